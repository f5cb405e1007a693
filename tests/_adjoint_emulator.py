"""NumPy transcription of the CUDA adjoint (pylabolt_gb300/csrc/lbm_adjoint.cuh
and lbm_adjoint_backward): the same transpose tables, the same reverse-mode
formulas, node by node, FP64.  Test helper: lets the adjoint's math be checked
against the torch autograd reference without a GPU."""
import numpy as np

from pylabolt_gb300.capi import LINK_PULL, LINK_BB, LINK_MBB
from pylabolt_gb300.lattice import CX, CY, W, INV
from _fused_emulator import FusedEmulator


def transpose_tables(em):
    """tr_reader / tr_self per record, as lbm_capi.cu builds them."""
    case, rec = em.case, em.rec
    nx, ny = case.nx, case.ny
    bulk = np.ones(nx * ny, dtype=bool)
    bulk[rec["node"]] = False
    bulk &= ~em.solid
    reader = {}
    for r in range(len(rec)):
        for k in range(1, 9):
            if rec["type"][r, k] == LINK_PULL:
                key = (int(rec["src"][r, k]), k)
                assert key not in reader
                reader[key] = int(rec["node"][r])
    tr_reader = np.full((len(rec), 9), -1, dtype=np.int64)
    tr_self = np.zeros((len(rec), 9), dtype=bool)
    for r in range(len(rec)):
        s = int(rec["node"][r])
        sx, sy = s // ny, s % ny
        tr_reader[r, 0] = s
        for m in range(1, 9):
            yx, yy = sx + CX[m], sy + CY[m]
            if 0 <= yx < nx and 0 <= yy < ny and bulk[yx * ny + yy]:
                tr_reader[r, m] = yx * ny + yy
            else:
                tr_reader[r, m] = reader.get((s, m), -1)
            tr_self[r, m] = rec["type"][r, INV[m]] in (LINK_BB, LINK_MBB)
    return tr_reader, tr_self


def adjoint(case, nsteps, grad_u, force=None):
    """Forward nsteps with the fused plan, then the reverse pass.
    Returns (dL/dF [n,2] or None, dL/dtau, dL/du_wall [2])."""
    em = FusedEmulator(case)
    em.initialize()
    ny = case.ny
    n = case.nx * case.ny
    states, sides = [em.fstar.copy()], [em.side.copy()]
    for t in range(1, nsteps + 1):
        em.step()
        states.append(em.fstar.copy())
        sides.append(em.side.copy())
    tr_reader, tr_self = transpose_tables(em)
    rec = em.rec
    spec_row = np.full(n, -1)
    spec_row[rec["node"]] = np.arange(len(rec))
    fluid = np.nonzero(~em.solid)[0]
    i2, i4, om = case.inv_cs_2, case.inv_cs_4, case.omega
    omh = 1 - 0.5 * om
    forc = {None: 0, "guo_linear": 1, "guo_second_order": 2}[case.forcing]
    gF = np.zeros((n, 2))
    g_om = 0.0
    g_uw = np.zeros(2)
    a_next = None
    for t in range(nsteps, 0, -1):
        # f^t from p_{t-1}: replay the emulator's pull
        em.fstar = states[t - 1]
        em.side = sides[t - 1]
        em.nopull = t == 1
        fin = em._incoming()
        a_cur = np.zeros((n, 9))
        for s in fluid:
            f = fin[s]
            r = spec_row[s]
            rho = f.sum()
            jx, jy = (CX * f).sum(), (CY * f).sum()
            if forc and force is not None:
                Fx, Fy = force[s]
                dFx = dFy = 0.0
            elif forc:
                dFx, dFy = case.gravity
                Fx, Fy = rho * dFx, rho * dFy
            else:
                Fx = Fy = dFx = dFy = 0.0
            ux, uy = (jx + 0.5 * Fx) / rho, (jy + 0.5 * Fy) / rho
            u2 = ux * ux + uy * uy
            A = np.zeros(9)
            if a_next is not None:
                for m in range(9):
                    if r < 0:
                        A[m] = a_next[(s // ny + CX[m]) * ny + s % ny + CY[m], m]
                    else:
                        rd = tr_reader[r, m]
                        A[m] = (a_next[rd, m] if rd >= 0 else 0.0) + \
                            (a_next[s, INV[m]] if tr_self[r, m] else 0.0)
            # moments of A (lbm_adjoint.cuh step 3)
            M0 = (W * A).sum()
            Mx, My = (W * CX * A).sum(), (W * CY * A).sum()
            Mxx, Myy, Mxy = (W * CX * CX * A).sum(), (W * CY * CY * A).sum(), (W * CX * CY * A).sum()
            uMc = ux * Mx + uy * My
            Mccux, Mccuy = Mxx * ux + Mxy * uy, Mxy * ux + Myy * uy
            uMccu = ux * Mccux + uy * Mccuy
            Bm1 = -0.5 * i2 * u2 * M0 + i2 * uMc + 0.5 * i4 * uMccu
            adj_rho = om * (M0 + Bm1)
            adj_ux = om * rho * (i2 * Mx + i4 * Mccux - i2 * ux * M0)
            adj_uy = om * rho * (i2 * My + i4 * Mccuy - i2 * uy * M0)
            adj_Fx = adj_Fy = 0.0
            g_om += rho * (M0 + Bm1) - (A * f).sum()
            if forc == 1:
                g_om -= 0.5 * i2 * (Mx * Fx + My * Fy)
                adj_Fx += omh * i2 * Mx
                adj_Fy += omh * i2 * My
            elif forc == 2:
                uF = ux * Fx + uy * Fy
                MccFx, MccFy = Mxx * Fx + Mxy * Fy, Mxy * Fx + Myy * Fy
                g_om -= 0.5 * (i2 * (Mx * Fx + My * Fy) - i2 * M0 * uF + i4 * (ux * MccFx + uy * MccFy))
                adj_Fx += omh * (i2 * Mx - i2 * M0 * ux + i4 * Mccux)
                adj_Fy += omh * (i2 * My - i2 * M0 * uy + i4 * Mccuy)
                adj_ux += omh * (-i2 * M0 * Fx + i4 * MccFx)
                adj_uy += omh * (-i2 * M0 * Fy + i4 * MccFy)
            if t == nsteps:
                adj_ux += grad_u[s, 0]
                adj_uy += grad_u[s, 1]
            adj_jx, adj_jy = adj_ux / rho, adj_uy / rho
            adj_Fx += 0.5 * adj_ux / rho
            adj_Fy += 0.5 * adj_uy / rho
            adj_rho -= (adj_ux * ux + adj_uy * uy) / rho
            if forc and force is None:
                adj_rho += adj_Fx * dFx + adj_Fy * dFy
            mbb = 0.0
            if r >= 0 and a_next is not None:
                for k in range(1, 9):
                    if rec["type"][r, k] != LINK_MBB:
                        continue
                    kb = INV[k]
                    coef = -2 * W[kb] * i2
                    mbb += coef * rec["param"][r, k] * a_next[s, k]
                    if rec["wall"][r]:
                        g_uw += coef * rho * np.array([CX[kb], CY[kb]]) * a_next[s, k]
            a_cur[s] = (1 - om) * A + adj_rho + adj_jx * CX + adj_jy * CY + mbb
            gF[s] += (adj_Fx, adj_Fy)
        a_next = a_cur
    return (gF if force is not None else None), -g_om * om * om, g_uw
