"""FP64 NumPy restatement of one fluidLB time step (test infrastructure only).

Every kernel below restates the reference CPU kernel named in its docstring,
vectorised over nodes but with the reference's per-node floating-point
operation order kept literally (same association, same constants, no fused
multiply-add), so that its results are bit-identical to the reference kernels
executed as Python.  Step order follows ``Solver.single_time_step``
(pylabolt/solvers/fluidLB.py:206-253): density -> gravity force -> velocity ->
collide -> periodic halo -> pull-stream (with solid bounce-back) -> boundary
elements in ``boundary_dict`` order.

Project extensions that have no reference kernel (restated here as the
project defines them): MRT collision with Guo forcing, the ``zero_gradient``
boundary type and a per-node body-force field.
"""
import numpy as np

from .setup import CX, CY, W, INV, INV_CS_2, INV_CS_4, EPS64

# MRT transform -- pylabolt/base/collision_operator.py:147-157 (rows rho, e,
# eps, jx, qx, jy, qy, pxx, pxy).
M_MRT = np.array([
    [1, 1, 1, 1, 1, 1, 1, 1, 1],
    [-4, -1, -1, -1, -1, 2, 2, 2, 2],
    [4, -2, -2, -2, -2, 1, 1, 1, 1],
    [0, 1, 0, -1, 0, 1, -1, -1, 1],
    [0, -2, 0, 2, 0, 1, -1, -1, 1],
    [0, 0, 1, 0, -1, 1, 1, -1, -1],
    [0, 0, -2, 0, 2, 1, 1, -1, -1],
    [0, 1, -1, 1, -1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 1, -1, 1, -1]], dtype=np.float64)
M_INV = np.linalg.inv(M_MRT)


def _seq_sum(values):
    """Left-to-right FP64 sum (the order of the reference's serial loop)."""
    if values.size == 0:
        return 0.0
    return float(np.cumsum(values)[-1])


def equilibrium(rho, ux, uy):
    """Second-order density-based equilibrium --
    pylabolt/parallel/cpu/equilibrium_kernels.py:6-35."""
    u2 = ux * ux + uy * uy
    feq = np.empty(rho.shape + (9,))
    for k in range(9):
        cu = CX[k] * ux + CY[k] * uy
        feq[..., k] = W[k] * rho * (
            1 + INV_CS_2 * cu + 0.5 * INV_CS_4 * cu * cu - 0.5 * INV_CS_2 * u2)
    return feq


def initialize(st):
    """pop = pop_new = f_eq(rho, u) on non-solid non-ghost nodes --
    pylabolt/parallel/cpu/equilibrium_kernels.py:38-78."""
    idx = np.nonzero(st.fluid)[0]
    feq = equilibrium(st.density[idx], st.velocity[idx, 0], st.velocity[idx, 1])
    st.pop[idx] = feq
    st.pop_new[idx] = feq


def compute_density(st, idx):
    """pylabolt/parallel/cpu/compute_fields_kernels.py:5-28."""
    pn = st.pop_new[idx]
    s = np.zeros(idx.size)
    for k in range(9):
        s = s + pn[:, k]
    st.density[idx] = s


def compute_force(st, idx):
    """F = rho * g -- pylabolt/parallel/cpu/force_field_kernels.py:5-25.
    Extension: a per-node body-force field replaces rho * g when given."""
    if st.body_force is not None:
        st.force[idx] = st.body_force[idx]
        return
    rho = st.density[idx]
    st.force[idx, 0] = rho * st.gravity[0]
    st.force[idx, 1] = rho * st.gravity[1]


def compute_velocity(st, idx):
    """pylabolt/parallel/cpu/compute_fields_kernels.py:31-65."""
    pn = st.pop_new[idx]
    sx = np.zeros(idx.size)
    sy = np.zeros(idx.size)
    for k in range(9):
        sx = sx + CX[k] * pn[:, k]
        sy = sy + CY[k] * pn[:, k]
    inv_density = 1 / (st.density[idx] + EPS64)
    st.velocity[idx, 0] = sx * inv_density + 0.5 * st.force[idx, 0] * inv_density
    st.velocity[idx, 1] = sy * inv_density + 0.5 * st.force[idx, 1] * inv_density


def collide_bgk(st, idx):
    """BGK_density_based_second_order_{None,guo_linear,guo_second_order} --
    pylabolt/parallel/cpu/collision_kernels.py:5-153."""
    rho = st.density[idx]
    ux = st.velocity[idx, 0]
    uy = st.velocity[idx, 1]
    fx = st.force[idx, 0]
    fy = st.force[idx, 1]
    omega = st.omega
    pn = st.pop_new[idx]
    u2 = ux * ux + uy * uy
    for k in range(9):
        cu = CX[k] * ux + CY[k] * uy
        pop_eq = W[k] * rho * (
            1 + INV_CS_2 * cu + 0.5 * INV_CS_4 * cu * cu - 0.5 * INV_CS_2 * u2)
        if st.forcing is None:
            st.pop[idx, k] = (1 - omega) * pn[:, k] + omega * pop_eq
            continue
        if st.forcing == "guo_linear":
            force_term = W[k] * (CX[k] * fx + CY[k] * fy) * INV_CS_2
        else:
            const_x = (CX[k] - ux) * INV_CS_2 + cu * CX[k] * INV_CS_4
            const_y = (CY[k] - uy) * INV_CS_2 + cu * CY[k] * INV_CS_4
            force_term = W[k] * (const_x * fx + const_y * fy)
        st.pop[idx, k] = ((1 - omega) * pn[:, k] + omega * pop_eq +
                          (1 - 0.5 * omega) * force_term)


def collide_mrt(st, idx):
    """MRT with Guo forcing in moment space (project restatement; the
    reference declares MRT but ships no kernel,
    pylabolt/base/collision_operator.py:92-100,136-165).

    m = M f ; m* = m - S (m - M f_eq) + (I - S/2) M Fbar ; f* = M^-1 m*,
    S = diag(1, s_e, s_eps, 1, s_q, 1, s_q, s_nu, s_nu), Fbar the Guo source of
    the configured forcing model in velocity space."""
    rho = st.density[idx]
    ux = st.velocity[idx, 0]
    uy = st.velocity[idx, 1]
    fx = st.force[idx, 0]
    fy = st.force[idx, 1]
    s_e, s_eps, s_q, s_nu = st.mrt_rates
    S = np.array([1.0, s_e, s_eps, 1.0, s_q, 1.0, s_q, s_nu, s_nu])
    f = st.pop_new[idx]
    m = f @ M_MRT.T
    meq = equilibrium(rho, ux, uy) @ M_MRT.T
    fbar = np.zeros_like(f)
    if st.forcing == "guo_linear":
        for k in range(9):
            fbar[:, k] = W[k] * (CX[k] * fx + CY[k] * fy) * INV_CS_2
    elif st.forcing == "guo_second_order":
        for k in range(9):
            cu = CX[k] * ux + CY[k] * uy
            const_x = (CX[k] - ux) * INV_CS_2 + cu * CX[k] * INV_CS_4
            const_y = (CY[k] - uy) * INV_CS_2 + cu * CY[k] * INV_CS_4
            fbar[:, k] = W[k] * (const_x * fx + const_y * fy)
    mstar = m - S * (m - meq) + (1 - 0.5 * S) * (fbar @ M_MRT.T)
    st.pop[idx] = mstar @ M_INV.T


def halo_pop(st):
    """Fill the ghost ring of the post-collision populations.

    ``wrap``: true periodic copy of the opposite inner column/row, x first
    then y, all ghost-inclusive -- pylabolt/parallel/gpu/MPI_kernels.py:51-99
    via MPI_operator.py:481-524.  ``selfcopy``: what the single-rank CPU path
    does (ghost <- adjacent inner column/row, MPI_operator.py:155-314)."""
    p = st.pop.reshape(st.nxp, st.nyp, 9)
    if st.x_periodic:
        if st.periodic_mode == "wrap":
            p[0, :, :] = p[st.nxp - 2, :, :]
            p[st.nxp - 1, :, :] = p[1, :, :]
        else:
            p[0, :, :] = p[1, :, :]
            p[st.nxp - 1, :, :] = p[st.nxp - 2, :, :]
    if st.y_periodic:
        if st.periodic_mode == "wrap":
            p[:, 0, :] = p[:, st.nyp - 2, :]
            p[:, st.nyp - 1, :] = p[:, 1, :]
        else:
            p[:, 0, :] = p[:, 1, :]
            p[:, st.nyp - 1, :] = p[:, st.nyp - 2, :]


def stream(st, idx):
    """Pull streaming with moving-solid bounce-back --
    pylabolt/parallel/cpu/streaming_kernels.py:5-47 (``scalar_based_kernel``)."""
    rho = st.density[idx]
    st.pop_new[idx, 0] = st.pop[idx, 0]
    for k in range(1, 9):
        nb = idx - CX[k] * st.nyp - CY[k]
        kinv = INV[k]
        temp = 2 * W[kinv] * rho * INV_CS_2 * (
            CX[kinv] * st.velocity[nb, 0] + CY[kinv] * st.velocity[nb, 1])
        bb = st.pop[idx, kinv] - temp
        st.pop_new[idx, k] = np.where(st.solid[nb], bb, st.pop[nb, k])


def apply_boundaries(st):
    """Boundary elements in ``boundary_dict`` order (last writer wins) --
    pylabolt/base/boundary_operator.py:138-164 with the kernels of
    pylabolt/parallel/cpu/fluid_boundary_kernels.py."""
    for el in st.elements:
        nodes = el.nodes[~st.solid[el.nodes]]
        if el.type == "periodic" or nodes.size == 0:
            continue
        if el.type == "bounce_back":
            # fluid_boundary_kernels.py:5-25
            for k in range(3):
                st.pop_new[nodes, el.inv_list[k]] = st.pop[nodes, el.out_list[k]]
        elif el.type == "fixed_velocity":
            # fluid_boundary_kernels.py:28-62
            uw = np.asarray(el.value, dtype=np.float64)
            rho = st.density[nodes]
            for k in range(3):
                o, i = el.out_list[k], el.inv_list[k]
                temp = 2 * W[o] * rho * INV_CS_2 * (CX[o] * uw[0] + CY[o] * uw[1])
                st.pop_new[nodes, i] = st.pop[nodes, o] - temp
        elif el.type == "fixed_pressure":
            # fluid_boundary_kernels.py:100-152, with the surface normal taken
            # as an integer offset (the reference indexes with a float normal
            # there, boundary.py:63-78, which cannot run).
            rho_w = np.float64(el.value)
            nrm = nodes + el.normal[0] * st.nyp + el.normal[1]
            ux = st.velocity[nodes, 0]
            uy = st.velocity[nodes, 1]
            uex = ux + 0.5 * (ux - st.velocity[nrm, 0])
            uey = uy + 0.5 * (uy - st.velocity[nrm, 1])
            u2 = uex * uex + uey * uey
            for k in range(3):
                o, i = el.out_list[k], el.inv_list[k]
                cu = CX[o] * uex + CY[o] * uey
                temp = 2 * W[o] * rho_w * (
                    1 + 0.5 * INV_CS_4 * cu * cu - 0.5 * INV_CS_2 * u2)
                st.pop_new[nodes, i] = -st.pop[nodes, o] + temp
        elif el.type == "zero_gradient":
            # Project extension (README.rst:83 names it, no kernel exists):
            # the unknown incoming population i at boundary node b takes the
            # post-collision value that reaches the inward neighbour b+n along
            # i, i.e. pop[b + n - c_i, i] (periodic wrap applied); when that
            # source is a ghost or a solid node, pop[b + n, i].
            for k in range(3):
                i = el.inv_list[k]
                src = _zg_source(st, nodes, el.normal, i)
                st.pop_new[nodes, i] = st.pop[src, i]


def _zg_source(st, nodes, normal, i):
    x = nodes // st.nyp - 1 + normal[0] - CX[i]
    y = nodes % st.nyp - 1 + normal[1] - CY[i]
    if st.x_periodic:
        x = np.mod(x, st.Nx)
    if st.y_periodic:
        y = np.mod(y, st.Ny)
    src = (x + 1) * st.nyp + (y + 1)
    inside = (x >= 0) & (x < st.Nx) & (y >= 0) & (y < st.Ny)
    src = np.where(inside, src, 0)
    ok = inside & ~st.solid[src]
    fallback = nodes + normal[0] * st.nyp + normal[1]
    return np.where(ok, src, fallback)


def step(st):
    """One ``Solver.single_time_step`` (fluidLB.py:206-253)."""
    idx = np.nonzero(st.fluid)[0]
    compute_density(st, idx)
    compute_force(st, idx)
    compute_velocity(st, idx)
    if st.collision == "MRT":
        collide_mrt(st, idx)
    else:
        collide_bgk(st, idx)
    halo_pop(st)
    stream(st, idx)
    apply_boundaries(st)


class Residue:
    """``ResidueOperator`` restated: pylabolt/utils/residues.py:60-62,171-222
    with the kernels of pylabolt/parallel/cpu/compute_residues_kernels.py:6-73.
    The old fields start at zero; sums run over non-solid non-ghost nodes in
    node order."""

    def __init__(self, st):
        self.density_old = np.zeros(st.size)
        self.velocity_old = np.zeros((st.size, 2))

    def compute(self, st):
        idx = np.nonzero(st.fluid)[0]
        out = []
        d, do = st.density[idx], self.density_old[idx]
        num = _seq_sum((d - do) * (d - do))
        den = _seq_sum(do * do)
        out.append(np.sqrt(num / (den + EPS64)))
        for c in range(2):
            v, vo = st.velocity[idx, c], self.velocity_old[idx, c]
            num = _seq_sum((v - vo) * (v - vo))
            den = _seq_sum(vo * vo)
            out.append(np.sqrt(num / (den + EPS64)))
        self.density_old[idx] = d
        self.velocity_old[idx] = st.velocity[idx]
        return np.array(out)


def run(st, nsteps, std_out_interval=None):
    """Initialise and advance ``nsteps`` steps (fluidLB.py:320-356).  Returns
    the residual history ``[(t, res_rho, res_ux, res_uy), ...]``."""
    initialize(st)
    res = Residue(st)
    hist = []
    for t in range(1, nsteps + 1):
        step(st)
        if std_out_interval and t % std_out_interval == 0:
            hist.append((t, *res.compute(st)))
    return hist


# ---------------------------------------------------------------------------
# momentum exchange (evaluated after a time step)

def obstacle_force_torque(pop, pop_new, solid, solid_id, fluid_boundary, nx, ny,
                          ref_point, obstacle_id, x_periodic, y_periodic):
    """compute_force_torque_single_phase,
    pylabolt/parallel/cpu/force_torque_kernels.py:11-90.  Padded AoS inputs
    ([(nx+2)*(ny+2)] flags, [.., 9] populations); sums in the serial loop
    order (node, then direction).  Returns [fx, fy, torque]."""
    nyp = ny + 2
    idx = np.arange((nx + 2) * nyp)
    x, y = idx // nyp, idx % nyp
    ghost = (x == 0) | (x == nx + 1) | (y == 0) | (y == ny + 1)
    sel = np.nonzero(~ghost & fluid_boundary & (solid_id == obstacle_id))[0]
    xs, ys = sel // nyp, sel % nyp
    rx = (xs - 1) - ref_point[0]
    ry = (ys - 1) - ref_point[1]
    rxm, rym = rx.astype(np.float64), ry.astype(np.float64)
    if x_periodic:
        a = rx + nx
        rxm = np.where(np.abs(a) < np.abs(rxm), a, rxm)
        b = rx - nx
        rxm = np.where(np.abs(b) < np.abs(rxm), b, rxm)
    if y_periodic:
        a = ry + ny
        rym = np.where(np.abs(a) < np.abs(rym), a, rym)
        b = ry - ny
        rym = np.where(np.abs(b) < np.abs(rym), b, rym)
    vx = np.zeros((sel.size, 9))
    vy = np.zeros((sel.size, 9))
    tq = np.zeros((sel.size, 9))
    for k in range(9):
        nb = (xs + CX[k]) * nyp + ys + CY[k]
        m = solid[nb]
        ki = INV[k]
        px = pop[sel, k] * CX[k] - pop_new[sel, ki] * CX[ki]
        py = pop[sel, k] * CY[k] - pop_new[sel, ki] * CY[ki]
        vx[m, k] = px[m]
        vy[m, k] = py[m]
        tq[m, k] = rxm[m] * py[m] - rym[m] * px[m]
    return np.array([_seq_sum(vx.ravel()), _seq_sum(vy.ravel()), _seq_sum(tq.ravel())])


def boundary_force(pop, pop_new, solid, boundary_nodes, out_list, inv_list):
    """compute_boundary_force_single_phase,
    pylabolt/parallel/cpu/force_torque_kernels.py:96-141 (padded node
    indices).  Returns [fx, fy]."""
    nodes = np.asarray(boundary_nodes)
    nodes = nodes[~solid[nodes]]
    vx = np.zeros((nodes.size, len(out_list)))
    vy = np.zeros((nodes.size, len(out_list)))
    for j, (ko, ki) in enumerate(zip(out_list, inv_list)):
        vx[:, j] = pop[nodes, ko] * CX[ko] - pop_new[nodes, ki] * CX[ki]
        vy[:, j] = pop[nodes, ko] * CY[ko] - pop_new[nodes, ki] * CY[ki]
    return np.array([_seq_sum(vx.ravel()), _seq_sum(vy.ravel())])
