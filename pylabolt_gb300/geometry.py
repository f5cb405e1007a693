"""Link table of the boundary ("special") nodes of a case.

The fused kernel pulls the nine incoming populations of a bulk node from its
neighbours.  Every node for which that is not true gets a record of nine links
(``LbmNodeLinks`` in include/lbm_gb300.h).  The rules restate, per node and
direction, what the reference's stream + boundary kernels write into
``pop_new``:

* streaming (pylabolt/parallel/cpu/streaming_kernels.py:5-47): pull
  ``pop[x - c_k, k]``; if that node is solid, moving-solid bounce-back
  ``pop[x, kbar] - 2 w rho(x) inv_cs_2 (c_kbar . u_solid)`` (a plain bounce-back
  when the solid is at rest);
* a source outside the grid reads the ghost ring: after the periodic wrap
  (pylabolt/parallel/gpu/MPI_kernels.py:51-99) it holds the opposite node's
  population (whose value is 0 if that node is solid); on non-periodic sides it
  holds 0.  Ghost nodes are never solid;
* boundary elements are applied after streaming, in ``boundary_dict`` order,
  to their non-solid nodes, last writer wins
  (pylabolt/base/boundary_operator.py:138-164): ``bounce_back`` -> BB,
  ``fixed_velocity`` -> MBB with ``c_kbar . u_w``
  (fluid_boundary_kernels.py:28-62), ``fixed_pressure`` -> ABB with rho_w and
  the inward neighbour x+n (fluid_boundary_kernels.py:100-152, integer normal),
  ``zero_gradient`` -> PULL from ``x + n - c_k`` (extension).
"""
import numpy as np

from .capi import NODE_LINKS_DTYPE, LINK_PULL, LINK_ZERO, LINK_BB, LINK_MBB, LINK_ABB
from .lattice import CX, CY, INV


def _dilate(mask, xper, yper):
    out = mask.copy()
    for k in range(1, 9):
        sh = np.roll(mask, (int(CX[k]), int(CY[k])), axis=(0, 1))
        if not xper:
            if CX[k] == 1:
                sh[0, :] = False
            elif CX[k] == -1:
                sh[-1, :] = False
        if not yper:
            if CY[k] == 1:
                sh[:, 0] = False
            elif CY[k] == -1:
                sh[:, -1] = False
        out |= sh
    return out


def build_links(case):
    """Returns (node_solid uint8 [nx*ny] inner x-major, records structured array)."""
    nx, ny = case.nx, case.ny
    solid = case.solid
    special = np.zeros((nx, ny), dtype=bool)
    special[0, :] = special[-1, :] = True
    special[:, 0] = special[:, -1] = True
    if solid.any():
        special |= _dilate(solid, case.x_periodic, case.y_periodic)
    for el in case.elements:
        if el.type == "fixed_pressure":
            ax = el.xs + el.normal[0]
            ay = el.ys + el.normal[1]
            ok = ~solid[el.xs, el.ys]
            if np.any(solid[ax[ok], ay[ok]]):
                raise ValueError("fixed_pressure boundary " + el.name +
                                 ": the inward neighbour of a boundary node is solid")
            special[ax, ay] = True
    special &= ~solid
    xs, ys = np.nonzero(special)
    node = xs * ny + ys
    n = node.size
    rec = np.zeros(n, dtype=NODE_LINKS_DTYPE)
    rec["node"] = node
    typ = np.zeros((n, 9), dtype=np.int8)
    src = np.zeros((n, 9), dtype=np.int64)
    aux = np.zeros((n, 9), dtype=np.int64)
    par = np.zeros((n, 9), dtype=np.float64)
    wall = np.zeros(n, dtype=np.int8)
    src[:, 0] = node
    u = case.velocity
    for k in range(1, 9):
        sx = xs - CX[k]
        sy = ys - CY[k]
        inx = (sx >= 0) & (sx < nx)
        iny = (sy >= 0) & (sy < ny)
        wrapped = ~(inx & iny)
        if case.x_periodic:
            sx = np.mod(sx, nx)
        if case.y_periodic:
            sy = np.mod(sy, ny)
        inside = (sx >= 0) & (sx < nx) & (sy >= 0) & (sy < ny)
        sxc = np.clip(sx, 0, nx - 1)
        syc = np.clip(sy, 0, ny - 1)
        ssol = inside & solid[sxc, syc]
        kb = INV[k]
        cu = CX[kb] * u[sxc, syc, 0] + CY[kb] * u[sxc, syc, 1]
        t = np.full(n, LINK_PULL, dtype=np.int8)
        t[~inside] = LINK_ZERO
        # through the ghost ring a solid source contributes its zero population
        t[inside & ssol & wrapped] = LINK_ZERO
        direct_solid = inside & ssol & ~wrapped
        t[direct_solid & (cu == 0)] = LINK_BB
        t[direct_solid & (cu != 0)] = LINK_MBB
        typ[:, k] = t
        src[:, k] = np.where(inside & ~ssol, sxc * ny + syc, 0)
        par[:, k] = np.where(direct_solid, cu, 0.0)
    for el in case.elements:
        if el.type == "periodic":
            continue
        keep = ~solid[el.xs, el.ys]
        ex, ey = el.xs[keep], el.ys[keep]
        rows = np.searchsorted(node, ex * ny + ey)
        for k in el.inv_list:
            kb = INV[k]
            src[rows, k] = 0
            par[rows, k] = 0.0
            aux[rows, k] = 0
            if el.type == "bounce_back":
                typ[rows, k] = LINK_BB
            elif el.type == "fixed_velocity":
                typ[rows, k] = LINK_MBB
                wall[rows] = 1
                par[rows, k] = CX[kb] * np.float64(el.value[0]) + CY[kb] * np.float64(el.value[1])
            elif el.type == "fixed_pressure":
                typ[rows, k] = LINK_ABB
                par[rows, k] = el.value
                aux[rows, k] = (ex + el.normal[0]) * ny + (ey + el.normal[1])
            elif el.type == "zero_gradient":
                sx = ex + el.normal[0] - CX[k]
                sy = ey + el.normal[1] - CY[k]
                if case.x_periodic:
                    sx = np.mod(sx, nx)
                if case.y_periodic:
                    sy = np.mod(sy, ny)
                inside = (sx >= 0) & (sx < nx) & (sy >= 0) & (sy < ny)
                sxc = np.clip(sx, 0, nx - 1)
                syc = np.clip(sy, 0, ny - 1)
                ok = inside & ~solid[sxc, syc]
                fb = (ex + el.normal[0]) * ny + (ey + el.normal[1])
                typ[rows, k] = LINK_PULL
                src[rows, k] = np.where(ok, sxc * ny + syc, fb)
            else:
                raise ValueError("Unsupported boundary condition for fluid: " + el.type)
    rec["type"] = typ
    rec["src"] = src
    rec["aux"] = aux
    rec["param"] = par
    rec["wall"] = wall
    node_solid = np.ascontiguousarray(solid.astype(np.uint8).ravel())
    return node_solid, rec
