"""Obstacle geometry fields and momentum-exchange link sets (host side).

Geometry: the fields the reference's ObstacleOperator derives once at set-up
and writes in every ``output/fields/t_<n>.npz``:

* ``solid_id``        obstacle id of solid nodes (construct_circle,
                      pylabolt/parallel/cpu/obstacle_kernels.py:43-93) and of
                      fluid boundary nodes (the first solid neighbour in
                      direction order, compute_obstacle_boundary :307-350);
                      -1 elsewhere
* ``solid_boundary``  solid node with a non-solid neighbour (:307-350)
* ``fluid_boundary``  fluid node with a solid neighbour (:307-350)
* ``surface_normals`` on the boundary nodes of each obstacle: the unit
                      vector from a circle's centre (minimum image on
                      periodic axes; compute_normals_circle :95-143), or an
                      ellipse's unit gradient of (x'/a)^2 + (y'/b)^2 turned
                      back by the inclination (compute_normals_ellipse
                      :244-302)

Ghost nodes carry what the reference's single-rank ``halo_exchange_cpu``
leaves there before these kernels run (pylabolt/base/obstacle_operator.py:
35-41 with pylabolt/parallel/MPI_operator.py:131-153,155-314): on a periodic
axis the ghost copies the adjacent inner node (the rank exchanges with
itself), on a non-periodic axis it stays non-solid with id -1.  The x
exchange runs first over all rows, then the y exchange over all columns.

Force links: the (node, direction) pairs over which the reference sums the
momentum exchange, grouped per obstacle (compute_force_torque_single_phase,
pylabolt/parallel/cpu/force_torque_kernels.py:11-90) and per wall boundary
element (compute_boundary_force_single_phase, :96-141).  They are evaluated on
the GPU by ``lbm_forces``.
"""
import numpy as np

from .capi import FORCE_LINK_DTYPE
from .lattice import CX, CY, INV


def _fill_ghosts(a, x_periodic, y_periodic):
    """Single-rank halo exchange of a padded [nx+2, ny+2] field in place."""
    if x_periodic:
        a[0, :] = a[1, :]
        a[-1, :] = a[-2, :]
    if y_periodic:
        a[:, 0] = a[:, 1]
        a[:, -1] = a[:, -2]


def _min_image(r, n, periodic):
    """The reference's minimum-image rule: try r + n, then r - n."""
    if not periodic:
        return r
    m = r.copy()
    a = r + n
    m = np.where(np.abs(a) < np.abs(m), a, m)
    b = r - n
    return np.where(np.abs(b) < np.abs(m), b, m)


class Geometry:
    """Padded geometry fields of a Case ([nx+2, ny+2] arrays, x-major).
    `solid`, `solid_id` [nx, ny], `centers` {obstacle id: (x, y)} and
    `angles` {obstacle id: radians} replace the case's set-up geometry
    (moving obstacles: the device's node flags, positions and ellipse
    orientations at the time of output)."""

    def __init__(self, case, solid=None, solid_id=None, centers=None, angles=None):
        nx, ny = case.nx, case.ny
        self.nx, self.ny = nx, ny
        self.x_periodic, self.y_periodic = case.x_periodic, case.y_periodic
        centers = centers or {}
        angles = angles or {}   # {obstacle id: inclination in radians} of moving ellipses
        solid_a = np.zeros((nx + 2, ny + 2), dtype=bool)
        solid_id_a = np.full((nx + 2, ny + 2), -1, dtype=np.int64)
        solid_a[1:-1, 1:-1] = case.solid if solid is None else solid
        solid_id_a[1:-1, 1:-1] = case.solid_id if solid_id is None else solid_id
        solid, solid_id = solid_a, solid_id_a
        _fill_ghosts(solid, self.x_periodic, self.y_periodic)
        _fill_ghosts(solid_id, self.x_periodic, self.y_periodic)
        inner = np.zeros_like(solid)
        inner[1:-1, 1:-1] = True
        solid_boundary = np.zeros_like(solid)
        fluid_boundary = np.zeros_like(solid)
        first_id = np.full_like(solid_id, -1)
        found = np.zeros_like(solid)
        for k in range(9):
            nb_solid = np.zeros_like(solid)
            nb_id = np.full_like(solid_id, -1)
            nb_solid[1:-1, 1:-1] = solid[1 + CX[k]:nx + 1 + CX[k], 1 + CY[k]:ny + 1 + CY[k]]
            nb_id[1:-1, 1:-1] = solid_id[1 + CX[k]:nx + 1 + CX[k], 1 + CY[k]:ny + 1 + CY[k]]
            solid_boundary |= inner & solid & ~nb_solid
            take = inner & ~solid & nb_solid & ~found
            first_id = np.where(take, nb_id, first_id)
            found |= take
        fluid_boundary = found
        solid_id = np.where(fluid_boundary, first_id, solid_id)
        self._check_overlap(solid_id, fluid_boundary, inner)
        normals = np.zeros((nx + 2, ny + 2, 2), dtype=np.float64)
        X, Y = np.meshgrid(np.arange(-1, nx + 1, dtype=np.float64),
                           np.arange(-1, ny + 1, dtype=np.float64), indexing="ij")
        for obs in case.obstacles:
            sel = inner & (solid_id == obs.id) & (solid_boundary | fluid_boundary)
            cx, cy = centers.get(obs.id, obs.center)
            rx = _min_image(X - cx, nx, self.x_periodic)
            ry = _min_image(Y - cy, ny, self.y_periodic)
            if obs.type == "ellipse":
                a, b = (np.float64(v) for v in obs.semi_axes)
                alpha = angles.get(obs.id, np.float64(obs.inclination) * np.pi / 180)
                cos_a, sin_a = np.cos(alpha), np.sin(alpha)
                xp = rx * cos_a + ry * sin_a
                yp = -rx * sin_a + ry * cos_a
                gx = xp / (a * a)
                gy = yp / (b * b)
                rx = gx * cos_a - gy * sin_a
                ry = gx * sin_a + gy * cos_a
            mag = np.sqrt(rx * rx + ry * ry)
            with np.errstate(invalid="ignore", divide="ignore"):
                normals[..., 0] = np.where(sel, rx / mag, normals[..., 0])
                normals[..., 1] = np.where(sel, ry / mag, normals[..., 1])
        self.solid = solid
        self.solid_id = solid_id
        self.solid_boundary = solid_boundary
        self.fluid_boundary = fluid_boundary
        self.surface_normals = normals

    @staticmethod
    def _check_overlap(solid_id, fluid_boundary, inner):
        """check_fluid_boundary_overlap (obstacle_kernels.py:353-380) and the
        message of obstacle_operator.py:168-183."""
        nx, ny = solid_id.shape[0] - 2, solid_id.shape[1] - 2
        bad = np.zeros_like(fluid_boundary)
        own = solid_id[1:-1, 1:-1]
        for k in range(9):
            nb = solid_id[1 + CX[k]:nx + 1 + CX[k], 1 + CY[k]:ny + 1 + CY[k]]
            bad[1:-1, 1:-1] |= ~((nb == own) | (nb == -1))
        n = int((bad & fluid_boundary & inner).sum())
        if n > 0:
            raise ValueError(
                f"Fluid Boundary node overlap detected for {n} nodes! This indicates two solid "
                "obstacles have a common fluid boundary node which is illegal! To avoid this "
                "issue, ensure solid particle surfaces have 2-3 lattice nodes in between.")

    def inner(self, name):
        """Inner-node field in the order the reference saves it
        (copy_inner_data, pylabolt/parallel/cpu/io_operator_kernels.py)."""
        a = getattr(self, name)[1:-1, 1:-1]
        n = self.nx * self.ny
        return np.ascontiguousarray(a.reshape(n, -1) if a.ndim == 3 else a.reshape(n))


def force_links(case, geometry=None):
    """Momentum-exchange links of every static obstacle (groups 0..nobs-1, in
    obstacle order; moving obstacles are summed on the device by the step
    itself) and every wall boundary element (the following groups, in element
    order).  Returns (links [FORCE_LINK_DTYPE], obstacle names, wall element
    names)."""
    geo = geometry or Geometry(case)
    nx, ny = case.nx, case.ny
    recs = []
    solid = geo.solid
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    fb = geo.fluid_boundary[1:-1, 1:-1]
    sid = geo.solid_id[1:-1, 1:-1]
    static = [o for o in case.obstacles if o not in case.moving]
    for g, obs in enumerate(static):
        ref = obs.center              # the reference's ref_point (obstacle.py:450)
        rx = _min_image(X - ref[0], nx, geo.x_periodic)
        ry = _min_image(Y - ref[1], ny, geo.y_periodic)
        sel = fb & (sid == obs.id)
        for k in range(9):
            nb = solid[1 + CX[k]:nx + 1 + CX[k], 1 + CY[k]:ny + 1 + CY[k]]
            m = sel & nb
            if not m.any():
                continue
            r = np.zeros(int(m.sum()), dtype=FORCE_LINK_DTYPE)
            r["node"] = (X[m] * ny + Y[m])
            r["group"] = g
            r["k_out"] = k
            r["k_in"] = INV[k]
            r["rx"] = rx[m]
            r["ry"] = ry[m]
            recs.append(r)
    walls = [el for el in case.elements if el.wall]
    for j, el in enumerate(walls):
        keep = ~case.solid[el.xs, el.ys]
        nodes = el.xs[keep] * ny + el.ys[keep]
        for ko, ki in zip(el.out_list, el.inv_list):
            r = np.zeros(nodes.size, dtype=FORCE_LINK_DTYPE)
            r["node"] = nodes
            r["group"] = len(static) + j
            r["k_out"] = ko
            r["k_in"] = ki
            recs.append(r)
    links = np.concatenate(recs) if recs else np.zeros(0, dtype=FORCE_LINK_DTYPE)
    return links, [o.name for o in static], [el.name for el in walls]

