"""Reference-layout state builder for the oracle (test infrastructure only).

Builds, from ``simulation.py``-style case dictionaries, the arrays the
reference's CPU kernels operate on, in the reference's own layout:

* padded grid ``(Nx+2) x (Ny+2)`` with a one-node ghost ring, node index
  ``ind = x * (Ny+2) + y`` (x-major, y fastest) -- pylabolt/base/fields.py:166-179,
  pylabolt/parallel/domain.py:80-85;
* populations AoS ``[node][q]`` -- pylabolt/base/fields.py:83-92;
* boundary elements with node lists on the first interior ring
  ``ind = (i+1)*(Ny+2) + (j+1)`` and the per-location out/inv direction lists
  -- pylabolt/base/boundary.py:63-127, :451-485;
* circle obstacles rasterised by ``dist^2 <= r^2`` and ellipses by
  ``(x'/a)^2 + (y'/b)^2 <= 1`` in the inclined frame, on global inner-node
  coordinates with the periodic minimum image --
  pylabolt/parallel/cpu/obstacle_kernels.py:11-93,151-241;
* initial fields ``fixed`` / ``func`` on non-ghost nodes --
  pylabolt/base/init_fields.py:274-375.  The extension type ``array`` takes an
  explicit inner-node array ``[Nx, Ny]`` (``[Nx, Ny, 2]`` for velocity).

Only FP64 (``precision: "double"``) is restated; the oracle is the FP64
reference for every precision mode of the product.
"""
import numpy as np

# D2Q9 tables -- pylabolt/base/lattice.py:45-60
CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], dtype=np.int64)
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1], dtype=np.int64)
W = np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 36, 1 / 36],
             dtype=np.float64)
INV = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6], dtype=np.int64)

# Sound-speed constants exactly as pylabolt/base/lattice.py:41-44 computes them
# in FP64 (inv_cs_2 == 2.999999999999999, not 3).
CS = np.float64(1 / np.sqrt(3))
CS_2 = CS * CS
INV_CS_2 = 1.0 / CS_2
INV_CS_4 = INV_CS_2 * INV_CS_2
EPS64 = np.finfo(np.float64).eps  # control.py:49 float_min

# location -> (inward normal, out_list, inv_list) -- boundary.py:63-78
LOCATIONS = {
    "bottom": ((0, 1), (4, 7, 8), (2, 5, 6)),
    "top": ((0, -1), (2, 5, 6), (4, 7, 8)),
    "left": ((1, 0), (3, 6, 7), (1, 8, 5)),
    "right": ((-1, 0), (1, 8, 5), (3, 6, 7)),
}

FLUID_BC_TYPES = ("bounce_back", "fixed_velocity", "fixed_pressure",
                  "periodic", "zero_gradient")


class Element:
    """One boundary element (one segment of one ``boundary_dict`` entry)."""

    def __init__(self, name, bc_type, location, nodes, value):
        self.name = name
        self.type = bc_type
        self.location = location
        normal, out_list, inv_list = LOCATIONS[location]
        self.normal = np.array(normal, dtype=np.int64)
        self.out_list = np.array(out_list, dtype=np.int64)
        self.inv_list = np.array(inv_list, dtype=np.int64)
        self.nodes = np.asarray(nodes, dtype=np.int64)
        self.value = value


class RefState:
    """Arrays of one case in the reference's padded AoS layout."""

    def __init__(self, nx, ny):
        self.Nx, self.Ny = int(nx), int(ny)
        self.nxp, self.nyp = self.Nx + 2, self.Ny + 2
        self.size = self.nxp * self.nyp
        ind = np.arange(self.size)
        i, j = ind // self.nyp, ind % self.nyp
        self.ghost = (i == 0) | (j == 0) | (i == self.nxp - 1) | (j == self.nyp - 1)
        self.solid = np.zeros(self.size, dtype=bool)
        self.density = np.zeros(self.size)
        self.velocity = np.zeros((self.size, 2))
        self.force = np.zeros((self.size, 2))
        self.pop = np.zeros((self.size, 9))
        self.pop_new = np.zeros((self.size, 9))
        self.elements = []
        self.x_periodic = False
        self.y_periodic = False
        self.collision = "BGK"
        self.forcing = None
        self.omega = 1.0
        self.gravity = np.zeros(2)
        self.body_force = None          # optional per-node force (size, 2)
        self.mrt_rates = None           # (s_e, s_eps, s_q, s_nu) for MRT
        self.periodic_mode = "wrap"     # "wrap" (GPU path) or "selfcopy" (1-rank CPU path)

    def padded_index(self, x, y):
        return (np.asarray(x) + 1) * self.nyp + (np.asarray(y) + 1)

    @property
    def fluid(self):
        return ~self.solid & ~self.ghost

    def inner(self, arr):
        """Inner-node view ``[Nx, Ny, ...]`` of a padded node array."""
        a = np.asarray(arr).reshape((self.nxp, self.nyp) + np.asarray(arr).shape[1:])
        return a[1:-1, 1:-1]


def _field_values(spec, st, vector):
    kind = spec["type"]
    X, Y = np.meshgrid(np.arange(st.Nx), np.arange(st.Ny), indexing="ij")
    if kind == "fixed":
        v = spec["value"]
        return np.broadcast_to(np.asarray(v, dtype=np.float64),
                               (st.Nx, st.Ny, 2) if vector else (st.Nx, st.Ny))
    if kind == "func":
        f = spec["func"]
        out = np.zeros((st.Nx, st.Ny, 2) if vector else (st.Nx, st.Ny))
        for x in range(st.Nx):
            for y in range(st.Ny):
                out[x, y] = f(x, y)
        return out
    if kind == "array":
        return np.asarray(spec["value"], dtype=np.float64)
    raise ValueError("Unsupported velocity initialization")


def build_state(sim, periodic_mode="wrap"):
    """``sim``: mapping with the reference's case dictionaries."""
    nx, ny = sim["mesh_dict"]["grid"]
    st = RefState(nx, ny)
    st.periodic_mode = periodic_mode
    # transport + collision -- collision_operator.py:89-91
    kin_visc = np.float64(sim["transport_dict"]["kin_visc"])
    tau = kin_visc * INV_CS_2 + 0.5
    st.omega = 1 / tau
    fl = sim["collision_dict"]["fluid"]
    st.collision = fl["model"]
    st.forcing = fl["forcing_model"]
    if st.collision == "MRT":
        r = fl.get("mrt_rates", {})
        st.mrt_rates = (float(r.get("s_e", 1.0)), float(r.get("s_eps", 1.0)),
                        float(r.get("s_q", 1.0)), float(r.get("s_nu", st.omega)))
    fd = sim.get("forcing_dict", {})
    if st.forcing is not None and "gravity" in fd:
        st.gravity = np.array(fd["gravity"], dtype=np.float64)
    if st.forcing is not None and "body_force_field" in fd:
        bf = np.asarray(fd["body_force_field"], dtype=np.float64)
        st.body_force = np.zeros((st.size, 2))
        st.inner(st.body_force)[...] = bf
    # initial fields (default, then overrides in dict order) -- init_fields.py:7-129
    ifd = sim["initial_fields_dict"]
    order = ["default"] + [k for k in ifd if k != "default"]
    for key in order:
        fdict = ifd[key].get("fluid", {})
        if "velocity" in fdict:
            st.inner(st.velocity)[...] = _field_values(fdict["velocity"], st, True)
        if "density" in fdict:
            st.inner(st.density)[...] = _field_values(fdict["density"], st, False)
    # boundaries -- boundary.py:283-519
    for name, bd in sim["boundary_dict"].items():
        if name == "options":
            continue
        bc_type = bd["fluid"]["type"]
        value = bd["fluid"].get("value")
        if bc_type == "periodic":
            (a, b) = bd["segments"][0]
            if a[0] == b[0]:
                st.x_periodic = True
            else:
                st.y_periodic = True
        for seg_no, seg in enumerate(bd["segments"]):
            (x1, y1), (x2, y2) = seg
            if x2 - x1 == 0:
                loc = "right" if x2 == nx - 1 else ("left" if x2 == 0 else None)
                xs = np.full(y2 - y1 + 1, x1)
                ys = np.arange(y1, y2 + 1)
            else:
                loc = "top" if y2 == ny - 1 else ("bottom" if y2 == 0 else None)
                xs = np.arange(x1, x2 + 1)
                ys = np.full(x2 - x1 + 1, y1)
            if loc is None:
                raise ValueError("segment is not on the domain edge: " + name)
            nodes = st.padded_index(xs, ys)
            st.elements.append(Element(f"{name}_{seg_no}", bc_type, loc, nodes, value))
    # obstacles -- obstacle.py:392-825, obstacle_kernels.py:43-93,151-241
    for name, od in sim.get("obstacle_dict", {}).items():
        if name == "options":
            continue
        if od["type"] not in ("circle", "ellipse"):
            raise ValueError("oracle restates circle and ellipse obstacles only")
        cx, cy = (np.float64(c) for c in od["center"])
        lin = np.zeros(2)
        ang = np.float64(0)
        if not od["static"]:
            sm = od["solid_motion_dict"]
            lin = np.array(sm["linear_velocity"], dtype=np.float64)
            ang = np.float64(sm["angular_velocity"])
        ind = np.nonzero(~st.ghost)[0]
        xg, yg = ind // st.nyp - 1, ind % st.nyp - 1
        rx, ry = xg - cx, yg - cy
        rxm, rym = rx.copy(), ry.copy()
        if st.x_periodic:
            rxm = np.where(np.abs(rx + nx) < np.abs(rxm), rx + nx, rxm)
            rxm = np.where(np.abs(rx - nx) < np.abs(rxm), rx - nx, rxm)
        if st.y_periodic:
            rym = np.where(np.abs(ry + ny) < np.abs(rym), ry + ny, rym)
            rym = np.where(np.abs(ry - ny) < np.abs(rym), ry - ny, rym)
        if od["type"] == "circle":
            r = np.float64(od["radius"])
            inside = rxm * rxm + rym * rym <= r * r
        else:
            # is_ellipse -- obstacle_kernels.py:151-189, angle in degrees
            # (obstacle.py:666-676)
            a = np.float64(od["semi_major_axis"])
            b = np.float64(od["semi_minor_axis"])
            alpha = np.float64(od["inclination_angle"]) * np.pi / 180
            ca, sa = np.cos(alpha), np.sin(alpha)
            xp = rxm * ca + rym * sa
            yp = -rxm * sa + rym * ca
            inside = (xp * xp) / (a * a) + (yp * yp) / (b * b) <= 1
        hit = ind[inside]
        st.solid[hit] = True
        st.velocity[hit, 0] = lin[0] - ang * rym[inside]
        st.velocity[hit, 1] = lin[1] + ang * rxm[inside]
        st.density[hit] = np.float64(od["density"])
    return st
