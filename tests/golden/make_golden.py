"""Generate the golden fixtures for the fluidLB step from the reference itself.

Run where a checkout of the reference is available:

    python tests/golden/make_golden.py --ref <path of the reference checkout>

The reference needs ``numba``, which is not installed here, so a stand-in
``numba`` module is placed in ``sys.modules`` first: ``njit`` returns the
function unchanged, ``prange`` is ``range`` and ``cuda.jit`` returns the
function unchanged (``cuda.grid`` reads a thread index that this script sets).
With it the reference's own modules run as plain FP64 Python:

* the case State (control, mesh, lattice, domain, fields, init_fields,
  boundary, obstacle) is built by ``pylabolt.base.state.State``;
* every step replays ``Solver.single_time_step``
  (pylabolt/solvers/fluidLB.py:206-253) with the reference CPU kernels:
  density, gravity force, velocity, BGK collision, the GPU periodic wrap
  kernels of pylabolt/parallel/gpu/MPI_kernels.py:51-99 (looped over thread
  indices), ``scalar_based_kernel`` and the boundary kernels in element order;
* residues come from ``compute_residue_scalar/vector``;
* the obstacle geometry fields (solid_id, solid_boundary, fluid_boundary,
  surface_normals) come from the reference's own ``ObstacleOperator``
  (pylabolt/base/obstacle_operator.py:19-45, with its single-rank
  ``halo_exchange_cpu``), built on a second State so that the stepping above
  keeps ghost nodes non-solid;
* momentum-exchange forces at t = 0 and at every checkpoint come from
  ``compute_force_torque_single_phase`` (every obstacle) and
  ``compute_boundary_force_single_phase`` (every wall element),
  pylabolt/parallel/cpu/force_torque_kernels.py:11-141, applied to the
  checkpointed pop / pop_new.

Deviations, each forced by a defect of the reference snapshot:
* ``move_obstacles`` is skipped (it calls the undefined
  ``reconstruct_obstacles``, pylabolt/base/obstacle_operator.py:67); obstacles
  here are rasterised once and never moved, so the call would be a no-op.
* ``fixed_pressure_density_based`` receives the surface normal as an int array
  (the reference passes the float normal of boundary.py:63-78, which fails to
  index).

Zero-gradient cases.  The reference has no ``zero_gradient`` kernel, but its
single-rank CPU halo exchange (``MPIOperator.halo_exchange_cpu``,
pylabolt/parallel/MPI_operator.py:155-314, with a one-rank communicator)
copies the first inner column / row of the post-collision populations into
the ghost column / row of a "periodic" edge instead of wrapping.  The pull
stream then gives an edge node b, for every population i entering from
outside, ``pop[b + n - c_i, i]``: exactly this package's ``zero_gradient``
definition.  The ``zero_gradient_*`` cases are therefore run by the
reference with ``periodic`` edges and the CPU self-copy halo, and stored with
the same dictionaries in which those edges are ``zero_gradient`` (listed
before the walls, so that the walls win at the corners as the wall kernels do
after streaming in the reference).  ``ref_case_json`` holds the dictionaries
the reference ran.

Each case is written to ``tests/golden/<name>.npz`` with the case
dictionaries (JSON), the initial padded fields the reference built, the
solid flags, checkpoints of density / velocity / pop / pop_new and the
per-step residual history.
"""
import argparse
import contextlib
import io
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


# --------------------------------------------------------------------------
# stand-in numba
_THREAD = [0]


def _identity_decorator(*args, **kwargs):
    if args and callable(args[0]) and len(args) == 1 and not kwargs:
        return args[0]
    return lambda f: f


def install_numba_stub():
    numba = types.ModuleType("numba")
    numba.njit = _identity_decorator
    numba.jit = _identity_decorator
    numba.prange = range
    cuda = types.ModuleType("numba.cuda")
    cuda.jit = _identity_decorator
    cuda.grid = lambda ndim: _THREAD[0]
    cuda.device_array = np.zeros
    cuda.device_array_like = np.zeros_like
    numba.cuda = cuda
    # type names imported by the GPU kernel modules (``from numba import int64``)
    numba.__getattr__ = lambda name: getattr(np, name) if hasattr(np, name) else object()
    cuda.__getattr__ = lambda name: object()
    sys.modules["numba"] = numba
    sys.modules["numba.cuda"] = cuda


def install_mpi4py_stub():
    """``mpi4py`` is not installed; the reference's MPIOperator imports it."""
    mpi4py = types.ModuleType("mpi4py")
    mpi = types.ModuleType("mpi4py.MPI")
    mpi.SUM = "sum"
    mpi4py.MPI = mpi
    sys.modules["mpi4py"] = mpi4py
    sys.modules["mpi4py.MPI"] = mpi


class DummyComm:
    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def Sendrecv(self, sendbuf, dest, sendtag, recvbuf, source, recvtag):
        recvbuf[...] = sendbuf          # one rank: it exchanges with itself

    def Allreduce(self, a, b, op=None):
        b[...] = a

    def Barrier(self):
        pass

    def Abort(self, *a):
        raise RuntimeError("reference State construction aborted")


# --------------------------------------------------------------------------
# cases
def base_case(nx, ny, kin_visc, model="BGK", forcing=None, gravity=None):
    case = {
        "control_dict": {"start_time": 0, "end_time": 0, "std_out_interval": 1,
                         "save_interval": None, "checkpoint_interval": None,
                         "precision": "double"},
        "mesh_dict": {"grid": [nx, ny]},
        "lattice_dict": {"lattice_type": "D2Q9"},
        "decompose_dict": {"nx": 1, "ny": 1},
        "transport_dict": {"kin_visc": kin_visc},
        "initial_fields_dict": {"default": {"fluid": {
            "velocity": {"type": "fixed", "value": [0.0, 0.0]},
            "density": {"type": "fixed", "value": 1.0},
            "pressure": {"type": "fixed", "value": 0.0}}}},
        "boundary_dict": {"options": {}},
        "obstacle_dict": {"options": {}},
        "collision_dict": {"fluid": {"model": model,
                                     "equilibrium": "density_based_second_order",
                                     "forcing_model": forcing}},
        "forcing_dict": {} if gravity is None else {"gravity": list(gravity)},
    }
    return case


def walls(nx, ny, order=("left", "right", "bottom", "top"), top=None, kinds=None):
    segs = {"left": [[0, 0], [0, ny - 1]], "right": [[nx - 1, 0], [nx - 1, ny - 1]],
            "bottom": [[0, 0], [nx - 1, 0]], "top": [[0, ny - 1], [nx - 1, ny - 1]]}
    out = {}
    for side in order:
        kind = (kinds or {}).get(side, {"type": "bounce_back"})
        out[side] = {"wall": True, "segments": [segs[side]], "fluid": dict(kind)}
    return out


def make_cases():
    rng = np.random.default_rng(12345)
    cases = {}

    # lid-driven cavity (C1 shape, reduced): walls first, lid last
    c = base_case(12, 10, 0.128)
    c["boundary_dict"].update(walls(12, 10, order=("left", "right", "bottom", "top"),
                                    kinds={"top": {"type": "fixed_velocity",
                                                   "value": [0.1, 0.0]}}))
    cases["cavity_lid_last"] = (c, 80, None)

    # same cavity, lid first: the side walls win at the two top corners
    c = base_case(12, 10, 0.128)
    c["boundary_dict"].update(walls(12, 10, order=("top", "left", "right", "bottom"),
                                    kinds={"top": {"type": "fixed_velocity",
                                                   "value": [0.1, 0.0]}}))
    cases["cavity_lid_first"] = (c, 60, None)

    # gravity-driven Poiseuille: periodic x, bounce-back y, Guo second order
    c = base_case(10, 8, 0.256, forcing="guo_second_order", gravity=[2e-5, 0.0])
    c["boundary_dict"]["inout"] = {"wall": False, "segments": [
        [[0, 0], [0, 7]], [[9, 0], [9, 7]]], "fluid": {"type": "periodic"}}
    c["boundary_dict"]["walls"] = {"wall": True, "segments": [
        [[0, 0], [9, 0]], [[0, 7], [9, 7]]], "fluid": {"type": "bounce_back"}}
    cases["poiseuille_guo2"] = (c, 80, None)

    # pressure-driven channel with a cylinder, Guo linear, random start
    nx, ny = 16, 11
    c = base_case(nx, ny, 0.05, forcing="guo_linear", gravity=[1e-5, 0.0])
    c["boundary_dict"]["inlet"] = {"wall": False, "segments": [[[0, 0], [0, ny - 1]]],
                                   "fluid": {"type": "fixed_pressure", "value": 1.0005}}
    c["boundary_dict"]["outlet"] = {"wall": False,
                                    "segments": [[[nx - 1, 0], [nx - 1, ny - 1]]],
                                    "fluid": {"type": "fixed_pressure", "value": 1.0}}
    c["boundary_dict"]["walls"] = {"wall": True, "segments": [
        [[0, 0], [nx - 1, 0]], [[0, ny - 1], [nx - 1, ny - 1]]],
        "fluid": {"type": "bounce_back"}}
    c["obstacle_dict"]["cyl"] = {"type": "circle", "radius": 2.0, "center": [5, 5],
                                 "density": 1.0, "static": True}
    pert = rng.uniform(-1e-4, 1e-4, (nx, ny, 2))
    c["initial_fields_dict"]["default"]["fluid"]["velocity"] = {"type": "array",
                                                                "value": pert}
    cases["channel_cylinder_abb"] = (c, 60, None)

    # doubly periodic box with a moving (non-static) circle, Guo 2nd order
    nx, ny = 14, 12
    c = base_case(nx, ny, 0.08, forcing="guo_second_order", gravity=[1e-5, -2e-6])
    c["boundary_dict"]["xper"] = {"wall": False, "segments": [
        [[0, 0], [0, ny - 1]], [[nx - 1, 0], [nx - 1, ny - 1]]],
        "fluid": {"type": "periodic"}}
    c["boundary_dict"]["yper"] = {"wall": False, "segments": [
        [[0, 0], [nx - 1, 0]], [[0, ny - 1], [nx - 1, ny - 1]]],
        "fluid": {"type": "periodic"}}
    c["obstacle_dict"]["options"] = {"compute_force_torque": True}
    c["obstacle_dict"]["disk"] = {
        "type": "circle", "radius": 2.5, "center": [12.5, 1.0], "density": 2.0,
        "static": False, "solid_motion_dict": {
            "type": "fixed_velocity", "degree_of_freedom": "both",
            "linear_velocity": [0.01, 0.005], "angular_velocity": 0.002}}
    pert = rng.uniform(-1e-3, 1e-3, (nx, ny, 2))
    c["initial_fields_dict"]["default"]["fluid"]["velocity"] = {"type": "array",
                                                                "value": pert}
    cases["periodic_moving_disk"] = (c, 60, None)

    # y-periodic, partial and mixed segments on the x edges, random density
    nx, ny = 12, 9
    c = base_case(nx, ny, 0.1)
    c["boundary_dict"]["yper"] = {"wall": False, "segments": [
        [[0, 0], [nx - 1, 0]], [[0, ny - 1], [nx - 1, ny - 1]]],
        "fluid": {"type": "periodic"}}
    c["boundary_dict"]["left_lid"] = {"wall": True, "segments": [[[0, 2], [0, 6]]],
                                      "fluid": {"type": "fixed_velocity",
                                                "value": [0.0, 0.05]}}
    c["boundary_dict"]["right_low"] = {"wall": True, "segments": [[[nx - 1, 0], [nx - 1, 4]]],
                                       "fluid": {"type": "bounce_back"}}
    c["boundary_dict"]["right_high"] = {"wall": False,
                                        "segments": [[[nx - 1, 5], [nx - 1, ny - 1]]],
                                        "fluid": {"type": "fixed_pressure", "value": 1.001}}
    dens = 1.0 + rng.uniform(-1e-3, 1e-3, (nx, ny))
    c["initial_fields_dict"]["default"]["fluid"]["density"] = {"type": "array",
                                                               "value": dens}
    cases["yperiodic_partial_edges"] = (c, 40, None)

    # zero-gradient x edges (reference: periodic x with the CPU self-copy
    # halo), bottom bounce-back, moving lid, cylinder, Guo linear, random start
    nx, ny = 18, 10
    c = base_case(nx, ny, 0.06, forcing="guo_linear", gravity=[1e-5, 0.0])
    c["boundary_dict"]["ends"] = {"wall": False, "segments": [
        [[0, 0], [0, ny - 1]], [[nx - 1, 0], [nx - 1, ny - 1]]],
        "fluid": {"type": "periodic"}}
    c["boundary_dict"]["bottom"] = {"wall": True, "segments": [[[0, 0], [nx - 1, 0]]],
                                    "fluid": {"type": "bounce_back"}}
    c["boundary_dict"]["lid"] = {"wall": True, "segments": [[[0, ny - 1], [nx - 1, ny - 1]]],
                                 "fluid": {"type": "fixed_velocity", "value": [0.02, 0.0]}}
    c["obstacle_dict"]["cyl"] = {"type": "circle", "radius": 2.0, "center": [8, 5],
                                 "density": 1.0, "static": True}
    pert = rng.uniform(-1e-3, 1e-3, (nx, ny, 2))
    c["initial_fields_dict"]["default"]["fluid"]["velocity"] = {"type": "array",
                                                                "value": pert}
    cases["zero_gradient_x"] = (c, 60, "selfcopy")

    # zero-gradient y edges next to a bounce-back wall (left) and a moving wall
    # (right), Guo second order along y, random density
    nx, ny = 10, 16
    c = base_case(nx, ny, 0.09, forcing="guo_second_order", gravity=[0.0, 1e-5])
    c["boundary_dict"]["ends"] = {"wall": False, "segments": [
        [[0, 0], [nx - 1, 0]], [[0, ny - 1], [nx - 1, ny - 1]]],
        "fluid": {"type": "periodic"}}
    c["boundary_dict"]["left"] = {"wall": True, "segments": [[[0, 0], [0, ny - 1]]],
                                  "fluid": {"type": "bounce_back"}}
    c["boundary_dict"]["right"] = {"wall": True, "segments": [[[nx - 1, 0], [nx - 1, ny - 1]]],
                                   "fluid": {"type": "fixed_velocity", "value": [0.0, 0.03]}}
    dens = 1.0 + rng.uniform(-1e-3, 1e-3, (nx, ny))
    c["initial_fields_dict"]["default"]["fluid"]["density"] = {"type": "array",
                                                               "value": dens}
    cases["zero_gradient_y"] = (c, 60, "selfcopy")

    # channel with two inclined ellipses (one static, one non-static held in
    # place, i.e. a moving wall), pressure inlet / outlet, Guo second order
    nx, ny = 26, 14
    c = base_case(nx, ny, 0.07, forcing="guo_second_order", gravity=[5e-6, 1e-6])
    c["boundary_dict"]["inlet"] = {"wall": False, "segments": [[[0, 0], [0, ny - 1]]],
                                   "fluid": {"type": "fixed_pressure", "value": 1.0004}}
    c["boundary_dict"]["outlet"] = {"wall": False,
                                    "segments": [[[nx - 1, 0], [nx - 1, ny - 1]]],
                                    "fluid": {"type": "fixed_pressure", "value": 1.0}}
    c["boundary_dict"]["walls"] = {"wall": True, "segments": [
        [[0, 0], [nx - 1, 0]], [[0, ny - 1], [nx - 1, ny - 1]]],
        "fluid": {"type": "bounce_back"}}
    c["obstacle_dict"]["options"] = {"compute_force_torque": True}
    c["obstacle_dict"]["wing"] = {"type": "ellipse", "semi_major_axis": 3.5,
                                  "semi_minor_axis": 1.5, "inclination_angle": 30.0,
                                  "center": [7, 6.5], "density": 1.0, "static": True}
    c["obstacle_dict"]["rotor"] = {
        "type": "ellipse", "semi_major_axis": 2.6, "semi_minor_axis": 1.7,
        "inclination_angle": -50, "center": [17.5, 7], "density": 1.5, "static": False,
        "solid_motion_dict": {"type": "fixed_velocity", "degree_of_freedom": "rotation",
                              "linear_velocity": [0.0, 0.0], "angular_velocity": 0.004}}
    pert = rng.uniform(-1e-4, 1e-4, (nx, ny, 2))
    c["initial_fields_dict"]["default"]["fluid"]["velocity"] = {"type": "array",
                                                                "value": pert}
    cases["channel_ellipses"] = (c, 60, None)
    return cases


def zero_gradient_twin(case):
    """The same dictionaries with every ``periodic`` edge ``zero_gradient``."""
    out = json.loads(jsonable(case))
    for region, rd in case["initial_fields_dict"].items():
        for fname, spec in rd["fluid"].items():
            if spec["type"] == "array":
                out["initial_fields_dict"][region]["fluid"][fname]["value"] = spec["value"]
    for name, ud in out["boundary_dict"].items():
        if name != "options" and ud["fluid"]["type"] == "periodic":
            ud["fluid"] = {"type": "zero_gradient"}
    return out


# --------------------------------------------------------------------------
def to_module(case):
    """Reference-facing ``simulation`` module; ``array`` fields become funcs."""
    mod = types.ModuleType("simulation")
    for key, val in case.items():
        setattr(mod, key, val)
    ifd = {}
    for region, rd in case["initial_fields_dict"].items():
        fl = {}
        for fname, spec in rd["fluid"].items():
            if spec["type"] == "array":
                arr = np.asarray(spec["value"])
                if arr.ndim == 3:
                    fl[fname] = {"type": "func",
                                 "func": (lambda a: lambda i, j: (float(a[i, j, 0]),
                                                                  float(a[i, j, 1])))(arr)}
                else:
                    fl[fname] = {"type": "func",
                                 "func": (lambda a: lambda i, j: float(a[i, j]))(arr)}
            else:
                fl[fname] = spec
        ifd[region] = {"fluid": fl}
    mod.initial_fields_dict = ifd
    return mod


def jsonable(case):
    def conv(o):
        if isinstance(o, dict):
            return {k: conv(v) for k, v in o.items()}
        if isinstance(o, (list, tuple)):
            return [conv(v) for v in o]
        if isinstance(o, np.ndarray):
            return "__array__"
        return o
    return json.dumps(conv(case))


def run_case(name, case, nsteps, ref, halo=None):
    """Steps `case` with the reference's kernels.  halo None: the GPU periodic
    wrap kernels; "selfcopy": the single-rank CPU halo exchange (the stored
    case is then the zero_gradient twin)."""
    from pylabolt.base.state import State
    from pylabolt.parallel.MPI_operator import MPIOperator
    import pylabolt.parallel.cpu.compute_fields_kernels as cfk
    import pylabolt.parallel.cpu.force_field_kernels as ffk
    import pylabolt.parallel.cpu.collision_kernels as colk
    import pylabolt.parallel.cpu.equilibrium_kernels as eqk
    import pylabolt.parallel.cpu.streaming_kernels as stk
    import pylabolt.parallel.cpu.fluid_boundary_kernels as fbk
    import pylabolt.parallel.cpu.compute_residues_kernels as crk
    import pylabolt.parallel.gpu.MPI_kernels as gmk

    sim = to_module(case)
    with contextlib.redirect_stdout(io.StringIO()):
        state = State(sim, DummyComm(), 0, fluid=True)
    lat, fld, dom, ctl = state.lattice, state.fields, state.domain, state.control
    mpi_op = MPIOperator(DummyComm(), state) if halo == "selfcopy" else None
    tau = state.transport.kin_visc * lat.inv_cs_2 + 0.5   # collision_operator.py:89
    omega = 1 / tau
    forcing = case["collision_dict"]["fluid"]["forcing_model"]
    gravity = np.zeros(2)
    if forcing is not None and "gravity" in case["forcing_dict"]:
        gravity = np.array(case["forcing_dict"]["gravity"], dtype=np.float64)
    collide = getattr(colk, "BGK_density_based_second_order_" + str(forcing))
    size, shape = dom.size, dom.shape

    rho0 = fld.density.copy()
    u0 = fld.velocity.copy()
    solid0 = fld.solid.copy()

    eqk.initialize_pop_density_based_second_order(
        size, lat.cx, lat.cy, lat.weights, lat.no_of_directions, lat.inv_cs_2,
        lat.inv_cs_4, fld.solid, fld.ghost_node, fld.density, fld.velocity,
        fld.pop_fluid, fld.pop_fluid_new)
    pop_init = fld.pop_fluid.copy()
    pop_new_init = fld.pop_fluid_new.copy()

    dens_old = np.zeros_like(fld.density)
    vel_old = np.zeros_like(fld.velocity)
    checkpoints = sorted({1, 2, nsteps // 2, nsteps})
    out = {}
    resid = []
    for t in range(1, nsteps + 1):
        cfk.density_compute_density_based(size, lat.no_of_directions, fld.solid,
                                          fld.ghost_node, fld.density, fld.pop_fluid_new)
        ffk.compute_gravity_force(size, fld.solid, fld.ghost_node, fld.density,
                                  fld.force_field, gravity)
        cfk.velocity_compute_density_based(ctl.float_min, size, lat.cx, lat.cy,
                                           lat.no_of_directions, fld.solid,
                                           fld.ghost_node, fld.density, fld.velocity,
                                           fld.force_field, fld.pop_fluid_new)
        collide(size, lat.cx, lat.cy, lat.weights, lat.no_of_directions, lat.inv_cs_2,
                lat.inv_cs_4, fld.solid, fld.ghost_node, fld.density, fld.velocity,
                fld.force_field, fld.pop_fluid, fld.pop_fluid_new, omega)
        if mpi_op is not None:
            # fluidLB.py:227-231 on the CPU backend: MPI_operator.py:155-259
            mpi_op.halo_exchange_cpu(state, None, float_buffers=["pop_fluid"])
        elif state.boundary.x_periodic:
            for tid in range(shape[1]):
                _THREAD[0] = tid
                gmk.exchange_y_vector(fld.pop_fluid, shape)
        if mpi_op is None and state.boundary.y_periodic:
            for tid in range(shape[0]):
                _THREAD[0] = tid
                gmk.exchange_x_vector(fld.pop_fluid, shape)
        stk.scalar_based_kernel(size, shape, lat.cx, lat.cy, lat.weights, lat.inv_list,
                                lat.no_of_directions, lat.inv_cs_2, fld.solid,
                                fld.ghost_node, fld.density, fld.velocity,
                                fld.pop_fluid, fld.pop_fluid_new)
        for el in state.boundary.boundary_elements:
            kind = el.type_fluid
            if kind == "periodic":
                continue
            if kind == "bounce_back":
                fbk.bounce_back(fld.solid, fld.pop_fluid, fld.pop_fluid_new,
                                el.boundary_nodes, el.out_list, el.inv_list)
            elif kind == "fixed_velocity":
                fbk.fixed_velocity_density_based(
                    lat.cx, lat.cy, lat.weights, lat.inv_cs_2, fld.solid, fld.density,
                    fld.pop_fluid, fld.pop_fluid_new, el.boundary_nodes, el.out_list,
                    el.inv_list, el.vector_fluid)
            elif kind == "fixed_pressure":
                fbk.fixed_pressure_density_based(
                    shape, lat.cx, lat.cy, lat.weights, lat.inv_cs_2, lat.inv_cs_4,
                    fld.solid, fld.velocity, fld.pop_fluid, fld.pop_fluid_new,
                    el.boundary_nodes, el.out_list, el.inv_list, el.scalar_fluid,
                    el.surface_normals.astype(np.int64))
            else:
                raise ValueError(kind)
        r = crk.compute_residue_scalar(size, fld.solid, fld.ghost_node, fld.density,
                                       dens_old)
        v = crk.compute_residue_vector(size, fld.solid, fld.ghost_node, fld.velocity,
                                       vel_old)
        eps = ctl.float_min
        resid.append([t, np.sqrt(r[0] / (r[1] + eps)), np.sqrt(v[0] / (v[1] + eps)),
                      np.sqrt(v[2] / (v[3] + eps))])
        if t in checkpoints:
            out[f"density_t{t}"] = fld.density.copy()
            out[f"velocity_t{t}"] = fld.velocity.copy()
            out[f"pop_t{t}"] = fld.pop_fluid.copy()
            out[f"pop_new_t{t}"] = fld.pop_fluid_new.copy()

    stored = case if halo is None else zero_gradient_twin(case)
    extra = {} if halo is None else {"ref_case_json": np.array(jsonable(case)),
                                     "halo": np.array(halo)}
    geo = geometry_and_forces(case, {0: (pop_init, pop_new_init),
                                     **{t: (out[f"pop_t{t}"], out[f"pop_new_t{t}"])
                                        for t in checkpoints}})
    arrays = {}
    for region, rd in case["initial_fields_dict"].items():
        for fname, spec in rd["fluid"].items():
            if spec["type"] == "array":
                arrays[f"init_{region}_{fname}"] = np.asarray(spec["value"])
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        case_json=np.array(jsonable(stored)), nsteps=np.array(nsteps), **extra,
        checkpoints=np.array(checkpoints), rho0=rho0, u0=u0, solid=solid0,
        residuals=np.array(resid), inv_cs_2=np.array(lat.inv_cs_2),
        inv_cs_4=np.array(lat.inv_cs_4), omega=np.array(omega), **arrays, **out, **geo)
    return len(resid)


def geometry_and_forces(case, states):
    """Obstacle geometry fields from the reference's ObstacleOperator and
    momentum-exchange forces of `states` {t: (pop, pop_new)}."""
    from pylabolt.base.state import State
    from pylabolt.parallel.MPI_operator import MPIOperator
    from pylabolt.base.obstacle_operator import ObstacleOperator
    import pylabolt.parallel.cpu.force_torque_kernels as ftk

    with contextlib.redirect_stdout(io.StringIO()):
        st = State(to_module(case), DummyComm(), 0, fluid=True)
        ObstacleOperator(None, st, None, MPIOperator(DummyComm(), st), None)
    lat, fld, dom = st.lattice, st.fields, st.domain
    out = {"geo_solid": fld.solid.copy(), "geo_solid_id": fld.solid_id.copy(),
           "geo_solid_boundary": fld.solid_boundary.copy(),
           "geo_fluid_boundary": fld.fluid_boundary.copy(),
           "geo_surface_normals": fld.surface_normals.copy()}
    walls = [el for el in st.boundary.boundary_elements if el.wall]
    out["wall_names"] = np.array([el.name for el in walls])
    out["obstacle_names"] = np.array([o.name for o in st.obstacle.obstacles])
    for t, (pop, pop_new) in states.items():
        obs = [ftk.compute_force_torque_single_phase(
            dom.size, dom.shape, dom.offset, st.mesh.grid_global_shape, lat.cx, lat.cy,
            lat.inv_list, lat.no_of_directions, st.boundary.x_periodic, st.boundary.y_periodic,
            fld.solid, fld.solid_id, fld.fluid_boundary, fld.ghost_node, pop, pop_new,
            o.ref_point, o.id) for o in st.obstacle.obstacles]
        wall = [ftk.compute_boundary_force_single_phase(
            lat.cx, lat.cy, fld.solid, pop, pop_new, el.boundary_nodes, el.out_list,
            el.inv_list) for el in walls]
        out[f"force_obstacles_t{t}"] = np.array(obs).reshape(-1, 3)
        out[f"force_walls_t{t}"] = np.array(wall).reshape(-1, 2)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="path of the reference checkout")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    install_numba_stub()
    install_mpi4py_stub()
    sys.path.insert(0, args.ref)
    for name, (case, nsteps, halo) in make_cases().items():
        if args.only and name != args.only:
            continue
        n = run_case(name, case, nsteps, args.ref, halo)
        print(f"{name}: {n} steps written")


if __name__ == "__main__":
    main()
