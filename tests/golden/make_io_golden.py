"""Generate the output-format fixture from the reference's own I/O code.

Run where a checkout of the reference is available:

    python tests/golden/make_io_golden.py --ref <path of the reference checkout>

It builds the reference State of the ``channel_cylinder_abb`` golden case with
output options switched on (std_out / save / history intervals of 30 steps,
compute_force and compute_force_torque), runs the reference's
ObstacleOperator set-up and InputOutputOperator (pylabolt/utils/io_operator.py)
in a scratch directory, and feeds it the golden density / velocity and the
reference-kernel forces of t = 0, 30 and 60 from ``channel_cylinder_abb.npz``.
The residues of t = 30 and 60 are what the reference's ResidueOperator
computes with a std_out interval of 30 (compute_residue_scalar/vector against
the fields of the previous residue step, zeros at first;
pylabolt/utils/residues.py:171-222), formatted by SimulationStatusLogger
(pylabolt/utils/helpers.py:37-56).

The stand-ins of make_golden.py are used (numba, mpi4py); the package
version that ``dump_metadata`` reads with importlib.metadata is fixed to
VERSION because the reference is not pip-installed here.

Written: ``tests/golden/io_channel_cylinder.npz`` with the case (JSON), the
text of metadata.json and of every history file, the status lines, and the
arrays and key order of every t_<n>.npz.
"""
import argparse
import contextlib
import importlib.metadata
import io
import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg   # noqa: E402

VERSION = "0.0.0+golden"
TIMES = (0, 30, 60)


def io_case():
    case, nsteps, _ = mg.make_cases()["channel_cylinder_abb"]
    case["control_dict"].update({"std_out_interval": 30, "save_interval": 30,
                                 "end_time": 60})
    case["boundary_dict"]["options"] = {"compute_force": True,
                                        "write_boundary_data": {"interval": 30}}
    case["obstacle_dict"]["options"] = {"compute_force_torque": True,
                                        "write_obstacle_data": {"interval": 30}}
    return case


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="path of the reference checkout")
    args = ap.parse_args()
    mg.install_numba_stub()
    mg.install_mpi4py_stub()
    sys.path.insert(0, args.ref)
    importlib.metadata.version = lambda name: VERSION
    from pylabolt.base.state import State
    from pylabolt.parallel.MPI_operator import MPIOperator
    from pylabolt.base.obstacle_operator import ObstacleOperator
    from pylabolt.utils.io_operator import InputOutputOperator
    from pylabolt.utils.helpers import SimulationStatusLogger
    from pylabolt.solvers.fluidLB import FluidLB
    import pylabolt.parallel.cpu.io_operator_kernels as iok
    import pylabolt.parallel.cpu.compute_residues_kernels as crk

    gold = np.load(os.path.join(HERE, "channel_cylinder_abb.npz"))
    case = io_case()
    out = {"case_json": np.array(mg.jsonable(case)), "version": np.array(VERSION)}
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            with contextlib.redirect_stdout(io.StringIO()):
                st = State(mg.to_module(case), mg.DummyComm(), 0, fluid=True)
                ObstacleOperator(None, st, None, MPIOperator(mg.DummyComm(), st), None)
                st.obstacle.set_backend(types.SimpleNamespace(backend_type="cpu"))
                iop = InputOutputOperator(FluidLB(), st, None, mg.DummyComm())
            iop.copy_inner_data_kernel_scalar = iok.copy_inner_data_scalar
            iop.copy_inner_data_kernel_vector = iok.copy_inner_data_vector
            walls = [el for el in st.boundary.boundary_elements if el.wall]
            lines = []
            residues = []
            logger = SimulationStatusLogger(0)
            dens_old = np.zeros_like(st.fields.density)
            vel_old = np.zeros_like(st.fields.velocity)
            eps = st.control.float_min
            for t in TIMES:
                if t == 0:
                    st.fields.density[:] = gold["rho0"]
                    st.fields.velocity[:] = gold["u0"]
                else:
                    st.fields.density[:] = gold[f"density_t{t}"]
                    st.fields.velocity[:] = gold[f"velocity_t{t}"]
                fo = gold[f"force_obstacles_t{t}"]
                st.obstacle.obstacle_data.force[:, :] = fo[:, :2]
                st.obstacle.obstacle_data.torque[:, 0] = fo[:, 2]
                for el, fw in zip(walls, gold[f"force_walls_t{t}"]):
                    el.force[:] = fw
                iop.write_fields_cpu(st, None, t)
                iop.write_histories_cpu(st, t)
                if t > 0:
                    fl = st.fields
                    a = crk.compute_residue_scalar(st.domain.size, fl.solid, fl.ghost_node,
                                                   fl.density, dens_old)
                    b = crk.compute_residue_vector(st.domain.size, fl.solid, fl.ghost_node,
                                                   fl.velocity, vel_old)
                    r = [np.sqrt(a[0] / (a[1] + eps)), np.sqrt(b[0] / (b[1] + eps)),
                         np.sqrt(b[2] / (b[3] + eps))]
                    residues.append([t] + r)
                    buf = io.StringIO()
                    with contextlib.redirect_stdout(buf):
                        logger.log_data(st, t, res_density=np.array(r[:1]),
                                        res_velocity=np.array(r[1:]))
                    lines.append(buf.getvalue().rstrip("\n"))
            out["status_lines"] = np.array(lines)
            out["residues"] = np.array(residues)
            with open("metadata.json") as f:
                out["metadata_json"] = np.array(f.read())
            hist = sorted(os.listdir("output/histories"))
            out["history_names"] = np.array(hist)
            for h in hist:
                with open(os.path.join("output/histories", h)) as f:
                    out[f"history:{h}"] = np.array(f.read())
            for t in TIMES:
                z = np.load(f"output/fields/t_{t}.npz")
                out[f"fields_t{t}_keys"] = np.array(list(z.files))
                for k in z.files:
                    out[f"fields_t{t}:{k}"] = z[k]
        finally:
            os.chdir(cwd)
    np.savez_compressed(os.path.join(HERE, "io_channel_cylinder.npz"), **out)
    print("io_channel_cylinder: metadata, %d history files, %d field files"
          % (len(out["history_names"]), len(TIMES)))


if __name__ == "__main__":
    main()
