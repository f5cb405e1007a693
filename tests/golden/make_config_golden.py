"""Generate the case-validation fixture from the reference's own classes.

Run where a checkout of the reference is available:

    python tests/golden/make_config_golden.py --ref <path of the reference checkout>

Each entry applies one mutation (a list of set / delete operations on a key
path) to a valid golden case and records the message (all lines) the
reference prints after "FATAL ERROR!" when it rejects it: its State
(pylabolt/base/state.py:31-125: Control, Mesh, Lattice, Domain, Transport,
Fields, init_fields, Boundary, Obstacle), then its CollisionOperator and
ForceOperator (pylabolt/base/collision_operator.py:11-42,
pylabolt/base/force_operator.py:9-44) as pylabolt/solvers/fluidLB.py:135-147
builds them.  A mutation the reference accepts is recorded with message None.
The reference calls comm.Abort() after printing; the stand-in communicator
raises instead so that the next case can run.  The stand-ins of
make_golden.py are used (numba, mpi4py).

Written: tests/golden/config_validation.json.
"""
import argparse
import contextlib
import copy
import io
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg   # noqa: E402

CYL, PER, ELL = "channel_cylinder_abb", "poiseuille_guo2", "channel_ellipses"
B = "boundary_dict"
O = "obstacle_dict"
F = ["initial_fields_dict", "default", "fluid"]

# (name, base case, [("set", path, value) | ("del", path)])
MUTATIONS = [
    ("no control_dict", CYL, [("del", ["control_dict"])]),
    *[(f"no {k}", CYL, [("del", ["control_dict", k])])
      for k in ("start_time", "end_time", "std_out_interval", "save_interval",
                "checkpoint_interval", "precision")],
    ("bad precision", CYL, [("set", ["control_dict", "precision"], "other")]),
    ("no mesh_dict", CYL, [("del", ["mesh_dict"])]),
    ("no grid", CYL, [("del", ["mesh_dict", "grid"])]),
    ("grid not a list", CYL, [("set", ["mesh_dict", "grid"], "16x11")]),
    ("zero grid", CYL, [("set", ["mesh_dict", "grid"], [0, 11])]),
    ("point grid", CYL, [("set", ["mesh_dict", "grid"], [1, 1])]),
    ("no lattice_dict", CYL, [("del", ["lattice_dict"])]),
    ("no lattice_type", CYL, [("del", ["lattice_dict", "lattice_type"])]),
    ("bad lattice_type", CYL, [("set", ["lattice_dict", "lattice_type"], "D3Q19")]),
    ("no decompose_dict", CYL, [("del", ["decompose_dict"])]),
    ("no transport_dict", CYL, [("del", ["transport_dict"])]),
    ("no kin_visc", CYL, [("del", ["transport_dict", "kin_visc"])]),
    ("kin_visc a string", CYL, [("set", ["transport_dict", "kin_visc"], "0.05")]),
    ("no initial_fields_dict", CYL, [("del", ["initial_fields_dict"])]),
    ("no default region", CYL, [("del", ["initial_fields_dict", "default"])]),
    ("no default fluid", CYL, [("del", F)]),
    ("no density field", CYL, [("del", F + ["density"])]),
    ("no field type", CYL, [("del", F + ["density", "type"])]),
    ("bad field type", CYL, [("set", F + ["density", "type"], "other")]),
    ("no fixed value", CYL, [("del", F + ["density", "value"])]),
    ("scalar velocity", CYL, [("set", F + ["velocity"], {"type": "fixed", "value": 0.0})]),
    ("no boundary_dict", CYL, [("del", [B])]),
    ("no boundary options", CYL, [("del", [B, "options"])]),
    ("compute_force not bool", CYL, [("set", [B, "options"], {"compute_force": 0})]),
    ("no segments", CYL, [("del", [B, "walls", "segments"])]),
    ("segments not a list", CYL, [("set", [B, "walls", "segments"], "x")]),
    ("empty segments", CYL, [("set", [B, "walls", "segments"], [])]),
    ("segment structure", CYL, [("set", [B, "walls", "segments"], [[0, 0], [15, 0]])]),
    ("segment reversed", CYL, [("set", [B, "walls", "segments"], [[[15, 0], [0, 0]]])]),
    ("segment diagonal", CYL, [("set", [B, "walls", "segments"], [[[0, 0], [15, 10]]])]),
    ("no boundary fluid", CYL, [("del", [B, "walls", "fluid"])]),
    ("no boundary type", CYL, [("del", [B, "walls", "fluid", "type"])]),
    ("bad boundary type", CYL, [("set", [B, "walls", "fluid", "type"], "other")]),
    ("no pressure value", CYL, [("del", [B, "inlet", "fluid", "value"])]),
    ("pressure a string", CYL, [("set", [B, "inlet", "fluid", "value"], "1.0")]),
    ("no velocity value", CYL, [("set", [B, "walls", "fluid"], {"type": "fixed_velocity"})]),
    ("velocity a scalar", CYL, [("set", [B, "walls", "fluid"],
                                 {"type": "fixed_velocity", "value": 0.1})]),
    ("periodic single segment", PER, [("set", [B, "inout", "segments"], [[[0, 0], [0, 7]]])]),
    ("periodic orientation", PER, [("set", [B, "inout", "segments"],
                                    [[[0, 0], [0, 7]], [[0, 0], [9, 0]]])]),
    ("periodic partial span", PER, [("set", [B, "inout", "segments"],
                                     [[[0, 0], [0, 3]], [[9, 0], [9, 3]]])]),
    ("periodic not opposite", PER, [("set", [B, "inout", "segments"],
                                     [[[0, 0], [0, 7]], [[5, 0], [5, 7]]])]),
    ("no obstacle_dict", CYL, [("del", [O])]),
    ("no obstacle options", CYL, [("del", [O, "options"])]),
    ("compute_force_torque not bool", CYL, [("set", [O, "options"], {"compute_force_torque": 1})]),
    ("no obstacle type", CYL, [("del", [O, "cyl", "type"])]),
    ("bad obstacle type", CYL, [("set", [O, "cyl", "type"], "square")]),
    ("no radius", CYL, [("del", [O, "cyl", "radius"])]),
    ("radius a string", CYL, [("set", [O, "cyl", "radius"], "2")]),
    ("center a scalar", CYL, [("set", [O, "cyl", "center"], 5)]),
    ("density a string", CYL, [("set", [O, "cyl", "density"], "1")]),
    ("static not bool", CYL, [("set", [O, "cyl", "static"], 1)]),
    ("moving without motion dict", CYL, [("set", [O, "cyl", "static"], False)]),
    *[(f"no ellipse {k}", ELL, [("del", [O, "wing", k])])
      for k in ("semi_major_axis", "semi_minor_axis", "inclination_angle", "center",
                "density", "static")],
    ("semi_major_axis a string", ELL, [("set", [O, "wing", "semi_major_axis"], "3")]),
    ("semi_minor_axis a list", ELL, [("set", [O, "wing", "semi_minor_axis"], [1.5])]),
    ("inclination a string", ELL, [("set", [O, "wing", "inclination_angle"], "30")]),
    ("ellipse center a string", ELL, [("set", [O, "wing", "center"], "7,6.5")]),
    ("ellipse density a string", ELL, [("set", [O, "wing", "density"], "1")]),
    ("ellipse static not bool", ELL, [("set", [O, "wing", "static"], 0)]),
    ("ellipse moving without motion dict", ELL, [("set", [O, "wing", "static"], False)]),
    ("ellipse bad motion type", ELL, [("set", [O, "rotor", "solid_motion_dict", "type"],
                                       "oscillating")]),
    ("ellipse no angular velocity", ELL, [("del", [O, "rotor", "solid_motion_dict",
                                                   "angular_velocity"])]),
    ("no collision_dict", CYL, [("del", ["collision_dict"])]),
    ("no collision fluid", CYL, [("del", ["collision_dict", "fluid"])]),
    ("no collision model", CYL, [("del", ["collision_dict", "fluid", "model"])]),
    ("bad collision model", CYL, [("set", ["collision_dict", "fluid", "model"], "TRT")]),
    ("bad equilibrium", CYL, [("set", ["collision_dict", "fluid", "equilibrium"], "other")]),
    ("bad forcing model", CYL, [("set", ["collision_dict", "fluid", "forcing_model"], "other")]),
    ("no forcing_dict", CYL, [("del", ["forcing_dict"])]),
    ("gravity a scalar", CYL, [("set", ["forcing_dict", "gravity"], 1e-5)]),
]


def apply(case, ops):
    """Applies set / delete operations on key paths to a deep copy of case."""
    c = copy.deepcopy(case)
    for op in ops:
        path = op[1]
        node = c
        for k in path[:-1]:
            node = node[k]
        if op[0] == "del":
            del node[path[-1]]
        else:
            node[path[-1]] = copy.deepcopy(op[2])
    return c


class Abort(Exception):
    pass


class AbortComm(mg.DummyComm):
    def Abort(self, *args):
        raise Abort()


def to_module(case):
    """make_golden.to_module, tolerant of a mutated initial_fields_dict: the
    "array" fields that are well formed become funcs, everything else is
    passed to the reference as it is."""
    import types
    import numpy as np
    mod = types.ModuleType("simulation")
    for key, val in case.items():
        setattr(mod, key, val)
    ifd = case.get("initial_fields_dict")
    if not isinstance(ifd, dict):
        return mod
    out = {}
    for region, rd in ifd.items():
        if not isinstance(rd, dict) or not isinstance(rd.get("fluid"), dict):
            out[region] = rd
            continue
        fl = {}
        for fname, spec in rd["fluid"].items():
            if isinstance(spec, dict) and spec.get("type") == "array":
                arr = np.asarray(spec["value"])
                if arr.ndim == 3:
                    fl[fname] = {"type": "func",
                                 "func": (lambda a: lambda i, j: (float(a[i, j, 0]),
                                                                  float(a[i, j, 1])))(arr)}
                else:
                    fl[fname] = {"type": "func", "func": (lambda a: lambda i, j: float(a[i, j]))(arr)}
            else:
                fl[fname] = spec
        out[region] = dict(rd, fluid=fl)
    mod.initial_fields_dict = out
    return mod


def reference_message(case):
    from pylabolt.base.state import State
    from pylabolt.base.collision_operator import CollisionOperator
    from pylabolt.base.force_operator import ForceOperator
    from pylabolt.solvers.fluidLB import FluidLB
    out = io.StringIO()
    comm = AbortComm()
    try:
        with contextlib.redirect_stdout(out):
            sim = to_module(case)
            st = State(sim, comm, 0, fluid=True)
            model = FluidLB()
            col = CollisionOperator(sim, model, st, comm)
            ForceOperator(sim, model, st, comm, collision_operator=col)
    except Abort:
        lines = out.getvalue().splitlines()
        return "\n".join(lines[lines.index("FATAL ERROR!") + 1:])
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="path of the reference checkout")
    args = ap.parse_args()
    mg.install_numba_stub()
    mg.install_mpi4py_stub()
    sys.path.insert(0, args.ref)
    cases = mg.make_cases()
    out = []
    for name, base, ops in MUTATIONS:
        msg = reference_message(apply(cases[base][0], ops))
        out.append({"name": name, "base": base, "ops": ops, "reference": msg})
        print(f"{name:32s} {msg}")
    with open(os.path.join(HERE, "config_validation.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
