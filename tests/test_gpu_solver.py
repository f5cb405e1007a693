"""The drop-in Solver and command line on the GPU.

The full run (FP64 storage) of the output-enabled channel_cylinder_abb case
against what the reference's own writers produced for the reference's fields:
field files bit-exact, metadata identical, history files and status lines
with the same layout and values within the reduction tolerance (forces and
residues are sums whose order differs, 1e-12 relative)."""
import json
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from _golden import GOLDEN_DIR
from pylabolt_gb300 import output, solver

pytestmark = pytest.mark.gpu

SUM_RTOL = 1e-12
SUM_ATOL = 1e-13   # forces are sums of O(0.1-1) link terms: small results (lift) carry
                   # an absolute, not relative, reduction-order error
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _io_case():
    import test_output_cpu
    return test_output_cpu._io()


def _numbers(text):
    return np.array([float(v) for v in re.findall(r"-?\d\.\d+e[+-]\d+", text)])


@pytest.mark.parametrize("layout", ["ab", "aa"])
def test_solver_run_matches_reference_output(tmp_path, monkeypatch, capsys, layout):
    case, d, _ = _io_case()
    monkeypatch.setattr(output, "package_version", lambda: str(d["version"]))
    s = solver.Solver(case, root=str(tmp_path), storage="fp64", layout=layout)
    try:
        s.run()
    finally:
        s.close()
    out = capsys.readouterr().out
    with open(tmp_path / "metadata.json") as f:
        assert f.read() == str(d["metadata_json"])
    for t in (0, 30, 60):
        z = np.load(tmp_path / "output" / "fields" / f"t_{t}.npz")
        assert list(z.files) == d[f"fields_t{t}_keys"].tolist()
        for k in z.files:
            ref = d[f"fields_t{t}:{k}"]
            assert z[k].dtype == ref.dtype and np.array_equal(z[k], ref), (t, k)
    for h in d["history_names"].tolist():
        with open(tmp_path / "output" / "histories" / h) as f:
            mine = f.read()
        ref = str(d[f"history:{h}"])
        assert re.sub(r"-?\d\.\d+e[+-]\d+", "X", mine) == re.sub(r"-?\d\.\d+e[+-]\d+", "X", ref)
        np.testing.assert_allclose(_numbers(mine), _numbers(ref), rtol=SUM_RTOL, atol=SUM_ATOL)
    lines = [l for l in out.splitlines() if l.startswith("time:")]
    ref_lines = d["status_lines"].tolist()
    assert len(lines) == len(ref_lines)
    for a, b in zip(lines, ref_lines):
        assert re.sub(r"-?\d\.\d+e[+-]\d+", "X", a) == re.sub(r"-?\d\.\d+e[+-]\d+", "X", b)
        np.testing.assert_allclose(_numbers(a), _numbers(b), rtol=1e-4)


def test_command_line_cavity(tmp_path):
    """``python -m pylabolt_gb300 -s fluidLB -b gpu`` in a directory holding a
    simulation.py, as the reference's ``pylabolt`` is run."""
    from pylabolt_gb300 import workloads
    from pylabolt_gb300.config import Case
    from pylabolt_gb300.lbm import FluidLBM
    c = workloads.cavity(64, re=100.0)
    c["control_dict"].update({"end_time": 200, "std_out_interval": 100, "save_interval": 100})
    with open(tmp_path / "simulation.py", "w") as f:
        for k, v in c.items():
            f.write(f"{k} = {json.dumps(v)}\n".replace("null", "None").replace("true", "True")
                    .replace("false", "False"))
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-m", "pylabolt_gb300", "-s", "fluidLB", "-b", "gpu"],
                       cwd=tmp_path, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("time:")]
    assert [l.split()[1] for l in lines] == ["100", "200"]
    assert sorted(os.listdir(tmp_path / "output" / "fields")) == ["t_0.npz", "t_100.npz", "t_200.npz"]
    z = np.load(tmp_path / "output" / "fields" / "t_200.npz")
    with FluidLBM(Case(c), storage="fp64") as sim:
        sim.initialize()
        sim.step(200, moments=True)
        rho, u = sim.moments()
    assert np.array_equal(z["density"], rho.reshape(-1))
    assert np.array_equal(z["velocity"], u.reshape(-1, 2))


def test_solver_moving_obstacle_outputs(tmp_path, capsys):
    """A translating disk: its history rows follow the device state and each
    field file carries the geometry of its own step."""
    from test_moving_cpu import disk_case
    c = disk_case(True, v=(0.05, 0.0))
    c["control_dict"].update({"end_time": 40, "std_out_interval": 20, "save_interval": 20})
    c["obstacle_dict"]["options"]["write_obstacle_data"] = {"interval": 20}
    s = solver.Solver(c, root=str(tmp_path), storage="fp64")
    try:
        s.run()
    finally:
        s.close()
    rows = [l.split() for l in open(tmp_path / "output" / "histories" / "disk.dat")
            if not l.startswith("#")]
    assert [int(r[0]) for r in rows] == [0, 20, 40]
    xs = [float(r[1]) for r in rows]
    np.testing.assert_allclose(xs, [14.0, 15.0, 16.0], atol=1e-12)
    z0 = np.load(tmp_path / "output" / "fields" / "t_0.npz")
    z40 = np.load(tmp_path / "output" / "fields" / "t_40.npz")
    ny = 32
    X, Y = np.divmod(np.arange(40 * ny), ny)
    cx40 = 14.0
    for _ in range(40):     # the device's motion update, in the same FP64 order
        cx40 = cx40 + (0.05 + 0.5 * (0.0 / 1.0 + 0.0))
    for z, cx in ((z0, 14.0), (z40, cx40)):
        assert np.array_equal(z["solid"], (X - cx) ** 2 + (Y - 16.0) ** 2 <= 16.0)
        assert np.all(z["solid_id"][z["solid"]] == 0)
        assert np.all(z["fluid_boundary"] <= ~z["solid"])


def test_residue_lines_read_while_the_next_steps_run(tmp_path, capsys, monkeypatch):
    """A status line on every step, field output every 20: the lines of steps
    with no other output are logged once the next step is queued, and carry
    the values of a run that reads each residual right after its step (one
    launch shape for both, so the sums are the same bits)."""
    from pylabolt_gb300 import workloads
    from pylabolt_gb300.config import Case
    from pylabolt_gb300.lbm import FluidLBM
    monkeypatch.setenv("LBM_VARIANT", "3,2,128,1")
    c = workloads.cavity(64, re=100.0)
    c["control_dict"].update({"end_time": 45, "std_out_interval": 1, "save_interval": 20})
    s = solver.Solver(c, root=str(tmp_path), storage="fp32_shifted")
    try:
        s.run()
    finally:
        s.close()
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("time:")]
    assert [int(l.split()[1]) for l in lines] == list(range(1, 46))
    dtype = s.out.dtype
    with FluidLBM(Case(c), storage="fp32_shifted") as sim:
        sim.initialize()
        for t, line in enumerate(lines, 1):
            sim.step(1, residual=True)
            r = sim.residual().astype(dtype)
            assert line == output.log_line(t, res_density=r[:1], res_velocity=r[1:]), t
