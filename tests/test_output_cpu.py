"""Solver run loop and output files without a GPU.

The step library is replaced by a stand-in that serves the golden fields,
forces and residues of ``channel_cylinder_abb``; the files the Solver writes
must equal, byte for byte, what the reference's own InputOutputOperator and
status logger wrote for the same values (tests/golden/io_channel_cylinder.npz,
made by tests/golden/make_io_golden.py)."""
import json
import os

import numpy as np
import pytest

from _golden import GOLDEN_DIR, load_golden
from pylabolt_gb300 import output, solver
from pylabolt_gb300.output import log_line


def _io():
    d = np.load(os.path.join(GOLDEN_DIR, "io_channel_cylinder.npz"))
    case = json.loads(str(d["case_json"]))
    _, g = load_golden("channel_cylinder_abb")
    for region, rd in case["initial_fields_dict"].items():
        for fname, spec in rd["fluid"].items():
            if spec["type"] == "array":
                spec["value"] = g[f"init_{region}_{fname}"]
    return case, d, g


class GoldenLBM:
    """Stands in for FluidLBM: replays the golden values of the time reached."""

    def __init__(self, case, storage=None, device=0, layout=None):
        self.case = case
        _, self.d, self.g = _io()
        self.t = 0
        self.calls = []

    def initialize(self):
        self.t = 0

    def step(self, n, moments=False, residual=False):
        self.calls.append((n, moments, residual))
        self.t += n

    def _inner(self, a):
        nx, ny = self.case.nx, self.case.ny
        return a.reshape(nx + 2, ny + 2, *a.shape[1:])[1:-1, 1:-1]

    def moments(self, dtype=np.float64):
        if self.t == 0:
            r, u = self._inner(self.g["rho0"]), self._inner(self.g["u0"])
        else:
            r, u = self._inner(self.g[f"density_t{self.t}"]), self._inner(self.g[f"velocity_t{self.t}"])
        return r.astype(dtype), u.astype(dtype)

    def forces(self):
        return {"obstacles": self.g[f"force_obstacles_t{self.t}"],
                "walls": self.g[f"force_walls_t{self.t}"]}

    def residual(self, step=None):
        res = {int(r[0]): r[1:] for r in self.d["residues"]}
        return np.array(res[self.t if step is None else step])

    def synchronize(self):
        pass

    def close(self):
        pass


@pytest.fixture
def golden_run(tmp_path, monkeypatch, capsys):
    case, d, _ = _io()
    monkeypatch.setattr(solver, "FluidLBM", GoldenLBM)
    monkeypatch.setattr(output, "package_version", lambda: str(d["version"]))
    s = solver.Solver(case, root=str(tmp_path))
    s.run()
    return s, d, tmp_path, capsys.readouterr().out


def test_files_match_reference_writer(golden_run):
    s, d, root, _ = golden_run
    with open(root / "metadata.json") as f:
        assert f.read() == str(d["metadata_json"])
    hist = sorted(os.listdir(root / "output" / "histories"))
    assert hist == d["history_names"].tolist()
    for h in hist:
        with open(root / "output" / "histories" / h) as f:
            assert f.read() == str(d[f"history:{h}"]), h
    assert sorted(os.listdir(root / "output" / "fields")) == ["t_0.npz", "t_30.npz", "t_60.npz"]
    for t in (0, 30, 60):
        z = np.load(root / "output" / "fields" / f"t_{t}.npz")
        assert list(z.files) == d[f"fields_t{t}_keys"].tolist()
        for k in z.files:
            ref = d[f"fields_t{t}:{k}"]
            assert z[k].dtype == ref.dtype and np.array_equal(z[k], ref), (t, k)


def test_status_lines_match_reference_logger(golden_run):
    _, d, _, out = golden_run
    lines = [l for l in out.splitlines() if l.startswith("time:")]
    assert lines == d["status_lines"].tolist()
    assert "Simulation complete, run time" in out


def test_steps_grouped_between_events(golden_run):
    s, _, _, _ = golden_run
    # two events (t = 30, 60): each advances 30 steps with moments + residual
    assert s.lbm.calls == [(30, True, True), (30, True, True)]


def test_log_line_format():
    assert log_line(7, res_density=np.array([1.0]), res_velocity=np.array([2.0, 3.0])) == \
        "time: 7          | res_density: 1.00000e+00 | res_velocity: (2.00000e+00, 3.00000e+00)"


def test_event_schedule_without_output(tmp_path, monkeypatch):
    case, d, _ = _io()
    case["control_dict"].update({"std_out_interval": None, "save_interval": None,
                                 "end_time": 50})
    case["boundary_dict"]["options"] = {}
    case["obstacle_dict"]["options"] = {}
    monkeypatch.setattr(solver, "FluidLBM", GoldenLBM)
    s = solver.Solver(case, root=str(tmp_path), verbose=False)
    s.run()
    assert s.lbm.calls == [(50, False, False)]
    assert os.listdir(tmp_path / "output" / "fields") == []
    assert not os.path.exists(tmp_path / "output" / "histories")


def test_cli_rejects_cpu_backend():
    from pylabolt_gb300.__main__ import main
    with pytest.raises(SystemExit, match="gpu backend only"):
        main(["-s", "fluidLB", "-b", "cpu"])


class CheckpointLBM(GoldenLBM):
    """GoldenLBM with a stand-in step state: the time it was saved at."""

    def save_state(self):
        return np.array([self.t], dtype=np.int64).view(np.uint8)

    def load_state(self, state):
        self.t = int(np.asarray(state).view(np.int64)[0])


def test_checkpoints_scheduled_and_resumed(tmp_path, monkeypatch, capsys):
    case, d, _ = _io()
    case["control_dict"]["checkpoint_interval"] = 20
    monkeypatch.setattr(solver, "FluidLBM", CheckpointLBM)
    monkeypatch.setattr(output, "package_version", lambda: str(d["version"]))
    s = solver.Solver(case, root=str(tmp_path))
    s.run()
    # checkpoint events join the output events without changing them
    assert s.lbm.calls == [(20, False, False), (10, True, True), (10, False, False),
                           (20, True, True)]
    ck = tmp_path / "output" / "checkpoints"
    assert sorted(os.listdir(ck)) == ["state_t20.npy", "state_t40.npy", "state_t60.npy"]
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("time:")]
    assert lines == d["status_lines"].tolist()
    hist = tmp_path / "output" / "histories"
    before = {h: (hist / h).read_text() for h in os.listdir(hist)}
    # a run started at t = 30 resumes from that file: the histories keep their
    # rows up to t = 30 and get the later ones again, as the first run wrote them
    np.save(ck / "state_t30.npy", np.array([30], dtype=np.int64).view(np.uint8))
    case["control_dict"]["start_time"] = 30
    s = solver.Solver(case, root=str(tmp_path))
    s.run()
    assert s.lbm.calls == [(10, False, False), (20, True, True)]
    assert "Resuming from" in capsys.readouterr().out
    for h, text in before.items():
        assert (hist / h).read_text() == text, h
