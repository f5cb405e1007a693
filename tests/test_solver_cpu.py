"""The drop-in Solver's run loop on the CPU, against a stand-in for the GPU
handle that records its calls: a status line on every std_out_interval step,
in time order; a line whose step has no other output is read (residual at
step t) only after the next steps have been queued, and the last one before
the run ends."""
import numpy as np

from pylabolt_gb300 import solver, workloads


class RecordingLBM:
    """Stands in for FluidLBM: advances a step counter, returns residuals
    that encode the step they belong to, and logs every call."""

    def __init__(self, case, storage=None, device=0, layout=None):
        self.case = case
        self.t = 0
        self.log = []

    def initialize(self):
        self.t = 0

    def step(self, n, moments=False, residual=False):
        self.t += n
        self.log.append(("step", self.t, moments, residual))

    def residual(self, step=None):
        t = self.t if step is None else step
        assert t <= self.t
        self.log.append(("residual", t))
        return np.array([1e-3 * t, 2e-3 * t, 3e-3 * t])

    def moments(self, dtype=np.float64):
        nx, ny = self.case.nx, self.case.ny
        self.log.append(("moments", self.t))
        return np.ones((nx, ny), dtype=dtype), np.zeros((nx, ny, 2), dtype=dtype)

    def forces(self):
        return {"obstacles": np.zeros((0, 3)), "walls": np.zeros((0, 2))}

    def synchronize(self):
        self.log.append(("sync", self.t))

    def close(self):
        pass


def test_status_lines_are_read_while_the_next_steps_run(tmp_path, monkeypatch, capsys):
    monkeypatch.setattr(solver, "FluidLBM", RecordingLBM)
    c = workloads.cavity(32, re=100.0)
    c["control_dict"].update({"end_time": 43, "std_out_interval": 5, "save_interval": 20})
    s = solver.Solver(c, root=str(tmp_path))
    s.run()
    out = capsys.readouterr().out
    lines = [l for l in out.splitlines() if l.startswith("time:")]
    std_steps = [5, 10, 15, 20, 25, 30, 35, 40]
    assert [int(l.split()[1]) for l in lines] == std_steps
    for t, line in zip(std_steps, lines):     # each line carries its own step's residual
        assert f"{1e-3 * t:.5e}" in line
    log = s.lbm.log
    reads = [e[1] for e in log if e[0] == "residual"]
    assert reads == std_steps
    for t in std_steps:
        i = log.index(("residual", t))
        queued = max(e[1] for e in log[:i] if e[0] == "step")
        if t in (20, 40):      # field output at the same step: read at once
            assert queued == t
        else:                  # read once the next event's steps are queued
            assert queued > t
    # every residual is read before the final synchronisation
    assert log.index(("residual", 40)) < log.index(("sync", 43))
    assert np.allclose(s.residues, [0.04, 0.08, 0.12])
