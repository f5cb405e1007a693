"""Drop-in fluidLB solver for ``pylabolt --solver fluidLB -b gpu``.

``Solver.run`` follows the reference's run loop (pylabolt/solvers/fluidLB.py:
306-384): initial populations, t = 0 forces and output, then per time step
the step itself, boundary forces, residues and the status line, field output
and histories, and the final run-time line.  The GPU library advances the
steps between two output events in one call (replayed CUDA graphs); steps
with an event record what the event reads (moments for field output, the
residual pass for the status line).  Outputs are the reference's files
(pylabolt_gb300.output).

Extension: ``control_dict["checkpoint_interval"]`` (read but unused by the
reference) writes the step state every that many steps to
``output/checkpoints/state_t<t>.npy`` (lbm_save_state), and a run whose
``start_time`` has such a file continues from it bit for bit instead of
starting from the initial fields.
"""
import os
import sys
import time

import numpy as np

from .config import Case
from .lbm import FluidLBM
from .obstacles import Geometry
from .output import Output, log_line


def load_simulation(path=None):
    """``import simulation`` from the working directory (helpers.py:10-24)."""
    d = path or os.getcwd()
    if d not in sys.path:
        sys.path.append(d)
    try:
        import simulation
    except ImportError:
        raise ImportError("Missing simulation.py file in current working directory")
    return simulation


def _next_multiple(t, interval):
    return (t // interval + 1) * interval


class Solver:
    """One fluidLB run on one GPU.  `simulation`: the ``simulation`` module
    (or a dict with its dictionaries); `root`: directory that receives
    ``metadata.json`` and ``output/``; `storage` / `layout` override
    ``control_dict["storage"]`` / ``["population_layout"]``."""

    def __init__(self, simulation, root=".", storage=None, device=0, verbose=True, layout=None):
        self.verbose = verbose
        self.case = Case(simulation)
        self.geometry = Geometry(self.case)
        self.out = Output(self.case, self.geometry, root)
        self.lbm = FluidLBM(self.case, storage=storage, device=device, layout=layout)
        self.root = root
        ci = self.case.checkpoint_interval
        self.checkpoint_interval = ci if isinstance(ci, int) and not isinstance(ci, bool) and ci > 0 \
            else None
        nobs = len(self.case.obstacles)
        self.nobs = nobs
        self.residues = None

    def log(self, msg):
        if self.verbose:
            print(msg, flush=True)

    # -- events of step t
    def _events(self, t):
        c = self.case
        std = c.std_out_interval is not None and t % c.std_out_interval == 0
        return std, self.out.save_due(t), self.out.boundary_due(t), self.out.obstacle_due(t)

    def _next_event(self, t):
        c = self.case
        cands = [c.end_time]
        for iv in (c.std_out_interval, c.save_interval):
            if iv is not None:
                cands.append(_next_multiple(t, iv))
        if c.write_boundary_data and c.boundary_write_interval is not None:
            cands.append(_next_multiple(t, c.boundary_write_interval))
        if c.write_obstacle_data and c.obstacle_write_interval is not None:
            cands.append(_next_multiple(t, c.obstacle_write_interval))
        if self.checkpoint_interval is not None:
            cands.append(_next_multiple(t, self.checkpoint_interval))
        return min(cands)

    def checkpoint_path(self, t):
        return os.path.join(self.root, "output", "checkpoints", f"state_t{t}.npy")

    def _log_residual(self, t):
        """The residue line of time step t (SimulationStatusLogger.log_data,
        pylabolt/solvers/fluidLB.py:370-375), from that step's residual sums:
        a step with no other output is logged after the next steps have been
        queued, so the GPU does not wait on the host between them."""
        r = self.lbm.residual(step=t).astype(self.out.dtype)
        self.residues = r
        self.log(log_line(t, res_density=r[:1], res_velocity=r[1:]))

    def _checkpoint(self, t):
        if self.checkpoint_interval is None or t % self.checkpoint_interval:
            return
        path = self.checkpoint_path(t)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        np.save(path, self.lbm.save_state())

    def _update_forces(self, obstacles, walls):
        """The reference computes obstacle forces every step when
        compute_force_torque is set (fluidLB.py:249-253) and wall forces on
        write steps when compute_force is set; here both are evaluated on the
        steps whose histories read them."""
        c = self.case
        want_obs = obstacles and c.compute_force_torque
        want_walls = walls and c.compute_boundary_force
        if not (want_obs or want_walls):
            return
        f = self.lbm.forces()
        if want_obs:
            self.obstacle_forces = f["obstacles"]
        if want_walls:
            self.wall_forces = f["walls"]

    def _moving_states(self):
        if not self.case.moving:
            return {}
        return {st["id"]: st for st in self.lbm.moving_obstacles()}

    def _moving_geometry(self):
        """Geometry fields of the current step: static solids from the case,
        moving ones from the device's node flags, normals about their current
        centres."""
        c = self.case
        flags = self.lbm.node_flags()
        solid = flags > 0
        solid_id = np.where(flags == 1, c.solid_id, -1)
        for j, o in enumerate(c.moving):
            solid_id[flags == 2 + j] = o.id
        states = self.lbm.moving_obstacles()
        centers = {st["id"]: st["center"] for st in states}
        angles = {st["id"]: st["angle"] for st in states}
        return Geometry(c, solid=solid, solid_id=solid_id, centers=centers, angles=angles)

    def run(self):
        c = self.case
        self.log("\n" + "-" * 80)
        self.log("Running simulation...\n")
        resume = self.checkpoint_path(c.start_time)
        resumed = c.start_time > 0 and os.path.exists(resume)
        self.out.write_metadata()
        self.out.setup_histories(resume_time=c.start_time if resumed else None)
        self.obstacle_forces = np.zeros((self.nobs, 3))
        self.wall_forces = np.zeros((len(self.out.walls), 2))
        self.lbm.initialize()
        if resumed:
            self.lbm.load_state(np.load(resume))
            self.log("Resuming from " + resume)
        # t = 0 forces and initial output (fluidLB.py:323-344); a resumed run
        # continues after them (the run that wrote the checkpoint wrote them)
        if not resumed:
            self._update_forces(self.out.obstacle_due(0), self.out.boundary_due(0))
            if self.out.save_due(c.start_time):
                rho, u = self.lbm.moments(dtype=self.out.dtype)
                if c.moving:
                    self.out.set_geometry(self._moving_geometry())
                self.out.write_fields(c.start_time, rho, u)
            if self.out.obstacle_due(0):
                self.out.write_obstacles(0, self.obstacle_forces, self._moving_states())
            if self.out.boundary_due(0):
                self.out.write_walls(0, self.wall_forces)
        t0 = time.perf_counter()
        t = c.start_time
        pending = None   # a residual step whose line is logged once the next steps are queued
        while t < c.end_time:
            te = self._next_event(t)
            std, save, bnd, obs = self._events(te)
            self.lbm.step(te - t, moments=save, residual=std)
            if pending is not None:   # read while the steps just queued run
                self._log_residual(pending)
                pending = None
            t = te
            self._checkpoint(t)
            self._update_forces(obs, bnd)
            if std:
                if save or obs or bnd or t >= c.end_time:
                    self._log_residual(t)
                else:
                    pending = t
            if save:
                rho, u = self.lbm.moments(dtype=self.out.dtype)
                if c.moving:
                    self.out.set_geometry(self._moving_geometry())
                self.out.write_fields(t, rho, u)
            if obs:
                self.out.write_obstacles(t, self.obstacle_forces, self._moving_states())
            if bnd:
                self.out.write_walls(t, self.wall_forces)
        self.lbm.synchronize()
        run_time = time.perf_counter() - t0
        self.log("\n" + "-" * 80)
        self.log(f"{'Simulation complete, run time':<30}: {str(run_time) + ' s':<30}")
        self.log("-" * 80)
        return run_time

    def close(self):
        self.lbm.close()


def main(backend="gpu", n_threads=1, debug_mode=False, root=None):
    """Entry point of ``pylabolt --solver fluidLB -b gpu`` (fluidLB.py:387-395)."""
    if backend != "gpu":
        raise SystemExit("pylabolt_gb300 provides the gpu backend only; "
                         "run the reference package for -b cpu")
    try:
        sim = load_simulation(root)
        solver = Solver(sim, root=root or ".")
    except (ValueError, ImportError) as e:
        print("-" * 80, flush=True)
        print("FATAL ERROR!", flush=True)
        print(str(e), flush=True)
        raise SystemExit(1)
    try:
        solver.run()
    finally:
        solver.close()
