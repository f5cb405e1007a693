"""Field and history output in the reference's on-disk layout.

Mirrors ``InputOutputOperator`` (pylabolt/utils/io_operator.py) for one rank:

* ``metadata.json`` (dump_metadata, :96-156)
* ``output/fields/t_<n>.npz`` with the fluidLB save fields (fluidLB.py:56-60),
  inner nodes x-major (copy_inner_data, parallel/cpu/io_operator_kernels.py),
  written every ``save_interval`` steps (write_fields_cpu, :158-190)
* ``output/histories/<obstacle>.dat`` and ``<boundary>_<segment>.dat``
  (setup_write_histories / write_histories_cpu, :236-372)

and the residue log line of ``SimulationStatusLogger``
(pylabolt/utils/helpers.py:37-56).  The formats are the reference's so that
its post-processing (reconstruct, npz2vtk) reads the output unchanged.
"""
import json
import os

import numpy as np

SAVE_FIELDS = ["density", "velocity", "solid", "solid_id", "solid_boundary",
               "fluid_boundary", "surface_normals"]


def package_version():
    """The version string written into metadata.json: the installed
    reference's when present (its readers compare nothing else), else this
    package's."""
    from importlib.metadata import version, PackageNotFoundError
    try:
        return version("pylabolt")
    except PackageNotFoundError:
        from . import __version__
        return __version__


def log_line(time_step, **values):
    """One status line: ``time: <t> | res_density: x | res_velocity: (x, y)``."""
    parts = [f"{'time:':<5} {time_step:<10}"]
    for key, value in values.items():
        value = np.atleast_1d(value)
        if len(value) == 1:
            text = f"{value[0]:.5e}"
        else:
            text = "(" + ", ".join(f"{v:.5e}" for v in value) + ")"
        parts.append(f"{key:<5}: {text}")
    return " | ".join(parts)


class Output:
    """Writers for one case; `root` is the run directory (the reference
    writes relative to the working directory)."""

    def __init__(self, case, geometry, root="."):
        self.case = case
        self.root = root
        self.dtype = np.float64 if case.precision_type == "double" else np.float32
        nx, ny = case.nx, case.ny
        self.n = nx * ny
        self.static = {
            "solid": geometry.inner("solid").astype(np.bool_),
            "solid_id": geometry.inner("solid_id").astype(np.dtype(int)),
            "solid_boundary": geometry.inner("solid_boundary").astype(np.bool_),
            "fluid_boundary": geometry.inner("fluid_boundary").astype(np.bool_),
            "surface_normals": geometry.inner("surface_normals").astype(self.dtype),
        }
        self.meta = {}
        for name in SAVE_FIELDS:
            if name in self.static:
                a = self.static[name]
            else:
                a = np.zeros((self.n, 2) if name == "velocity" else self.n, dtype=self.dtype)
            self.meta[name] = {"components": 1 if a.ndim == 1 else int(a.shape[1]),
                               "dtype": str(a.dtype)}
        self.field_dir = os.path.join(root, "output", "fields")
        os.makedirs(self.field_dir, exist_ok=True)
        self.history_dir = os.path.join(root, "output", "histories")
        self.walls = [el for el in case.elements if el.wall]

    # -- metadata.json
    def write_metadata(self):
        c = self.case
        meta = {
            "pylabolt": {"version": package_version(), "solver": "fluidLB"},
            "control": {"end_time": c.end_time, "start_time": c.start_time,
                        "save_interval": c.save_interval,
                        "checkpoint_interval": c.checkpoint_interval},
            "mesh": {"size": int(c.nx * c.ny), "shape": (int(c.nx), int(c.ny))},
            "decomposition": {"nx": 1, "ny": 1},   # one rank (decompose_dict is 1 x 1)
            "fields_saved": self.meta,
        }
        with open(os.path.join(self.root, "metadata.json"), "w") as f:
            json.dump(meta, f, indent=4)

    # -- fields
    def save_due(self, t):
        si = self.case.save_interval
        return si is not None and t % si == 0

    def write_fields(self, t, rho, u):
        """rho [nx, ny], u [nx, ny, 2] (FP64) of step t."""
        fields = {"density": np.asarray(rho, dtype=self.dtype).reshape(self.n),
                  "velocity": np.asarray(u, dtype=self.dtype).reshape(self.n, 2)}
        out = {name: fields[name] if name in fields else self.static[name]
               for name in SAVE_FIELDS}
        np.savez(os.path.join(self.field_dir, f"t_{t}.npz"), **out)

    # -- histories
    @staticmethod
    def _keep_until(path, t):
        """A resumed run keeps a history file's header and its rows up to time
        t (rows after t are written again).  True if the file was kept."""
        if t is None or not os.path.exists(path):
            return False
        with open(path) as f:
            lines = f.readlines()
        kept = [l for l in lines if l.startswith("#") or (l.split() and float(l.split()[0]) <= t)]
        with open(path, "w") as f:
            f.writelines(kept)
        return True

    def setup_histories(self, resume_time=None):
        c = self.case
        if not (c.write_obstacle_data or c.write_boundary_data):
            return
        os.makedirs(self.history_dir, exist_ok=True)
        if c.write_obstacle_data:
            for o in c.obstacles:
                path = os.path.join(self.history_dir, o.name + ".dat")
                if self._keep_until(path, resume_time):
                    continue
                with open(path, "w") as f:
                    f.write(f"{'#':5} {'PyLaBolt obstacle history'}\n"
                            f"{'#':5} {'ID':8}: {o.id}\n"
                            f"{'#':5} {'Name':8}: {o.name}\n"
                            f"{'#':5} {'Type':8}: {o.type}\n"
                            f"{'#':5} {'Columns':8}:\n")
                    f.write(f"{'#':5}{'time':<21}{'pos_x':<30}{'pos_y':<30}{'alpha':<30}"
                            f"{'vel_x':<30}{'vel_y':<30}{'omega':<30}{'force_x':<30}"
                            f"{'force_y':<30}{'torque':<30}\n")
        if c.write_boundary_data:
            for el in self.walls:
                path = os.path.join(self.history_dir, el.name + ".dat")
                if self._keep_until(path, resume_time):
                    continue
                with open(path, "w") as f:
                    f.write(f"{'#':5} {'PyLaBolt boundary history'}\n"
                            f"{'#':5} {'Name':8}: {el.name}\n"
                            f"{'#':5} {'Columns':8}:\n")
                    f.write(f"{'#':5}{'time':<21}{'force_x':<30}{'force_y':<30}\n")

    def obstacle_due(self, t):
        c = self.case
        return (c.write_obstacle_data and c.obstacle_write_interval is not None
                and t % c.obstacle_write_interval == 0)

    def boundary_due(self, t):
        """Wall histories are written on multiples of the write interval
        (io_operator.py:323-343); their forces are computed there only when
        compute_force is set (boundary_operator.py:204-237), else they stay 0."""
        c = self.case
        return (c.write_boundary_data and c.boundary_write_interval is not None
                and t % c.boundary_write_interval == 0)

    def set_geometry(self, geometry):
        """New geometry fields for the following field files (moving obstacles)."""
        for name in ("solid", "solid_id", "solid_boundary", "fluid_boundary", "surface_normals"):
            self.static[name] = geometry.inner(name).astype(self.static[name].dtype)

    def write_obstacles(self, t, force_torque, states=None):
        """force_torque [nobs, 3] (zeros when compute_force_torque is off);
        states {obstacle id: dict(center, angle, velocity, omega)} of moving
        obstacles (the others report their set-up values)."""
        d = self.dtype
        states = states or {}
        for o, ft in zip(self.case.obstacles, force_torque):
            st = states.get(o.id)
            if st is None:
                pos, alpha, vel, om = o.center, 0.0, o.linear_velocity, o.angular_velocity
            else:
                pos, alpha, vel, om = st["center"], st["angle"], st["velocity"], st["omega"]
            vals = [pos[0], pos[1], alpha, vel[0], vel[1], om, ft[0], ft[1], ft[2]]
            line = f"{t:<24}" + "".join(f"{float(d(v)):<30.16e}" for v in vals) + "\n"
            with open(os.path.join(self.history_dir, o.name + ".dat"), "a") as f:
                f.write(line)

    def write_walls(self, t, forces):
        """forces [nwalls, 2] in wall-element order."""
        d = self.dtype
        for el, fw in zip(self.walls, forces):
            line = f"{t:<24}{float(d(fw[0])):<30.16e}{float(d(fw[1])):<30.16e}\n"
            with open(os.path.join(self.history_dir, el.name + ".dat"), "a") as f:
                f.write(line)
