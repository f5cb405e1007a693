"""Case set-up from ``simulation.py`` dictionaries.

Reads the same dictionaries as the reference's ``State``
(pylabolt/base/state.py:14-125) and validates them with the same rules and
messages: control (pylabolt/base/control.py:29-49), mesh (mesh.py:20-42),
lattice (lattice.py:29-74), decomposition (parallel/domain.py:32-48),
transport (transport.py:23-37), initial fields (init_fields.py:7-375),
boundaries (boundary.py:202-603), obstacles (obstacle.py:91-588), collision
(collision_operator.py:46-104) and forcing (force_operator.py:46-81).

Project extensions (no reference key exists for them):
* ``control_dict["storage"]`` in ``{"fp64", "fp32_shifted", "fp16_shifted"}``
  selects the population storage (default: ``fp64`` for precision
  ``double``, ``fp32_shifted`` for ``single``), ``control_dict["fp16_scale"]``
  the FP16 storage scale;
* ``control_dict["population_layout"]`` in ``{"ab", "aa"}``: two population
  buffers (default) or one buffer updated in place (AA pattern; half the
  population memory, not with moving obstacles, the adjoint or
  zero_gradient boundaries);
* ``collision_dict["fluid"]["mrt_rates"] = {"s_e", "s_eps", "s_q", "s_nu"}``
  (defaults: the reference's S = [1,...,1, omega, omega]);
* boundary type ``zero_gradient``;
* ``forcing_dict["body_force_field"]``: per-node force ``[Nx, Ny, 2]``;
* initial field type ``array``: explicit ``[Nx, Ny]`` / ``[Nx, Ny, 2]`` values.
"""
import numpy as np

from .lattice import INV_CS_2, INV_CS_4, EPS64, LOCATIONS

SUPPORTED_FLUID_BCS = ["bounce_back", "fixed_velocity", "fixed_pressure", "periodic",
                       "zero_gradient"]
COLLISION_MODELS = ["BGK", "MRT"]
EQUILIBRIUM_MODELS = ["density_based_second_order"]
FORCING_MODELS = [None, "guo_linear", "guo_second_order"]
STORAGES = ["fp64", "fp32_shifted", "fp16_shifted"]
POPULATION_LAYOUTS = ["ab", "aa"]


def _get(sim, name):
    if isinstance(sim, dict):
        if name not in sim:
            raise ValueError(f"{name} not found in simulation.py file")
        return sim[name]
    if not hasattr(sim, name):
        raise ValueError(f"{name} not found in simulation.py file")
    return getattr(sim, name)


def _has(sim, name):
    return name in sim if isinstance(sim, dict) else hasattr(sim, name)


def _write_interval(opts, where):
    """``write_*_data: {"interval": int | None}`` (boundary.py:254-272,
    obstacle.py:169-184); 1 when the option is absent."""
    key = "write_boundary_data" if where == "boundary_dict" else "write_obstacle_data"
    if key not in opts:
        return 1
    d = opts[key]
    if "interval" not in d:
        raise ValueError(f"interval missing {where} options!")
    iv = d["interval"]
    if not isinstance(iv, (int, type(None))):
        raise ValueError(f"interval must be int or None in {where} options")
    if isinstance(iv, int) and iv <= 0:
        raise ValueError(f"if interval is int then it must be > 0 in {where} options")
    return iv


class BoundaryElement:
    """One segment of one ``boundary_dict`` entry (boundary.py:7-127)."""

    def __init__(self, name, seg_no, segment, bc_type, location, value, wall):
        self.name = f"{name}_{seg_no}"
        self.type = bc_type
        self.location = location
        self.segment = segment
        self.value = value
        self.wall = wall
        normal, out_list, inv_list = LOCATIONS[location]
        self.normal = normal
        self.out_list = out_list
        self.inv_list = inv_list
        (x1, y1), (x2, y2) = segment
        if x1 == x2:
            self.orientation = "vertical"
            self.ys = np.arange(y1, y2 + 1, dtype=np.int64)
            self.xs = np.full(self.ys.size, x1, dtype=np.int64)
        else:
            self.orientation = "horizontal"
            self.xs = np.arange(x1, x2 + 1, dtype=np.int64)
            self.ys = np.full(self.xs.size, y1, dtype=np.int64)


class Obstacle:
    def __init__(self, obstacle_id, name, kind, center, radius, density, static,
                 linear_velocity, angular_velocity, semi_axes=None, inclination=0.0):
        self.id = obstacle_id
        self.name = name
        self.type = kind
        self.center = np.asarray(center, dtype=np.float64)
        self.radius = radius
        self.semi_axes = semi_axes
        self.inclination = inclination
        self.density = density
        self.static = static
        self.linear_velocity = np.asarray(linear_velocity, dtype=np.float64)
        self.angular_velocity = float(angular_velocity)
        # solid_motion_dict (obstacle.py:478-538); mass and moment of inertia
        # of a disc of the obstacle's density (obstacle.py:475-476)
        self.motion_type = None
        self.calculated = False
        self.rotation_allowed = False
        self.translation_allowed = False
        if semi_axes is not None:
            # obstacle.py:703-710
            a, b = (float(v) for v in semi_axes)
            self.mass = np.pi * a * b * density
            self.moment_of_inertia = self.mass * (a * a + b * b) / 4
        else:
            r = float(radius) if radius is not None else 0.0
            self.mass = np.pi * r * r * density
            self.moment_of_inertia = self.mass * r * r / 2


class Case:
    """Validated case: parameters, boundary elements, obstacles and initial
    fields on inner nodes ``[Nx, Ny]`` (x-major)."""

    def __init__(self, sim):
        self._control(_get(sim, "control_dict"))
        self._mesh(_get(sim, "mesh_dict"))
        self._lattice(_get(sim, "lattice_dict"))
        self._decompose(_get(sim, "decompose_dict"))
        self._transport(_get(sim, "transport_dict"))
        self._initial_fields(_get(sim, "initial_fields_dict"))
        self._boundaries(_get(sim, "boundary_dict"))
        self._obstacles(_get(sim, "obstacle_dict"))
        self._collision(_get(sim, "collision_dict"))
        self._forcing(_get(sim, "forcing_dict") if _has(sim, "forcing_dict") else None)

    # ---- control_dict -- control.py:29-49
    def _control(self, cd):
        try:
            self.start_time = cd["start_time"]
            self.end_time = cd["end_time"]
            self.std_out_interval = cd["std_out_interval"]
            self.save_interval = cd["save_interval"]
            self.checkpoint_interval = cd["checkpoint_interval"]
            self.precision_type = cd["precision"]
        except KeyError as e:
            raise ValueError(e.args[0] + " missing in control_dict")
        if self.precision_type not in ("single", "double"):
            raise ValueError("unsupported precision specified." +
                             "available precision (single, double)")
        default = "fp64" if self.precision_type == "double" else "fp32_shifted"
        self.storage = cd.get("storage", default)
        if self.storage not in STORAGES:
            raise ValueError(f"unsupported storage {self.storage!r}; available {STORAGES}")
        self.fp16_scale = float(cd.get("fp16_scale", 4096.0))
        self.population_layout = cd.get("population_layout", "ab")
        if self.population_layout not in POPULATION_LAYOUTS:
            raise ValueError(f"unsupported population_layout {self.population_layout!r}; "
                             f"available {POPULATION_LAYOUTS}")

    # ---- mesh_dict -- mesh.py:20-42
    def _mesh(self, md):
        if "grid" not in md:
            raise ValueError("grid missing in mesh_dict")
        grid = md["grid"]
        if not isinstance(grid, list) or len(grid) != 2:
            raise ValueError("grid entry in mesh_dict must be a list [Nx, Ny]")
        grid = np.array(grid, dtype=int)
        if np.any(grid == 0):
            raise ValueError("grid dimensions cannot be zero")
        if np.all(grid == 1):
            raise ValueError("grid specified is a point")
        if grid[0] == 1 or grid[1] == 1:
            raise ValueError("fluidLB on this backend needs a 2-D grid (D2Q9)")
        self.nx, self.ny = int(grid[0]), int(grid[1])

    def _lattice(self, ld):
        if "lattice_type" not in ld:
            raise ValueError("lattice_type missing in lattice_dict")
        if ld["lattice_type"] != "D2Q9":
            raise ValueError("Unsupported lattice type")

    def _decompose(self, dd):
        if "nx" not in dd or "ny" not in dd:
            raise ValueError("nx or ny missing decompose_dict")
        if dd["nx"] * dd["ny"] != 1:
            raise ValueError("invalid domain decomposition. this backend runs one "
                             "case per GPU (decompose_dict nx = ny = 1)")

    # ---- transport_dict -- transport.py:23-37, collision_operator.py:89-91
    def _transport(self, td):
        if "kin_visc" not in td:
            raise ValueError("kin_visc missing in transport_dict")
        kv = td["kin_visc"]
        if not isinstance(kv, (float, int)):
            raise ValueError("kin_visc must be a float/int")
        self.kin_visc = float(np.float64(kv))
        self.inv_cs_2 = float(INV_CS_2)
        self.inv_cs_4 = float(INV_CS_4)
        self.eps = float(EPS64)
        self.tau = float(np.float64(self.kin_visc) * INV_CS_2 + 0.5)
        self.omega = float(1 / np.float64(self.tau))

    # ---- initial_fields_dict -- init_fields.py:7-375
    def _initial_fields(self, ifd):
        self.density = np.zeros((self.nx, self.ny))
        self.velocity = np.zeros((self.nx, self.ny, 2))
        if "default" not in ifd:
            raise ValueError("default missing in initial_fields_dict")
        default = ifd["default"]
        if "fluid" not in default:
            raise ValueError("fluid missing in initial_fields_dict - default")
        for key in ("velocity", "density", "pressure"):
            if key not in default["fluid"]:
                raise ValueError(f"'{key}' is missing in default")
        for region, rd in ifd.items():
            if region != "default" and "fluid" not in rd:
                continue
            fd = rd["fluid"]
            if "velocity" in fd:
                self.velocity[...] = self._field(fd["velocity"], vector=True)
            if "density" in fd:
                self.density[...] = self._field(fd["density"], vector=False)

    def _field(self, spec, vector):
        if "type" not in spec:
            raise ValueError("type missing in field definition")
        kind = spec["type"]
        shape = (self.nx, self.ny, 2) if vector else (self.nx, self.ny)
        if kind == "fixed":
            if "value" not in spec:
                raise ValueError("value missing for fixed type field definition")
            v = spec["value"]
            ok = (isinstance(v, list) and len(v) == 2) if vector else isinstance(v, (int, float))
            if not ok:
                raise ValueError("vector value must be a list (ux, uy)" +
                                 " and scalar value must be a float or int")
            return np.broadcast_to(np.asarray(v, dtype=np.float64), shape)
        if kind == "func":
            if "func" not in spec:
                raise ValueError("func missing for func type field definition")
            f = spec["func"]
            out = np.zeros(shape)
            for x in range(self.nx):
                for y in range(self.ny):
                    out[x, y] = f(x, y)
            return out
        if kind == "array":
            arr = np.asarray(spec["value"], dtype=np.float64)
            if arr.shape != shape:
                raise ValueError(f"array field must have shape {shape}")
            return arr
        raise ValueError("Unsupported velocity initialization")

    # ---- boundary_dict -- boundary.py:202-603
    def _boundaries(self, bd):
        self.elements = []
        self.x_periodic = False
        self.y_periodic = False
        if "options" not in bd:
            raise ValueError("options missing in boundary_dict")
        opts = bd["options"]
        self.compute_boundary_force = opts.get("compute_force", False)
        if not isinstance(self.compute_boundary_force, (bool, np.bool_)):
            raise ValueError("compute_force must be a bool: True/False (default: False)")
        self.write_boundary_data = "write_boundary_data" in opts
        self.boundary_write_interval = _write_interval(opts, "boundary_dict")
        for name, ud in bd.items():
            if name == "options":
                continue
            self._boundary_entry(name, ud)

    def _boundary_entry(self, name, ud):
        if "wall" not in ud:
            raise ValueError("wall missing in boundary: " + name)
        wall = ud["wall"]
        if not isinstance(wall, (bool, np.bool_)):
            raise ValueError("wall entry must be True/False: " + name)
        if "segments" not in ud:
            raise ValueError("segments missing in boundary: " + name)
        segments = ud["segments"]
        if not isinstance(segments, list):
            raise ValueError("segments must be a list object: " + name)
        if len(segments) == 0:
            raise ValueError("segments cannot be an empty list: " + name)
        for seg in segments:
            if not (isinstance(seg, list) and len(seg) == 2 and
                    all(isinstance(pt, list) and len(pt) == 2 for pt in seg)):
                raise ValueError("segment must have structure [[x1, y1], [x2, y2]]: " + name)
            (x1, y1), (x2, y2) = seg
            if not (x2 >= x1 and y2 >= y1):
                raise ValueError("segment must satisfy x2 >= x1 and y2 >= y1: " + name)
            if not (x1 == x2 or y1 == y2):
                raise ValueError("segment must be axis-aligned (horizontal or vertical): " + name)
        if "fluid" not in ud:
            raise ValueError("fluid missing in boundary: " + name)
        fd = ud["fluid"]
        if "type" not in fd:
            raise ValueError("type missing in fluid section of boundary: " + name)
        bc = fd["type"]
        if bc not in SUPPORTED_FLUID_BCS:
            raise ValueError("Unsupported boundary condition for fluid: " + str(bc))
        value = None
        if bc == "fixed_velocity":
            if "value" not in fd:
                raise ValueError("value missing in fluid section of boundary: " + name)
            value = fd["value"]
            if not isinstance(value, list) or len(value) != 2:
                raise ValueError("value for fixed_velocity must be a list (ux, uy): " + name)
            value = [float(np.float64(v)) for v in value]
        elif bc == "fixed_pressure":
            if "value" not in fd:
                raise ValueError("value missing in fluid section of boundary: " + name)
            value = fd["value"]
            if not isinstance(value, (int, float)):
                raise ValueError("value for fixed_pressure must be a float or int: " + name)
            value = float(np.float64(value))
        if bc == "periodic":
            self._validate_periodic(name, segments)
        for seg_no, seg in enumerate(segments):
            (x1, y1), (x2, y2) = seg
            loc = None
            if x2 - x1 == 0:
                loc = "right" if x2 == self.nx - 1 else ("left" if x2 == 0 else None)
            elif y2 - y1 == 0:
                loc = "top" if y2 == self.ny - 1 else ("bottom" if y2 == 0 else None)
            if loc is None:
                raise ValueError("segment must lie on the domain edge: " + name)
            if x1 < 0 or y1 < 0 or x2 >= self.nx or y2 >= self.ny:
                raise ValueError("segment outside the grid: " + name)
            self.elements.append(BoundaryElement(name, seg_no, seg, bc, loc, value, wall))

    def _validate_periodic(self, name, segments):
        if len(segments) != 2:
            raise ValueError("For periodic boundary, each segment should be" +
                             " followed by a corresponding periodic pair: " + name)
        s1, s2 = segments
        ly1 = abs(s1[1][1] - s1[0][1])
        lx1 = abs(s1[1][0] - s1[0][0])
        ly2 = abs(s2[1][1] - s2[0][1])
        lx2 = abs(s2[1][0] - s2[0][0])
        horizontal, vertical = ly1 == 0, lx1 == 0
        if horizontal and ly2 != 0:
            raise ValueError("invalid periodic pair - different orientation: " + name)
        if vertical and lx2 != 0:
            raise ValueError("invalid periodic pair - different orientation: " + name)
        if horizontal:
            if ((s1[0][0], s1[1][0]) != (0, self.nx - 1) or
                    (s2[0][0], s2[1][0]) != (0, self.nx - 1)):
                raise ValueError("horizontal periodic boundaries must span" +
                                 " the entire x-direction: " + name)
            if sorted([s1[0][1], s2[0][1]]) != [0, self.ny - 1]:
                raise ValueError("horizontal periodic boundaries must connect" +
                                 " top-bottom boundaries: " + name)
            self.y_periodic = True
        elif vertical:
            if ((s1[0][1], s1[1][1]) != (0, self.ny - 1) or
                    (s2[0][1], s2[1][1]) != (0, self.ny - 1)):
                raise ValueError("vertical periodic boundaries must span" +
                                 " the entire y-direction: " + name)
            if sorted([s1[0][0], s2[0][0]]) != [0, self.nx - 1]:
                raise ValueError("vertical periodic boundaries must connect" +
                                 " left-right boundaries: " + name)
            self.x_periodic = True

    # ---- obstacle_dict -- obstacle.py:91-588, obstacle_kernels.py:11-93
    def _obstacles(self, od):
        self.obstacles = []
        self.solid = np.zeros((self.nx, self.ny), dtype=bool)
        self.solid_id = np.full((self.nx, self.ny), -1, dtype=np.int64)
        if "options" not in od:
            raise ValueError("options missing in obstacle_dict")
        opts = od["options"]
        self.compute_force_torque = opts.get("compute_force_torque", False)
        if not isinstance(self.compute_force_torque, (bool, np.bool_)):
            raise ValueError("compute_force_torque must be bool: True/False (default: False)")
        if "ref_point_torque" in opts and self.compute_force_torque:
            # parsed and validated as obstacle.py:147-163 does; like the
            # reference, the torque is taken about each obstacle's centre
            if not isinstance(opts["ref_point_torque"], list):
                raise ValueError("ref_point_torque must be list: (x, y)")
        self.write_obstacle_data = "write_obstacle_data" in opts
        self.obstacle_write_interval = _write_interval(opts, "obstacle_dict")
        names = [k for k in od if k != "options"]
        for oid, name in enumerate(names):
            d = od[name]
            if "type" not in d:
                raise ValueError("type missing in obstacle: " + name)
            if d["type"] == "ellipse":
                self._check_ellipse(name, d)
            elif d["type"] != "circle":
                raise ValueError("Unsupported obstacle type: " + str(d["type"]))
            else:
                for key in ("radius", "center", "density", "static"):
                    if key not in d:
                        raise ValueError(f"{key} missing in obstacle: " + name)
                if type(d["radius"]) not in (float, int):
                    raise ValueError("radius must be float or int for obstacle type circle: " + name)
                if not isinstance(d["center"], list):
                    raise ValueError("center must be list for obstacle type circle: " + name)
                if type(d["density"]) not in (float, int):
                    raise ValueError("density must be float or int for obstacle type circle: " + name)
                if not isinstance(d["static"], (bool, np.bool_)):
                    raise ValueError("static must be True/False for obstacle type circle: " + name)
            lin, ang = [0.0, 0.0], 0.0
            if not d["static"]:
                if "solid_motion_dict" not in d:
                    raise ValueError("solid_motion_dict missing in obstacle: " + name)
                sm = d["solid_motion_dict"]
                for key in ("type", "degree_of_freedom", "linear_velocity", "angular_velocity"):
                    if key not in sm:
                        raise ValueError(key + " missing in solid_motion_dict: " + name)
                lin, ang = sm["linear_velocity"], sm["angular_velocity"]
                if sm["type"] not in ("fixed_velocity", "calculated"):
                    raise ValueError("Unsupported motion type: " + str(sm["type"]) +
                                     " in obstacle: " + name)
                if sm["degree_of_freedom"] not in ("rotation", "translation", "both"):
                    raise ValueError("Unsupported degree of freedom: " +
                                     str(sm["degree_of_freedom"]) + " in obstacle: " + name)
                if not isinstance(lin, list):
                    raise ValueError("linear_velocity must be list [ux, uy]: " + name)
                if not isinstance(ang, (int, float)):
                    raise ValueError("angular_velocity must be int/float: " + name)
            if d["type"] == "ellipse":
                obs = Obstacle(oid, name, "ellipse", d["center"], None, float(d["density"]),
                               bool(d["static"]), lin, ang,
                               semi_axes=(float(d["semi_major_axis"]), float(d["semi_minor_axis"])),
                               inclination=float(d["inclination_angle"]))
            else:
                obs = Obstacle(oid, name, "circle", d["center"], float(d["radius"]),
                               float(d["density"]), bool(d["static"]), lin, ang)
            if not d["static"]:
                sm = d["solid_motion_dict"]
                obs.motion_type = sm["type"]
                obs.calculated = sm["type"] == "calculated"
                obs.rotation_allowed = sm["degree_of_freedom"] in ("rotation", "both")
                obs.translation_allowed = sm["degree_of_freedom"] in ("translation", "both")
            self.obstacles.append(obs)
            moving = (not obs.static) and bool(opts.get("move_obstacles", False))
            if obs.type == "ellipse":
                self._rasterise_ellipse(obs, solid=not moving)
            else:
                self._rasterise_circle(obs, solid=not moving)
        if any(not o.static for o in self.obstacles) and not self.compute_force_torque:
            raise ValueError("If any obstacle is not static, "
                             "then compute_force_torque must be True")
        # extension: move the non-static obstacles (the reference's moving path
        # cannot run; without this key they keep their place and act as moving
        # walls, which is what the reference's kernels do for one step)
        self.move_obstacles = bool(opts.get("move_obstacles", False))
        if not isinstance(opts.get("move_obstacles", False), (bool, np.bool_)):
            raise ValueError("move_obstacles must be bool: True/False (default: False)")
        self.moving = [o for o in self.obstacles if not o.static] if self.move_obstacles else []

    @staticmethod
    def _check_ellipse(name, d):
        """Keys, types and messages of the reference's Ellipse
        (pylabolt/base/obstacle.py:591-701), in its order."""
        for key in ("semi_major_axis", "semi_minor_axis"):
            if key not in d:
                raise ValueError(key + " missing in obstacle: " + name)
            if type(d[key]) not in (float, int):
                raise ValueError(key + " must be float or int for obstacle type ellipse: " + name)
        if "inclination_angle" not in d:
            raise ValueError("inclination_angle missing in obstacle: " + name)
        if type(d["inclination_angle"]) not in (float, int):
            raise ValueError("inclination_angle must be float or int for obstacle type ellipse "
                             "representing angle in degrees: " + name)
        if "center" not in d:
            raise ValueError("center missing in obstacle: " + name)
        if not isinstance(d["center"], list):
            raise ValueError("center must be list for obstacle type ellipse: " + name)
        if "density" not in d:
            raise ValueError("density missing in obstacle: " + name)
        if type(d["density"]) not in (float, int):
            raise ValueError("density must be float or int for obstacle type ellipse: " + name)
        if "static" not in d:
            raise ValueError("static missing in obstacle: " + name)
        if not isinstance(d["static"], (bool, np.bool_)):
            raise ValueError("static must be True/False for obstacle type ellipse: " + name)

    def _min_image_offsets(self, obs):
        """Node offsets from the obstacle centre with the reference's periodic
        minimum image (try r + N, then r - N), [nx, ny] each."""
        X, Y = np.meshgrid(np.arange(self.nx, dtype=np.float64),
                           np.arange(self.ny, dtype=np.float64), indexing="ij")
        rx = X - obs.center[0]
        ry = Y - obs.center[1]
        rxm, rym = rx.copy(), ry.copy()
        if self.x_periodic:
            a = rx + self.nx
            rxm = np.where(np.abs(a) < np.abs(rxm), a, rxm)
            b = rx - self.nx
            rxm = np.where(np.abs(b) < np.abs(rxm), b, rxm)
        if self.y_periodic:
            a = ry + self.ny
            rym = np.where(np.abs(a) < np.abs(rym), a, rym)
            b = ry - self.ny
            rym = np.where(np.abs(b) < np.abs(rym), b, rym)
        return rxm, rym

    def _mark_solid(self, obs, inside, rxm, rym, solid=True):
        if solid:
            self.solid |= inside
            self.solid_id[inside] = obs.id
        lin = obs.linear_velocity
        ang = np.float64(obs.angular_velocity)
        self.velocity[inside, 0] = lin[0] - ang * rym[inside]
        self.velocity[inside, 1] = lin[1] + ang * rxm[inside]
        self.density[inside] = obs.density

    def _rasterise_ellipse(self, obs, solid=True):
        """(x'/a)^2 + (y'/b)^2 <= 1 in the frame turned by the inclination,
        with the periodic minimum image (is_ellipse / construct_ellipse,
        pylabolt/parallel/cpu/obstacle_kernels.py:151-241, same operation
        order); solid nodes take the body velocity and density.  solid=False
        (a moving obstacle) sets only the fields: the device places it."""
        a, b = (np.float64(v) for v in obs.semi_axes)
        alpha = np.float64(obs.inclination) * np.pi / 180
        cos_a, sin_a = np.cos(alpha), np.sin(alpha)
        rxm, rym = self._min_image_offsets(obs)
        xp = rxm * cos_a + rym * sin_a
        yp = -rxm * sin_a + rym * cos_a
        inside = (xp * xp) / (a * a) + (yp * yp) / (b * b) <= 1
        self._mark_solid(obs, inside, rxm, rym, solid)

    def _rasterise_circle(self, obs, solid=True):
        """dist^2 <= r^2 with the periodic minimum image (obstacle_kernels.py:11-93);
        solid nodes take the body velocity and density.  solid=False (a moving
        obstacle) sets only the fields: the device places it."""
        rxm, rym = self._min_image_offsets(obs)
        r = np.float64(obs.radius)
        inside = rxm * rxm + rym * rym <= r * r
        self._mark_solid(obs, inside, rxm, rym, solid)

    # ---- collision_dict -- collision_operator.py:46-104
    def _collision(self, cd):
        if "fluid" not in cd:
            raise ValueError("fluid missing in collision_dict")
        fd = cd["fluid"]
        for key in ("model", "equilibrium", "forcing_model"):
            if key not in fd:
                raise ValueError(key + " missing in fluid: collision_dict")
        self.collision = fd["model"]
        self.equilibrium = fd["equilibrium"]
        self.forcing = fd["forcing_model"]
        if self.collision not in COLLISION_MODELS:
            raise ValueError("Unsupported fluid collision model: " + str(self.collision) +
                             "\nAvailable models: " + str(COLLISION_MODELS))
        if self.equilibrium not in EQUILIBRIUM_MODELS:
            raise ValueError("Unsupported fluid equilibrium model: " + str(self.equilibrium) +
                             "\nAvailable models: " + str(EQUILIBRIUM_MODELS))
        if self.forcing not in FORCING_MODELS:
            raise ValueError("Unsupported fluid forcing model: " + str(self.forcing) +
                             "\nAvailable models: " + str(FORCING_MODELS))
        rates = fd.get("mrt_rates", {})
        self.mrt_rates = (float(rates.get("s_e", 1.0)), float(rates.get("s_eps", 1.0)),
                          float(rates.get("s_q", 1.0)), float(rates.get("s_nu", self.omega)))

    # ---- forcing_dict -- force_operator.py:46-81
    def _forcing(self, fd):
        if fd is None:
            raise ValueError("forcing_dict not found in simulation.py file")
        self.gravity = np.zeros(2)
        self.body_force_field = None
        if self.forcing is None:
            return
        if "gravity" in fd:
            g = fd["gravity"]
            if not isinstance(g, list) or len(g) != 2:
                raise ValueError("gravity must be a list (gx, gy) in forcing dict")
            self.gravity = np.array(g, dtype=np.float64)
        if "body_force_field" in fd:
            bf = np.asarray(fd["body_force_field"], dtype=np.float64)
            if bf.shape != (self.nx, self.ny, 2):
                raise ValueError("body_force_field must have shape [Nx, Ny, 2]")
            self.body_force_field = bf
