"""Case dictionaries of the benchmark workloads (synthetic inputs).

No dataset is involved: every workload is a lattice-Boltzmann case generated
here from its stated shape and parameters, with seeded random perturbations.

* ``cavity``     lid-driven cavity, BGK, bounce-back walls + moving lid
* ``poiseuille`` gravity-driven channel, MRT + Guo forcing, periodic in x
* ``cylinder_shedding`` velocity-inlet channel with a cylinder at Re 100
  (vortex shedding: Strouhal number and drag coefficient)
* ``cylinder``   channel with a cylinder, anti-bounce-back pressure inlet /
                 outlet, bounce-back walls and cylinder, seeded +-1e-4 velocity
                 perturbation (numpy default_rng(seed))
* ``outlet_channel`` the same channel with a zero_gradient outlet
* ``ellipse_channel`` the same channel with an inclined ellipse
"""
import numpy as np


def _base(nx, ny, kin_visc, precision="double", storage=None, model="BGK",
          forcing=None, gravity=None, mrt_rates=None):
    cd = {"start_time": 0, "end_time": 0, "std_out_interval": None,
          "save_interval": None, "checkpoint_interval": None, "precision": precision}
    if storage:
        cd["storage"] = storage
    col = {"model": model, "equilibrium": "density_based_second_order",
           "forcing_model": forcing}
    if mrt_rates:
        col["mrt_rates"] = dict(mrt_rates)
    return {
        "control_dict": cd,
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
        "collision_dict": {"fluid": col},
        "forcing_dict": {} if gravity is None else {"gravity": list(gravity)},
    }


def cavity(n=128, re=100.0, lid=0.1, storage=None, lid_last=True, ny=None):
    """Lid-driven cavity, nu = U N / Re, tau = 3 nu + 1/2 (128^2, Re 100 ->
    nu = 0.128, tau = 0.884); `ny` (default n) makes it n wide and ny high."""
    kin_visc = lid * n / re
    m = n if ny is None else ny
    c = _base(n, m, kin_visc, storage=storage)
    walls = {"wall": True, "segments": [[[0, 0], [0, m - 1]], [[n - 1, 0], [n - 1, m - 1]],
                                         [[0, 0], [n - 1, 0]]],
             "fluid": {"type": "bounce_back"}}
    lid_d = {"wall": True, "segments": [[[0, m - 1], [n - 1, m - 1]]],
             "fluid": {"type": "fixed_velocity", "value": [lid, 0.0]}}
    if lid_last:
        c["boundary_dict"]["walls"] = walls
        c["boundary_dict"]["lid"] = lid_d
    else:
        c["boundary_dict"]["lid"] = lid_d
        c["boundary_dict"]["walls"] = walls
    return c


def poiseuille(nx=1024, ny=512, u_c=0.05, re=100.0, model="MRT", storage=None,
               rates=(1.4, 1.4, 1.2), forcing="guo_second_order"):
    """Gravity-driven plane Poiseuille flow, periodic in x, bounce-back walls in
    y.  The walls sit half a link outside the first and last rows, so the
    channel height is H = ny; nu = u_c H / Re, g_x = 8 nu u_c / H^2."""
    h = float(ny)
    kin_visc = u_c * h / re
    gx = 8.0 * kin_visc * u_c / (h * h)
    c = _base(nx, ny, kin_visc, model=model, forcing=forcing, gravity=[gx, 0.0],
              storage=storage,
              mrt_rates={"s_e": rates[0], "s_eps": rates[1], "s_q": rates[2]}
              if model == "MRT" else None)
    c["boundary_dict"]["inout"] = {"wall": False, "segments": [
        [[0, 0], [0, ny - 1]], [[nx - 1, 0], [nx - 1, ny - 1]]], "fluid": {"type": "periodic"}}
    c["boundary_dict"]["walls"] = {"wall": True, "segments": [
        [[0, 0], [nx - 1, 0]], [[0, ny - 1], [nx - 1, ny - 1]]], "fluid": {"type": "bounce_back"}}
    return c, {"gx": gx, "kin_visc": kin_visc, "H": h, "u_c": u_c}


def poiseuille_profile(ny, gx, kin_visc):
    """Analytic u_x(y) for walls at y = -1/2 and y = ny - 1/2."""
    y = np.arange(ny) + 0.5
    return gx / (2.0 * kin_visc) * y * (ny - y)


def poiseuille_startup_profile(ny, gx, kin_visc, t, terms=200):
    """u_x(y, t) of plane Poiseuille flow started from rest at t = 0 (walls at
    y = -1/2 and y = ny - 1/2): the parabola minus its decaying Fourier
    series, sum over odd n of 4 g H^2 / (nu (n pi)^3) sin(n pi y / H)
    exp(-nu (n pi / H)^2 t)."""
    h = float(ny)
    y = np.arange(ny) + 0.5
    u = gx / (2.0 * kin_visc) * y * (h - y)
    for n in range(1, 2 * terms, 2):
        u -= (4.0 * gx * h * h / (kin_visc * (n * np.pi) ** 3) * np.sin(n * np.pi * y / h) *
              np.exp(-kin_visc * (n * np.pi / h) ** 2 * t))
    return u


def cylinder(nx=8192, ny=2048, model="BGK", storage=None, kin_visc=0.04, radius=128.0,
             center=(2048, 1027), rho_in=1.0005, rho_out=1.0, seed=0, amp=1e-4,
             rates=(1.4, 1.4, 1.2)):
    """Channel with a cylinder of diameter 256 at (2048, 1024+3): anti-bounce-back
    pressure inlet (rho 1.0005) / outlet (rho 1.0), bounce-back top / bottom and
    cylinder, u0 ~ U(-amp, amp) per component from default_rng(seed)."""
    c = _base(nx, ny, kin_visc, model=model, storage=storage,
              mrt_rates={"s_e": rates[0], "s_eps": rates[1], "s_q": rates[2]}
              if model == "MRT" else None)
    b = c["boundary_dict"]
    b["inlet"] = {"wall": False, "segments": [[[0, 0], [0, ny - 1]]],
                  "fluid": {"type": "fixed_pressure", "value": rho_in}}
    b["outlet"] = {"wall": False, "segments": [[[nx - 1, 0], [nx - 1, ny - 1]]],
                   "fluid": {"type": "fixed_pressure", "value": rho_out}}
    b["walls"] = {"wall": True, "segments": [[[0, 0], [nx - 1, 0]],
                                              [[0, ny - 1], [nx - 1, ny - 1]]],
                  "fluid": {"type": "bounce_back"}}
    c["obstacle_dict"]["cylinder"] = {"type": "circle", "radius": float(radius),
                                      "center": [int(center[0]), int(center[1])],
                                      "density": 1.0, "static": True}
    rng = np.random.default_rng(seed)
    u0 = rng.uniform(-amp, amp, size=(nx, ny, 2))
    c["initial_fields_dict"]["default"]["fluid"]["velocity"] = {"type": "array", "value": u0}
    return c


def ellipse_channel(nx=512, ny=128, semi_axes=(24.0, 8.0), inclination=20.0, seed=0,
                    kin_visc=0.04, rho_in=1.0005, storage=None, model="BGK"):
    """The cylinder channel with an inclined ellipse (semi-axes a, b, angle
    in degrees) at (nx/4, ny/2 + 3) in place of the cylinder."""
    c = cylinder(nx=nx, ny=ny, model=model, storage=storage, kin_visc=kin_visc,
                 rho_in=rho_in, seed=seed)
    c["obstacle_dict"].pop("cylinder")
    c["obstacle_dict"]["wing"] = {"type": "ellipse", "semi_major_axis": float(semi_axes[0]),
                                  "semi_minor_axis": float(semi_axes[1]),
                                  "inclination_angle": float(inclination),
                                  "center": [nx // 4, ny // 2 + 3], "density": 1.0,
                                  "static": True}
    return c


def outlet_channel(nx, ny, outlet_last=True, seed=0):
    """The cylinder channel with a zero_gradient outlet in place of the
    fixed-pressure one: anti-bounce-back inlet (rho 1.0005), bounce-back
    walls, cylinder of radius ny/8 at (nx/4, ny/2 + 3).  outlet_last: the
    outlet is listed after the walls and wins at its two corners, where its
    sources leave the grid; otherwise the walls win there."""
    c = cylinder(nx=nx, ny=ny, radius=ny / 8.0, center=(nx // 4, ny // 2 + 3), seed=seed)
    b = c["boundary_dict"]
    outlet = b.pop("outlet")
    outlet["fluid"] = {"type": "zero_gradient"}
    walls = b.pop("walls")
    if outlet_last:
        b["walls"] = walls
        b["outlet"] = outlet
    else:
        b["outlet"] = outlet
        b["walls"] = walls
    return c


def cylinder_shedding(nx=800, ny=200, diameter=20, u_in=0.1, re=100.0, model="MRT",
                      storage=None, seed=0, amp=1e-3):
    """Vortex shedding behind a cylinder: velocity inlet (moving-wall
    bounce-back at u_in), anti-bounce-back outlet (rho 1), bounce-back walls
    (blockage diameter / ny), cylinder of the given diameter at (nx/5,
    ny/2 + 1), Re = u_in * diameter / nu.  Starts from u = (u_in, 0) plus a
    U(-amp, amp) perturbation per component (default_rng(seed)), rho = 1."""
    kin_visc = u_in * diameter / re
    c = _base(nx, ny, kin_visc, model=model, storage=storage,
              mrt_rates={"s_e": 1.4, "s_eps": 1.4, "s_q": 1.2} if model == "MRT" else None)
    b = c["boundary_dict"]
    b["inlet"] = {"wall": False, "segments": [[[0, 0], [0, ny - 1]]],
                  "fluid": {"type": "fixed_velocity", "value": [float(u_in), 0.0]}}
    b["outlet"] = {"wall": False, "segments": [[[nx - 1, 0], [nx - 1, ny - 1]]],
                   "fluid": {"type": "fixed_pressure", "value": 1.0}}
    b["walls"] = {"wall": True, "segments": [[[0, 0], [nx - 1, 0]],
                                              [[0, ny - 1], [nx - 1, ny - 1]]],
                  "fluid": {"type": "bounce_back"}}
    c["obstacle_dict"]["cylinder"] = {"type": "circle", "radius": diameter / 2.0,
                                      "center": [nx // 5, ny // 2 + 1],
                                      "density": 1.0, "static": True}
    rng = np.random.default_rng(seed)
    u0 = rng.uniform(-amp, amp, size=(nx, ny, 2))
    u0[..., 0] += u_in
    c["initial_fields_dict"]["default"]["fluid"]["velocity"] = {"type": "array", "value": u0}
    return c


def smooth_noise(nx, ny, sigma, seed):
    """Unit-variance Gaussian-smoothed N(0,1) field (periodic FFT filter)."""
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((nx, ny))
    kx = np.fft.fftfreq(nx)[:, None]
    ky = np.fft.rfftfreq(ny)[None, :]
    filt = np.exp(-2.0 * (np.pi * sigma) ** 2 * (kx ** 2 + ky ** 2))
    s = np.fft.irfft2(np.fft.rfft2(z) * filt, s=(nx, ny))
    return s / s.std()


def adjoint_channel(nx=512, ny=512, tau=0.8, mean_force=5e-6, amp=1e-6, sigma=8.0,
                    seed=1, storage=None, forcing="guo_second_order"):
    """Channel, periodic in x, bounce-back walls in y, BGK with Guo forcing and
    a per-node body force F = mean_force x + amp * smoothed noise (both
    components), tau fixed.  Returns the case dictionaries."""
    kin_visc = (tau - 0.5) / 3.0
    c = _base(nx, ny, kin_visc, forcing=forcing, storage=storage)
    c["boundary_dict"]["inout"] = {"wall": False, "segments": [
        [[0, 0], [0, ny - 1]], [[nx - 1, 0], [nx - 1, ny - 1]]], "fluid": {"type": "periodic"}}
    c["boundary_dict"]["walls"] = {"wall": True, "segments": [
        [[0, 0], [nx - 1, 0]], [[0, ny - 1], [nx - 1, ny - 1]]], "fluid": {"type": "bounce_back"}}
    F = np.zeros((nx, ny, 2))
    F[..., 0] = mean_force + amp * smooth_noise(nx, ny, sigma, seed)
    F[..., 1] = amp * smooth_noise(nx, ny, sigma, seed + 1000)
    c["forcing_dict"] = {"body_force_field": F}
    return c
