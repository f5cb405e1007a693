"""Moving obstacles on the CPU: the restatement of the moving-obstacle step
(tests/_moving_emulator.py) against the static fused plan when the obstacle
does not move, and its geometry bookkeeping when it does."""
import numpy as np
import pytest

from pylabolt_gb300 import workloads
from pylabolt_gb300.config import Case
from _fused_emulator import FusedEmulator
from _moving_emulator import MovingEmulator


def disk_case(moving, v=(0.0, 0.0), om=0.0, kind="fixed_velocity", dof="both", nx=40, ny=32,
              center=(14, 16), radius=4.0, density=1.0, lid=0.05):
    c = workloads.cavity(nx, re=lid * nx / 0.05, lid=lid)
    if nx != ny:
        c["mesh_dict"]["grid"] = [nx, ny]
        b = c["boundary_dict"]
        b["walls"]["segments"] = [[[0, 0], [0, ny - 1]], [[nx - 1, 0], [nx - 1, ny - 1]],
                                  [[0, 0], [nx - 1, 0]]]
        b["lid"]["segments"] = [[[0, ny - 1], [nx - 1, ny - 1]]]
    c["obstacle_dict"]["options"] = {"compute_force_torque": True, "move_obstacles": moving}
    d = {"type": "circle", "radius": radius, "center": list(center), "density": density,
         "static": False, "solid_motion_dict": {"type": kind, "degree_of_freedom": dof,
                                                "linear_velocity": list(v),
                                                "angular_velocity": om}}
    c["obstacle_dict"]["disk"] = d
    return c


def wing_case(moving, v=(0.0, 0.0), om=0.0, kind="fixed_velocity", dof="both", axes=(6.0, 2.5),
              incl=30.0, density=1.0, nx=48, ny=40, center=(18, 20)):
    """The disk case with an inclined ellipse in place of the disk."""
    c = disk_case(moving, v=v, om=om, kind=kind, dof=dof, nx=nx, ny=ny, center=center,
                  density=density)
    d = c["obstacle_dict"].pop("disk")
    del d["radius"]
    d.update({"type": "ellipse", "semi_major_axis": axes[0], "semi_minor_axis": axes[1],
              "inclination_angle": incl})
    c["obstacle_dict"]["wing"] = d
    return c


def test_resting_moving_ellipse_equals_static_ellipse():
    """An ellipse that does not move: the device-placed raster and its run-time
    links reproduce the static rasteriser and link records bit for bit."""
    st = FusedEmulator(Case(wing_case(False)))
    mv = MovingEmulator(Case(wing_case(True)))
    st.initialize()
    mv.initialize()
    assert np.array_equal(mv.dsolid > 0, st.solid)
    for _ in range(40):
        st.step()
        mv.step()
    fl = ~st.solid
    assert np.array_equal(st.fstar[fl], mv.fstar[fl])
    assert np.array_equal(st.rho[fl], mv.rho[fl])


def test_rotating_ellipse_geometry():
    """A spinning ellipse: after t steps at omega its solid set is the static
    raster at inclination alpha + omega t."""
    om = 0.02
    mv = MovingEmulator(Case(wing_case(True, om=om, dof="rotation")))
    mv.initialize()
    for _ in range(25):
        mv.step()
    o = mv.obs[0]
    assert o["angle"] == pytest.approx(np.pi / 6 + 25 * om)
    turned = Case(wing_case(False, incl=float(np.degrees(o["angle"]))))
    assert abs(int((mv.dsolid > 0).sum()) - int(turned.solid.sum())) <= 4
    assert (mv.dsolid.reshape(turned.solid.shape) > 0)[turned.solid].mean() > 0.95


def test_resting_moving_disk_equals_static_disk():
    """A moving obstacle that does not move: the run-time links reproduce the
    static link records bit for bit."""
    st = FusedEmulator(Case(disk_case(False)))
    mv = MovingEmulator(Case(disk_case(True)))
    st.initialize()
    mv.initialize()
    for _ in range(60):
        st.step()
        mv.step()
    fl = ~st.solid
    assert np.array_equal(st.fstar[fl], mv.fstar[fl])
    assert np.array_equal(st.rho[fl], mv.rho[fl])


def test_translating_disk_geometry():
    mv = MovingEmulator(Case(disk_case(True, v=(0.3, 0.1))))
    mv.initialize()
    n0 = int((mv.dsolid > 0).sum())
    for _ in range(20):
        mv.step()
    o = mv.obs[0]
    assert o["cx"] == pytest.approx(14 + 20 * 0.3) and o["cy"] == pytest.approx(16 + 20 * 0.1)
    # the solid set follows the disk and keeps its size up to the lattice
    X, Y = np.divmod(np.arange(mv.n), mv.case.ny)
    inside = (X - o["cx"]) ** 2 + (Y - o["cy"]) ** 2 <= o["r"] ** 2
    assert np.array_equal(mv.dsolid > 0, inside)
    assert abs(int(inside.sum()) - n0) <= 8
    # classes: solid 2, its fluid neighbours 4
    assert np.all(mv.cls[inside] == 2)
    assert np.all(np.isfinite(mv.fstar[~inside]))


def test_motion_dict_validation_messages():
    """solid_motion_dict errors as obstacle.py:478-538 words them."""
    c = disk_case(True)
    c["obstacle_dict"]["disk"]["solid_motion_dict"]["type"] = "spinning"
    with pytest.raises(ValueError, match="Unsupported motion type: spinning in obstacle: disk"):
        Case(c)
    c = disk_case(True)
    c["obstacle_dict"]["disk"]["solid_motion_dict"]["degree_of_freedom"] = "all"
    with pytest.raises(ValueError, match="Unsupported degree of freedom: all in obstacle: disk"):
        Case(c)
    c = disk_case(True)
    del c["obstacle_dict"]["disk"]["solid_motion_dict"]["linear_velocity"]
    with pytest.raises(ValueError, match="linear_velocity missing in solid_motion_dict: disk"):
        Case(c)
    c = disk_case(True)
    c["obstacle_dict"]["options"]["move_obstacles"] = "yes"
    with pytest.raises(ValueError, match="move_obstacles must be bool"):
        Case(c)


def test_moving_ellipse_parameters():
    case = Case(wing_case(True, kind="calculated", dof="both", density=2.0))
    o = case.moving[0]
    assert o.type == "ellipse" and o.semi_axes == (6.0, 2.5)
    assert o.mass == pytest.approx(np.pi * 6.0 * 2.5 * 2.0)
    assert o.moment_of_inertia == pytest.approx(o.mass * (36.0 + 6.25) / 4)
    assert not case.solid.any()


def test_moving_obstacle_parameters():
    case = Case(disk_case(True, kind="calculated", dof="rotation", density=2.0))
    o = case.moving[0]
    assert o.calculated and o.rotation_allowed and not o.translation_allowed
    assert o.mass == pytest.approx(np.pi * 16.0 * 2.0)
    assert o.moment_of_inertia == pytest.approx(o.mass * 16.0 / 2)
    # a moving obstacle is not part of the static solid: the device places it
    assert not case.solid.any()
    static = Case(disk_case(False))
    assert static.solid.sum() > 0 and not static.moving
