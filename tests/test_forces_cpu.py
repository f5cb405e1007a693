"""Obstacle geometry fields and momentum-exchange forces on the CPU.

The product's geometry (pylabolt_gb300.obstacles.Geometry) against the
fields the reference's own ObstacleOperator built for the golden cases
(bit-exact); the oracle's force restatement against the reference's force
kernels applied to the golden populations; the product's force link sets,
summed over the same populations, against both."""
import numpy as np
import pytest

from _golden import golden_names, load_golden
from oracle import lbm_np
from pylabolt_gb300.config import Case
from pylabolt_gb300.lattice import CX, CY
from pylabolt_gb300.obstacles import Geometry, force_links

GEO_FIELDS = ["solid_id", "solid_boundary", "fluid_boundary", "surface_normals"]


def _times(d):
    return [0] + sorted(d["checkpoints"].tolist())


def _inner_mask(case):
    m = np.zeros((case.nx + 2, case.ny + 2), dtype=bool)
    m[1:-1, 1:-1] = True
    return m.ravel()


@pytest.mark.parametrize("name", golden_names())
def test_geometry_fields_match_reference(name):
    case_d, d = load_golden(name)
    case = Case(case_d)
    geo = Geometry(case)
    inner = _inner_mask(case)
    npad = (case.nx + 2) * (case.ny + 2)
    for f in GEO_FIELDS:
        mine = getattr(geo, f)
        mine = mine.reshape(npad, -1) if mine.ndim == 3 else mine.reshape(npad)
        assert np.array_equal(mine[inner], d["geo_" + f][inner]), f


@pytest.mark.parametrize("name", golden_names())
def test_oracle_forces_match_reference(name):
    case_d, d = load_golden(name)
    case = Case(case_d)
    ny = case.ny
    walls = [el for el in case.elements if el.wall]
    assert [el.name for el in walls] == d["wall_names"].tolist()
    for t in _times(d):
        if t == 0:       # the reference initialises pop = pop_new = f_eq(rho0, u0)
            fl = _inner_mask(case) & ~d["solid"]
            pop = np.zeros((fl.size, 9))
            pop[fl] = lbm_np.equilibrium(d["rho0"][fl], d["u0"][fl, 0], d["u0"][fl, 1])
            pn = pop
        else:
            pop, pn = d[f"pop_t{t}"], d[f"pop_new_t{t}"]
        for i, o in enumerate(case.obstacles):
            got = lbm_np.obstacle_force_torque(pop, pn, d["geo_solid"], d["geo_solid_id"],
                                               d["geo_fluid_boundary"], case.nx, ny, o.center,
                                               o.id, case.x_periodic, case.y_periodic)
            np.testing.assert_allclose(got, d[f"force_obstacles_t{t}"][i], rtol=1e-12, atol=1e-15)
        for j, el in enumerate(walls):
            nodes = (el.xs + 1) * (ny + 2) + el.ys + 1
            got = lbm_np.boundary_force(pop, pn, d["geo_solid"], nodes, el.out_list, el.inv_list)
            np.testing.assert_allclose(got, d[f"force_walls_t{t}"][j], rtol=1e-12, atol=1e-15)


def _sum_links(links, ngroups, pop, pop_new, ny):
    p = (links["node"] // ny + 1) * (ny + 2) + links["node"] % ny + 1
    ko, ki = links["k_out"].astype(int), links["k_in"].astype(int)
    fo, fi = pop[p, ko], pop_new[p, ki]
    vx = fo * CX[ko] - fi * CX[ki]
    vy = fo * CY[ko] - fi * CY[ki]
    out = np.zeros((ngroups, 3))
    np.add.at(out[:, 0], links["group"], vx)
    np.add.at(out[:, 1], links["group"], vy)
    np.add.at(out[:, 2], links["group"], links["rx"] * vy - links["ry"] * vx)
    return out


@pytest.mark.parametrize("name", golden_names())
def test_force_links_reproduce_reference_sums(name):
    case_d, d = load_golden(name)
    case = Case(case_d)
    links, obs, walls = force_links(case)
    assert walls == d["wall_names"].tolist() and obs == d["obstacle_names"].tolist()
    ng = len(obs) + len(walls)
    for t in _times(d):
        if t == 0:
            continue
        got = _sum_links(links, ng, d[f"pop_t{t}"], d[f"pop_new_t{t}"], case.ny)
        ref_o = d[f"force_obstacles_t{t}"]
        ref_w = d[f"force_walls_t{t}"]
        np.testing.assert_allclose(got[:len(obs)], ref_o, rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(got[len(obs):, :2], ref_w, rtol=1e-12, atol=1e-15)


def test_overlapping_fluid_boundaries_rejected():
    from pylabolt_gb300 import workloads
    c = workloads.cavity(40)
    c["obstacle_dict"]["a"] = {"type": "circle", "radius": 5.0, "center": [12, 20],
                               "density": 1.0, "static": True}
    c["obstacle_dict"]["b"] = {"type": "circle", "radius": 5.0, "center": [23, 20],
                               "density": 1.0, "static": True}
    with pytest.raises(ValueError, match="Fluid Boundary node overlap detected"):
        Geometry(Case(c))
