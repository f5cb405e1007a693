"""AA (in-place) population layout: index algebra and race freedom on the CPU.

Restates the addressing of the AA step kernel (step_aa_kernel /
special_link_aa in pylabolt_gb300/csrc/lbm_kernels.cuh) and of
``aa_post_index`` (lbm_internal.h), and checks on the link tables of the
golden cases that

* every access stays inside the population allocation;
* within one phase no thread reads a slot another thread writes, and no two
  threads write the same slot (the update is race-free in place);
* with any node update in place of the collision, the AA even / odd phases
  hand every node the same incoming populations as the two-buffer pull, and
  ``aa_post_index`` finds the same post-update populations.

The GPU tests check the real kernels against the reference fixtures.
"""
import ctypes

import numpy as np
import pytest

from _golden import golden_names, load_golden
from pylabolt_gb300 import capi
from pylabolt_gb300.config import Case
from pylabolt_gb300.geometry import build_links

CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])
INV = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6])


def aa_pitch(nx, eb):
    """Row pitch of the AA layout: 128-byte rows with a padding column."""
    align = 128 // eb
    return (nx + 1 + align - 1) // align * align


class Grid:
    def __init__(self, case, eb=8):
        self.nx, self.ny = nx, ny = case.nx, case.ny
        self.pitch = aa_pitch(nx, eb)
        self.plane = (ny + 2) * self.pitch
        solid, rec = build_links(case)
        self.rec = rec
        self.solid = solid.reshape(nx, ny).astype(bool)
        self.rec_of = {int(r["node"]): i for i, r in enumerate(rec)}
        xs, ys = np.nonzero(~self.solid)
        self.x, self.y = xs, ys
        self.ni = (ys + 1) * self.pitch + xs
        self.r = np.array([self.rec_of.get(int(x) * ny + int(y), -1) for x, y in zip(xs, ys)])

    def dev(self, inner):
        return (inner % self.ny + 1) * self.pitch + inner // self.ny

    def off(self, k):
        return CY[k] * self.pitch + CX[k]


def accesses(G, phase, nopull=False):
    """(reads, writes): lists of (flat index, node) pairs of one phase;
    flat index = k * plane + storage index, as the kernel forms it."""
    reads, writes = [], []
    odd = phase == 1
    for n, r in zip(G.ni, G.r):
        if not odd and (nopull or r < 0):
            reads += [(k * G.plane + n, n) for k in range(9)]
        elif odd and r < 0:
            reads += [(INV[k] * G.plane + n - G.off(k), n) for k in range(9)]
        else:
            reads.append((n, n))
            L = G.rec[r]
            for k in range(1, 9):
                t = L["type"][k]
                if t == capi.LINK_PULL:
                    s = G.dev(int(L["src"][k]))
                    reads.append((INV[k] * G.plane + s, n) if odd else (k * G.plane + s + G.off(k), n))
                elif t != capi.LINK_ZERO:
                    reads.append((k * G.plane + n, n) if odd else (INV[k] * G.plane + n - G.off(k), n))
        if odd:
            writes += [(k * G.plane + n + G.off(k), n) for k in range(9)]
        else:
            writes += [(INV[k] * G.plane + n, n) for k in range(9)]
    return reads, writes


AA_CASES = golden_names(zero_gradient=False)   # AA refuses zero_gradient edges


@pytest.mark.parametrize("name", AA_CASES)
@pytest.mark.parametrize("eb", [8, 4, 2])
def test_aa_accesses_in_bounds_and_race_free(name, eb):
    G = Grid(Case(load_golden(name)[0]), eb)
    lo, hi = -G.pitch, 9 * G.plane + G.pitch
    for phase, nopull in ((0, True), (0, False), (1, False)):
        reads, writes = accesses(G, phase, nopull)
        idx = np.array([i for i, _ in reads + writes])
        assert idx.min() >= lo and idx.max() < hi
        owner = {}
        for i, n in writes:
            assert owner.setdefault(i, n) == n, "two writers"
        for i, n in reads:
            assert owner.get(i, n) == n, "a slot read by one node is written by another"


def _update(fin, ni):
    """Stand-in node update: any deterministic map of the incoming values."""
    rot = np.roll(fin, 1, axis=0)
    return 0.5 * fin + 0.25 * rot + 1e-3 * (ni[None, :] % 97) + np.arange(9)[:, None]


def _incoming_ab(G, P, nopull):
    F = np.empty((9, G.ni.size))
    for j, (n, r) in enumerate(zip(G.ni, G.r)):
        for k in range(9):
            if nopull:
                F[k, j] = P[k, n]
            elif r < 0 or k == 0:
                F[k, j] = P[k, n - G.off(k)]
            else:
                t = G.rec[r]["type"][k]
                if t == capi.LINK_PULL:
                    F[k, j] = P[k, G.dev(int(G.rec[r]["src"][k]))]
                elif t == capi.LINK_ZERO:
                    F[k, j] = 0.0
                else:
                    F[k, j] = P[INV[k], n]   # the raw value a boundary rule transforms
    return F


def _incoming_aa(G, A, phase, nopull):
    base = G.pitch
    F = np.empty((9, G.ni.size))
    odd = phase == 1
    for j, (n, r) in enumerate(zip(G.ni, G.r)):
        for k in range(9):
            if not odd and (nopull or r < 0 or k == 0):
                i = k * G.plane + n
            elif odd and (r < 0 or k == 0):
                i = INV[k] * G.plane + n - G.off(k)
            else:
                t = G.rec[r]["type"][k]
                if t == capi.LINK_ZERO:
                    F[k, j] = 0.0
                    continue
                if t == capi.LINK_PULL:
                    s = G.dev(int(G.rec[r]["src"][k]))
                    i = INV[k] * G.plane + s if odd else k * G.plane + s + G.off(k)
                else:
                    i = k * G.plane + n if odd else INV[k] * G.plane + n - G.off(k)
            F[k, j] = A[base + i]
    return F


def aa_post_index(G, state, n, k):
    if state == 1:
        return INV[k] * G.plane + n
    if state == 2:
        return k * G.plane + n + G.off(k)
    return k * G.plane + n


@pytest.mark.parametrize("name", AA_CASES)
def test_aa_phases_match_two_buffer_pull(name):
    G = Grid(Case(load_golden(name)[0]), 8)
    rng = np.random.default_rng(7)
    P = np.zeros((9, G.plane))
    A = np.full(9 * G.plane + 2 * G.pitch, np.nan)   # unwritten slots poison the result
    init = rng.random((9, G.ni.size))
    P[:, G.ni] = init
    for k in range(9):
        A[G.pitch + k * G.plane + G.ni] = init[k]
    state = 0
    for step in range(7):
        nopull = step == 0
        phase = step % 2
        Fab = _incoming_ab(G, P, nopull)
        Faa = _incoming_aa(G, A, phase, nopull)
        assert np.array_equal(Fab, Faa), step
        post = _update(Fab, G.ni)
        P = np.zeros_like(P)
        P[:, G.ni] = post
        for k in range(9):
            if phase == 0:
                A[G.pitch + INV[k] * G.plane + G.ni] = post[k]
            else:
                A[G.pitch + k * G.plane + G.ni + G.off(k)] = post[k]
        state = 1 if phase == 0 else 2
        for k in range(9):
            got = A[G.pitch + np.array([aa_post_index(G, state, n, k) for n in G.ni])]
            assert np.array_equal(got, post[k])


def _cfg(case, layout):
    from pylabolt_gb300.lbm import make_config
    return make_config(case, "fp64", 0, layout)


def test_aa_rejects_zero_gradient(lbm_lib):
    """A zero_gradient boundary pulls populations that another fluid node
    overwrites in place: lbm_create refuses the AA layout before any device
    work."""
    case_d, _ = load_golden("channel_cylinder_abb")
    case_d["boundary_dict"]["outlet"]["fluid"] = {"type": "zero_gradient"}
    case = Case(case_d)
    solid, rec = build_links(case)
    h = ctypes.c_void_p()
    rc = lbm_lib.lbm_create(ctypes.byref(_cfg(case, "aa")), capi.ptr(solid), capi.ptr(rec), len(rec),
                            ctypes.byref(h))
    assert rc == capi.LBM_ERR_ARG
    assert "AA layout" in lbm_lib.lbm_last_error().decode()


def test_unknown_layout_rejected(lbm_lib):
    case = Case(load_golden("cavity_lid_first")[0])
    solid, rec = build_links(case)
    cfg = _cfg(case, "ab")
    cfg.layout = 5
    h = ctypes.c_void_p()
    rc = lbm_lib.lbm_create(ctypes.byref(cfg), capi.ptr(solid), capi.ptr(rec), len(rec), ctypes.byref(h))
    assert rc == capi.LBM_ERR_ARG and "population layout" in lbm_lib.lbm_last_error().decode()


def test_population_layout_key():
    d = load_golden("cavity_lid_first")[0]
    assert Case(d).population_layout == "ab"
    d["control_dict"]["population_layout"] = "aa"
    assert Case(d).population_layout == "aa"
    d["control_dict"]["population_layout"] = "abc"
    with pytest.raises(ValueError, match="population_layout"):
        Case(d)
