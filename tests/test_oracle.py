"""The oracle (CPU restatement) against the reference's own RNG outputs and against
known answers derived from the reference formulas. CPU only."""
import json
import math
import os

import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "dsfmt_random_golden.json")


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def small_params(**kw):
    p = S.base_params(2, 0, [20.0, 20.0])
    p.update(kw)
    return p


def make(O, p, cap=64, seed=1, threads=0):
    return O.Oracle(p, cap, seed, threads=threads)


def test_dsfmt_and_random_functions_match_reference(oracle_lib, golden):
    o = make(oracle_lib, small_params())
    for s, rec in golden["seeds"].items():
        for kind in ("close_open", "open_open", "uniform", "normal"):
            o.rng_seed(int(s))
            np.testing.assert_array_equal(o.rng(kind, len(rec[kind])), np.array(rec[kind]))
        o.rng_seed(int(s))
        np.testing.assert_array_equal(o.on_dsphere(2, len(rec["on_dsphere2_then3"]["d2"])),
                                      np.array(rec["on_dsphere2_then3"]["d2"]))
        np.testing.assert_array_equal(o.on_dsphere(3, len(rec["on_dsphere2_then3"]["d3"])),
                                      np.array(rec["on_dsphere2_then3"]["d3"]))


def test_division_draw_sequence_matches_reference(oracle_lib, golden):
    """Axis, axis, two cycle lengths, one apoptosis test: the per-division draw order of
    CIL.cu:392-424 followed by CIL.cu:636."""
    o = make(oracle_lib, small_params())
    for s, rec in golden["seeds"].items():
        o.rng_seed(int(s))
        for row in rec["division_sequence"]:
            a = o.on_dsphere(2, 1)[0]
            b = o.on_dsphere(2, 1)[0]
            n1 = 1.0 + 0.1 * o.rng("normal", 1)[0]
            n2 = 1.0 + 0.1 * o.rng("normal", 1)[0]
            u = o.rng("close_open", 1)[0] * 1.0
            assert [a[0], a[1], b[0], b[1], n1, n2, u] == row


def two_cells(p, r, sig=1.0, D=2):
    """Cell 0 at the origin side, cell 1 placed so that only back elements interact at r."""
    L = p["box"][0]
    pos = np.zeros((2, 2, D))
    pos[0, 0, 0], pos[0, 1, 0] = L / 2, L / 2 - 3.0
    pos[1, 0, 0], pos[1, 1, 0] = L / 2 + r, L / 2 + r + 3.0
    for c in range(2):
        for j in range(2):
            pos[c, j, 1] = L / 2
    return pos, np.full((2, 2), sig)


@pytest.mark.parametrize("law,r,expect", [
    (0, 1.0, 24.0),                      # WCA at r = sigma: 24 eps (2 - 1) / sigma
    (0, 2 ** (1 / 6) * 1.0000001, 0.0),  # beyond the cutoff
    (1, 0.5, 5.0 * 0.25),                # soft-core eps (1 - r/rc)^2
    (1, 1.0, 0.0),
    (2, 0.9, 100.0 * 0.1 ** 1.5),        # Hertz E delta^1.5
])
def test_pair_force_known_answers(oracle_lib, law, r, expect):
    eps = {0: 1.0, 1: 5.0, 2: 100.0}[law]
    rcs = {0: 2 ** (1 / 6), 1: 1.0, 2: 1.0}[law]
    p = small_params(force_law=law, epsilon=eps, rcut_scale=rcs, noise_D=0.0, motility=[0.0, 0.0],
                     kappa=0.0)
    o = make(oracle_lib, p)
    pos, sig = two_cells(p, r)
    o.set_state(pos, sig, np.zeros(2, np.int32), np.full(2, S.NEVER, np.int32))
    f = o.compute_forces()
    # repulsion pushes the back element of cell 0 to -x and of cell 1 to +x
    assert f[0, 0, 0] == pytest.approx(-expect, rel=1e-12, abs=1e-300)
    assert f[1, 0, 0] == pytest.approx(expect, rel=1e-12, abs=1e-300)
    assert np.all(f[:, 1] == 0.0)


def test_spring_and_motility(oracle_lib):
    p = small_params(noise_D=0.0, motility=[0.25, 1.0], kappa=10.0, rest0=0.5)
    o = make(oracle_lib, p)
    pos = np.array([[[5.0, 5.0], [5.8, 5.0]]])  # stretched by 0.3 along +x
    o.set_state(pos, np.ones((1, 2)), np.zeros(1, np.int32), np.full(1, S.NEVER, np.int32))
    f = o.compute_forces()
    assert f[0, 0, 0] == pytest.approx(10.0 * 0.3 - 0.25)
    assert f[0, 1, 0] == pytest.approx(-10.0 * 0.3 + 1.0)
    assert f[0, 0, 1] == 0.0 and f[0, 1, 1] == 0.0


@pytest.mark.parametrize("sep,cil", [(0.7, 0), (1.05, 0), (1.05, 1), (0.3, 1)])
def test_fene_bond_known_answers(oracle_lib, sep, cil):
    """binaryCellForce (MD.cu:525-598) for a crawling cell, worked by hand: r2max = max(RMAX^2,
    larger diameter); push spring kappa_push |r^2 - r2max ratio| below r2max ratio, FENE
    -kappa / (1 - q^2), q = (r^2 - r2max ratio) / (r2max (1 - ratio)), above; the bond acts twice;
    motility along rij, scaled by rss / r without CIL."""
    kappa, kpush, ratio, rmax = 0.2, 0.5, 0.5, 1.2
    p = small_params(noise_D=0.0, motility=[0.25, 1.0], intra_law=1, cil=cil, fene_kappa=kappa,
                     fene_kappa_push=kpush, fene_spring_ratio=ratio, fene_rmax=rmax)
    o = make(oracle_lib, p)
    pos = np.array([[[5.0, 5.0], [5.0 + sep * 0.8, 5.0 + sep * 0.6]]])
    sig = np.array([[1.3, 0.9]])
    o.set_state(pos, sig, np.zeros(1, np.int32), np.full(1, S.NEVER, np.int32))
    f = o.compute_forces()
    rij = pos[0, 1] - pos[0, 0]
    r2 = float(rij @ rij)
    r2max = max(rmax * rmax, 1.3)
    if r2 <= r2max * ratio:
        spring = kpush * abs(r2 - r2max * ratio)
        assert spring > 0.0  # pushes the elements apart
    else:
        q = (r2 - r2max * ratio) / (r2max * (1.0 - ratio))
        spring = -kappa / (1.0 - q * q)
    rss = math.sqrt(rmax * rmax * (1.0 - 2.0 / 1.25 * kappa))  # alpha = 2, beta = 0.25 + 1
    nij = rij if cil else rij * (rss / math.sqrt(r2))
    np.testing.assert_allclose(f[0, 0], -(0.25 * nij + 2.0 * spring * rij), rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(f[0, 1], 1.0 * nij + 2.0 * spring * rij, rtol=1e-14, atol=1e-15)


def cell_machine_params(**kw):
    """Two-element cells with the reference's bond and its crawling/dividing states; spans exact
    (sigma 0): division 30 steps, migration 50."""
    p = small_params(noise_D=0.0, motility=[0.0, 1.0], intra_law=1, cil=1, fene_kappa=0.2, fene_kappa_push=0.5,
                     fene_spring_ratio=0.5, fene_rmax=1.2, fene_rmax_division=1.6, divide=1, dt=1e-3,
                     div_tau_mu=0.03, div_tau_sigma=0.0, mig_tau_mu=0.05, mig_tau_sigma=0.0,
                     growth_k0=[0.0, 0.0], growth_k1=[1.0, 1.0], growth_k2=[0.0, 0.0], div_r0=0.25,
                     div_rmin=1.05, sigma_core=[1.0, 0.9])
    p.update(kw)
    return p


def test_cell_state_machine_transitions(oracle_lib):
    """calculDivisions (CIL.cu:369-455) for the reference's two-element cells, worked by hand on
    three isolated cells after one step: a crawling cell whose time ends starts dividing
    (time += 30); a dividing cell whose elements are Rmin apart divides (a daughter appended,
    both crawling, both born now, the daughter's time now + 50 and the mother's own + 50, the
    elements 2 R0 apart, the diameters reset to SIGMA_CORE); a dividing cell short of Rmin whose
    time ends fails (crawling, time += 50, elements 2 R0 apart)."""
    p = cell_machine_params()
    o = make(oracle_lib, p)
    pos = np.array([[[3.0, 3.0], [3.9, 3.0]],     # crawling, time ends
                    [[10.0, 10.0], [11.3, 10.0]],  # dividing, 1.3 apart
                    [[16.0, 16.0], [16.9, 16.0]]])  # dividing, 0.9 apart, time ends
    sig = np.array([[1.0, 1.0], [1.1, 1.0], [1.0, 1.0]])
    o.set_state(pos, sig, np.zeros(3, np.int32), np.array([1, 500, 1], np.int32), cell_state=[1, 0, 0])
    assert o.step(1) == 0
    s = o.state()
    assert o.ncells == 4
    np.testing.assert_array_equal(s["cell_state"], [0, 1, 1, 1])
    np.testing.assert_array_equal(s["tswitch"], [1 + 30, 500 + 50, 1 + 50, 1 + 50])
    np.testing.assert_array_equal(s["t0"], [0, 1, 0, 1])
    for c in (1, 2, 3):
        d = s["pos"][c, 1] - s["pos"][c, 0]
        assert np.sqrt(d @ d) == pytest.approx(0.5, abs=1e-12)
    np.testing.assert_array_equal(s["sigma"][1], [1.0, 0.9])
    np.testing.assert_array_equal(s["sigma"][3], [1.0, 0.9])
    ev = o.events()
    assert sorted(ev[:, 1].tolist()) == [0, 2, 3]


def test_dividing_bond_known_answer(oracle_lib):
    """binaryCellForce (MD.cu:545-567) for a dividing cell: r2max from RMAX_DIVISION, the growth
    activity -k0 feneDivMax + k1 + k2 r^4 along rij (no rss scaling), the bond acting once."""
    p = cell_machine_params(growth_k0=[0.3, 0.1], growth_k1=[0.2, 0.7], growth_k2=[0.05, 0.02], divide=0)
    o = make(oracle_lib, p)
    pos = np.array([[[5.0, 5.0], [5.0 + 0.8 * 1.1, 5.0 + 0.6 * 1.1]]])
    o.set_state(pos, np.ones((1, 2)), np.zeros(1, np.int32), np.full(1, S.NEVER, np.int32), cell_state=[0])
    f = o.compute_forces()
    rij = pos[0, 1] - pos[0, 0]
    r2 = float(rij @ rij)
    r2max = 1.6 * 1.6
    lim = 0.5 * r2max
    spring = 0.5 * abs(r2 - lim) if r2 <= lim else -0.2 / (1 - ((r2 - lim) / (0.5 * r2max)) ** 2)
    fdm = -0.2 / (1 - (1.05 * 1.05 / r2max) ** 2)
    act = [-0.3 * fdm + 0.2 + 0.05 * r2 * r2, -0.1 * fdm + 0.7 + 0.02 * r2 * r2]
    np.testing.assert_allclose(f[0, 0], -(act[0] * rij + spring * rij), rtol=1e-14)
    np.testing.assert_allclose(f[0, 1], act[1] * rij + spring * rij, rtol=1e-14)


def test_binning_formula_known_answers(oracle_lib):
    """min((int)((r * (1/L)) * Ns), Ns-1) with Ns = (int)(L / (w + 1e-8 min L)), ids
    ls0 * Ns1 + ls1 (Utils.hpp:872-876, 990, 1020-1022)."""
    p = small_params(box=[10.0, 6.0, 0.0])
    o = make(oracle_lib, p, cap=4)
    pos = np.array([[[0.0, 0.0], [9.999999, 5.999999]], [[2.0, 2.0], [4.99, 0.1]]])
    o.set_state(pos, np.ones((2, 2)), np.zeros(2, np.int32), np.full(2, S.NEVER, np.int32))
    # (int)(10/2.00000006) = 4 but (int)(6/2.00000006) = 2 < 3: the grid collapses to one
    # bin and every axis reports 1 (Utils.hpp:897-901)
    ns, head, lst = o.bin_elements(2.0)
    assert list(ns[:2]) == [1, 1]
    assert len(head) == 1
    ns, head, lst = o.bin_elements(1.9)
    assert list(ns[:2]) == [5, 3]
    bins = oracle_lib.bins_as_sets(head, lst)
    expect = {0: 0, 1: 4 * 3 + 2, 2: 1 * 3 + 1, 3: 2 * 3 + 0}
    for e, b in expect.items():
        assert e in bins[b]


def test_newton_third_law_and_parallel_variant(oracle_lib):
    p, st = S.config1(256, seed=3)
    p.update(noise_D=0.0, motility=[0.0, 0.0], force_law=1, epsilon=5.0, rcut_scale=1.0)
    o = make(oracle_lib, p, cap=256)
    o.set_state(**st)
    f = o.compute_forces()
    scale = np.abs(f).max()
    assert np.abs(f.sum(axis=(0, 1))).max() < 1e-12 * scale * 512
    o8 = make(oracle_lib, p, cap=256, threads=4)
    o8.set_state(**st)
    f8 = o8.compute_forces()
    assert np.abs(f8 - f).max() <= 1e-13 * scale


def test_apoptosis_replay_matches_sequential_swap_remove(oracle_lib):
    """The oracle's apoptosis events equal an independent replay of CIL.cu:627-649 on the
    same dSFMT stream (noise draws first, then one test per slot with re-test after a
    swap-with-last removal)."""
    p = small_params(noise_D=0.0, apop_rate=2000.0, dt=1e-4)  # 0.2 per step
    n = 40
    rng = np.random.default_rng(0)
    pos = rng.uniform(0, 20, size=(n, 2, 2))
    o = make(oracle_lib, p, cap=n, seed=99)
    o.set_state(pos, np.ones((n, 2)), np.zeros(n, np.int32), np.full(n, S.NEVER, np.int32))
    o.step(3)
    ev = o.events()
    ref = make(oracle_lib, p, cap=n, seed=99)
    slots = list(range(n))
    expect = []
    for ts in range(1, 4):
        i = 0
        while i < len(slots):
            u = ref.rng("close_open", 1)[0]
            if u <= 2000.0 * 1e-4:
                last = len(slots) - 1
                expect.append((ts, 1, i, last))
                slots[i] = slots[last]
                slots.pop()
            else:
                i += 1
    assert [tuple(e) for e in ev] == expect
    assert o.ncells == len(slots)


def test_division_replay(oracle_lib):
    """Due cells divide in slot order, daughters are appended, both get new cycles drawn
    daughter-first (CIL.cu:392-424, MD.cuh:434-436)."""
    p = small_params(noise_D=0.0, divide=1, dt=1e-3, div_tau_mu=0.01, div_tau_sigma=0.002)
    n = 6
    rng = np.random.default_rng(1)
    pos = rng.uniform(2, 18, size=(n, 2, 2))
    tsw = np.array([1, 3, 1, 5, 2, 1], np.int32)
    o = make(oracle_lib, p, cap=64, seed=5)
    o.set_state(pos, np.ones((n, 2)), np.zeros(n, np.int32), tsw)
    o.step(4)
    ev = o.events()
    ref = make(oracle_lib, p, cap=64, seed=5)
    t = list(tsw)
    expect = []
    for ts in range(1, 5):
        n0 = len(t)
        for i in range(n0):
            if t[i] != ts:
                continue
            k = len(t)
            ref.on_dsphere(2, 2)
            sd = max(int(math.floor(ref.rng("normal", 1)[0] * 0.002 / 1e-3 + 0.01 / 1e-3 + 0.5)), 1)
            sm = max(int(math.floor(ref.rng("normal", 1)[0] * 0.002 / 1e-3 + 0.01 / 1e-3 + 0.5)), 1)
            t.append(ts + sd)
            t[i] = ts + sm
            expect.append((ts, 0, i, k))
    assert [tuple(e) for e in ev] == expect
    st = o.state()
    assert list(st["tswitch"]) == t


def test_heun_is_two_half_euler_steps(oracle_lib):
    """Without noise and events, a StochasticHeun step of dt (CIL.cu:1028-1050) is two Euler
    steps of dt/2: bit for bit."""
    from cil_cuda_gb300 import synthetic as S
    p = S.growth_params(box=40.0, dt=1e-3, divide=0, apop_rate=0.0, noise_D=0.0)
    st = S.disk_colony(200, p, seed=3)
    a = oracle_lib.Oracle(p, 800, 5, integrator=1)
    a.set_state(**st)
    a.step(50)
    q = dict(p)
    q["dt"] = 0.5e-3
    b = oracle_lib.Oracle(q, 800, 5)
    b.set_state(**st)
    b.step(100)
    np.testing.assert_array_equal(a.state()["pos"], b.state()["pos"])
