"""CUDA path against the oracle, through the C ABI.

Tolerances (FP64, oracle mode = the reference's dSFMT stream uploaded):
* bin contents: identical sets per bin (bit-exact integer work)
* per-step forces: max_i |F_gpu - F_oracle| <= 1e-12 * max_i |F_oracle| (norm-wise; the
  two sides sum the same pair forces in different orders)
* 100-step trajectories: max |x_gpu - x_oracle| (minimum image) <= 1e-9
* division / apoptosis: identical cell counts, birth steps and division steps
* mixed precision forces: norm-wise relative error <= 2e-5 against the FP64 oracle
* mixed precision 100-step trajectories (FP32 forces, FP64 positions, local coordinates
  re-anchored on the FP64 positions every 32 steps): max |x - x_oracle| <= 1e-5
"""
import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-12
TRAJ_TOL = 1e-9
MIXED_TOL = 2e-5
MIXED_TRAJ_TOL = 1e-5


def minimage(a, b, p):
    d = np.asarray(a) - np.asarray(b)
    for k in range(p["dim"]):
        if p["periodic"][k]:
            L = p["box"][k]
            d[..., k] -= np.round(d[..., k] / L) * L
    return d


def engine(G, p, cap, **kw):
    return G.Engine([p], [cap], **kw)


@pytest.fixture(scope="module")
def lj(gpu_lib):
    p, st = S.config1(1024, seed=7)
    st = S.relax(p, st)
    return p, st


@pytest.fixture(scope="module")
def growth(gpu_lib):
    p = S.growth_params(box=120.0)
    st = S.disk_colony(2500, p, seed=11)
    return p, st


@pytest.fixture(scope="module")
def sc(gpu_lib):
    """The soft-core cubic well: a dense disk, so pairs sit in the core and in the well."""
    p = S.sc_params(box=90.0)
    st = S.disk_colony(1500, p, seed=13)
    return p, st


@pytest.fixture(scope="module")
def fene(gpu_lib):
    """Two-element cells held by the reference's FENE / push bond, soft-core contacts."""
    p = S.fene_params(box=90.0)
    st = S.disk_colony(2000, p, seed=4)
    return p, st


@pytest.fixture(scope="module")
def channel(gpu_lib):
    p = S.channel_params(lxy=40.0, height=10.0)
    st = S.channel_colony(1500, p, seed=5)
    return p, st


def bins_gpu(G, p, st, width):
    eng = engine(G, p, len(st["sigma"]), bin_width=width)
    eng.upload(0, **st)
    ns, start, elems = eng.bins(0)
    eng.close()
    return ns, start, elems


@pytest.mark.parametrize("width", [1.8, 2.6, 5.0])
def test_bin_contents_match_oracle_2d(gpu_lib, oracle_lib, lj, width):
    p, st = lj
    ns, start, elems = bins_gpu(gpu_lib, p, st, width)
    o = oracle_lib.Oracle(p, len(st["sigma"]), 1)
    o.set_state(**st)
    ons, head, lst = o.bin_elements(width)
    assert list(ns) == list(ons)
    ref = oracle_lib.bins_as_sets(head, lst)
    assert len(start) == len(ref) + 1
    for b, s in enumerate(ref):
        got = elems[start[b]:start[b + 1]]
        assert set(got.tolist()) == s
        assert np.all(np.diff(got) > 0)  # ascending element ids within a bin


def test_bin_contents_match_oracle_3d_walls(gpu_lib, oracle_lib, channel):
    p, st = channel
    ns, start, elems = bins_gpu(gpu_lib, p, st, 1.3)
    o = oracle_lib.Oracle(p, len(st["sigma"]), 1)
    o.set_state(**st)
    ons, head, lst = o.bin_elements(1.3)
    assert list(ns) == list(ons)
    for b, s in enumerate(oracle_lib.bins_as_sets(head, lst)):
        assert set(elems[start[b]:start[b + 1]].tolist()) == s


def test_single_bin_collapse(gpu_lib, oracle_lib):
    p, st = S.config1(12, seed=1, phi=0.3)
    ns, start, elems = bins_gpu(gpu_lib, p, st, 4.0)
    assert list(ns[:2]) == [1, 1] and len(start) == 2
    assert sorted(elems.tolist()) == list(range(24))


def forces_pair(G, O, p, st, seed=42, **kw):
    n = len(st["sigma"])
    eng = engine(G, p, n, rng=G.RNG_DSFMT, seed=seed, **kw)
    eng.upload(0, **st)
    fg = eng.forces(0)
    eng.close()
    o = O.Oracle(p, n, seed)
    o.set_state(**st)
    fo = o.compute_forces()
    return fg, fo


def lj_attraction(lj, shifted=1):
    """The LJ law with the reference's ATTRACTION ON: cutoff 2.5 sigma_ij, SHIFT FORCE."""
    p, st = lj
    return dict(p, rcut_scale=2.5, force_shifted=shifted), st


@pytest.mark.parametrize("case", ["lj", "growth", "channel", "lj_cellnoise", "sc", "sc_shifted", "lj_attr",
                                  "lj_attr_plain", "fene", "fene_cil"])
def test_forces_match_oracle(gpu_lib, oracle_lib, lj, growth, channel, sc, fene, case):
    p, st = {"lj": lj, "growth": growth, "channel": channel, "lj_cellnoise": lj,
             "sc": sc, "sc_shifted": sc, "lj_attr": lj_attraction(lj), "lj_attr_plain": lj_attraction(lj, 0),
             "fene": fene, "fene_cil": (dict(fene[0], cil=1), fene[1])}[case]
    if case == "lj_cellnoise":
        p = dict(p, noise_per_cell=1)
    if case == "sc_shifted":
        p = dict(p, force_shifted=1)
    fg, fo = forces_pair(gpu_lib, oracle_lib, p, st)
    assert np.isfinite(fo).all()
    scale = np.abs(fo).max()
    err = np.abs(fg - fo).max()
    assert err <= FORCE_TOL * scale, (err, scale)


def channel_variants():
    """The 3D walled channel with the other laws: the cubic well, and the FENE / push bond (the
    colony placed at its steady-state length), divisions off."""
    import cil_cuda_gb300 as CG
    base = S.channel_params(lxy=40.0, height=10.0, divide=0)
    sc = dict(base, force_law=CG.FORCE_SC, epsilon=10.0, well_epsilon=0.5, well_sigma=0.3, rcut_scale=1.0)
    fp = S.fene_params(box=40.0)
    fene = dict(base, intra_law=fp["intra_law"], cil=0, fene_kappa=fp["fene_kappa"],
                fene_kappa_push=fp["fene_kappa_push"], fene_spring_ratio=fp["fene_spring_ratio"],
                fene_rmax=fp["fene_rmax"], motility=fp["motility"], zeta=fp["zeta"], rest0=fp["rest0"],
                rest1=fp["rest0"])
    lja = dict(base, force_law=CG.FORCE_LJ_WCA, epsilon=1.0, rcut_scale=2.5, force_shifted=1)
    return {"sc3": (sc, S.channel_colony(1500, sc, seed=6)), "fene3": (fene, S.channel_colony(1500, fene, seed=7)),
            "lj_attr3": (lja, S.channel_colony(1500, lja, seed=8))}


@pytest.mark.parametrize("case", ["sc3", "fene3", "lj_attr3"])
def test_forces_3d_other_laws(gpu_lib, oracle_lib, case):
    p, st = channel_variants()[case]
    fg, fo = forces_pair(gpu_lib, oracle_lib, p, st)
    scale = np.abs(fo).max()
    assert np.isfinite(fo).all() and np.abs(fg - fo).max() <= FORCE_TOL * scale
    fg, fo = forces_pair(gpu_lib, oracle_lib, dict(p, noise_D=0.0), st, precision=gpu_lib.PREC_MIXED)
    assert np.abs(fg - fo).max() / np.abs(fo).max() <= MIXED_TOL


def test_mixed_precision_forces(gpu_lib, oracle_lib, lj, growth, sc, fene):
    for p, st in (lj, growth, sc, (dict(sc[0], force_shifted=1), sc[1]), lj_attraction(lj), lj_attraction(lj, 0),
                  fene, (dict(fene[0], cil=1), fene[1])):
        p = dict(p, noise_D=0.0)
        fg, fo = forces_pair(gpu_lib, oracle_lib, p, st, precision=gpu_lib.PREC_MIXED)
        err = np.abs(fg - fo).max() / np.abs(fo).max()
        assert err <= MIXED_TOL, err


def run_pair(G, O, p, st, nsteps, seed=3, cap=None, **kw):
    n = len(st["sigma"])
    cap = cap or n
    eng = engine(G, p, cap, rng=G.RNG_DSFMT, seed=seed, **kw)
    eng.upload(0, **st)
    eng.step(nsteps)
    g = eng.download(0)
    eng.close()
    o = O.Oracle(p, cap, seed)
    o.set_state(**st)
    rc = o.step(nsteps)
    return g, o.state(), rc, o


def test_trajectory_100_steps(gpu_lib, oracle_lib, lj):
    p, st = lj
    g, s, rc, _ = run_pair(gpu_lib, oracle_lib, p, st, 100)
    assert rc == 0
    assert g["ncells"] == len(s["sigma"])
    err = np.abs(minimage(g["pos"], s["pos"], p)).max()
    assert err <= TRAJ_TOL, err
    verr = np.abs(g["vel"] - s["vel"]).max() / np.abs(s["vel"]).max()
    assert verr <= 1e-9


def test_trajectory_100_steps_3d_channel(gpu_lib, oracle_lib, channel):
    p, st = channel
    g, s, rc, _ = run_pair(gpu_lib, oracle_lib, p, st, 100, cap=2 * len(st["sigma"]))
    assert rc == 0
    err = np.abs(minimage(g["pos"], s["pos"], p)).max()
    assert err <= TRAJ_TOL, err


def test_trajectory_100_steps_soft_core_well(gpu_lib, oracle_lib, sc):
    p, st = sc
    g, s, rc, _ = run_pair(gpu_lib, oracle_lib, p, st, 100, cap=2 * len(st["sigma"]))
    assert rc == 0
    assert g["ncells"] == len(s["sigma"])
    err = np.abs(minimage(g["pos"], s["pos"], p)).max()
    assert err <= TRAJ_TOL, err


def test_trajectory_100_steps_lj_attraction(gpu_lib, oracle_lib, lj):
    p, st = lj_attraction(lj)
    g, s, rc, _ = run_pair(gpu_lib, oracle_lib, p, st, 100)
    assert rc == 0
    err = np.abs(minimage(g["pos"], s["pos"], p)).max()
    assert err <= TRAJ_TOL, err


def test_trajectory_100_steps_fene_bond(gpu_lib, oracle_lib, fene):
    p, st = fene
    g, s, rc, _ = run_pair(gpu_lib, oracle_lib, p, st, 100)
    assert rc == 0
    err = np.abs(minimage(g["pos"], s["pos"], p)).max()
    assert err <= TRAJ_TOL, err


def test_soft_core_well_events_fp64(gpu_lib, oracle_lib):
    """The cubic well with division and apoptosis over 300 steps: events exact, FP64 positions."""
    p = S.sc_params(box=80.0, dt=1e-4, divide=1, div_tau_mu=0.05, div_tau_sigma=0.005, apop_rate=2.0)
    st = S.disk_colony(1200, p, seed=9)
    g, s, rc, o = run_pair(gpu_lib, oracle_lib, p, st, 300, seed=11, cap=4 * len(st["sigma"]))
    assert rc == 0
    ev = o.events()
    assert (ev[:, 1] == 0).sum() > 100 and (ev[:, 1] == 1).sum() > 5
    assert g["ncells"] == len(s["sigma"])
    np.testing.assert_array_equal(g["t0"], s["t0"])
    np.testing.assert_array_equal(g["tswitch"], s["tswitch"])
    err = np.abs(minimage(g["pos"], s["pos"], p)).max()
    assert err <= TRAJ_TOL, err


@pytest.mark.parametrize("case", ["lj", "growth", "channel", "sc", "lj_attr", "fene"])
def test_mixed_precision_trajectory(gpu_lib, oracle_lib, lj, growth, channel, sc, fene, case):
    p, st = {"lj": lj, "growth": growth, "channel": channel, "sc": sc, "lj_attr": lj_attraction(lj), "fene": fene}[case]
    g, s, rc, _ = run_pair(gpu_lib, oracle_lib, p, st, 100, cap=2 * len(st["sigma"]),
                           precision=gpu_lib.PREC_MIXED)
    assert rc == 0
    assert g["ncells"] == len(s["sigma"])
    np.testing.assert_array_equal(g["tswitch"], s["tswitch"])
    err = np.abs(minimage(g["pos"], s["pos"], p)).max()
    assert err <= MIXED_TRAJ_TOL, err


def test_division_and_apoptosis_events_exact(gpu_lib, oracle_lib):
    p = S.growth_params(box=80.0, dt=1e-3, div_tau_mu=0.05, div_tau_sigma=0.01, apop_rate=1.0)
    st = S.disk_colony(400, p, seed=2)
    g, s, rc, o = run_pair(gpu_lib, oracle_lib, p, st, 120, seed=17, cap=4000)
    assert rc == 0
    ev = o.events()
    assert (ev[:, 1] == 0).sum() > 100 and (ev[:, 1] == 1).sum() > 5  # both kinds happened
    assert g["ncells"] == len(s["sigma"])
    np.testing.assert_array_equal(g["t0"], s["t0"])
    np.testing.assert_array_equal(g["tswitch"], s["tswitch"])
    np.testing.assert_array_equal(g["sigma"], s["sigma"])
    err = np.abs(minimage(g["pos"], s["pos"], p)).max()
    assert err <= TRAJ_TOL, err


def test_philox_mode_deterministic_and_growing(gpu_lib):
    p = S.growth_params(box=150.0, dt=1e-3, div_tau_mu=0.1, div_tau_sigma=0.01, apop_rate=0.5)
    st = S.disk_colony(1500, p, seed=4)
    outs = []
    for _ in range(2):
        eng = engine(gpu_lib, p, 20000, seed=123)
        eng.upload(0, **st)
        eng.step(150)
        outs.append(eng.download(0))
        ob = eng.observables(0)
        eng.close()
    a, b = outs
    assert a["ncells"] == b["ncells"] > 1500
    np.testing.assert_array_equal(a["pos"], b["pos"])
    np.testing.assert_array_equal(a["tswitch"], b["tswitch"])
    assert ob["ndiv_total"] > 0 and ob["ncells"] == a["ncells"]


def test_batched_colonies_equal_single(gpu_lib):
    """Colonies of uneven size stepped in one handle give the same states as separate
    handles (no noise, no events: a deterministic force field)."""
    ps, sts = [], []
    for i, n in enumerate((300, 1200, 700)):
        p = S.growth_params(box=0.0, noise_D=0.0, divide=0, apop_rate=0.0)
        p, st = S.square_colony(n, p, seed=i)
        ps.append(p)
        sts.append(st)
    eng = gpu_lib.Engine(ps, [len(s["sigma"]) for s in sts])
    for c, st in enumerate(sts):
        eng.upload(c, **st)
    eng.step(20)
    batched = [eng.download(c) for c in range(3)]
    eng.close()
    for c in range(3):
        e1 = engine(gpu_lib, ps[c], len(sts[c]["sigma"]))
        e1.upload(0, **sts[c])
        e1.step(20)
        single = e1.download(0)
        e1.close()
        np.testing.assert_array_equal(batched[c]["pos"], single["pos"])


@pytest.mark.parametrize("precision", [0, 1])
def test_batched_colonies_with_different_bonds(gpu_lib, precision):
    """One handle holding a colony with the linear spring and one with the reference's FENE /
    push bond (the bond is a per-colony parameter) gives each the state it has alone."""
    ps, sts = [], []
    for i, n in enumerate((500, 900)):
        p = S.growth_params(box=0.0, noise_D=0.0, divide=0, apop_rate=0.0)
        if i == 1:
            f = S.fene_params()
            p.update({k: f[k] for k in ("intra_law", "cil", "fene_kappa", "fene_kappa_push", "fene_spring_ratio",
                                        "fene_rmax", "motility", "zeta", "rest0", "rest1")})
        p, st = S.square_colony(n, p, seed=10 + i)
        ps.append(p)
        sts.append(st)
    eng = gpu_lib.Engine(ps, [len(s["sigma"]) for s in sts], precision=precision)
    for c, st in enumerate(sts):
        eng.upload(c, **st)
    eng.step(20)
    batched = [eng.download(c) for c in range(2)]
    eng.close()
    for c in range(2):
        e1 = engine(gpu_lib, ps[c], len(sts[c]["sigma"]), precision=precision)
        e1.upload(0, **sts[c])
        e1.step(20)
        single = e1.download(0)
        e1.close()
        if precision == 0:
            np.testing.assert_array_equal(batched[c]["pos"], single["pos"])
        else:  # the mixed kernel may sum a cell's FP32 pair terms in another order in a batch
            assert np.abs(minimage(batched[c]["pos"], single["pos"], ps[c])).max() <= 1e-6


def test_error_nan(gpu_lib):
    p = S.base_params(2, gpu_lib.FORCE_LJ_WCA, [10.0, 10.0], noise_D=0.0)
    pos = np.array([[[5.0, 5.0], [5.5, 5.0]], [[5.0, 5.0], [4.5, 5.0]]])  # coincident back elements
    eng = engine(gpu_lib, p, 2)
    eng.upload(0, pos, np.ones((2, 2)), np.zeros(2, np.int32), np.full(2, S.NEVER, np.int32))
    with pytest.raises(gpu_lib.CilError) as e:
        eng.step(1)
    assert e.value.status == 4
    eng.close()


def test_error_capacity_and_box(gpu_lib):
    p = S.growth_params(box=30.0, dt=1e-3)
    st = S.disk_colony(50, p, seed=1)
    st["tswitch"][:] = 1  # everyone divides at the first step
    eng = engine(gpu_lib, p, 60)
    eng.upload(0, **st)
    with pytest.raises(gpu_lib.CilError) as e:
        eng.step(1)
    assert e.value.status == 3
    bad = dict(st)
    bad["pos"] = st["pos"].copy()
    bad["pos"][0, 0, 0] = 31.0
    with pytest.raises(gpu_lib.CilError) as e:
        eng.upload(0, **bad)
    assert e.value.status == 5
    eng.close()


def test_refused_upload_changes_nothing_and_pinned_upload(gpu_lib):
    """cil_upload checks its input on the device before writing any of the colony's arrays: a
    refused upload (a position outside the box, a non-positive diameter) leaves the colony as it
    was, and stepping goes on; an upload from registered (pinned) host arrays gives the same
    state as one from ordinary arrays."""
    p = S.growth_params(box=30.0, dt=1e-3)
    st = S.disk_colony(50, p, seed=2)
    eng = engine(gpu_lib, p, 200)
    eng.upload(0, **st)
    eng.step(3)
    before = eng.download(0)
    bad_box = dict(st, pos=st["pos"].copy())
    bad_box["pos"][7, 1, 0] = -1e-9
    bad_sigma = dict(st, sigma=st["sigma"].copy())
    bad_sigma["sigma"][3, 0] = 0.0
    for bad, status in ((bad_box, 5), (bad_sigma, 1)):
        with pytest.raises(gpu_lib.CilError) as e:
            eng.upload(0, **bad)
        assert e.value.status == status
        after = eng.download(0)
        for k in ("pos", "sigma", "t0", "tswitch"):
            np.testing.assert_array_equal(after[k], before[k])
    eng.step(3)
    eng.close()
    outs = []
    for pin in (False, True):
        arrs = {"pos": np.ascontiguousarray(st["pos"], np.float64), "sigma": np.ascontiguousarray(st["sigma"], np.float64),
                "t0": np.ascontiguousarray(st["t0"], np.int32), "tswitch": np.ascontiguousarray(st["tswitch"], np.int32)}
        if pin:
            for v in arrs.values():
                gpu_lib.host_register(v)
        e2 = engine(gpu_lib, p, 200)
        e2.upload(0, **arrs)
        e2.step(5)
        outs.append(e2.download(0))
        e2.close()
        if pin:
            for v in arrs.values():
                gpu_lib.host_unregister(v)
    for k in ("pos", "sigma", "t0", "tswitch"):
        np.testing.assert_array_equal(outs[0][k], outs[1][k])
