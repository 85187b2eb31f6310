"""Parity of the form the benchmark times, at the sizes it runs, against the FP64 oracle.

The headline number comes from the mixed-precision step with Verlet lists, the learned skin
scheduler, CUDA-graph replay and an autotuned list-kernel variant, in Philox mode. These tests
cover that form (and the plain form at the benchmark's first configuration) beyond the small
colonies of test_gpu_parity.py:

* ensemble statistics of the headline form, every list-kernel variant the autotuner can return,
  against the FP64 oracle over 16 seeds: cell count, mean cell area, MSD and VACF each within
  2 standard errors (z = |difference of the ensemble means| / SE of that difference, SEs from
  the 16-sample spreads as the reference's block errors, tools/utils.py:82-130);
* the fast-mode event samplers against their distributions with large samples: division
  times (randomTimeSpan, MD.cuh:434-436: max(Nint(N(mu, sigma) / dt), 1)) and apoptosis
  counts (each cell dies with probability rate dt per step, CIL.cu:627-649);
* observables in oracle mode equal to the oracle's (cell and event counts exact, mean area to
  1e-12, MSD and VACF to 1e-9: they carry the 1e-9 trajectory tolerance);
* the first benchmark configuration at its stated size (4096 cells, WCA, packing 0.8): bins
  exact, forces 1e-12, a 1000-step trajectory 1e-9;
* a 256k-cell colony: bins exact, FP64 forces 1e-12, mixed forces 2e-5 (norm-wise);
* batching in Philox mode with lists: every colony of a batch draws what it draws alone
  (colony-local random streams), so events are equal and positions agree to FP32 summation
  order.
"""
import math

import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

SEEDS = list(range(1, 17))
OBS = ("ncells", "mean_area", "msd", "vacf")


def minimage(a, b, p):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    for k in range(p["dim"]):
        if p["periodic"][k]:
            L = p["box"][k]
            d[..., k] -= np.round(d[..., k] / L) * L
    return d


def headline_engine(G, p, cap, seed, variant, **kw):
    """The benchmark's form: mixed precision, Philox, Verlet lists with the learned scheduler,
    graph-replayed steps, the given list-kernel variant."""
    from cil_cuda_gb300 import skin_scheduler as SS
    skin = SS.load()[2]
    eng = G.Engine([p], [cap], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=seed, skin=skin,
                   staging=variant[0], occupancy=variant[1], **kw)
    return eng


# ---------------------------------------------------------------- ensemble statistics

STAT_WARM, STAT_STEPS = 20, 300


def stat_case():
    p = S.growth_params(box=400.0, dt=1e-3, div_tau_mu=0.5, div_tau_sigma=0.1, apop_rate=0.5, noise_D=0.02)
    st = S.disk_colony(20000, p, seed=31)
    return p, st


def test_headline_form_statistics_within_two_standard_errors(gpu_lib, oracle_lib):
    from cil_cuda_gb300 import autotune as AT
    from cil_cuda_gb300 import skin_scheduler as SS
    from oracle import ensembles as E
    p, st = stat_case()
    cap = 40000
    ora = np.array(E.run_pool([(p, st, cap, s, STAT_WARM, STAT_STEPS) for s in SEEDS]))
    m_o, se_o = ora.mean(0), ora.std(0, ddof=1) / math.sqrt(len(SEEDS))
    assert m_o[0] > 1.1 * 20000 and m_o[2] > 0 and abs(m_o[3]) > 0  # growth; MSD and VACF non-trivial
    report = {}
    for variant in AT.VARIANTS:
        rows = []
        for s in SEEDS:
            eng = headline_engine(gpu_lib, p, cap, s, variant)
            eng.upload(0, **st)
            SS.install(eng)
            eng.step(STAT_WARM)
            eng.obs_reset(0)
            eng.step(STAT_STEPS)
            ob = eng.observables(0)
            gi = eng.graph_info()
            eng.close()
            assert gi["graph_steps"] > 0  # the steps ran from captured graphs
            rows.append([float(ob[k]) for k in OBS])
        g = np.array(rows)
        m_g, se_g = g.mean(0), g.std(0, ddof=1) / math.sqrt(len(SEEDS))
        z = np.abs(m_g - m_o) / np.sqrt(se_o**2 + se_g**2)
        report[str(variant)] = {k: (float(m_g[i]), float(m_o[i]), round(float(z[i]), 3)) for i, k in enumerate(OBS)}
    print(report)
    for v, r in report.items():
        for k, (mg, mo, z) in r.items():
            assert z <= 2.0, (v, k, mg, mo, z)


# ---------------------------------------------------------------- event samplers

def test_division_time_sampler(gpu_lib):
    """Cycle lengths drawn at divisions (mother and daughter) in steps follow
    max(Nint(N(mu, sigma) / dt), 1): mean, spread and shape (chi-square over 5-step bins)."""
    # a sparse colony (packing 0.1): six-fold growth in 260 steps without apoptosis stays far
    # from crowding (the cycle lengths do not depend on positions)
    p = S.growth_params(box=400.0, dt=1e-3, div_tau_mu=0.1, div_tau_sigma=0.02, apop_rate=0.0, noise_D=0.0)
    st = S.disk_colony(5000, p, seed=3, phi=0.1)
    eng = headline_engine(gpu_lib, p, 60000, 5, (0, 0))
    eng.upload(0, **st)
    spans = []
    for k in range(1, 261):
        eng.step(1)
        d = eng.download(0, want=("t0", "tswitch"))
        t0, tsw = d["t0"][: d["ncells"]], d["tswitch"][: d["ncells"]]
        spans.append(tsw[t0 == k] - k)
    eng.close()
    x = np.concatenate(spans).astype(np.float64)
    n = x.size
    assert n > 40000
    mu, sd = 100.0, 20.0
    var = sd * sd + 1.0 / 12.0  # rounding to whole steps
    assert abs(x.mean() - mu) <= 3.5 * math.sqrt(var / n), (x.mean(), n)
    assert abs(x.std() - math.sqrt(var)) <= 3.5 * math.sqrt(var / (2 * n)), (x.std(), n)
    edges = np.arange(37.5, 167.5, 5.0)
    obs, _ = np.histogram(x, bins=edges)
    z = (edges - mu) / sd
    cdf = 0.5 * (1.0 + np.array([math.erf(v / math.sqrt(2.0)) for v in z]))
    exp = n * np.diff(cdf)
    keep = exp > 20
    chi2 = float(np.sum((obs[keep] - exp[keep]) ** 2 / exp[keep]))
    dof = int(keep.sum()) - 1
    # chi-square above mean + 5 sd (dof + 5 sqrt(2 dof)) would reject a correct sampler with
    # probability well below 1e-4
    assert chi2 <= dof + 5.0 * math.sqrt(2.0 * dof), (chi2, dof)


def test_apoptosis_count_sampler(gpu_lib):
    """Deaths per step among n cells follow Binomial(n, rate dt): their sum and their
    dispersion over 200 steps."""
    p = S.growth_params(box=1024.0, dt=1e-3, apop_rate=1.0, divide=0, noise_D=0.0)
    st = S.disk_colony(100000, p, seed=4)
    eng = headline_engine(gpu_lib, p, 100000, 6, (0, 0))
    eng.upload(0, **st)
    q = p["apop_rate"] * p["dt"]
    ob = eng.observables(0)
    n_prev, a_prev = ob["ncells"], ob["napo_total"]
    d, m = [], []
    for _ in range(200):
        eng.step(1)
        ob = eng.observables(0)
        d.append(ob["napo_total"] - a_prev)
        m.append(n_prev * q)
        assert ob["ncells"] == n_prev - d[-1]
        n_prev, a_prev = ob["ncells"], ob["napo_total"]
    eng.close()
    d, m = np.array(d, np.float64), np.array(m)
    assert abs(d.sum() - m.sum()) <= 3.5 * math.sqrt(m.sum() * (1 - q)), (d.sum(), m.sum())
    disp = float(np.sum((d - m) ** 2) / np.sum(m * (1 - q)))
    assert abs(disp - 1.0) <= 3.5 * math.sqrt(2.0 / len(d)), disp


# ---------------------------------------------------------------- exact observables

def test_observables_equal_oracle_in_oracle_mode(gpu_lib, oracle_lib):
    p = S.growth_params(box=120.0, dt=1e-3, div_tau_mu=0.05, div_tau_sigma=0.01, apop_rate=2.0, noise_D=0.02)
    st = S.disk_colony(2500, p, seed=11)
    cap = 12000
    eng = gpu_lib.Engine([p], [cap], precision=gpu_lib.PREC_FP64, rng=gpu_lib.RNG_DSFMT, seed=9)
    eng.upload(0, **st)
    ora = oracle_lib.Oracle(p, cap, 9)
    ora.set_state(**st)
    for side in (eng, ora):
        side.step(20)
    eng.obs_reset(0)
    ora.obs_reset()
    eng.step(60)
    ora.step(60)
    g, o = eng.observables(0), ora.observables()
    eng.close()
    for k in ("ncells", "ndiv_total", "napo_total"):
        assert g[k] == o[k], (k, g[k], o[k])
    assert g["ndiv_total"] > 0 and g["napo_total"] > 0
    assert abs(g["mean_area"] - o["mean_area"]) <= 1e-12 * abs(o["mean_area"])
    for k in ("msd", "vacf"):
        assert abs(g[k] - o[k]) <= 1e-9 * abs(o[k]), (k, g[k], o[k])


# ---------------------------------------------------------------- the first configuration at size

def test_first_configuration_at_stated_size(gpu_lib, oracle_lib):
    """4096 cells x 2 elements, WCA, packing 0.8 (relaxed from uniform centres): bins at three
    widths identical, forces 1e-12 (norm-wise), 1000 steps of the oracle-mode trajectory 1e-9."""
    p, st = S.config1(4096, seed=12345)
    st = S.relax(p, st)
    n = len(st["sigma"])
    ora = oracle_lib.Oracle(p, n, 1)
    ora.set_state(**st)
    for width in (1.8, 2.6, 5.0):  # at least the largest cutoff (the engine's minimum width)
        eng = gpu_lib.Engine([p], [n], bin_width=width)
        eng.upload(0, **st)
        ns, start, elems = eng.bins(0)
        eng.close()
        ons, head, lst = ora.bin_elements(width)
        assert list(ns) == list(ons)
        ref = oracle_lib.bins_as_sets(head, lst)
        for b, s in enumerate(ref):
            assert set(elems[start[b]:start[b + 1]].tolist()) == s
    ora.close()
    eng = gpu_lib.Engine([p], [n], rng=gpu_lib.RNG_DSFMT, seed=9)
    eng.upload(0, **st)
    ora = oracle_lib.Oracle(p, n, 9)
    ora.set_state(**st)
    fg, fo = eng.forces(0), ora.compute_forces()
    assert np.abs(fg - fo).max() <= 1e-12 * np.abs(fo).max()
    eng.step(1000)
    assert ora.step(1000) == 0
    g, o = eng.download(0), ora.state()
    eng.close()
    assert g["ncells"] == len(o["sigma"])
    err = np.abs(minimage(g["pos"], o["pos"], p)).max()
    print("1000-step trajectory max |dx|", err)
    assert err <= 1e-9


# ---------------------------------------------------------------- near the benchmark's size

def test_256k_cells_bins_and_forces(gpu_lib, oracle_lib):
    p = S.growth_params(box=1024.0)
    st = S.disk_colony(256000, p, seed=13)
    n = len(st["sigma"])
    ora = oracle_lib.Oracle(p, n, 9)
    ora.set_state(**st)
    eng = gpu_lib.Engine([p], [n], bin_width=1.5)
    eng.upload(0, **st)
    ns, start, elems = eng.bins(0)
    eng.close()
    ons, head, lst = ora.bin_elements(1.5)
    assert list(ns) == list(ons)
    ref = oracle_lib.bins_as_sets(head, lst)
    assert len(start) == len(ref) + 1
    for b, s in enumerate(ref):
        assert set(elems[start[b]:start[b + 1]].tolist()) == s
    fo = ora.compute_forces()
    scale = np.abs(fo).max()
    for prec, tol in ((gpu_lib.PREC_FP64, 1e-12), (gpu_lib.PREC_MIXED, 2e-5)):
        eng = gpu_lib.Engine([p], [n], precision=prec, rng=gpu_lib.RNG_DSFMT, seed=9)
        eng.upload(0, **st)
        fg = eng.forces(0)
        eng.close()
        assert np.abs(fg - fo).max() <= tol * scale, (prec, np.abs(fg - fo).max() / scale)
    ora.close()


# ---------------------------------------------------------------- batching

def test_batched_colonies_draw_what_they_draw_alone(gpu_lib):
    """Four colonies of uneven size in one Philox handle with lists and the scheduler, against
    each colony alone with its random stream: the same divisions and apoptoses (cell counts,
    cycle arrays), positions equal to FP32 summation order."""
    from cil_cuda_gb300 import skin_scheduler as SS
    sizes = (3000, 6500, 1500, 9000)
    ps, sts = [], []
    for i, n in enumerate(sizes):
        p = S.growth_params(box=260.0, dt=1e-3, div_tau_mu=0.1, div_tau_sigma=0.02, apop_rate=1.0, noise_D=0.02)
        ps.append(p)
        sts.append(S.disk_colony(n, p, seed=40 + i))
    caps = [3 * n for n in sizes]
    eng = gpu_lib.Engine(ps, caps, precision=gpu_lib.PREC_MIXED, rng=gpu_lib.RNG_PHILOX, seed=21,
                         skin=SS.load()[2])
    for c, st in enumerate(sts):
        eng.upload(c, **st)
    SS.install(eng)
    eng.step(100)
    batched = [eng.download(c) for c in range(len(sizes))]
    eng.close()
    for c, st in enumerate(sts):
        one = gpu_lib.Engine([ps[c]], [caps[c]], precision=gpu_lib.PREC_MIXED, rng=gpu_lib.RNG_PHILOX, seed=21,
                             skin=SS.load()[2], rng_stream_base=c)
        one.upload(0, **st)
        SS.install(one)
        one.step(100)
        alone = one.download(0)
        one.close()
        b = batched[c]
        assert b["ncells"] == alone["ncells"] and b["ncells"] > sizes[c]
        n = b["ncells"]
        np.testing.assert_array_equal(b["t0"][:n], alone["t0"][:n])
        np.testing.assert_array_equal(b["tswitch"][:n], alone["tswitch"][:n])
        err = np.abs(minimage(b["pos"][:n], alone["pos"][:n], ps[c])).max()
        assert err <= 1e-3, (c, err)
