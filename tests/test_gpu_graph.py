"""CUDA-graph replay of steady steps against the same steps launched one by one.

Philox mode only (oracle mode draws on the host every step). The FP64 form is deterministic,
so the two runs must agree bit for bit; the mixed forms sum pair forces in a scheduling-
dependent FP32 order, so they agree to FP32 rounding over the run."""
import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
STEPS = 101  # an odd count: graph pairs, stand-alone steps and the last step


def run(G, p, st, precision, graphs, skin=0.0, steps=STEPS):
    n = len(st["sigma"])
    eng = G.Engine([p], [3 * n], precision=precision, rng=G.RNG_PHILOX, seed=5, skin=skin, graphs=graphs)
    eng.upload(0, **st)
    eng.step(steps)
    out = eng.download(0)
    info = eng.graph_info()
    ob = eng.observables(0)
    eng.close()
    return out, info, ob


@pytest.fixture(scope="module")
def growth():
    p = S.growth_params(box=120.0, dt=1e-3, div_tau_mu=0.2, div_tau_sigma=0.02, apop_rate=0.5)
    return p, S.disk_colony(3000, p, seed=4)


def test_fp64_graph_bitwise(gpu_lib, growth):
    p, st = growth
    a, ia, oa = run(gpu_lib, p, st, gpu_lib.PREC_FP64, graphs=False)
    b, ib, ob = run(gpu_lib, p, st, gpu_lib.PREC_FP64, graphs=True)
    assert ia["graph_steps"] == 0 and ib["graph_steps"] >= STEPS - 3
    assert a["ncells"] == b["ncells"] and oa["ndiv_total"] == ob["ndiv_total"] > 0
    np.testing.assert_array_equal(a["pos"], b["pos"])
    np.testing.assert_array_equal(a["vel"], b["vel"])
    np.testing.assert_array_equal(a["tswitch"], b["tswitch"])


@pytest.mark.parametrize("skin", [0.0, 0.3])
def test_mixed_graph_matches_launches(gpu_lib, growth, skin):
    p, st = growth
    a, ia, oa = run(gpu_lib, p, st, gpu_lib.PREC_MIXED, graphs=False, skin=skin)
    b, ib, ob = run(gpu_lib, p, st, gpu_lib.PREC_MIXED, graphs=True, skin=skin)
    assert ib["graph_steps"] > 0 and ib["graphs_captured"] >= 1
    # divisions and apoptosis follow the same Philox streams
    assert a["ncells"] == b["ncells"] and oa["ndiv_total"] == ob["ndiv_total"]
    np.testing.assert_array_equal(a["tswitch"], b["tswitch"])
    d = np.asarray(a["pos"]) - np.asarray(b["pos"])
    d -= np.round(d / p["box"][0]) * p["box"][0]
    assert np.abs(d).max() < 1e-4


def test_rebuild_node_and_plain_launches_agree(gpu_lib, growth):
    """Skin mode with graphs: the list-rebuild kernels in a conditional graph node (run on
    rebuild steps only, CIL_FLAG_REBUILD_NODE) and the same kernels launched every step
    (returning at once when no colony rebuilds) give the same run: the same rebuilds, divisions
    and apoptoses, positions to FP32 summation order; the node saves the seven launches on steps
    without a rebuild."""
    p, st = growth
    n = len(st["sigma"])
    res = []
    for node in (True, False):
        eng = gpu_lib.Engine([p], [3 * n], precision=gpu_lib.PREC_MIXED, rng=gpu_lib.RNG_PHILOX, seed=5, skin=0.3,
                             rebuild_node=node)
        eng.upload(0, **st)
        eng.step(STEPS)
        launches = eng.timings()["launches"]
        res.append((eng.download(0), launches, eng.skin_stats(0), eng.graph_info(), eng.observables(0)))
        eng.close()
    (a, la, ska, ga, oa), (b, lb, skb, gb, ob) = res
    assert ga["graph_steps"] > 0 and gb["graph_steps"] == ga["graph_steps"]
    assert ska["nrebuild"] == skb["nrebuild"] and 1 <= ska["nrebuild"] < STEPS // 2
    assert a["ncells"] == b["ncells"] and oa["ndiv_total"] == ob["ndiv_total"] > 0
    np.testing.assert_array_equal(a["tswitch"], b["tswitch"])
    d = np.asarray(a["pos"]) - np.asarray(b["pos"])
    d -= np.round(d / p["box"][0]) * p["box"][0]
    assert np.abs(d).max() < 1e-4
    # replayed steps without a rebuild launch the node's seven kernels fewer
    assert 7 * (ga["graph_steps"] - ska["nrebuild"]) <= lb - la <= 7 * ga["graph_steps"]


def test_graphs_follow_buffers_allocated_between_calls(gpu_lib, growth):
    """Observables are allocated at the first obs_reset; steps captured before it must not be
    replayed after it (they would hold no observable arrays and divisions would not carry the
    tracks to the daughters)."""
    p, st = growth
    res = []
    for graphs in (False, True):
        n = len(st["sigma"])
        eng = gpu_lib.Engine([p], [3 * n], precision=gpu_lib.PREC_FP64, rng=gpu_lib.RNG_PHILOX, seed=5,
                             graphs=graphs)
        eng.upload(0, **st)
        eng.step(21)
        eng.obs_reset(0)
        eng.step(61)
        res.append(eng.observables(0))
        eng.close()
    assert res[0]["ndiv_total"] > 0
    for k in ("ncells", "mean_area", "msd", "vacf"):
        assert res[0][k] == res[1][k], (k, res[0][k], res[1][k])


def test_deferred_status(gpu_lib):
    """CIL_FLAG_DEFERRED_STATUS: the same run, and a capacity overflow reported by the call
    after the step that overflowed."""
    G = gpu_lib
    p = S.growth_params(box=80.0, dt=1e-3, div_tau_mu=0.02, div_tau_sigma=0.002, apop_rate=0.0)
    st = S.disk_colony(600, p, seed=9)
    res = []
    for deferred in (False, True):
        eng = G.Engine([p], [700], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=5, skin=0.3,
                       deferred_status=deferred)
        eng.upload(0, **st)
        fail_at = None
        for k in range(60):
            try:
                eng.step(1)
            except G.CilError as e:
                assert e.status == 3  # CIL_ERR_CAPACITY
                fail_at = k
                break
        res.append(fail_at)
        eng.close()
    assert res[0] is not None and res[1] == res[0] + 1
    out = []
    for deferred in (False, True):
        eng = G.Engine([p], [4000], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=5, skin=0.3,
                       deferred_status=deferred)
        eng.upload(0, **st)
        for _ in range(40):
            eng.step(1)
        out.append(eng.download(0))
        eng.close()
    assert out[0]["ncells"] == out[1]["ncells"]
    d = out[0]["pos"] - out[1]["pos"]
    d -= np.round(d / 80.0) * 80.0
    assert np.abs(d).max() < 1e-4
