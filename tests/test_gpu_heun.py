"""The reference's StochasticHeun integrator (CIL.cu:1028-1050), cil_config.integrator =
CIL_INTEGRATOR_HEUN: two half steps per step, each a force evaluation with its own noise draw.

* oracle mode (the reference's host draws, FP64) against the oracle's Heun, with division,
  apoptosis and noise;
* without noise and events a Heun step of dt is two Euler steps of dt/2, bit for bit (FP64);
* the two half steps draw independent noise: free diffusion spreads half as fast as with
  Euler (each half step moves (dt/2) sqrt(2D/dt) N), which a repeated draw would not;
* the mixed skin form with graph replay agrees with its launch-by-launch run."""
import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def wrapdiff(a, b, L):
    d = np.asarray(a) - np.asarray(b)
    return d - np.round(d / L) * L


def test_heun_oracle_mode_matches_oracle(gpu_lib, oracle_lib):
    G = gpu_lib
    p = S.growth_params(box=60.0, dt=1e-3, div_tau_mu=0.06, div_tau_sigma=0.01, apop_rate=2.0, noise_D=0.002)
    st = S.disk_colony(400, p, seed=21)
    cap = 8000
    eng = G.Engine([p], [cap], precision=G.PREC_FP64, rng=G.RNG_DSFMT, seed=17, integrator=G.INTEGRATOR_HEUN)
    eng.upload(0, **st)
    eng.step(120)
    g = eng.download(0)
    eng.close()
    o = oracle_lib.Oracle(p, cap, 17, integrator=1)
    o.set_state(**st)
    assert o.step(120) == 0
    s = o.state()
    assert g["ncells"] == len(s["sigma"]) and g["ncells"] != 400
    np.testing.assert_array_equal(g["tswitch"], s["tswitch"])
    assert np.abs(wrapdiff(g["pos"], s["pos"], 60.0)).max() <= 1e-9
    assert np.abs(g["vel"] - s["vel"]).max() <= 1e-7 * max(1.0, np.abs(s["vel"]).max())


def test_heun_fene_bond_oracle_mode(gpu_lib, oracle_lib):
    """The reference's two-element integrator with its own bond (binaryCellForce, FENE / push
    spring, no division) against the oracle, oracle-mode noise, FP64."""
    G = gpu_lib
    p = S.fene_params(box=80.0, dt=1e-3, noise_D=0.002)
    st = S.disk_colony(1200, p, seed=23)
    eng = G.Engine([p], [1200], precision=G.PREC_FP64, rng=G.RNG_DSFMT, seed=19, integrator=G.INTEGRATOR_HEUN)
    eng.upload(0, **st)
    eng.step(150)
    g = eng.download(0)
    eng.close()
    o = oracle_lib.Oracle(p, 1200, 19, integrator=1)
    o.set_state(**st)
    assert o.step(150) == 0
    s = o.state()
    assert np.abs(wrapdiff(g["pos"], s["pos"], 80.0)).max() <= 1e-9


def test_heun_is_two_half_euler_steps(gpu_lib):
    G = gpu_lib
    p = S.growth_params(box=60.0, dt=1e-3, divide=0, apop_rate=0.0, noise_D=0.0)
    st = S.disk_colony(1000, p, seed=22)
    q = dict(p)
    q["dt"] = 0.5e-3
    out = []
    for params, integ, n in ((p, G.INTEGRATOR_HEUN, 60), (q, G.INTEGRATOR_EULER, 120)):
        eng = G.Engine([params], [1100], precision=G.PREC_FP64, rng=G.RNG_PHILOX, seed=3, integrator=integ)
        eng.upload(0, **st)
        eng.step(n)
        out.append(eng.download(0)["pos"])
        eng.close()
    np.testing.assert_array_equal(out[0], out[1])


@pytest.mark.parametrize("precision", [0, 1])
def test_heun_half_steps_draw_independent_noise(gpu_lib, precision):
    G = gpu_lib
    D = 0.05
    p = S.growth_params(box=1000.0, dt=1e-3, divide=0, apop_rate=0.0, noise_D=D, kappa=0.0, motility=[0.0, 0.0],
                        epsilon=0.0)
    st = S.disk_colony(20000, p, seed=23, phi=0.05)
    msd = {}
    for integ in (G.INTEGRATOR_EULER, G.INTEGRATOR_HEUN):
        eng = G.Engine([p], [20100], precision=precision, rng=G.RNG_PHILOX, seed=4, integrator=integ)
        eng.upload(0, **st)
        eng.obs_reset(0)
        eng.step(200)
        msd[integ] = eng.observables(0)["msd"]
        eng.close()
    ratio = msd[G.INTEGRATOR_HEUN] / msd[G.INTEGRATOR_EULER]
    assert abs(ratio - 0.5) < 0.05, (ratio, msd)


def test_heun_mixed_skin_graphs(gpu_lib):
    G = gpu_lib
    p = S.growth_params(box=120.0, dt=1e-3, div_tau_mu=0.2, div_tau_sigma=0.02, apop_rate=0.5)
    st = S.disk_colony(3000, p, seed=24)
    res = []
    for graphs in (False, True):
        eng = G.Engine([p], [9000], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=5, skin=0.3, graphs=graphs,
                       integrator=G.INTEGRATOR_HEUN)
        eng.upload(0, **st)
        eng.step(101)
        res.append((eng.download(0), eng.graph_info(), eng.observables(0)))
        eng.close()
    (a, ia, oa), (b, ib, ob) = res
    assert ia["graph_steps"] == 0 and ib["graph_steps"] > 0
    assert a["ncells"] == b["ncells"] and oa["ndiv_total"] == ob["ndiv_total"] > 0
    np.testing.assert_array_equal(a["tswitch"], b["tswitch"])
    assert np.abs(wrapdiff(a["pos"], b["pos"], 120.0)).max() < 1e-4
