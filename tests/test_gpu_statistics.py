"""Long-run statistics of the Philox (fast) mode of the forms without Verlet lists (FP64 and
mixed precision, the plain forms the headline is compared with) against the oracle over 16
seeds, on a 400-cell colony.

Both sides start from the same colony; the oracle runs with dSFMT seeds 1..16 (the
reference's stream), the library with Philox seeds 1..16. Cell count, mean cell area, MSD and
VACF at the end are compared through z = |difference of the ensemble means| / SE of that
difference (SE from the 16-sample spreads, as tools/utils.py's block errors). This test is a
guard against gross errors of these forms: every z <= 3. The strict bar (every observable
within 2 SE) is applied to the form the benchmark times, on a 20k-cell colony, in
test_gpu_headline_parity.py, which also tests the event samplers directly with large samples.
The z values are printed per observable.
"""
import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
SEEDS = list(range(1, 17))
OBS = ("ncells", "mean_area", "msd", "vacf")
STEPS = 300
WARM = 20


def setup_case():
    p = S.growth_params(box=70.0, dt=1e-3, div_tau_mu=0.1, div_tau_sigma=0.02, apop_rate=1.0, noise_D=0.02)
    st = S.disk_colony(400, p, seed=21)
    return p, st


def run_oracle(O, p, st, seed):
    o = O.Oracle(p, 4000, seed)
    o.set_state(**st)
    o.step(WARM)  # velocities exist before the VACF origin is taken
    o.obs_reset()
    assert o.step(STEPS) == 0
    return o.observables()


def run_gpu(G, p, st, seed, precision):
    eng = G.Engine([p], [4000], precision=precision, rng=G.RNG_PHILOX, seed=seed)
    eng.upload(0, **st)
    eng.step(WARM)
    eng.obs_reset(0)
    eng.step(STEPS)
    ob = eng.observables(0)
    eng.close()
    return ob


def stats(rows):
    a = np.array([[r[k] for k in OBS] for r in rows], dtype=np.float64)
    return a.mean(axis=0), a.std(axis=0, ddof=1) / np.sqrt(len(rows))


def test_observables_within_three_standard_errors(gpu_lib, oracle_lib):
    p, st = setup_case()
    ora = [run_oracle(oracle_lib, p, st, s) for s in SEEDS]
    m_o, se_o = stats(ora)
    report = {}
    for name, prec in (("fp64", gpu_lib.PREC_FP64), ("mixed", gpu_lib.PREC_MIXED)):
        gpu = [run_gpu(gpu_lib, p, st, s, prec) for s in SEEDS]
        m_g, se_g = stats(gpu)
        se = np.sqrt(se_o**2 + se_g**2)
        z = np.abs(m_g - m_o) / np.where(se > 0, se, 1.0)
        report[name] = {k: (float(m_g[i]), float(m_o[i]), float(z[i])) for i, k in enumerate(OBS)}
        print(name, report[name])
        for i, k in enumerate(OBS):
            assert z[i] <= 3.0, (name, k, m_g[i], m_o[i], se[i])
    # growth actually happened; MSD and VACF are non-trivial
    assert m_o[0] > 400 and m_o[2] > 0 and abs(m_o[3]) > 0
