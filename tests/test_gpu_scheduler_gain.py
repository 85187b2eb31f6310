"""What the trained skin scheduler gains: device time per step of the mixed-precision step on
held-out growth colonies (seeds and motilities not used in training) with

  * per-step rebuild (no lists: the reference's method, CIL.cu:180),
  * Verlet lists with a fixed skin of 0.3 sigma (guard on),
  * Verlet lists with the skin and cadence chosen by the trained network (guard on).

The three runs start from the same state with the same Philox stream; the displacement guard
keeps the scheduled run's physics that of the others (trajectory parity of the skin mode
against the oracle is tested in test_gpu_skin.py). Times are summed over the colonies."""
import math
import os

import numpy as np
import pytest

from cil_cuda_gb300 import skin_scheduler as SS
from cil_cuda_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
STEPS, WARMUP = 400, 40


def held_out():
    rng = np.random.default_rng(987654)
    out = []
    for ncells, mot in ((1000000, 1.0), (150000, 0.3), (150000, 1.5), (60000, 1.0)):
        tau = math.exp(rng.uniform(math.log(0.3), math.log(3.0)))
        p = S.growth_params(box=2048.0 if ncells > 500000 else 1024.0, div_tau_mu=tau, div_tau_sigma=0.1 * tau,
                            apop_rate=0.01 / tau, motility=[0.0, mot])
        out.append((p, S.disk_colony(ncells, p, seed=int(rng.integers(1, 2**31 - 1)))))
    return out


def timed(G, p, st, skin, sched):
    n = len(st["sigma"])
    eng = G.Engine([p], [int(1.3 * n) + 64], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=3, skin=skin)
    eng.upload(0, **st)
    if sched:
        SS.install(eng)
    eng.step(WARMUP)
    eng.step(STEPS)
    ms = eng.timings()["total_ms"] / STEPS
    n1 = eng.observables(0)["ncells"]
    info = eng.skin_stats(0) if skin > 0 else None
    eng.close()
    return ms, n1, info


def test_scheduler_beats_fixed_skin_and_per_step_rebuild(gpu_lib):
    assert os.path.exists(SS.WEIGHTS), "trained scheduler weights missing (python -m cil_cuda_gb300.skin_scheduler)"
    skin_max = SS.load()[2]
    tot = {"rebuild": 0.0, "fixed": 0.0, "sched": 0.0}
    rows = []
    for p, st in held_out():
        r, nr, _ = timed(gpu_lib, p, st, 0.0, False)
        f, nf, fi = timed(gpu_lib, p, st, 0.3, False)
        m, nm, mi = timed(gpu_lib, p, st, skin_max, True)
        assert nr == nf == nm  # same division / apoptosis stream
        tot["rebuild"] += r
        tot["fixed"] += f
        tot["sched"] += m
        rows.append((len(st["sigma"]), p["motility"][1], r, f, m, fi["nrebuild"], mi["nrebuild"], mi["skin"]))
    for row in rows:
        print("cells %d motility %.2f  ms/step: rebuild %.4f fixed %.4f scheduled %.4f  rebuilds fixed %d "
              "scheduled %d  last skin %.3f" % row)
    print("total ms/step", tot)
    assert tot["sched"] < tot["rebuild"]
    assert tot["sched"] < tot["fixed"]
