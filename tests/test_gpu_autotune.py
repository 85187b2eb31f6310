"""Autotuner: every candidate (bin size x list-kernel variant) runs the same physics, and the
tuner returns settings an Engine accepts."""
import numpy as np
import pytest

from cil_cuda_gb300 import autotune as AT
from cil_cuda_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def test_variants_agree_and_tuner_picks_one(gpu_lib):
    p = S.growth_params(box=256.0, div_tau_mu=0.3, div_tau_sigma=0.03, apop_rate=0.1)
    st = S.disk_colony(20000, p, seed=8)
    cap = 26000
    outs = []
    for f, (stg, occ) in [(1.0, (4, 3)), (1.3, (1, 3)), (1.15, (2, 3)), (1.0, (1, 4))]:
        w = 0.0 if f == 1.0 else f * AT.needed_width([p], [st], 0.3)
        eng = gpu_lib.Engine([p], [cap], precision=gpu_lib.PREC_MIXED, rng=gpu_lib.RNG_PHILOX, seed=4, skin=0.3,
                             bin_width=w, staging=stg, occupancy=occ)
        eng.upload(0, **st)
        eng.step(60)
        outs.append(eng.download(0))
        eng.close()
    for o in outs[1:]:
        assert o["ncells"] == outs[0]["ncells"]
        np.testing.assert_array_equal(o["tswitch"], outs[0]["tswitch"])
        d = o["pos"] - outs[0]["pos"]
        d -= np.round(d / p["box"][0]) * p["box"][0]
        assert np.abs(d).max() < 1e-4
    kw, trials = AT.autotune([p], [st], [cap], skin=0.3, steps=10, warmup=3, bin_factors=(1.0, 1.15))
    assert len(trials) == 2 * len(AT.VARIANTS) + len(AT.BLOCK_SIZES) - 1
    assert all(t["ms_per_step"] > 0 for t in trials)
    eng = gpu_lib.Engine([p], [cap], precision=gpu_lib.PREC_MIXED, rng=gpu_lib.RNG_PHILOX, seed=4, skin=0.3, **kw)
    eng.upload(0, **st)
    eng.step(5)
    eng.close()


def test_block_sizes_agree(gpu_lib):
    """The list force kernel at 128, 256 and 512 cells per block runs the same physics."""
    p = S.growth_params(box=256.0, div_tau_mu=0.3, div_tau_sigma=0.03, apop_rate=0.1)
    st = S.disk_colony(20000, p, seed=9)
    outs = []
    for block in (256, 128, 512):
        eng = gpu_lib.Engine([p], [26000], precision=gpu_lib.PREC_MIXED, rng=gpu_lib.RNG_PHILOX, seed=4, skin=0.3,
                             block_size=block)
        eng.upload(0, **st)
        eng.step(60)
        outs.append(eng.download(0))
        eng.close()
    for o in outs[1:]:
        assert o["ncells"] == outs[0]["ncells"]
        np.testing.assert_array_equal(o["tswitch"], outs[0]["tswitch"])
        d = o["pos"] - outs[0]["pos"]
        d -= np.round(d / p["box"][0]) * p["box"][0]
        assert np.abs(d).max() < 1e-4


def test_invalid_variant_rejected(gpu_lib):
    p = S.growth_params(box=64.0)
    for stg, occ in ((8, 4), (2, 2)):  # (2, 2): a pair no longer compiled
        with pytest.raises(gpu_lib.CilError):
            gpu_lib.Engine([p], [100], precision=gpu_lib.PREC_MIXED, skin=0.3, staging=stg, occupancy=occ)
    with pytest.raises(gpu_lib.CilError):
        gpu_lib.Engine([p], [100], precision=gpu_lib.PREC_MIXED, skin=0.3, block_size=384)
    with pytest.raises(gpu_lib.CilError):  # other block sizes only for the list kernel of skin mode
        gpu_lib.Engine([p], [100], precision=gpu_lib.PREC_MIXED, block_size=512)
