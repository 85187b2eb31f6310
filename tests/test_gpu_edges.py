"""Edge cases of the step and its outputs: empty and single-cell colonies in a batch, a
colony at its capacity, frames of an empty colony, and the cell-cycle model with no cells or
one cell."""
import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S
from cil_cuda_gb300.gsd import GSDFile

pytestmark = pytest.mark.gpu


def empty_state():
    return dict(pos=np.zeros((0, 2, 2)), sigma=np.zeros((0, 2)), t0=np.zeros(0, np.int32),
                tswitch=np.zeros(0, np.int32))


@pytest.mark.parametrize("precision,skin", [(0, 0.0), (1, 0.3)])
def test_batch_with_empty_and_single_cell_colonies(gpu_lib, precision, skin):
    """Colony 0 holds no cell, colony 2 a single cell: the batch steps, they stay as they are,
    and colony 1 runs as it does alone (a deterministic force field: no noise, no events; bit
    for bit in FP64)."""
    G = gpu_lib
    p = S.growth_params(box=60.0, dt=1e-3, noise_D=0.0, divide=0, apop_rate=0.0)
    st = S.disk_colony(500, p, seed=31)
    one = S.disk_colony(1, p, seed=32)
    eng = G.Engine([p, p, p], [64, 2000, 64], precision=precision, rng=G.RNG_PHILOX, seed=4, skin=skin)
    eng.upload(0, **empty_state())
    eng.upload(1, **st)
    eng.upload(2, **one)
    eng.step(80)
    a = [eng.download(c) for c in range(3)]
    eng.close()
    assert a[0]["ncells"] == 0 and a[2]["ncells"] == 1
    assert np.all(np.isfinite(a[2]["pos"]))
    alone = G.Engine([p], [2000], precision=precision, rng=G.RNG_PHILOX, seed=4, skin=skin)
    alone.upload(0, **st)
    alone.step(80)
    b = alone.download(0)
    alone.close()
    assert b["ncells"] == a[1]["ncells"] == 500
    if precision == 0:
        np.testing.assert_array_equal(a[1]["pos"], b["pos"])
    else:
        np.testing.assert_allclose(a[1]["pos"], b["pos"], rtol=0, atol=1e-6)


def test_full_capacity_in_captured_skin_steps(gpu_lib):
    """A colony that fills its capacity inside graph-replayed Verlet-list steps: the call returns
    CIL_ERR_CAPACITY, and the state stays readable with no more cells than the capacity."""
    G = gpu_lib
    p = S.growth_params(box=60.0, dt=1e-3, div_tau_mu=0.02, div_tau_sigma=0.002, apop_rate=0.0)
    st = S.disk_colony(300, p, seed=33)
    eng = G.Engine([p], [300], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=4, skin=0.3)
    eng.upload(0, **st)
    with pytest.raises(G.CilError) as e:
        eng.step(40)
    assert e.value.status == 3
    with pytest.raises(G.CilError):
        eng.download(0)
    s = eng.download(0, strict=False)
    assert s["status"] == 3 and s["ncells"] == 300
    assert np.all(np.isfinite(s["pos"])) and np.all(s["sigma"] > 0)
    eng.close()


def test_frames_of_an_empty_colony(gpu_lib, tmp_path):
    G = gpu_lib
    p = S.growth_params(box=60.0, dt=1e-3)
    st = S.disk_colony(100, p, seed=34)
    eng = G.Engine([p, p], [64, 400], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=4, skin=0.3)
    eng.upload(0, **empty_state())
    eng.upload(1, **st)
    path = str(tmp_path / "empty.gsd")
    with eng.frame_writer(0, path) as w:
        w.write()
        eng.step(5)
        w.write()
    eng.close()
    f = GSDFile(path)
    assert f.nframes == 2
    for k in range(2):
        assert int(f.read(k, "particles/N")[0]) == 0
        assert f.read(k, "particles/position") is None
    assert f.chunk_names(1) == ["configuration/step", "configuration/dimensions", "configuration/box", "particles/N"]


def test_cycle_model_without_cells_and_with_one(gpu_lib):
    G = gpu_lib
    prm = dict(box=[20.0, 20.0, 0.0], dt=2e-4, motility=1.0, zeta=0.2)
    eng = G.CycleEngine(prm, 64, seed=1)
    eng.upload(pos=np.zeros((0, 2)))
    eng.step(20)
    eng.check_positions()
    assert eng.download()["ncells"] == 0
    eng.upload(pos=np.array([[10.0, 10.0]]), theta=np.zeros(1))  # far from its division
    eng.step(20)
    s = eng.download()
    eng.close()
    assert s["ncells"] == 1 and np.all(np.isfinite(s["pos"])) and s["pressure"][0] == 0.0


@pytest.mark.parametrize("flags", [0, 1])
def test_cycle_model_capacity_overflow(gpu_lib, flags):
    """Divisions beyond the capacity inside replayed (or launched) steps: the call reports
    CIL_ERR_CAPACITY, the colony never holds more cells than its capacity, and its state stays
    finite."""
    G = gpu_lib
    rng = np.random.default_rng(5)
    n, cap = 60, 80
    prm = dict(box=[20.0, 20.0, 0.0], dt=2e-4, motility=1.0, zeta=0.2, flags=flags)
    eng = G.CycleEngine(prm, cap, seed=2)
    eng.upload(pos=rng.uniform(0, 20.0, size=(n, 2)), theta=np.full(n, 0.999), rho=np.ones(n),
               angvel=np.full(n, 0.01), sigma=np.full(n, 1.1283791670955126))
    with pytest.raises(G.CilError) as e:
        eng.step(5)
    assert e.value.status == 3
    L = eng.L
    v = G.CycleView(ncells=0, capacity=0)
    L.cil_cycle_download(eng.h, v)  # the cell count, whatever the status
    assert v.ncells == cap
    eng.close()
