"""Device-fed GSD frame writer (cil_frame_*, include/cil_gsd.h) against the state cil_download
returns at the same point of the run: every frame's chunks must be the reference's
outputGSDFrame (OutputWriter.cpp:505-644) of that state, bit for bit (FP64 shift by half the
box, then one rounding to FP32). Frames are written while the run goes on, with graph-replayed
steps in between, and writing them must not change the run."""
import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S
from cil_cuda_gb300.gsd import GSDFile

pytestmark = pytest.mark.gpu

BITS = lambda a: np.ascontiguousarray(a, np.float32).view(np.uint32)  # noqa: E731


def expected_frame(state, p, dim, lz):
    n = state["ncells"]
    E = 2 * n
    L = np.asarray(p["box"], np.float64)
    pos = np.zeros((E, 3), np.float32)
    vel = np.zeros((E, 3), np.float32)
    x = state["pos"].reshape(E, dim)
    v = state["vel"].reshape(E, dim)
    for d in range(dim):
        pos[:, d] = (x[:, d] - 0.5 * L[d]).astype(np.float32)
        vel[:, d] = v[:, d].astype(np.float32)
    if dim == 2:
        pos[0::2, 2] = np.float32(0.0 * -0.01)  # -0.0
        pos[1::2, 2] = np.float32(1.0 * -0.01)
    box = np.array([L[0], L[1], L[2] if dim == 3 else lz, 0, 0, 0], np.float32)
    return dict(N=E, pos=pos, vel=vel, dia=state["sigma"].reshape(E).astype(np.float32), box=box)


def check_frame(f, k, exp, step, *, types, per_elem, charge):
    assert int(f.read(k, "configuration/step")[0]) == step
    assert int(f.read(k, "configuration/dimensions")[0]) == 3
    np.testing.assert_array_equal(BITS(f.read(k, "configuration/box")), BITS(exp["box"]))
    assert int(f.read(k, "particles/N")[0]) == exp["N"]
    assert (f.read(k, "particles/types") is not None) == types
    if types:
        assert f.types(k) == ["A_BACK", "A_FRONT"]
    for nm in ("particles/Z", "particles/diameter", "particles/typeid"):
        assert (f.read(k, nm) is not None) == per_elem, nm
    if per_elem:
        np.testing.assert_array_equal(BITS(f.read(k, "particles/Z")), BITS(exp["dia"]))
        np.testing.assert_array_equal(BITS(f.read(k, "particles/diameter")), BITS(exp["dia"]))
        np.testing.assert_array_equal(f.read(k, "particles/typeid"), np.tile([0, 1], exp["N"] // 2))
    ch = f.read(k, "particles/charge")
    assert (ch is not None) == charge
    if charge:
        assert np.all(ch == -1.0)
    np.testing.assert_array_equal(BITS(f.read(k, "particles/position")), BITS(exp["pos"]))
    np.testing.assert_array_equal(BITS(f.read(k, "particles/velocity")), BITS(exp["vel"]))
    assert np.all(f.read(k, "particles/mass") == 0.0)


@pytest.mark.parametrize("precision,skin", [(0, 0.0), (1, 0.3)])
def test_frames_of_a_growing_colony(gpu_lib, tmp_path, precision, skin):
    G = gpu_lib
    p = S.growth_params(box=160.0, dt=1e-3, div_tau_mu=0.3, div_tau_sigma=0.03, apop_rate=0.3)
    st = S.disk_colony(4000, p, seed=11)
    lz = float(st["sigma"].max())
    path = str(tmp_path / "run.gsd")
    eng = G.Engine([p], [4 * len(st["sigma"])], precision=precision, rng=G.RNG_PHILOX, seed=9, skin=skin)
    eng.upload(0, **st)
    w = eng.frame_writer(0, path)
    steps, expect = [], []
    for k in range(7):
        expect.append(expected_frame(eng.download(0), p, 2, lz))
        steps.append(k * 60)
        assert w.write() == k
        eng.step(60)
    w.close()
    f = GSDFile(path)
    assert f.nframes == 7 and (f.application, f.schema) == ("CIL", "hoomd")
    assert expect[-1]["N"] != expect[0]["N"]  # divisions and apoptoses happened between frames
    for k in range(7):
        check_frame(f, k, expect[k], steps[k], types=steps[k] == 0, per_elem=True, charge=True)
    eng.close()


def test_writer_does_not_change_the_run(gpu_lib, tmp_path):
    G = gpu_lib
    p = S.growth_params(box=160.0, dt=1e-3, div_tau_mu=0.3, div_tau_sigma=0.03, apop_rate=0.3)
    st = S.disk_colony(3000, p, seed=12)
    out = []
    for write in (False, True):
        eng = G.Engine([p], [4 * len(st["sigma"])], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=3, skin=0.3)
        eng.upload(0, **st)
        w = eng.frame_writer(0, str(tmp_path / "w.gsd")) if write else None
        for _ in range(10):
            if w:
                w.write()
            eng.step(31)
        if w:
            w.close()
        out.append(eng.download(0))
        eng.close()
    assert out[0]["ncells"] == out[1]["ncells"]
    np.testing.assert_array_equal(out[0]["t0"], out[1]["t0"])
    # the mixed form sums pair forces in a schedule-dependent FP32 order
    L = np.asarray(p["box"][:2])
    d = out[0]["pos"] - out[1]["pos"]
    d -= np.round(d / L) * L
    assert np.abs(d).max() < 1e-4


def test_frames_3d_channel_static_colony(gpu_lib, tmp_path):
    """No division, no apoptosis: per-element chunks only in the frame of step 0, no charge."""
    G = gpu_lib
    p = S.channel_params(lxy=40.0, height=8.0, divide=0, apop_rate=0.0)
    st = S.channel_colony(1500, p, seed=5)
    path = str(tmp_path / "ch.gsd")
    eng = G.Engine([p], [len(st["sigma"]) + 64], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=2, skin=0.2)
    eng.upload(0, **st)
    w = eng.frame_writer(0, path)
    expect, steps = [], []
    for k in range(4):
        expect.append(expected_frame(eng.download(0), p, 3, 0.0))
        steps.append(k * 40)
        w.write()
        eng.step(40)
    # several frames queued back to back: the third waits for a free staging slot
    for k in range(3):
        w.write()
        expect.append(expect[-1] if k else expected_frame(eng.download(0), p, 3, 0.0))
        steps.append(160)
    s = w.stats()
    w.close()
    assert s["frames_queued"] == 7
    f = GSDFile(path)
    assert f.nframes == 7
    for k in range(7):
        check_frame(f, k, expect[k], steps[k], types=steps[k] == 0, per_elem=steps[k] == 0, charge=False)
    eng.close()


def test_final_state_file_and_options(gpu_lib, tmp_path):
    """The reference's final-state file writes one frame labelled step 0 (OutputWriter.cpp:735);
    options: names, length unit, lz, types in a first frame of another step."""
    G = gpu_lib
    p = S.growth_params(box=120.0, dt=1e-3, div_tau_mu=0.3, div_tau_sigma=0.03, apop_rate=0.0)
    st = S.disk_colony(1000, p, seed=13)
    eng = G.Engine([p], [4 * len(st["sigma"])], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=1, skin=0.3)
    eng.upload(0, **st)
    eng.step(50)
    state = eng.download(0)
    last = str(tmp_path / "cil.Last.gsd")
    with eng.frame_writer(0, last) as w:
        w.write(0)
    f = GSDFile(last)
    check_frame(f, 0, expected_frame(state, p, 2, float(st["sigma"].max())), 0, types=True, per_elem=True,
                charge=True)
    opt = str(tmp_path / "opt.gsd")
    with eng.frame_writer(0, opt, cell_name="MDCK", elem_names=("REAR", "LEAD"), length_unit=2.5, lz=3.0,
                          types_in_first=True) as w:
        w.write()
        eng.step(10)
        w.write()
    f = GSDFile(opt)
    assert f.types(0) == ["MDCK_REAR", "MDCK_LEAD"] and f.read(1, "particles/types") is None
    assert f.read(0, "configuration/box")[2] == np.float32(3.0)
    z = f.read(0, "particles/position")[:, 2]
    assert np.all(BITS(z[0::2]) == BITS(np.float32(-0.0)))
    assert np.all(z[1::2] == np.float32(1.0 * (-0.01 * 2.5)))
    assert int(f.read(1, "configuration/step")[0]) == 60
    eng.close()


def test_writer_opened_before_upload(gpu_lib, tmp_path):
    """The output opens before the colony is uploaded (initializeOutput precedes the run); the
    2D box z is the largest uploaded diameter, read at the first frame."""
    G = gpu_lib
    p = S.growth_params(box=120.0, dt=1e-3, div_tau_mu=0.3, div_tau_sigma=0.03, apop_rate=0.0)
    st = S.disk_colony(800, p, seed=14)
    eng = G.Engine([p], [4 * len(st["sigma"])], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=2, skin=0.3)
    path = str(tmp_path / "early.gsd")
    w = eng.frame_writer(0, path)
    eng.upload(0, **st)
    exp0 = expected_frame(eng.download(0), p, 2, float(st["sigma"].max()))
    w.write()
    eng.step(20)
    exp1 = expected_frame(eng.download(0), p, 2, float(st["sigma"].max()))
    w.write()
    w.close()
    f = GSDFile(path)
    check_frame(f, 0, exp0, 0, types=True, per_elem=True, charge=True)
    check_frame(f, 1, exp1, 20, types=False, per_elem=True, charge=True)
    eng.close()
