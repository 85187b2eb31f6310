"""cil_bin_elements_noalloc: the binning entry point for callers that cannot allocate device
memory (a host framework that owns its device pool and forbids outside cudaMalloc, or a
real-time loop that cannot risk an allocation's latency or failure). It must give exactly what
cil_bins gives for the same positions and bin width (integer results: bit-exact), on calls in
a row that share its fixed scratch, and must refuse inputs beyond its stated limits before
touching the GPU.

Cases: a 2D colony on a grid of more than 1024 bins (two radix passes) and then a different
colony on the same scratch; a grid of at most 1024 bins (one pass); a grid collapsed to one
bin (width above a third of the box: every element in one bin, ordered by id); a 3D colony;
an empty input.

Kept in a file that pytest collects last; it passes alone in a fresh process and after the
other tests."""
import ctypes as C

import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

MAX_ELEMS = 1 << 20
CAPACITY = 3
CONFIG = 1


def reference_bins(G, p, st, width):
    eng = G.Engine([p], [len(st["sigma"])], bin_width=width)
    eng.upload(0, **st)
    ns, start, elems = eng.bins(0)
    eng.close()
    return ns, start, elems


def call_noalloc(lib, torch, pos, n, dim, box, width, max_bins):
    bin_start = torch.full((max_bins + 1,), -7, dtype=torch.int32, device="cuda")
    elems = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    box = np.array(box[:dim], np.float64)
    ns = np.zeros(3, np.int32)
    stream = torch.cuda.current_stream().cuda_stream
    code = lib.cil_bin_elements_noalloc(
        C.c_void_p(pos.data_ptr()), n, dim, box.ctypes.data_as(C.POINTER(C.c_double)), width,
        ns.ctypes.data_as(C.POINTER(C.c_int32)), C.c_void_p(bin_start.data_ptr()),
        C.c_void_p(elems.data_ptr()), max_bins, C.c_void_p(stream))
    torch.cuda.synchronize()
    assert code == 0, code
    nb = int(np.prod(ns[:dim]))
    return ns, bin_start[: nb + 1].cpu().numpy(), elems[:n].cpu().numpy()


def noalloc_bins(G, torch, p, st, width, max_bins):
    pos = torch.tensor(np.ascontiguousarray(st["pos"]).reshape(-1, p["dim"]), dtype=torch.float64, device="cuda")
    return call_noalloc(G.lib(), torch, pos, pos.shape[0], p["dim"], p["box"], width, max_bins)


def check_same(G, torch, p, st, width, max_bins=1 << 16):
    ns_r, start_r, elems_r = reference_bins(G, p, st, width)
    ns_n, start_n, elems_n = noalloc_bins(G, torch, p, st, width, max_bins)
    assert list(ns_n) == list(ns_r)
    np.testing.assert_array_equal(start_n, start_r)
    np.testing.assert_array_equal(elems_n, elems_r)
    return ns_n


def test_noalloc_binning_matches_cil_bins_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    p, st1 = S.config1(3000, seed=5)
    p2, st2 = S.config1(3000, seed=6)  # a second, different colony for the second call
    for params, st in ((p, st1), (p2, st2)):
        ns = check_same(gpu_lib, torch, params, st, 1.7)
        assert ns[0] * ns[1] > 1024  # the two-pass radix path


def test_noalloc_small_grid_collapsed_grid_and_3d(gpu_lib):
    torch = pytest.importorskip("torch")
    p, st = S.config1(2000, seed=8)
    ns = check_same(gpu_lib, torch, p, st, 5.0)  # at most 1024 bins: one radix pass
    assert 9 <= ns[0] * ns[1] <= 1024
    # width above a third of the box: the grid collapses to one bin holding every element
    ns = check_same(gpu_lib, torch, p, st, 0.4 * p["box"][0])
    assert list(ns) == [1, 1, 1]
    q = S.channel_params(lxy=24.0, height=10.0)
    st3 = S.channel_colony(1200, q, seed=4)
    ns = check_same(gpu_lib, torch, q, st3, 1.6)
    assert ns[2] > 1


def test_noalloc_empty_input(gpu_lib):
    torch = pytest.importorskip("torch")
    pos = torch.zeros((1, 2), dtype=torch.float64, device="cuda")  # a real buffer; n = 0 reads none of it
    ns, start, elems = call_noalloc(gpu_lib.lib(), torch, pos, 0, 2, [50.0, 50.0], 2.0, 1 << 12)
    k = int(50.0 / (2.0 + 50.0 * 1.0e-8))  # LinkListOrtho::get_opt_size with its 1e-8 margin
    assert list(ns) == [k, k, 1]
    assert start.shape == (k * k + 1,) and not start.any()
    assert elems.size == 0


def test_noalloc_refuses_oversize_inputs(gpu_lib):
    torch = pytest.importorskip("torch")
    lib = gpu_lib.lib()
    # real (small) device buffers: the size checks refuse before anything is enqueued, so
    # none of them is read or written
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    ptr = C.c_void_p(buf.data_ptr())
    box = np.array([100.0, 100.0], np.float64)
    ns = np.zeros(3, np.int32)
    bp = box.ctypes.data_as(C.POINTER(C.c_double))
    nsp = ns.ctypes.data_as(C.POINTER(C.c_int32))
    assert lib.cil_bin_elements_noalloc(ptr, MAX_ELEMS + 1, 2, bp, 1.0, nsp, ptr, ptr, 1 << 20, None) == CAPACITY
    # 100 x 100 bins of width 1 exceed max_bins = 50
    assert lib.cil_bin_elements_noalloc(ptr, 10, 2, bp, 1.0, nsp, ptr, ptr, 50, None) == CAPACITY
    # more bins along one axis than the scratch holds (and than an int holds)
    assert lib.cil_bin_elements_noalloc(ptr, 10, 2, bp, 1e-12, nsp, ptr, ptr, 1 << 20, None) == CAPACITY
    assert lib.cil_bin_elements_noalloc(ptr, 10, 4, bp, 1.0, nsp, ptr, ptr, 50, None) == CONFIG
    assert lib.cil_bin_elements_noalloc(None, 10, 2, bp, 1.0, nsp, ptr, ptr, 1 << 20, None) == CONFIG
    torch.cuda.synchronize()
