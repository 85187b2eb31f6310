"""cil_bin_elements_noalloc: the binning entry point for callers that cannot allocate device
memory (a host framework that owns its device pool, code running during CUDA graph capture,
real-time loops). It must give exactly what cil_bins gives for the same positions and bin
width (integer results: bit-exact), on two calls in a row that share its fixed scratch, and
must refuse inputs beyond its stated limits before touching the GPU.

Kept in a file that pytest collects last; it passes alone in a fresh process and after the
other tests."""
import ctypes as C

import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

MAX_ELEMS = 1 << 20


def reference_bins(G, p, st, width):
    eng = G.Engine([p], [len(st["sigma"])], bin_width=width)
    eng.upload(0, **st)
    ns, start, elems = eng.bins(0)
    eng.close()
    return ns, start, elems


def noalloc_bins(G, torch, p, st, width, max_bins):
    lib = G.lib()
    pos = torch.tensor(np.ascontiguousarray(st["pos"]).reshape(-1, p["dim"]), dtype=torch.float64, device="cuda")
    n = pos.shape[0]
    bin_start = torch.full((max_bins + 1,), -7, dtype=torch.int32, device="cuda")
    elems = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    box = np.array(p["box"][: p["dim"]], np.float64)
    ns = np.zeros(3, np.int32)
    stream = torch.cuda.current_stream().cuda_stream
    st_code = lib.cil_bin_elements_noalloc(
        C.c_void_p(pos.data_ptr()), n, p["dim"], box.ctypes.data_as(C.POINTER(C.c_double)), width,
        ns.ctypes.data_as(C.POINTER(C.c_int32)), C.c_void_p(bin_start.data_ptr()),
        C.c_void_p(elems.data_ptr()), max_bins, C.c_void_p(stream))
    torch.cuda.synchronize()
    assert st_code == 0, st_code
    nb = int(np.prod(ns[: p["dim"]]))
    return ns, bin_start[: nb + 1].cpu().numpy(), elems.cpu().numpy()


def test_noalloc_binning_matches_cil_bins_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    p, st1 = S.config1(3000, seed=5)
    p2, st2 = S.config1(3000, seed=6)  # a second, different colony for the second call
    width = 1.7
    for params, st in ((p, st1), (p2, st2)):
        ns_r, start_r, elems_r = reference_bins(gpu_lib, params, st, width)
        ns_n, start_n, elems_n = noalloc_bins(gpu_lib, torch, params, st, width, max_bins=1 << 16)
        assert list(ns_n) == list(ns_r)
        np.testing.assert_array_equal(start_n, start_r)
        np.testing.assert_array_equal(elems_n, elems_r)


def test_noalloc_refuses_oversize_inputs(gpu_lib):
    lib = gpu_lib.lib()
    box = np.array([100.0, 100.0], np.float64)
    ns = np.zeros(3, np.int32)
    dummy = C.c_void_p(16)  # never dereferenced: the size checks come first
    bp = box.ctypes.data_as(C.POINTER(C.c_double))
    nsp = ns.ctypes.data_as(C.POINTER(C.c_int32))
    assert lib.cil_bin_elements_noalloc(dummy, MAX_ELEMS + 1, 2, bp, 1.0, nsp, dummy, dummy, 1 << 20, None) == 3
    # 100 x 100 bins of width 1 exceed max_bins = 50
    assert lib.cil_bin_elements_noalloc(dummy, 10, 2, bp, 1.0, nsp, dummy, dummy, 50, None) == 3
    assert lib.cil_bin_elements_noalloc(dummy, 10, 4, bp, 1.0, nsp, dummy, dummy, 50, None) == 1
