"""The C-ABI library loads without a GPU and exports every entry point the public headers
declare; argument validation and the oracle-mode host stream work without a device."""
import glob
import json
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = sorted(glob.glob(os.path.join(ROOT, "include", "*.h")))


@pytest.fixture(scope="module")
def G():
    import cil_cuda_gb300 as G
    if not os.path.exists(G.LIB_PATH):
        from cil_cuda_gb300 import build
        build.build()
    return G


def declared_functions():
    text = "".join(open(h).read() for h in HEADERS)
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cil_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    for n in ("cil_create", "cil_destroy", "cil_upload", "cil_download", "cil_step", "cil_forces",
              "cil_bins", "cil_observables", "cil_obs_reset", "cil_last_error", "cil_gsd_create",
              "cil_gsd_write_chunk", "cil_gsd_end_frame", "cil_frame_open", "cil_frame_write", "cil_frame_close"):
        assert n in names


def test_library_exports_every_declared_symbol(G):
    out = subprocess.run(["nm", "-D", "--defined-only", G.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    lib = G.lib()
    for n in declared_functions():
        assert hasattr(lib, n)


def test_version(G):
    assert "sm_103a" in G.version()


def test_bad_configs_rejected_without_device(G):
    import ctypes as C
    lib = G.lib()
    p = G.make_params(dim=2, force_law=0, box=[10, 10, 0], periodic=[1, 1, 0], zeta=[1, 1], dt=1e-4,
                      rcut_scale=1.0)
    caps = np.array([10], np.int32)
    h = C.c_void_p()
    for kw in (dict(dim=4), dict(num_colonies=0), dict(precision=7), dict(force_law=9)):
        cfg = G.Config(dim=2, force_law=0, precision=0, rng_mode=0, seed=0, num_colonies=1, device=0)
        for k, v in kw.items():
            setattr(cfg, k, v)
        st = lib.cil_create(C.byref(cfg), C.byref(p), caps.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(h))
        assert st == 1  # CIL_ERR_CONFIG
    # apoptosis probability per step >= 1 is refused as the reference refuses it (CIL.cuh:235)
    bad = G.make_params(dim=2, force_law=0, box=[10, 10, 0], periodic=[1, 1, 0], zeta=[1, 1], dt=1.0,
                        rcut_scale=1.0, apop_rate=2.0)
    cfg = G.Config(dim=2, force_law=0, precision=0, rng_mode=0, seed=0, num_colonies=1, device=0)
    assert lib.cil_create(C.byref(cfg), C.byref(bad), caps.ctypes.data_as(C.POINTER(C.c_int32)),
                          C.byref(h)) == 1


def test_host_stream_matches_reference_golden(G):
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "dsfmt_random_golden.json")))
    for s, rec in g["seeds"].items():
        for kind in ("close_open", "open_open", "uniform", "normal"):
            np.testing.assert_array_equal(G.host_rng_draw(int(s), kind, len(rec[kind])), np.array(rec[kind]))
        d2 = rec["on_dsphere2_then3"]["d2"]
        np.testing.assert_array_equal(G.host_rng_draw(int(s), "sphere2", len(d2)), np.array(d2))
