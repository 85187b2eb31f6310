"""The reference-side C++ plug-in (cil_cuda_gb300/host/gpu_euler.hpp) driven by a
reference-shaped main loop (frames of GTS mdStep calls), compiled with g++ against
libcilgpu.so, in oracle mode, against the oracle."""
import os
import struct
import subprocess
import tempfile

import numpy as np
import pytest

from cil_cuda_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_plugin_matches_oracle(gpu_lib, oracle_lib, tmp_path):
    libdir = os.path.dirname(gpu_lib.LIB_PATH)
    exe = tmp_path / "demo"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "cil_cuda_gb300", "host"),
                    os.path.join(ROOT, "cil_cuda_gb300", "host", "demo_main.cpp"),
                    "-L", libdir, "-lcilgpu", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    p = S.growth_params(box=60.0, dt=1e-3, div_tau_mu=0.03, div_tau_sigma=0.005, apop_rate=2.0)
    st = S.disk_colony(300, p, seed=8)
    n, cap = 300, 3000
    q = [p["force_law"], p["divide"], p["box"][0], p["box"][1], 0.0, p["epsilon"], p["rcut_scale"],
         p["motility"][0], p["motility"][1], p["kappa"], p["rest0"], p["rest1"], p["noise_D"], p["dt"],
         p["div_tau_mu"], p["div_tau_sigma"], p["apop_rate"]]
    fin = tmp_path / "in.bin"
    with open(fin, "wb") as f:
        f.write(struct.pack("iii", n, 2, cap))
        f.write(struct.pack("17d", *q))
        f.write(st["pos"].astype(np.float64).tobytes())
        f.write(st["sigma"].astype(np.float64).tobytes())
        f.write(st["t0"].astype(np.int32).tobytes())
        f.write(st["tswitch"].astype(np.int32).tobytes())
    fout = tmp_path / "out.bin"
    frames, gts, seed = 4, 25, 31
    fgsd = tmp_path / "frames.gsd"
    r = subprocess.run([str(exe), str(fin), str(fout), str(frames), str(gts), str(seed), str(fgsd)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = open(fout, "rb").read()
    ng, ts = struct.unpack_from("ii", raw, 0)
    off = 8
    pos = np.frombuffer(raw, np.float64, ng * 4, off).reshape(ng, 2, 2)
    off += ng * 32
    sig = np.frombuffer(raw, np.float64, ng * 2, off).reshape(ng, 2)
    off += ng * 16 + ng * 32
    t0 = np.frombuffer(raw, np.int32, ng, off)
    tsw = np.frombuffer(raw, np.int32, ng, off + 4 * ng)

    o = oracle_lib.Oracle(p, cap, seed)
    o.set_state(**st)
    assert o.step(frames * gts) == 0
    s = o.state()
    assert ts == frames * gts
    assert ng == len(s["sigma"]) and ng != n
    np.testing.assert_array_equal(t0, s["t0"])
    np.testing.assert_array_equal(tsw, s["tswitch"])
    np.testing.assert_array_equal(sig, s["sigma"])
    d = pos - s["pos"]
    d -= np.round(d / 60.0) * 60.0
    assert np.abs(d).max() <= 1e-9
    # the GSD frames written along the way: the last one is the final state
    from cil_cuda_gb300.gsd import GSDFile
    g = GSDFile(str(fgsd))
    assert g.nframes == frames + 1
    assert [int(g.read(k, "configuration/step")[0]) for k in range(g.nframes)] == [k * gts for k in range(frames + 1)]
    assert int(g.read(0, "particles/N")[0]) == 2 * n and int(g.read(frames, "particles/N")[0]) == 2 * ng
    exp = (pos.reshape(-1, 2) - 30.0).astype(np.float32)
    np.testing.assert_array_equal(g.read(frames, "particles/position")[:, :2], exp)
    np.testing.assert_array_equal(g.read(frames, "particles/diameter"), sig.reshape(-1).astype(np.float32))
