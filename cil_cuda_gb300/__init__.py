"""cil_cuda_gb300 — GB300 (sm_103a) cell-colony step library.

Python binding of the C ABI in include/cil_gpu.h (libcilgpu.so, built in-tree by
cil_cuda_gb300/build.py). The library is the product; this module only marshals arrays.
There is no CPU fallback: if the CUDA library is missing or no GPU is present the calls
raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcilgpu.so")

FORCE_LJ_WCA, FORCE_SOFTCORE, FORCE_HERTZ = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
RNG_PHILOX, RNG_DSFMT = 0, 1

STATUS = {0: "CIL_OK", 1: "CIL_ERR_CONFIG", 2: "CIL_ERR_CUDA", 3: "CIL_ERR_CAPACITY", 4: "CIL_ERR_NAN",
          5: "CIL_ERR_OUT_OF_BOX", 6: "CIL_ERR_TIMEOUT", 7: "CIL_ERR_STATE"}

EXPORTED = ["cil_create", "cil_destroy", "cil_upload", "cil_download", "cil_step", "cil_forces",
            "cil_bins", "cil_obs_reset", "cil_observables", "cil_timings", "cil_last_error",
            "cil_version", "cil_host_rng_draw", "cil_bin_elements_noalloc"]


class CilError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class ColonyParams(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("force_law", C.c_int32),
        ("noise_per_cell", C.c_int32),
        ("divide", C.c_int32),
        ("box", C.c_double * 3),
        ("periodic", C.c_int32 * 3),
        ("nwalls", C.c_int32),
        ("wall_dir", C.c_int32 * 2),
        ("wall_pos", C.c_double * 2),
        ("wall_E", C.c_double),
        ("epsilon", C.c_double),
        ("rcut_scale", C.c_double),
        ("zeta", C.c_double * 2),
        ("motility", C.c_double * 2),
        ("kappa", C.c_double),
        ("rest0", C.c_double),
        ("rest1", C.c_double),
        ("noise_D", C.c_double),
        ("dt", C.c_double),
        ("div_tau_mu", C.c_double),
        ("div_tau_sigma", C.c_double),
        ("apop_rate", C.c_double),
    ]


class Config(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("force_law", C.c_int32),
        ("precision", C.c_int32),
        ("rng_mode", C.c_int32),
        ("seed", C.c_uint64),
        ("num_colonies", C.c_int32),
        ("device", C.c_int32),
        ("bin_width", C.c_double),
        ("skin", C.c_double),
        ("block_size", C.c_int32),
        ("flags", C.c_int32),
    ]


class ColonyView(C.Structure):
    _fields_ = [
        ("ncells", C.c_int32),
        ("capacity", C.c_int32),
        ("ts", C.c_int32),
        ("pad", C.c_int32),
        ("pos", C.POINTER(C.c_double)),
        ("sigma", C.POINTER(C.c_double)),
        ("vel", C.POINTER(C.c_double)),
        ("t0", C.POINTER(C.c_int32)),
        ("tswitch", C.POINTER(C.c_int32)),
    ]


class Obs(C.Structure):
    _fields_ = [
        ("ncells", C.c_int32),
        ("pad", C.c_int32),
        ("mean_area", C.c_double),
        ("msd", C.c_double),
        ("vacf", C.c_double),
        ("ndiv_total", C.c_int64),
        ("napo_total", C.c_int64),
    ]


_lib = None


def lib():
    """Loads libcilgpu.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with cil_cuda_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        vp, i32, dp, ip = C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int32)
        L.cil_create.restype = i32
        L.cil_create.argtypes = [C.POINTER(Config), C.POINTER(ColonyParams), ip, C.POINTER(vp)]
        L.cil_destroy.restype = None
        L.cil_destroy.argtypes = [vp]
        L.cil_upload.restype = i32
        L.cil_upload.argtypes = [vp, i32, C.POINTER(ColonyView)]
        L.cil_download.restype = i32
        L.cil_download.argtypes = [vp, i32, C.POINTER(ColonyView)]
        L.cil_step.restype = i32
        L.cil_step.argtypes = [vp, i32, C.POINTER(C.c_int64)]
        L.cil_forces.restype = i32
        L.cil_forces.argtypes = [vp, i32, dp]
        L.cil_bins.restype = i32
        L.cil_bins.argtypes = [vp, i32, ip, ip, ip, i32]
        L.cil_obs_reset.restype = i32
        L.cil_obs_reset.argtypes = [vp, i32]
        L.cil_observables.restype = i32
        L.cil_observables.argtypes = [vp, i32, C.POINTER(Obs)]
        L.cil_timings.restype = i32
        L.cil_timings.argtypes = [vp, dp, dp, dp, dp, C.POINTER(C.c_int64)]
        L.cil_last_error.restype = None
        L.cil_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
        L.cil_version.restype = C.c_char_p
        L.cil_version.argtypes = []
        L.cil_bin_elements_noalloc.restype = i32
        L.cil_bin_elements_noalloc.argtypes = [vp, i32, i32, dp, C.c_double, ip, vp, vp, i32, vp]
        L.cil_host_rng_draw.restype = i32
        L.cil_host_rng_draw.argtypes = [C.c_uint32, i32, C.c_int64, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def make_params(**kw) -> ColonyParams:
    p = ColonyParams()
    for k, v in kw.items():
        f = getattr(p, k)
        if isinstance(f, C.Array):
            for i, x in enumerate(v):
                f[i] = x
        else:
            setattr(p, k, v)
    return p


class Engine:
    """One handle: B colonies stepped together on one GPU."""

    def __init__(self, params: list, caps: list, *, precision: int = PREC_FP64, rng: int = RNG_PHILOX,
                 seed: int = 0, device: int = 0, bin_width: float = 0.0, skin: float = 0.0):
        self.L = lib()
        self.B = len(params)
        self.dim = params[0]["dim"]
        self.caps = [int(c) for c in caps]
        cfg = Config(dim=self.dim, force_law=params[0]["force_law"], precision=precision, rng_mode=rng,
                     seed=seed, num_colonies=self.B, device=device, bin_width=bin_width, skin=skin,
                     block_size=0, flags=0)
        arr = (ColonyParams * self.B)(*[make_params(**p) for p in params])
        caps_a = np.array(self.caps, np.int32)
        h = C.c_void_p()
        st = self.L.cil_create(C.byref(cfg), arr, _ip(caps_a), C.byref(h))
        if st != 0:
            raise CilError(st, "cil_create failed")
        self.h = h

    def _check(self, st: int):
        if st != 0:
            buf = C.create_string_buffer(512)
            self.L.cil_last_error(self.h, buf, 512)
            raise CilError(st, buf.value.decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.cil_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, colony: int, pos, sigma, t0, tswitch, ts: int = 0):
        pos = np.ascontiguousarray(pos, np.float64)
        sigma = np.ascontiguousarray(sigma, np.float64)
        t0 = np.ascontiguousarray(t0, np.int32)
        tswitch = np.ascontiguousarray(tswitch, np.int32)
        v = ColonyView(ncells=sigma.shape[0], capacity=sigma.shape[0], ts=ts, pad=0, pos=_dp(pos),
                       sigma=_dp(sigma), vel=None, t0=_ip(t0), tswitch=_ip(tswitch))
        self._check(self.L.cil_upload(self.h, colony, C.byref(v)))

    def step(self, n: int = 1) -> int:
        ts = C.c_int64()
        self._check(self.L.cil_step(self.h, n, C.byref(ts)))
        return ts.value

    def forces(self, colony: int = 0) -> np.ndarray:
        n = self.download(colony, want=("ncells",))["ncells"]
        out = np.zeros((n, 2, self.dim))
        self._check(self.L.cil_forces(self.h, colony, _dp(out)))
        return out

    def bins(self, colony: int = 0, max_bins: int = 1 << 24):
        ns = np.zeros(3, np.int32)
        start = np.zeros(max_bins + 1, np.int32)
        cap = 2 * self.caps[colony]
        elems = np.zeros(max(cap, 1), np.int32)
        self._check(self.L.cil_bins(self.h, colony, _ip(ns), _ip(start), _ip(elems), max_bins))
        nb = int(np.prod(ns[: self.dim]))
        start = start[: nb + 1].copy()
        return ns, start, elems[: start[-1]].copy()

    def download(self, colony: int = 0, want=("pos", "sigma", "vel", "t0", "tswitch")) -> dict:
        cap = self.caps[colony]
        D = self.dim
        pos = np.zeros((cap, 2, D))
        sig = np.zeros((cap, 2))
        vel = np.zeros((cap, 2, D))
        t0 = np.zeros(cap, np.int32)
        tsw = np.zeros(cap, np.int32)
        v = ColonyView(ncells=0, capacity=cap, ts=0, pad=0, pos=_dp(pos), sigma=_dp(sig), vel=_dp(vel),
                       t0=_ip(t0), tswitch=_ip(tsw))
        self._check(self.L.cil_download(self.h, colony, C.byref(v)))
        n = v.ncells
        out = dict(ncells=n, ts=v.ts, pos=pos[:n], sigma=sig[:n], vel=vel[:n], t0=t0[:n], tswitch=tsw[:n])
        return {k: out[k] for k in out if k in want or k in ("ncells", "ts")}

    def obs_reset(self, colony: int = 0):
        self._check(self.L.cil_obs_reset(self.h, colony))

    def observables(self, colony: int = 0) -> dict:
        o = Obs()
        self._check(self.L.cil_observables(self.h, colony, C.byref(o)))
        return dict(ncells=o.ncells, mean_area=o.mean_area, msd=o.msd, vacf=o.vacf,
                    ndiv_total=o.ndiv_total, napo_total=o.napo_total)

    def timings(self) -> dict:
        a, b, c, t = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        n = C.c_int64()
        self._check(self.L.cil_timings(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(t), C.byref(n)))
        return dict(rebuild_ms=a.value, force_ms=b.value, events_ms=c.value, total_ms=t.value,
                    launches=n.value)


def host_rng_draw(seed: int, kind: str, n: int) -> np.ndarray:
    """Draws from the oracle-mode host stream (no GPU needed)."""
    k = {"close_open": 0, "open_open": 1, "uniform": 2, "normal": 3, "sphere2": 4, "sphere3": 5}[kind]
    width = 2 if k == 4 else (3 if k == 5 else 1)
    out = np.zeros(n * width)
    st = lib().cil_host_rng_draw(seed, k, n, _dp(out))
    if st != 0:
        raise CilError(st, "cil_host_rng_draw failed")
    return out.reshape(n, width) if width > 1 else out


def version() -> str:
    return lib().cil_version().decode()
