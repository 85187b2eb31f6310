"""ORACLE — test infrastructure only.

ctypes wrapper around oracle/_build/liboracle.so, the CPU restatement of the reference's
cell-colony step (see oracle/cil_oracle.h for what is pinned against the reference and
what is "parity unpinned"). Only tests/, __graft_entry__.smoke() and bench.py's CPU legs
import this module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

FORCE_LJ_WCA, FORCE_SOFTCORE, FORCE_HERTZ, FORCE_SC = 0, 1, 2, 3


class OraParams(C.Structure):
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
        ("well_epsilon", C.c_double),
        ("well_sigma", C.c_double),
        ("force_shifted", C.c_int32),
        ("intra_law", C.c_int32),
        ("cil", C.c_int32),
        ("fene_kappa", C.c_double),
        ("fene_kappa_push", C.c_double),
        ("fene_spring_ratio", C.c_double),
        ("fene_rmax", C.c_double),
        ("fene_rmax_division", C.c_double),
        ("growth_k0", C.c_double * 2),
        ("growth_k1", C.c_double * 2),
        ("growth_k2", C.c_double * 2),
        ("div_r0", C.c_double),
        ("div_rmin", C.c_double),
        ("div_rmin_ratio", C.c_double),
        ("mig_tau_mu", C.c_double),
        ("mig_tau_sigma", C.c_double),
        ("sigma_core", C.c_double * 2),
        ("noise_radial", C.c_double),
        ("noise_angular", C.c_double),
        ("div_swelling", C.c_int32),
        ("pad_swell", C.c_int32),
    ]


class OraEvent(C.Structure):
    _fields_ = [("ts", C.c_int32), ("kind", C.c_int32), ("a", C.c_int32), ("b", C.c_int32)]


class OraObs(C.Structure):
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


def build() -> str:
    subprocess.run(["bash", os.path.join(HERE, "build.sh")], check=True, capture_output=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp, i32, u32, dp, ip = C.c_void_p, C.c_int32, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_int32)
        L.ora_create.restype = vp
        L.ora_create.argtypes = [C.POINTER(OraParams), i32, u32]
        L.ora_destroy.argtypes = [vp]
        L.ora_set_threads.argtypes = [vp, i32]
        L.ora_set_integrator.restype = None
        L.ora_set_integrator.argtypes = [vp, i32]
        L.ora_set_state.restype = i32
        L.ora_set_state.argtypes = [vp, i32, dp, dp, ip, ip, i32]
        L.ora_num_cells.restype = i32
        L.ora_num_cells.argtypes = [vp]
        L.ora_timestep.restype = i32
        L.ora_timestep.argtypes = [vp]
        L.ora_get_state.argtypes = [vp, dp, dp, dp, dp, ip, ip]
        L.ora_set_cell_states.restype = None
        L.ora_set_cell_states.argtypes = [vp, i32, ip]
        L.ora_get_cell_states.restype = None
        L.ora_get_cell_states.argtypes = [vp, ip]
        L.ora_compute_forces.argtypes = [vp]
        L.ora_step.restype = i32
        L.ora_step.argtypes = [vp, i32]
        L.ora_bin_elements.restype = i32
        L.ora_bin_elements.argtypes = [vp, C.c_double, ip, ip, ip, i32]
        L.ora_num_events.restype = i32
        L.ora_num_events.argtypes = [vp]
        L.ora_get_events.argtypes = [vp, C.POINTER(OraEvent)]
        L.ora_clear_events.argtypes = [vp]
        L.ora_obs_reset.argtypes = [vp]
        L.ora_observables.argtypes = [vp, C.POINTER(OraObs)]
        L.ora_rng_seed.argtypes = [vp, u32]
        for name in ("ora_rng_close_open", "ora_rng_open_open", "ora_rng_uniform", "ora_rng_normal"):
            getattr(L, name).restype = C.c_double
            getattr(L, name).argtypes = [vp]
        L.ora_rng_on_dsphere.argtypes = [vp, i32, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def make_params(**kw) -> OraParams:
    p = OraParams()
    for k, v in kw.items():
        f = getattr(p, k)
        if isinstance(f, C.Array):
            for i, x in enumerate(v):
                f[i] = x
        else:
            setattr(p, k, v)
    return p


class Oracle:
    """One colony on the CPU, reference layout pos[cell][elem][dim]."""

    def __init__(self, params: dict, cap_cells: int, seed: int, threads: int = 0, integrator: int = 0):
        self.L = lib()
        self.params = make_params(**params)
        self.dim = params["dim"]
        self.h = self.L.ora_create(C.byref(self.params), cap_cells, seed)
        if not self.h:
            raise ValueError("ora_create failed")
        self.L.ora_set_threads(self.h, threads)
        self.L.ora_set_integrator(self.h, integrator)

    def close(self):
        if self.h:
            self.L.ora_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, pos, sigma, t0, tswitch, ts=0, cell_state=None):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        sigma = np.ascontiguousarray(sigma, dtype=np.float64)
        t0 = np.ascontiguousarray(t0, dtype=np.int32)
        tswitch = np.ascontiguousarray(tswitch, dtype=np.int32)
        n = sigma.shape[0]
        rc = self.L.ora_set_state(self.h, n, _dp(pos), _dp(sigma), _ip(t0), _ip(tswitch), ts)
        if rc != 0:
            raise ValueError(f"ora_set_state rc={rc}")
        if cell_state is not None:
            cs = np.ascontiguousarray(cell_state, dtype=np.int32)
            self.L.ora_set_cell_states(self.h, n, _ip(cs))

    @property
    def ncells(self) -> int:
        return self.L.ora_num_cells(self.h)

    @property
    def ts(self) -> int:
        return self.L.ora_timestep(self.h)

    def state(self) -> dict:
        n, D = self.ncells, self.dim
        pos = np.zeros((n, 2, D))
        vel = np.zeros((n, 2, D))
        frc = np.zeros((n, 2, D))
        sig = np.zeros((n, 2))
        t0 = np.zeros(n, np.int32)
        tsw = np.zeros(n, np.int32)
        self.L.ora_get_state(self.h, _dp(pos), _dp(sig), _dp(vel), _dp(frc), _ip(t0), _ip(tsw))
        cs = np.zeros(n, np.int32)
        self.L.ora_get_cell_states(self.h, _ip(cs))
        return dict(pos=pos, sigma=sig, vel=vel, frc=frc, t0=t0, tswitch=tsw, cell_state=cs)

    def compute_forces(self) -> np.ndarray:
        self.L.ora_compute_forces(self.h)
        return self.state()["frc"]

    def step(self, nsteps: int = 1) -> int:
        return self.L.ora_step(self.h, nsteps)

    def bin_elements(self, width: float, max_bins: int = 1 << 22):
        ns = np.zeros(3, np.int32)
        head = np.zeros(max_bins, np.int32)
        lst = np.zeros(2 * max(self.ncells, 1), np.int32)
        nb = self.L.ora_bin_elements(self.h, width, _ip(ns), _ip(head), _ip(lst), max_bins)
        if nb < 0:
            raise ValueError(f"too many bins: {-nb}")
        return ns, head[:nb].copy(), lst

    def events(self) -> np.ndarray:
        m = self.L.ora_num_events(self.h)
        out = (OraEvent * max(m, 1))()
        self.L.ora_get_events(self.h, out)
        return np.array([(e.ts, e.kind, e.a, e.b) for e in out[:m]], dtype=np.int64).reshape(-1, 4)

    def obs_reset(self):
        self.L.ora_obs_reset(self.h)

    def observables(self) -> dict:
        o = OraObs()
        self.L.ora_observables(self.h, C.byref(o))
        return dict(ncells=o.ncells, mean_area=o.mean_area, msd=o.msd, vacf=o.vacf,
                    ndiv_total=o.ndiv_total, napo_total=o.napo_total)

    # RNG passthrough for golden-vector checks
    def rng_seed(self, s):
        self.L.ora_rng_seed(self.h, s)

    def rng(self, kind: str, n: int) -> np.ndarray:
        f = {"close_open": self.L.ora_rng_close_open, "open_open": self.L.ora_rng_open_open,
             "uniform": self.L.ora_rng_uniform, "normal": self.L.ora_rng_normal}[kind]
        return np.array([f(self.h) for _ in range(n)])

    def on_dsphere(self, dim: int, n: int) -> np.ndarray:
        out = np.zeros((n, dim))
        buf = np.zeros(dim)
        for i in range(n):
            self.L.ora_rng_on_dsphere(self.h, dim, _dp(buf))
            out[i] = buf
        return out


def bins_as_sets(head: np.ndarray, lst: np.ndarray) -> list:
    """Per-bin sets of element ids from a LIFO head/list pair."""
    out = []
    for h in head:
        s = set()
        i = int(h)
        while i >= 0:
            s.add(i)
            i = int(lst[i])
        out.append(s)
    return out


class CycleOracle:
    """The single-element cell-cycle model on the CPU (oracle/cil_cycle_oracle.cpp), with the
    GPU model's counter-based draws. Test infrastructure."""

    def __init__(self, params, capacity: int, seed: int):
        from cil_cuda_gb300 import cycle_params
        self.L = lib()
        L = self.L
        vp, i32, dp, ip = C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int32)
        L.cyo_create.restype = vp
        L.cyo_create.argtypes = [vp, i32, C.c_uint64]
        L.cyo_destroy.argtypes = [vp]
        L.cyo_set_state.argtypes = [vp, i32, i32] + [dp] * 8 + [ip]
        L.cyo_step.restype = i32
        L.cyo_step.argtypes = [vp, i32]
        L.cyo_check_positions.restype = i32
        L.cyo_check_positions.argtypes = [vp]
        L.cyo_num_cells.restype = i32
        L.cyo_num_cells.argtypes = [vp]
        L.cyo_get_state.argtypes = [vp] + [dp] * 8 + [ip, C.POINTER(C.c_int64)]
        L.cyo_get_forces.argtypes = [vp, dp, dp, dp]
        self.p = cycle_params(**params)
        self.dim = self.p.dim
        self.h = L.cyo_create(C.byref(self.p), capacity, seed)

    def set_state(self, pos, sigma, theta, rho, angvel, sigma_t=None, vel=None, pressure=None, tpressure=None, ts=0):
        def d(a):
            return None if a is None else np.ascontiguousarray(a, np.float64)
        arrs = [d(pos), d(vel), d(sigma), d(sigma_t), d(theta), d(rho), d(angvel), d(pressure)]
        tp = None if tpressure is None else np.ascontiguousarray(tpressure, np.int32)
        self._keep = (arrs, tp)
        ptrs = [None if a is None else a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]
        self.L.cyo_set_state(self.h, len(arrs[0]), ts, *ptrs,
                             None if tp is None else tp.ctypes.data_as(C.POINTER(C.c_int32)))

    def step(self, n: int) -> int:
        return self.L.cyo_step(self.h, n)

    def check_positions(self) -> int:
        return self.L.cyo_check_positions(self.h)

    def state(self) -> dict:
        n = self.L.cyo_num_cells(self.h)
        D = self.dim
        a = {k: np.zeros(n) for k in ("sigma", "sigma_t", "theta", "rho", "angvel", "pressure")}
        a["pos"] = np.zeros((n, D))
        a["vel"] = np.zeros((n, D))
        a["tpressure"] = np.zeros(n, np.int32)
        counts = np.zeros(3, np.int64)
        P = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        self.L.cyo_get_state(self.h, P(a["pos"]), P(a["vel"]), P(a["sigma"]), P(a["sigma_t"]), P(a["theta"]),
                             P(a["rho"]), P(a["angvel"]), P(a["pressure"]),
                             a["tpressure"].ctypes.data_as(C.POINTER(C.c_int32)),
                             counts.ctypes.data_as(C.POINTER(C.c_int64)))
        a.update(ncells=n, ts=int(counts[0]), ndiv=int(counts[1]), napo=int(counts[2]))
        for k in ("force", "force_dis", "force_ran"):
            a[k] = np.zeros((n, D))
        self.L.cyo_get_forces(self.h, P(a["force"]), P(a["force_dis"]), P(a["force_ran"]))
        return a

    def close(self):
        if getattr(self, "h", None):
            self.L.cyo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
