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

FORCE_LJ_WCA, FORCE_SOFTCORE, FORCE_HERTZ, FORCE_SC = 0, 1, 2, 3
PREC_FP64, PREC_MIXED = 0, 1
RNG_PHILOX, RNG_DSFMT = 0, 1
FLAG_NO_GRAPH = 1
FLAG_DEFERRED_STATUS = 2
FLAG_REBUILD_NODE = 4
INTEGRATOR_EULER, INTEGRATOR_HEUN = 0, 1
INTRA_SPRING, INTRA_FENE = 0, 1

STATUS = {0: "CIL_OK", 1: "CIL_ERR_CONFIG", 2: "CIL_ERR_CUDA", 3: "CIL_ERR_CAPACITY", 4: "CIL_ERR_NAN",
          5: "CIL_ERR_OUT_OF_BOX", 6: "CIL_ERR_TIMEOUT", 7: "CIL_ERR_STATE", 8: "CIL_ERR_IO"}

EXPORTED = ["cil_create", "cil_destroy", "cil_upload", "cil_download", "cil_step", "cil_forces", "cil_host_register",
            "cil_host_unregister",
            "cil_bins", "cil_obs_reset", "cil_observables", "cil_timings", "cil_last_error",
            "cil_version", "cil_host_rng_draw", "cil_bin_elements_noalloc", "cil_skin_stats",
            "cil_set_skin", "cil_set_scheduler", "cil_sched_state", "cil_mlp_num_params",
            "cil_mlp_workspace_floats", "cil_mlp_forward", "cil_mlp_grad", "cil_mlp_adam",
            "cil_graph_info", "cil_gsd_create", "cil_gsd_write_chunk", "cil_gsd_end_frame", "cil_gsd_nframes",
            "cil_gsd_close", "cil_gsd_last_error", "cil_frame_open", "cil_frame_write", "cil_frame_flush",
            "cil_frame_close", "cil_frame_get_stats", "cil_frame_last_error", "cil_input_load", "cil_input_config",
            "cil_input_initial_state", "cil_input_last_error", "cil_input_free", "cil_cycle_create",
            "cil_cycle_destroy", "cil_cycle_upload", "cil_cycle_step", "cil_cycle_check_positions",
            "cil_cycle_download", "cil_cycle_timings", "cil_cycle_last_error", "cil_input_elements",
            "cil_input_cycle_config", "cil_input_cycle_initial_state", "cil_h5_shape", "cil_h5_read",
            "cil_h5_last_error", "cil_h5_write_state", "cil_h5_attr", "cil_h5_frames_create", "cil_h5_frames_write",
            "cil_h5_frames_close"]


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
        ("staging", C.c_int32),
        ("occupancy", C.c_int32),
        ("integrator", C.c_int32),
        ("rng_stream_base", C.c_int32),
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
        ("cell_state", C.POINTER(C.c_int32)),
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


class SkinInfo(C.Structure):
    _fields_ = [
        ("skin", C.c_double),
        ("interval", C.c_int32),
        ("nrebuild", C.c_int32),
        ("ntrip", C.c_int32),
        ("last_interval", C.c_int32),
        ("nfresh", C.c_int32),
        ("list_overflow", C.c_int32),
        ("npairs", C.c_int64),
        ("max_disp", C.c_double),
    ]


class SchedInfo(C.Structure):
    _fields_ = [
        ("features", C.c_float * 12),
        ("div_rate", C.c_float),
        ("apo_rate", C.c_float),
        ("trip_share", C.c_float),
        ("nsched", C.c_int32),
    ]


class FrameOptions(C.Structure):
    _fields_ = [
        ("cell_name", C.c_char_p),
        ("elem_names", C.c_char_p * 2),
        ("length_unit", C.c_double),
        ("lz", C.c_double),
        ("flags", C.c_int32),
        ("pad", C.c_int32),
    ]


class FrameStats(C.Structure):
    _fields_ = [
        ("frames_queued", C.c_int64),
        ("frames_written", C.c_int64),
        ("d2h_bytes", C.c_int64),
        ("file_bytes", C.c_int64),
        ("enqueue_ms", C.c_double),
        ("slot_wait_ms", C.c_double),
        ("write_ms", C.c_double),
        ("pack_ms", C.c_double),
        ("copy_ms", C.c_double),
    ]


class RunInfo(C.Structure):
    _fields_ = [
        ("gts", C.c_int32),
        ("frames", C.c_int32),
        ("output_gsd", C.c_int32),
        ("output_h5", C.c_int32),
        ("ncells", C.c_int32),
        ("capacity", C.c_int32),
        ("use_scheduler", C.c_int32),
        ("seed", C.c_int32),
        ("output_dir", C.c_char * 256),
        ("output_name", C.c_char * 256),
        ("cell_name", C.c_char * 64),
        ("elem_names", (C.c_char * 64) * 2),
    ]


FRAME_TYPES_IN_FIRST = 1
APOP_NONE, APOP_CYCLE_PRESSURE, APOP_PRESSURE_TIME, APOP_RATE, APOP_CYCLE, APOP_CYCLE_EXTRUDE = 0, 1, 2, 3, 4, 5
CYCLE_EULER, CYCLE_DPD = 0, 1
CYCLE_NO_GRAPH = 1

CYCLE_FIELDS = [
    ("dim", C.c_int32), ("periodic", C.c_int32 * 3), ("box", C.c_double * 3), ("dt", C.c_double),
    ("sigma_core", C.c_double), ("E", C.c_double), ("nu", C.c_double), ("adhesion", C.c_double),
    ("motility", C.c_double), ("zeta", C.c_double), ("zeta_p", C.c_double), ("zeta_p_beta", C.c_double),
    ("noise_D", C.c_double), ("divide", C.c_int32), ("apoptosis", C.c_int32),
    ("tau_div_mu", C.c_double), ("tau_div_sigma", C.c_double), ("tau_mig_mu", C.c_double),
    ("tau_mig_sigma", C.c_double), ("v1", C.c_double), ("cycle_tau_r", C.c_double), ("cycle_tau_v", C.c_double),
    ("cycle_tau_p", C.c_double), ("cycle_sigma_min", C.c_double), ("cycle_p0", C.c_double),
    ("cycle_beta_vs", C.c_double), ("cycle_rho_ratio", C.c_double), ("cycle_r_maxed", C.c_double),
    ("cycle_p_shift", C.c_double), ("cycle_p_shift_tau", C.c_double), ("osmotic_pressure", C.c_double),
    ("apop_pressure", C.c_double), ("apop_duration", C.c_double), ("apop_rate", C.c_double),
    ("extr_gamma", C.c_double), ("drain", C.c_int32), ("precision", C.c_int32),
    ("integrator", C.c_int32), ("flags", C.c_int32), ("mass", C.c_double), ("kbt", C.c_double),
    ("dis_same", C.c_double), ("dis_diff", C.c_double), ("dis_bg", C.c_double), ("extr_rate", C.c_double),
]


class CycleParams(C.Structure):
    _fields_ = CYCLE_FIELDS


class CycleView(C.Structure):
    _fields_ = [("ncells", C.c_int32), ("capacity", C.c_int32), ("ts", C.c_int32), ("pad", C.c_int32)] + [
        (k, C.POINTER(C.c_double)) for k in ("pos", "vel", "sigma", "sigma_t", "theta", "rho", "angvel", "pressure")
    ] + [("tpressure", C.POINTER(C.c_int32))] + [
        (k, C.POINTER(C.c_double)) for k in ("force", "force_dis", "force_ran")
    ] + [("t0", C.POINTER(C.c_int32)), ("pad2", C.c_int32)]


class H5State(C.Structure):
    _fields_ = [("ncells", C.c_int32), ("nelem", C.c_int32), ("dim", C.c_int32), ("pad", C.c_int32)] + [
        (k, C.POINTER(C.c_double)) for k in ("pos", "vel", "force", "force_dis", "force_ran", "sigma", "rho", "theta",
                                             "pressure")
    ] + [("state", C.POINTER(C.c_int32)), ("t0", C.POINTER(C.c_int32)), ("cpu_time", C.c_double)]


def _h5_check(L, st: int):
    if st != 0:
        buf = C.create_string_buffer(1024)
        L.cil_h5_last_error(buf, 1024)
        raise CilError(st, buf.value.decode())


def h5_read(path: str, dataset: str) -> np.ndarray:
    """A dataset of an HDF5 final-state file (the reference's <NAME>.Last.h5) as float64, read by
    the library's own reader (cil_h5_read, include/cil_input.h)."""
    L = lib()
    rank = C.c_int32()
    dims = (C.c_int64 * 8)()
    _h5_check(L, L.cil_h5_shape(path.encode(), dataset.encode(), C.byref(rank), dims))
    shape = tuple(int(dims[k]) for k in range(rank.value))
    out = np.zeros(int(np.prod(shape)) if shape else 1)
    _h5_check(L, L.cil_h5_read(path.encode(), dataset.encode(), _dp(out), out.size))
    return out.reshape(shape)


def h5_attr(path: str, obj: str, name: str) -> np.ndarray:
    """A numeric attribute of an HDF5 object (cil_h5_attr)."""
    L = lib()
    out = np.zeros(64)
    n = C.c_int64()
    _h5_check(L, L.cil_h5_attr(path.encode(), obj.encode(), name.encode(), _dp(out), out.size, C.byref(n)))
    return out[:n.value].copy()


class H5Frames:
    """The HDF5 frame file (cil_h5_frames_*): /params, then /snapshots/t_<frame> per write."""

    def __init__(self, path: str, box, dt: float, gts: int):
        self.L = lib()
        b = np.ascontiguousarray(box, np.float64)
        h = C.c_void_p()
        _h5_check(self.L, self.L.cil_h5_frames_create(path.encode(), len(b), _dp(b), dt, gts, C.byref(h)))
        self.h = h

    def write(self, frame: int, ts: int, **state):
        keep, st = _h5_state(state)
        _h5_check(self.L, self.L.cil_h5_frames_write(self.h, frame, ts, C.byref(st)))

    def close(self):
        if getattr(self, "h", None):
            h, self.h = self.h, None
            _h5_check(self.L, self.L.cil_h5_frames_close(h))


def _h5_state(state: dict):
    pos = np.ascontiguousarray(state["pos"], np.float64)
    n, E, D = pos.shape
    keep = [pos]

    def d(a, shape):
        if a is None:
            return None
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float64).reshape(shape), shape), np.float64)
        keep.append(a)
        return _dp(a)

    def i(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, np.int32).reshape(n)
        keep.append(a)
        return _ip(a)

    g = state.get
    st = H5State(ncells=n, nelem=E, dim=D, pad=0, pos=_dp(pos), vel=d(g("vel"), (n, E, D)),
                 force=d(g("force"), (n, E, D)), force_dis=d(g("force_dis"), (n, E, D)),
                 force_ran=d(g("force_ran"), (n, E, D)), sigma=d(g("sigma"), (n, E)), rho=d(g("rho"), (n,)),
                 theta=d(g("theta"), (n,)), pressure=d(g("pressure"), (n,)), state=i(g("state")), t0=i(g("t0")),
                 cpu_time=float(g("cpu_time", 0.0)))
    return keep, st


def h5_write_state(path: str, pos, sigma, vel=None, force=None, force_dis=None, force_ran=None, rho=None, theta=None,
                   pressure=None, state=None, t0=None, cpu_time: float = 0.0):
    """A final-state file as outputHDF5Frame writes it with id -1 (cil_h5_write_state). pos:
    [cell][elem][dim]; sigma: [cell][elem]."""
    L = lib()
    pos = np.ascontiguousarray(pos, np.float64)
    n, E, D = pos.shape
    keep = [pos]

    def d(a, shape):
        if a is None:
            return None
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float64).reshape(shape), shape), np.float64)
        keep.append(a)
        return _dp(a)

    def i(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, np.int32).reshape(n)
        keep.append(a)
        return _ip(a)

    st = H5State(ncells=n, nelem=E, dim=D, pad=0, pos=_dp(pos), vel=d(vel, (n, E, D)), force=d(force, (n, E, D)),
                 force_dis=d(force_dis, (n, E, D)), force_ran=d(force_ran, (n, E, D)), sigma=d(sigma, (n, E)),
                 rho=d(rho, (n,)), theta=d(theta, (n,)), pressure=d(pressure, (n,)), state=i(state), t0=i(t0),
                 cpu_time=cpu_time)
    _h5_check(L, L.cil_h5_write_state(path.encode(), C.byref(st)))


def cycle_params(**kw) -> CycleParams:
    """cil_cycle_params with the reference's defaults (Cell.cuh:236-260) for what is not given."""
    base = dict(dim=2, periodic=[1, 1, 0], box=[100.0, 100.0, 0.0], dt=1e-5, sigma_core=1.1283791670955126, E=100.0,
                nu=0.5, adhesion=0.2, motility=0.0, zeta=0.01, zeta_p=0.0, zeta_p_beta=0.0, noise_D=0.0, divide=1,
                apoptosis=APOP_NONE, tau_div_mu=1.0, tau_div_sigma=0.1, tau_mig_mu=0.0, tau_mig_sigma=0.0, v1=15.0,
                cycle_tau_r=1.0, cycle_tau_v=1.0, cycle_tau_p=0.0, cycle_sigma_min=1.1283791670955126, cycle_p0=5.0,
                cycle_beta_vs=0.0, cycle_rho_ratio=1.0, cycle_r_maxed=1.0, cycle_p_shift=0.0, cycle_p_shift_tau=0.0,
                osmotic_pressure=0.0, apop_pressure=1.0, apop_duration=8.0, apop_rate=0.0, extr_gamma=0.0, drain=0,
                precision=0, integrator=CYCLE_EULER, flags=0, mass=1.0, kbt=0.0, dis_same=0.0, dis_diff=0.0,
                dis_bg=0.0, extr_rate=0.0)
    base.update(kw)
    q = CycleParams()
    for k, v in base.items():
        f = getattr(q, k)
        if isinstance(f, C.Array):
            for i, x in enumerate(v):
                f[i] = x
        else:
            setattr(q, k, v)
    return q

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
        L.cil_host_register.restype = i32
        L.cil_host_register.argtypes = [vp, C.c_size_t]
        L.cil_host_unregister.restype = i32
        L.cil_host_unregister.argtypes = [vp]
        L.cil_bin_elements_noalloc.restype = i32
        L.cil_bin_elements_noalloc.argtypes = [vp, i32, i32, dp, C.c_double, ip, vp, vp, i32, vp]
        L.cil_skin_stats.restype = i32
        L.cil_skin_stats.argtypes = [vp, i32, C.POINTER(SkinInfo)]
        L.cil_set_skin.restype = i32
        L.cil_set_skin.argtypes = [vp, i32, C.c_double, i32]
        L.cil_graph_info.restype = i32
        L.cil_graph_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.cil_set_scheduler.restype = i32
        L.cil_set_scheduler.argtypes = [vp, C.POINTER(C.c_float), C.c_double, C.c_double, i32]
        L.cil_sched_state.restype = i32
        L.cil_sched_state.argtypes = [vp, i32, C.POINTER(SchedInfo)]
        L.cil_mlp_num_params.restype = i32
        L.cil_mlp_num_params.argtypes = []
        L.cil_mlp_workspace_floats.restype = C.c_int64
        L.cil_mlp_workspace_floats.argtypes = [i32]
        L.cil_mlp_forward.restype = i32
        L.cil_mlp_forward.argtypes = [vp, vp, i32, vp]
        L.cil_mlp_grad.restype = i32
        L.cil_mlp_grad.argtypes = [vp, vp, vp, vp, i32, vp, vp, vp]
        L.cil_mlp_adam.restype = i32
        L.cil_mlp_adam.argtypes = [vp, vp, vp, vp, i32, C.c_float]
        L.cil_gsd_create.restype = i32
        L.cil_gsd_create.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_uint32, C.POINTER(vp)]
        L.cil_gsd_write_chunk.restype = i32
        L.cil_gsd_write_chunk.argtypes = [vp, C.c_char_p, i32, C.c_uint64, C.c_uint32, vp]
        L.cil_gsd_end_frame.restype = i32
        L.cil_gsd_end_frame.argtypes = [vp]
        L.cil_gsd_nframes.restype = C.c_uint64
        L.cil_gsd_nframes.argtypes = [vp]
        L.cil_gsd_close.restype = i32
        L.cil_gsd_close.argtypes = [vp]
        L.cil_gsd_last_error.restype = None
        L.cil_gsd_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
        L.cil_frame_open.restype = i32
        L.cil_frame_open.argtypes = [vp, i32, C.c_char_p, C.POINTER(FrameOptions), C.POINTER(vp)]
        L.cil_frame_write.restype = i32
        L.cil_frame_write.argtypes = [vp, C.c_int64, C.POINTER(C.c_int64)]
        L.cil_frame_flush.restype = i32
        L.cil_frame_flush.argtypes = [vp]
        L.cil_frame_close.restype = i32
        L.cil_frame_close.argtypes = [vp]
        L.cil_frame_get_stats.restype = i32
        L.cil_frame_get_stats.argtypes = [vp, C.POINTER(FrameStats)]
        L.cil_frame_last_error.restype = None
        L.cil_frame_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
        L.cil_input_load.restype = i32
        L.cil_input_load.argtypes = [C.c_char_p, i32, C.POINTER(vp)]
        L.cil_input_config.restype = i32
        L.cil_input_config.argtypes = [vp, C.POINTER(Config), C.POINTER(ColonyParams), C.POINTER(RunInfo)]
        L.cil_input_initial_state.restype = i32
        L.cil_input_initial_state.argtypes = [vp, C.POINTER(ColonyView)]
        L.cil_input_last_error.restype = None
        L.cil_input_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
        L.cil_input_free.restype = None
        L.cil_input_free.argtypes = [vp]
        L.cil_input_elements.restype = i32
        L.cil_input_elements.argtypes = [vp]
        L.cil_input_cycle_config.restype = i32
        L.cil_input_cycle_config.argtypes = [vp, C.c_void_p, C.c_void_p]
        L.cil_input_cycle_initial_state.restype = i32
        L.cil_input_cycle_initial_state.argtypes = [vp, C.c_void_p]
        L.cil_cycle_create.restype = i32
        L.cil_cycle_create.argtypes = [C.POINTER(CycleParams), i32, C.c_uint64, i32, C.POINTER(vp)]
        L.cil_cycle_destroy.restype = None
        L.cil_cycle_destroy.argtypes = [vp]
        L.cil_cycle_upload.restype = i32
        L.cil_cycle_upload.argtypes = [vp, C.POINTER(CycleView)]
        L.cil_cycle_step.restype = i32
        L.cil_cycle_step.argtypes = [vp, i32, C.POINTER(C.c_int64)]
        L.cil_cycle_check_positions.restype = i32
        L.cil_cycle_check_positions.argtypes = [vp]
        L.cil_cycle_download.restype = i32
        L.cil_cycle_download.argtypes = [vp, C.POINTER(CycleView)]
        L.cil_cycle_timings.restype = i32
        L.cil_cycle_timings.argtypes = [vp, dp, C.POINTER(C.c_int64)]
        L.cil_cycle_last_error.restype = None
        L.cil_cycle_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
        L.cil_h5_shape.restype = i32
        L.cil_h5_shape.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
        L.cil_h5_read.restype = i32
        L.cil_h5_read.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_double), C.c_int64]
        L.cil_h5_last_error.restype = None
        L.cil_h5_last_error.argtypes = [C.c_char_p, C.c_size_t]
        L.cil_h5_write_state.restype = i32
        L.cil_h5_write_state.argtypes = [C.c_char_p, C.POINTER(H5State)]
        L.cil_h5_attr.restype = i32
        L.cil_h5_attr.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_double), C.c_int64,
                                  C.POINTER(C.c_int64)]
        L.cil_h5_frames_create.restype = i32
        L.cil_h5_frames_create.argtypes = [C.c_char_p, i32, C.POINTER(C.c_double), C.c_double, i32, C.POINTER(vp)]
        L.cil_h5_frames_write.restype = i32
        L.cil_h5_frames_write.argtypes = [vp, i32, i32, C.POINTER(H5State)]
        L.cil_h5_frames_close.restype = i32
        L.cil_h5_frames_close.argtypes = [vp]
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
                 seed: int = 0, device: int = 0, bin_width: float = 0.0, skin: float = 0.0,
                 graphs: bool = True, staging: int = 0, occupancy: int = 0, integrator: int = INTEGRATOR_EULER,
                 deferred_status: bool = False, rng_stream_base: int = 0, block_size: int = 0,
                 rebuild_node: bool = False):
        self.L = lib()
        self.B = len(params)
        self.dim = params[0]["dim"]
        self.caps = [int(c) for c in caps]
        cfg = Config(dim=self.dim, force_law=params[0]["force_law"], precision=precision, rng_mode=rng,
                     seed=seed, num_colonies=self.B, device=device, bin_width=bin_width, skin=skin,
                     block_size=block_size,
                     flags=(0 if graphs else FLAG_NO_GRAPH) | (FLAG_DEFERRED_STATUS if deferred_status else 0)
                     | (FLAG_REBUILD_NODE if rebuild_node else 0),
                     staging=staging,
                     occupancy=occupancy, integrator=integrator, rng_stream_base=rng_stream_base)
        arr = (ColonyParams * self.B)(*[make_params(**p) for p in params])
        caps_a = np.array(self.caps, np.int32)
        h = C.c_void_p()
        st = self.L.cil_create(C.byref(cfg), arr, _ip(caps_a), C.byref(h))
        if st != 0:
            raise CilError(st, "cil_create failed")
        self.h = h
        self._writers = []

    def _check(self, st: int):
        if st != 0:
            buf = C.create_string_buffer(512)
            self.L.cil_last_error(self.h, buf, 512)
            raise CilError(st, buf.value.decode())

    def close(self):
        for w in list(getattr(self, "_writers", ())):
            w.close()
        if getattr(self, "h", None):
            self.L.cil_destroy(self.h)
            self.h = None

    def frame_writer(self, colony: int, path: str, *, cell_name: str = "A", elem_names=("BACK", "FRONT"),
                     length_unit: float = 1.0, lz: float = 0.0, types_in_first: bool = False) -> "FrameWriter":
        """GSD frame output of one colony (cil_frame_open, include/cil_gsd.h)."""
        w = FrameWriter(self, colony, path, cell_name=cell_name, elem_names=elem_names, length_unit=length_unit,
                        lz=lz, types_in_first=types_in_first)
        self._writers.append(w)
        return w

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, colony: int, pos, sigma, t0, tswitch, ts: int = 0, cell_state=None):
        pos = np.ascontiguousarray(pos, np.float64)
        sigma = np.ascontiguousarray(sigma, np.float64)
        t0 = np.ascontiguousarray(t0, np.int32)
        tswitch = np.ascontiguousarray(tswitch, np.int32)
        cs = None if cell_state is None else np.ascontiguousarray(cell_state, np.int32)
        v = ColonyView(ncells=sigma.shape[0], capacity=sigma.shape[0], ts=ts, pad=0, pos=_dp(pos),
                       sigma=_dp(sigma), vel=None, t0=_ip(t0), tswitch=_ip(tswitch),
                       cell_state=_ip(cs) if cs is not None else None)
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

    def download(self, colony: int = 0, want=("pos", "sigma", "vel", "t0", "tswitch", "cell_state"),
                 strict: bool = True, out: dict = None) -> dict:
        """The colony's state. strict=False keeps the state that a failed step left (its status
        under "status") instead of raising. out: caller-owned C-contiguous arrays to fill
        (pos [cap][2][dim] and sigma [cap][2] float64, t0 and tswitch [cap] int32, vel optional;
        cap = their first dimension), e.g. pinned with host_register; views of them come back."""
        D = self.dim
        if out is None:
            cap = self.caps[colony]
            pos = np.zeros((cap, 2, D))
            sig = np.zeros((cap, 2))
            vel = np.zeros((cap, 2, D))
            t0 = np.zeros(cap, np.int32)
            tsw = np.zeros(cap, np.int32)
            cst = np.zeros(cap, np.int32) if "cell_state" in want else None
        else:
            pos, sig, t0, tsw, vel = out["pos"], out["sigma"], out["t0"], out["tswitch"], out.get("vel")
            cst = out.get("cell_state")
            cap = len(pos)
            for a, dt in ((pos, np.float64), (sig, np.float64), (t0, np.int32), (tsw, np.int32)) + \
                    (((vel, np.float64),) if vel is not None else ()):
                if a.dtype != dt or not a.flags["C_CONTIGUOUS"] or len(a) != cap:
                    raise ValueError("download: out arrays must be C-contiguous, of one capacity and typed")
            if pos.shape[1:] != (2, D) or sig.shape[1:] != (2,) or (vel is not None and vel.shape[1:] != (2, D)):
                raise ValueError("download: out arrays have the wrong shape")
        v = ColonyView(ncells=0, capacity=cap, ts=0, pad=0, pos=_dp(pos), sigma=_dp(sig),
                       vel=_dp(vel) if vel is not None else None, t0=_ip(t0), tswitch=_ip(tsw),
                       cell_state=_ip(cst) if cst is not None else None)
        st = self.L.cil_download(self.h, colony, C.byref(v))
        if strict or st not in (3, 4, 5) or v.ncells > cap:
            self._check(st)
        n = v.ncells
        res = dict(ncells=n, ts=v.ts, pos=pos[:n], sigma=sig[:n], vel=vel[:n] if vel is not None else None,
                   t0=t0[:n], tswitch=tsw[:n], cell_state=cst[:n] if cst is not None else None)
        res = {k: res[k] for k in res if k in want or k in ("ncells", "ts")}
        if st != 0:
            res["status"] = st
        return res

    def obs_reset(self, colony: int = 0):
        self._check(self.L.cil_obs_reset(self.h, colony))

    def observables(self, colony: int = 0) -> dict:
        o = Obs()
        self._check(self.L.cil_observables(self.h, colony, C.byref(o)))
        return dict(ncells=o.ncells, mean_area=o.mean_area, msd=o.msd, vacf=o.vacf,
                    ndiv_total=o.ndiv_total, napo_total=o.napo_total)

    def skin_stats(self, colony: int = 0) -> dict:
        k = SkinInfo()
        self._check(self.L.cil_skin_stats(self.h, colony, C.byref(k)))
        return {f: getattr(k, f) for f, _ in SkinInfo._fields_}

    def set_skin(self, colony: int, skin: float, interval: int = 0):
        self._check(self.L.cil_set_skin(self.h, colony, skin, interval))

    def set_scheduler(self, params, skin_min: float = 0.05, interval_scale: float = 100.0,
                      use_interval: bool = True):
        """Installs the skin-scheduler network (a float32 vector of mlp_num_params() values),
        or removes it with params=None."""
        if params is None:
            self._check(self.L.cil_set_scheduler(self.h, None, 0.0, 0.0, 0))
            return
        w = np.ascontiguousarray(params, dtype=np.float32)
        if w.size != mlp_num_params():
            raise ValueError(f"expected {mlp_num_params()} parameters, got {w.size}")
        self._check(self.L.cil_set_scheduler(self.h, w.ctypes.data_as(C.POINTER(C.c_float)), skin_min,
                                             interval_scale, 1 if use_interval else 0))

    def sched_state(self, colony: int = 0) -> dict:
        q = SchedInfo()
        self._check(self.L.cil_sched_state(self.h, colony, C.byref(q)))
        return dict(features=np.array(q.features[:], dtype=np.float32), div_rate=q.div_rate,
                    apo_rate=q.apo_rate, trip_share=q.trip_share, nsched=q.nsched)

    def graph_info(self) -> dict:
        a, b = C.c_int64(), C.c_int64()
        self._check(self.L.cil_graph_info(self.h, C.byref(a), C.byref(b)))
        return dict(graph_steps=a.value, graphs_captured=b.value)

    def timings(self) -> dict:
        a, b, c, t = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        n = C.c_int64()
        self._check(self.L.cil_timings(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(t), C.byref(n)))
        return dict(rebuild_ms=a.value, force_ms=b.value, events_ms=c.value, total_ms=t.value,
                    launches=n.value)


def host_register(arr: np.ndarray):
    """Pins a C-contiguous numpy array's memory (cil_host_register), so uploads from it and
    downloads into it are direct copies; release it with host_unregister before it is freed."""
    if not arr.flags["C_CONTIGUOUS"] or arr.nbytes == 0:
        raise ValueError("host_register: a non-empty C-contiguous array is needed")
    st = lib().cil_host_register(arr.ctypes.data_as(C.c_void_p), arr.nbytes)
    if st != 0:
        raise CilError(st, "cil_host_register failed")


def host_unregister(arr: np.ndarray):
    st = lib().cil_host_unregister(arr.ctypes.data_as(C.c_void_p))
    if st != 0:
        raise CilError(st, "cil_host_unregister failed")


def host_rng_draw(seed: int, kind: str, n: int) -> np.ndarray:
    """Draws from the oracle-mode host stream (no GPU needed)."""
    k = {"close_open": 0, "open_open": 1, "uniform": 2, "normal": 3, "sphere2": 4, "sphere3": 5}[kind]
    width = 2 if k == 4 else (3 if k == 5 else 1)
    out = np.zeros(n * width)
    st = lib().cil_host_rng_draw(seed, k, n, _dp(out))
    if st != 0:
        raise CilError(st, "cil_host_rng_draw failed")
    return out.reshape(n, width) if width > 1 else out


def mlp_num_params() -> int:
    return int(lib().cil_mlp_num_params())


def _mlp_call(st, what):
    if st != 0:
        raise CilError(st, what + " failed")


def mlp_forward(params, X, Y):
    """Y[n,2] = net(X[n,12]); float32 CUDA tensors (torch), current device."""
    _mlp_call(lib().cil_mlp_forward(params.data_ptr(), X.data_ptr(), X.shape[0], Y.data_ptr()), "cil_mlp_forward")


def mlp_grad(params, X, T, out_weights, workspace, grad, loss):
    """Loss (weighted mean squared error) and its gradient; float32 CUDA tensors. workspace
    holds mlp_workspace_floats(n) floats."""
    _mlp_call(lib().cil_mlp_grad(params.data_ptr(), X.data_ptr(), T.data_ptr(), out_weights.data_ptr(),
                                 X.shape[0], workspace.data_ptr(), grad.data_ptr(), loss.data_ptr()),
              "cil_mlp_grad")


def mlp_workspace_floats(n: int) -> int:
    return int(lib().cil_mlp_workspace_floats(n))


def mlp_adam(params, grad, m, v, t: int, lr: float):
    _mlp_call(lib().cil_mlp_adam(params.data_ptr(), grad.data_ptr(), m.data_ptr(), v.data_ptr(), t, lr),
              "cil_mlp_adam")


def version() -> str:
    return lib().cil_version().decode()


class FrameWriter:
    """Device-fed GSD frame writer of one colony (include/cil_gsd.h, cil_frame_*): write()
    enqueues a pack kernel and an asynchronous copy and returns; a host thread writes the
    file. Close it (or the engine) to flush."""

    def __init__(self, engine: Engine, colony: int, path: str, *, cell_name="A", elem_names=("BACK", "FRONT"),
                 length_unit=1.0, lz=0.0, types_in_first=False):
        self.engine = engine
        self.L = engine.L
        o = FrameOptions(cell_name=cell_name.encode(), length_unit=length_unit, lz=lz,
                         flags=FRAME_TYPES_IN_FIRST if types_in_first else 0)
        o.elem_names[0] = elem_names[0].encode()
        o.elem_names[1] = elem_names[1].encode()
        w = C.c_void_p()
        engine._check(self.L.cil_frame_open(engine.h, colony, os.fsencode(path), C.byref(o), C.byref(w)))
        self.w = w
        self.path = path

    def _check(self, st: int):
        if st != 0:
            buf = C.create_string_buffer(512)
            self.L.cil_frame_last_error(self.w, buf, 512)
            msg = buf.value.decode()
            if not msg and self.engine.h:
                self.L.cil_last_error(self.engine.h, buf, 512)
                msg = buf.value.decode()
            raise CilError(st, msg)

    def write(self, step: int = -1) -> int:
        """Queues a frame of the current state; step < 0 labels it with the engine's step."""
        idx = C.c_int64()
        self._check(self.L.cil_frame_write(self.w, step, C.byref(idx)))
        return idx.value

    def flush(self):
        self._check(self.L.cil_frame_flush(self.w))

    def stats(self) -> dict:
        s = FrameStats()
        self._check(self.L.cil_frame_get_stats(self.w, C.byref(s)))
        return {k: getattr(s, k) for k, _ in FrameStats._fields_}

    def close(self):
        """Flushes and closes; the final counters stay in last_stats."""
        if getattr(self, "w", None):
            fst = self.L.cil_frame_flush(self.w)
            s = FrameStats()
            self.L.cil_frame_get_stats(self.w, C.byref(s))
            self.last_stats = {k: getattr(s, k) for k, _ in FrameStats._fields_}
            buf = C.create_string_buffer(512)
            self.L.cil_frame_last_error(self.w, buf, 512)
            w, self.w = self.w, None
            if self in self.engine._writers:
                self.engine._writers.remove(self)
            st = self.L.cil_frame_close(w)
            if fst != 0 or st != 0:
                raise CilError(fst or st, "cil_frame_close: " + buf.value.decode())

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class GSDWriter:
    """The library's GSD 1.0 file writer (cil_gsd_*): chunks of the open frame, end_frame()
    closes it. Needs no GPU."""

    def __init__(self, path: str, application: str = "CIL", schema: str = "hoomd", schema_version=(1, 1)):
        self.L = lib()
        f = C.c_void_p()
        ver = (schema_version[0] << 16) | schema_version[1]
        st = self.L.cil_gsd_create(os.fsencode(path), application.encode(), schema.encode(), ver, C.byref(f))
        if st != 0:
            raise CilError(st, f"cil_gsd_create({path}) failed")
        self.f = f

    def _check(self, st: int):
        if st != 0:
            buf = C.create_string_buffer(512)
            self.L.cil_gsd_last_error(self.f, buf, 512)
            raise CilError(st, buf.value.decode())

    def write_chunk(self, name: str, data, gsd_type: int | None = None):
        """data: numpy array of 1 or 2 dimensions (N rows x M columns)."""
        a = np.ascontiguousarray(data)
        if gsd_type is None:
            gsd_type = GSD_TYPE_OF[a.dtype.str.lstrip("<=|")]
        n = a.shape[0] if a.ndim else 1
        m = a.shape[1] if a.ndim > 1 else 1
        ptr = a.ctypes.data_as(C.c_void_p) if a.size else None
        self._check(self.L.cil_gsd_write_chunk(self.f, name.encode(), gsd_type, n, m, ptr))

    def end_frame(self):
        self._check(self.L.cil_gsd_end_frame(self.f))

    @property
    def nframes(self) -> int:
        return int(self.L.cil_gsd_nframes(self.f))

    def close(self):
        if getattr(self, "f", None):
            f, self.f = self.f, None
            st = self.L.cil_gsd_close(f)
            if st != 0:
                raise CilError(st, "cil_gsd_close failed")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


GSD_TYPE_OF = {"u1": 1, "u2": 2, "u4": 3, "u8": 4, "i1": 5, "i2": 6, "i4": 7, "i8": 8, "f4": 9, "f8": 10}


def _struct_dict(st) -> dict:
    out = {}
    for k, _ in st._fields_:
        v = getattr(st, k)
        if isinstance(v, C.Array):
            v = [x.value.decode() if isinstance(x, C.Array) else x for x in v]
        elif isinstance(v, bytes):
            v = v.decode()
        out[k] = v
    return out


class RunInput:
    """The reference's JSON run description read by the library (include/cil_input.h):
    .config (cil_config fields), .params (cil_colony_params fields, the dict Engine takes),
    .run (GTS, FRAMES, output names ...), .initial_state() (INIT, reference layout)."""

    def __init__(self, source: str, is_path: bool = True):
        self.L = lib()
        h = C.c_void_p()
        data = os.fsencode(source) if is_path else source.encode()
        st = self.L.cil_input_load(data, 1 if is_path else 0, C.byref(h))
        self.h = h
        if st != 0:
            buf = C.create_string_buffer(1024)
            self.L.cil_input_last_error(h, buf, 1024)
            self.close()
            raise CilError(st, buf.value.decode())
        self.elements = int(self.L.cil_input_elements(h))
        run = RunInfo()
        if self.elements == 1:  # single-element cells: the cell-cycle model (cil_cycle.h)
            q = CycleParams()
            self._check(self.L.cil_input_cycle_config(h, C.byref(q), C.byref(run)))
            self.config = None
            self.params = _struct_dict(q)
        else:
            cfg, prm = Config(), ColonyParams()
            self._check(self.L.cil_input_config(h, C.byref(cfg), C.byref(prm), C.byref(run)))
            self.config = _struct_dict(cfg)
            self.params = _struct_dict(prm)
        self.run = _struct_dict(run)

    def _check(self, st: int):
        if st != 0:
            buf = C.create_string_buffer(1024)
            self.L.cil_input_last_error(self.h, buf, 1024)
            raise CilError(st, buf.value.decode())

    def initial_state(self) -> dict:
        n, D = self.run["ncells"], self.config["dim"]
        pos = np.zeros((n, 2, D))
        sig = np.zeros((n, 2))
        t0 = np.zeros(n, np.int32)
        tsw = np.zeros(n, np.int32)
        cst = np.zeros(n, np.int32)
        v = ColonyView(ncells=0, capacity=n, ts=0, pad=0, pos=_dp(pos), sigma=_dp(sig), vel=None, t0=_ip(t0),
                       tswitch=_ip(tsw), cell_state=_ip(cst))
        self._check(self.L.cil_input_initial_state(self.h, C.byref(v)))
        return dict(pos=pos, sigma=sig, t0=t0, tswitch=tsw, cell_state=cst)

    def cycle_initial_state(self) -> dict:
        """INIT and the cell status of a single-element run (cil_input_cycle_initial_state)."""
        n, D = self.run["ncells"], self.params["dim"]
        a = {k: np.zeros(n) for k in ("sigma", "sigma_t", "theta", "rho", "angvel")}
        a["pos"] = np.zeros((n, D))
        a["vel"] = np.zeros((n, D))  # INIT H5 ALL restarts the velocities; zero otherwise
        v = CycleView(ncells=0, capacity=n, ts=0, pad=0, pressure=None, tpressure=None,
                      **{k: _dp(x) for k, x in a.items()})
        self._check(self.L.cil_input_cycle_initial_state(self.h, C.byref(v)))
        return a

    def cycle_engine(self, device: int = 0) -> "CycleEngine":
        return CycleEngine(self.params, self.run["capacity"], seed=self.run["seed"], device=device)

    def engine(self, device: int = 0, **over) -> Engine:
        """An Engine configured from the run description (keyword arguments override)."""
        c = self.config
        kw = dict(precision=c["precision"], rng=c["rng_mode"], seed=c["seed"], device=device, skin=c["skin"],
                  integrator=c["integrator"])
        kw.update(over)
        return Engine([self.params], [self.run["capacity"]], **kw)

    def close(self):
        if getattr(self, "h", None):
            self.L.cil_input_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CycleEngine:
    """The single-element cell-cycle model (include/cil_cycle.h) of one colony on one GPU."""

    def __init__(self, params: dict, capacity: int, *, seed: int = 0, device: int = 0):
        self.L = lib()
        self.params = dict(params)
        self.p = cycle_params(**params)
        self.dim = self.p.dim
        self.cap = int(capacity)
        h = C.c_void_p()
        st = self.L.cil_cycle_create(C.byref(self.p), self.cap, seed, device, C.byref(h))
        if st != 0:
            raise CilError(st, "cil_cycle_create failed")
        self.h = h

    def _check(self, st):
        if st != 0:
            buf = C.create_string_buffer(512)
            self.L.cil_cycle_last_error(self.h, buf, 512)
            raise CilError(st, buf.value.decode())

    def upload(self, pos, sigma=None, sigma_t=None, theta=None, rho=None, angvel=None, pressure=None,
               tpressure=None, ts: int = 0, vel=None):
        pos = np.ascontiguousarray(pos, np.float64)
        n = pos.shape[0]
        keep = []

        def ptr(a, dt=np.float64):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dt)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_double if dt == np.float64 else C.c_int32))

        v = CycleView(ncells=n, capacity=n, ts=ts, pad=0, pos=_dp(pos), vel=ptr(vel), sigma=ptr(sigma),
                      sigma_t=ptr(sigma_t), theta=ptr(theta), rho=ptr(rho), angvel=ptr(angvel),
                      pressure=ptr(pressure), tpressure=ptr(tpressure, np.int32))
        self._check(self.L.cil_cycle_upload(self.h, C.byref(v)))

    def step(self, n: int = 1) -> int:
        ts = C.c_int64()
        self._check(self.L.cil_cycle_step(self.h, n, C.byref(ts)))
        return ts.value

    def check_positions(self):
        self._check(self.L.cil_cycle_check_positions(self.h))

    def download(self) -> dict:
        cap, D = self.cap, self.dim
        a = {k: np.zeros(cap) for k in ("sigma", "sigma_t", "theta", "rho", "angvel", "pressure")}
        for k in ("pos", "vel", "force", "force_dis", "force_ran"):
            a[k] = np.zeros((cap, D))
        a["tpressure"] = np.zeros(cap, np.int32)
        a["t0"] = np.zeros(cap, np.int32)
        v = CycleView(ncells=0, capacity=cap, ts=0, pad=0, tpressure=_ip(a["tpressure"]), t0=_ip(a["t0"]),
                      **{k: _dp(a[k]) for k in ("pos", "vel", "sigma", "sigma_t", "theta", "rho", "angvel", "pressure",
                                                "force", "force_dis", "force_ran")})
        self._check(self.L.cil_cycle_download(self.h, C.byref(v)))
        n = v.ncells
        out = {k: x[:n] for k, x in a.items()}
        out["ncells"] = n
        out["ts"] = v.ts
        return out

    def timings(self) -> dict:
        t = C.c_double()
        nl = C.c_int64()
        self._check(self.L.cil_cycle_timings(self.h, C.byref(t), C.byref(nl)))
        return dict(total_ms=t.value, launches=nl.value)

    def close(self):
        if getattr(self, "h", None):
            self.L.cil_cycle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
