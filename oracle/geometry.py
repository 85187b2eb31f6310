"""ORACLE — test infrastructure only: numpy calls over the box and link-list geometry.

Two libraries export the same C signatures:
  * the oracle's restatement (oracle/_build/liboracle.so, ora_geom_*);
  * the reference's own Utils.hpp compiled by oracle/ref_build.sh
    (oracle/_ref/libref_utils.so, ref_*): Nint (Utils.hpp:173-175), BoundingBox::distance /
    updatePos (Utils.hpp:536-566), LinkListOrtho2D/3D (Utils.hpp:872-1069).
Geometry(lib, prefix) wraps either, so the golden vectors the reference produces
(tests/golden/make_geometry_golden.py) and the oracle's outputs go through one code path.
The Lennard-Jones element force has one wrapper per side: lj_force_oracle (the oracle's law
table, ora_geom_pair_force) and lj_force_reference (the reference's LJParams::elemForce,
likewise the soft-core cubic well: sc_force_oracle and sc_force_reference (SCParams),
MD.cuh:98-113, in oracle/_ref/libref_force.so)."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_UTILS = os.path.join(HERE, "_ref", "libref_utils.so")


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Geometry:
    def __init__(self, lib: C.CDLL, prefix: str):
        dp, ip, i32, i64 = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_int32, C.c_int64
        self._nint = getattr(lib, prefix + "nint")
        self._nint.restype = i32
        self._nint.argtypes = [C.c_double]
        self._dist = getattr(lib, prefix + "box_distance" if prefix == "ref_" else prefix + "distance")
        self._dist.restype = None
        self._dist.argtypes = [i32, dp, ip, i64, dp, dp, dp, dp]
        self._upd = getattr(lib, prefix + "box_update_pos" if prefix == "ref_" else prefix + "update_pos")
        self._upd.restype = None
        self._upd.argtypes = [i32, dp, ip, i64, dp, dp, C.c_double]
        self._ll = getattr(lib, prefix + "link_list")
        self._ll.restype = i32
        self._ll.argtypes = [i32, C.c_double, dp, ip, i32, dp, ip, ip, ip, ip, ip, i32]

    def nint(self, a):
        return np.array([self._nint(float(x)) for x in np.asarray(a, np.float64)], np.int64)

    def distance(self, dim, box, periodic, r1, r2):
        r1 = np.ascontiguousarray(r1, np.float64).reshape(-1, dim)
        r2 = np.ascontiguousarray(r2, np.float64).reshape(-1, dim)
        n = r1.shape[0]
        box = np.ascontiguousarray(box, np.float64)
        per = np.ascontiguousarray(periodic, np.int32)
        r12 = np.zeros((n, dim))
        d2 = np.zeros(n)
        self._dist(dim, _dp(box), _ip(per), n, _dp(r1), _dp(r2), _dp(r12), _dp(d2))
        return r12, d2

    def update_pos(self, dim, box, periodic, r, v, dt):
        r = np.array(r, np.float64).reshape(-1, dim).copy()
        v = np.ascontiguousarray(v, np.float64).reshape(-1, dim)
        box = np.ascontiguousarray(box, np.float64)
        per = np.ascontiguousarray(periodic, np.int32)
        self._upd(dim, _dp(box), _ip(per), r.shape[0], _dp(r), _dp(v), float(dt))
        return r

    def link_list(self, dim, rcut, box, periodic, r, max_bins=1 << 20):
        r = np.ascontiguousarray(r, np.float64).reshape(-1, dim)
        n = r.shape[0]
        box = np.ascontiguousarray(box, np.float64)
        per = np.ascontiguousarray(periodic, np.int32)
        ns = np.zeros(3, np.int32)
        head = np.zeros(max_bins, np.int32)
        lst = np.zeros(max(n, 1), np.int32)
        nst = 5 if dim == 2 else 14
        coords = np.zeros(max_bins * dim, np.int32)
        nbr = np.zeros(max_bins * nst, np.int32)
        nb = self._ll(dim, float(rcut), _dp(box), _ip(per), n, _dp(r), _ip(ns), _ip(head), _ip(lst), _ip(coords),
                      _ip(nbr), max_bins)
        if nb < 0:
            raise ValueError(f"{-nb} bins exceed max_bins={max_bins}")
        return dict(ns=ns, head=head[:nb].copy(), list=lst[:n].copy(), coords=coords[: nb * dim].reshape(nb, dim),
                    neighbor_ids=nbr[: nb * nst].reshape(nb, nst))


def lj_force_oracle(eps, rcut_scale, r2, si, sj):
    from oracle import oracle as O
    L = O.lib()
    f = L.ora_geom_pair_force
    f.restype = None
    f.argtypes = [C.c_int32, C.c_double, C.c_double, C.c_int64] + [C.POINTER(C.c_double)] * 4 + [C.POINTER(C.c_int32)]
    r2, si, sj = (np.ascontiguousarray(a, np.float64) for a in (r2, si, sj))
    f0 = np.zeros(r2.size)
    inside = np.zeros(r2.size, np.int32)
    f(0, float(eps), float(rcut_scale), r2.size, _dp(r2), _dp(si), _dp(sj), _dp(f0), _ip(inside))
    return f0, inside


REF_FORCE = os.path.join(HERE, "_ref", "libref_force.so")


def lj_force_reference(eps, r2, si, sj):
    """The reference's LJParams::elemForce with its WCA cutoff (pow(2, 1/3), Input.cpp:296-301),
    or None when oracle/ref_build.sh has not built it here."""
    if not os.path.exists(REF_FORCE):
        return None
    L = C.CDLL(REF_FORCE)
    L.ref_lj_wca_rc2.restype = C.c_double
    f = L.ref_lj_force
    f.restype = None
    f.argtypes = [C.c_double, C.c_double, C.c_int64] + [C.POINTER(C.c_double)] * 4 + [C.POINTER(C.c_int32)]
    r2, si, sj = (np.ascontiguousarray(a, np.float64) for a in (r2, si, sj))
    f0 = np.zeros(r2.size)
    inside = np.zeros(r2.size, np.int32)
    f(float(eps), L.ref_lj_wca_rc2(), r2.size, _dp(r2), _dp(si), _dp(sj), _dp(f0), _ip(inside))
    return f0, inside


def lj_attr_force_oracle(eps, rcut, shifted, r2, si, sj):
    """The oracle's Lennard-Jones law with cutoff rcut (in sigma_ij) and the optional force shift
    (ora_geom_lj_force)."""
    from oracle import oracle as O
    L = O.lib()
    f = L.ora_geom_lj_force
    f.restype = None
    f.argtypes = [C.c_double, C.c_double, C.c_int32, C.c_int64] + [C.POINTER(C.c_double)] * 4 + [C.POINTER(C.c_int32)]
    r2, si, sj = (np.ascontiguousarray(a, np.float64) for a in (r2, si, sj))
    f0 = np.zeros(r2.size)
    inside = np.zeros(r2.size, np.int32)
    f(float(eps), float(rcut), int(shifted), r2.size, _dp(r2), _dp(si), _dp(sj), _dp(f0), _ip(inside))
    return f0, inside


def lj_attr_force_reference(eps, rcut, shifted, r2, si, sj):
    """The reference's LJParams::elemForce with ATTRACTION ON (rcut2 = RCUT^2, SHIFT FORCE when
    shifted), or None when oracle/ref_build.sh has not built it here."""
    if not os.path.exists(REF_FORCE):
        return None
    L = C.CDLL(REF_FORCE)
    f = L.ref_lj_attr_force
    f.restype = None
    f.argtypes = [C.c_double, C.c_double, C.c_int32, C.c_int64] + [C.POINTER(C.c_double)] * 4 + [C.POINTER(C.c_int32)]
    r2, si, sj = (np.ascontiguousarray(a, np.float64) for a in (r2, si, sj))
    f0 = np.zeros(r2.size)
    inside = np.zeros(r2.size, np.int32)
    f(float(eps), float(rcut), int(shifted), r2.size, _dp(r2), _dp(si), _dp(sj), _dp(f0), _ip(inside))
    return f0, inside


def sc_force_oracle(eps_core, eps_well, xi, rcut_scale, shifted, r2, si, sj):
    """The oracle's restatement of the reference's soft-core cubic well (ora_geom_sc_force)."""
    from oracle import oracle as O
    L = O.lib()
    f = L.ora_geom_sc_force
    f.restype = None
    f.argtypes = [C.c_double] * 4 + [C.c_int32, C.c_int64] + [C.POINTER(C.c_double)] * 4 + [C.POINTER(C.c_int32)]
    r2, si, sj = (np.ascontiguousarray(a, np.float64) for a in (r2, si, sj))
    f0 = np.zeros(r2.size)
    inside = np.zeros(r2.size, np.int32)
    f(float(eps_core), float(eps_well), float(xi), float(rcut_scale), int(shifted), r2.size, _dp(r2), _dp(si), _dp(sj),
      _dp(f0), _ip(inside))
    return f0, inside


def sc_force_reference(eps_core, eps_well, xi, rcut_scale, shifted, r2, si, sj):
    """The reference's SCParams::elemForce (one element type, rcut2 = rcut_scale^2), or None when
    oracle/ref_build.sh has not built it here."""
    if not os.path.exists(REF_FORCE):
        return None
    L = C.CDLL(REF_FORCE)
    f = L.ref_sc_force
    f.restype = None
    f.argtypes = [C.c_double] * 4 + [C.c_int32, C.c_int64] + [C.POINTER(C.c_double)] * 4 + [C.POINTER(C.c_int32)]
    r2, si, sj = (np.ascontiguousarray(a, np.float64) for a in (r2, si, sj))
    f0 = np.zeros(r2.size)
    inside = np.zeros(r2.size, np.int32)
    rcs = float(rcut_scale)
    f(float(eps_core), float(eps_well), float(xi), rcs * rcs, int(shifted), r2.size, _dp(r2), _dp(si), _dp(sj),
      _dp(f0), _ip(inside))
    return f0, inside


def oracle_geometry():
    from oracle import oracle as O
    return Geometry(O.lib(), "ora_geom_")


def reference_geometry():
    """The reference's own Utils.hpp, when oracle/ref_build.sh has built it here; else None."""
    if not os.path.exists(REF_UTILS):
        return None
    return Geometry(C.CDLL(REF_UTILS), "ref_")
