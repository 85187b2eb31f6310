"""The reference's initial configuration draws (INIT RANDOM, Input.cpp:736-757, read twice
around initializeCellStatus, CIL.cuh:253-330 and 374-378), restated step by step on top of
the reference's own Random:: functions (oracle/_ref/libref_random.so, built from the
reference's Random.cpp and vendored dSFMT by oracle/ref_build.sh). Test infrastructure: it
writes input_random_init_golden.json (make_input_golden.py) and checks the library's
cil_input_initial_state live."""
import ctypes as C
import math
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
LIB = os.path.join(ROOT, "oracle", "_ref", "libref_random.so")


def load():
    L = C.CDLL(LIB)
    for name in ("ref_uniform", "ref_close_open"):
        getattr(L, name).restype = C.c_double
    L.ref_uniform0x.restype = C.c_double
    L.ref_uniform0x.argtypes = [C.c_double]
    L.ref_normal_ms.restype = C.c_double
    L.ref_normal_ms.argtypes = [C.c_double, C.c_double]
    L.ref_init.argtypes = [C.c_int]
    return L


def nint(a):  # Utils.hpp:172-174
    return int(a + 0.5) if a >= 0.0 else int(a - 0.5)


def reference_init(seed, n, dim, box, pbc, rss, divide, const_force, tau_div, tau_mig, dt):
    L = load()
    L.ref_init(seed)

    def positions():
        pos = np.zeros((n, 2, dim))
        for i in range(n):
            for j in range(2):
                for d in range(dim):
                    pos[i, j, d] = L.ref_uniform0x(box[d])
            radius = L.ref_normal_ms(rss, 0.25 * rss)
            theta = L.ref_uniform() * math.pi
            sinphi = 1.0 if dim == 2 else L.ref_uniform() * math.pi
            z2 = 1.0 - sinphi * sinphi
            direction = [sinphi * math.cos(theta), sinphi * math.sin(theta), math.sqrt(z2) if z2 >= 0 else math.nan]
            for d in range(dim):
                r = pos[i, 1, d]
                pos[i, 1, d] = math.fmod(r + radius * direction[d] + box[d], box[d]) if pbc[d] else r + direction[d] * radius
        return pos

    positions()
    tsw = np.full(n, -1, np.int32)
    if divide:
        p_mig = tau_mig[0] / (tau_mig[0] + tau_div[0])

        def span_of(tau):
            return max(nint(L.ref_normal_ms(tau[0], tau[1]) / dt), 1)

        for i in range(n):
            if const_force:
                span = span_of(tau_mig)
            elif L.ref_uniform0x(1.0) <= p_mig:
                span = span_of(tau_mig)
            else:
                span = span_of(tau_div)
            L.ref_uniform0x(1.0)  # theta
            span -= nint(L.ref_uniform0x(float(span))) - 1
            tsw[i] = span
    pos = positions()
    return pos, tsw


def from_fixture(doc):
    """reference_init's arguments from a run description (the fixture's keys)."""
    md, sp = doc["MD"], doc["SPECIES"]
    cell = sp["DEFINE"][0]
    loc = sp[cell]
    m, z = loc["MOTILITY"], loc["FRICTION"]
    alpha = 1.0 / z[0] + 1.0 / z[1]
    beta = m[0] * (1.0 / z[0]) + m[1] * (1.0 / z[1])
    rmax, kappa = loc["FENE"]["RMAX"][0], loc["FENE"]["KAPPA_PULL"][0]
    rss = math.sqrt(rmax * rmax * (1.0 - alpha / beta * kappa))
    dv = loc["DIVISION"]
    return dict(seed=doc["RUNTIME"]["RNG"]["SEED"], n=doc["INIT"][cell]["RANDOM"]["NUMBER"], dim=md["DIM"],
                box=md["BOX"], pbc=md["PBC"], rss=rss, divide=dv["ENABLED"], const_force=dv.get("CONST_FORCE", False),
                tau_div=(dv["TAU_DIVISION"]["AVG"], dv["TAU_DIVISION"]["SIGMA"]),
                tau_mig=(dv["TAU_MIGRATION"]["AVG"], dv["TAU_MIGRATION"]["SIGMA"]), dt=md["DT"]["MANUAL"])


def reference_cycle_init(seed, n, dim, box, tau_div, dt, random=True):
    """INIT RANDOM and the cell status of a single-element species (Input.cpp:736-757 with
    one element; CIL.cuh:253-330), on the reference's Random:: functions."""
    L = load()
    L.ref_init(seed)

    def positions():
        pos = np.zeros((n, dim))
        for i in range(n):
            for d in range(dim):
                pos[i, d] = L.ref_uniform0x(box[d])
        return pos

    if random:
        positions()
    theta = np.zeros(n)
    angvel = np.zeros(n)
    for i in range(n):
        L.ref_uniform0x(1.0)  # the migration test
        span = max(nint(L.ref_normal_ms(tau_div[0], tau_div[1]) / dt), 1)
        angvel[i] = 1.0 / span
        theta[i] = L.ref_uniform0x(1.0)
        L.ref_uniform0x(float(span))
    pos = positions() if random else None
    return pos, theta, angvel
