"""Seeded synthetic colonies with the shapes of the reference's benchmark configurations.

The reference ships no input states for its step (its stored .gsd/.h5 outputs come from a
different physics); these generators stand in for them. Conventions:

* sigma is the element diameter (the reference's sigmaCore, Utils.hpp:232-234); the
  contact distance of two elements is sigma_ij = (sigma_i + sigma_j)/2 (MD.cuh:78).
* packing fraction phi = sum over elements of pi sigma^2 / 4 divided by the area
  (2D) or sum of pi sigma^3 / 6 divided by the volume (3D).
* element 0 is the back, element 1 the front of a cell; the spring rest length is in
  absolute units (0.5 = half a nominal diameter).
"""
from __future__ import annotations

import math

import numpy as np

from . import FORCE_HERTZ, FORCE_LJ_WCA, FORCE_SOFTCORE

NEVER = 2**30  # cycle end of a cell that never divides


def base_params(dim: int, force_law: int, box, **over) -> dict:
    p = dict(dim=dim, force_law=force_law, noise_per_cell=0, divide=0,
             box=list(box) + [0.0] * (3 - len(box)), periodic=[1] * dim + [0] * (3 - dim),
             nwalls=0, wall_dir=[1, -1], wall_pos=[0.0, 0.0], wall_E=0.0,
             epsilon=1.0, rcut_scale=2 ** (1 / 6), zeta=[1.0, 1.0], motility=[0.0, 1.0],
             kappa=10.0, rest0=0.5, rest1=1.0, noise_D=0.01, dt=1e-4,
             div_tau_mu=1.0, div_tau_sigma=0.1, apop_rate=0.0,
             well_epsilon=0.0, well_sigma=0.0, force_shifted=0)
    p.update(over)
    return p


def sc_params(box=60.0, **over) -> dict:
    """The reference's soft-core cubic well (SCParams, MD.cuh:134-232) in a 2D colony: core
    energy E0 = 10, well depth Em = 0.5, well width xi = 0.3 (its SIGMA_RATIO times a unit
    diameter), the reference's rc2 = 1."""
    from . import FORCE_SC
    kw = dict(epsilon=10.0, well_epsilon=0.5, well_sigma=0.3, rcut_scale=1.0)
    kw.update(over)
    return base_params(2, FORCE_SC, [box, box], **kw)


def fene_params(box=60.0, **over) -> dict:
    """Two-element cells held by the reference's own bond (binaryCellForce, MD.cu:525-598): FENE
    above half of RMAX^2 = 1.44, the push spring below it, no contact inhibition (motility
    along the axis scaled by rss / r), the front element pulling; soft-core contacts (eps 5,
    cutoff at contact), no division. rest0 is the steady-state length rss, used only to place
    the elements."""
    from . import FORCE_SOFTCORE, INTRA_FENE
    kw = dict(epsilon=5.0, rcut_scale=1.0, intra_law=INTRA_FENE, cil=0, fene_kappa=0.2, fene_kappa_push=0.5,
              fene_spring_ratio=0.5, fene_rmax=1.2, motility=[0.0, 1.0], zeta=[1.0, 1.0])
    kw.update(over)
    p = base_params(2, FORCE_SOFTCORE, [box, box], **kw)
    zi = [1.0 / z for z in p["zeta"]]
    beta = p["motility"][0] * zi[0] + p["motility"][1] * zi[1]
    rss = math.sqrt(p["fene_rmax"] ** 2 * (1.0 - (zi[0] + zi[1]) / beta * p["fene_kappa"]))
    p.update(rest0=rss, rest1=rss)
    return p


def polydisperse(rng, n, mu=1.0, sd=0.1, lo=0.7, hi=1.3):
    """Gaussian diameters, redrawn outside [lo, hi]."""
    s = rng.normal(mu, sd, size=n)
    bad = (s < lo) | (s > hi)
    while bad.any():
        s[bad] = rng.normal(mu, sd, size=bad.sum())
        bad = (s < lo) | (s > hi)
    return s


def unit_vectors(rng, n, dim):
    if dim == 2:
        th = rng.uniform(0, 2 * np.pi, n)
        return np.stack([np.cos(th), np.sin(th)], axis=1)
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def place_cells(centres, axes, sep, box, periodic):
    """Elements at centre -/+ sep/2 along the axis, wrapped on periodic axes."""
    half = (0.5 * np.asarray(sep))[:, None] * axes
    pos = np.stack([centres - half, centres + half], axis=1)
    dim = centres.shape[1]
    for d in range(dim):
        if periodic[d]:
            pos[..., d] = np.mod(pos[..., d], box[d])
            pos[..., d] = np.where(pos[..., d] >= box[d], 0.0, pos[..., d])
    return pos


def cycle_state(rng, n, divide, dt, tau_mu=1.0, tau_sd=0.1, ts=0):
    """Birth and division steps: ages uniform over a drawn cycle length (a colony in
    steady growth), or a cycle that never ends when division is off."""
    if not divide:
        return np.full(n, ts, np.int32), np.full(n, NEVER, np.int32)
    span = np.maximum(np.rint(rng.normal(tau_mu, tau_sd, n) / dt), 1).astype(np.int64)
    age = (rng.uniform(0, 1, n) * span).astype(np.int64)
    t0 = ts - age
    return t0.astype(np.int32), (t0 + span).astype(np.int32)


def rest_lengths(p, t0, tsw, ts):
    if not p["divide"]:
        return np.full(len(t0), p["rest0"])
    span = np.maximum(tsw - t0, 1)
    frac = np.clip((ts - t0) / span, 0.0, 1.0)
    return p["rest0"] + (p["rest1"] - p["rest0"]) * frac


def config1(ncells=4096, seed=12345, phi=0.8):
    """Plain 2D periodic square, WCA-LJ, no division (first benchmark configuration)."""
    rng = np.random.default_rng(seed)
    sigma = polydisperse(rng, 2 * ncells, lo=0.5, hi=1.5).reshape(ncells, 2)
    L = math.sqrt(float(np.sum(np.pi * sigma**2 / 4)) / phi)
    p = base_params(2, FORCE_LJ_WCA, [L, L])
    centres = rng.uniform(0, L, size=(ncells, 2))
    axes = unit_vectors(rng, ncells, 2)
    t0, tsw = cycle_state(rng, ncells, False, p["dt"])
    pos = place_cells(centres, axes, np.full(ncells, p["rest0"]), p["box"], p["periodic"])
    return p, dict(pos=pos, sigma=sigma, t0=t0, tswitch=tsw)


def growth_params(box=2048.0, **over):
    """2D colony growth: soft-core eps=5 with cutoff at contact, linear growth, division,
    apoptosis 0.01/tau_d (second benchmark configuration)."""
    kw = dict(epsilon=5.0, rcut_scale=1.0, divide=1, apop_rate=0.01)
    kw.update(over)
    return base_params(2, FORCE_SOFTCORE, [box, box], **kw)


def disk_colony(ncells, p, seed=1, phi=0.8, ts=0, centre=None):
    """A grown colony: cells uniform in a central disk of packing fraction phi, random
    orientations, cycle ages uniform, rest lengths matching the ages."""
    rng = np.random.default_rng(seed)
    sigma = polydisperse(rng, 2 * ncells).reshape(ncells, 2)
    area = float(np.sum(np.pi * sigma**2 / 4)) / phi
    R = math.sqrt(area / np.pi)
    box = p["box"]
    if centre is None:
        centre = np.array([box[0] / 2, box[1] / 2])
    if 2 * R >= min(box[0], box[1]):
        raise ValueError("colony does not fit the box")
    r = R * np.sqrt(rng.uniform(0, 1, ncells))
    th = rng.uniform(0, 2 * np.pi, ncells)
    centres = centre + np.stack([r * np.cos(th), r * np.sin(th)], axis=1)
    axes = unit_vectors(rng, ncells, 2)
    t0, tsw = cycle_state(rng, ncells, p["divide"], p["dt"], p["div_tau_mu"], p["div_tau_sigma"], ts)
    sep = rest_lengths(p, t0, tsw, ts)
    pos = place_cells(centres, axes, sep, box, p["periodic"])
    return dict(pos=pos, sigma=sigma, t0=t0, tswitch=tsw)


def square_colony(ncells, p, seed=1, phi=0.8, ts=0):
    """Cells uniform in a periodic square sized for packing fraction phi."""
    rng = np.random.default_rng(seed)
    sigma = polydisperse(rng, 2 * ncells).reshape(ncells, 2)
    L = math.sqrt(float(np.sum(np.pi * sigma**2 / 4)) / phi)
    p = dict(p)
    p["box"] = [L, L, 0.0]
    centres = rng.uniform(0, L, size=(ncells, 2))
    axes = unit_vectors(rng, ncells, 2)
    t0, tsw = cycle_state(rng, ncells, p["divide"], p["dt"], p["div_tau_mu"], p["div_tau_sigma"], ts)
    sep = rest_lengths(p, t0, tsw, ts)
    pos = place_cells(centres, axes, sep, p["box"], p["periodic"])
    return p, dict(pos=pos, sigma=sigma, t0=t0, tswitch=tsw)


def channel_params(lxy=1024.0, height=20.0, **over):
    """3D Hertzian channel: E=100, walls at z=0 and z=height (third configuration)."""
    kw = dict(epsilon=100.0, rcut_scale=1.0, divide=1, apop_rate=0.01, dt=5e-5, noise_D=0.005,
              periodic=[1, 1, 0], nwalls=2, wall_dir=[1, -1], wall_pos=[0.0, height], wall_E=100.0)
    kw.update(over)
    return base_params(3, FORCE_HERTZ, [lxy, lxy, height], **kw)


def channel_colony(ncells, p, seed=1, phi=0.6, ts=0):
    """Cells on a jittered cubic lattice filling a slab of the channel at packing
    fraction phi, isotropic orientations, sigma uniform on [0.9, 1.1]."""
    rng = np.random.default_rng(seed)
    sigma = rng.uniform(0.9, 1.1, size=(ncells, 2))
    vol = float(np.sum(np.pi * sigma**3 / 6)) / phi
    lx, ly, lz = p["box"]
    h = min(lz - 1.5, (vol / (lx * ly)))
    a = (lx * ly * h / ncells) ** (1 / 3)
    nx, ny = max(1, int(lx / a)), max(1, int(ly / a))
    nz = int(math.ceil(ncells / (nx * ny)))
    idx = np.arange(ncells)
    ix, iy, iz = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    zs = 0.75 + (iz + 0.5) * (lz - 1.5) / max(nz, 1)
    centres = np.stack([(ix + 0.5) * lx / nx, (iy + 0.5) * ly / ny, zs], axis=1)
    centres[:, :2] += rng.uniform(-0.1, 0.1, size=(ncells, 2)) * a
    axes = unit_vectors(rng, ncells, 3)
    t0, tsw = cycle_state(rng, ncells, p["divide"], p["dt"], p["div_tau_mu"], p["div_tau_sigma"], ts)
    sep = rest_lengths(p, t0, tsw, ts)
    pos = place_cells(centres, axes, sep, p["box"], p["periodic"])
    pos[..., 2] = np.clip(pos[..., 2], 0.5, lz - 0.5)
    return dict(pos=pos, sigma=sigma, t0=t0, tswitch=tsw)


def relax(p, state, stages=9, steps=300, final=1000, E=1000.0, seed=0, device=0):
    """Removes inter-cell overlaps of a random start: the diameters are inflated from 60 %
    to 100 % in `stages` stages while a stiff Hertz repulsion (no noise, no motility, no
    division) relaxes the packing, then `final` steps at full size. Runs on the GPU through
    the library. Returns a copy of the state with relaxed positions."""
    from . import FORCE_HERTZ as HZ
    from . import PREC_FP64, RNG_PHILOX, Engine

    q = dict(p)
    q.update(force_law=HZ, epsilon=E, rcut_scale=1.0, noise_D=0.0, motility=[0.0, 0.0], divide=0,
             apop_rate=0.0, dt=min(1e-3, 0.3 / E), nwalls=0)
    n = len(state["sigma"])
    eng = Engine([q], [n], precision=PREC_FP64, rng=RNG_PHILOX, seed=seed, device=device)
    pos = np.asarray(state["pos"], np.float64)
    try:
        lams = list(np.linspace(0.6, 1.0, stages)) + [1.0]
        for k, lam in enumerate(lams):
            eng.upload(0, pos, np.asarray(state["sigma"]) * lam, np.zeros(n, np.int32), np.full(n, NEVER, np.int32))
            eng.step(final if k == len(lams) - 1 else steps)
            pos = eng.download(0)["pos"]
    finally:
        eng.close()
    s = dict(state)
    s["pos"] = pos
    return s


def batched_sweep(ncolonies=256, seed=2024, cells_lo=1000, cells_hi=64000, steps=5000, dt=1e-4):
    """The batched sweep (fourth configuration): colonies of log-uniform size in
    [cells_lo, cells_hi], each in its own periodic square at packing fraction 0.8, soft-core
    growth physics with motility U[0.1, 2] and division time log-U[0.3, 3] (sd 10 %),
    apoptosis 0.01/tau. Returns (params, states, capacities); capacities cover the growth
    over `steps` steps with a 25 % margin."""
    rng = np.random.default_rng(seed)
    out_p, out_s, caps = [], [], []
    for k in range(ncolonies):
        n = int(round(math.exp(rng.uniform(math.log(cells_lo), math.log(cells_hi)))))
        tau = math.exp(rng.uniform(math.log(0.3), math.log(3.0)))
        p = growth_params(box=1.0, dt=dt, div_tau_mu=tau, div_tau_sigma=0.1 * tau, apop_rate=0.01 / tau,
                          motility=[0.0, float(rng.uniform(0.1, 2.0))])
        p, st = square_colony(n, p, seed=int(rng.integers(1, 2**31 - 1)))
        growth = 2.0 ** (steps * dt / tau)
        out_p.append(p)
        out_s.append(st)
        caps.append(int(n * growth * 1.25) + 64)
    return out_p, out_s, caps
