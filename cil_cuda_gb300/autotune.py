"""Autotuner for the step's launch parameters.

Tries, on the caller's own colonies, every combination of
  * bin size: the bin width as a factor of the smallest allowed one (largest cutoff + skin),
  * the Verlet-list force kernel's variant: chunks of 32 flattened list entries in flight per
    warp (staging depth) and CTAs per SM it is compiled for (which sets its register budget,
    hence block residency),
and times a short run of each with CUDA events (graph-replayed steps, as in production).
Every candidate runs the same physics; only the time differs. Returns the fastest settings
as keyword arguments for Engine and the table of all trials.
"""
from __future__ import annotations

import itertools

from . import Engine, PREC_MIXED, RNG_PHILOX

BIN_FACTORS = (1.0, 1.15, 1.3)
VARIANTS = ((2, 3), (1, 3), (2, 2), (1, 4))  # (chunks of 32 list entries in flight per warp, CTAs per SM)


def needed_width(params, states, skin):
    w = 0.0
    for p, st in zip(params, states):
        w = max(w, p["rcut_scale"] * float(st["sigma"].max()) + skin)
    return w


def autotune(params, states, caps, *, skin=0.3, steps=40, warmup=10, seed=3, device=0, scheduler=None,
             bin_factors=BIN_FACTORS, variants=VARIANTS):
    """scheduler: None, or a callable installing the learned scheduler into an engine."""
    base = needed_width(params, states, skin)
    trials = []
    for f, (stg, occ) in itertools.product(bin_factors, variants):
        eng = Engine(params, caps, precision=PREC_MIXED, rng=RNG_PHILOX, seed=seed, device=device, skin=skin,
                     bin_width=0.0 if f == 1.0 else f * base, staging=stg, occupancy=occ)
        try:
            for c, st in enumerate(states):
                eng.upload(c, **st)
            if scheduler is not None:
                scheduler(eng)
            eng.step(warmup)
            eng.step(steps)
            ms = eng.timings()["total_ms"] / steps
        finally:
            eng.close()
        trials.append(dict(bin_factor=f, staging=stg, occupancy=occ, ms_per_step=ms))
    best = min(trials, key=lambda t: t["ms_per_step"])
    kw = dict(bin_width=0.0 if best["bin_factor"] == 1.0 else best["bin_factor"] * base,
              staging=best["staging"], occupancy=best["occupancy"])
    return kw, trials
