"""Autotuner for the step's launch parameters.

Tries, on the caller's own colonies, every combination of
  * bin size: the bin width as a factor of the smallest allowed one (largest cutoff + skin),
  * the Verlet-list force kernel's variant: chunks of 32 flattened list entries in flight per
    warp (staging depth) and CTAs per SM it is compiled for (which sets its register budget,
    hence block residency),
then, for the fastest of those, the kernel's block size (128, 256 or 512 cells per block),
and times a short run of each with CUDA events (graph-replayed steps, as in production).
Every candidate runs the same physics; only the time differs. Returns the fastest settings
as keyword arguments for Engine and the table of all trials.
"""
from __future__ import annotations

import itertools

from . import Engine, PREC_MIXED, RNG_PHILOX

BIN_FACTORS = (1.0, 1.15, 1.3)
BLOCK_SIZES = (128, 256, 512)  # threads (cells) per block of the list force kernel; stage 1 runs the first
VARIANTS = ((4, 3), (2, 3), (1, 3), (1, 4))  # (chunks of 32 list entries in flight per warp, CTAs per SM)


def needed_width(params, states, skin):
    w = 0.0
    for p, st in zip(params, states):
        w = max(w, p["rcut_scale"] * float(st["sigma"].max()) + skin)
    return w


def _trial(params, states, caps, *, skin, steps, warmup, seed, device, scheduler, bin_width, stg, occ, block):
    eng = Engine(params, caps, precision=PREC_MIXED, rng=RNG_PHILOX, seed=seed, device=device, skin=skin,
                 bin_width=bin_width, staging=stg, occupancy=occ, block_size=block)
    try:
        for c, st in enumerate(states):
            eng.upload(c, **st)
        if scheduler is not None:
            scheduler(eng)
        eng.step(warmup)
        eng.step(steps)
        return eng.timings()["total_ms"] / steps
    finally:
        eng.close()


def autotune(params, states, caps, *, skin=0.3, steps=40, warmup=10, seed=3, device=0, scheduler=None,
             bin_factors=BIN_FACTORS, variants=VARIANTS, block_sizes=BLOCK_SIZES):
    """scheduler: None, or a callable installing the learned scheduler into an engine.
    Stage 1 tries every bin size x list-kernel variant at the first block size (128 threads);
    stage 2 tries the other block sizes with the stage-1 winner."""
    base = needed_width(params, states, skin)
    common = dict(skin=skin, steps=steps, warmup=warmup, seed=seed, device=device, scheduler=scheduler)
    trials = []
    for f, (stg, occ) in itertools.product(bin_factors, variants):
        ms = _trial(params, states, caps, bin_width=0.0 if f == 1.0 else f * base, stg=stg, occ=occ,
                    block=block_sizes[0], **common)
        trials.append(dict(bin_factor=f, staging=stg, occupancy=occ, block_size=block_sizes[0], ms_per_step=ms))
    best = min(trials, key=lambda t: t["ms_per_step"])
    for b in block_sizes[1:]:
        f = best["bin_factor"]
        ms = _trial(params, states, caps, bin_width=0.0 if f == 1.0 else f * base, stg=best["staging"],
                    occ=best["occupancy"], block=b, **common)
        trials.append(dict(bin_factor=f, staging=best["staging"], occupancy=best["occupancy"], block_size=b,
                           ms_per_step=ms))
    best = min(trials, key=lambda t: t["ms_per_step"])
    kw = dict(bin_width=0.0 if best["bin_factor"] == 1.0 else best["bin_factor"] * base,
              staging=best["staging"], occupancy=best["occupancy"], block_size=best["block_size"])
    return kw, trials
