"""ORACLE — test infrastructure only: end-of-run observables of oracle ensembles, one seed per
worker process. The GPU statistics tests run the oracle side of a comparison in a process pool
started with the spawn method (a pool forked from a process that has initialised CUDA can
hang), so the worker is a module-level function that receives everything it needs as plain
data."""
import os

OBS = ("ncells", "mean_area", "msd", "vacf")


def observables_after(args):
    """args = (params dict, state dict of arrays, capacity, seed, warm steps, measured steps):
    the oracle's observables after `warm` steps, an observable reset, and `steps` more steps."""
    params, state, cap, seed, warm, steps = args
    from oracle import oracle as O
    o = O.Oracle(params, cap, seed, threads=0)
    o.set_state(**state)
    o.step(warm)
    o.obs_reset()
    err = o.step(steps)
    if err != 0:
        raise RuntimeError(f"oracle step failed with {err} (seed {seed})")
    r = o.observables()
    o.close()
    return [float(r[k]) for k in OBS]


def run_pool(jobs, processes=None):
    import multiprocessing as mp
    n = processes or min(len(jobs), os.cpu_count() or 1)
    with mp.get_context("spawn").Pool(n) as pool:
        return pool.map(observables_after, jobs)
