"""Learned Verlet-skin scheduler: traces, labels, training and the trained network.

The network (12 -> 64 -> 64 -> 2, SiLU, FP32) runs on the device at every list rebuild of a
colony (cil_set_scheduler); its inputs are the 12 per-colony features the step maintains
(cil_sched_info: cells, mean/max bin occupancy, mean/max step displacement, division and
apoptosis rates, current skin, steps since the last rebuild, displacement at the rebuild,
guard-trip share, fresh elements). Output 0 sets the skin in [skin_min, skin_max], output 1
the rebuild cadence. The displacement guard (|u - u_ref| > skin/2 forces a rebuild) runs
every step whatever the network says, so the trajectory is the one of any other skin; only
the cost of a step depends on the choice.

Training data (make_dataset): trace runs of the library's skin mode, one colony per run,
under the growth physics with randomised seeds, motility in [0.1, 2], noise, division time
and colony size, each at a grid of fixed skins. Every list rebuild of a run gives one input
row (the features at that decision). A run's per-step cost at each skin is modelled from
its exact counters as
    t(s) = A * list_entries(s) + R * elements * rebuilds_per_step(s) + F * fresh(s) + B * elements,
with the unit costs A, R, F, B fitted by least squares to device-timed runs of a large
colony (fit_unit_costs, each run advanced in one call with graph-replayed steps). The label
of every row of a configuration is the skin of least modelled cost over the grid and the
cadence that balances rebuild cost against the accumulating fresh elements at that skin
(cadence_target). Training (train) uses only the project's CUDA kernels (cil_mlp_grad,
cil_mlp_adam).
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

from . import synthetic as S

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "skin_mlp.npz")

N_IN, N_H, N_OUT = 12, 64, 2
SKIN_MIN, SKIN_MAX = 0.1, 0.3            # output range; SKIN_MAX also sizes the bins
INTERVAL_SCALE = 100.0                    # cadence = INTERVAL_SCALE * softplus(y1)
SKIN_GRID = (0.1, 0.15, 0.2, 0.25, 0.3)
FEATURES = ("log_cells", "mean_occupancy", "max_occupancy", "mean_step", "max_step", "div_rate",
            "apo_rate", "skin", "log_interval", "disp_ratio", "trip_share", "fresh_share")


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation in the kernels' layout W1 b1 W2 b2 W3 b3."""
    rng = np.random.default_rng(seed)
    parts = []
    for rows, cols in ((N_H, N_IN), (N_H, N_H), (N_OUT, N_H)):
        parts.append(rng.normal(0.0, math.sqrt(1.0 / cols), size=rows * cols))
        parts.append(np.zeros(rows))
    return np.concatenate(parts).astype(np.float32)


def skin_to_y0(skin, lo=SKIN_MIN, hi=SKIN_MAX):
    f = np.clip((np.asarray(skin) - lo) / (hi - lo), 0.02, 0.98)
    return np.log(f / (1.0 - f))


def interval_to_y1(interval, scale=INTERVAL_SCALE):
    v = np.maximum(np.asarray(interval, dtype=np.float64) / scale, 1e-3)
    return np.where(v > 20.0, v, np.log(np.expm1(v)))


# ---------------------------------------------------------------- trace configurations

def trace_config(rng, ncells=None):
    """One growth-physics configuration: motility U[0.1, 2], noise D log-U[1e-3, 3e-2],
    division time log-U[0.3, 3] (sd 10 %), apoptosis 0.01/tau, cells log-U[8k, 64k]."""
    if ncells is None:
        ncells = int(round(math.exp(rng.uniform(math.log(8000), math.log(64000)))))
    tau = math.exp(rng.uniform(math.log(0.3), math.log(3.0)))
    area = ncells * 2 * math.pi / 4 / 0.8
    box = float(max(64.0, 2 ** math.ceil(math.log2(4.0 * math.sqrt(area / math.pi)))))
    p = S.growth_params(box=box, div_tau_mu=tau, div_tau_sigma=0.1 * tau, apop_rate=0.01 / tau,
                        noise_D=math.exp(rng.uniform(math.log(1e-3), math.log(3e-2))),
                        motility=[0.0, float(rng.uniform(0.1, 2.0))])
    st = S.disk_colony(ncells, p, seed=int(rng.integers(1, 2**31 - 1)))
    return p, st


def run_trace(G, p, st, skin, steps, warmup=20, seed=1, skin_max=SKIN_MAX, timed=False):
    """Runs one colony at a fixed skin (guard on, no cadence). Returns the feature rows of
    its list rebuilds and its counters, step by step; when timed, a second run of the same
    colony and seed advances all steps in one call (graph-replayed, as in production) and
    gives the device time per step."""
    n = len(st["sigma"])
    cap = int(1.3 * n) + 64
    ms = None
    if timed:
        eng = G.Engine([p], [cap], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=seed, skin=skin_max)
        try:
            eng.upload(0, **st)
            eng.set_skin(0, skin, 0)
            eng.step(warmup)
            eng.step(steps)
            ms = eng.timings()["total_ms"] / steps
        finally:
            eng.close()
    eng = G.Engine([p], [cap], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=seed, skin=skin_max)
    try:
        eng.upload(0, **st)
        eng.set_skin(0, skin, 0)
        eng.step(warmup)
        k0 = eng.skin_stats(0)
        rows, entries, fresh = [], 0.0, 0.0
        last = k0["nrebuild"]
        for _ in range(steps):
            eng.step(1)
            k = eng.skin_stats(0)
            entries += k["npairs"]
            fresh += k["nfresh"]
            if k["nrebuild"] != last:
                rows.append(eng.sched_state(0)["features"])
                last = k["nrebuild"]
        k1 = eng.skin_stats(0)
        ne = 2 * eng.download(0, want=("ncells",))["ncells"]
    finally:
        eng.close()
    nreb = k1["nrebuild"] - k0["nrebuild"]
    return dict(rows=np.array(rows, dtype=np.float32).reshape(-1, N_IN), elements=ne,
                entries=entries / steps, fresh=fresh / steps, rebuild_rate=nreb / steps,
                interval=steps / max(nreb, 1), ms_per_step=ms)


def fit_unit_costs(G, ncells=400000, steps=150, seed=7):
    """Device-timed runs of one large colony over the skin grid and a few noise levels;
    least-squares fit of t = A*entries + R*elements*rate + F*fresh + B*elements."""
    rng = np.random.default_rng(seed)
    obs = []
    for D in (3e-3, 1e-2, 3e-2):
        p, st = trace_config(rng, ncells)
        p["noise_D"] = D
        for s in SKIN_GRID:
            r = run_trace(G, p, st, s, steps, seed=seed, timed=True)
            obs.append(r)
    Xm = np.array([[r["entries"], r["elements"] * r["rebuild_rate"], r["fresh"], r["elements"]] for r in obs])
    y = np.array([r["ms_per_step"] for r in obs])
    coef, *_ = np.linalg.lstsq(Xm, y, rcond=None)
    coef = np.maximum(coef, 0.0)
    resid = float(np.sqrt(np.mean((Xm @ coef - y) ** 2)))
    return dict(A=float(coef[0]), R=float(coef[1]), F=float(coef[2]), B=float(coef[3]), rms_ms=resid,
                runs=[{k: (float(v) if isinstance(v, (int, float, np.floating)) else None)
                       for k, v in r.items() if k != "rows"} for r in obs])


def modelled_ms(costs, r):
    return (costs["A"] * r["entries"] + costs["R"] * r["elements"] * r["rebuild_rate"] + costs["F"] * r["fresh"]
            + costs["B"] * r["elements"])


def cadence_target(costs, r):
    """Rebuild cadence that balances the cost of a rebuild against the growing cost of the
    fresh elements between rebuilds: with fresh elements accumulating at rate q per step,
    an interval T costs R*N/T + F*q*T/2 per step, least at T* = sqrt(2 R N / (F q)). The
    guard still rebuilds earlier when elements move too far. q is read off the run's mean
    fresh count over its mean interval (a sawtooth from 0 to q*T)."""
    q = 2.0 * r["fresh"] / max(r["interval"], 1.0)
    if q <= 0.0 or costs["F"] <= 0.0:
        return 1000.0
    t = math.sqrt(2.0 * costs["R"] * r["elements"] / (costs["F"] * q))
    return float(min(max(t, 10.0), 1000.0))


def make_dataset(G, costs, nconfigs=200, steps=300, seed=11, max_rows=24):
    """Inputs and labels from trace runs of nconfigs random configurations."""
    rng = np.random.default_rng(seed)
    X, T, meta = [], [], []
    for k in range(nconfigs):
        p, st = trace_config(rng)
        runs = {s: run_trace(G, p, st, s, steps, seed=k + 1) for s in SKIN_GRID}
        cost = {s: modelled_ms(costs, r) for s, r in runs.items()}
        best = min(cost, key=cost.get)
        cadence = cadence_target(costs, runs[best])
        target = (float(skin_to_y0(best)), float(interval_to_y1(cadence)))
        for s, r in runs.items():
            rows = r["rows"]
            if len(rows) > max_rows:
                rows = rows[rng.choice(len(rows), max_rows, replace=False)]
            X.append(rows)
            T.append(np.tile(target, (len(rows), 1)))
        meta.append(dict(cells=len(st["sigma"]), motility=p["motility"][1], noise_D=p["noise_D"],
                         tau=p["div_tau_mu"], best_skin=best, interval=runs[best]["interval"], cadence=cadence,
                         cost_ms={str(s): c for s, c in cost.items()}))
    return np.concatenate(X).astype(np.float32), np.concatenate(T).astype(np.float32), meta


def train(G, X, T, epochs=3000, lr=3e-3, seed=0, out_weights=(1.0, 0.25)):
    """Full-batch Adam on the device with the project's kernels; returns the parameters and
    the loss history (every 100 epochs)."""
    import torch
    dev = torch.device("cuda:0")
    Xt = torch.tensor(X, device=dev)
    Tt = torch.tensor(T, device=dev)
    ow = torch.tensor(np.asarray(out_weights, dtype=np.float32), device=dev)
    w = torch.tensor(init_params(seed), device=dev)
    m, v = torch.zeros_like(w), torch.zeros_like(w)
    ws = torch.zeros(G.mlp_workspace_floats(len(X)), device=dev)
    grad, loss = torch.zeros_like(w), torch.zeros(1, device=dev)
    hist = []
    for t in range(1, epochs + 1):
        G.mlp_grad(w, Xt, Tt, ow, ws, grad, loss)
        rate = lr * (0.1 ** (t / epochs))  # exponential decay to lr/10
        G.mlp_adam(w, grad, m, v, t, rate)
        if t % 100 == 0 or t == 1:
            hist.append((t, float(loss.item())))
    return w.cpu().numpy(), hist


def save(params, path=WEIGHTS, **info):
    np.savez(path, params=np.asarray(params, dtype=np.float32), skin_min=SKIN_MIN, skin_max=SKIN_MAX,
             interval_scale=INTERVAL_SCALE, features=np.array(FEATURES), info=json.dumps(info))


def load(path=WEIGHTS):
    """The trained network: (params, skin_min, skin_max, interval_scale)."""
    z = np.load(path)
    return (z["params"].astype(np.float32), float(z["skin_min"]), float(z["skin_max"]),
            float(z["interval_scale"]))


def install(engine, path=WEIGHTS, use_interval=True):
    """Installs the trained network into a skin-mode engine created with skin = skin_max."""
    params, lo, hi, scale = load(path)
    engine.set_scheduler(params, skin_min=lo, interval_scale=scale, use_interval=use_interval)
    return hi


def main():
    """Fits the unit costs, generates the traces, trains and writes the weights file."""
    import argparse
    import time

    import cil_cuda_gb300 as G
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", type=int, default=200)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--report", default=None)
    a = ap.parse_args()
    t0 = time.time()
    costs = fit_unit_costs(G)
    t1 = time.time()
    X, T, meta = make_dataset(G, costs, nconfigs=a.configs, steps=a.steps)
    t2 = time.time()
    params, hist = train(G, X, T, epochs=a.epochs)
    t3 = time.time()
    info = dict(costs={k: costs[k] for k in ("A", "R", "F", "B", "rms_ms")}, rows=int(len(X)),
                configs=a.configs, steps=a.steps, epochs=a.epochs, loss=hist[-1][1], loss0=hist[0][1],
                seconds=dict(costs=t1 - t0, traces=t2 - t1, train=t3 - t2))
    save(params, a.out, **info)
    if a.report:
        with open(a.report, "w") as f:
            json.dump(dict(info=info, costs=costs, history=hist, configs=meta), f, indent=1)
    print(json.dumps(info))


if __name__ == "__main__":
    main()
