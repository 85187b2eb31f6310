"""Benchmark: particle-steps/s of the 2D colony-growth step at 2M particles on one GB300.

Workload (the reference's headline configuration): 2D soft-core colony growth
(eps = 5, cutoff at contact, linear growth, division ~ N(1, 0.1), apoptosis 0.01/tau_d,
D = 0.01, dt = 1e-4, periodic 2048 x 2048 box) at the checkpoint of 1M cells
(2M particles), division and apoptosis on. The checkpoint is a seeded synthetic grown
colony (cells uniform in a central disk at packing fraction 0.8, cycle ages uniform).

Arms:
  default            the library: plain FP64 form and mixed FP32-force/FP64-position form
                     (value = mixed), device-timed with CUDA events, plus an end-to-end
                     run through the C ABI with host buffers, plus the CPU baseline (the
                     oracle on the host cores, bounded sample)
  --impl reference   the reference's CPU path (the oracle restatement, all host threads,
                     the reference itself does not build) on the same workload

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Multi-GPU (torchrun): one independent replica per rank (the path does not shard a single
colony); value = all ranks' particle-steps / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s @2M particles 2D: mixed+batched+skin-MLP vs plain FP64, 1 GB300"
UNIT = "particle-steps/s"
NCELLS = 1_000_000
BOX = 2048.0
CAP = 1_200_000
GTS = 100  # steps per output frame in the end-to-end arm
FRAME_CAP = 1_600_000  # cells: the frame-output leg grows the colony for 3000 steps
# ncu summary of the dominant kernel on this workload; roofline.traffic is read from its
# dram__bytes_read.sum + dram__bytes_write.sum rows (one launch, one capture)
TRAFFIC_PROFILE = os.path.join(ROOT, "profiles", "k_force_cells_2d_softcore_2M.md")
WORKLOAD = ("2D colony growth, soft-core eps=5, 1M cells / 2M particles checkpoint, "
            "division+apoptosis on, dt=1e-4, 2048^2 periodic box")


def bench_config(world: int) -> dict:
    """The workload as both arms report it: the checkpoint's size before any step (the two arms
    warm up differently, so counts taken later differ by the divisions in between)."""
    return {"workload": WORKLOAD, "particles": 2 * NCELLS, "cells": NCELLS,
            "l2": "working set ~230 MB per step > 126 MB L2, no flush",
            "parallelism": f"replicas x{world}"}


def profile_traffic(path: str = TRAFFIC_PROFILE):
    """DRAM bytes of one launch from a committed ncu summary (markdown table rows
    `| dram__bytes_read.sum | v | unit |`), or None when the file has no such rows."""
    scale = {"byte": 1.0, "kbyte": 1e3, "mbyte": 1e6, "gbyte": 1e9}
    got = {}
    try:
        with open(path) as f:
            for line in f:
                cells = [c.strip().strip("`") for c in line.strip().strip("|").split("|")]
                if len(cells) >= 3 and cells[0] in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
                    got[cells[0]] = float(cells[1].replace(",", "")) * scale.get(cells[2].lower(), 1.0)
    except OSError:
        return None
    if len(got) != 2:
        return None
    return got["dram__bytes_read.sum"] + got["dram__bytes_write.sum"]


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(self.device)], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def workload(seed: int):
    from cil_cuda_gb300 import synthetic as S
    p = S.growth_params(box=BOX)
    st = S.disk_colony(NCELLS, p, seed=seed)
    return p, st


def dist_init(n_gpus: int):
    if n_gpus <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="env://")
    return dist.get_rank(), dist.get_world_size(), dist


def allreduce_max(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def run_form(G, p, st, precision, steps, warmup, device, seed, dist, skin=0.0, sched=False, graphs=True,
             tune=None, integrator=0):
    """Device-timed run of one form; returns particle-steps/s and the timing details."""
    eng = G.Engine([p], [CAP], precision=precision, rng=G.RNG_PHILOX, seed=seed, device=device, skin=skin,
                   graphs=graphs, integrator=integrator, **(tune or {}))
    eng.upload(0, **st)
    if sched:
        from cil_cuda_gb300 import skin_scheduler as SS
        SS.install(eng)
    if warmup:
        eng.step(warmup)
    n0 = eng.observables(0)["ncells"]
    sk0 = eng.skin_stats(0) if skin > 0 else None
    barrier(dist)
    t0 = time.perf_counter()
    eng.step(steps)  # synchronises the handle's stream before returning
    wall = time.perf_counter() - t0
    tm = eng.timings()
    gi = eng.graph_info()
    n1 = eng.observables(0)["ncells"]
    sk = eng.skin_stats(0) if skin > 0 else None
    if sk is not None:
        sk["rebuilds_in_timed_window"] = sk["nrebuild"] - sk0["nrebuild"]
        sk["guard_trips_in_timed_window"] = sk["ntrip"] - sk0["ntrip"]
    eng.close()
    dev_s = tm["total_ms"] * 1e-3
    psteps = (n0 + n1) * steps  # 2 elements per cell, trapezoid over the (slow) growth
    return dict(psteps=psteps, dev_s=dev_s, wall_s=wall, n0=n0, n1=n1, timings=tm, skin=sk, graphs=gi)


def run_channel(G, device, steps, warmup):
    """The 3D Hertzian channel (third configuration): 2M cells / 4M particles between flat
    walls at z = 0 and 20 sigma, periodic 1024^2 in x and y, division on, dt = 5e-5; mixed
    precision with Verlet lists (0.3 sigma), and the plain FP64 form on a tenth of the steps."""
    from cil_cuda_gb300 import synthetic as S
    p = S.channel_params(lxy=1024.0, height=20.0)
    st = S.channel_colony(2_000_000, p, seed=3)
    cap = 2_400_000
    out = {}
    for name, prec, skin, k in (("mixed_skin", G.PREC_MIXED, 0.3, steps),
                                ("plain_fp64", G.PREC_FP64, 0.0, max(1, steps // 10))):
        eng = G.Engine([p], [cap], precision=prec, rng=G.RNG_PHILOX, seed=5, device=device, skin=skin)
        eng.upload(0, **st)
        eng.step(warmup)
        n0 = eng.observables(0)["ncells"]
        eng.step(k)
        tm = eng.timings()
        n1 = eng.observables(0)["ncells"]
        eng.close()
        out[name] = (n0 + n1) * k / (tm["total_ms"] * 1e-3)
        out[name + "_ms_per_step"] = tm["total_ms"] / k
    # phase split of the mixed skin form: the same steps launched one by one (graph replay
    # records no per-phase events)
    eng = G.Engine([p], [cap], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=5, device=device, skin=0.3,
                   graphs=False)
    eng.upload(0, **st)
    eng.step(warmup)
    eng.timings()
    eng.step(steps)
    tm = eng.timings()
    eng.close()
    phases = {key: v / steps for key, v in tm.items() if key.endswith("_ms")}
    return {"value": out["mixed_skin"], "unit": UNIT, "particles": 2 * len(st["sigma"]), "steps": steps,
            "forms": out, "speedup_vs_plain_fp64": out["mixed_skin"] / out["plain_fp64"],
            "mixed_skin_phase_ms_per_step_launched": phases,
            "config": "3D Hertz E=100, walls z=0 and 20, periodic 1024^2, phi=0.6 slab, dt=5e-5, D=0.005, division on"}


def run_batched(G, device, steps, warmup, sched):
    """The batched sweep: 256 colonies of log-uniform size in one handle (skin mode, learned
    scheduler when available, graph-replayed steps, launch parameters from the autotuner),
    device-timed."""
    from cil_cuda_gb300 import autotune as AT
    from cil_cuda_gb300 import synthetic as S
    ps, sts, caps = S.batched_sweep(256, steps=steps + warmup + 100)
    skin = 0.3
    inst = None
    if sched:
        from cil_cuda_gb300 import skin_scheduler as SS
        skin = SS.load()[2]
        inst = SS.install
    tune, trials = AT.autotune(ps, sts, caps, skin=skin, steps=30, warmup=5, device=device, scheduler=inst)
    eng = G.Engine(ps, caps, precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=11, device=device, skin=skin, **tune)
    for c, st in enumerate(sts):
        eng.upload(c, **st)
    if sched:
        SS.install(eng)
    eng.step(warmup)
    n0 = [eng.observables(c)["ncells"] for c in range(len(ps))]
    eng.step(steps)
    tm = eng.timings()
    n1 = [eng.observables(c)["ncells"] for c in range(len(ps))]
    gi = eng.graph_info()
    eng.close()
    dev_s = tm["total_ms"] * 1e-3
    psteps = (sum(n0) + sum(n1)) * steps
    sizes = np.array([len(s["sigma"]) for s in sts])
    batch_ms = dev_s / steps * 1e3
    # per colony: five colonies (smallest, quartiles, largest) run alone on their own random
    # streams with the same settings, against their share of the batched step (by particles)
    order = np.argsort(sizes)
    picks = [int(order[int(round(q * (len(order) - 1)))]) for q in (0.0, 0.25, 0.5, 0.75, 1.0)]
    tot = float(sum(n0) + sum(n1))
    alone = []
    for c in picks:
        e1 = G.Engine([ps[c]], [caps[c]], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=11, device=device, skin=skin,
                      rng_stream_base=c, **tune)
        e1.upload(0, **sts[c])
        if sched:
            SS.install(e1)
        e1.step(warmup)
        e1.step(steps)
        ms1 = e1.timings()["total_ms"] / steps
        e1.close()
        share = (n0[c] + n1[c]) / tot * batch_ms
        alone.append({"colony": c, "cells": int(sizes[c]), "ms_per_step_alone": ms1,
                      "ms_per_step_share_in_batch": share, "speedup_in_batch": ms1 / share})
    return {"value": psteps / dev_s, "unit": UNIT, "colonies": len(ps), "steps": steps,
            "particles": 2 * int(sum(n0)), "cells_min_median_max": [int(sizes.min()), int(np.median(sizes)),
                                                                    int(sizes.max())],
            "ms_per_step": batch_ms, "ms_per_colony_step": batch_ms / len(ps),
            "per_colony": alone,
            "form": "mixed precision, Verlet skin" + (" + learned scheduler" if sched else " 0.3 sigma"),
            "autotuned": tune, "autotune_trials_ms_per_step": {f"{t['bin_factor']}/{t['staging']}/{t['occupancy']}/{t['block_size']}":
                                                              round(t["ms_per_step"], 4) for t in trials},
            "graph_steps": gi["graph_steps"], "gpu_launches": tm["launches"]}


def run_e2e(G, p, st, precision, steps, device, seed, skin=0.0, sched=False, tune=None):
    """The same metric through the reference-facing calls with host buffers: upload the
    colony from pinned host memory, one cil_step per Euler step (the reference's mdStep
    call; every step's counters are read back to the host, and with CIL_FLAG_DEFERRED_STATUS
    each call returns the previous call's status, so the host queues the next step while the
    GPU runs this one), a GSD frame after every GTS steps written by the device-fed frame
    writer (outputFrame, OutputWriter.cpp:640-644; its copy to the host and its file writes
    overlap the next steps; none in a run shorter than GTS steps), and the final state
    downloaded into pinned host arrays. Every queued frame is written to the file (flush) inside
    the timed region; the file is closed after it, as the reference closes its output after
    its step loop (finalizeOutput), and the engine (learned scheduler included) is configured
    before it, as the reference reads its parameters before the loop."""
    import tempfile
    n = len(st["sigma"])
    eng = G.Engine([p], [CAP], precision=precision, rng=G.RNG_PHILOX, seed=seed, device=device, skin=skin,
                   deferred_status=True, **(tune or {}))
    h2d = st["pos"].nbytes + st["sigma"].nbytes + st["t0"].nbytes + st["tswitch"].nbytes
    d2h = 0
    # the step's inputs sit in pinned host memory (registered before the timed region)
    types = {"pos": np.float64, "sigma": np.float64, "t0": np.int32, "tswitch": np.int32}
    st = {k: np.ascontiguousarray(v, types.get(k)) for k, v in st.items()}
    pinned = [v for k, v in st.items() if k in ("pos", "sigma", "t0", "tswitch") and v.nbytes]
    # the result: the final state, into pinned host arrays of the run's capacity
    res = dict(pos=np.zeros((CAP, 2, p["dim"])), sigma=np.zeros((CAP, 2)), t0=np.zeros(CAP, np.int32),
               tswitch=np.zeros(CAP, np.int32))
    pinned += list(res.values())
    for v in pinned:
        G.host_register(v)
    with tempfile.TemporaryDirectory() as tmp:
        # the output file and its staging are opened before the run, as the reference's
        # initializeOutput is (outside its simulation timer)
        w = eng.frame_writer(0, os.path.join(tmp, "e2e.gsd"))
        if sched:
            from cil_cuda_gb300 import skin_scheduler as SS
            SS.install(eng)
        t0 = time.perf_counter()
        eng.upload(0, **st)
        for k in range(steps):
            eng.step(1)
            d2h += 56  # the per-call status read of the colony counters
            if (k + 1) % GTS == 0:
                w.write()
        w.flush()
        fin = eng.download(0, want=("pos", "sigma", "t0", "tswitch"), out=res)
        wall = time.perf_counter() - t0
        w.close()
        fs = w.last_stats
    n1 = fin["ncells"]
    d2h += n1 * (res["pos"][0].nbytes + res["sigma"][0].nbytes + 8)
    eng.close()
    for v in pinned:
        G.host_unregister(v)
    d2h += fs["d2h_bytes"]
    return dict(value=(n + n1) * steps / wall, wall_s=wall, h2d=h2d / steps, d2h=d2h / steps,
                frames=fs["frames_written"], file_bytes=fs["file_bytes"])


def run_frames(G, p, st, steps, device, seed, skin, sched, tune):
    """Cost of frame output at the headline workload: steps in cil_step(GTS) calls (graph
    replay) with a GSD frame after every call, written (a) by the device-fed frame writer, whose
    copy and file writes overlap the following steps, and (b) synchronously, the way the
    reference's outputFrame runs: download the frame, then write the chunks on the host (the
    library's GSD file layer) before stepping on; (c) no frames. Wall-clock times."""
    import tempfile
    out = {}
    nframes = max(1, steps // GTS)
    with tempfile.TemporaryDirectory() as tmp:
        for mode in ("none", "async", "sync"):
            eng = G.Engine([p], [FRAME_CAP], precision=G.PREC_MIXED, rng=G.RNG_PHILOX, seed=seed, device=device,
                           skin=skin, **(tune or {}))
            eng.upload(0, **st)
            if sched:
                from cil_cuda_gb300 import skin_scheduler as SS
                SS.install(eng)
            eng.step(GTS)
            path = os.path.join(tmp, mode + ".gsd")
            w = eng.frame_writer(0, path) if mode == "async" else None
            gw = G.GSDWriter(path) if mode == "sync" else None  # both opened before the timed steps
            L = np.asarray(p["box"], np.float64)
            t0 = time.perf_counter()
            for _ in range(nframes):
                eng.step(GTS)
                if w is not None:
                    w.write()
                elif gw is not None:
                    fr = eng.download(0, want=("pos", "sigma", "vel"))
                    E = 2 * fr["ncells"]
                    pos = np.zeros((E, 3), np.float32)
                    x = fr["pos"].reshape(E, 2)
                    pos[:, 0] = x[:, 0] - 0.5 * L[0]
                    pos[:, 1] = x[:, 1] - 0.5 * L[1]
                    pos[0::2, 2] = np.float32(-0.0)
                    pos[1::2, 2] = np.float32(-0.01)
                    vel = np.zeros((E, 3), np.float32)
                    vel[:, :2] = fr["vel"].reshape(E, 2)
                    dia = fr["sigma"].reshape(E).astype(np.float32)
                    gw.write_chunk("configuration/step", np.array([0], np.uint64))
                    gw.write_chunk("configuration/dimensions", np.array([3], np.uint8))
                    gw.write_chunk("configuration/box", np.array([L[0], L[1], 1.0, 0, 0, 0], np.float32))
                    gw.write_chunk("particles/N", np.array([E], np.uint32))
                    gw.write_chunk("particles/Z", dia)
                    gw.write_chunk("particles/diameter", dia)
                    gw.write_chunk("particles/typeid", np.tile(np.array([0, 1], np.uint32), E // 2))
                    gw.write_chunk("particles/charge", np.full(E, -1.0, np.float32))
                    gw.write_chunk("particles/position", pos)
                    gw.write_chunk("particles/velocity", vel)
                    gw.write_chunk("particles/mass", np.zeros(E, np.float32))
                    gw.end_frame()
            if w is not None:
                w.flush()  # every frame in the file
            eng.step(1)  # drains the stream
            wall = time.perf_counter() - t0
            if w is not None:
                w.close()
                st_w = w.last_stats
            if gw is not None:
                gw.close()
            out[mode] = wall
            if mode == "async":
                out["async_stats"] = st_w
            eng.close()
    base = out["none"]
    return {"frames": nframes, "steps_per_frame": GTS, "particles": 2 * len(st["sigma"]),
            "bytes_per_frame_d2h": out["async_stats"]["d2h_bytes"] / nframes,
            "file_bytes_per_frame": out["async_stats"]["file_bytes"] / nframes,
            "wall_s": {k: out[k] for k in ("none", "async", "sync")},
            "overhead_ms_per_frame": {"async_writer": (out["async"] - base) / nframes * 1e3,
                                      "sync_download_and_write": (out["sync"] - base) / nframes * 1e3},
            "writer_thread_ms_per_frame": out["async_stats"]["write_ms"] / nframes,
            "pack_kernel_ms_per_frame": out["async_stats"]["pack_ms"] / nframes,
            "d2h_copy_ms_per_frame": out["async_stats"]["copy_ms"] / nframes,
            "enqueue_ms_per_frame": out["async_stats"]["enqueue_ms"] / nframes}


def run_cycle(G, device, steps, warmup, precision=0, dpd=False):
    """The single-element cell-cycle model that the shipped configurations run
    (PRX_MDCK_2D.json: Hertz contacts E = 100 with adhesion 0.2, motility 1, friction 0.01,
    dt = 1e-5, V1 15, P0 5), 1M cells on a jittered square lattice of spacing 1.1 in a periodic
    1100^2 box, cycle phases uniform; device-timed, and the restatement on one host thread over
    a 20k-cell sample of the same packing for scale. dpd: the DPD integrator instead of Euler
    (mass 1, KBT 0.003 as in the shipped files, DISDIFCEL 1, DISBG 0.01)."""
    side = 1000
    rng = np.random.default_rng(17)
    n = side * side
    g = (np.arange(n) % side, np.arange(n) // side)
    pos = np.stack([(g[0] + 0.5) * 1.1, (g[1] + 0.5) * 1.1], axis=1) + rng.uniform(-0.05, 0.05, size=(n, 2))
    prm = dict(box=[1100.0, 1100.0, 0.0], dt=1e-5, motility=1.0, zeta=0.01, v1=15.0, precision=precision)
    if dpd:
        prm.update(integrator=G.CYCLE_DPD, mass=1.0, kbt=0.003, dis_diff=1.0, dis_bg=0.01)
    st = dict(pos=pos, sigma=np.full(n, 1.1283791670955126), theta=rng.uniform(0, 1, n), rho=np.ones(n),
              angvel=np.full(n, 1e-5))
    eng = G.CycleEngine(prm, int(1.2 * n), seed=3, device=device)
    eng.upload(**st)
    eng.step(warmup)
    n0 = eng.download()["ncells"]
    eng.step(steps)
    tm = eng.timings()
    n1 = eng.download()["ncells"]
    eng.close()
    dev_s = tm["total_ms"] * 1e-3
    out = {"value": (n0 + n1) / 2 * steps / dev_s, "unit": "cell-steps/s", "cells": n0, "cells_end": n1,
           "steps": steps, "ms_per_step": tm["total_ms"] / steps, "gpu_launches": tm["launches"],
           "config": "single-element cell-cycle model (PRX_MDCK_2D.json parameters), "
                     + ("DPD, " if dpd else "")
                     + (("FP32 pair terms" if dpd else "FP32 contacts") + " / FP64 state" if precision else "FP64")
                     + ", 1M cells"}
    if precision or dpd:
        return out
    try:
        from oracle import oracle as O
        O.build()
        m = 140  # a 140 x 140 corner of the lattice in its own periodic box
        sel = (g[0] < m) & (g[1] < m)
        k = int(sel.sum())
        so = dict(pos=pos[sel], sigma=np.full(k, 1.1283791670955126), theta=st["theta"][sel], rho=np.ones(k),
                  angvel=np.full(k, 1e-5))
        q = dict(prm)
        q["box"] = [m * 1.1, m * 1.1, 0.0]
        o = O.CycleOracle(q, 2 * k, 3)
        o.set_state(**so)
        t0 = time.perf_counter()
        o.step(10)
        cpu_s = time.perf_counter() - t0
        out["cpu_restatement_1_thread"] = {"value": k * 10 / cpu_s, "unit": "cell-steps/s", "cells": k, "steps": 10}
    except Exception as e:  # reported, not fatal
        out["cpu_restatement_1_thread"] = {"error": str(e)}
    return out


def run_cycle_small(G, device, steps=3000, warmup=3):
    """The cell-cycle model at the sizes the shipped runs spend their time at (they start from
    one or two cells): 1024 cells on the same lattice in a periodic 35.2^2 box, FP64, with the
    step replayed as a captured CUDA graph (the default) and launched kernel by kernel."""
    side = 32
    rng = np.random.default_rng(19)
    n = side * side
    g = (np.arange(n) % side, np.arange(n) // side)
    pos = np.stack([(g[0] + 0.5) * 1.1, (g[1] + 0.5) * 1.1], axis=1) + rng.uniform(-0.05, 0.05, size=(n, 2))
    st = dict(pos=pos, sigma=np.full(n, 1.1283791670955126), theta=rng.uniform(0, 1, n), rho=np.ones(n),
              angvel=np.full(n, 1e-5))
    out = {"cells": n, "steps": steps, "unit": "ms per step"}
    for name, flags in (("graphs", 0), ("launches", G.CYCLE_NO_GRAPH)):
        prm = dict(box=[side * 1.1, side * 1.1, 0.0], dt=1e-5, motility=1.0, zeta=0.01, v1=15.0, flags=flags)
        eng = G.CycleEngine(prm, 4 * n, seed=3, device=device)
        eng.upload(**st)
        eng.step(warmup)
        eng.step(steps)
        tm = eng.timings()
        eng.close()
        out[name] = tm["total_ms"] / steps
    out["speedup"] = out["launches"] / out["graphs"]
    return out


def run_c1(G, device, steps, warmup, threads):
    """The first configuration at its stated size: 4096 two-element cells (8192 particles), WCA LJ,
    packing 0.8 in a periodic square (relaxed from uniform centres), D = 0.01, dt = 1e-4, no
    division or apoptosis; `steps` steps on the GPU (plain FP64 and mixed with lists, device
    time) and on the host cores (the oracle restatement on all threads and on one)."""
    from cil_cuda_gb300 import synthetic as S
    from oracle import oracle as O
    p, st = S.config1(4096, seed=12345)
    st = S.relax(p, st, device=device)
    n = len(st["sigma"])
    out = {"particles": 2 * n, "steps": steps, "unit": UNIT}
    for name, prec, skin in (("plain_fp64", G.PREC_FP64, 0.0), ("mixed_skin_0.3", G.PREC_MIXED, 0.3)):
        eng = G.Engine([p], [n], precision=prec, rng=G.RNG_PHILOX, seed=5, device=device, skin=skin)
        eng.upload(0, **st)
        eng.step(warmup)
        eng.step(steps)
        ms = eng.timings()["total_ms"]
        eng.close()
        out[name] = {"value": 2 * n * steps / (ms * 1e-3), "ms_per_step": ms / steps}
    if not os.path.exists(O.LIB_PATH):
        O.build()
    for key, th in (("cpu_all_threads", threads), ("cpu_one_thread", 1)):
        o = O.Oracle(p, n, 1, threads=th)
        o.set_state(**st)
        t0 = time.perf_counter()
        k = 0
        while k < steps and time.perf_counter() - t0 < 12.0:
            o.step(50)
            k += 50
        wall = time.perf_counter() - t0
        o.close()
        out[key] = {"value": 2 * n * k / wall, "cores": th, "kind": "port",
                    "sample": f"{k} Euler steps of the 8192-particle configuration, {wall:.1f} s"}
    out["config"] = "4096 cells x 2 elements, WCA LJ eps=1, packing 0.8, periodic, D=0.01, dt=1e-4"
    return out


def cpu_baseline(p, st, threads: int, budget_s: float = 20.0):
    """The oracle (race-free OpenMP variant of the reference's step) on the host cores on
    the same 2M-particle state, as many whole steps as fit the budget (at least 1)."""
    from oracle import oracle as O
    if not os.path.exists(O.LIB_PATH):
        O.build()
    o = O.Oracle(p, CAP, 1, threads=threads)
    o.set_state(**st)
    t0 = time.perf_counter()
    o.step(1)
    first = time.perf_counter() - t0
    n = max(0, int(budget_s / max(first, 1e-3)) - 1)
    n = min(n, 20)
    if n:
        o.step(n)
    wall = time.perf_counter() - t0
    steps = n + 1
    value = 2 * (len(st["sigma"]) + o.ncells) / 2 * steps / wall
    o.close()
    return dict(value=value, unit=UNIT, cores=threads, kind="port",
                sample=f"{steps} Euler steps of the 2M-particle checkpoint (full step: forces, "
                       f"integration, division, apoptosis), {wall:.1f} s")


def reference_arm(args):
    rank, world, dist = dist_init(args.gpus)
    if rank != 0:
        return 0
    p, st = workload(seed=1)
    threads = os.cpu_count() or 1
    from oracle import oracle as O
    if not os.path.exists(O.LIB_PATH):
        O.build()
    o = O.Oracle(p, CAP, 1, threads=threads)
    o.set_state(**st)
    # bounded sample: each bench step is one full Euler step of the 2M-particle colony;
    # the number of timed steps is capped so that the run ends within a few minutes
    # bounded sample: each bench step is one full Euler step of the 2M-particle colony; the
    # warm-up is the requested one, and the number of timed steps is capped so that the run
    # ends within a few minutes
    t0 = time.perf_counter()
    o.step(1)
    per = time.perf_counter() - t0
    warm = args.warmup
    if warm > 1:
        o.step(warm - 1)
    k = max(1, min(args.steps, int(90.0 / max(per, 1e-3))))
    n0 = o.ncells
    t0 = time.perf_counter()
    o.step(k)
    wall = time.perf_counter() - t0
    n1 = o.ncells
    value = (n0 + n1) * k / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": k, "warmup": warm, "ms_per_step": wall / k * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(world),
        "steps_requested": args.steps, "cells_timed": [n0, n1],
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{k} full Euler steps of the 2M-particle state on {threads} host threads "
                                   f"(oracle restatement; the reference's step does not compile)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--skin", type=float, default=0.3, help="Verlet skin of the skin form (sigma units)")
    ap.add_argument("--no-sched", action="store_true", help="fixed skin instead of the learned scheduler")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched 256-colony leg")
    ap.add_argument("--no-frames", action="store_true", help="skip the frame-output leg")
    ap.add_argument("--no-tune", action="store_true", help="default launch parameters (no autotuner)")
    ap.add_argument("--staging", type=int, default=0, help="profile: list entries in flight (0: default)")
    ap.add_argument("--occupancy", type=int, default=0, help="profile: CTAs per SM of the list kernel (0: default)")
    ap.add_argument("--only", choices=["mixed", "plain", "skin", "cycle", "cycle_fp64", "cycle_small", "dpd", "profile",
                                       "channel"],
                    default=None, help="run one form only (profiling); profile: the headline form alone, "
                                       "launched step by step, nothing else")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)

    rank, world, dist = dist_init(args.gpus)
    device = int(os.environ.get("LOCAL_RANK", "0"))
    import cil_cuda_gb300 as G
    if not os.path.exists(G.LIB_PATH):
        from cil_cuda_gb300 import build
        build.build()
    if args.only == "channel":
        print(json.dumps(run_channel(G, device, args.steps, args.warmup)))
        return 0
    if args.only == "cycle_small":
        print(json.dumps(run_cycle_small(G, device, steps=args.steps, warmup=args.warmup)))
        return 0
    if args.only == "dpd":
        print(json.dumps(run_cycle(G, device, args.steps, args.warmup, 0, dpd=True)))
        print(json.dumps(run_cycle(G, device, args.steps, args.warmup, 1, dpd=True)))
        return 0
    if args.only == "cycle_fp64":  # the 1M-cell FP64 form alone (profiling)
        print(json.dumps(run_cycle(G, device, args.steps, args.warmup)))
        return 0
    if args.only == "cycle":
        print(json.dumps(run_cycle_small(G, device)))
        print(json.dumps(run_cycle(G, device, args.steps, args.warmup)))
        print(json.dumps(run_cycle(G, device, args.steps, args.warmup, 1)))
        print(json.dumps(run_cycle(G, device, args.steps, args.warmup, 0, dpd=True)))
        return 0
    p, st = workload(seed=1 + rank)
    hbm, peak_kind = peaks()
    if args.only == "profile":
        from cil_cuda_gb300 import skin_scheduler as SS
        tune = {"staging": args.staging, "occupancy": args.occupancy}
        r = run_form(G, p, st, G.PREC_MIXED, args.steps, args.warmup, device, 7 + rank, dist, skin=SS.load()[2],
                     sched=True, graphs=False, tune=tune)
        print(json.dumps({"profile_run": {"ms_per_step": r["dev_s"] / args.steps * 1e3, "timings": r["timings"],
                                          "skin": r["skin"]}}))
        return 0

    plain_steps = max(1, args.steps // 10)
    from cil_cuda_gb300 import skin_scheduler as SS
    have_mlp = os.path.exists(SS.WEIGHTS) and not args.no_sched
    mlp_skin = SS.load()[2] if have_mlp else args.skin
    if args.only == "mixed":
        plain = None
    else:
        # individually launched steps: the phase timings (FP64 pair kernel) stay complete
        plain = run_form(G, p, st, G.PREC_FP64, plain_steps, args.warmup, device, 7 + rank, dist, graphs=False)
    if args.only == "plain":
        print(json.dumps({"plain_fp64": plain["psteps"] / plain["dev_s"], "timings": plain["timings"]}))
        return 0
    mixed = None
    fixed = None
    if args.only in (None, "mixed"):
        mixed = run_form(G, p, st, G.PREC_MIXED, args.steps, args.warmup, device, 7 + rank, dist)
    if args.only is None and have_mlp:
        fixed = run_form(G, p, st, G.PREC_MIXED, args.steps, args.warmup, device, 7 + rank, dist, skin=args.skin)
    tune, trials = None, []
    if args.only is None and not args.no_tune:
        from cil_cuda_gb300 import autotune as AT
        tune, trials = AT.autotune([p], [st], [CAP], skin=mlp_skin if have_mlp else args.skin, steps=50,
                                   warmup=5, device=device, scheduler=SS.install if have_mlp else None)
    with Clocks(device) as clk:
        skinf = run_form(G, p, st, G.PREC_MIXED, args.steps, args.warmup, device, 7 + rank, dist,
                         skin=mlp_skin if have_mlp else args.skin,
                         sched=have_mlp, tune=tune) if args.only in (None, "skin") else None
    clocks = clk.summary()
    # kernel phases from individually launched steps (graph replays carry no phase events)
    phases = run_form(G, p, st, G.PREC_MIXED, min(args.steps, 200), args.warmup, device, 7 + rank, dist,
                      skin=mlp_skin if have_mlp else args.skin, sched=have_mlp, graphs=False, tune=tune) \
        if skinf is not None else None
    if mixed is None:
        mixed = skinf
    if skinf is None:
        skinf = phases = mixed
    if plain is None:
        plain = mixed
    if fixed is None:
        fixed = skinf

    t_max = allreduce_max(dist, skinf["dev_s"])
    ps_all = allreduce_sum(dist, skinf["psteps"])
    value = ps_all / t_max
    mixed_value = allreduce_sum(dist, mixed["psteps"]) / allreduce_max(dist, mixed["dev_s"])
    fixed_value = allreduce_sum(dist, fixed["psteps"]) / allreduce_max(dist, fixed["dev_s"])
    t_plain = allreduce_max(dist, plain["dev_s"])
    plain_value = allreduce_sum(dist, plain["psteps"]) / t_plain

    # roofline of the dominant kernel (the fused pair-force + integrate kernel)
    tm = phases["timings"]
    psteps_ph = min(args.steps, 200)
    force_s = tm["force_ms"] * 1e-3 / psteps_ph
    nelem = phases["n0"] + phases["n1"]  # mean elements per step (2 * mean cells)
    bytes_per_elem = 40  # pos in 16 + sigma 4 + id 4 + pos out 16 (2D, FP32-force form)
    achieved = bytes_per_elem * nelem / force_s / 1e9
    tp = plain["timings"]
    plain_force_s = tp["force_ms"] * 1e-3 / plain_steps
    traffic = profile_traffic()
    form = ("mixed precision, Philox noise, Verlet skin with the learned scheduler" if have_mlp
            else f"mixed precision, Philox noise, Verlet skin {args.skin} sigma")

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-force/f64-position", "data": "synthetic",
        "config": bench_config(world),
        "form": form + ", CUDA-graph replay of steady steps",
        "cells_timed": [skinf["n0"], skinf["n1"]],
        "forms": {"mixed_skin_scheduled" if have_mlp else "mixed_skin": value,
                  "mixed_skin_fixed_0.3": fixed_value,
                  "mixed_rebuild_every_step": mixed_value, "plain_fp64": plain_value,
                  "speedup_vs_plain_fp64": value / plain_value},
        "skin_stats": skinf["skin"],
        "graph_steps": skinf["graphs"]["graph_steps"],
        "autotuned": tune, "autotune_trials_ms_per_step": {f"{t['bin_factor']}/{t['staging']}/{t['occupancy']}/{t['block_size']}":
                                                          round(t["ms_per_step"], 4) for t in trials},
        "phases_ms_per_step": {k: tm[k] / psteps_ph for k in ("rebuild_ms", "force_ms", "events_ms")},
        "plain_fp64_phases_ms_per_step": {k: tp[k] / plain_steps for k in ("rebuild_ms", "force_ms", "events_ms")},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic,
                     "traffic_unit": "bytes per launch (ncu: dram__bytes_read.sum + dram__bytes_write.sum)",
                     "traffic_source": os.path.relpath(TRAFFIC_PROFILE, ROOT),
                     "peak_kind": peak_kind,
                     "kernel": "k_force_cells<2, softcore>", "algorithmic_bytes_per_element": bytes_per_elem,
                     "timed_on": f"{psteps_ph} individually launched steps (CUDA events around the force phase)",
                     "plain_fp64_kernel_GBps": 44 * nelem / plain_force_s / 1e9},
        "gpu_launches": skinf["timings"]["launches"],
        "clocks": clocks,
    }
    if args.only is None:
        # the reference's StochasticHeun (two force passes per step) in the headline form
        heun = run_form(G, p, st, G.PREC_MIXED, args.steps, args.warmup, device, 7 + rank, dist,
                        skin=mlp_skin if have_mlp else args.skin, sched=have_mlp, tune=tune,
                        integrator=G.INTEGRATOR_HEUN)
        line["forms"]["mixed_skin_heun"] = allreduce_sum(dist, heun["psteps"]) / allreduce_max(dist, heun["dev_s"])
        line["forms"]["mixed_skin_heun_ms_per_step"] = heun["dev_s"] / args.steps * 1e3
    if args.only is None and not args.no_batched:
        line["batched_sweep"] = run_batched(G, device, min(args.steps, 300), args.warmup, have_mlp)
        try:
            line["channel_3d"] = run_channel(G, device, min(args.steps, 200), args.warmup)
        except G.CilError as e:  # reported, not fatal to the headline line
            line["channel_3d"] = {"error": str(e)}
        try:
            line["cycle_model"] = run_cycle(G, device, min(args.steps, 200), args.warmup)
            line["cycle_model"]["fp32_contacts"] = run_cycle(G, device, min(args.steps, 200), args.warmup, 1)
            line["cycle_model"]["small_colony"] = run_cycle_small(G, device)
            line["cycle_model"]["dpd"] = run_cycle(G, device, min(args.steps, 200), args.warmup, 0, dpd=True)
            line["cycle_model"]["dpd"]["fp32_pair_terms"] = run_cycle(G, device, min(args.steps, 200), args.warmup, 1,
                                                                      dpd=True)
        except G.CilError as e:
            line["cycle_model"] = {"error": str(e)}
    if not args.no_e2e:
        e2e = run_e2e(G, p, st, G.PREC_MIXED, args.steps, device, 7 + rank, mlp_skin if have_mlp else args.skin,
                      sched=have_mlp, tune=tune)
        line["e2e"] = {"value": allreduce_sum(dist, e2e["value"]), "unit": UNIT,
                       "h2d_bytes_per_step": e2e["h2d"], "d2h_bytes_per_step": e2e["d2h"],
                       "frames": e2e["frames"], "frame_every": GTS, "gsd_file_bytes": e2e["file_bytes"]}
    if args.only is None and not args.no_batched:
        try:
            line["first_configuration"] = run_c1(G, device, min(args.steps, 1000), args.warmup,
                                                 os.cpu_count() or 1)
        except G.CilError as e:
            line["first_configuration"] = {"error": str(e)}
    if args.only is None and not args.no_frames:
        line["frame_output"] = run_frames(G, p, st, 3000, device, 7 + rank,
                                          mlp_skin if have_mlp else args.skin, have_mlp, tune)
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(p, st, os.cpu_count() or 1)
        # the same restatement on one host thread (a short sample: one or two steps)
        one = cpu_baseline(p, st, 1, budget_s=8.0)
        line["cpu_baseline"]["one_thread"] = {k: one[k] for k in ("value", "unit", "cores", "sample")}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
