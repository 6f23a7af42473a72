#!/usr/bin/env python3
"""Benchmark of the EMC hot path on GB300.

Workload (one "step" = one EMC time step of every particle): bulk silicon,
three paired Delta valleys (m_l 0.916, m_t 0.19, alpha 0.5 /eV), acoustic
(9 eV) + 3 g + 3 f zero-order intervalley phonons, T = 300 K, field 1e6 V/m
along <100>, dt = 1 fs, N = 2^20 electrons, 5000 steps; FP32 particle state,
FP64 observable sums.  Synthetic data (Maxwellian initial electrons).

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl engine|reference]

Prints one JSON line.  --impl reference times the reference's CPU algorithm
(the oracle port, bit-identical to the reference on the golden vectors) on the
host cores for the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s, FP32-batched vs plain GPU at ≤1% v_d error; Poisson ms/solve"
UNIT = "particle-steps/s"
BYTES_PER_PARTICLE_STEP = {"fp32": 72, "fp64": 136}  # state read + written once


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_over_ranks(ms: float, units: float, ws: int):
    """Max time and summed units over ranks (barrier included)."""
    if ws <= 1:
        return ms, units
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms, -units], dtype=torch.float64)
    dist.barrier()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([units], dtype=torch.float64)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t[0]), float(u[0])


class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.p = None
        self.path = os.path.join("/tmp", f"emcg_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        rows = []
        for ln in open(self.path):
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def silicon_model(v, precision):
    return v.silicon_electron("jacoboni", temperature=300.0, n_levels=1000, max_energy=1.0)


def run_engine(args):
    ws, rank, local = _dist()
    import torch
    torch.cuda.set_device(local)
    if ws > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl")
    import viennaemc_gb300 as v
    from viennaemc_gb300.bulk import BulkBatch, EnsembleSpec
    N, K, W, per = args.n, args.steps, args.warmup, args.steps_per_launch
    pt = silicon_model(v, "fp32")
    spec = EnsembleSpec(0, N, 1e6, (1, 0, 0), (1e-6,) * 3, 1e-15, 1234 + rank, 0, 300.0)
    b = BulkBatch([pt], [spec], "fp32")
    b.set_launch(args.block, per, args.min_blocks,
                 queued=args.scatter_mode, pass_actions=args.pass_actions)
    b.init_particles(0)
    # warm-up (untimed)
    b.step(W)
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB > L2
    sampler = ClockSampler(local)
    n_launch = (K + per - 1) // per
    kernel_ms = 0.0
    obs_all = []
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    sampler.start()
    t0 = time.perf_counter()
    done = 0
    for _ in range(n_launch):
        ns = min(per, K - done)
        flush.zero_()
        torch.cuda.synchronize()
        obs_all.append(b.step(ns))
        kernel_ms += b.last_kernel_ms()
        done += ns
    args.block_used = b.launch()["block_threads"]
    args.pass_actions_used = b.pass_actions()  # of the timed launch
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    ms, units = reduce_over_ranks(kernel_ms, float(N) * K, ws)
    value = units / (ms / 1e3)
    b.close()

    if args.skip_e2e:
        e2e_s, e2e_units, h2d, d2h = float("nan"), 0.0, 0, 0
    else:
        e2e_s, e2e_units, h2d, d2h = _e2e(v, pt, spec, args, N, K)
    if args.fp64_steps > 0:
        value64, precision, k64 = _precision(v, pt, args, N, per, rank)
    else:
        value64 = precision = k64 = None
    small = _small_bench(args, rank) if args.small_steps > 0 else None
    batched = _batched_bench(args, rank) if args.batch_steps > 0 else None
    device = _device_bench(args, rank) if args.device_steps > 0 else None
    if device is not None and args.mosfet_steps > 0:
        device["mosfet_sweep"] = _mosfet_bench(args, rank)
    p2p = _p2p_bench(args, rank) if args.p2p_n > 0 else None
    _report(args, ws, rank, N, K, W, per, ms, value, n_launch, e2e_s, e2e_units, h2d, d2h,
            value64, precision, k64, wall, clocks, device, batched, p2p, small)
    if ws > 1:
        torch.distributed.destroy_process_group()


E2E_CALLS = 5


def _e2e(v, pt, spec, args, N, K):
    """End to end through the C ABI: the host state in, in the float engine's
    own layout in page-locked memory, per-step observables out."""
    import torch
    from viennaemc_gb300.bulk import BulkBatch, ParticleStateF32
    st = ParticleStateF32.from_state(_host_state(v, N), pinned=True)
    b2 = BulkBatch([pt], [spec], "fp32")
    b2.set_launch(args.block, args.steps_per_launch, args.min_blocks,
                  pass_actions=args.pass_actions)
    # warm-up through the same call (untimed)
    b2.step_from_host(0, st, max(args.warmup, 3))
    torch.cuda.synchronize()
    # one call per pass: the first launch reads the start state from the
    # page-locked host block, the upload overlapping the steps; each pass
    # starts again from the same host state, and the median of E2E_CALLS
    # passes is reported
    times = []
    for _ in range(E2E_CALLS):
        t0 = time.perf_counter()
        o2 = b2.step_from_host(0, st, K, step0=0)
        times.append(time.perf_counter() - t0)
    e2e_s = statistics.median(times)
    b2.close()
    e2e_units = float(N) * K
    h2d = N * (9 * 4 + 4) / K
    d2h = o2.shape[-2] * 3 * 8
    return e2e_s, e2e_units, h2d, d2h


def _run_steps(b, k, per):
    """k steps in launches of at most per; (per-step sums, kernel ms)."""
    ms, obs = 0.0, []
    for d0 in range(0, k, per):
        obs.append(b.step(min(per, k - d0)))
        ms += b.last_kernel_ms()
    return np.concatenate(obs, axis=1), ms


def _run_snapshots(b, k, per, win, every=100):
    """k steps in launches of at most per, with the subvalley occupancy of
    the ensemble taken every `every` steps inside the window; (per-step sums,
    kernel ms, mean occupancy, final state)."""
    ms, obs, occ, done = 0.0, [], [], 0
    while done < k:
        ns = min(per, k - done)
        if done >= win.start:
            ns = min(ns, every)
        elif done + ns > win.start:
            ns = win.start - done
        obs.append(b.step(ns))
        ms += b.last_kernel_ms()
        done += ns
        if done > win.start and (done - win.start) % every == 0:
            st = b.get_state(0)
            occ.append(np.bincount(np.asarray(st.sub), minlength=3)[:3] / max(st.n, 1))
    return np.concatenate(obs, axis=1), ms, np.mean(occ, axis=0), b.get_state(0)


def _observables(obs, occ, n, win):
    """Mean drift velocity and energy over the step window, and the mean
    subvalley occupancy of the snapshots in it (the valley repopulation a
    field along <100> drives)."""
    from viennaemc_gb300.bulk import BulkBatch
    a = BulkBatch.averages(obs, [n])
    return {"drift_velocity": float(a["drift_velocity"][0, win, 0].mean()),
            "energy": float(a["energy"][0, win, 0].mean()),
            "subvalley_occupancy": [float(x) for x in occ]}


def _precision(v, pt, args, N, per, rank):
    """The FP32 engine against its precision oracle, the FP64 engine run from the
    same initial electrons with the same seed and the same random numbers
    (EMCG_ENS_FLOAT_DRAWS), per observable; the seed-to-seed sigma of the FP32
    observables (extra seeds) beside it; and the plain FP64 engine's speed."""
    from viennaemc_gb300.bulk import BulkBatch, EnsembleSpec
    k64 = args.fp64_steps
    win = slice(max(0, k64 - 500), k64)
    seed = 4321 + rank

    def spec(s, fd=False):
        return EnsembleSpec(0, N, 1e6, (1, 0, 0), (1e-6,) * 3, 1e-15, s, 0, 300.0, fd)
    b32 = BulkBatch([pt], [spec(seed)], "fp32")
    b32.set_launch(args.block, per, args.min_blocks, queued=args.scatter_mode)
    b32.init_particles(0)
    st0 = b32.get_state(0)
    o32, _, occ32, s32 = _run_snapshots(b32, k64, per, win)
    b32.close()
    b64 = BulkBatch([pt], [spec(seed, True)], "fp64")
    b64.set_launch(args.block, per)
    b64.set_state(0, st0)
    o64, _, occ64, s64 = _run_snapshots(b64, k64, per, win)
    b64.close()
    r32, r64 = _observables(o32, occ32, N, win), _observables(o64, occ64, N, win)
    # electrons still on the same path: same subvalley, energy within float
    # rounding grown over the run (the others branched on a rounding)
    same = (s32.sub == s64.sub) & (np.abs(s32.energy - s64.energy)
                                   <= 1e-3 * np.abs(s64.energy) + 1e-5)
    # seed-to-seed spread of one FP32 run's observables
    extra = []
    for k in range(args.precision_seeds):
        b = BulkBatch([pt], [spec(seed + 1 + k)], "fp32")
        b.set_launch(args.block, per, args.min_blocks, queued=args.scatter_mode)
        b.init_particles(0)
        o, _, occ, _ = _run_snapshots(b, k64, per, win)
        extra.append(_observables(o, occ, N, win))
        b.close()
    out = {"oracle": "FP64 engine, same initial electrons, same seed, same random numbers "
                     "(float draws widened to double)",
           "steps": k64, "window_steps": [win.start, win.stop],
           "occupancy": "mean of 5 snapshots of the ensemble, every 100 steps in the window",
           "same_path_fraction": float(same.mean()), "observables": {}}
    for key in ("drift_velocity", "energy"):
        x32, x64 = r32[key], r64[key]
        sd = float(np.std([e[key] for e in extra + [r32]], ddof=1)) if extra else None
        out["observables"][key] = {"fp32": x32, "fp64": x64, "rel": abs(x32 - x64) / abs(x64),
                                   "seed_sigma_rel": sd / abs(x64) if sd is not None else None}
    o32v, o64v = np.array(r32["subvalley_occupancy"]), np.array(r64["subvalley_occupancy"])
    sd = (np.std([e["subvalley_occupancy"] for e in extra + [r32]], axis=0, ddof=1).max()
          if extra else None)
    out["observables"]["subvalley_occupancy"] = {
        "fp32": r32["subvalley_occupancy"], "fp64": r64["subvalley_occupancy"],
        "abs": float(np.abs(o32v - o64v).max()),
        "seed_sigma_abs": float(sd) if sd is not None else None}
    out["seeds_for_sigma"] = len(extra) + 1
    # the plain FP64 engine (its own 64-bit draws) on the same workload: speed
    b = BulkBatch([pt], [spec(999 + rank)], "fp64")
    b.set_launch(args.block, per)
    b.set_state(0, st0)
    _, ms_plain = _run_steps(b, k64, per)
    b.close()
    return N * k64 / (ms_plain / 1e3), out, k64


def _report(args, ws, rank, N, K, W, per, ms, value, n_launch, e2e_s, e2e_units, h2d, d2h,
            value64, precision, k64, wall, clocks, device=None, batched=None, p2p=None,
            small=None):
    peak, peak_src = _peaks()
    bpp = BYTES_PER_PARTICLE_STEP["fp32"]
    achieved = bpp * value / 1e9  # algorithmic GB/s (72 B per particle-step)
    kernel = {0: "lockstep", 1: "block-queued", 2: "warp-asynchronous"}[args.scatter_mode]
    ns_launch = min(per, K)  # steps of each timed launch
    prof = _profiled(kernel, ns_launch)
    traffic = prof["dram_bytes_per_electron"] * N if prof else None
    sms, sm_mhz = _sm_count(), (clocks or {}).get("sm_mhz") or 2070.0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "bulk Si, 2^20 electrons, 1e6 V/m <100>, dt 1 fs (the "
                               "5000-step configuration; the timed steps below)",
                   "particles": N, "steps_timed": K, "launches_timed": n_launch,
                   "steps_per_launch": ns_launch,
                   "block_threads": getattr(args, "block_used", args.block),
                   "min_blocks_per_sm": args.min_blocks,
                   "scatter_kernel": kernel,
                   "pass_actions": getattr(args, "pass_actions_used", None),
                   "l2": "flushed (256 MB write) between timed launches",
                   "observables": "per-step FP64 sums of E, v.dir, count"},
        "e2e": {"value": e2e_units / e2e_s if e2e_units else None, "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "emcg_bulk_step_from_host: float-layout host state (40 B per "
                        "electron, page-locked) read by the first launch, per-step "
                        "observables back; host wall clock, median of "
                        f"{E2E_CALLS} calls of the timed steps"},
        "gpu_launches": n_launch,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_src,
                     "bytes_per_unit": bpp, "unit_of_work": "particle-step",
                     "algorithmic_bytes_per_launch": bpp * N * ns_launch,
                     "traffic_per": "timed launch (steps_per_launch steps), from the ncu "
                                    "capture of the closest launch length",
                     "traffic_source": prof["source"] if prof else None},
        "wall_s": wall,
    }
    if prof:
        # the kernel's real limit: instruction issue (one warp instruction per
        # scheduler and cycle, four schedulers per SM)
        ipu = prof["warp_instructions_per_particle_step"]
        ipeak = sms * 4 * sm_mhz * 1e6
        line["roofline_issue"] = {"bound": "issue", "achieved": ipu * value, "peak": ipeak,
                                  "unit": "warp instructions/s", "frac": ipu * value / ipeak,
                                  "instructions_per_unit": ipu, "unit_of_work": "particle-step",
                                  "peak_basis": f"{sms} SMs x 4 schedulers x {sm_mhz:.0f} MHz",
                                  "source": prof["source"]}
    if value64:
        line["fp64_engine"] = {"value": value64, "unit": UNIT, "steps": k64,
                               "fp32_speedup": value / value64}
        line["fp32_error"] = precision
    if clocks:
        line["clocks"] = clocks
    if small:
        line["small"] = small
    if batched:
        line["batched"] = batched
    if device:
        line["device"] = device
    if p2p:
        line["p2p_coulomb"] = p2p
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(N, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)


def sweep_specs(seed=2024):
    """64 bulk Si ensembles: {<100>, <111>} x T in {77, 200, 300, 400} K x 8
    fields log-spaced over 1e4 .. 1e7 V/m, particle counts log-uniform in
    [1e4, 1e6] drawn from the seed."""
    from viennaemc_gb300.bulk import EnsembleSpec
    rs = np.random.default_rng(seed)
    temps = (77.0, 200.0, 300.0, 400.0)
    specs = []
    for d in ((1, 0, 0), (1, 1, 1)):
        for m, T in enumerate(temps):
            for f in np.logspace(4, 7, 8):
                n = int(round(10 ** rs.uniform(4, 6)))
                specs.append(EnsembleSpec(m, n, float(f), d, (1e-6,) * 3, 1e-15,
                                          int(rs.integers(1, 2 ** 31)), 0, T))
    return temps, specs


def _rate_rebuild_timing(b, models, reps=50):
    """reinitScatterTables on the GPU from rates already in device memory:
    host wall time per model rebuild (the call, the stream-ordered kernel),
    averaged over reps rebuilds of every model, the stream drained at the end."""
    import torch
    raws = [torch.tensor(m.raw_rates(), dtype=torch.float64, device="cuda") for m in models]
    b.get_rates(0)  # drains the handle's stream
    t0 = time.perf_counter()
    for _ in range(reps):
        for mi, r in enumerate(raws):
            b.reinit_scatter_tables(mi, r)
    b.get_rates(0)
    us = (time.perf_counter() - t0) / (reps * len(raws)) * 1e6
    h = models[0].scatterHandler
    return {"us_per_model": us, "tables": sum(len(v) for v in h.table_mechs.values()),
            "levels": h.n_levels, "source": "device rates (CUDA tensor)",
            "timing": "host wall clock, call + kernel, %d rebuilds of %d models" %
                      (reps, len(raws))}


def _p2p_bench(args, rank):
    """Particle-particle Coulomb sums of the FMM handlers, direct on the GPU:
    n electrons and donors in a cube with the 1 nm cutoff; FP32 and FP64 pair
    terms; the oracle's direct sum on the host cores for a bounded sample of
    targets."""
    from viennaemc_gb300 import p2p
    n = args.p2p_n
    rs = np.random.default_rng(7 + rank)
    box = 1e-7
    pos = rs.random((3, n)) * box
    q = np.where(np.arange(n) % 2 == 0, -1.0, 1.0) * 1.60219e-19
    out = {"workload": f"{n} charges (electrons and donors alternating) in a {box:g} m cube, "
                       "1 nm cutoff, no periodic copies", "pairs": n * (n - 1)}
    for prec in ("fp32", "fp64"):
        p2p.coulomb(pos[:, :2048], q[:2048], precision=prec)  # warm-up
        ms = []
        for _ in range(3 if prec == "fp32" else 1):
            _, _, k = p2p.coulomb(pos, q, precision=prec, return_ms=True)
            ms.append(k)
        out[prec] = {"kernel_ms": min(ms), "pairs_per_s": n * (n - 1) / (min(ms) / 1e3)}
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle as po
        po.build()
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        po.p2p_coulomb(pos, q, 1e9, threads=threads)
        el = time.perf_counter() - t0
        out["cpu_oracle"] = {"pairs_per_s": n * (n - 1) / el, "cores": threads,
                             "kind": "port", "sample": f"the same {n} charges, double"}
    return out


def _small_bench(args, rank):
    """The plain method's small case: bulk Si, 10,000 electrons, 1e5 V/m
    along <100>, dt 1 fs, 3,000 steps, FP64 engine; the FP32 engine beside
    it; the reference algorithm (oracle port, FP64) on the host cores for the
    same workload."""
    import viennaemc_gb300 as v
    from viennaemc_gb300.bulk import BulkBatch, EnsembleSpec
    n, K, per = 10000, args.small_steps, 500
    pt = silicon_model(v, "fp64")
    out = {"workload": "bulk Si, 10,000 electrons, 1e5 V/m <100>, dt 1 fs, 3,000 steps, FP64",
           "particles": n, "steps": K}
    for prec, block in (("fp64", 64), ("fp32", 64)):
        spec = EnsembleSpec(0, n, 1e5, (1, 0, 0), (1e-6,) * 3, 1e-15, 77 + rank, 0, 300.0)
        b = BulkBatch([pt], [spec], prec)
        b.set_launch(block, per)
        b.init_particles(0)
        o, ms, occ, _ = _run_snapshots(b, K, per, slice(K // 2, K), every=K // 10)
        r = _observables(o, occ, n, slice(K // 2, K))
        b.close()
        out[prec] = {"value": n * K / (ms / 1e3), "unit": UNIT, "kernel_ms": ms,
                     "block_threads": block, **r}
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle as po
        po.build()
        threads = os.cpu_count() or 1
        m = po.silicon_model("jacoboni")
        st = _oracle_state(po, n)
        t0 = time.perf_counter()
        m.bulk_run_philox(st, 1e-15, [-1.60219e-19 * 1e5, 0, 0], [1e-6] * 3, [1, 0, 0], 7, 0,
                          0, K, threads, True)
        el = time.perf_counter() - t0
        out["cpu_reference"] = {"value": n * K / el, "unit": UNIT, "cores": threads,
                                "kind": "port", "sample": "the whole workload, FP64"}
    return out


def _batched_bench(args, rank):
    """The velocity-field sweep in one launch per chunk of steps: FP32 state,
    autotuned launch shape, CUDA-graph replay; the plain FP64 engine on the same
    batch for the speed ratio and the drift-velocity error."""
    import torch
    import viennaemc_gb300 as v
    from viennaemc_gb300.bulk import BulkBatch
    temps, specs = sweep_specs(2024 + rank)
    models = [v.silicon_electron("jacoboni", temperature=T, n_levels=3000, max_energy=3.0)
              for T in temps]
    ntot = sum(s.n_particles for s in specs)
    b = BulkBatch(models, specs, "fp32")
    for e in range(len(specs)):
        b.init_particles(e)
    b.set_launch(256, args.steps_per_launch)
    tuned = b.autotune(args.batch_trial)
    b.set_graph(True)
    b.step(max(args.warmup // 4, 3))
    K = args.batch_steps
    torch.cuda.synchronize()
    ms, done, obs = 0.0, 0, []
    while done < K:
        ns = min(args.steps_per_launch, K - done)
        obs.append(b.step(ns))
        ms += b.last_kernel_ms()
        done += ns
    rebuild = _rate_rebuild_timing(b, models)
    b.close()
    value = ntot * K / (ms / 1e3)
    out = {"workload": "64 bulk Si ensembles: <100>,<111> x 77/200/300/400 K x 8 fields "
                       "1e4-1e7 V/m, counts log-uniform 1e4-1e6, dt 1 fs",
           "ensembles": len(specs), "particles_total": ntot, "steps": K, "value": value,
           "unit": UNIT, "ms_per_step": ms / K, "autotune": tuned, "graph_replay": True,
           "steps_per_launch": args.steps_per_launch,
           "l2": "working set larger than L2 (%.0f MB of particle state)" % (ntot * 40 / 1e6),
           "rate_rebuild": rebuild}
    if args.batch_fp64_steps > 0:
        out.update(_batched_precision(args, models, specs, ntot))
    return out


def _batched_precision(args, models, specs, ntot):
    """The sweep's FP32 run against the FP64 engine from the same initial
    electrons with the same seeds and random numbers (float draws), per
    ensemble: mean energy and drift velocity over the second half of the
    steps; and the plain FP64 engine's speed on the same batch."""
    import dataclasses
    from viennaemc_gb300.bulk import BulkBatch
    k64, per = args.batch_fp64_steps, args.steps_per_launch
    b32 = BulkBatch(models, specs, "fp32")
    for e in range(len(specs)):
        b32.init_particles(e)
    st0 = [b32.get_state(e) for e in range(len(specs))]
    b32.set_launch(256, min(k64, per))
    o32, ms32 = _run_steps(b32, k64, per)
    s32 = [b32.get_state(e) for e in range(len(specs))]
    b32.close()
    runs = {}
    for mode, fd in (("same_draws", True), ("plain", False)):
        b64 = BulkBatch(models, [dataclasses.replace(s, float_draws=fd) for s in specs], "fp64")
        for e in range(len(specs)):
            b64.set_state(e, st0[e])
        b64.set_launch(256, min(k64, per))
        runs[mode] = _run_steps(b64, k64, per)
        if fd:
            s64 = [b64.get_state(e) for e in range(len(specs))]
        b64.close()
    win = slice(k64 // 2, k64)
    e_err, v_err, same = [], [], []
    for e, sp in enumerate(specs):
        a, r = s32[e], s64[e]
        same.append(float(((a.sub == r.sub) & (np.abs(a.energy - r.energy)
                                                <= 1e-3 * np.abs(r.energy) + 1e-5)).mean()))
        a32 = BulkBatch.averages(o32[e:e + 1], [sp.n_particles])
        a64 = BulkBatch.averages(runs["same_draws"][0][e:e + 1], [sp.n_particles])
        e32, e64 = a32["energy"][0, win, 0].mean(), a64["energy"][0, win, 0].mean()
        e_err.append(abs(e32 - e64) / e64)
        if sp.field_strength >= 1e5:
            v32, v64 = (a["drift_velocity"][0, win, 0].mean() for a in (a32, a64))
            v_err.append(abs(v32 - v64) / abs(v64))
    return {"fp64_engine": {"value": ntot * k64 / (runs["plain"][1] / 1e3), "steps": k64,
                            "fp32_speedup_same_steps": runs["plain"][1] / ms32},
            "fp32_error": {"oracle": "FP64 engine, same initial electrons, seeds and random "
                                     "numbers (float draws widened to double)",
                           "energy_max_rel": float(max(e_err)), "ensembles": len(e_err),
                           "drift_velocity_max_rel": float(max(v_err)),
                           "drift_velocity_ensembles": len(v_err),
                           "same_path_fraction_min": float(min(same)),
                           "window_steps": [win.start, win.stop],
                           "rule": "energy: every ensemble; drift velocity: fields >= 1e5 V/m"}}


def resistor_device(D, P):
    """2-D n+ Si resistor: 100 nm x 50 nm, 0.5 nm spacing (201 x 101 nodes),
    Nd = 1e24 m^-3, ohmic contacts at both ends with 0.5 V across, width
    1e-4 m so that about 5e5 electrons fill it."""
    dev = D.Device(P.silicon_material(), (100e-9, 50e-9), (0.5e-9, 0.5e-9))
    dev.setDeviceWidth(1e-4)
    dev.addConstantDopingRegion((0, 0), (100e-9, 50e-9), 1e24)
    dev.addOhmicContact(D.XMAX, 0.0, (0,), (50e-9,))
    dev.addOhmicContact(D.XMIN, 0.5, (0,), (50e-9,))
    return dev


def _device_bench(args, rank):
    """The device path on the resistor: performEMCStep (Poisson -> E -> move ->
    contacts -> CIC assignment) every 0.1 fs in FP32 with the float-multigrid /
    double-Newton Poisson solve to 1e-8 relative residual; the reference's SOR
    (omega 1.8, 1e-4 V) is timed on the host on the same potential and
    concentration."""
    from viennaemc_gb300 import device as D
    from viennaemc_gb300 import physics as P
    dev = resistor_device(D, P)
    pt = P.silicon_electron("refbulk", n_levels=1000, max_energy=4.0, regions=[0], coulomb=True,
                            region_doping=dev.getDopingRegionDoping)
    sim = D.DeviceSimulation(dev, pt, scheme=D.CIC, dt=1e-16, seed=11 + rank, precision="fp32",
                             poisson_rtol=1e-8, poisson_max_cycles=60, poisson_fp32=True)
    sim.calcEquilibriumCharacteristics()
    sim.performEMCStep(args.device_warmup)
    n0 = sim.num_particles()
    K = args.device_steps
    t0 = time.perf_counter()
    sim.performEMCStep(K)
    wall = time.perf_counter() - t0
    n1 = sim.num_particles()
    step_ms, pois_ms = sim.timing()
    cycles, solves = sim.poisson_counts()
    cur = sim.current()
    out = {"workload": "2-D Si resistor 100 x 50 nm, 201 x 101 nodes, Nd 1e24, 0.5 V, CIC, "
                       "dt 0.1 fs, acoustic + zero/first-order IV + Coulomb",
           "particles": [n0, n1], "steps": K, "warmup": args.device_warmup,
           "value": 0.5 * (n0 + n1) * K / (step_ms / 1e3), "unit": UNIT,
           "ms_per_step": step_ms / K, "poisson_ms_per_solve": pois_ms / K,
           "poisson_newton_per_solve": cycles / max(solves, 1),
           "poisson": "double Newton steps, each with 3 float multigrid V-cycles; stop at 1e-8 "
                      "relative residual",
           "wall_s": wall, "current_A": [float(c) for c in cur]}
    out.update(_device_rooflines(out["value"], pois_ms / K, cycles / max(solves, 1),
                                 dev.nx * dev.ny))
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_reference_sor"] = _cpu_sor(dev, sim.potential, sim.concentration)
    # the same steps with the reference SOR's stopping rule (no update above 1e-4 V)
    sim.set_poisson(update_tol=1e-4)
    K2 = max(K // 4, 1)
    sim.performEMCStep(K2)
    step2, pois2 = sim.timing()
    cyc2, sol2 = sim.poisson_counts()
    out["reference_rule"] = {"steps": K2, "ms_per_step": step2 / K2,
                             "poisson_ms_per_solve": pois2 / K2,
                             "poisson_newton_per_solve": cyc2 / max(sol2, 1),
                             "rule": "stop once a Newton update moves no node by more than "
                                     "1e-4 V (the reference SOR's rule at its accuracy)"}
    sim.close()
    return out


def _device_rooflines(psteps, pois_ms, newton, nodes, pre=3, post=3, vcycles=3):
    """The device step's two bounds: the particle kernels against HBM
    (64 B per particle-step, the 2-D float state read and written once) and
    the Poisson solve's algorithmic bytes (per V-cycle and level, pre + post
    sweeps and one residual of 16 B per node, levels adding a third) against
    the same peak: the grids stay in shared memory and L2, so both report how
    far the step is from a bandwidth bound, not the bound itself (launch and
    barrier latency)."""
    peak, src = _peaks()
    pbytes = (pre + post + 1) * 16.0 * nodes * 4.0 / 3.0 * vcycles * newton
    pgbs = pbytes / (pois_ms * 1e-3) / 1e9
    agbs = psteps * 64.0 / 1e9
    return {"particle_roofline": {"bound": "hbm", "bytes_per_unit": 64,
                                  "unit_of_work": "particle-step", "achieved": agbs,
                                  "peak": peak, "unit": "GB/s", "frac": agbs / peak,
                                  "peak_source": src},
            "poisson_roofline": {"bound": "latency", "algorithmic_bytes_per_solve": pbytes,
                                 "achieved": pgbs, "peak": peak, "unit": "GB/s",
                                 "frac": pgbs / peak, "peak_source": src,
                                 "note": "grids resident in shared memory and L2; the solve "
                                         "waits on barriers (profiles/poisson_cluster_"
                                         "resistor_201x101_full.md)"}}


def mosfet_device(D, P, vds, vgs=1.0, width=1.3e-6):
    """2-D Si n-MOSFET: 200 nm x 100 nm at 0.5 nm (401 x 201 nodes), gate
    length 50 nm over 1 nm SiO2 (eps_r 3.9, barrier Eg/2), source and drain
    Nd = 1e26 m^-3 to 20 nm depth, channel and bulk Na = 1e24 m^-3, substrate
    contact at the back; the contact layout of the reference mosfet2D.  The
    device width sets the superparticle count (about 3.9e5 at 1.3 um)."""
    mat = P.silicon_material()
    dev = D.Device(mat, (200e-9, 100e-9), (0.5e-9, 0.5e-9))
    dev.setDeviceWidth(width)
    dev.addConstantDopingRegion((0, 20e-9), (200e-9, 100e-9), -1e24)
    dev.addConstantDopingRegion((0, 0), (75e-9, 20e-9), 1e26)
    dev.addConstantDopingRegion((75e-9, 0), (125e-9, 20e-9), -1e24)
    dev.addConstantDopingRegion((125e-9, 0), (200e-9, 20e-9), 1e26)
    dev.addOhmicContact(D.YMAX, 0.0, (0,), (200e-9,))
    dev.addOhmicContact(D.YMIN, 0.0, (0,), (75e-9,))
    dev.addGateContact(D.YMIN, vgs, (75e-9,), (125e-9,), 3.9, 1e-9, 1.12 / 2)
    dev.addOhmicContact(D.YMIN, vds, (125e-9,), (200e-9,))
    return dev


# uneven superparticle counts of the eight bias points, 2e5 .. 6e5 (device
# width in proportion), in an order unrelated to the bias
MOSFET_COUNTS = (4.3e5, 2.0e5, 6.0e5, 3.1e5, 5.4e5, 2.6e5, 4.9e5, 3.6e5)


def _mosfet_bench(args, rank):
    """Eight drain biases 0..1 V at Vgs = 1 V stepped together as one batch
    of uneven ensembles (2e5 to 6e5 superparticles, one engine per bias, each
    on its own stream), FP32 particles, per-step Poisson to 1e-8."""
    from viennaemc_gb300 import device as D
    from viennaemc_gb300 import physics as P
    sims, widths = [], []
    for k, vds in enumerate(np.linspace(0.0, 1.0, 8)):
        widths.append(1.3e-6 * MOSFET_COUNTS[k] / 3.9e5)
        dev = mosfet_device(D, P, float(vds), width=widths[-1])
        regs = list(range(dev.n_regions))
        pt = P.silicon_electron("refbulk", n_levels=1000, max_energy=4.0, regions=regs,
                                coulomb=True, region_doping=dev.getDopingRegionDoping,
                                first_order=False)
        sim = D.DeviceSimulation(dev, pt, scheme=D.CIC, dt=1e-16, seed=100 + k + 8 * rank,
                                 precision="fp32", poisson_rtol=1e-8, poisson_max_cycles=200,
                                 tau_region_is_valley=True)
        sim.calcEquilibriumCharacteristics()
        sims.append(sim)
    D.DeviceSimulation.performEMCStepMany(sims, args.device_warmup)
    n0 = [s.num_particles() for s in sims]
    K = args.mosfet_steps
    t0 = time.perf_counter()
    D.DeviceSimulation.performEMCStepMany(sims, K)
    wall = time.perf_counter() - t0
    n1 = [s.num_particles() for s in sims]
    pois = [s.timing()[1] / K for s in sims]
    step = [s.timing()[0] / K for s in sims]
    drain = [float(s.current(args.device_warmup)[3]) for s in sims]
    for s in sims:
        s.close()
    tot = sum(0.5 * (a + b) for a, b in zip(n0, n1))
    return {"workload": "Si n-MOSFET 401 x 201 nodes (0.5 nm), Lg 50 nm, 1 nm SiO2, S/D 1e26, "
                        "channel 1e24, Vgs 1 V, Vds = 0..1 V in 8 steps, one engine per bias, "
                        "uneven superparticle counts 2e5-6e5",
            "steps": K, "particles": n1, "wall_ms_per_step": 1e3 * wall / K,
            "value": tot * K / wall, "unit": UNIT,
            "device_ms_per_step_each": step, "poisson_ms_per_solve_each": pois,
            "drain_current_A": drain,
            "drain_current_A_per_m": [i / w for i, w in zip(drain, widths)],
            "note": "value = particles of all 8 engines x steps / wall time of the batch "
                    "(host-timed, the engines overlap on the GPU)"}


def _cpu_sor(dev, pot, conc, repeats=3):
    """The reference's SOR solve (oracle port, one thread like the reference)
    from the engine's potential with its latest concentration."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    ct = np.array([c[0] for c in dev.contacts], np.int32)
    cv = np.array([c[1] for c in dev.contacts], np.float64)
    cp = np.array([p for c in dev.contacts for p in c[2]], np.float64).reshape(-1, 3)
    od = po.Device(dev.nx, dev.ny, dev.spacing[0], dev.spacing[1], dev.width, dev.doping,
                   dev.region, dev.bnd, ct, cv, cp)
    od.set_max(*dev.max_pos)
    times, sweeps = [], []
    for _ in range(repeats):
        t0 = time.perf_counter()
        _, n = od.sor(pot, conc, 1.8, 1e-4, False)
        times.append(time.perf_counter() - t0)
        sweeps.append(int(n))
    out = {"ms_per_solve": 1e3 * statistics.median(times), "sweeps": sweeps, "cores": 1,
           "kind": "port", "sample": f"{repeats} solves on the engine's last potential and "
                                     "concentration, omega 1.8, accuracy 1e-4 V"}
    # the same solve run to the engine's accuracy (1e-8 relative residual):
    # tighten the SOR accuracy until the residual meets it (bounded time)
    r0 = rel_residual(dev, pot, conc)
    t_all = 0.0
    for acc in (1e-5, 1e-6, 1e-7, 1e-8, 1e-9, 1e-10, 1e-11, 1e-12):
        t0 = time.perf_counter()
        sol, n = od.sor(pot, conc, 1.8, acc, False)
        dt = time.perf_counter() - t0
        t_all += dt
        r = rel_residual(dev, sol, conc)
        if r <= 1e-8 or t_all > 60:
            out["equal_accuracy"] = {"ms_per_solve": 1e3 * dt, "sweeps": int(n), "accuracy_V": acc,
                                     "rel_residual": r, "start_rel_residual": r0,
                                     "met": bool(r <= 1e-8)}
            break
    return out


def rel_residual(dev, pot, conc):
    """max |F| / max hP (|C| + n + p) of the reference's discrete Poisson
    equation (no gate contacts) over the nodes that are not ohmic reservoirs."""
    kB, q, eps0 = 1.38066e-23, 1.60219e-19, 8.85419e-12
    mat = dev.material
    Vt = kB / q * dev.temperature
    Ld = np.sqrt(eps0 * mat.epsR * Vt / q / mat.Ni)
    h0, h1 = dev.spacing[0] / Ld, dev.spacing[1] / Ld
    nx, ny = dev.nx, dev.ny
    phi = np.asarray(pot).reshape(ny, nx)
    n = np.asarray(conc).reshape(ny, nx)
    C = (dev.doping / mat.Ni).reshape(ny, nx)
    w = np.concatenate([phi[:, 1:2], phi[:, :-1]], axis=1)
    e = np.concatenate([phi[:, 1:], phi[:, -2:-1]], axis=1)
    so = np.concatenate([phi[1:2, :], phi[:-1, :]], axis=0)
    no = np.concatenate([phi[1:, :], phi[-2:-1, :]], axis=0)
    p = np.exp(-phi)
    F = h1 / h0 * (w + e - 2 * phi) + h0 / h1 * (so + no - 2 * phi) + h0 * h1 * (p - n + C)
    free = np.ones((ny, nx), bool)
    for b, idx in ((0, (slice(None), 0)), (1, (slice(None), nx - 1))):
        cont = np.asarray(dev.bnd[b])
        ohmic = np.array([c >= 0 and dev.contacts[c][0] == 0 for c in cont])
        free[idx] &= ~ohmic
    for b, idx in ((2, (0, slice(1, nx - 1))), (3, (ny - 1, slice(1, nx - 1)))):
        cont = np.asarray(dev.bnd[b])[1:nx - 1]
        ohmic = np.array([c >= 0 and dev.contacts[c][0] == 0 for c in cont])
        free[idx] &= ~ohmic
    scale = np.max(h0 * h1 * (np.abs(C) + n + p)[free])
    return float(np.max(np.abs(F[free])) / scale)


def _host_state(v, N):
    """A host-side Maxwellian state (the public API's input form), in
    page-locked memory."""
    rs = np.random.default_rng(5)
    from viennaemc_gb300.bulk import ParticleState
    st = ParticleState(N, pinned=True)
    E = -1.5 * (1.38066e-23 / 1.60219e-19 * 300.0) * np.log(rs.uniform(1e-6, 1, N))
    k = np.sqrt(2 * 0.2586 * 9.11e-31 * E * (1 + 0.5 * E) * 1.60219e-19) / 1.05459e-34
    ct = 1 - 2 * rs.random(N)
    ph = 2 * np.pi * rs.random(N)
    stt = np.sqrt(1 - ct * ct)
    st.kx[:], st.ky[:], st.kz[:] = k * stt * np.cos(ph), k * stt * np.sin(ph), k * ct
    st.px[:], st.py[:], st.pz[:] = (rs.random((3, N)) * 1e-6)
    st.energy[:] = E
    st.tau[:] = -np.log(rs.uniform(1e-6, 1, N)) * 8.7e-15
    st.grain_tau[:] = 1.0
    st.sub[:] = rs.integers(0, 3, N)
    return st


def _profiled(kernel, steps):
    """The committed ncu figures of the bulk kernel's launch closest in length
    to `steps` steps: DRAM bytes per electron per launch (the fused kernel
    reads and writes the state once per launch) and issued warp instructions
    per particle-step; None when no capture of the kernel is committed."""
    p = os.path.join(ROOT, "profiles", "bulk_step_fp32_counters.json")
    try:
        with open(p) as f:
            caps = json.load(f)["kernels"][kernel]["launches"]
        return min(caps, key=lambda c: abs(np.log(c["steps"] / max(steps, 1))))
    except (OSError, KeyError, ValueError):
        return None


def _sm_count():
    try:
        import torch
        return torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        return 152


def cpu_baseline(N, seconds):
    """The reference algorithm (oracle port) on all host cores, bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    threads = os.cpu_count() or 1
    m = po.silicon_model("jacoboni")
    n = min(N, 1 << 18)
    st = _oracle_state(po, n)
    force = [-1.60219e-19 * 1e6, 0, 0]
    t0 = time.perf_counter()
    m.bulk_run_philox(st, 1e-15, force, [1e-6] * 3, [1, 0, 0], 7, 0, 0, 20, threads, False)
    dt20 = time.perf_counter() - t0
    steps = int(max(20, min(2000, seconds / max(dt20 / 20, 1e-9))))
    t0 = time.perf_counter()
    m.bulk_run_philox(st, 1e-15, force, [1e-6] * 3, [1, 0, 0], 7, 0, 20, steps, threads, True)
    el = time.perf_counter() - t0
    return {"value": n * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} electrons x {steps} steps of the same workload (FP64, per-step "
                      f"observables), OpenMP over particles"}


def _oracle_state(po, n):
    rs = np.random.default_rng(3)
    st = po.State(n)
    E = -1.5 * (1.38066e-23 / 1.60219e-19 * 300.0) * np.log(rs.uniform(1e-6, 1, n))
    k = np.sqrt(2 * 0.2586 * 9.11e-31 * E * (1 + 0.5 * E) * 1.60219e-19) / 1.05459e-34
    ct = 1 - 2 * rs.random(n)
    ph = 2 * np.pi * rs.random(n)
    stt = np.sqrt(1 - ct * ct)
    st.kx[:], st.ky[:], st.kz[:] = k * stt * np.cos(ph), k * stt * np.sin(ph), k * ct
    st.E[:] = E
    st.tau[:] = -np.log(rs.uniform(1e-6, 1, n)) * 8.7e-15
    st.gtau[:] = 1.0
    st.sub[:] = rs.integers(0, 3, n)
    return st


def run_reference(args):
    ws, rank, local = _dist()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    threads = os.cpu_count() or 1
    m = po.silicon_model("jacoboni")
    N, K, W = args.n, args.steps, args.warmup
    st = _oracle_state(po, N)
    force = [-1.60219e-19 * 1e6, 0, 0]
    m.bulk_run_philox(st, 1e-15, force, [1e-6] * 3, [1, 0, 0], 7, 0, 0, max(W, 3), threads, True)
    # each timed step is the full 2^20-electron step; cap the count so the run
    # stays within a few minutes
    t0 = time.perf_counter()
    m.bulk_run_philox(st, 1e-15, force, [1e-6] * 3, [1, 0, 0], 7, 0, W, 5, threads, True)
    per = (time.perf_counter() - t0) / 5
    k_run = int(max(5, min(K, 120.0 / max(per, 1e-9))))
    t0 = time.perf_counter()
    m.bulk_run_philox(st, 1e-15, force, [1e-6] * 3, [1, 0, 0], 7, 0, W + 5, k_run, threads, True)
    el = time.perf_counter() - t0
    value = N * k_run / el
    sample = (f"{N} electrons x {k_run} steps (of {K} requested) of the same workload, "
              f"FP64, per-step observables, OpenMP over particles on {threads} threads")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": k_run,
            "warmup": W, "ms_per_step": el / k_run * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "bulk Si, 2^20 electrons, 1e6 V/m <100>, dt 1 fs, 5000 steps",
                       "particles": N},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def build_parser():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=200)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--steps-per-launch", type=int, default=500)
    ap.add_argument("--block", type=int, default=-1,
                    help="threads per block (-1: the library's choice for the launch length)")
    ap.add_argument("--min-blocks", type=int, default=4, help="register cap variant (1, 3, 4)")
    ap.add_argument("--pass-actions", type=int, default=None,
                    help="free flights per drift pass of the warp-asynchronous kernel "
                         "(default: the library's)")
    ap.add_argument("--scatter-mode", type=int, default=2, choices=(0, 1, 2),
                    help="step kernel: 0 lockstep, 1 block-queued, 2 warp-asynchronous")
    ap.add_argument("--batch-steps", type=int, default=4000,
                    help="timed steps of the 64-ensemble sweep (0: skip it)")
    ap.add_argument("--batch-trial", type=int, default=50,
                    help="autotuner steps per shape and pass")
    ap.add_argument("--batch-fp64-steps", type=int, default=400)
    ap.add_argument("--device-steps", type=int, default=1000,
                    help="timed resistor device steps (0: skip the device path)")
    ap.add_argument("--device-warmup", type=int, default=20)
    ap.add_argument("--mosfet-steps", type=int, default=200,
                    help="timed steps of the 8-bias MOSFET batch (0: skip it)")
    ap.add_argument("--fp64-steps", type=int, default=1500)
    ap.add_argument("--small-steps", type=int, default=3000,
                    help="steps of the 10,000-electron FP64 case (0: skip it)")
    ap.add_argument("--precision-seeds", type=int, default=4,
                    help="extra FP32 seeds for the seed-to-seed sigma of the observables")
    ap.add_argument("--p2p-n", type=int, default=32768,
                    help="charges of the particle-particle Coulomb leg (0: skip it)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    return ap


def main(argv=None):
    args = build_parser().parse_args(argv)
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
