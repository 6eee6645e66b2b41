"""Benchmark: replica-exchange Monte Carlo throughput on one GB300.

Metric: MC steps/s and residue-pair evaluations/s.  A bench "step" is one exchange
block of the workload: every replica advances `--block` Monte Carlo steps (move, energy
of the moved molecule, Metropolis) on the GPU, then one even/odd temperature exchange
runs.  value = replica MC steps per second over the timed steps.

Default workload: the batched uneven configuration -- 96 independent simulations of
2-12 rigid molecules with log-uniform lengths 40-400 residues and 8-40 replicas each
(2,218 replicas, 101,651 residues), seeded synthetic inputs, all in one launch.  Its
resident state (~110 MB) is below the 129 MB L2, so every timed step is preceded by an
L2 flush (a 256 MiB write) inside the timed region.  The flexible-linker (c1), crowded
(c2) and identical-copies (c4) configurations run as extra legs of the same line.

Arms:
  default            the GB300 engine (libcgppd_gb300.so), CUDA-graph replays
  --impl reference   the reference CPU algorithm (full energy recomputation every
                     step, reference precision) timed on this host's cores: the
                     oracle's port of the reference loop, rank 0 only.  For the
                     batched configuration a bench step is one MC step of every
                     replica of a stratified share of the simulations, so that the
                     timed steps together sweep every simulation
Launched with torchrun for N > 1, each rank runs an independent set of replicas
("replicas only": the path has no cross-GPU exchange step), value = sum over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MC steps/s & pair-evals/s on 1 GB300: plain vs surrogate-screened, 1e-5 rel E"
FLOP_PER_PAIR = 80  # 40 FP32-pipe ops (FMA-counted as 2 FLOP) per Kim-Hummer pair term


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="c3")
    p.add_argument("--legs", default="c1,c2,c4", help="extra workloads timed in the same line ('' for none)")
    p.add_argument("--leg-blocks", type=int, default=10, help="timed blocks of each extra leg")
    p.add_argument("--block", type=int, default=1000, help="MC steps per exchange block")
    p.add_argument("--cluster", type=int, default=0)
    p.add_argument("--threads", type=int, default=0)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-surrogate", action="store_true")
    p.add_argument("--no-dropin", action="store_true", help="skip the drop-in energy-module leg")
    p.add_argument("--surrogate-workload", default="c4")
    p.add_argument("--surrogate-samples", type=int, default=2_000_000)
    p.add_argument("--surrogate-epochs", type=int, default=8)
    p.add_argument("--surrogate-blocks", type=int, default=10, help="timed blocks of each surrogate-leg arm")
    return p.parse_args()


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi samples during the timed region (read-only queries)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower() in ("active", "1"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ ranks

def reduce_over_ranks(seconds, counts, dist=None, device="cpu"):
    """Whole-job figures of a timed region: the slowest rank's time (max over ranks) and
    the sum of every rank's work; value = summed work / slowest time."""
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    c = torch.tensor([float(x) for x in counts], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(c)
    return float(t.item()), [float(x) for x in c.tolist()]


# ------------------------------------------------------------------ CPU arm

class CpuPort:
    """The oracle's port of the reference CPU loop (full energy recomputation every MC
    step, reference precision) over the simulations of a workload.  Every replica runs
    on its own host thread and the simulations of a sample run concurrently, so the OS
    spreads the work over all host cores."""

    def __init__(self, wl):
        from oracle.remc import OracleRemc
        self.wl = wl
        self.sims = [OracleRemc(s.molecules, wl.lj_raw, s.box, s.temperatures, s.translate_steps, s.rotate_steps,
                                s.move_weights, s.rigid_rotate_prob, wl.torsion_V, wl.torsion_phase, seed=wl.seed,
                                repulsive_crowding=s.repulsive_crowding)
                     for s in wl.sims]
        self.cores = os.cpu_count() or 1

    def sample(self, sim_ids, steps=1):
        """`steps` MC steps of every replica of the simulations `sim_ids`: (replica MC
        steps, seconds)."""
        from concurrent.futures import ThreadPoolExecutor
        sel = [self.sims[i] for i in sim_ids]
        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=max(1, len(sel))) as ex:
            list(ex.map(lambda o: o.run(1, steps, False, threads=o.R), sel))
        dt = time.perf_counter() - t0
        return sum(o.R for o in sel) * steps, dt

    def strata(self, k):
        """k shares of the simulations, each a mix of large and small ones (simulations
        ranked by pair work per step, dealt round-robin)."""
        work = [o.R * (o.N * o.N) for o in self.sims]
        order = sorted(range(len(self.sims)), key=lambda i: -work[i])
        return [order[j::k] for j in range(k) if order[j::k]]


def cpu_sweep(wl, min_seconds):
    """CPU baseline of the bench line: whole sweeps (one MC step of every replica of every
    simulation), repeated until `min_seconds` have passed."""
    port = CpuPort(wl)
    every = list(range(len(wl.sims)))
    port.sample([min(every, key=lambda i: port.sims[i].N)])  # warm-up
    done, secs, sweeps = 0, 0.0, 0
    while secs < min_seconds or sweeps == 0:
        n, dt = port.sample(every, 1 if len(every) > 1 else 16)
        done, secs, sweeps = done + n, secs + dt, sweeps + 1
    return {"value": done / secs, "unit": "replica MC steps/s", "cores": port.cores, "kind": "port",
            "sample": "%d sweep(s) of %d MC step(s) of all %d replicas of all %d simulation(s) of the same "
                      "workload (%.1f s; one host thread per replica)" % (sweeps, 1 if len(every) > 1 else 16,
                                                                          sum(o.R for o in port.sims), len(every),
                                                                          secs)}


def reference_arm(args):
    import cgppd_gb300.workloads as workloads
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wl = workloads.make(args.workload)
    port = CpuPort(wl)
    if len(wl.sims) > 1:
        # each bench step: one MC step of every replica of one stratum; the timed steps
        # together cover every simulation (strata repeat when steps > simulations)
        shares = port.strata(min(args.steps, len(wl.sims)))
        plan = [(shares[i % len(shares)], 1) for i in range(args.steps)]
        warm = [([min(range(len(wl.sims)), key=lambda i: port.sims[i].N)], 1)] * args.warmup
    else:
        # one simulation: each bench step a bounded block of MC steps of all replicas
        o = port.sims[0]
        _, dt = port.sample([0], 2)
        per = max(0.25, args.cpu_seconds / max(1, args.steps))
        n = max(4, int(per / max(dt / 2.0, 1e-4)))
        plan = [([0], n)] * args.steps
        warm = [([0], max(1, n // 4))] * args.warmup
    for ids, n in warm:
        port.sample(ids, n)
    rates = [port.sample(ids, n) for ids, n in plan]
    total_steps = sum(r[0] for r in rates)
    total_t = sum(r[1] for r in rates)
    value = total_steps / total_t
    covered = sorted(set(i for ids, _ in plan for i in ids))
    sample = ("%d bench steps, each one MC step of every replica of a stratified share of the %d simulations "
              "(%d of %d simulations covered, %d replica MC steps in %.1f s; full energy recomputation each "
              "step, as the reference CPU path)" % (args.steps, len(wl.sims), len(covered), len(wl.sims),
                                                    total_steps, total_t)) if len(wl.sims) > 1 else \
        ("%d replicas x %s MC steps per bench step (full energy recomputation each step, as the reference CPU "
         "path)" % (port.sims[0].R, plan[0][1]))
    out = {"metric": METRIC, "impl": "reference", "value": value, "unit": "replica MC steps/s", "n_gpus": 0,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total_t / len(rates),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64/fp32 (reference mix)",
           "data": "synthetic (seeded, configuration shapes)",
           "config": {"workload": wl.name, "replicas": wl.n_replicas, "simulations": len(wl.sims),
                      "mc_steps_per_bench_step": [n for _, n in plan]},
           "cpu_baseline": {"value": value, "unit": "replica MC steps/s", "cores": port.cores, "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "replica MC steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ------------------------------------------------------------------ surrogate leg

def surrogate_leg(args, torch, flush):
    """Plain vs surrogate-screened throughput on the identical-copies configuration: time
    the plain engine, train the surrogate on (pose, exact energy) samples drawn from that
    plain run, attach it, time the screened engine.  Both arms run the same workload from
    the same starting state with the same Philox stream; the screened arm's statistics
    are those of the exact distribution (delayed acceptance)."""
    from cgppd_gb300 import engine as eng
    from cgppd_gb300 import surrogate as sg
    from cgppd_gb300 import workloads
    wl = workloads.make(args.surrogate_workload)
    K = args.block
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream

    def timed(e, blocks):
        with torch.cuda.stream(stream):
            for _ in range(max(3, args.warmup)):
                flush.fill_(1.0)
                e.run(1, K, True, stream=sh)
        torch.cuda.synchronize()
        s0, p0 = e.counters()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
            for _ in range(blocks):
                flush.fill_(1.0)
                e.run(1, K, True, stream=sh)
            b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        s1, p1 = e.counters()
        return (s1 - s0) / (ms / 1000.0), (p1 - p0) / max(1, s1 - s0), ms

    plain = eng.from_workload(wl)
    plain_rate, plain_pairs, _ = timed(plain, args.surrogate_blocks)
    t0 = time.perf_counter()
    s, hist = sg.train_on_engine(plain, 0, n_samples=args.surrogate_samples, blocks=20, steps_per_block=K,
                                 epochs=args.surrogate_epochs, batch=8192, lr=1e-3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    plain.close()
    screened = eng.from_workload(wl)
    n_on = sg.attach(screened, s, rmse_threshold=0.5)
    st0 = sg.stats(screened, 0)
    da_rate, da_pairs, _ = timed(screened, args.surrogate_blocks)
    st = sg.stats(screened, 0)
    d = {k: st[k] - st0.get(k, 0.0) for k in ("proposals", "stage1_reject", "stage2_eval", "stage2_accept")}
    shape = screened.launch_shape()
    screened.close()
    # the same with the fallback disabled: what delayed acceptance itself does on this
    # system (the sampled distribution is exact either way)
    always = eng.from_workload(wl)
    sg.attach(always, s, rmse_threshold=1e30)
    a0 = sg.stats(always, 0)
    always_rate, always_pairs, _ = timed(always, args.surrogate_blocks)
    a1 = sg.stats(always, 0)
    da_always = {k: a1[k] - a0.get(k, 0.0) for k in ("proposals", "stage1_reject", "stage2_eval")}
    out = {"workload": wl.name, "plain_replica_mc_steps_per_s": plain_rate,
           "screened_replica_mc_steps_per_s": da_rate, "speedup": da_rate / plain_rate,
           "exact_pairs_per_step_plain": plain_pairs, "exact_pairs_per_step_screened": da_pairs,
           "stage1_reject_fraction": d["stage1_reject"] / max(1.0, d["proposals"]),
           "stage2_accept_fraction": d["stage2_accept"] / max(1.0, d["stage2_eval"]),
           "screened_proposals": d["proposals"], "online_rmse_kcal": st["rmse"], "still_screening": bool(st["screening"]),
           "simulations_screened": n_on, "train_samples": s.n_samples, "train_epochs": args.surrogate_epochs,
           "train_seconds_incl_sampling": train_s, "heldout_rmse_per_epoch": [float(x) for x in hist[:, 1]],
           "cluster_ctas_per_replica": shape[0], "threads_per_cta": shape[1],
           "no_fallback": {"replica_mc_steps_per_s": always_rate, "speedup": always_rate / plain_rate,
                           "exact_pairs_per_step": always_pairs,
                           "stage1_reject_fraction": da_always["stage1_reject"] / max(1.0, da_always["proposals"]),
                           "online_rmse_kcal": a1["rmse"]}}
    always.close()
    s.close()
    out["crowded_bound"] = crowded_screen_bound(args, torch, flush)
    return out


def crowded_screen_bound(args, torch, flush):
    """What any delayed-acceptance screen can gain on the crowded configuration: its first
    stage saves only the exact evaluations of proposals it rejects, and a correct first
    stage rejects at most what the exact test rejects, so the effective speed-up of a
    free, perfect screen is 1 / acceptance.  Measured on the plain engine (acceptance per
    temperature over 10 exchange blocks after 5 blocks of equilibration)."""
    from cgppd_gb300 import engine as eng
    from cgppd_gb300 import workloads
    wl = workloads.make("c2")
    e = eng.from_workload(wl)
    e.run(5, args.block, True)
    r0 = e.replicas(0)
    e.run(10, args.block, True)
    e.synchronize()
    r1 = e.replicas(0)
    # the counters travel with the temperature on exchange: totals per ladder index
    before = {int(t): (a, n) for t, a, n in zip(r0["tindex"], r0["totalAccept"], r0["totalAcceptReject"])}
    acc = [0.0] * len(r1["tindex"])
    for t, a, n in zip(r1["tindex"], r1["totalAccept"], r1["totalAcceptReject"]):
        a0, n0 = before[int(t)]
        acc[int(t)] = float(a - a0) / max(1, int(n - n0))
    e.close()
    return {"workload": wl.name, "acceptance_by_temperature": acc, "acceptance_mean": float(np.mean(acc)),
            "max_speedup_of_any_screen": 1.0 / float(np.mean(acc)),
            "note": "a first stage can skip only the exact evaluations of proposals it rejects; a correct one "
                    "rejects at most the ones the exact test rejects, so even a free, perfect screen gains at "
                    "most 1 / acceptance"}


# ------------------------------------------------------------------ drop-in energy module

def dropin_leg(args, torch, flush, wl, peak_tflops):
    """The reference's energy entry point (CUDA_EonDevice / _async, the drop-in C ABI) on
    one replica of the workload packed as the reference uploads it: pairs of residues in
    different molecules (rigid molecules; each molecule its own domain and chain id).
    Kernel time with events on the call's stream (async form), and the synchronous call
    (result copied to the host) timed on the host."""
    import ctypes
    import cgppd_gb300
    L = cgppd_gb300.lib()
    sim = wl.sims[0]
    mols = sim.molecules
    N = sum(m.n for m in mols)
    P = ((N + 31) // 32) * 32
    pos = np.zeros((P, 4), np.float32)
    meta = np.zeros((P, 4), np.float32)
    pos[:, 3] = -2.0   # padding
    meta[:, 0] = 20.0
    i0 = 0
    for k, m in enumerate(mols):
        sl = slice(i0, i0 + m.n)
        pos[sl, :3] = m.xyz
        pos[sl, 3] = k + 1
        meta[sl, 0] = np.minimum(m.types, 19)
        meta[sl, 1] = m.charges
        meta[sl, 2] = m.radii
        meta[sl, 3] = (k + 1) + (k + 1) / 1024.0
        i0 += m.n
    sizes = np.array([m.n for m in mols], np.float64)
    pairs = float((sizes.sum() ** 2 - (sizes ** 2).sum()) / 2)
    t20 = np.ascontiguousarray(np.asarray(wl.lj_raw, np.float32)[:20, :20])
    a = L.cgppd_aminoacids_create()
    L.cgppd_aminoacids_set_table(a, t20.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    dev = L.LJPotentialDataToDevice(a)
    L.bindLJTexture(dev)
    L.CUDA_setBoxDimension(ctypes.c_float(sim.box))
    dp = torch.from_numpy(pos.reshape(-1)).cuda()
    dm = torch.from_numpy(meta.reshape(-1)).cuda()
    rs = P // 32
    out = torch.zeros(rs * rs, dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    args_async = (ctypes.c_void_p(dp.data_ptr()), ctypes.c_void_p(dm.data_ptr()), None, None, None, None,
                  ctypes.c_void_p(out.data_ptr()), rs, 32, P, 0, ctypes.c_void_p(stream.cuda_stream))
    reps, burst = 20, 20
    with torch.cuda.stream(stream):
        for _ in range(3):
            L.CUDA_EonDevice_async(*args_async)
        times, singles = [], []
        for _ in range(reps):
            # a burst of calls enqueued back to back (as replicas issue them on a stream):
            # the host's launch work overlaps the previous call's kernel, so the events
            # time the kernels; the packed arrays (113 KB) stay in L2 as they do for a caller
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(burst):
                L.CUDA_EonDevice_async(*args_async)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / burst)
            # one call alone between the events (launch latency included)
            flush.fill_(1.0)
            e0.record(stream)
            L.CUDA_EonDevice_async(*args_async)
            e1.record(stream)
            e1.synchronize()
            singles.append(e0.elapsed_time(e1))
    cgppd_gb300.check("dropin leg")
    k_ms = float(np.median(times))
    res = ctypes.c_double(0.0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        L.CUDA_EonDevice(ctypes.c_void_p(dp.data_ptr()), ctypes.c_void_p(dm.data_ptr()), None, None, None, None,
                         ctypes.byref(res), 32, P, 0)
    sync_ms = (time.perf_counter() - t0) * 1000.0 / reps
    cgppd_gb300.check("dropin leg")
    L.unbindLJTexture()
    L.cgppd_aminoacids_destroy(a)
    tflops = pairs * FLOP_PER_PAIR / (k_ms / 1000.0) / 1e12
    return {"entry": "CUDA_EonDevice(_async)", "kernel": "k_tile_energy", "workload": wl.name + ", replica 0",
            "residues": N, "padded": P, "pairs_per_call": pairs, "kernel_ms": k_ms,
            "kernel_ms_note": "median over 20 bursts of 20 back-to-back async calls on one stream, per call "
                              "(each a dependent launch that waits for the previous call to end)",
            "single_call_ms": float(np.median(singles)), "sync_call_ms": sync_ms,
            "pair_evals_per_s": pairs / (k_ms / 1000.0), "achieved_tflops": tflops, "frac": tflops / peak_tflops,
            "energy_kcal": res.value}


# ------------------------------------------------------------------ GPU arm

def profile_counters(workload):
    """Per-launch ncu figures of k_mc on `workload` committed under profiles/ (DRAM
    traffic, FMA-pipe utilisation), or {}."""
    path = os.path.join(ROOT, "profiles", "k_mc_counters.json")
    try:
        return json.load(open(path)).get(workload, {})
    except (OSError, ValueError):
        return {}


def kernel_roofline(e, torch, stream, flush, K, peak_tflops, sfu_peak, workload):
    """The MC block kernel alone (one k_mc launch of K steps of every replica, no exchange)
    timed with CUDA events on its stream: pair-evals x 80 FLOP / duration."""
    sh = stream.cuda_stream
    ktimes = []
    with torch.cuda.stream(stream):
        for _ in range(3):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            p0 = e.counters()[1]
            a.record(stream)
            e.run(1, K, False, stream=sh)
            b.record(stream)
            b.synchronize()
            ktimes.append((a.elapsed_time(b), e.counters()[1] - p0))
    k_ms = float(np.mean([x[0] for x in ktimes]))
    k_pairs = float(np.mean([x[1] for x in ktimes]))
    achieved = k_pairs * FLOP_PER_PAIR / (k_ms / 1000.0) / 1e12
    sfu = k_pairs * 2 / (k_ms / 1000.0) / 1e9
    prof = profile_counters(workload)
    return {"bound": "fp32", "achieved": achieved, "peak": peak_tflops, "unit": "TFLOP/s",
            "frac": achieved / peak_tflops, "traffic": prof.get("traffic"),
            "fma_pipe_frac": prof.get("fma_pipe_frac"),
            "fma_pipe_note": "ncu sm__pipe_fma_cycles_active (fraction of peak sustained) of one k_mc launch, "
                             "from the committed profile of this workload",
            "kernel": "k_mc", "kernel_ms_per_launch": k_ms, "pairs_per_launch": k_pairs,
            "flop_per_pair": FLOP_PER_PAIR,
            "peak_note": "nominal FP32 pipe: SMs x 128 lanes x 2 x max SM clock (no FP32 figure in the measured "
                         "peaks); 80 FLOP per pair evaluation is the algorithmic count (40 FP32-pipe operations)",
            "sfu": {"ops_per_pair": 2, "achieved_gops": sfu, "peak_gops": sfu_peak, "frac": sfu / sfu_peak,
                    "note": "secondary ceiling: rsqrt and ex2 per pair against SMs x 16 MUFU lanes x max SM "
                            "clock"}}


def timed_blocks(e, torch, stream, flush, K, warmup, blocks):
    """Replica MC steps/s and pair-evals/s of `blocks` exchange blocks after `warmup`
    untimed ones, an L2 flush before each, CUDA events on the engine's stream."""
    sh = stream.cuda_stream
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            flush.fill_(1.0)
            e.run(1, K, True, stream=sh)
    torch.cuda.synchronize()
    s0, p0 = e.counters()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        a.record(stream)
        for _ in range(blocks):
            flush.fill_(1.0)
            e.run(1, K, True, stream=sh)
        b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    s1, p1 = e.counters()
    return (s1 - s0) / (ms / 1000.0), (p1 - p0) / (ms / 1000.0), ms


def leg(name, args, torch, flush, peak_tflops, sfu_peak):
    """One extra workload of the line: throughput over --leg-blocks blocks and its k_mc
    roofline."""
    from cgppd_gb300 import engine as eng
    from cgppd_gb300 import workloads
    wl = workloads.make(name)
    e = eng.from_workload(wl)
    stream = torch.cuda.Stream()
    rate, pair_rate, ms = timed_blocks(e, torch, stream, flush, args.block, max(3, args.warmup), args.leg_blocks)
    roof = kernel_roofline(e, torch, stream, flush, args.block, peak_tflops, sfu_peak, name)
    shape = e.launch_shape()
    e.close()
    return {"workload": wl.name, "replicas": wl.n_replicas, "replica_mc_steps_per_s": rate,
            "pair_evals_per_s": pair_rate, "blocks": args.leg_blocks, "mc_steps_per_block": args.block,
            "ms_per_block": ms / args.leg_blocks, "cluster_ctas_per_replica": shape[0], "threads_per_cta": shape[1],
            "state_in_shared_memory": shape[2], "roofline": roof}


def gpu_arm(args):
    import torch
    import cgppd_gb300
    from cgppd_gb300 import engine as eng
    from cgppd_gb300 import workloads

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    cgppd_gb300.lib()  # fails loudly if the library is missing

    wl = workloads.make(args.workload, seed=None if rank == 0 else 20261203 + 1000 * rank + int(args.workload[1:]))
    e = eng.from_workload(wl, cluster=args.cluster, threads=args.threads)
    R = e.total_replicas
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    K = args.block
    props = torch.cuda.get_device_properties(local)

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.fill_(1.0)
            e.run(1, K, True, stream=sh)
    barrier()
    steps0, pairs0 = e.counters()
    launches = 0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        with torch.cuda.stream(stream):
            ev0.record(stream)
            for _ in range(args.steps):
                flush.fill_(1.0)
                e.run(1, K, True, stream=sh)
                launches += e.last_launches()
            ev1.record(stream)
        barrier()
    steps1, pairs1 = e.counters()
    ms, (all_steps, all_pairs) = reduce_over_ranks(ev0.elapsed_time(ev1), [steps1 - steps0, pairs1 - pairs0],
                                                   dist, "cuda")
    value = all_steps / (ms / 1000.0)
    pair_rate = all_pairs / (ms / 1000.0)
    clocks = clk.summary()
    max_mhz = clocks["sm_max_mhz"] or 2070.0
    peak_tflops = props.multi_processor_count * 128 * 2 * max_mhz * 1e6 / 1e12
    sfu_peak = props.multi_processor_count * 16 * max_mhz * 1e6 / 1e9

    # the dominant kernel alone, timed with events on its stream
    roofline = kernel_roofline(e, torch, stream, flush, K, peak_tflops, sfu_peak, args.workload)

    # end to end through the public API with host buffers: upload every replica's state
    # from pinned memory (with a fresh energy evaluation), run the block, download state
    # and potentials, every step
    e2e = None
    if not args.no_e2e:
        sims = []
        for si in range(len(wl.sims)):
            N, M, Rs = e.sim_info(si)
            bufs = (torch.empty((Rs * N * 4,), dtype=torch.float32).pin_memory(),
                    torch.empty((Rs * N * 4,), dtype=torch.float32).pin_memory(),
                    torch.empty((Rs * M * 4,), dtype=torch.float32).pin_memory(),
                    torch.empty((Rs,), dtype=torch.float64).pin_memory())
            sims.append((si, N, M, Rs, bufs))
            e.download(si, bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(), bufs[3].data_ptr(), stream=sh)
        stream.synchronize()
        n_e2e = max(2, args.steps // 2)
        barrier()
        t0 = time.perf_counter()
        s0 = e.counters()[0]
        for _ in range(n_e2e):
            # the last upload re-evaluates every replica of every simulation (one launch)
            for si, N, M, Rs, b in sims:
                e.upload(si, b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr(), recompute=(si == len(sims) - 1),
                         stream=sh)
            e.run(1, K, True, stream=sh)
            for si, N, M, Rs, b in sims:
                e.download(si, b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr(), b[3].data_ptr(), stream=sh)
            stream.synchronize()
        t1 = time.perf_counter()
        h2d = sum((2 * Rs * N + Rs * M) * 16 for _, N, M, Rs, _ in sims)
        d2h = h2d + sum(Rs * 8 for _, _, _, Rs, _ in sims)
        secs, (done,) = reduce_over_ranks(t1 - t0, [e.counters()[0] - s0], dist, "cuda")
        e2e = {"value": done / secs, "unit": "replica MC steps/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    shape = e.launch_shape()
    tuning = [list(x) for x in e.tuning()]
    e.close()

    solo = rank == 0 and world == 1
    cpu = cpu_sweep(wl, args.cpu_seconds) if solo and not args.no_cpu_baseline else None
    legs = {}
    if solo:
        for name in [x for x in args.legs.split(",") if x and x != args.workload]:
            legs[name] = leg(name, args, torch, flush, peak_tflops, sfu_peak)
    sur = surrogate_leg(args, torch, flush) if solo and not args.no_surrogate else None
    dropin = dropin_leg(args, torch, flush, workloads.make("c2"), peak_tflops) \
        if solo and not args.no_dropin else None
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "replica MC steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded, configuration shapes)",
            "config": {"workload": wl.name, "simulations": len(wl.sims), "replicas": R,
                       "residues": sum(s.n_residues for s in wl.sims), "mc_steps_per_bench_step": K,
                       "exchange": "after every block", "l2": "256 MiB flush before every timed step, inside the "
                                                             "timed region", "cluster_ctas_per_replica": shape[0],
                       "threads_per_cta": shape[1], "state_in_shared_memory": shape[2],
                       "parallelism": "replicas on one GPU" if world == 1 else
                       "dp%d (independent replica sets)" % world},
            "pair_evals_per_s": pair_rate,
            "autotune_us_per_mc_step": tuning,
            "roofline": roofline,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
            "legs": legs, "surrogate": sur, "dropin": dropin,
        }
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        reference_arm(a)
    else:
        gpu_arm(a)
