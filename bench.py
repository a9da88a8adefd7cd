#!/usr/bin/env python
"""Key Gbit/s of the privacy-amplification hot path on GB300.

Workload (the reference's default size): n = 2^27 key/seed bits, h = 83,886,080, v = 50,331,648,
static seed with cached FP32 spectrum, do_xor_key_rest + do_compress, i.i.d. Bernoulli(0.5) bits
from a fixed PCG64 seed.  One step = one block.  Metric: key Gbit/s = n / time per block, the
reference's definition (PrivacyAmplification.cu:1213, 2081).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

* value  -- device-timed (CUDA events around the batch on the caller's stream) K blocks with inputs
            resident in HBM, two in flight (pa_batch_run over two slots, the seed spectrum cached once),
            working set 1.5 GiB per block, so every step streams from HBM.  value_one_stream: the same
            blocks one after another (pa_process_device), which also gives the per-block latency and
            the per-kernel times of the roofline.
* e2e    -- the same K blocks from pinned host buffers through the C ABI: per block the H2D copy of
            key_start and key_rest, the kernels, and the D2H copy of the v/8 output bytes.  value:
            pa_submit / pa_poll with four blocks in flight (copies overlap the other blocks' kernels);
            sync_value: pa_process, one block at a time.
* roofline -- the dominant kernel's algorithmic bytes per launch / its mean CUDA-event duration in
            the timed region, against MEASURED_PEAKS.json's hbm_gbs.
* cpu_baseline -- the exact NTT convolution of the oracle on all host cores, one whole block.
* reference_cuda -- the reference's own kernels (compiled from PrivacyAmplification.cu for sm_103a by
            baseline/ref_cuda.py) in its mainloop order on cuFFT, with its launch shapes, pinned
            zero-copy slots and host syncs, on the same GPU and inputs, static and dynamic seed, host
            wall time per block as the reference's speedtest measures it; plus whether its output
            bytes equal the engine's.  cufft_plain: the same sequence with restated kernels.
* other_configs -- short forms of configs 4 (the 512-block uneven mix as one CUDA graph) and 5 (2000
            requests at 2000/s, host-driven serving); --workload batch / serve run them in full.
* --impl reference -- the reference has no CPU implementation of the path, so this arm times the CPU
            port (the oracle's exact NTT convolution, all host threads) on the same workload, one whole
            block per step.

For N > 1 (torchrun) every rank runs an independent replica on its own GPU (blocks are independent;
no collective on the data path); value = all blocks of all ranks / max over ranks of the time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_BITS = 1 << 27
V_BITS = 50331648
H_BITS = N_BITS - V_BITS
METRIC = "key Gbit/s"
UNIT = "Gbit/s"
DATA = "synthetic: i.i.d. Bernoulli(0.5) seed and key bits, PCG64 seed 0x5EED"
WORKLOAD = ("n=2^27 (h=83886080, v=50331648), static seed with cached FP32 spectrum, do_xor_key_rest, "
            "do_compress; one block per step")
KEY_BUFFERS = 4  # distinct keys cycled through the timed blocks
IN_FLIGHT = 2    # device-resident blocks in flight for the headline value (slots of the engine's pool)
E2E_IN_FLIGHT = 4  # host-resident blocks in flight for e2e


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profiles(kernel):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel:
                return float(parts[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def make_inputs(nkeys):
    import privacyamplification_gb300 as pa
    from privacyamplification_gb300.workloads import random_block
    seed, _ = random_block(N_BITS, V_BITS, 0x5EED)
    keys = []
    for i in range(nkeys):
        _, recv = random_block(N_BITS, V_BITS, 0x5EED + 1 + i)
        keys.append(pa.key_split(recv, N_BITS, V_BITS))
    return seed, keys


class CpuBlocks:
    """The oracle's exact NTT port on the bench workload with the seed transform kept (the static-seed
    case: the reference caches its seed spectrum the same way), so that one call is one whole key block
    -- forward transform of the key, product, inverse transform, parity, key_rest XOR, packing -- on
    `threads` host threads."""

    def __init__(self, threads=0):
        from oracle import oracle as O
        self.O = O
        self.cores = threads or os.cpu_count() or 1
        seed, _ = O.random_block(N_BITS, V_BITS, 0x5EED)
        t = time.perf_counter()
        self.ref = O.NttSeed(seed, N_BITS, V_BITS, threads=self.cores)
        self.seed_s = time.perf_counter() - t
        self.keys = []
        for i in range(KEY_BUFFERS):
            _, recv = O.random_block(N_BITS, V_BITS, 0x5EED + 1 + i)
            self.keys.append(O.key_split(recv, N_BITS, V_BITS))

    def block(self, i):
        """One whole block; returns (seconds, output bytes)."""
        ks, kr = self.keys[i % len(self.keys)]
        t = time.perf_counter()
        out = self.ref.block(ks, kr, threads=self.cores)
        return time.perf_counter() - t, out

    def close(self):
        self.ref.close()


def cpu_baseline(threads=0, blocks=2):
    """The CPU port timed on whole n=2^27 blocks (the median of `blocks`), seed transform excluded."""
    cb = CpuBlocks(threads)
    try:
        times = [cb.block(i)[0] for i in range(blocks)]
    finally:
        cb.close()
    dt = statistics.median(times)
    sample = ("%d whole n=2^27 blocks (exact NTT convolution mod 2^64-2^32+1, seed transform kept as in the "
              "static-seed path; %.1f s once), median %.2f s per block on %d threads"
              % (blocks, cb.seed_s, dt, cb.cores))
    return N_BITS / dt / 1e9, cb.cores, sample


def workload_config(world):
    """The `config` of both arms' lines (identical, so that the two lines describe the same workload)."""
    return {"workload": WORKLOAD, "n": N_BITS, "h": H_BITS, "v": V_BITS, "blocks_per_step": 1,
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2: 512 MiB work array + 512 MiB seed spectrum per block"}


def cufft_plain_leg(seed, keys, eng, steps, ref_fatbin=None):
    """Times the cuFFT pipeline baseline (4 warm-up blocks, then `steps` blocks per seed mode) and
    checks its output bytes against the engine's on the same key.  With ref_fatbin the pipeline launches
    the reference's own kernels (compiled from PrivacyAmplification.cu) instead of its restated ones."""
    import numpy as np
    from baseline import cufft_plain
    cufft_plain.build()
    cp = cufft_plain.CufftPlain(N_BITS, V_BITS)
    if ref_fatbin:
        cp.use_reference_kernels(ref_fatbin)
    try:
        cp.load(seed=seed)
        res = {}
        for mode, recalc in (("static", False), ("dynamic", True)):
            times = []
            for i in range(4 + steps):
                ks, kr = keys[i % len(keys)]
                cp.load(key_start=ks, key_rest=kr)  # outside the timed call, like a filled ring slot
                ms = cp.process(recalc_seed=recalc or i == 0)
                if i >= 4:
                    times.append(ms)
            times.sort()
            p50 = times[len(times) // 2]
            p99 = times[min(len(times) - 1, int(round(0.99 * (len(times) - 1))))]
            res[mode] = {"value": N_BITS / (p50 / 1e3) / 1e9, "unit": UNIT, "p50_ms": p50, "p99_ms": p99,
                         "blocks": len(times), "last_block_steps_ms": cp.step_ms()}
        ks, kr = keys[0]
        cp.load(key_start=ks, key_rest=kr)
        cp.process(recalc_seed=False)
        nbytes = V_BITS // 8
        theirs = cp.output(nbytes)
        resid = cp.residual(V_BITS)
        mine = eng.process(ks, kr, N_BITS, V_BITS)
        res["output_equal"] = bool(np.array_equal(theirs, mine))
        res["output_sha3"] = O_sha3(theirs)
        res["max_residual"] = resid
        if ref_fatbin:
            res["what"] = ("the reference's own kernels (PrivacyAmplification.cu compiled for sm_103a by "
                           "baseline/ref_cuda.py) in its mainloop order on cuFFT: zero-copy pinned slots, per-step "
                           "host syncs; wall ms per block, value at p50")
        else:
            res["what"] = ("reference mainloop sequence restated on cuFFT (baseline/cufft_plain.cu): zero-copy "
                           "pinned slots, per-step host syncs; wall ms per block, value at p50")
        return res
    finally:
        if ref_fatbin:
            cp.use_restated_kernels()
        cp.close()


def O_sha3(data):
    import hashlib
    return hashlib.sha3_256(bytes(data)).hexdigest().upper()


def pct(xs, q):
    """Nearest-rank percentile."""
    import math
    ys = sorted(xs)
    return ys[min(len(ys) - 1, max(0, math.ceil(q / 100.0 * len(ys)) - 1))]


def max_over_ranks(values, dist, device):
    """Element-wise maximum of per-rank times (the slowest replica sets the job's time)."""
    if dist is None:
        return [float(x) for x in values]
    import torch
    t = torch.tensor([float(x) for x in values], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_value(world, steps, bits, seconds):
    """Whole-job key Gbit/s: every rank processed `steps` blocks of `bits` in at most `seconds`."""
    return world * steps * bits / seconds / 1e9


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    """The reference arm, on the host cores: the reference ships no CPU implementation of the path, so this
    times the CPU port (oracle, exact NTT, all host threads) on the same workload, one whole block per
    step.  The reference's own CUDA kernels on the GPU are timed by the engine arm (`reference_cuda`).
    Under torchrun only rank 0 runs it."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    cb = CpuBlocks()
    try:
        for i in range(args.warmup):
            cb.block(i)
        times = [cb.block(args.warmup + i)[0] for i in range(args.steps)]
    finally:
        cb.close()
    total = sum(times)
    value = args.steps * N_BITS / total / 1e9
    sample = ("%d whole n=2^27 blocks after %d warm-up blocks, exact NTT convolution mod 2^64-2^32+1 on %d "
              "threads (seed transform computed once, %.1f s, as the static-seed path caches it); per block "
              "median %.2f s, min %.2f s, max %.2f s" % (args.steps, args.warmup, cb.cores, cb.seed_s,
                                                          statistics.median(times), min(times), max(times)))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64 (mod p)", "data": DATA,
        "config": workload_config(world),
        "implementation": "CPU port of the path (oracle/pa_oracle.c: exact NTT convolution, OpenMP); the "
                          "reference itself has no CPU path",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cb.cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def spread(xs):
    """Median and spread of repeated measurements."""
    ys = sorted(xs)
    return {"median": statistics.median(ys), "min": ys[0], "max": ys[-1], "p10": pct(ys, 10), "p90": pct(ys, 90),
            "repeats": len(ys)}


def rate_spread(seconds, to_rate):
    """Spread of repeated timed regions as rates (min/max of the rate, not of the time)."""
    out = spread([to_rate(t) for t in seconds])
    out["median"] = to_rate(statistics.median(seconds))
    return out


def run_ours(args):
    import numpy as np
    import torch
    import privacyamplification_gb300 as pa
    from privacyamplification_gb300 import build as pa_build

    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    torch.cuda.set_device(local)
    pa_build.build()
    dev = torch.device("cuda", local)
    R, K = args.repeats, args.steps

    def fence():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    seed, keys = make_inputs(KEY_BUFFERS)
    eng = pa.Engine(max_sample_size=N_BITS, device_id=local)
    eng.set_seed(seed, N_BITS, -1)

    # ---------------------------------------------------------------- device-resident, one stream
    # The same K blocks one after another through pa_process_device, the timed region repeated R times:
    # per-block device latency (an event after every block) and the per-kernel times of the roofline.
    d_keys = [(torch.from_numpy(ks.view(np.int32)).to(dev), torch.from_numpy(kr.view(np.int32)).to(dev))
              for ks, kr in keys]
    nbytes_out = pa.output_bytes(N_BITS, V_BITS)
    d_out = torch.empty((nbytes_out + 3) // 4, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream

    def block(i):
        ks, kr = d_keys[i % len(d_keys)]
        eng.process_device(ks.data_ptr(), kr.data_ptr(), N_BITS, V_BITS, d_out.data_ptr(), stream=sh)

    for i in range(args.warmup):
        block(i)
    eng.sync()
    fence()
    eng.set_timing(True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev_blk = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    t_one, blk_ms, stage_sum, stage_n = [], [], None, 0
    with ClockSampler(local) as clk_one:
        for rep in range(R):
            fence()
            with torch.cuda.stream(stream):
                ev0.record(stream)
                for i in range(K):
                    block(i)
                    ev_blk[i].record(stream)
                ev1.record(stream)
            ev1.synchronize()
            t_one.append(max_over_ranks([ev0.elapsed_time(ev1) / 1e3], dist, dev)[0])
            blk_ms += [ev0.elapsed_time(ev_blk[0])] + [ev_blk[i - 1].elapsed_time(ev_blk[i]) for i in range(1, K)]
            sm, nb = eng.stage_times()
            stage_sum = [a + b * nb for a, b in zip(stage_sum, sm)] if stage_sum else [b * nb for b in sm]
            stage_n += nb
    stats = eng.sync()
    eng.set_timing(False)
    stage_ms = [x / stage_n for x in stage_sum] if stage_n else []

    # ---------------------------------------------------------------- device-resident, blocks in flight
    # The headline value: the same K blocks, IN_FLIGHT at a time (pa_batch_run over that many slots, the
    # seed spectrum cached once), so that one block's kernel tails and short kernels overlap the next
    # block's work; the timed region repeated R times, value = the median repeat.
    sid = eng.seed_cache_add(seed, N_BITS, V_BITS)
    n_out = 16
    d_outs = [torch.empty((nbytes_out + 3) // 4, dtype=torch.int32, device=dev) for _ in range(n_out)]

    def jobs_for(count):
        return [pa.PAJob(None, sid, d_keys[i % len(d_keys)][0].data_ptr(), d_keys[i % len(d_keys)][1].data_ptr(),
                         N_BITS, V_BITS, pa.DEFAULT_FLAGS, d_outs[i % n_out].data_ptr()) for i in range(count)]

    eng.set_pool(0, 16, IN_FLIGHT)
    eng.batch_run(jobs_for(args.warmup), 0, sh)
    eng.batch_sync(args.warmup)
    timed_jobs = jobs_for(K)
    t_conc = []
    with ClockSampler(local) as clk:
        for rep in range(R):
            fence()
            eng.batch_run(timed_jobs, 0, sh)
            bst = eng.batch_sync(K)
            t_conc.append(max_over_ranks([bst[0].gpu_ms / 1e3], dist, dev)[0])
    torch.cuda.synchronize()
    conc_equal = bool(torch.equal(d_outs[(K - 1) % n_out], d_out))
    if dist:
        dist.barrier()

    # ---------------------------------------------------------------- e2e through the C ABI
    pin_keys = []
    for ks, kr in keys:
        pk = torch.from_numpy(ks.view(np.int32)).pin_memory().numpy().view(np.uint32)
        pr = torch.from_numpy(kr.view(np.int32)).pin_memory().numpy().view(np.uint32)
        pin_keys.append((pk, pr))
    pin_out = torch.empty(nbytes_out, dtype=torch.uint8).pin_memory().numpy()
    for i in range(args.warmup):
        ks, kr = pin_keys[i % len(pin_keys)]
        eng.process(ks, kr, N_BITS, V_BITS, out=pin_out)
    t_e2e_sync, sync_ms = [], []
    for rep in range(R):
        fence()
        t0 = time.perf_counter()
        for i in range(K):
            ks, kr = pin_keys[i % len(pin_keys)]
            t1 = time.perf_counter()
            eng.process(ks, kr, N_BITS, V_BITS, out=pin_out)
            sync_ms.append((time.perf_counter() - t1) * 1e3)
        t_e2e_sync.append(max_over_ranks([time.perf_counter() - t0], dist, dev)[0])

    # pipelined form of the same calls: pa_submit / pa_poll with E2E_IN_FLIGHT blocks in flight, so one
    # block's host copies overlap the others' kernels (same pinned host buffers, same bytes per block)
    depth = E2E_IN_FLIGHT
    pin_outs = [torch.empty(nbytes_out, dtype=torch.uint8).pin_memory().numpy() for _ in range(depth)]

    def pipelined(count):
        inflight = []
        for i in range(count):
            ks, kr = pin_keys[i % len(pin_keys)]
            job = pa.PAJob(None, sid, ks.ctypes.data, kr.ctypes.data, N_BITS, V_BITS, pa.DEFAULT_FLAGS,
                           pin_outs[i % depth].ctypes.data)
            while len(inflight) >= depth:
                while eng.poll(inflight[0]) is None:
                    pass
                inflight.pop(0)
            t = eng.submit(job)
            while t is None:  # a slot frees up when the oldest block is collected
                while eng.poll(inflight[0]) is None:
                    pass
                inflight.pop(0)
                t = eng.submit(job)
            inflight.append(t)
        for t in inflight:
            while eng.poll(t) is None:
                pass

    pipelined(args.warmup)
    t_e2e = []
    with ClockSampler(local) as clk_e2e:
        for rep in range(R):
            fence()
            t0 = time.perf_counter()
            pipelined(K)
            t_e2e.append(max_over_ranks([time.perf_counter() - t0], dist, dev)[0])
    same_out = bool((pin_outs[(K - 1) % depth] == eng.process(*keys[(K - 1) % len(keys)], N_BITS, V_BITS)).all())
    h2d = (H_BITS // 32 + 1) * 4 + (V_BITS // 32) * 4
    d2h = nbytes_out

    if rank != 0:
        eng.close()
        if dist:
            dist.destroy_process_group()
        return 0

    # ---------------------------------------------------------------- roofline of the dominant kernel
    names = ["pass_a", "pass_b", "pass_c", "finish"]
    n = N_BITS
    # algorithmic bytes per launch: the minimum HBM traffic of each pass
    algo = {
        "pass_a": 4 * n + (H_BITS + 1) // 8,        # key bits in, Y (n/2 complex64) out
        "pass_b": 12 * n,                           # Y in, seed spectrum in, Y out
        "pass_c": 4 * n + n // 8,                   # Y in, two parity planes out
        "finish": n // 8 + V_BITS // 8 * 2,         # planes in, key_rest in, output out
    }
    kern = {names[i]: stage_ms[i] for i in range(min(len(stage_ms), len(names)))}
    top = max(kern, key=kern.get) if kern else None
    peak, peak_kind = peaks()
    roof = None
    if top:
        achieved = algo[top] / (kern[top] / 1e3) / 1e9
        tr = traffic_from_profiles(top)
        roof = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": tr, "algorithmic_bytes": algo[top],
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                else "fallback 6.8 TB/s",
                "kernel_fracs": {k: algo[k] / (kern[k] / 1e3) / 1e9 / peak for k in kern}}
    block_bytes = 20 * n + ((H_BITS + 1) + 2 * V_BITS) // 8
    total_s = sum(stage_ms) / 1e3 if stage_ms else None

    plain = None if args.no_cufft else cufft_plain_leg(seed, keys, eng, min(K, 20))
    ref_cuda = None
    if not args.no_cufft:
        from baseline import ref_cuda as RC
        fb = RC.fatbin()
        ref_cuda = (cufft_plain_leg(seed, keys, eng, min(K, 20), ref_fatbin=fb) if fb else
                    {"unavailable": "the reference's kernels were not compiled: its source tree was absent at build "
                                    "time"})

    if args.no_cpu:
        cpu = None
    else:
        cb, cores, sample = cpu_baseline()
        cpu = {"value": cb, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}

    s_conc, s_one, s_e2e, s_sync = spread(t_conc), spread(t_one), spread(t_e2e), spread(t_e2e_sync)
    gbit = lambda secs: job_value(world, K, N_BITS, secs)
    value = gbit(s_conc["median"])
    block_gbs = block_bytes / (s_conc["median"] / K) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": s_conc["median"] / K * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": DATA,
        "config": workload_config(world),
        "blocks_in_flight": IN_FLIGHT,
        "repeats": {"count": R, "what": "the K-step timed region is run R times (each bracketed by a sync); "
                                        "value = median repeat",
                    "gbit_s": rate_spread(t_conc, gbit)},
        "e2e": {"value": gbit(s_e2e["median"]), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "api": "pa_submit/pa_poll, %d blocks in flight, pinned host buffers" % E2E_IN_FLIGHT,
                "repeats_gbit_s": rate_spread(t_e2e, gbit),
                "output_equals_pa_process": same_out, "clocks": clk_e2e.summary(),
                "sync_value": gbit(s_sync["median"]), "sync_api": "pa_process, one block at a time"},
        "gpu_launches": K * pa.kernels_per_block(N_BITS, V_BITS),
        "value_one_stream": {"value": gbit(s_one["median"]), "unit": UNIT,
                             "repeats_gbit_s": rate_spread(t_one, gbit),
                             "api": "pa_process_device, one block after another on one stream",
                             "output_equals_in_flight": conc_equal, "clocks": clk_one.summary()},
        "latency_ms": {"device_p50": pct(blk_ms, 50), "device_p99": pct(blk_ms, 99), "device_max": max(blk_ms),
                       "blocks": len(blk_ms),
                       "pa_process_p50": pct(sync_ms, 50), "pa_process_p99": pct(sync_ms, 99),
                       "what": "device: CUDA events between consecutive blocks on the engine stream; "
                               "pa_process: host wall time of one synchronous call (copies in, block, copy out)"},
        "kernels_ms": kern, "kernel_blocks_timed": stage_n,
        "block_hbm_model": {"bytes": block_bytes, "GB_per_s_in_flight": block_gbs,
                            "frac_in_flight": block_gbs / peak,
                            "GB_per_s_at_kernel_sum": block_bytes / total_s / 1e9 if total_s else None},
        "roofline": roof,
        "cpu_baseline": cpu,
        "cufft_plain": plain,
        "reference_cuda": ref_cuda,
        "clocks": clk.summary(),
        "max_residual": stats.max_residual,
    }
    eng.close()
    if world == 1 and not args.no_configs:
        line["other_configs"] = other_configs_leg(args)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def other_configs_leg(args):
    """Short forms of configs 4 and 5 in the default run (their full forms are --workload batch / serve):
    the 512-block uneven mix as one CUDA graph (device-timed, median of `steps` batches), and 2000
    requests arriving at 2000/s with their own seeds (host-driven serving, p50 / p99)."""
    import privacyamplification_gb300 as pa
    from privacyamplification_gb300 import workloads as W
    out = {}
    with pa.Engine(max_sample_size=1 << 25) as eng:
        eng.autotune(1 << 18, 1 << 26)
        blocks = W.uneven_mix()
        mix = W.DeviceMix(eng, blocks)
        bits = sum(b.n for b in blocks)
        for _ in range(args.warmup):
            mix.run(pa.BATCH_GRAPH)
        with ClockSampler(0) as clk:
            ms = [mix.run(pa.BATCH_GRAPH)[0].gpu_ms for _ in range(max(3, min(args.steps, 10)))]
        out["config4_batch"] = {
            "workload": "512 blocks, n log-uniform [2^18, 2^25] (multiple of 1024), v/n ~ U[0.1,0.9], half with "
                        "a cached static seed, half with their own; one CUDA graph per batch",
            "gbit_s": bits / (statistics.median(ms) / 1e3) / 1e9, "ms_median": statistics.median(ms),
            "ms_min": min(ms), "ms_max": max(ms), "batches": len(ms), "clocks": clk.summary()}
    with pa.Engine(max_sample_size=1 << 27) as eng:
        eng.pool_reserve(1 << 27, 16)
        reqs = W.poisson_requests(2000, 2000, rng_seed=2000)
        words = max(r.n // 32 + max(r.seed_word0, r.key_word0) for r in reqs) + 64
        banks = W.HostBanks(words)
        warm = W.poisson_requests(5000, 24, rng_seed=1)
        for r in warm:
            r.seed_word0 = r.key_word0 = 0
        W.serve(eng, warm, banks)
        with ClockSampler(0) as clk:
            res = W.serve(eng, reqs, banks)
        out["config5_serve_2000_per_s"] = {
            "workload": "2000 requests, Poisson arrivals at 2000/s, n log-uniform [2^20, 2^27] (multiple of 1024), "
                        "v/n ~ U[0.2,0.8], each with its own seed; host-driven pa_submit / pa_poll, 16 slots",
            "p50_ms": res.pct(50), "p99_ms": res.pct(99), "sustained_gbit_s": res.bits / res.wall_s / 1e9,
            "offered_gbit_s": sum(r.n for r in reqs) / reqs[-1].arrival / 1e9, "exact_recomputed": res.exact,
            "clocks": clk.summary()}
    return out


# ------------------------------------------------------------------------------------ other workloads
def _line(metric, value, unit, steps, warmup, ms_per_step, workload, extra, higher=True):
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": steps, "warmup": warmup,
            "ms_per_step": ms_per_step, "higher_is_better": higher, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": DATA, "config": {"workload": workload}}
    line.update(extra)
    print(json.dumps(line))


def run_dynamic27(args):
    """Precision-stress size with a fresh seed per block: seed spectrum + key block, n = 2^27."""
    import numpy as np
    import torch
    import privacyamplification_gb300 as pa
    from privacyamplification_gb300.workloads import random_block
    pa.load_library()
    dev = torch.device("cuda", 0)
    eng = pa.Engine(max_sample_size=N_BITS)
    seeds, keys = [], []
    for i in range(KEY_BUFFERS):
        sd, recv = random_block(N_BITS, V_BITS, 0xD1 + i)
        ks, kr = pa.key_split(recv, N_BITS, V_BITS)
        seeds.append(torch.from_numpy(sd.view(np.int32)).to(dev))
        keys.append((torch.from_numpy(ks.view(np.int32)).to(dev), torch.from_numpy(kr.view(np.int32)).to(dev)))
    d_out = torch.empty(V_BITS // 32, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def block(i):
        eng.set_seed_device(seeds[i % len(seeds)].data_ptr(), N_BITS, 1, stream=stream.cuda_stream)
        ks, kr = keys[i % len(keys)]
        eng.process_device(ks.data_ptr(), kr.data_ptr(), N_BITS, V_BITS, d_out.data_ptr(), stream=stream.cuda_stream)

    for i in range(args.warmup):
        block(i)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        ev0.record(stream)
        for i in range(args.steps):
            block(i)
        ev1.record(stream)
        ev1.synchronize()
    st = eng.sync(check=False)
    t = ev0.elapsed_time(ev1) / 1e3
    # the same blocks, IN_FLIGHT at a time (each job brings its own seed; pa_batch_run over slots)
    outs = [torch.empty(V_BITS // 32, dtype=torch.int32, device=dev) for _ in range(8)]
    jobs = [pa.PAJob(seeds[i % len(seeds)].data_ptr(), -1, keys[i % len(keys)][0].data_ptr(),
                     keys[i % len(keys)][1].data_ptr(), N_BITS, V_BITS, pa.DEFAULT_FLAGS, outs[i % 8].data_ptr())
               for i in range(args.steps)]
    eng.set_pool(0, 16, IN_FLIGHT)
    eng.batch_run(jobs[: args.warmup], 0, stream.cuda_stream)
    eng.batch_sync(args.warmup)
    with ClockSampler(0) as clk2:
        eng.batch_run(jobs, 0, stream.cuda_stream)
        bst = eng.batch_sync(args.steps)
    t2 = bst[0].gpu_ms / 1e3
    _line(METRIC, args.steps * N_BITS / t2 / 1e9, UNIT, args.steps, args.warmup, t2 / args.steps * 1e3,
          "n=2^27 (h=83886080, v=50331648), dynamic seed: a fresh seed spectrum every block, do_xor, do_compress; "
          "%d blocks in flight" % IN_FLIGHT,
          {"max_residual": max(st.max_residual, max(x.max_residual for x in bst)), "clocks": clk2.summary(),
           "value_one_stream": args.steps * N_BITS / t / 1e9, "clocks_one_stream": clk.summary(),
           "gpu_launches": args.steps * (3 + pa.kernels_per_block(N_BITS, V_BITS))})
    eng.close()


def run_big29(args, force_exact):
    """n = 2^29 (beyond one FP32 pass), fresh seed per block: 2^27-bit FP32 chunk blocks under the
    residual guard, or (force_exact) the exact NTT path."""
    import numpy as np
    import torch
    import privacyamplification_gb300 as pa
    n = 1 << 29
    v = n // 4 + n // 8
    pa.load_library()
    dev = torch.device("cuda", 0)
    eng = pa.Engine(max_sample_size=n)
    rng = np.random.default_rng(29)
    words = lambda k: rng.integers(0, 1 << 32, size=k, dtype=np.uint64).astype(np.uint32)
    seeds = [torch.from_numpy(words(n // 32).view(np.int32)).to(dev) for _ in range(2)]
    ks = torch.from_numpy(words(n // 32).view(np.int32)).to(dev)
    kr = torch.from_numpy(words(v // 32).view(np.int32)).to(dev)
    d_out = torch.empty(v // 32, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def block(i):
        eng.set_seed_device(seeds[i % 2].data_ptr(), n, 1, stream=stream.cuda_stream)
        eng.process_device(ks.data_ptr(), kr.data_ptr(), n, v, d_out.data_ptr(),
                           flags=pa.DEFAULT_FLAGS | (pa.FLAG_EXACT if force_exact else 0), stream=stream.cuda_stream)

    for i in range(args.warmup):
        block(i)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        ev0.record(stream)
        for i in range(args.steps):
            block(i)
        ev1.record(stream)
        ev1.synchronize()
    st = eng.sync(check=False)
    t = ev0.elapsed_time(ev1) / 1e3
    path = "exact NTT path mod 3*2^30+1" if force_exact else "FP32 path in 2^27-bit chunk blocks, residual guard"
    _line(METRIC, args.steps * n / t / 1e9, UNIT, args.steps, args.warmup, t / args.steps * 1e3,
          "n=2^29 (h=n/2+n/8, v=n/4+n/8), dynamic seed, " + path,
          {"exact": st.exact, "max_residual": st.max_residual, "clocks": clk.summary(),
           "dtype": "u32 (mod p)" if force_exact else "f32"})
    eng.close()


def run_batch(args):
    """Uneven mix: 512 blocks, n log-uniform in [2^18, 2^25], v/n ~ U[0.1, 0.9], half static seeds."""
    import torch
    import privacyamplification_gb300 as pa
    from privacyamplification_gb300 import workloads as W
    pa.load_library()
    eng = pa.Engine(max_sample_size=1 << 25)
    t = time.perf_counter()
    tuned = eng.autotune(1 << 18, 1 << 26)
    tune_s = time.perf_counter() - t
    blocks = W.uneven_mix()
    mix = W.DeviceMix(eng, blocks)
    bits = sum(b.n for b in blocks)
    res = {}
    modes = (("serial", pa.BATCH_SERIAL), ("concurrent", 0), ("graph", pa.BATCH_GRAPH),
             ("persistent", pa.BATCH_PERSISTENT), ("persistent_graph", pa.BATCH_PERSISTENT | pa.BATCH_GRAPH))
    outs = {}
    for name, flags in modes:
        for _ in range(args.warmup):
            mix.run(flags)
        ms = []
        with ClockSampler(0) as clk:
            for _ in range(args.steps):
                st = mix.run(flags)
                ms.append(st[0].gpu_ms)
        res[name] = {"gbit_s": bits / (statistics.median(ms) / 1e3) / 1e9, "ms_median": statistics.median(ms),
                     "ms_max": max(ms), "max_residual": max(x.max_residual for x in st),
                     "exact_recomputed": sum(x.exact for x in st), "clocks": clk.summary()}
        outs[name] = mix.outputs()
    same = {name: all((a == b).all() for a, b in zip(outs[name], outs["serial"])) for name in outs}
    best = max(("graph", "persistent_graph"), key=lambda k: res[k]["gbit_s"])
    g = res[best]
    _line(METRIC, g["gbit_s"], UNIT, args.steps, args.warmup, g["ms_median"],
          "uneven mix: 512 blocks, n log-uniform [2^18, 2^25] (multiple of 1024), v/n ~ U[0.1,0.9] (multiple "
          "of 128), even blocks static seed (cached spectrum), odd blocks dynamic; one batch per step",
          {"batch_bits": bits, "modes": res, "headline_mode": best,
           "persistent_vs_graph": res["persistent_graph"]["gbit_s"] / res["graph"]["gbit_s"],
           "graph_vs_serial": res["graph"]["gbit_s"] / res["serial"]["gbit_s"],
           "outputs_equal_serial": same, "autotune_s": tune_s, "lanes": eng.set_lanes(0, 0),
           "splits": {str(k): v[0] for k, v in tuned.items()}, "clocks": g["clocks"]})
    eng.close()


def run_banked(args):
    """Equal sub-blocks of a 2^27-bit bank (the reference's sub-block variant): the engine's batch of B
    equal blocks (one CUDA graph) against the bank on batched cuFFT plans, static and dynamic seeds."""
    import privacyamplification_gb300 as pa
    from privacyamplification_gb300 import workloads as W
    from baseline import cufft_plain
    pa.load_library()
    cufft_plain.build()
    sizes, total_bits, total_s = [], 0, 0.0
    for log_s in (15, 18, 20, 22, 25):
        s, v, seeds, ks, kr = W.sub_block_bank(log_s)
        B = seeds.shape[0]
        bits = B * s
        row = {"log_s": log_s, "sub_blocks": B, "v": v}
        bank = cufft_plain.CufftBank(s, v, B)
        bank.load(seeds, ks, kr)
        eng = pa.Engine(max_sample_size=s)
        try:
            for static in (True, False):
                tag = "static" if static else "dynamic"
                for _ in range(args.warmup):
                    bank.run(recalc_seed=not static)
                with ClockSampler(0) as clk:
                    ms = [bank.run(recalc_seed=not static) for _ in range(args.steps)]
                row["cufft_bank_" + tag] = {"gbit_s": bits / (statistics.median(ms) / 1e3) / 1e9,
                                            "ms_median": statistics.median(ms), "clocks": clk.summary()}
                ref_out = bank.outputs()
                db = W.DeviceBank(eng, s, v, seeds, ks, kr, static)
                for _ in range(args.warmup):
                    db.run(pa.BATCH_GRAPH)
                with ClockSampler(0) as clk:
                    sts = [db.run(pa.BATCH_GRAPH) for _ in range(args.steps)]
                ms = [st[0].gpu_ms for st in sts]
                mine = db.outputs()
                row["engine_graph_" + tag] = {
                    "gbit_s": bits / (statistics.median(ms) / 1e3) / 1e9, "ms_median": statistics.median(ms),
                    "max_residual": max(x.max_residual for x in sts[-1]), "clocks": clk.summary(),
                    "blocks_equal_cufft_bank": int(sum((mine[i] == ref_out[i]).all() for i in range(B)))}
                row["engine_over_cufft_" + tag] = row["engine_graph_" + tag]["gbit_s"] / row["cufft_bank_" + tag]["gbit_s"]
                # group sizes: one launch per pass for 2^20 .. 2^27 bits of the bank's blocks
                if static:
                    sweep = {}
                    for lb in (20, 22, 24, 27):
                        if lb <= log_s:
                            continue
                        eng.set_groups(0, lb)
                        for _ in range(args.warmup):
                            db.run(pa.BATCH_GRAPH)
                        ms = [db.run(pa.BATCH_GRAPH)[0].gpu_ms for _ in range(args.steps)]
                        sweep["2^%d" % lb] = bits / (statistics.median(ms) / 1e3) / 1e9
                    eng.set_groups(0, 0)
                    row["engine_group_bits_sweep_gbit_s"] = sweep
                # the same bank launched block by block (no groups), and as one persistent lane launch
                # (lanes hold cyclic lengths from 2^20)
                alt = [("graph_no_group", pa.BATCH_GRAPH | pa.BATCH_NO_GROUP)]
                if log_s >= 20:
                    alt.append(("persistent", pa.BATCH_PERSISTENT))
                for name, fl in alt:
                    for _ in range(args.warmup):
                        db.run(fl)
                    sts = [db.run(fl) for _ in range(args.steps)]
                    ms = [st[0].gpu_ms for st in sts]
                    row["engine_%s_%s" % (name, tag)] = {
                        "gbit_s": bits / (statistics.median(ms) / 1e3) / 1e9, "ms_median": statistics.median(ms),
                        "blocks_equal_cufft_bank": int(sum((db.outputs()[i] == ref_out[i]).all() for i in range(B)))}
                if static:
                    total_bits += bits
                    total_s += row["engine_graph_static"]["ms_median"] / 1e3
                del db
        finally:
            eng.close()
            bank.close()
        sizes.append(row)
    value = total_bits / total_s / 1e9
    _line(METRIC, value, UNIT, args.steps, args.warmup, total_s / len(sizes) * 1e3,
          "sub-block banks: 2^27 bits as B equal blocks of s = 2^15 / 2^18 / 2^20 / 2^22 / 2^25 bits (B = 4096 / 512 / "
          "128 / 32 / 4), v = 3s/8, each block with its own seed and key; value: the engine's static-seed banks (one "
          "CUDA graph of the bank's groups: one launch per pass for up to 2^27 bits of equal blocks) over all "
          "five sizes",
          {"sizes": sizes, "baseline": "the reference's sub-block variant (PrivacyAmplification_subblocks.cu) "
                                       "restated on batched cuFFT plans, device inputs, no host syncs "
                                       "(baseline/cufft_plain.cu cb_*)"})


def run_serve(args, static):
    """Poisson arrivals; p50/p99 latency and sustained Gbit/s per rate; sampled same-alone-vs-in-mix check."""
    import privacyamplification_gb300 as pa
    from privacyamplification_gb300 import workloads as W
    pa.load_library()
    eng = pa.Engine(max_sample_size=1 << 27)
    reserved = eng.pool_reserve(1 << 27, 16)  # every slot's working set exists before the first request
    rates = [(10, 100), (100, 400), (500, 1000), (2000, 2000)]
    all_reqs = {rate: W.poisson_requests(rate, count, static=static, rng_seed=rate) for rate, count in rates}
    words = max(r.n // 32 + max(r.seed_word0, r.key_word0) for rs in all_reqs.values() for r in rs) + 64
    banks = W.HostBanks(words)
    seed_ids = None
    if static:
        seed_ids = {}
        for rs in all_reqs.values():
            for r in rs:
                if W.seed_key(r.n, r.v, r.flags) not in seed_ids:
                    seed_ids[W.seed_key(r.n, r.v, r.flags)] = eng.seed_cache_add(banks.seed_words(r), r.n, r.v, r.flags)
    warm = W.poisson_requests(5000, 24, static=static, rng_seed=1)
    for r in warm:
        r.seed_word0 = r.key_word0 = 0
        if static and W.seed_key(r.n, r.v, r.flags) not in seed_ids:
            seed_ids[W.seed_key(r.n, r.v, r.flags)] = eng.seed_cache_add(banks.seed_words(r), r.n, r.v, r.flags)
    W.serve(eng, warm, banks, seed_ids=seed_ids)
    lines = []
    checked = mismatched = 0
    for rate, count in rates:
        reqs = all_reqs[rate]
        with ClockSampler(0) as clk:
            res = W.serve(eng, reqs, banks, keep=lambda r: r.rid % 50 == 7, seed_ids=seed_ids)
        for r in reqs:
            if r.rid in res.outputs:
                eng.set_seed(banks.seed_words(r), r.n, -1)
                alone = eng.process(banks.key_start(r), banks.key_rest(r), r.n, r.v, r.flags)
                checked += 1
                mismatched += int(not (alone == res.outputs[r.rid]).all())
        offered = sum(r.n for r in reqs) / reqs[-1].arrival / 1e9
        lines.append({"rate_per_s": rate, "requests": count, "p50_ms": res.pct(50), "p99_ms": res.pct(99),
                      "sustained_gbit_s": res.bits / res.wall_s / 1e9, "offered_gbit_s": offered,
                      "wall_s": res.wall_s, "exact_recomputed": res.exact, "clocks": clk.summary()})
    # the same arrivals through the device-resident loop: lanes of the persistent kernel take requests from
    # a ring in pinned host memory; no launch or copy per request
    dev_lines = []
    lanes = eng.serve_start(ctas_per_lane=38, max_np=1 << 27, ring_slots=64)
    W.serve_device(eng, warm, banks, seed_ids=seed_ids)
    dchecked = dmismatched = 0
    for rate, count in rates:
        reqs = all_reqs[rate]
        with ClockSampler(0) as clk:
            res = W.serve_device(eng, reqs, banks, keep=lambda r: r.rid % 50 == 7, seed_ids=seed_ids)
        eng.serve_stop()
        for r in reqs:
            if r.rid in res.outputs:
                eng.set_seed(banks.seed_words(r), r.n, -1)
                alone = eng.process(banks.key_start(r), banks.key_rest(r), r.n, r.v, r.flags)
                dchecked += 1
                dmismatched += int(not (alone == res.outputs[r.rid]).all())
        eng.serve_start(ctas_per_lane=38, max_np=1 << 27, ring_slots=64)
        offered = sum(r.n for r in reqs) / reqs[-1].arrival / 1e9
        dev_lines.append({"rate_per_s": rate, "requests": count, "p50_ms": res.pct(50), "p99_ms": res.pct(99),
                          "sustained_gbit_s": res.bits / res.wall_s / 1e9, "offered_gbit_s": offered,
                          "wall_s": res.wall_s, "exact_recomputed": res.exact, "clocks": clk.summary()})
    eng.serve_stop()
    top = lines[-1]
    _line("p99 latency", top["p99_ms"], "ms", len(rates), 1, None,
          "serving: Poisson arrivals at 10/100/500/2000 blocks/s, n log-uniform [2^20, 2^27] "
          + ("rounded to a power of two, static seed spectra cached per size" if static
             else "(multiple of 1024), each request with its own seed")
          + ", v/n ~ U[0.2,0.8]; continuous admission to slots",
          {"rates": lines, "mix_equals_alone": {"checked": checked, "mismatched": mismatched},
           "slots_reserved": reserved,
           "device_loop": {"what": "pa_serve_*: %d lanes of 38 CTAs of the persistent kernel take requests from a "
                                   "ring in pinned host memory, read inputs from and write outputs to host memory"
                                   % lanes, "rates": dev_lines,
                           "mix_equals_alone": {"checked": dchecked, "mismatched": dmismatched}}}, higher=False)
    eng.close()


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--repeats", type=int, default=25, help="runs of the K-step timed region (value: median)")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-cufft", action="store_true", help="skip the cuFFT pipeline baseline leg")
    ap.add_argument("--no-configs", action="store_true", help="skip the short config-4 / config-5 legs")
    ap.add_argument("--workload", default="static27",
                    choices=["static27", "dynamic27", "dynamic29", "exact29", "batch", "banked", "serve", "serve-static"],
                    help="static27 (default): the headline line; the others print their own line")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "dynamic27":
        return run_dynamic27(args)
    if args.workload in ("dynamic29", "exact29"):
        return run_big29(args, force_exact=args.workload == "exact29")
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "banked":
        return run_banked(args)
    if args.workload in ("serve", "serve-static"):
        return run_serve(args, static=args.workload == "serve-static")
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
