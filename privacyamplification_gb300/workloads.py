"""Multi-block workloads on one engine: the uneven batched mix and the Poisson-arrival serving loop.

Both run through the C ABI's slot pool (pa_batch_run / pa_submit / pa_poll); nothing here computes
hash bits.  Key material is drawn from fixed-seed PCG64 streams as i.i.d. Bernoulli(0.5) words.

* uneven_mix(): blocks with n log-uniform in [2^lo, 2^hi] rounded to a multiple of 1024, v = ratio * n
  rounded to a multiple of 128 with ratio ~ U[r0, r1], h = n - v; even-numbered blocks use a static seed
  (spectrum cached before the run), odd-numbered ones bring their own seed (spectrum computed in the run).
* poisson_requests() + serve(): requests arrive at exponential inter-arrival times; serve() admits
  each to a free slot as soon as one is free (continuous batching: blocks of different sizes overlap on
  the GPU), polls for completions and records latency = completion - arrival.
* serve_device(): the same arrivals through the device-resident serving loop (pa_serve_*): the host
  only publishes request descriptors and reads completions; lanes on the GPU take requests as they free
  up, read the inputs from pinned host memory and write the outputs there.
* sub_block_bank() + DeviceBank: equal sub-blocks of a 2^27-bit bank, the batched form of the reference's
  sub-block variant, as one pa_batch_run.
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import FLAG_COMPRESS, FLAG_XOR_KEY_REST, PAJob, output_bytes

DEFAULT = FLAG_XOR_KEY_REST | FLAG_COMPRESS


def random_block(n: int, v: int, rng_seed: int = 0x5EED):
    """Seeded i.i.d. Bernoulli(0.5) seed and received-key words of one block (PCG64 stream `rng_seed`):
    the synthetic inputs of every benchmark workload.  Returns (seed[n/32], recv_key[n/32+1])."""
    rng = np.random.Generator(np.random.PCG64(rng_seed))
    seed = rng.integers(0, 2 ** 32, size=n // 32, dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2 ** 32, size=n // 32 + 1, dtype=np.uint64).astype(np.uint32)
    return seed, key


def sub_block_bank(log_s: int, bank_bits: int = 1 << 27, rng_seed: int = 0xBA4C):
    """The sub-block bank of the reference's sub-block variant: bank_bits cut into B = bank_bits / s
    blocks of s = 2^log_s bits with v = s/4 + s/8, each with its own seed and key (key2StartRest of its
    own received key).  Returns (s, v, seeds[B, s/32], key_start[B, s/32], key_rest[B, v/32])."""
    from . import key_split
    s = 1 << log_s
    v = s // 4 + s // 8
    B = bank_bits // s
    seeds = np.empty((B, s // 32), np.uint32)
    ks = np.empty((B, s // 32), np.uint32)
    kr = np.empty((B, v // 32), np.uint32)
    for i in range(B):
        seeds[i], recv = random_block(s, v, rng_seed + i)
        ks[i], kr[i] = key_split(recv, s, v)
    return s, v, seeds, ks, kr


class DeviceBank:
    """A sub-block bank on the device as pa_batch_run jobs: static seeds (one cached spectrum per block,
    as the bank keeps one per sub-block) or each block's own seed."""

    def __init__(self, engine, s, v, seeds, ks, kr, static: bool, device="cuda"):
        import torch
        self.engine, self.s, self.v, self.B = engine, s, v, seeds.shape[0]
        dev = torch.device(device)
        as_dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).reshape(-1).view(np.int32)).to(dev)
        self.d_seed, self.d_ks, self.d_kr = as_dev(seeds), as_dev(ks), as_dev(kr)
        self.d_out = torch.zeros(self.B * (v // 8), dtype=torch.uint8, device=dev)
        w, wr = s // 32, v // 32
        sids = [engine.seed_cache_add(seeds[i], s, v, DEFAULT) for i in range(self.B)] if static else None
        torch.cuda.synchronize()
        self.jobs = [PAJob(None if static else self.d_seed.data_ptr() + 4 * w * i, sids[i] if static else -1,
                           self.d_ks.data_ptr() + 4 * w * i, self.d_kr.data_ptr() + 4 * wr * i, s, v, DEFAULT,
                           self.d_out.data_ptr() + (v // 8) * i) for i in range(self.B)]

    def run(self, batch_flags=0, stream=0):
        self.engine.batch_run(self.jobs, batch_flags, stream)
        return self.engine.batch_sync(len(self.jobs))

    def outputs(self):
        return self.d_out.cpu().numpy().reshape(self.B, self.v // 8)


@dataclass
class Block:
    n: int
    v: int
    static: bool
    flags: int = DEFAULT
    seed_word0: int = 0  # offset of this block's seed in the shared seed bank (dynamic blocks)
    key_word0: int = 0   # offset of its key material in the key bank

    @property
    def h(self):
        return self.n - self.v


def seed_key(n, v, flags):
    """Blocks that can share one cached seed spectrum: a power-of-two n places the seed identically for
    every v and flags; otherwise the placement depends on h and the output length."""
    return (n,) if n & (n - 1) == 0 else (n, v, flags)


def _round_n(x, quantum=1024):
    return max(quantum, int(round(x / quantum)) * quantum)


def draw_sizes(rng, count, lo, hi, r0, r1):
    out = []
    for _ in range(count):
        n = _round_n(2.0 ** rng.uniform(lo, hi))
        ratio = rng.uniform(r0, r1)
        v = int(round(ratio * n / 128)) * 128
        v = min(max(v, 128), n - 128)
        out.append((n, v))
    return out


def uneven_mix(count=512, lo=18, hi=25, r0=0.1, r1=0.9, rng_seed=0xC0F4):
    """Config-4 block list (deterministic)."""
    rng = np.random.default_rng(rng_seed)
    sizes = draw_sizes(rng, count, lo, hi, r0, r1)
    blocks = []
    for i, (n, v) in enumerate(sizes):
        blocks.append(Block(n=n, v=v, static=(i % 2 == 0), seed_word0=int(rng.integers(0, 1 << 20)) * 8,
                            key_word0=int(rng.integers(0, 1 << 20)) * 8))
    return blocks


def bank(words, rng_seed):
    """Random uint32 words (the shared seed / key banks blocks take windows of)."""
    return np.random.default_rng(rng_seed).integers(0, 1 << 32, size=words, dtype=np.uint64).astype(np.uint32)


def bank_words_for(blocks):
    return max(b.n // 32 + max(b.seed_word0, b.key_word0) + 64 for b in blocks)


class DeviceMix:
    """Device-resident inputs/outputs of a block list for pa_batch_run (torch tensors hold the memory)."""

    def __init__(self, engine, blocks, device="cuda", rng_seed=0xB10C):
        import torch
        self.engine, self.blocks = engine, blocks
        words = bank_words_for(blocks)
        self.seed_bank = bank(words, rng_seed)
        self.key_bank = bank(words + 64, rng_seed + 1)
        self.rest_bank = bank(words + 64, rng_seed + 2)
        dev = torch.device(device)
        as_dev = lambda a: torch.from_numpy(a.view(np.int32)).to(dev)
        self.d_seed, self.d_key, self.d_rest = as_dev(self.seed_bank), as_dev(self.key_bank), as_dev(self.rest_bank)
        self.out_bytes = [output_bytes(b.n, b.v, b.flags) for b in blocks]
        self.out_off = np.concatenate([[0], np.cumsum([(x + 255) // 256 * 256 for x in self.out_bytes])])
        self.d_out = torch.zeros(int(self.out_off[-1]), dtype=torch.uint8, device=dev)
        self.seed_ids = {}
        for b in blocks:
            if b.static:
                key = seed_key(b.n, b.v, b.flags)
                if key not in self.seed_ids:
                    self.seed_ids[key] = engine.seed_cache_add(self.seed_words(b), b.n, b.v, b.flags)
        torch.cuda.synchronize()
        self.jobs = [self._job(i, b) for i, b in enumerate(blocks)]

    def seed_words(self, b):
        """The seed a block uses (static blocks: the one cached for their geometry)."""
        if b.static:
            return self.seed_bank[: b.n // 32]
        return self.seed_bank[b.seed_word0: b.seed_word0 + b.n // 32]

    def key_start(self, b):
        return self.key_bank[b.key_word0: b.key_word0 + b.n // 32]

    def key_rest(self, b):
        return self.rest_bank[b.key_word0: b.key_word0 + b.v // 32]

    def _job(self, i, b):
        seed_ptr = 0 if b.static else self.d_seed.data_ptr() + 4 * b.seed_word0
        sid = self.seed_ids[seed_key(b.n, b.v, b.flags)] if b.static else -1
        return PAJob(seed_ptr or None, sid, self.d_key.data_ptr() + 4 * b.key_word0,
                     self.d_rest.data_ptr() + 4 * b.key_word0, b.n, b.v, b.flags,
                     self.d_out.data_ptr() + int(self.out_off[i]))

    def outputs(self):
        host = self.d_out.cpu().numpy()
        return [host[self.out_off[i]: self.out_off[i] + self.out_bytes[i]].copy() for i in range(len(self.blocks))]

    def run(self, batch_flags=0, stream=0):
        self.engine.batch_run(self.jobs, batch_flags, stream)
        return self.engine.batch_sync(len(self.jobs))


# ------------------------------------------------------------------------------------------ serving
@dataclass
class Request:
    rid: int
    arrival: float  # seconds from the start of the run
    n: int
    v: int
    static: bool
    seed_word0: int
    key_word0: int
    flags: int = DEFAULT
    done: float = -1.0
    exact: int = 0


def poisson_requests(rate, count, lo=20, hi=27, r0=0.2, r1=0.8, static=False, rng_seed=0x5E7E):
    """Config-5 request stream.  static=True rounds n to a power of two (one cached seed per size)."""
    rng = np.random.default_rng(rng_seed)
    t = 0.0
    reqs = []
    for i, (n, v) in enumerate(draw_sizes(rng, count, lo, hi, r0, r1)):
        if static:
            ratio = v / n
            n = 1 << int(round(np.log2(n)))
            v = min(max(int(round(ratio * n / 128)) * 128, 128), n - 128)
        t += rng.exponential(1.0 / rate)
        reqs.append(Request(rid=i, arrival=t, n=n, v=v, static=static, seed_word0=int(rng.integers(0, 1 << 20)) * 8,
                            key_word0=int(rng.integers(0, 1 << 20)) * 8))
    return reqs


@dataclass
class ServeResult:
    latency_ms: list
    wall_s: float
    bits: int
    outputs: dict = field(default_factory=dict)  # rid -> output bytes for the kept requests
    exact: int = 0

    def pct(self, q):
        return float(np.percentile(np.asarray(self.latency_ms), q)) if self.latency_ms else None


class HostBanks:
    """Pinned host banks the served requests take their seed / key / key_rest windows from."""

    def __init__(self, words, rng_seed=0x5EED):
        import torch
        pin = lambda a: torch.from_numpy(a.view(np.int32)).pin_memory().numpy().view(np.uint32)
        self.seed = pin(bank(words, rng_seed))
        self.key = pin(bank(words + 64, rng_seed + 1))
        self.rest = pin(bank(words + 64, rng_seed + 2))

    def seed_words(self, r):
        return self.seed[: r.n // 32] if r.static else self.seed[r.seed_word0: r.seed_word0 + r.n // 32]

    def key_start(self, r):
        return self.key[r.key_word0: r.key_word0 + r.n // 32]

    def key_rest(self, r):
        return self.rest[r.key_word0: r.key_word0 + r.v // 32]


def serve(engine, reqs, banks, out_slots=24, keep=lambda r: False, seed_ids=None, idle_sleep=20e-6):
    """Serves `reqs` in real time on `engine`; returns latencies and the outputs of requests `keep` selects.

    Admission is FIFO: a request waits until pa_submit finds it a slot (and a free pinned output
    buffer); completed blocks free their slot immediately, so later arrivals overlap with running ones.
    """
    import torch
    max_out = max(output_bytes(r.n, r.v, r.flags) for r in reqs)
    outs = [torch.empty(max_out + 4, dtype=torch.uint8).pin_memory().numpy() for _ in range(out_slots)]
    free_out = list(range(out_slots))
    pending = deque(sorted(reqs, key=lambda r: r.arrival))
    waiting = deque()
    inflight = {}
    res = ServeResult(latency_ms=[], wall_s=0.0, bits=0)
    t0 = time.perf_counter()
    remaining = len(reqs)
    while remaining:
        now = time.perf_counter() - t0
        progressed = False
        while pending and pending[0].arrival <= now:
            waiting.append(pending.popleft())
        while waiting and free_out:
            r = waiting[0]
            ob = free_out[-1]
            sid = seed_ids[seed_key(r.n, r.v, r.flags)] if (r.static and seed_ids is not None) else -1
            seed = None if sid >= 0 else banks.seed_words(r)
            job = PAJob(seed.ctypes.data if seed is not None else None, sid, banks.key_start(r).ctypes.data,
                        banks.key_rest(r).ctypes.data, r.n, r.v, r.flags, outs[ob].ctypes.data)
            t = engine.submit(job)
            if t is None:
                break
            free_out.pop()
            waiting.popleft()
            inflight[t] = (r, ob)
            progressed = True
        for t in list(inflight):
            st = engine.poll(t)
            if st is None:
                continue
            r, ob = inflight.pop(t)
            r.done = time.perf_counter() - t0
            r.exact = st.exact
            res.exact += st.exact
            res.latency_ms.append((r.done - r.arrival) * 1e3)
            res.bits += r.n
            if keep(r):
                res.outputs[r.rid] = outs[ob][: output_bytes(r.n, r.v, r.flags)].copy()
            free_out.append(ob)
            remaining -= 1
            progressed = True
        if not progressed:
            if not inflight and not waiting and pending:
                time.sleep(max(0.0, min(pending[0].arrival - (time.perf_counter() - t0), 1e-3)))
            else:
                time.sleep(idle_sleep)
    res.wall_s = time.perf_counter() - t0
    return res


def serve_device(engine, reqs, banks, out_slots=24, keep=lambda r: False, seed_ids=None, idle_sleep=20e-6,
                 stall_s=60.0):
    """Serves `reqs` in real time through the device-resident loop (engine.serve_start() first); returns
    latencies and the outputs of requests `keep` selects.  Admission is FIFO: a request waits for a free
    pinned output buffer and a free ring slot; the device takes published requests as lanes free up.
    Raises TimeoutError when no request completes for stall_s seconds."""
    import torch
    max_out = max(output_bytes(r.n, r.v, r.flags) for r in reqs)
    outs = [torch.empty(max_out + 4, dtype=torch.uint8).pin_memory().numpy() for _ in range(out_slots)]
    free_out = list(range(out_slots))
    pending = deque(sorted(reqs, key=lambda r: r.arrival))
    waiting = deque()
    inflight = {}
    res = ServeResult(latency_ms=[], wall_s=0.0, bits=0)
    t0 = time.perf_counter()
    remaining = len(reqs)
    last_done = t0
    while remaining:
        now = time.perf_counter() - t0
        if inflight and time.perf_counter() - last_done > stall_s:
            raise TimeoutError("the serving loop completed no request in %.0f s" % stall_s)
        progressed = False
        while pending and pending[0].arrival <= now:
            waiting.append(pending.popleft())
        while waiting and free_out:
            r = waiting[0]
            ob = free_out[-1]
            sid = seed_ids[seed_key(r.n, r.v, r.flags)] if (r.static and seed_ids is not None) else -1
            seed = None if sid >= 0 else banks.seed_words(r)
            job = PAJob(seed.ctypes.data if seed is not None else None, sid, banks.key_start(r).ctypes.data,
                        banks.key_rest(r).ctypes.data, r.n, r.v, r.flags, outs[ob].ctypes.data)
            t = engine.serve_submit(job)
            if t is None:
                break
            free_out.pop()
            waiting.popleft()
            inflight[t] = (r, ob)
            progressed = True
        for t in list(inflight):
            st = engine.serve_poll(t)
            if st is None:
                continue
            r, ob = inflight.pop(t)
            r.done = time.perf_counter() - t0
            last_done = time.perf_counter()
            r.exact = st.exact
            res.exact += st.exact
            res.latency_ms.append((r.done - r.arrival) * 1e3)
            res.bits += r.n
            if keep(r):
                res.outputs[r.rid] = outs[ob][: output_bytes(r.n, r.v, r.flags)].copy()
            free_out.append(ob)
            remaining -= 1
            progressed = True
        if not progressed:
            if not inflight and not waiting and pending:
                time.sleep(max(0.0, min(pending[0].arrival - (time.perf_counter() - t0), 1e-3)))
            else:
                time.sleep(idle_sleep)
    res.wall_s = time.perf_counter() - t0
    return res
