"""Runs a few device-resident blocks of one size back to back, for a profiler's launch list or capture.

    python -m privacyamplification_gb300.profile_block [--log-n 27] [--blocks 4] [--v-frac 0.375]
                                                       [--lanes [--ctas-per-lane T]] [--one-use-seed]

Seed and keys are i.i.d. Bernoulli(0.5) bits from fixed PCG64 seeds (the bench's inputs at n = 2^27); the
seed spectrum is computed once, then `blocks` key blocks run through pa_process_device on one stream
(or, with --lanes, as one persistent lane batch of that many blocks).  With --one-use-seed the seed is
set again before every block for that block only, so each block transforms it in its own column pass.  Prints the per-kernel mean device
times the engine records, so a profiled run can be matched with the unprofiled one.
"""
from __future__ import annotations

import argparse
import json


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--log-n", type=int, default=27)
    ap.add_argument("--blocks", type=int, default=4)
    ap.add_argument("--v-frac", type=float, default=0.375)
    ap.add_argument("--lanes", action="store_true", help="run the blocks as one persistent lane batch")
    ap.add_argument("--ctas-per-lane", type=int, default=0, help="lane width (0: the engine's default)")
    ap.add_argument("--repeat", type=int, default=1, help="lane batches run (the last one is reported)")
    ap.add_argument("--one-use-seed", action="store_true",
                    help="set the seed before every block for that block only (the fused column pass)")
    args = ap.parse_args()
    import numpy as np
    import torch
    import privacyamplification_gb300 as pa

    n = 1 << args.log_n
    v = int(n * args.v_frac) // 32 * 32
    rng = np.random.Generator(np.random.PCG64(0x5EED))
    words = lambda k: rng.integers(0, 2 ** 32, size=k, dtype=np.uint64).astype(np.uint32)
    seed = words(n // 32)
    keys = [pa.key_split(words(n // 32 + 1), n, v) for _ in range(2)]
    dev = torch.device("cuda", 0)
    d = lambda a: torch.from_numpy(a.view(np.int32)).to(dev)
    d_keys = [(d(ks), d(kr)) for ks, kr in keys]
    out = torch.empty((pa.output_bytes(n, v) + 3) // 4, dtype=torch.int32, device=dev)
    with pa.Engine(max_sample_size=n) as eng:
        if args.lanes:
            eng.set_lanes(args.ctas_per_lane, n)
            sid = eng.seed_cache_add(seed, n, v)
            outs = [torch.empty_like(out) for _ in range(args.blocks)]
            jobs = [pa.PAJob(None, sid, d_keys[i % 2][0].data_ptr(), d_keys[i % 2][1].data_ptr(), n, v,
                             pa.DEFAULT_FLAGS, outs[i].data_ptr()) for i in range(args.blocks)]
            for _ in range(args.repeat):
                eng.batch_run(jobs, pa.BATCH_PERSISTENT)
                st = eng.batch_sync(len(jobs))
            print(json.dumps({"n": n, "v": v, "blocks": args.blocks, "lanes": eng.set_lanes(0, 0),
                              "batch_ms": st[0].gpu_ms, "max_residual": max(s.max_residual for s in st)}))
            return
        s = torch.cuda.Stream(device=dev)
        d_seed = d(seed)
        if not args.one_use_seed:
            eng.set_seed(seed, n, -1)
        eng.set_timing(True)
        for i in range(args.blocks):
            if args.one_use_seed:  # queued on the blocks' stream, after the previous block's reads
                eng.set_seed_device(d_seed.data_ptr(), n, 1, stream=s.cuda_stream)
            ks, kr = d_keys[i % 2]
            eng.process_device(ks.data_ptr(), kr.data_ptr(), n, v, out.data_ptr(), stream=s.cuda_stream)
        st = eng.sync()
        ms, nb = eng.stage_times()
        print(json.dumps({"n": n, "v": v, "blocks": nb, "kernels_ms": ms, "max_residual": st.max_residual}))


if __name__ == "__main__":
    main()
