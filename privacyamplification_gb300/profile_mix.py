"""Runs the config-4 uneven mix (512 blocks, n log-uniform in [2^18, 2^25], half with their own seed) as one
batch, for a profiler's launch list.

    python -m privacyamplification_gb300.profile_mix [--runs 1] [--flags graph|concurrent|persistent]

The mix is the bench's `batch` workload (same block list and inputs); after one untimed warm-up batch and
one marker launch (the bounded-wait self-test kernel, k_wait_expires, so a launch list can be cut there)
it runs `runs` batches and prints the batch device time of the last, so a profiled run can be matched
with the unprofiled one.
"""
from __future__ import annotations

import argparse
import json


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--runs", type=int, default=1)
    ap.add_argument("--flags", choices=["graph", "concurrent", "persistent"], default="graph")
    args = ap.parse_args()
    import privacyamplification_gb300 as pa
    from privacyamplification_gb300 import workloads as W
    flags = {"graph": pa.BATCH_GRAPH, "concurrent": 0, "persistent": pa.BATCH_PERSISTENT}[args.flags]
    with pa.Engine(max_sample_size=1 << 25) as eng:
        eng.autotune(1 << 18, 1 << 26)
        blocks = W.uneven_mix()
        mix = W.DeviceMix(eng, blocks)
        mix.run(flags)
        pa.selftest_wait_timeout(0, rounds=1)  # a marker launch (k_wait_expires) before the measured batches
        for _ in range(args.runs):
            st = mix.run(flags)
        print(json.dumps({"blocks": len(blocks), "bits": sum(b.n for b in blocks), "flags": args.flags,
                          "batch_ms": st[0].gpu_ms, "max_residual": max(s.max_residual for s in st)}))


if __name__ == "__main__":
    main()
