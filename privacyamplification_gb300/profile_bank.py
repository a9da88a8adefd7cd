"""Runs one sub-block bank (2^27 bits as equal blocks) as one batch, for a profiler's launch list.

    python -m privacyamplification_gb300.profile_bank [--log-s 18] [--no-group] [--dynamic]

The blocks are workloads.sub_block_bank's (each with its own seed and key).  One untimed warm-up batch,
then a marker launch (the bounded-wait self-test kernel, k_wait_expires), then one batch; prints its
device time.
"""
from __future__ import annotations

import argparse
import json


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--log-s", type=int, default=18)
    ap.add_argument("--no-group", action="store_true", help="launch every block on its own")
    ap.add_argument("--dynamic", action="store_true", help="every block brings its own seed")
    args = ap.parse_args()
    import privacyamplification_gb300 as pa
    from privacyamplification_gb300 import workloads as W
    s, v, seeds, ks, kr = W.sub_block_bank(args.log_s)
    flags = pa.BATCH_GRAPH | (pa.BATCH_NO_GROUP if args.no_group else 0)
    with pa.Engine(max_sample_size=s) as eng:
        bank = W.DeviceBank(eng, s, v, seeds, ks, kr, static=not args.dynamic)
        bank.run(flags)
        pa.selftest_wait_timeout(0, rounds=1)  # marker launch
        st = bank.run(flags)
        print(json.dumps({"s": s, "blocks": bank.B, "grouped": not args.no_group, "dynamic": args.dynamic,
                          "batch_ms": st[0].gpu_ms}))


if __name__ == "__main__":
    main()
