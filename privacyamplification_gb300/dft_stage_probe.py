"""Times one radix-16 DFT stage on the tensor cores against the FP32 butterflies (pa_dft16_stages).

    python -m privacyamplification_gb300.dft_stage_probe [--log-butterflies 22] [--reps 8 72] [--once]

The cost of a stage is taken from two runs that differ only in the number of stages, so the loads and
stores of the data cancel: (t(reps_hi) - t(reps_lo)) / (reps_hi - reps_lo).  2^22 butterflies of 16
complex values are the 2^26 points one radix-16 stage of a 2^27-bit block touches.  Accuracy: relative
RMS error after reps_hi stages (reps % 4 == 0 returns the input) and after one stage against numpy's FFT.
Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import statistics

import numpy as np

import privacyamplification_gb300 as pa

METHODS = {"fp32_butterflies": pa.DFT16_FP32, "tcgen05_tf32_split3": pa.DFT16_TC_SPLIT,
           "tcgen05_tf32_single": pa.DFT16_TC_TF32}


def main(argv=None) -> int:
    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("--log-butterflies", type=int, default=22)
    ap.add_argument("--reps", type=int, nargs=2, default=[8, 72])
    ap.add_argument("--repeats", type=int, default=7)
    ap.add_argument("--once", action="store_true", help="one launch per method (16 stages, 4 CTAs/SM), no timing")
    args = ap.parse_args(argv)
    lo, hi = args.reps
    assert lo % 4 == 0 and hi % 4 == 0 and hi > lo
    b = 1 << args.log_butterflies
    pa.load_library()
    dev = torch.device("cuda")
    g = torch.Generator(device="cpu").manual_seed(0xDF7)
    x = (torch.rand(b * 32, generator=g, dtype=torch.float64) * 2 - 1).float().to(dev)
    y = torch.empty_like(x)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream().cuda_stream

    def timed(method, reps, cps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ts = []
        for _ in range(args.repeats):
            torch.cuda.synchronize()
            ev[0].record()
            pa.dft16_stages(x.data_ptr(), y.data_ptr(), b, reps, method, err.data_ptr(), cps, s)
            ev[1].record()
            torch.cuda.synchronize()
            ts.append(ev[0].elapsed_time(ev[1]) * 1e3)
        return statistics.median(ts)

    if args.once:  # one launch of each kernel, e.g. for a profiler
        for m in METHODS.values():
            pa.dft16_stages(x.data_ptr(), y.data_ptr(), b, 16, m, err.data_ptr(), 4, s)
        torch.cuda.synchronize()
        print(json.dumps({"once": True, "err_word": int(err.item())}))
        return 0 if int(err.item()) == 0 else 1
    xs = x[: 128 * 32].cpu().double().numpy().view(np.complex128).reshape(128, 16)
    want1 = np.fft.fft(xs, axis=1)
    out = {"butterflies": b, "reps": [lo, hi], "methods": {}}
    for name, m in METHODS.items():
        res = {}
        for cps in ([2, 4, 8, 16] if m == pa.DFT16_FP32 else [1, 2, 4]):
            pa.dft16_stages(x.data_ptr(), y.data_ptr(), b, 4, m, err.data_ptr(), cps, s)  # warm-up
            t_lo, t_hi = timed(m, lo, cps), timed(m, hi, cps)
            res[str(cps)] = {"us_lo": t_lo, "us_hi": t_hi, "us_per_stage": (t_hi - t_lo) / (hi - lo)}
        best = min(res.values(), key=lambda r: r["us_per_stage"])
        pa.dft16_stages(x.data_ptr(), y.data_ptr(), b, hi, m, err.data_ptr(), 2, s)
        torch.cuda.synchronize()
        rel_hi = float(torch.linalg.vector_norm((y - x).double()) / torch.linalg.vector_norm(x.double()))
        pa.dft16_stages(x.data_ptr(), y.data_ptr(), 128, 1, m, err.data_ptr(), 1, s)
        torch.cuda.synchronize()
        got1 = y[: 128 * 32].cpu().double().numpy().view(np.complex128).reshape(128, 16)
        rel_1 = float(np.linalg.norm(got1 - want1) / np.linalg.norm(want1))
        out["methods"][name] = {"by_ctas_per_sm": res, "us_per_stage": best["us_per_stage"],
                                "rel_rms_error_one_stage": rel_1, "rel_rms_error_after_reps_hi": rel_hi}
    out["err_word"] = int(err.item())
    f = out["methods"]["fp32_butterflies"]["us_per_stage"]
    out["tensor_split3_over_fp32"] = out["methods"]["tcgen05_tf32_split3"]["us_per_stage"] / f
    out["tensor_single_over_fp32"] = out["methods"]["tcgen05_tf32_single"]["us_per_stage"] / f
    print(json.dumps(out))
    return 0 if out["err_word"] == 0 else 1


if __name__ == "__main__":
    raise SystemExit(main())
