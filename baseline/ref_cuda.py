"""The reference's own CUDA kernels for the cuFFT pipeline baseline (cufft_plain.cu).

    python -m baseline.ref_cuda      # where the reference tree is present: build the fatbin

Compiles the device code of PrivacyAmplification/PrivacyAmplification.cu, where it lies in the reference
tree (never copied), for sm_103a into baseline/_ref_cuda/pa_ref_sm103a.fatbin (git-ignored).  The fatbin
holds GPU code only, so it serves the Arm GPU host as it is; its host side is cufft_plain.cu, which
loads it with cudaLibraryLoadFromFile and launches binInt2float, calculateCorrectionFloat,
setFirstElementToZero, ElementWiseProduct and ToBinaryArray[NoXOR] in the reference's mainloop order
(PrivacyAmplification.cu:1797-2042).  The reference's host program itself cannot run there: it is a
ZeroMQ service (libzmq is absent) and a binary built here is x86.

The tree's location: $PA_REFERENCE_TREE, else the default below; without it, build() does nothing and
the baseline runs its restated kernels.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref_cuda")
FATBIN = os.path.join(OUT_DIR, "pa_ref_sm103a.fatbin")
DEFAULT_TREE = "/root/reference"


def tree() -> str | None:
    t = os.environ.get("PA_REFERENCE_TREE", DEFAULT_TREE)
    src = os.path.join(t, "PrivacyAmplification", "PrivacyAmplification.cu")
    return t if os.path.exists(src) else None


def build(force: bool = False) -> str | None:
    """Builds the fatbin when the reference tree is present; returns its path if it exists."""
    t = tree()
    if t is None:
        return FATBIN if os.path.exists(FATBIN) else None
    src = os.path.join(t, "PrivacyAmplification", "PrivacyAmplification.cu")
    if not force and os.path.exists(FATBIN) and os.path.getmtime(FATBIN) >= os.path.getmtime(src):
        return FATBIN
    from privacyamplification_gb300.build import ARCH, nvcc
    os.makedirs(OUT_DIR, exist_ok=True)
    # -std=c++14 as the reference's MakefileCuda; its vendored libzmq headers let the host part parse
    cmd = [nvcc(), "--fatbin", *ARCH, "-O3", "-std=c++14", "-I" + os.path.join(t, "PrivacyAmplification"),
           "-I" + os.path.join(t, "libzmq", "include"), "-w", src, "-o", FATBIN]
    subprocess.run(cmd, check=True, cwd=OUT_DIR)
    return FATBIN


def fatbin() -> str | None:
    return FATBIN if os.path.exists(FATBIN) else None


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
