"""Generates tests/golden/large_block_kat.npz from the reference's large-block example.

Source (read as text, never compiled): examples/LargeBlocksizeExample/Matrix.h of
nicoboss/PrivacyAmplification.  It holds

* ``key_input[16384]`` and ``toeplitz_seed_input[16384]`` (Matrix.h:4-5) -- 0/1 bytes, packed MSB-first
  into uint32 words by ``binTo4byteLittleEndian`` (examples/LargeBlocksizeExample/main.cpp:220-230);
* ``ampOutInData_hash[60][32]`` (Matrix.h:7) -- SHA3-256 of the 60 chunk outputs
  (n=2^11, v=h=1024, do_xor_key_rest=false, do_compress=false);
* ``amp_out_intermediate_hash[70][32]`` (Matrix.h:250) -- SHA3-256 of the row-XOR accumulator;
* ``amp_out_pre_hash``, ``key_rest_hash``, ``amp_out_reult`` (Matrix.h:533,540,547) -- the n=2^14
  (v=6144, h=10240) composite before the key_rest XOR, the key_rest bytes, and the final result.

Usage: python tests/golden/make_golden.py path/to/Matrix.h
       (or PA_REFERENCE_TREE=<root of the reference tree> python tests/golden/make_golden.py)
The fixture is committed; this script only has to be re-run if the source changes.
"""
import os
import re
import sys

import numpy as np

MATRIX_H = os.path.join("examples", "LargeBlocksizeExample", "Matrix.h")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "large_block_kat.npz")


def _array_body(text, name):
    m = re.search(r"%s\s*\[[^\]]*\](?:\s*\[[^\]]*\])?\s*=\s*\{(.*?)\};" % re.escape(name), text, re.S)
    if not m:
        raise SystemExit("array %s not found" % name)
    return m.group(1)


def _ints(body):
    return [int(t, 0) for t in re.findall(r"0x[0-9A-Fa-f]+|\d+", body)]


def main(src):
    text = open(src).read()
    key = np.array(_ints(_array_body(text, "key_input")), dtype=np.uint8)
    seed = np.array(_ints(_array_body(text, "toeplitz_seed_input")), dtype=np.uint8)
    assert key.size == 16384 and seed.size == 16384, (key.size, seed.size)
    assert set(np.unique(key)) <= {0, 1} and set(np.unique(seed)) <= {0, 1}
    chunk = np.array(_ints(_array_body(text, "ampOutInData_hash")), dtype=np.uint8).reshape(-1, 32)
    inter = np.array(_ints(_array_body(text, "amp_out_intermediate_hash")), dtype=np.uint8).reshape(-1, 32)
    pre = np.array(_ints(_array_body(text, "amp_out_pre_hash")), dtype=np.uint8)
    krh = np.array(_ints(_array_body(text, "key_rest_hash")), dtype=np.uint8)
    res = np.array(_ints(_array_body(text, "amp_out_reult")), dtype=np.uint8)
    assert chunk.shape == (60, 32) and inter.shape == (70, 32), (chunk.shape, inter.shape)
    assert pre.size == krh.size == res.size == 32
    np.savez_compressed(OUT, key_bits=np.packbits(key), seed_bits=np.packbits(seed), chunk_hash=chunk,
                        intermediate_hash=inter, pre_hash=pre, key_rest_hash=krh, result_hash=res)
    print("wrote", OUT)


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    elif os.environ.get("PA_REFERENCE_TREE"):
        main(os.path.join(os.environ["PA_REFERENCE_TREE"], MATRIX_H))
    else:
        raise SystemExit(__doc__)
