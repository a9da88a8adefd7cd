"""The host loop end to end on the GPU: seed server, key server and ampout client speak the reference's
ZeroMQ message layouts (examples/MatrixSeedServerExample, SendKeysExample, ReceiveAmpOutExample) over
ZMTP; every block that comes back equals the oracle.  File inputs, SHA3 verification and the exit codes
101/103/104/105/106, and the `pa_service` executable."""
import os
import subprocess
import threading

import numpy as np
import pytest

from privacyamplification_gb300 import service as S
from oracle import oracle as O
from zmtp_peer import Peer, free_port

pytestmark = pytest.mark.gpu

N = 1 << 16


def cfg_for(**kw):
    base = dict(factor_exp=16, show_ampout=-1, show_zeromq_status=0, verify_ampout=0,
                store_first_ampouts_in_file=0, input_blocks_to_cache=4, output_blocks_to_cache=4)
    base.update(kw)
    return S.default_config(**base)


def run_service(cfg, blocks):
    res = {}
    t = threading.Thread(target=lambda: res.setdefault("rc", S.run(cfg, blocks)), daemon=True)
    t.start()
    return t, res


def test_zeromq_loop_matches_oracle(pa_lib):
    """4 seeds with reuse amounts 2, 0, 1, -1 and 6 key blocks of mixed v / flags: block i uses the seed
    the reference's reuse rule assigns (2 blocks, 1, 1, then the last one for good)."""
    eps = ["tcp://127.0.0.1:%d" % free_port() for _ in range(3)]
    seed_srv, key_srv = Peer("PUSH", eps[0], bind=True), Peer("PUSH", eps[1], bind=True)
    cfg = cfg_for(address_seed_in=eps[0], address_key_in=eps[1], address_amp_out=eps[2])
    t, res = run_service(cfg, 6)
    rng = np.random.default_rng(5)
    seeds = [rng.integers(0, 1 << 32, N // 32, dtype=np.uint64).astype(np.uint32) for _ in range(4)]
    reuse = [2, 0, 1, -1]
    blocks = [(24576, True, True), (24576, False, True), (8192, True, False), (40960, False, False),
              (24576, True, True), (32768, True, True)]
    recv_keys = [rng.integers(0, 1 << 32, N // 32 + 1, dtype=np.uint64).astype(np.uint32) for _ in blocks]

    def seed_server():
        for s, r in zip(seeds, reuse):
            seed_srv.send(np.int32(r).tobytes(), s.tobytes())

    def key_server():
        for (v, xor, comp), rk in zip(blocks, recv_keys):
            h = N - v
            data = rk if xor else O.key_split(rk, N, v)[0][: h // 32 + 1]
            key_srv.send(bytes([xor]), bytes([comp]), np.uint32(v // 32).tobytes(), data.tobytes())

    threads = [threading.Thread(target=f, daemon=True) for f in (seed_server, key_server)]
    for th in threads:
        th.start()
    client = Peer("PULL", eps[2], bind=False)
    try:
        seed_of_block = [0, 0, 1, 2, 3, 3]
        for i, ((v, xor, comp), rk) in enumerate(zip(blocks, recv_keys)):
            (got,) = client.recv()
            ks, kr = O.key_split(rk, N, v)
            flags = (O.FLAG_XOR_KEY_REST if xor else 0) | (O.FLAG_COMPRESS if comp else 0)
            want = O.direct(seeds[seed_of_block[i]], ks, kr, N, v, flags)
            assert np.array_equal(np.frombuffer(got, np.uint8), want), i
        t.join(60)
        assert res.get("rc") == 0
    finally:
        for p in (client, seed_srv, key_srv):
            p.close()


@pytest.fixture()
def files(tmp_path):
    rng = np.random.default_rng(9)
    seed = rng.integers(0, 1 << 32, N // 32, dtype=np.uint64).astype(np.uint32)
    recv = rng.integers(0, 1 << 32, N // 32 + 1, dtype=np.uint64).astype(np.uint32)
    (tmp_path / "toeplitz_seed.bin").write_bytes(seed.tobytes())
    (tmp_path / "keyfile.bin").write_bytes(recv.tobytes())
    v = 24576
    ks, kr = O.key_split(recv, N, v)
    want = O.direct(seed, ks, kr, N, v)
    (tmp_path / "ampout.sh3").write_text("; SHA3-256 of the first block\n%s *ampout.bin\n" % O.sha3_256(want.tobytes()))
    return tmp_path, want


def file_cfg(d, **kw):
    base = dict(use_matrix_seed_server=0, use_key_server=0, host_ampout_server=0, vertical_len=24576,
                toeplitz_seed_path=str(d / "toeplitz_seed.bin"), keyfile_path=str(d / "keyfile.bin"),
                ampout_sha3_path=str(d / "ampout.sh3"), ampout_path=str(d / "ampout.bin"))
    base.update(kw)
    return cfg_for(**base)


def test_file_inputs_verify_and_store(pa_lib, files):
    d, want = files
    rc = S.run(file_cfg(d, verify_ampout=1, store_first_ampouts_in_file=2), 3)
    assert rc == 0
    stored = np.frombuffer((d / "ampout.bin").read_bytes(), np.uint8)
    assert np.array_equal(stored, np.concatenate([want, want]))


def test_exit_codes(pa_lib, files):
    d, _ = files
    (d / "bad.sh3").write_text("%s *ampout.bin\n" % ("00" * 32))
    assert S.run(file_cfg(d, verify_ampout=1, ampout_sha3_path=str(d / "bad.sh3")), 2) == 101
    assert S.run(file_cfg(d, toeplitz_seed_path=str(d / "none.bin")), 1) == 103
    (d / "short.bin").write_bytes(b"\x00" * 100)
    assert S.run(file_cfg(d, toeplitz_seed_path=str(d / "short.bin")), 1) == 104
    assert S.run(file_cfg(d, keyfile_path=str(d / "none.bin")), 1) == 105
    assert S.run(file_cfg(d, keyfile_path=str(d / "short.bin")), 1) == 106


def test_service_executable(pa_lib, files):
    d, want = files
    (d / "config.yaml").write_text(
        "factor_exp: 16\nvertical_len: 24576\nuse_matrix_seed_server: false\nuse_key_server: false\n"
        "host_ampout_server: false\nverify_ampout: true\nstore_first_ampouts_in_file: 1\nshow_ampout: 4\n")
    r = subprocess.run([S.SERVICE_BIN, "config.yaml", "--blocks", "2"], cwd=d, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "VERIFIED!" in r.stdout
    assert np.array_equal(np.frombuffer((d / "ampout.bin").read_bytes(), np.uint8), want)
    r = subprocess.run([S.SERVICE_BIN, "missing.yaml"], cwd=d, capture_output=True, text=True, timeout=60)
    assert r.returncode == 102
