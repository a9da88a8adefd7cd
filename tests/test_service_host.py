"""Host loop pieces that need no GPU: SHA3-256, the config.yaml reader, ZMTP 3.0 sockets (C++ against
C++ and against the independent Python peer in zmtp_peer.py), and the exported symbols of pa_service.h."""
import hashlib
import os
import re
import threading

import numpy as np
import pytest

from privacyamplification_gb300 import service as S
from zmtp_peer import Peer, free_port

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_service_header_matches_binding(pa_lib):
    text = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "pa_service.h")).read(), flags=re.S)
    declared = sorted(set(re.findall(r"\b(pa_[a-z0-9_]+)\s*\(", text)))
    assert declared == sorted(S.SERVICE_EXPORTS)
    for name in declared:
        assert hasattr(pa_lib, name), name
    assert os.access(S.SERVICE_BIN, os.X_OK)


@pytest.mark.parametrize("size", [0, 1, 135, 136, 137, 272, 1000, 1 << 20])
def test_sha3_256_matches_hashlib(pa_lib, size):
    data = np.random.default_rng(size).integers(0, 256, size, dtype=np.uint8).tobytes()
    assert S.sha3_256(data) == hashlib.sha3_256(data).digest()


def test_config_reader(pa_lib, tmp_path):
    p = tmp_path / "config.yaml"
    p.write_text(
        "# privacy amplification settings\n"
        "factor_exp: 16\n"
        "reuse_seed_amount: -1   # keep the seed\n"
        "vertical_len: 24576\n"
        "do_xor_key_rest: false\n"
        "do_compress: True\n"
        "show_ampout: -1\n"
        "use_matrix_seed_server: no\n"
        "address_seed_in: 'tcp://127.0.0.1:45999'\n"
        "toeplitz_seed_path: \"seed # not a comment.bin\"\n"
        "store_first_ampouts_in_file: true\n"
        "unknown_key: 5\n")
    cfg = S.load_config(str(p))
    assert cfg.factor_exp == 16 and cfg.reuse_seed_amount == -1 and cfg.vertical_len == 24576
    assert cfg.do_xor_key_rest == 0 and cfg.do_compress == 1 and cfg.show_ampout == -1
    assert cfg.use_matrix_seed_server == 0 and cfg.use_key_server == 1  # default kept
    assert cfg.address_seed_in == b"tcp://127.0.0.1:45999"
    assert cfg.toeplitz_seed_path == b"seed # not a comment.bin"
    assert cfg.store_first_ampouts_in_file == 1
    assert cfg.address_amp_out == b"tcp://127.0.0.1:48888"  # default
    with pytest.raises(OSError) as ei:
        S.load_config(str(tmp_path / "missing.yaml"))
    assert ei.value.errno == 102


def run_bg(fn, *args):
    out = {}
    t = threading.Thread(target=lambda: out.setdefault("r", fn(*args)), daemon=True)
    t.start()
    return t, out


def test_zmtp_cpp_push_to_python_pull(pa_lib):
    ep = "tcp://127.0.0.1:%d" % free_port()
    push = S.Socket(S.ZMQ_PUSH, ep, bind=True)
    payload = np.random.default_rng(1).integers(0, 256, 70000, dtype=np.uint8).tobytes()
    t, res = run_bg(lambda: (push.send(b"\x01", more=True), push.send(payload)))
    peer = Peer("PULL", ep, bind=False)
    try:
        assert peer.recv() == [b"\x01", payload]
    finally:
        t.join(10)
        peer.close()
        push.close()
    assert res["r"] == (0, 0)


def test_zmtp_python_push_to_cpp_pull(pa_lib):
    ep = "tcp://127.0.0.1:%d" % free_port()
    peer = Peer("PUSH", ep, bind=True)
    pull = S.Socket(S.ZMQ_PULL, ep, bind=False)
    seed = np.arange(2048, dtype=np.uint32).tobytes()
    t = threading.Thread(target=lambda: peer.send(np.int32(3).tobytes(), seed), daemon=True)
    t.start()
    try:
        a, na, more_a = pull.recv(4)
        b, nb, more_b = pull.recv(len(seed))
        assert (a, na, more_a) == (np.int32(3).tobytes(), 4, True)
        assert (b, nb, more_b) == (seed, len(seed), False)
    finally:
        t.join(10)
        pull.close()
        peer.close()


def test_zmtp_cpp_to_cpp_multipart_and_truncation(pa_lib):
    ep = "tcp://127.0.0.1:%d" % free_port()
    push = S.Socket(S.ZMQ_PUSH, ep, bind=True)
    pull = S.Socket(S.ZMQ_PULL, ep, bind=False)
    t, _ = run_bg(lambda: [push.send(bytes([i]) * (300 * i + 1), more=i < 3) for i in range(4)])
    try:
        for i in range(4):
            data, n, more = pull.recv(16)
            assert n == 300 * i + 1 and data == bytes([i]) * min(16, n) and more == (i < 3)
    finally:
        t.join(10)
        pull.close()
        push.close()


def test_zmtp_rejects_wrong_socket_type(pa_lib):
    """A PUSH peer talking to a PUSH socket fails the READY check; the C++ side keeps waiting for a
    proper peer instead of accepting the data."""
    ep = "tcp://127.0.0.1:%d" % free_port()
    pull = S.Socket(S.ZMQ_PULL, ep, bind=False)
    bad = Peer("PULL", ep, bind=True, timeout=5)  # a PULL server: wrong partner for a PULL client
    with pytest.raises((AssertionError, ConnectionError, OSError)):
        bad.accept()
    bad.close()
    good = Peer("PUSH", ep, bind=True)
    t = threading.Thread(target=lambda: good.send(b"ok"), daemon=True)
    t.start()
    try:
        assert pull.recv(8)[:2] == (b"ok", 2)
    finally:
        t.join(10)
        pull.close()
        good.close()
