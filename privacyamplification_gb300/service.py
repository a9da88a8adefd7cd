"""ctypes binding of include/pa_service.h: config.yaml surface, host loop, SHA3-256, ZMTP sockets.

The loop itself is native (pa_service.cpp); `pa_service` next to this file is the executable form
(`pa_service [config.yaml] [--blocks K]`).
"""
from __future__ import annotations

import ctypes
import os

from . import HERE as _HERE, load_library

SERVICE_EXPORTS = ("pa_service_config_default", "pa_service_config_load", "pa_service_run", "pa_sha3_256",
                   "pa_zmq_open", "pa_zmq_recv", "pa_zmq_send", "pa_zmq_close")
SERVICE_BIN = os.path.join(_HERE, "pa_service")
ZMQ_PULL, ZMQ_PUSH = 7, 8


class ServiceConfig(ctypes.Structure):
    """pa_service_config: the reference's config.yaml keys (strings as bytes)."""
    _fields_ = [("factor_exp", ctypes.c_uint32), ("reuse_seed_amount", ctypes.c_int32),
                ("vertical_len", ctypes.c_uint32), ("do_xor_key_rest", ctypes.c_int32),
                ("do_compress", ctypes.c_int32), ("reduction_exp", ctypes.c_uint32),
                ("pre_mul_reduction_exp", ctypes.c_uint32), ("gpu_device_id_to_use", ctypes.c_int32),
                ("input_blocks_to_cache", ctypes.c_uint32), ("output_blocks_to_cache", ctypes.c_uint32),
                ("show_ampout", ctypes.c_int32), ("show_zeromq_status", ctypes.c_int32),
                ("use_matrix_seed_server", ctypes.c_int32), ("address_seed_in", ctypes.c_char * 256),
                ("toeplitz_seed_path", ctypes.c_char * 1024), ("use_key_server", ctypes.c_int32),
                ("address_key_in", ctypes.c_char * 256), ("keyfile_path", ctypes.c_char * 1024),
                ("host_ampout_server", ctypes.c_int32), ("address_amp_out", ctypes.c_char * 256),
                ("store_first_ampouts_in_file", ctypes.c_int32), ("verify_ampout", ctypes.c_int32),
                ("verify_ampout_threads", ctypes.c_uint32), ("ampout_sha3_path", ctypes.c_char * 1024),
                ("ampout_path", ctypes.c_char * 1024)]


_bound = False


def _lib():
    global _bound
    lib = load_library()
    if not _bound:
        vp = ctypes.c_void_p
        sig = {
            "pa_service_config_default": ([ctypes.POINTER(ServiceConfig)], None),
            "pa_service_config_load": ([ctypes.c_char_p, ctypes.POINTER(ServiceConfig)], ctypes.c_int),
            "pa_service_run": ([ctypes.POINTER(ServiceConfig), ctypes.c_int64], ctypes.c_int),
            "pa_sha3_256": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint8)], None),
            "pa_zmq_open": ([ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(vp)], ctypes.c_int),
            "pa_zmq_recv": ([vp, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_int)], ctypes.c_int64),
            "pa_zmq_send": ([vp, vp, ctypes.c_size_t, ctypes.c_int], ctypes.c_int),
            "pa_zmq_close": ([vp], None),
        }
        for name, (args, res) in sig.items():
            fn = getattr(lib, name)
            fn.argtypes, fn.restype = args, res
        _bound = True
    return lib


def default_config(**overrides) -> ServiceConfig:
    cfg = ServiceConfig()
    _lib().pa_service_config_default(ctypes.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v.encode() if isinstance(v, str) else v)
    return cfg


def load_config(path: str) -> ServiceConfig:
    cfg = default_config()
    rc = _lib().pa_service_config_load(path.encode(), ctypes.byref(cfg))
    if rc:
        raise OSError(rc, "cannot read %s" % path)
    return cfg


def run(cfg: ServiceConfig, max_blocks: int = -1) -> int:
    """Runs the host loop (blocking; releases the GIL); returns its exit code."""
    return int(_lib().pa_service_run(ctypes.byref(cfg), max_blocks))


def sha3_256(data) -> bytes:
    buf = bytes(data)
    out = (ctypes.c_uint8 * 32)()
    _lib().pa_sha3_256(buf, len(buf), out)
    return bytes(out)


class Socket:
    """pa_zmq_* socket: ZMTP 3.0 PUSH or PULL, one peer."""

    def __init__(self, kind: int, endpoint: str, bind: bool):
        self._lib = _lib()
        h = ctypes.c_void_p()
        rc = self._lib.pa_zmq_open(kind, endpoint.encode(), int(bind), ctypes.byref(h))
        if rc:
            raise ValueError("pa_zmq_open(%s) failed: %d" % (endpoint, rc))
        self._h = h

    def send(self, data: bytes, more: bool = False) -> int:
        buf = bytes(data)
        return int(self._lib.pa_zmq_send(self._h, buf, len(buf), int(more)))

    def recv(self, cap: int):
        """(frame bytes, size on the wire, more); size < 0 on error."""
        buf = ctypes.create_string_buffer(max(1, cap))
        more = ctypes.c_int()
        n = int(self._lib.pa_zmq_recv(self._h, buf, cap, ctypes.byref(more)))
        return buf.raw[: max(0, min(n, cap))], n, bool(more.value)

    def close(self):
        if self._h:
            self._lib.pa_zmq_close(self._h)
            self._h = None
