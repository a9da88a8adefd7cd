"""A small, independent ZMTP 3.0 PUSH/PULL peer (NULL mechanism) for the host-loop tests.

Written from the ZMTP 3.0 specification separately from privacyamplification_gb300/csrc/pa_zmtp.cpp,
so that the two implementations check each other: greeting (FF 00*8 7F, version 3.0, "NULL"), READY
command with Socket-Type, frames with MORE / LONG / COMMAND flag bits.
"""
import socket
import struct
import time


def _recv_exact(sock, n):
    buf = bytearray()
    while len(buf) < n:
        chunk = sock.recv(n - len(buf))
        if not chunk:
            raise ConnectionError("peer closed")
        buf += chunk
    return bytes(buf)


class Peer:
    def __init__(self, kind, endpoint, bind, timeout=30.0):
        assert kind in ("PUSH", "PULL")
        host, port = endpoint[len("tcp://"):].rsplit(":", 1)
        self.kind, self.timeout = kind, timeout
        if bind:
            self._lsock = socket.socket(socket.AF_INET, socket.SOCK_STREAM)
            self._lsock.setsockopt(socket.SOL_SOCKET, socket.SO_REUSEADDR, 1)
            self._lsock.bind((host if host != "*" else "0.0.0.0", int(port)))
            self._lsock.listen(1)
            self._lsock.settimeout(timeout)
            self.sock = None
        else:
            self._lsock = None
            deadline = time.monotonic() + timeout
            while True:  # the bound side may not be listening yet
                try:
                    self.sock = socket.create_connection((host, int(port)), timeout=timeout)
                    break
                except ConnectionRefusedError:
                    if time.monotonic() > deadline:
                        raise
                    time.sleep(0.05)
            self._handshake()

    def accept(self):
        if self.sock is None:
            self.sock, _ = self._lsock.accept()
            self.sock.settimeout(self.timeout)
            self._handshake()

    def _handshake(self):
        greeting = b"\xff" + b"\x00" * 8 + b"\x7f" + bytes([3, 0]) + b"NULL".ljust(20, b"\x00") + b"\x00" + b"\x00" * 31
        assert len(greeting) == 64
        self.sock.sendall(greeting)
        g = _recv_exact(self.sock, 64)
        assert g[0] == 0xFF and g[9] & 1 and g[10] >= 3 and g[12:16] == b"NULL", g
        body = b"\x05READY" + bytes([11]) + b"Socket-Type" + struct.pack(">I", len(self.kind)) + self.kind.encode()
        self._send_frame(0x04, body)
        flags, body = self._recv_frame()
        assert flags & 0x04 and body[:6] == b"\x05READY", body
        props, i = {}, 6
        while i < len(body):
            nl = body[i]
            name = body[i + 1: i + 1 + nl].decode()
            (vl,) = struct.unpack(">I", body[i + 1 + nl: i + 5 + nl])
            props[name] = body[i + 5 + nl: i + 5 + nl + vl].decode()
            i += 5 + nl + vl
        assert props.get("Socket-Type") == ("PULL" if self.kind == "PUSH" else "PUSH"), props

    def _send_frame(self, flags, body):
        if len(body) > 255:
            self.sock.sendall(bytes([flags | 0x02]) + struct.pack(">Q", len(body)) + body)
        else:
            self.sock.sendall(bytes([flags, len(body)]) + body)

    def _recv_frame(self):
        flags = _recv_exact(self.sock, 1)[0]
        if flags & 0x02:
            (size,) = struct.unpack(">Q", _recv_exact(self.sock, 8))
        else:
            size = _recv_exact(self.sock, 1)[0]
        return flags, _recv_exact(self.sock, size)

    def send(self, *parts):
        """One message of one or more frames."""
        assert self.kind == "PUSH"
        self.accept()
        for i, p in enumerate(parts):
            self._send_frame(0x01 if i + 1 < len(parts) else 0x00, bytes(p))

    def recv(self):
        """One message: the list of its frames."""
        assert self.kind == "PULL"
        self.accept()
        parts = []
        while True:
            flags, body = self._recv_frame()
            if flags & 0x04:
                continue
            parts.append(body)
            if not flags & 0x01:
                return parts

    def close(self):
        for s in (self.sock, self._lsock):
            if s is not None:
                try:
                    s.close()
                except OSError:
                    pass


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port
