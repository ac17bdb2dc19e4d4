"""The TCP renderer endpoint (nes_tcp_serve) on paths that never reach the
renderer, so no GPU is needed: a malformed FrameRequest and a length above
the request limit each close the connection (a failed parse makes neserver's
client reconnect, src/server.cpp:174-180), and a long-running endpoint joins
the threads of ended connections instead of holding them until shutdown."""
import ctypes
import socket
import struct
import time

import pytest


class _StandIn:
    """A zeroed buffer in place of a renderer context; the requests sent
    here are refused before the context is used."""

    def __init__(self):
        self.buf = ctypes.create_string_buffer(4096)
        self.h = ctypes.cast(self.buf, ctypes.c_void_p)


def _vm_kb():
    with open("/proc/self/status") as f:
        for line in f:
            if line.startswith("VmSize:"):
                return int(line.split()[1])
    pytest.skip("no /proc/self/status")


def _closed_after(port, payload):
    with socket.create_connection(("127.0.0.1", port), timeout=10) as s:
        s.sendall(payload)
        s.settimeout(10)
        try:
            return s.recv(1) == b""
        except ConnectionResetError:
            return True


def test_tcp_endpoint_closes_bad_requests_and_reaps_connections(nes_lib):
    bad = b"\x08"  # truncated varint
    malformed = struct.pack("=Q", len(bad)) + bad  # host-endian size_t length, as neserver sends it
    ep = nes_lib.TcpEndpoint(_StandIn())
    try:
        port = ep.port.value
        assert _closed_after(port, malformed)
        assert _closed_after(port, struct.pack("=Q", 1 << 21))  # above the 1 MiB request limit
        assert _closed_after(port, struct.pack("=Q", 0))  # empty request: no camera
        for _ in range(20):
            _closed_after(port, malformed)
        v0 = _vm_kb()
        for _ in range(200):
            assert _closed_after(port, malformed)
        time.sleep(0.3)
        grown_mb = (_vm_kb() - v0) / 1024
    finally:
        served = ep.close()
    assert served == 0
    # 200 ended connections whose threads were never joined would keep their
    # stacks mapped (8 MiB each by default): well over a gigabyte.
    assert grown_mb < 400, grown_mb  # allows a few malloc arenas of new threads (64 MiB each)
