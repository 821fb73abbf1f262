"""Party mode: one RSS party per process, messages over TCP in the
reference's wire format (``pg_party_*`` of the C ABI).

The reference runs one process per party (``./piranha -p <party>``) and
connects them with ``initializeCommunication`` (src/util/connect.cu:109-123):
for every ordered pair the receiver listens on ``base + sender * n +
receiver`` (base 32000), three TCP connections per pair, a message being the
raw bytes of the vector on the first. ``Party`` sets up the same connections
and sends the same bytes, so a reference party can be a peer; every wait is
bounded and every failure is a ``PartyError`` with the library's status.

A party holds only its own share pair: an RSS tensor of n elements is a
(2, n) int64 CUDA tensor, [shareA, shareB] (src/mpc/RSS.h:74-75).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import PiranhaError, lib

PG_ERR_TIMEOUT = 5
PG_ERR_COMM = 7
FAULT_NONE, FAULT_DROP, FAULT_DUPLICATE, FAULT_TRUNCATE = 0, 1, 2, 3
REFERENCE_BASE_PORT = 32000


class PartyError(PiranhaError):
    def __init__(self, status, msg):
        super().__init__(f"party status {status}: {msg}")
        self.status = status


class Party:
    """This process's party ``party`` of ``num_parties``; ``hosts[i]`` is
    party i's address. ``timeout_ms`` bounds every wait (connection set-up
    included)."""

    def __init__(self, party: int, num_parties: int = 3, hosts=None, base_port: int = REFERENCE_BASE_PORT,
                 timeout_ms: int = 10000):
        hosts = hosts or ["127.0.0.1"] * num_parties
        arr = (ctypes.c_char_p * num_parties)(*[h.encode() for h in hosts])
        self._h = ctypes.c_void_p()
        self.party, self.n = party, num_parties
        st = lib().pg_party_create(ctypes.byref(self._h), party, num_parties, ctypes.cast(arr, ctypes.c_void_p),
                                   base_port, timeout_ms)
        if st:
            raise PartyError(st, lib().pg_party_last_error(None).decode())

    def _check(self, st):
        if st:
            raise PartyError(st, lib().pg_party_last_error(self._h).decode())

    def close(self):
        if self._h:
            lib().pg_party_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --------------------------------------------------------- transport
    def send(self, to: int, data: np.ndarray):
        """sendVector (connect.h:41-47): the array's raw bytes."""
        a = np.ascontiguousarray(data)
        self._check(lib().pg_party_send(self._h, to, a.ctypes.data_as(ctypes.c_void_p), a.nbytes))

    def recv(self, frm: int, like: np.ndarray) -> np.ndarray:
        """receiveVector (connect.h:49-55) into an array shaped like ``like``."""
        out = np.empty_like(like)
        self._check(lib().pg_party_recv(self._h, frm, out.ctypes.data_as(ctypes.c_void_p), out.nbytes))
        return out

    def exchange(self, ctx, to, dev_out, frm, dev_in):
        """DeviceData::transmit(to) of one CUDA tensor while receiving another
        from ``frm`` (either may be None)."""
        self._check(lib().pg_party_exchange(
            self._h, ctx.handle, -1 if to is None else to,
            ctypes.c_void_p(dev_out.data_ptr()) if dev_out is not None else None,
            dev_out.numel() * dev_out.element_size() if dev_out is not None else 0,
            -1 if frm is None else frm,
            ctypes.c_void_p(dev_in.data_ptr()) if dev_in is not None else None,
            dev_in.numel() * dev_in.element_size() if dev_in is not None else 0))

    def counters(self) -> dict:
        buf = (ctypes.c_uint64 * (2 * self.n + 1))()
        self._check(lib().pg_party_counters(self._h, buf))
        return {"tx": list(buf[:self.n]), "rx": list(buf[self.n:2 * self.n]), "rounds": buf[2 * self.n]}

    def check(self):
        """Swap byte counters with every peer and look for unread bytes:
        PartyError(PG_ERR_COMM) when a message was lost, duplicated or cut."""
        self._check(lib().pg_party_check(self._h))

    def inject(self, kind: int, nth: int = 1):
        """Host-side fault injection: the nth send from now is dropped,
        duplicated or truncated (FAULT_NONE clears it)."""
        self._check(lib().pg_party_inject(self._h, kind, nth))

    # ------------------------------------------------------ protocol steps
    @staticmethod
    def _p2(t):
        return (ctypes.c_void_p * 2)(t[0].data_ptr(), t[1].data_ptr())

    def reconstruct(self, ctx, shares, out):
        """reconstruct (RSS.inl:457-479) of this party's (2, n) shares into out (n,)."""
        self._check(lib().pg_party_rss_reconstruct_u64(self._h, ctx.handle, self._p2(shares), shares.shape[1],
                                                       ctypes.c_void_p(out.data_ptr())))
        return out

    def reshare(self, ctx, c, out):
        """reshare (RSS.inl:1052-1074) of this party's 3-out-of-3 share c (n,) into out (2, n)."""
        self._check(lib().pg_party_rss_reshare_u64(self._h, ctx.handle, ctypes.c_void_p(c.data_ptr()), c.numel(),
                                                   self._p2(out)))
        return out

    def matmul(self, ctx, a, b, c, M, N, K, transpose_a, transpose_b, transpose_c, truncation):
        """matmul (RSS.inl:481-540) of this party's shares: localMatMul,
        dividePublic3out3 with reconstruct3out3 over the network."""
        self._check(lib().pg_party_rss_matmul_u64(self._h, ctx.handle, self._p2(a), self._p2(b), self._p2(c), M, N, K,
                                                  int(transpose_a), int(transpose_b), int(transpose_c),
                                                  int(truncation)))
        return c
