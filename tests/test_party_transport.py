"""The TCP party mode's transport on the CPU: three (or two) party processes
on localhost, messages in the reference's wire format, and host-side fault
injection. No call here touches a GPU.

* a ring of messages arrives intact, the reference's byte accounting holds
  and the end-of-step check passes;
* a dropped message makes the receiver's bounded wait run out
  (PG_ERR_TIMEOUT), a truncated one too, a duplicated one is caught by the
  end-of-step check (PG_ERR_COMM), and a peer that leaves mid-protocol is a
  PG_ERR_COMM at the party waiting for it; a party whose peers never come
  up gives up with PG_ERR_TIMEOUT;
* wire compatibility: a peer written here from the reference's socket code
  (listen on base + sender * n + receiver, three connections per ordered
  pair, raw bytes with no header) exchanges messages with a Party.
"""
import multiprocessing as mp
import os
import random
import socket
import sys
import time

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PG_ERR_TIMEOUT, PG_ERR_COMM = 5, 7


def _free_base(n):
    """A base port whose n * n ports are free now."""
    for _ in range(200):
        base = random.randint(20000, 60000 - n * n)
        socks = []
        try:
            for k in range(n * n):
                s = socket.socket()
                s.setsockopt(socket.SOL_SOCKET, socket.SO_REUSEADDR, 1)
                s.bind(("127.0.0.1", base + k))
                socks.append(s)
            return base
        except OSError:
            continue
        finally:
            for s in socks:
                s.close()
    raise RuntimeError("no free ports")


def _party_main(party, n, base, timeout_ms, script, q):
    sys.path.insert(0, ROOT)
    from piranha_gb300 import party as pm

    out = {"party": party}
    try:
        p = pm.Party(party, n, base_port=base, timeout_ms=timeout_ms)
    except pm.PartyError as e:
        q.put({"party": party, "create": e.status})
        return
    try:
        script(pm, p, party, n, out)
    except pm.PartyError as e:
        out["error"] = e.status
        out["msg"] = str(e)
    if p._h:
        out["counters"] = p.counters()
        p.close()
    q.put(out)


def _run(script, n=3, timeout_ms=3000, parties=None):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    base = _free_base(n)
    procs = [ctx.Process(target=_party_main, args=(i, n, base, timeout_ms, script, q))
             for i in (parties if parties is not None else range(n))]
    for pr in procs:
        pr.start()
    res = {}
    for _ in procs:
        r = q.get(timeout=60)
        res[r["party"]] = r
    for pr in procs:
        pr.join(timeout=30)
    return res


def _payload(party, size=1000):
    return (np.arange(size, dtype=np.uint64) * np.uint64(2654435761) + np.uint64(party * 7919 + 1)).astype(np.uint64)


# scripts run in the party processes (module-level, picklable by name)

def ring(pm, p, party, n, out, fault=None):
    nxt, prv = (party + 1) % n, (party + n - 1) % n
    if fault and party == 0:
        p.inject(fault, 1)
    # the lower-numbered of each pair sends first (the host API blocks on each call)
    if party == 0:
        p.send(nxt, _payload(party))
        if fault in (1, 3):
            time.sleep(3.0)  # stay connected while the receiver's wait runs out
        got = p.recv(prv, _payload(0))
    else:
        got = p.recv(prv, _payload(0))
        p.send(nxt, _payload(party))
    out["ok"] = bool(np.array_equal(got, _payload(prv)))
    p.check()
    out["checked"] = True


def ring_drop(pm, p, party, n, out):
    ring(pm, p, party, n, out, fault=1)


def ring_duplicate(pm, p, party, n, out):
    ring(pm, p, party, n, out, fault=2)


def ring_truncate(pm, p, party, n, out):
    ring(pm, p, party, n, out, fault=3)


def leave_early(pm, p, party, n, out):
    if party == 0:
        p.close()  # leaves without sending its message
        return
    out["got"] = p.recv(0, _payload(0)).tolist()[:1]


def test_ring_messages_counters_and_check():
    res = _run(ring)
    for i in range(3):
        r = res[i]
        assert r.get("ok") and r.get("checked"), r
        nxt, prv = (i + 1) % 3, (i + 2) % 3
        assert r["counters"]["tx"][nxt] == 8000 and r["counters"]["rx"][prv] == 8000
        assert sum(r["counters"]["tx"]) == 8000 and sum(r["counters"]["rx"]) == 8000


def test_dropped_message_times_out_at_the_receiver():
    res = _run(ring_drop, timeout_ms=1500)
    assert res[1].get("error") == PG_ERR_TIMEOUT, res[1]
    assert "stopped after 0 of 8000 bytes" in res[1]["msg"]


def test_truncated_message_times_out_at_the_receiver():
    res = _run(ring_truncate, timeout_ms=1500)
    assert res[1].get("error") == PG_ERR_TIMEOUT, res[1]
    assert "stopped after 4000 of 8000 bytes" in res[1]["msg"]


def test_duplicated_message_is_caught_by_the_check():
    res = _run(ring_duplicate, timeout_ms=3000)
    assert res[1].get("ok") is True  # the first copy arrives as the message
    assert res[1].get("error") == PG_ERR_COMM, res[1]
    assert "unexpected bytes from party 0" in res[1]["msg"]


def test_peer_that_leaves_is_a_communication_error():
    res = _run(leave_early, n=2, timeout_ms=5000)
    assert res[1].get("error") == PG_ERR_COMM, res[1]
    assert "closed the connection" in res[1]["msg"]


def test_party_without_peers_gives_up():
    res = _run(ring, n=3, timeout_ms=500, parties=[0])
    assert res[0].get("create") == PG_ERR_TIMEOUT, res[0]


def _reference_style_peer(base, n, me, peer, payload, want, q):
    """Party `me` of n as the reference's BmrNet sets it up for one peer with a
    lower number: connect first (to base + me * n + peer, three connections),
    then listen on base + peer * n + me and accept three; a message is the raw
    bytes on the first connection."""
    try:
        send = []
        deadline = time.time() + 10
        for _ in range(3):
            while True:
                s = socket.socket()
                s.setsockopt(socket.IPPROTO_TCP, socket.TCP_NODELAY, 1)
                try:
                    s.connect(("127.0.0.1", base + me * n + peer))
                    break
                except OSError:
                    s.close()
                    if time.time() > deadline:
                        raise
                    time.sleep(0.02)
            send.append(s)
        srv = socket.socket()
        srv.setsockopt(socket.SOL_SOCKET, socket.SO_REUSEADDR, 1)
        srv.bind(("0.0.0.0", base + peer * n + me))
        srv.listen(10)
        srv.settimeout(10)
        recv = [srv.accept()[0] for _ in range(3)]
        srv.close()
        buf = b""
        recv[0].settimeout(10)
        while len(buf) < want:
            chunk = recv[0].recv(want - len(buf))
            if not chunk:
                break
            buf += chunk
        send[0].sendall(payload.tobytes())
        q.put(buf)
        time.sleep(0.5)
        for s in send + recv:
            s.close()
    except Exception as e:  # reported to the test
        q.put(repr(e))


def _wire_party0(pm, p, party, n, out):
    p.send(1, _payload(0, 513))
    out["got"] = p.recv(1, _payload(1, 77)).tolist()


def test_wire_format_matches_the_reference_sockets():
    ctx = mp.get_context("spawn")
    q, q2 = ctx.Queue(), ctx.Queue()
    base = _free_base(2)
    peer = ctx.Process(target=_reference_style_peer, args=(base, 2, 1, 0, _payload(1, 77), 513 * 8, q2))
    p0 = ctx.Process(target=_party_main, args=(0, 2, base, 10000, _wire_party0, q))
    peer.start()
    p0.start()
    got_by_peer = q2.get(timeout=60)
    res = q.get(timeout=60)
    p0.join(timeout=30)
    peer.join(timeout=30)
    assert isinstance(got_by_peer, bytes), got_by_peer
    assert got_by_peer == _payload(0, 513).tobytes()  # raw bytes, no header
    assert res.get("got") == _payload(1, 77).tolist(), res
