"""The TCP party mode on the GPU: three party processes on localhost, each
with its own context on the one GPU and only its own share pair, run the
reference's RSS matmul (localMatMul, dividePublic3out3 with
reconstruct3out3 over the network), reconstruct and reshare. Every share
of every party equals the oracle's per-party views, the byte and round
counters follow the reference's accounting, and the end-of-step check
passes. The parties wait on one another only on the host (sockets); no
kernel waits on another process."""
import multiprocessing as mp
import os
import sys

import numpy as np
import pytest

import oracle as orc
from tests.test_party_transport import _free_base

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
U64 = np.uint64
CASES = [(64, 48, 96, 1, 1, 1, 26), (33, 70, 130, 0, 1, 0, 20)]


def _inputs():
    out = []
    for i, (M, N, K, tA, tB, tC, t) in enumerate(CASES):
        out.append((orc.random_views(M * K, U64, 10 + i), orc.random_views(K * N, U64, 20 + i)))
    return out, orc.random_views(300, U64, 30)[0, 0].copy()


def _party_proc(party, base, q):
    sys.path.insert(0, ROOT)
    try:
        import torch

        import piranha_gb300 as pg
        from piranha_gb300 import party as pm

        ins, c3 = _inputs()
        ctx = pg.Context(0)
        p = pm.Party(party, 3, base_port=base, timeout_ms=60000)
        res = {"party": party, "matmul": [], "reconstruct": []}
        dev = lambda x: torch.from_numpy(np.ascontiguousarray(x).view(np.int64)).cuda()  # noqa: E731
        for (M, N, K, tA, tB, tC, t), (a, b) in zip(CASES, ins):
            c = torch.empty((2, M * N), dtype=torch.int64, device="cuda")
            p.matmul(ctx, dev(a[party]), dev(b[party]), c, M, N, K, tA, tB, tC, t)
            rec = torch.empty(M * N, dtype=torch.int64, device="cuda")
            p.reconstruct(ctx, c, rec)
            ctx.sync()
            res["matmul"].append(c.cpu().numpy().view(U64))
            res["reconstruct"].append(rec.cpu().numpy().view(U64))
        out = torch.empty((2, 300), dtype=torch.int64, device="cuda")
        # a 3-out-of-3 share per party: party p's slice of a seeded vector
        p.reshare(ctx, dev(c3 + U64(party)), out)
        ctx.sync()
        res["reshare"] = out.cpu().numpy().view(U64)
        p.check()
        res["counters"] = p.counters()
        p.close()
        ctx.close()
        q.put(res)
    except Exception as e:  # reported to the test
        q.put({"party": party, "error": repr(e)})


@pytest.fixture(scope="module")
def results():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    base = _free_base(3)
    procs = [ctx.Process(target=_party_proc, args=(i, base, q)) for i in range(3)]
    for pr in procs:
        pr.start()
    res = {}
    for _ in procs:
        r = q.get(timeout=300)
        res[r["party"]] = r
    for pr in procs:
        pr.join(timeout=60)
    for r in res.values():
        assert "error" not in r, r
    return res


def test_party_matmul_and_reconstruct_equal_oracle(results):
    ins, _ = _inputs()
    for ci, ((M, N, K, tA, tB, tC, t), (a, b)) in enumerate(zip(CASES, ins)):
        want = orc.matmul(a, b, M, N, K, tA, tB, tC, t)
        rec = orc.reconstruct(want)
        for party in range(3):
            assert np.array_equal(results[party]["matmul"][ci], want[party]), (ci, party)
            assert np.array_equal(results[party]["reconstruct"][ci], rec[party]), (ci, party)


def test_party_reshare_equals_oracle(results):
    _, c3 = _inputs()
    cin = np.stack([c3 + U64(p) for p in range(3)])
    want = orc.reshare(cin)
    for party in range(3):
        assert np.array_equal(results[party]["reshare"], want[party])


def test_party_counters_follow_the_reference_accounting(results):
    per = [M * N * 8 for (M, N, *_rest) in CASES]
    for party in range(3):
        nxt, prv = (party + 1) % 3, (party + 2) % 3
        c = results[party]["counters"]
        # matmul: reconstruct3out3 sends M*N to both neighbours; reconstruct: M*N to
        # the next party; reshare: 300 values to the previous one
        assert c["tx"][nxt] == sum(per) + sum(per) and c["tx"][prv] == sum(per) + 300 * 8
        assert c["rx"][prv] == sum(per) + sum(per) and c["rx"][nxt] == sum(per) + 300 * 8
        assert c["rounds"] == 2 * len(CASES) + 1
