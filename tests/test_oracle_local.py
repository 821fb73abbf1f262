"""The oracle's restatement of RSSBase's local operators
(src/mpc/RSS.inl:168-345, functors.cuh:48-90) checked on the CPU through the
reconstruction algebra and slot-by-slot known answers."""
import numpy as np
import pytest

import oracle as orc


def _rec(a):
    return orc.reconstruct(a)


@pytest.mark.parametrize("op", ["add", "sub", "mul", "xor", "and", "shr", "shl"])
def test_rss_local_public_semantics(op):
    """Reconstruction algebra of RSSBase's local operators on a consistent
    sharing: public + - act once on the value, * & >> << on every share."""
    n = 257
    rng = np.random.default_rng(3)
    x = rng.integers(0, 2**64 - 1, n, dtype=np.uint64, endpoint=True)
    a = orc.share_random(x, seed=4)
    r = rng.integers(0, 70, n, dtype=np.uint64) if op in ("shr", "shl") else \
        rng.integers(0, 2**64 - 1, n, dtype=np.uint64, endpoint=True)
    out = orc.rss_local(op, a, r)
    rec = _rec(out)[0]
    with np.errstate(over="ignore"):
        if op == "add":
            assert np.array_equal(rec, x + r)
        elif op == "sub":
            assert np.array_equal(rec, x - r)
        elif op == "mul":
            assert np.array_equal(rec, x * r)
        else:
            # & ^ and shifts are share-wise: check every slot directly
            for p in range(3):
                for s in range(2):
                    v, w = a[p, s], out[p, s]
                    if op == "xor":
                        want = v ^ r if (p, s) in ((0, 0), (2, 1)) else v
                    elif op == "and":
                        want = v & r
                    elif op == "shl":
                        want = np.array([0 if int(k) >= 64 else (int(u) << int(k)) % 2**64 for u, k in zip(v, r)],
                                        dtype=np.uint64)
                    else:
                        want = np.array([(2**64 - 1 if int(u) >= 2**63 else 0) if int(k) >= 64 else
                                         ((int(u) - (2**64 if int(u) >= 2**63 else 0)) >> int(k)) % 2**64
                                         for u, k in zip(v, r)], dtype=np.uint64)
                    assert np.array_equal(w, want)


def test_rss_local_scalar_and_shares():
    n = 100
    rng = np.random.default_rng(5)
    x = rng.integers(0, 2**64 - 1, n, dtype=np.uint64, endpoint=True)
    y = rng.integers(0, 2**64 - 1, n, dtype=np.uint64, endpoint=True)
    a, b = orc.share_random(x, seed=6), orc.share_random(y, seed=7)
    with np.errstate(over="ignore"):
        assert np.array_equal(_rec(orc.rss_local("add", a, 12345))[0], x + np.uint64(12345))
        assert np.array_equal(_rec(orc.rss_local("add", a, b))[0], x + y)
        assert np.array_equal(_rec(orc.rss_local("sub", a, b))[0], x - y)
        assert np.array_equal(_rec(orc.rss_local("mul", a, 3))[0], x * np.uint64(3))


def test_tpc_fpc_local_public_add_reconstructs():
    rng = np.random.default_rng(9)
    n = 50
    x = rng.integers(0, 2**63, n, dtype=np.uint64)
    r = rng.integers(0, 2**63, n, dtype=np.uint64)
    t = orc.tpc_local("add", np.stack([x, np.zeros(n, np.uint64)]), r)  # party A holds the public value
    with np.errstate(over="ignore"):
        assert np.array_equal(t[0] + t[1], x + r)
    f = np.zeros((4, 3, n), dtype=np.uint64)
    f[1, 2] = f[2, 1] = f[3, 0] = x  # setPublic(x)
    g = orc.fpc_local("add", f, r)
    with np.errstate(over="ignore"):
        for p, s in ((1, 2), (2, 1), (3, 0)):
            assert np.array_equal(g[p, s], x + r)
        assert not g[0].any()


def test_empty_inputs_count_the_protocol_rounds():
    """Zero-length inputs: empty outputs, no bytes, and the rounds of the
    reference's call sequence on empty vectors (reconstruct 1, dReLU 1 + 12,
    ReLU 15); maxpool of no rows returns without dividing by the row count."""
    U64 = np.uint64
    e = np.zeros((3, 2, 0), dtype=U64)
    for fn, rounds in ((lambda c: orc.reconstruct(e, c), 1), (lambda c: orc.mul(e, e, c), 1),
                       (lambda c: orc.drelu(e, comm=c), 13), (lambda c: orc.relu(e, comm=c), 15)):
        c = orc.Comm()
        fn(c)
        assert c.rounds == rounds and c.tx == [0, 0, 0] and c.rx == [0, 0, 0]
    c = orc.Comm()
    out, d = orc.maxpool(e, 4, comm=c)
    assert out.shape[-1] == 0 and d.shape[-1] == 0 and c.tx == [0, 0, 0]
