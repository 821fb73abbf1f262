"""The device AES counter-mode generator and the live resharing masks against
the oracle: the uint64 stream of AESObject from any counter, and reshare /
*= / &= with pairwise keys, which equal the unmasked steps plus zero-sum masks
(so reconstructions are unchanged) and advance the context's counter."""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

U8, U64 = np.uint8, np.uint64
KEYS = [bytes([17 * p + i for i in range(32)]) for p in range(3)]


@pytest.fixture(scope="module")
def pg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    pg.lib()
    return pg


@pytest.fixture()
def ctx(pg):
    c = pg.Context(0)
    yield c
    c.close()


def _dev(a):
    import torch

    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(np.int64 if a.dtype == U64 else np.uint8)).cuda()


def _host(t):
    a = t.cpu().numpy()
    return a.view(U64) if a.dtype == np.int64 else a


@pytest.mark.parametrize("counter,n", [(0, 1), (0, 2), (7, 1001), (2**33 + 5, 4096)])
def test_prg_fill_matches_oracle(pg, ctx, counter, n):
    import torch

    key = bytes(range(100, 132))
    out = torch.empty(n, dtype=torch.int64, device="cuda")
    ctx.prg_fill(key, counter, out)
    ctx.sync()
    assert np.array_equal(_host(out), orc.prg_fill_u64(key, counter, n))


def _masked(base, alpha, xor):
    """shares (3, 2, n) of a reshared value plus the masks: party p's pair is (z_p + a_p, z_p+1 + a_p+1)."""
    out = base.copy()
    with np.errstate(over="ignore"):
        for p in range(3):
            for s, q in ((0, p), (1, (p + 1) % 3)):
                out[p, s] = (out[p, s] ^ alpha[q]) if xor else (out[p, s] + alpha[q])
    return out.astype(base.dtype)


@pytest.mark.parametrize("n", [1, 999, 65537])
def test_masked_reshare_mul_and(pg, ctx, n):
    import torch

    c0 = 11
    ctx.set_prg_keys(KEYS, c0)
    blocks = (n + 1) // 2
    c3 = np.random.default_rng(n).integers(0, 2**64 - 1, (3, n), dtype=U64, endpoint=True)
    out = pg.empty_shares(n)
    pg.reshare(ctx, torch.from_numpy(c3.view(np.int64)).cuda(), out)
    want = _masked(orc.reshare(c3), orc.prg_masks(KEYS, c0, n), False)
    assert np.array_equal(_host(out), want)
    assert np.array_equal(orc.reconstruct(_host(out)), orc.reconstruct(orc.reshare(c3)))
    assert ctx.prg_counter() == c0 + blocks

    a, b = orc.random_views(n, U64, 40), orc.random_views(n, U64, 41)
    da = _dev(a)
    pg.mul_(ctx, da, _dev(b))
    want = _masked(orc.mul(a, b), orc.prg_masks(KEYS, c0 + blocks, n), False)
    assert np.array_equal(_host(da), want)
    da = _dev(a)
    pg.and_(ctx, da, _dev(b))
    want = _masked(orc.and_(a, b), orc.prg_masks(KEYS, c0 + 2 * blocks, n, xor=True), True)
    assert np.array_equal(_host(da), want)

    ab = (orc.random_views(n, U64, 42) & U64(1)).astype(U8)
    bb = (orc.random_views(n, U64, 43) & U64(1)).astype(U8)
    db = _dev(ab)
    pg.and_(ctx, db, _dev(bb))
    z = [(ab[p, 0] & (bb[p, 0] ^ bb[p, 1])) ^ (ab[p, 1] & bb[p, 0]) for p in range(3)]  # RSS.inl:331-345
    base = np.stack([np.stack([z[p], z[(p + 1) % 3]]) for p in range(3)]).astype(U8)
    want = _masked(base, orc.prg_masks(KEYS, c0 + 3 * blocks, n, xor=True, bits=True).astype(U8), True)
    got = _host(db)
    assert np.array_equal(got, want) and set(np.unique(got)) <= {0, 1}
    assert ctx.prg_counter() == c0 + 4 * blocks

    # off again: the reference's unfilled masks
    ctx.set_prg_keys(None)
    da = _dev(a)
    pg.mul_(ctx, da, _dev(b))
    assert np.array_equal(_host(da), orc.mul(a, b))
