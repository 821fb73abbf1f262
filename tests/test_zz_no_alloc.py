"""pg_rss_matmul_u64_noalloc (the limb-form share-GEMM whose scratch is one
fixed device array) against pg_rss_matmul_u64, bit for bit, through the C ABI.

The file name sorts last, so in a full run these calls come after every other
test has used the library in the same process; it passes on its own as well.
"""
import ctypes

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

U64 = np.uint64
P6 = ctypes.c_void_p * 6
PG_ERR_SIZE = 2


@pytest.fixture(scope="module")
def pg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    fn = pg.lib().pg_rss_matmul_u64_noalloc
    fn.argtypes = [ctypes.c_void_p, P6, P6, P6] + [ctypes.c_int] * 7
    fn.restype = ctypes.c_int
    return pg


@pytest.fixture()
def ctx(pg):
    c = pg.Context(0, form=pg.FORM_LIMB_TC)
    yield c
    c.check_device_errors()
    c.close()


def _p6(t):
    return P6(*[t[p, s].data_ptr() for p in range(3) for s in range(2)])


def _noalloc(pg, ctx, a, b, c, M, N, K, tA, tB, tC, trunc):
    return pg.lib().pg_rss_matmul_u64_noalloc(ctx.handle, _p6(a), _p6(b), _p6(c), M, N, K, tA, tB, tC, trunc)


CASES = [
    (256, 192, 512, 1, 1, 1, 26),   # several tiles, one K' slice per tile
    (64, 128, 1024, 1, 0, 1, 20),   # few tiles: split-K with partial sums
]


def test_noalloc_matches_regular_two_calls(pg, ctx):
    import torch

    ins, want = [], []
    for i, (M, N, K, tA, tB, tC, t) in enumerate(CASES):
        a = orc.random_views(M * K, U64, 100 + i)
        b = orc.random_views(K * N, U64, 200 + i)
        da, db = pg.to_device(a), pg.to_device(b)
        ref = pg.empty_shares(M * N)
        pg.matmul(ctx, da, db, ref, M, N, K, tA, tB, tC, t)
        ins.append((da, db))
        want.append(pg.to_host(ref))
        if i == 0:
            assert np.array_equal(want[0], orc.matmul(a, b, M, N, K, tA, tB, tC, t))
    outs = [pg.empty_shares(M * N) for (M, N, *_) in CASES]
    # set-up call (the first on this device in a fresh process): loads the
    # module that holds the fixed scratch
    (M, N, K, tA, tB, tC, t), (da, db) = CASES[0], ins[0]
    ctx._check(_noalloc(pg, ctx, da, db, outs[0], M, N, K, tA, tB, tC, t))
    ctx.sync()
    comm0 = ctx.comm()
    free0 = torch.cuda.mem_get_info()[0]
    # two calls in a row on one stream: the second reuses the scratch the first just used
    for (M, N, K, tA, tB, tC, t), (da, db), out in zip(CASES, ins, outs):
        ctx._check(_noalloc(pg, ctx, da, db, out, M, N, K, tA, tB, tC, t))
    ctx.check_device_errors()
    for got, w in zip(outs, want):
        assert np.array_equal(pg.to_host(got), w)
    comm1 = ctx.comm()
    per = [2 * M * N * 8 for (M, N, *_) in CASES]
    assert [x - y for x, y in zip(comm1["tx"], comm0["tx"])] == [sum(per)] * 3
    assert comm1["rounds"] - comm0["rounds"] == 2
    # after the set-up of the first call, a call reserves no device memory
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_repeat_is_stable(pg, ctx):
    M, N, K, tA, tB, tC, t = CASES[1]
    a, b = orc.random_views(M * K, U64, 7), orc.random_views(K * N, U64, 8)
    want = orc.matmul(a, b, M, N, K, tA, tB, tC, t)
    da, db = pg.to_device(a), pg.to_device(b)
    for _ in range(2):
        out = pg.zeros_shares(M * N)
        ctx._check(_noalloc(pg, ctx, da, db, out, M, N, K, tA, tB, tC, t))
        ctx.check_device_errors()
        assert np.array_equal(pg.to_host(out), want)


def test_noalloc_refuses_what_does_not_fit(pg, ctx):
    # sizes are checked before any device memory is touched, so small buffers do
    d = pg.zeros_shares(16)
    st = _noalloc(pg, ctx, d, d, d, 4096, 4096, 4096, 1, 1, 1, 26)
    assert st == PG_ERR_SIZE
    msg = pg.lib().pg_last_error(ctx.handle)
    msg = msg.decode() if isinstance(msg, bytes) else str(msg)
    assert "fixed scratch" in msg


def test_noalloc_any_k(pg, ctx):
    # K not a multiple of 16: zero digits pad the contraction
    M, N, K = 40, 24, 25
    a, b = orc.random_views(M * K, U64, 11), orc.random_views(K * N, U64, 12)
    out = pg.zeros_shares(M * N)
    ctx._check(_noalloc(pg, ctx, pg.to_device(a), pg.to_device(b), out, M, N, K, 1, 1, 1, 20))
    ctx.check_device_errors()
    assert np.array_equal(pg.to_host(out), orc.matmul(a, b, M, N, K, 1, 1, 1, 20))
