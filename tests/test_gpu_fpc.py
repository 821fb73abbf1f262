"""FPC (4PC) entry points against the CPU oracle's restatement of src/mpc/FPC.inl.

All twelve arrays (four parties x three shares) must match bit for bit, and
the communication counters must equal the bytes and rounds of the
reference's reconstructs and reshares. Inputs are either consistent 4-party
sharings or arbitrary views (parties that disagree), which the reference
processes party by party all the same.
"""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

U64, U32, U8 = np.uint64, np.uint32, np.uint8
_VIEW = {np.dtype(U64): np.int64, np.dtype(U32): np.int32, np.dtype(U8): np.uint8}
_BACK = {np.int64: U64, np.int32: U32, np.uint8: U8}


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


def dev(a):
    import torch

    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(_VIEW[a.dtype])).cuda()


def host(t):
    a = t.cpu().numpy()
    return a.view(_BACK[a.dtype.type])


def views(n, dt, seed):
    """Arbitrary (inconsistent) views: every party's every share random."""
    rng = np.random.default_rng(seed)
    return rng.integers(0, np.iinfo(dt).max, (4, 3, n), dtype=dt, endpoint=True)


def check_comm(ctx, comm):
    cc = ctx.comm(4)
    assert cc["tx"] == comm.tx and cc["rx"] == comm.rx and cc["rounds"] == comm.rounds, (cc, comm.tx, comm.rx)


@pytest.mark.parametrize("dt", [U64, U32])
@pytest.mark.parametrize("M,N,K,tA,tB,tC", [(5, 7, 9, 1, 1, 1), (16, 8, 33, 0, 1, 0), (3, 64, 17, 1, 0, 1),
                                            (128, 128, 784, 1, 1, 1)])
def test_fpc_matmul(pg, ctx, dt, M, N, K, tA, tB, tC):
    a, b = views(M * K, dt, 1), views(K * N, dt, 2)
    trunc = 26 if dt == U64 else 10
    comm = orc.Comm(4)
    want = orc.fpc_matmul(a, b, M, N, K, tA, tB, tC, trunc, comm)
    c = pg.fpc.empty(M * N, "u64" if dt == U64 else "u32")
    pg.fpc.matmul(ctx, dev(a), dev(b), c, M, N, K, tA, tB, tC, trunc)
    ctx.sync()
    assert np.array_equal(host(c), want)
    check_comm(ctx, comm)


def test_fpc_matmul_public_inputs_reveal_the_product(pg, ctx):
    """Inputs loaded as the reference loads them (setPublic: values in x0):
    every party reveals the truncated product. (With fully random 4-party
    sharings the reference's zero-mask reshare does not give the product;
    the shares still match the oracle, as test_fpc_matmul checks.)"""
    M, N, K, fp = 32, 24, 100, 26
    rng = np.random.default_rng(3)
    xv, wv = rng.normal(0, 1, M * K), rng.normal(0, 1, K * N)
    a, b = orc.fpc_from_list(xv, fp=fp), orc.fpc_from_list(wv, fp=fp)
    want = orc.fpc_matmul(a, b, M, N, K, 1, 1, 1, fp)
    c = pg.fpc.empty(M * N)
    pg.fpc.matmul(ctx, dev(a), dev(b), c, M, N, K, 1, 1, 1, fp)
    ctx.sync()
    got = host(c)
    assert np.array_equal(got, want)
    ref = orc.decode(orc.gemm(M, N, K, orc.encode(xv, fp=fp), 1, orc.encode(wv, fp=fp), 1, 1), 2 * fp)
    rec = orc.fpc_reconstruct(got)
    for p in range(4):
        assert np.max(np.abs(orc.decode(rec[p], fp) - ref)) < 1e-3


@pytest.mark.parametrize("dt", [U64, U32])
def test_fpc_fc_forward_bias(pg, ctx, dt):
    batch, din, dout = 32, 100, 24
    fp = 26 if dt == U64 else 10
    x, w, bias = views(batch * din, dt, 6), views(din * dout, dt, 7), views(dout, dt, 8)
    want = orc.fpc_matmul(x, w, batch, dout, din, 1, 1, 1, fp)
    want = (want.reshape(4, 3, batch, dout) + bias[:, :, None, :]).reshape(4, 3, -1).astype(dt)
    out = pg.fpc.empty(batch * dout, "u64" if dt == U64 else "u32")
    pg.fpc.fc_forward(ctx, dev(x), dev(w), dev(bias), out, batch, din, dout, fp)
    ctx.sync()
    assert np.array_equal(host(out), want)


@pytest.mark.parametrize("op", [orc.FPROP, orc.DGRAD, orc.WGRAD])
def test_fpc_convolution(pg, ctx, op):
    batch, H, W, f, Din, Dout, stride, pad = 2, 6, 5, 3, 4, 3, 1, 1
    P = (H + 2 * pad - f) // stride + 1
    Q = (W + 2 * pad - f) // stride + 1
    nx, nw, ny = batch * H * W * Din, Dout * f * f * Din, batch * P * Q * Dout
    na = nx if op == orc.FPROP else ny
    nb = nx if op == orc.WGRAD else nw
    A, B = views(na, U64, 9), views(nb, U64, 10)
    comm = orc.Comm(4)
    want = orc.fpc_convolution(A, B, op, batch, H, W, f, Din, Dout, stride, pad, 20, comm)
    C = pg.fpc.empty(want.shape[2])
    pg.fpc.convolution(ctx, dev(A), dev(B), C, op, batch, H, W, f, Din, Dout, stride, pad, 20)
    ctx.sync()
    assert np.array_equal(host(C), want)
    check_comm(ctx, comm)


def test_fpc_wgrad_small_output(pg, ctx):
    """A weight gradient with few outputs and a long K (the u64 form's
    small-output kernel over the 4PC party segments)."""
    batch, H, W, f, Din, Dout, stride, pad = 64, 20, 20, 5, 1, 8, 1, 0
    P = Q = H - f + 1
    A, B = views(batch * P * Q * Dout, U64, 18), views(batch * H * W * Din, U64, 19)
    comm = orc.Comm(4)
    want = orc.fpc_convolution(A, B, orc.WGRAD, batch, H, W, f, Din, Dout, stride, pad, 20, comm)
    C = pg.fpc.empty(want.shape[2])
    pg.fpc.convolution(ctx, dev(A), dev(B), C, orc.WGRAD, batch, H, W, f, Din, Dout, stride, pad, 20)
    ctx.sync()
    assert np.array_equal(host(C), want)
    check_comm(ctx, comm)


def test_fpc_convolution_strided(pg, ctx):
    batch, H, W, f, Din, Dout, stride, pad = 3, 9, 7, 3, 2, 5, 2, 1
    P = (H + 2 * pad - f) // stride + 1
    Q = (W + 2 * pad - f) // stride + 1
    A, B = views(batch * H * W * Din, U64, 11), views(Dout * f * f * Din, U64, 12)
    want = orc.fpc_convolution(A, B, orc.FPROP, batch, H, W, f, Din, Dout, stride, pad, 26)
    C = pg.fpc.empty(batch * P * Q * Dout)
    pg.fpc.convolution(ctx, dev(A), dev(B), C, orc.FPROP, batch, H, W, f, Din, Dout, stride, pad, 26)
    ctx.sync()
    assert np.array_equal(host(C), want)


@pytest.mark.parametrize("d", [1 << 26, 3, 1000])
def test_fpc_divide_public(pg, ctx, d):
    a = views(999, U64, 13)
    comm = orc.Comm(4)
    want = orc.fpc_divide_public(a, d, comm)
    t = dev(a)
    pg.fpc.dividePublic(ctx, t, d)
    ctx.sync()
    assert np.array_equal(host(t), want)
    check_comm(ctx, comm)


def test_fpc_divide_public_vector_and_u32(pg, ctx):
    a = views(300, U64, 14)
    d = (np.uint64(1) << np.random.default_rng(15).integers(1, 40, 300).astype(U64)).astype(U64)
    want = orc.fpc_divide_public(a, d)
    t = dev(a)
    pg.fpc.dividePublic(ctx, t, dev(d))
    ctx.sync()
    assert np.array_equal(host(t), want)
    a32 = views(300, U32, 16)
    t32 = dev(a32)
    pg.fpc.dividePublic(ctx, t32, 1 << 10)
    ctx.sync()
    assert np.array_equal(host(t32), orc.fpc_divide_public(a32, 1 << 10))


@pytest.mark.parametrize("dt", [U64, U32, U8])
def test_fpc_reconstruct(pg, ctx, dt):
    a = views(513, dt, 17)
    comm = orc.Comm(4)
    want = orc.fpc_reconstruct(a, comm)
    out = dev(np.zeros((4, 513), dtype=dt))
    pg.fpc.reconstruct(ctx, dev(a), out)
    ctx.sync()
    assert np.array_equal(host(out), want)
    check_comm(ctx, comm)


def test_fpc_mul(pg, ctx):
    a, b = views(777, U64, 18), views(777, U64, 19)
    comm = orc.Comm(4)
    want = orc.fpc_mul(a, b, comm)
    t = dev(a)
    pg.fpc.mul_(ctx, t, dev(b))
    ctx.sync()
    assert np.array_equal(host(t), want)
    check_comm(ctx, comm)


def test_fpc_and_u8(pg, ctx):
    a, b = views(777, U8, 20), views(777, U8, 21)
    comm = orc.Comm(4)
    want = orc.fpc_and(a, b, comm)
    t = dev(a)
    pg.fpc.and_(ctx, t, dev(b))
    ctx.sync()
    assert np.array_equal(host(t), want)
    check_comm(ctx, comm)


def _edge_values(dt):
    W = np.iinfo(dt).bits
    e = [0, 1, 2, (1 << (W - 1)) - 2, (1 << (W - 1)) - 1, 1 << (W - 1), (1 << (W - 1)) + 1, (1 << W) - 2, (1 << W) - 1]
    return np.array(e, dtype=dt)


@pytest.mark.parametrize("dt", [U64, U32])
def test_fpc_drelu(pg, ctx, dt):
    rng = np.random.default_rng(22)
    vals = np.concatenate([_edge_values(dt), rng.integers(0, np.iinfo(dt).max, 2000, dtype=dt, endpoint=True)])
    x = orc.fpc_share_random(vals, dtype=dt, seed=23)
    comm = orc.Comm(4)
    want = orc.fpc_drelu(x, comm=comm)
    out = dev(np.zeros((4, 3, vals.size), dtype=U8))
    pg.fpc.dReLU(ctx, dev(x), out)
    ctx.sync()
    assert np.array_equal(host(out), want)
    check_comm(ctx, comm)


def test_fpc_drelu_inconsistent_views(pg, ctx):
    x = views(1500, U64, 24)
    want = orc.fpc_drelu(x)
    out = dev(np.zeros((4, 3, 1500), dtype=U8))
    pg.fpc.dReLU(ctx, dev(x), out)
    ctx.sync()
    assert np.array_equal(host(out), want)


@pytest.mark.parametrize("dt", [U64, U32])
def test_fpc_relu(pg, ctx, dt):
    fp = 26 if dt == U64 else 10
    vals = orc.encode(np.random.default_rng(25).normal(0, 4, 3000), dtype=dt, fp=fp)
    vals = np.concatenate([_edge_values(dt), vals])
    x = orc.fpc_share_random(vals, dtype=dt, seed=26)
    comm = orc.Comm(4)
    want, dwant = orc.fpc_relu(x, comm=comm)
    out = pg.fpc.empty(vals.size, "u64" if dt == U64 else "u32")
    dout = dev(np.zeros((4, 3, vals.size), dtype=U8))
    pg.fpc.ReLU(ctx, dev(x), out, dout)
    ctx.sync()
    assert np.array_equal(host(out), want)
    assert np.array_equal(host(dout), dwant)
    check_comm(ctx, comm)


def test_fpc_relu_inconsistent_views(pg, ctx):
    x = views(1200, U64, 27)
    want, dwant = orc.fpc_relu(x)
    out = pg.fpc.empty(1200)
    dout = dev(np.zeros((4, 3, 1200), dtype=U8))
    pg.fpc.ReLU(ctx, dev(x), out, dout)
    ctx.sync()
    assert np.array_equal(host(out), want)
    assert np.array_equal(host(dout), dwant)


def test_fpc_select_share(pg, ctx):
    n = 1000
    x, y = views(n, U64, 28), views(n, U64, 29)
    b = views(n, U8, 30) % 3  # shares that reveal to 1 at some parties and not at others
    comm = orc.Comm(4)
    want = orc.fpc_select_share(x, y, b, comm)
    z = pg.fpc.empty(n)
    pg.fpc.selectShare(ctx, dev(x), dev(y), dev(b), z)
    ctx.sync()
    assert np.array_equal(host(z), want)
    check_comm(ctx, comm)


@pytest.mark.parametrize("k", [2, 4, 16])
def test_fpc_maxpool(pg, ctx, k):
    rows = 200
    vals = orc.encode(np.random.default_rng(31).normal(0, 3, rows * k))
    vals[:k] = vals[0]  # ties
    x = orc.fpc_share_random(vals, seed=32)
    comm = orc.Comm(4)
    want, dwant = orc.fpc_maxpool(x, k, comm=comm)
    out = pg.fpc.empty(rows)
    dout = dev(np.zeros((4, 3, rows * k), dtype=U8))
    xd = dev(x)
    pg.fpc.maxpool(ctx, xd, out, dout, k)
    ctx.sync()
    assert np.array_equal(host(out), want)
    assert np.array_equal(host(dout), dwant)
    assert np.array_equal(host(xd), x)  # the input is left as it was
    check_comm(ctx, comm)


def test_fpc_maxpool_inconsistent_views(pg, ctx):
    rows, k = 300, 4
    x = views(rows * k, U64, 33)
    want, dwant = orc.fpc_maxpool(x, k)
    out = pg.fpc.empty(rows)
    dout = dev(np.zeros((4, 3, rows * k), dtype=U8))
    pg.fpc.maxpool(ctx, dev(x), out, dout, k)
    ctx.sync()
    assert np.array_equal(host(out), want)
    assert np.array_equal(host(dout), dwant)


def test_fpc_fc_net_u32_fp10(pg, ctx):
    """The 4PC FC net (784-128-128-10, ReLU between layers) at batch 128 on
    uint32 shares with 10 fractional bits, layer by layer against the oracle."""
    batch, fp, dims = 128, 10, [784, 128, 128, 10]
    rng = np.random.default_rng(34)
    x = orc.fpc_from_list(rng.uniform(0, 1, batch * 784), dtype=U32, fp=fp)  # setPublic, as the reference loads
    cur_h, cur_d = x, dev(x)
    for li in range(3):
        din, dout = dims[li], dims[li + 1]
        bound = np.sqrt(6.0 / din)
        w = orc.fpc_from_list(rng.uniform(-bound, bound, din * dout), dtype=U32, fp=fp)
        bias = orc.fpc_from_list(rng.uniform(-bound, bound, dout), dtype=U32, fp=fp)
        want = orc.fpc_matmul(cur_h, w, batch, dout, din, 1, 1, 1, fp)
        want = (want.reshape(4, 3, batch, dout) + bias[:, :, None, :]).reshape(4, 3, -1).astype(U32)
        out = pg.fpc.empty(batch * dout, "u32")
        pg.fpc.fc_forward(ctx, cur_d, dev(w), dev(bias), out, batch, din, dout, fp)
        ctx.sync()
        assert np.array_equal(host(out), want), f"fc {li}"
        cur_h, cur_d = want, out
        if li < 2:
            want_r, _ = orc.fpc_relu(cur_h)
            r = pg.fpc.empty(batch * dout, "u32")
            dr = dev(np.zeros((4, 3, batch * dout), dtype=U8))
            pg.fpc.ReLU(ctx, cur_d, r, dr)
            ctx.sync()
            assert np.array_equal(host(r), want_r), f"relu {li}"
            cur_h, cur_d = want_r, r


@pytest.mark.parametrize("op,kind", [("add", "scalar"), ("sub", "public"), ("xor", "public"), ("and", "public"),
                                     ("shr", "public"), ("mul", "scalar"), ("sub", "shares"), ("xor", "shares")])
def test_fpc_local(pg, ctx, op, kind):
    import torch

    n = 555
    a = views(n, U64, 80)
    rng = np.random.default_rng(81)
    shift = op in ("shr", "shl")
    if kind == "scalar":
        r_np = int(rng.integers(0, 70)) if shift else int(rng.integers(0, 2**63))
        r_dev = r_np
    elif kind == "public":
        r_np = rng.integers(0, 70, n, dtype=U64) if shift else rng.integers(0, 2**63, n, dtype=U64)
        r_dev = torch.from_numpy(r_np.view(np.int64)).cuda()
    else:
        r_np = views(n, U64, 82)
        r_dev = dev(r_np)
    ops = {"add": pg.OP_ADD, "sub": pg.OP_SUB, "mul": pg.OP_MUL, "xor": pg.OP_XOR, "and": pg.OP_AND,
           "shr": pg.OP_SHR}
    da = dev(a)
    pg.fpc.local_(ctx, ops[op], da, r_dev)
    ctx.sync()
    assert np.array_equal(host(da), orc.fpc_local(op, a, r_np))


def test_fpc_empty_inputs(pg, ctx):
    """Zero-length inputs: no launch, the oracle's rounds with empty messages."""
    e = np.zeros((4, 3, 0), U64)
    comm = orc.Comm(4)
    a, b = pg.fpc.empty(0), pg.fpc.empty(0)
    pg.fpc.reconstruct(ctx, a, dev(np.zeros((4, 0), U64)))
    orc.fpc_reconstruct(e, comm)
    pg.fpc.mul_(ctx, a, b)
    orc.fpc_mul(e, e, comm)
    pg.fpc.dividePublic(ctx, a, 3)
    orc.fpc_divide_public(e.copy(), 3, comm)
    pg.fpc.dReLU(ctx, a, pg.fpc.empty(0, "u8"))
    orc.fpc_drelu(e, comm=comm)
    pg.fpc.ReLU(ctx, a, pg.fpc.empty(0), pg.fpc.empty(0, "u8"))
    orc.fpc_relu(e, comm=comm)
    pg.fpc.selectShare(ctx, a, b, pg.fpc.empty(0, "u8"), pg.fpc.empty(0))
    orc.fpc_select_share(e, e, np.zeros((4, 3, 0), U8), comm)
    pg.fpc.local_(ctx, pg.OP_ADD, a, 5)
    pg.fpc.maxpool(ctx, a, pg.fpc.empty(0), pg.fpc.empty(0, "u8"), 4)
    ctx.sync()
    check_comm(ctx, comm)
    assert comm.rounds > 20
