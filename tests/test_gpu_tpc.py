"""TPC (2PC) entry points against the CPU oracle's restatement of src/mpc/TPC.inl.

Every share of both parties must match bit for bit, and the communication
counters must equal the bytes and rounds of the reference's reveals.
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


def rnd(n, dt, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.integers(0, np.iinfo(dt).max, n, dtype=dt, endpoint=True) for _ in range(2)])


def check_comm(ctx, comm):
    cc = ctx.comm()
    assert cc["tx"][:2] == comm.tx[:2] and cc["rx"][:2] == comm.rx[:2] and cc["rounds"] == comm.rounds


@pytest.mark.parametrize("dt", [U64, U32])
@pytest.mark.parametrize("M,N,K,tA,tB,tC", [(5, 7, 9, 1, 1, 1), (16, 8, 33, 0, 1, 0), (3, 64, 17, 1, 0, 1),
                                            (128, 128, 784, 1, 1, 1)])
def test_tpc_matmul(pg, ctx, dt, M, N, K, tA, tB, tC):
    a, b = rnd(M * K, dt, 1), rnd(K * N, dt, 2)
    trunc = 26 if dt == U64 else 10
    comm = orc.Comm()
    want = orc.tpc_matmul(a, b, M, N, K, tA, tB, tC, trunc, comm)
    c = pg.tpc.empty(M * N, "u64" if dt == U64 else "u32")
    pg.tpc.matmul(ctx, dev(a), dev(b), c, M, N, K, tA, tB, tC, trunc)
    ctx.sync()
    assert np.array_equal(host(c), want)
    check_comm(ctx, comm)


@pytest.mark.parametrize("dt", [U64, U32])
def test_tpc_fc_forward_bias(pg, ctx, dt):
    batch, din, dout = 32, 100, 24
    fp = 26 if dt == U64 else 10
    x, w, bias = rnd(batch * din, dt, 3), rnd(din * dout, dt, 4), rnd(dout, dt, 5)
    want = orc.tpc_matmul(x, w, batch, dout, din, 1, 1, 1, fp)
    want = (want.reshape(2, batch, dout) + bias[:, None, :]).reshape(2, -1).astype(dt)
    out = pg.tpc.empty(batch * dout, "u64" if dt == U64 else "u32")
    pg.tpc.fc_forward(ctx, dev(x), dev(w), dev(bias), out, batch, din, dout, fp)
    ctx.sync()
    assert np.array_equal(host(out), want)


@pytest.mark.parametrize("op", [orc.FPROP, orc.DGRAD, orc.WGRAD])
def test_tpc_convolution(pg, ctx, op):
    batch, H, W, f, Din, Dout, stride, pad = 2, 6, 5, 3, 4, 3, 1, 1
    P = (H + 2 * pad - f) // stride + 1
    Q = (W + 2 * pad - f) // stride + 1
    nx, nw, ny = batch * H * W * Din, Dout * f * f * Din, batch * P * Q * Dout
    na = nx if op == orc.FPROP else ny
    nb = nx if op == orc.WGRAD else nw
    A, B = rnd(na, U64, 6), rnd(nb, U64, 7)
    comm = orc.Comm()
    want = orc.tpc_convolution(A, B, op, batch, H, W, f, Din, Dout, stride, pad, 20, comm)
    C = pg.tpc.empty(want.shape[1])
    pg.tpc.convolution(ctx, dev(A), dev(B), C, op, batch, H, W, f, Din, Dout, stride, pad, 20)
    ctx.sync()
    assert np.array_equal(host(C), want)
    check_comm(ctx, comm)


def test_tpc_wgrad_small_output(pg, ctx):
    """A weight gradient with few outputs and a long K (the u64 form's
    small-output kernel over the 2PC segments)."""
    batch, H, W, f, Din, Dout, stride, pad = 64, 20, 20, 5, 1, 8, 1, 0
    P = Q = H - f + 1
    A, B = rnd(batch * P * Q * Dout, U64, 16), rnd(batch * H * W * Din, U64, 17)
    comm = orc.Comm()
    want = orc.tpc_convolution(A, B, orc.WGRAD, batch, H, W, f, Din, Dout, stride, pad, 20, comm)
    C = pg.tpc.empty(want.shape[1])
    pg.tpc.convolution(ctx, dev(A), dev(B), C, orc.WGRAD, batch, H, W, f, Din, Dout, stride, pad, 20)
    ctx.sync()
    assert np.array_equal(host(C), want)
    check_comm(ctx, comm)


@pytest.mark.parametrize("d", [1 << 26, 3, 1000])
def test_tpc_divide_public(pg, ctx, d):
    a = rnd(999, U64, 8)
    comm = orc.Comm()
    want = orc.tpc_divide_public(a, d, comm)
    t = dev(a)
    pg.tpc.dividePublic(ctx, t, d)
    ctx.sync()
    assert np.array_equal(host(t), want)
    check_comm(ctx, comm)


def test_tpc_divide_public_vector_and_u32(pg, ctx):
    a = rnd(300, U64, 9)
    d = (np.uint64(1) << np.random.default_rng(10).integers(1, 40, 300).astype(U64)).astype(U64)
    want = orc.tpc_divide_public(a, d)
    t = dev(a)
    pg.tpc.dividePublic(ctx, t, dev(d))
    ctx.sync()
    assert np.array_equal(host(t), want)
    a32 = rnd(300, U32, 11)
    t32 = dev(a32)
    pg.tpc.dividePublic(ctx, t32, 1 << 10)
    ctx.sync()
    assert np.array_equal(host(t32), orc.tpc_divide_public(a32, 1 << 10))


@pytest.mark.parametrize("dt", [U64, U32, U8])
def test_tpc_reconstruct(pg, ctx, dt):
    a = rnd(513, dt, 12)
    comm = orc.Comm()
    want = orc.tpc_reconstruct(a, comm)
    out = dev(np.zeros((2, 513), dtype=dt))
    pg.tpc.reconstruct(ctx, dev(a), out)
    ctx.sync()
    assert np.array_equal(host(out), want)
    check_comm(ctx, comm)


def test_tpc_mul(pg, ctx):
    a, b = rnd(777, U64, 13), rnd(777, U64, 14)
    comm = orc.Comm()
    want = orc.tpc_mul(a, b, comm)
    t = dev(a)
    pg.tpc.mul_(ctx, t, dev(b))
    ctx.sync()
    assert np.array_equal(host(t), want)
    check_comm(ctx, comm)


def _edge_values(dt):
    W = np.iinfo(dt).bits
    e = [0, 1, 2, (1 << (W - 1)) - 2, (1 << (W - 1)) - 1, 1 << (W - 1), (1 << (W - 1)) + 1, (1 << W) - 2, (1 << W) - 1]
    return np.array(e, dtype=dt)


@pytest.mark.parametrize("dt", [U64, U32])
def test_tpc_drelu(pg, ctx, dt):
    vals = np.concatenate([_edge_values(dt), rnd(2000, dt, 15)[0]])
    x = orc.tpc_share_random(vals, dtype=dt, seed=16)
    comm = orc.Comm()
    want = orc.tpc_drelu(x, comm=comm)
    out = dev(np.zeros((2, vals.size), dtype=U8))
    pg.tpc.dReLU(ctx, dev(x), out)
    ctx.sync()
    assert np.array_equal(host(out), want)
    check_comm(ctx, comm)


@pytest.mark.parametrize("dt", [U64, U32])
def test_tpc_relu(pg, ctx, dt):
    fp = 26 if dt == U64 else 10
    vals = orc.encode(np.random.default_rng(17).normal(0, 4, 3000), dtype=dt, fp=fp)
    vals = np.concatenate([_edge_values(dt), vals])
    x = orc.tpc_share_random(vals, dtype=dt, seed=18)
    comm = orc.Comm()
    want, dwant = orc.tpc_relu(x, comm=comm)
    out = pg.tpc.empty(vals.size, "u64" if dt == U64 else "u32")
    dout = dev(np.zeros((2, vals.size), dtype=U8))
    pg.tpc.ReLU(ctx, dev(x), out, dout)
    ctx.sync()
    assert np.array_equal(host(out), want)
    assert np.array_equal(host(dout), dwant)
    check_comm(ctx, comm)


def test_tpc_select_share(pg, ctx):
    n = 1000
    x, y = rnd(n, U64, 19), rnd(n, U64, 20)
    rng = np.random.default_rng(21)
    b = np.stack([rng.integers(0, 2, n).astype(U8), np.zeros(n, U8)])
    b[1, :10] = 1  # shares that do not sum to a bit: the e == 1 test decides
    comm = orc.Comm()
    want = orc.tpc_select_share(x, y, b, comm)
    z = pg.tpc.empty(n)
    pg.tpc.selectShare(ctx, dev(x), dev(y), dev(b), z)
    ctx.sync()
    assert np.array_equal(host(z), want)
    check_comm(ctx, comm)


@pytest.mark.parametrize("k", [4, 16])
def test_tpc_maxpool(pg, ctx, k):
    rows = 200
    vals = orc.encode(np.random.default_rng(22).normal(0, 3, rows * k))
    vals[:k] = vals[0]  # ties
    x = orc.tpc_share_random(vals, seed=23)
    comm = orc.Comm()
    want, dwant = orc.tpc_maxpool(x, k, comm=comm)
    out = pg.tpc.empty(rows)
    dout = dev(np.zeros((2, rows * k), dtype=U8))
    pg.tpc.maxpool(ctx, dev(x), out, dout, k)
    ctx.sync()
    assert np.array_equal(host(out), want)
    assert np.array_equal(host(dout), dwant)
    check_comm(ctx, comm)


def test_tpc_fc_net_u32_fp10(pg, ctx):
    """The 2PC FC net (784-128-128-10, ReLU between layers) at batch 128 on
    uint32 shares with 10 fractional bits, layer by layer against the oracle."""
    batch, fp, dims = 128, 10, [784, 128, 128, 10]
    rng = np.random.default_rng(24)
    x = orc.tpc_share_random(orc.encode(rng.uniform(0, 1, batch * 784), dtype=U32, fp=fp), dtype=U32, seed=25)
    cur_h, cur_d = x, dev(x)
    for li in range(3):
        din, dout = dims[li], dims[li + 1]
        bound = np.sqrt(6.0 / din)
        w = orc.tpc_from_list(rng.uniform(-bound, bound, din * dout), dtype=U32, fp=fp)
        bias = orc.tpc_from_list(rng.uniform(-bound, bound, dout), dtype=U32, fp=fp)
        want = orc.tpc_matmul(cur_h, w, batch, dout, din, 1, 1, 1, fp)
        want = (want.reshape(2, batch, dout) + bias[:, None, :]).reshape(2, -1).astype(U32)
        out = pg.tpc.empty(batch * dout, "u32")
        pg.tpc.fc_forward(ctx, cur_d, dev(w), dev(bias), out, batch, din, dout, fp)
        ctx.sync()
        assert np.array_equal(host(out), want), f"fc {li}"
        cur_h, cur_d = want, out
        if li < 2:
            want_r, _ = orc.tpc_relu(cur_h)
            r = pg.tpc.empty(batch * dout, "u32")
            dr = dev(np.zeros((2, batch * dout), dtype=U8))
            pg.tpc.ReLU(ctx, cur_d, r, dr)
            ctx.sync()
            assert np.array_equal(host(r), want_r), f"relu {li}"
            cur_h, cur_d = want_r, r


@pytest.mark.parametrize("op,kind", [("add", "scalar"), ("sub", "public"), ("xor", "public"), ("mul", "public"),
                                     ("shr", "scalar"), ("shl", "public"), ("add", "shares"), ("xor", "shares")])
def test_tpc_local(pg, ctx, op, kind):
    import torch

    n = 777
    a = rnd(n, U64, 70)
    rng = np.random.default_rng(71)
    shift = op in ("shr", "shl")
    if kind == "scalar":
        r_np = int(rng.integers(0, 70)) if shift else int(rng.integers(0, 2**63))
        r_dev = r_np
    elif kind == "public":
        r_np = rng.integers(0, 70, n, dtype=U64) if shift else rng.integers(0, 2**63, n, dtype=U64)
        r_dev = torch.from_numpy(r_np.view(np.int64)).cuda()
    else:
        r_np = rnd(n, U64, 72)
        r_dev = dev(r_np)
    ops = {"add": pg.OP_ADD, "sub": pg.OP_SUB, "mul": pg.OP_MUL, "xor": pg.OP_XOR, "shr": pg.OP_SHR, "shl": pg.OP_SHL}
    da = dev(a)
    pg.tpc.local_(ctx, ops[op], da, r_dev)
    ctx.sync()
    assert np.array_equal(host(da), orc.tpc_local(op, a, r_np))


def test_tpc_empty_inputs(pg, ctx):
    """Zero-length inputs: no launch, the oracle's rounds with empty messages."""
    e = np.zeros((2, 0), U64)
    comm = orc.Comm()
    a, b = pg.tpc.empty(0), pg.tpc.empty(0)
    pg.tpc.reconstruct(ctx, a, pg.tpc.empty(0))
    orc.tpc_reconstruct(e, comm)
    pg.tpc.mul_(ctx, a, b)
    orc.tpc_mul(e, e, comm)
    pg.tpc.dividePublic(ctx, a, 3)
    orc.tpc_divide_public(e.copy(), 3, comm)
    pg.tpc.dReLU(ctx, a, pg.tpc.empty(0, "u8"))
    orc.tpc_drelu(e, comm=comm)
    pg.tpc.ReLU(ctx, a, pg.tpc.empty(0), pg.tpc.empty(0, "u8"))
    orc.tpc_relu(e, comm=comm)
    pg.tpc.selectShare(ctx, a, b, pg.tpc.empty(0, "u8"), pg.tpc.empty(0))
    orc.tpc_select_share(e, e, np.zeros((2, 0), U8), comm)
    pg.tpc.local_(ctx, pg.OP_ADD, a, 5)
    pg.tpc.maxpool(ctx, a, pg.tpc.empty(0), pg.tpc.empty(0, "u8"), 4)
    ctx.sync()
    check_comm(ctx, comm)
    assert comm.rounds > 20
