"""GPU parity: every CUDA entry point against the CPU oracle, bit for bit.

Inputs are seeded. Share views are either a consistent RSS sharing or six
independent random slots (arbitrary per-party views, which exercise every
party-local code path the reference has). Every output share of every party
must equal the oracle's exactly, and so must the communication counters.
"""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

U64, U32, U8 = np.uint64, np.uint32, np.uint8


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


def rnd(shape, dt, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, np.iinfo(dt).max, size=shape, dtype=dt, endpoint=True)


def small_fixed_views(n, seed, scale=4.0, fp=26):
    """Consistent RSS sharing of small fixed-point values (meaningful ReLU/maxpool inputs)."""
    rng = np.random.default_rng(seed)
    vals = rng.normal(0, scale, size=n)
    return orc.share_random(orc.encode(vals, U64, fp), U64, seed=seed + 1)


def dev(pg, a):
    return pg.to_device(a)


def host(pg, t, ring="u64"):
    return pg.to_host(t, ring)


def comm_equal(ctx, comm):
    c = ctx.comm()
    assert c["tx"] == comm.tx and c["rx"] == comm.rx and c["rounds"] == comm.rounds, (c, comm.tx, comm.rounds)


# ------------------------------------------------------------------ gpu::gemm

@pytest.mark.parametrize("tA,tB,tC", [(a, b, c) for a in (0, 1) for b in (0, 1) for c in (0, 1)])
@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (2, 4, 3), (129, 65, 17), (200, 70, 300)])
def test_gemm_layouts(pg, ctx, M, N, K, tA, tB, tC):
    import torch

    A = rnd(M * K, U64, 1)
    B = rnd(K * N, U64, 2)
    C = torch.empty(M * N, dtype=torch.int64, device="cuda")
    pg.gpu.gemm(ctx, M, N, K, torch.from_numpy(A.view(np.int64)).cuda(), tA, torch.from_numpy(B.view(np.int64)).cuda(),
                tB, C, tC)
    ctx.sync()
    assert np.array_equal(C.cpu().numpy().view(U64), orc.gemm(M, N, K, A, tA, B, tB, tC))


def test_gemm_u32(pg, ctx):
    import torch

    M, N, K = 70, 33, 129
    A, B = rnd(M * K, U32, 3), rnd(K * N, U32, 4)
    C = torch.empty(M * N, dtype=torch.int32, device="cuda")
    pg.gpu.gemm(ctx, M, N, K, torch.from_numpy(A.view(np.int32)).cuda(), 1, torch.from_numpy(B.view(np.int32)).cuda(),
                0, C, 1)
    ctx.sync()
    assert np.array_equal(C.cpu().numpy().view(U32), orc.gemm(M, N, K, A, 1, B, 0, 1, dtype=U32))


def test_gemm_kats(pg, ctx, golden):
    import torch

    kat = golden[0]
    c = kat["CutlassGemmTranspose2"]
    M, N, K, tA, tB, tC = c["params"]["calls"][0]
    a = torch.tensor([int(v) for v in c["arrays"]["a"]], dtype=torch.int64, device="cuda")
    b = torch.tensor([int(v) for v in c["arrays"]["b"]], dtype=torch.int64, device="cuda")
    out = torch.empty(M * N, dtype=torch.int64, device="cuda")
    pg.gpu.gemm(ctx, M, N, K, a, tA, b, tB, out, tC)
    ctx.sync()
    assert out.cpu().tolist() == [int(v) for v in c["arrays"]["expected"]]


# ------------------------------------------------------------------- gpu::conv

CONV_SHAPES = [
    # N, H, W, C, K, R, pad, stride
    (1, 3, 3, 1, 1, 3, 1, 1),
    (2, 5, 5, 4, 10, 3, 1, 2),
    (3, 7, 6, 5, 7, 3, 0, 1),
    (2, 8, 8, 3, 17, 5, 2, 2),
    (1, 4, 4, 70, 9, 1, 0, 1),
]


@pytest.mark.parametrize("op", [orc.FPROP, orc.DGRAD, orc.WGRAD])
@pytest.mark.parametrize("shape", CONV_SHAPES)
def test_conv_single(pg, ctx, op, shape):
    import torch

    N, H, W, C, K, R, pad, stride = shape
    P, Q = (H + 2 * pad - R) // stride + 1, (W + 2 * pad - R) // stride + 1
    sizes = {orc.FPROP: (N * H * W * C, K * R * R * C), orc.DGRAD: (N * P * Q * K, K * R * R * C),
             orc.WGRAD: (N * P * Q * K, N * H * W * C)}[op]
    a, b = rnd(sizes[0], U64, 5), rnd(sizes[1], U64, 6)
    want = orc.conv(op, N, H, W, C, K, R, R, pad, stride, a, b)
    out = torch.empty(want.size, dtype=torch.int64, device="cuda")
    pg.gpu.conv(ctx, op, N, H, W, C, K, R, R, pad, stride, torch.from_numpy(a.view(np.int64)).cuda(),
                torch.from_numpy(b.view(np.int64)).cuda(), out)
    ctx.sync()
    assert np.array_equal(out.cpu().numpy().view(U64), want)


@pytest.mark.parametrize("name,op,a,b", [("CutlassConvDgrad2", orc.DGRAD, "delta", "filters"),
                                         ("CutlassConvWgrad2", orc.WGRAD, "delta", "input"),
                                         ("CutlassConvFprop", orc.FPROP, "im", "f")])
def test_conv_kats(pg, ctx, golden, name, op, a, b):
    import torch

    c = golden[0][name]
    p = c["params"]
    ta = torch.tensor([int(v) for v in c["arrays"][a]], dtype=torch.int64, device="cuda")
    tb = torch.tensor([int(v) for v in c["arrays"][b]], dtype=torch.int64, device="cuda")
    out = torch.empty(len(c["arrays"]["expected"]), dtype=torch.int64, device="cuda")
    pg.gpu.conv(ctx, op, p["N"], p["H"], p["W"], p["C"], p["K"], p["R"], p["R"], p["pad"], p["stride"], ta, tb, out)
    ctx.sync()
    assert out.cpu().tolist() == [int(v) for v in c["arrays"]["expected"]]


# ------------------------------------------------------------------ RSS matmul

@pytest.mark.parametrize("tA,tB,tC", [(1, 1, 1), (0, 0, 0), (1, 0, 1), (0, 1, 0)])
@pytest.mark.parametrize("M,N,K,trunc", [(2, 4, 3, 26), (128, 10, 784, 26), (33, 130, 65, 13), (257, 64, 16, 0),
                                         (64, 64, 64, 62)])
def test_rss_matmul_random_views(pg, ctx, M, N, K, trunc, tA, tB, tC):
    a, b = orc.random_views(M * K, U64, 10), orc.random_views(K * N, U64, 11)
    comm = orc.Comm()
    want = orc.matmul(a, b, M, N, K, tA, tB, tC, trunc, comm)
    c = pg.empty_shares(M * N)
    pg.matmul(ctx, dev(pg, a), dev(pg, b), c, M, N, K, tA, tB, tC, trunc)
    ctx.sync()
    assert np.array_equal(host(pg, c), want)
    comm_equal(ctx, comm)


def test_rss_matmul_u32(pg, ctx):
    M, N, K = 128, 10, 128
    a, b = orc.random_views(M * K, U32, 12), orc.random_views(K * N, U32, 13)
    want = orc.matmul(a, b, M, N, K, 1, 1, 1, 10)
    c = pg.empty_shares(M * N, "u32")
    pg.matmul(ctx, dev(pg, a), dev(pg, b), c, M, N, K, 1, 1, 1, 10)
    ctx.sync()
    assert np.array_equal(host(pg, c, "u32"), want)


def test_fc_forward_bias(pg, ctx):
    batch, din, dout = 128, 200, 70
    x = small_fixed_views(batch * din, 20)
    w = orc.set_public(np.random.default_rng(21).normal(0, 0.1, din * dout))
    bias = orc.set_public(np.full(dout, 0.01))
    act = orc.matmul(x, w, batch, dout, din, 1, 1, 1, 26)
    for p in range(3):
        for s in range(2):
            act[p, s] = orc.element_vector_add(act[p, s], bias[p, s], False, dout, batch)
    out = pg.empty_shares(batch * dout)
    pg.fc_forward(ctx, dev(pg, x), dev(pg, w), dev(pg, bias), out, batch, din, dout)
    ctx.sync()
    assert np.array_equal(host(pg, out), act)


# -------------------------------------------------------------------- RSS conv

@pytest.mark.parametrize("op", [orc.FPROP, orc.DGRAD, orc.WGRAD])
@pytest.mark.parametrize("batch,H,W,f,Din,Dout,stride,pad", [(2, 5, 5, 3, 4, 10, 2, 1), (3, 8, 8, 3, 16, 24, 1, 1),
                                                             (2, 12, 12, 5, 20, 50, 1, 0)])
def test_rss_conv_random_views(pg, ctx, op, batch, H, W, f, Din, Dout, stride, pad):
    P, Q = (H + 2 * pad - f) // stride + 1, (W + 2 * pad - f) // stride + 1
    na = {orc.FPROP: batch * H * W * Din, orc.DGRAD: batch * P * Q * Dout, orc.WGRAD: batch * P * Q * Dout}[op]
    nb = {orc.FPROP: Dout * f * f * Din, orc.DGRAD: Dout * f * f * Din, orc.WGRAD: batch * H * W * Din}[op]
    A, B = orc.random_views(na, U64, 30), orc.random_views(nb, U64, 31)
    comm = orc.Comm()
    want = orc.convolution(A, B, op, batch, H, W, f, Din, Dout, stride, pad, 26, comm)
    C = pg.empty_shares(want.shape[2])
    pg.convolution(ctx, dev(pg, A), dev(pg, B), C, op, batch, H, W, f, Din, Dout, stride, pad, 26)
    ctx.sync()
    assert np.array_equal(host(pg, C), want)
    comm_equal(ctx, comm)


@pytest.mark.parametrize("batch,H,W,f,Din,Dout,stride,pad", [(4, 12, 12, 5, 20, 50, 1, 0), (3, 9, 7, 3, 10, 70, 1, 1),
                                                             (128, 4, 4, 3, 20, 24, 1, 1)])
def test_rss_fprop_padded_channels_limb_form(pg, batch, H, W, f, Din, Dout, stride, pad):
    """Implicit limb-form convolutions over input channels that are not a
    multiple of 16 (the image's channels zero-padded to 32 or 16; the last
    case on position-major tiles), with the form fixed to the limb kernel."""
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    ctx.set_autotune(False)
    A = orc.random_views(batch * H * W * Din, U64, 42)
    B = orc.random_views(Dout * f * f * Din, U64, 43)
    comm = orc.Comm()
    want = orc.convolution(A, B, orc.FPROP, batch, H, W, f, Din, Dout, stride, pad, 26, comm)
    C = pg.empty_shares(want.shape[2])
    pg.convolution(ctx, dev(pg, A), dev(pg, B), C, orc.FPROP, batch, H, W, f, Din, Dout, stride, pad, 26)
    ctx.sync()
    assert np.array_equal(host(pg, C), want)
    comm_equal(ctx, comm)
    ctx.check_device_errors()
    ctx.close()


@pytest.mark.parametrize("batch,H,W,f,Din,Dout,stride,pad", [(128, 4, 4, 3, 32, 48, 1, 1), (4, 10, 9, 3, 16, 24, 1, 1),
                                                             (4, 12, 12, 5, 20, 50, 1, 0)])
def test_rss_dgrad_flipped_filter_limb_form(pg, tmp_path, batch, H, W, f, Din, Dout, stride, pad):
    """The input gradient as an implicit convolution of dY with the flipped,
    transposed filter (the third form the set-up timing can pick; here forced
    through a tuning-cache entry): position-major tiles at 128 images,
    rectangle tiles below, and a valid convolution whose dY is padded by
    f - 1 and whose 50 channels are zero-padded to 64."""
    import torch

    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    cache = tmp_path / "tune.txt"
    cache.write_text(f"pg-tune {sms}\nsform/conv/1/{batch}/{H}/{W}/{f}/{Din}/{Dout}/{stride}/{pad} 3 1\n")
    ctx.tune_load(str(cache))
    P, Q = (H + 2 * pad - f) // stride + 1, (W + 2 * pad - f) // stride + 1
    A = orc.random_views(batch * P * Q * Dout, U64, 44)
    B = orc.random_views(Dout * f * f * Din, U64, 45)
    comm = orc.Comm()
    want = orc.convolution(A, B, orc.DGRAD, batch, H, W, f, Din, Dout, stride, pad, 26, comm)
    C = pg.empty_shares(want.shape[2])
    pg.convolution(ctx, dev(pg, A), dev(pg, B), C, orc.DGRAD, batch, H, W, f, Din, Dout, stride, pad, 26)
    ctx.sync()
    assert np.array_equal(host(pg, C), want)
    comm_equal(ctx, comm)
    ctx.check_device_errors()
    ctx.close()


@pytest.mark.parametrize("batch,H,W,f,Din,Dout,stride,pad", [(8, 28, 28, 5, 1, 20, 1, 0), (64, 17, 17, 3, 3, 6, 2, 1),
                                                             (40, 10, 10, 3, 2, 30, 1, 1), (2, 3, 600, 3, 20, 4, 1, 1)])
def test_rss_wgrad_small_output_u64_form(pg, batch, H, W, f, Din, Dout, stride, pad):
    """Weight gradients with few outputs and a long K (LeNet's first
    convolution at batch 8; a strided, padded one; one with 30 filters) run the
    u64 form's row-staged small-output kernel; the last case's input rows
    (600 pixels x 20 channels) are too long to stage and take the gathering
    kernel: every share equal to the oracle's."""
    ctx = pg.Context(0, form=pg.FORM_U64)
    P, Q = (H + 2 * pad - f) // stride + 1, (W + 2 * pad - f) // stride + 1
    assert 6 * batch * P * Q >= 16384
    A = orc.random_views(batch * P * Q * Dout, U64, 40)
    B = orc.random_views(batch * H * W * Din, U64, 41)
    comm = orc.Comm()
    want = orc.convolution(A, B, orc.WGRAD, batch, H, W, f, Din, Dout, stride, pad, 26, comm)
    C = pg.empty_shares(want.shape[2])
    pg.convolution(ctx, dev(pg, A), dev(pg, B), C, orc.WGRAD, batch, H, W, f, Din, Dout, stride, pad, 26)
    ctx.sync()
    assert np.array_equal(host(pg, C), want)
    comm_equal(ctx, comm)
    ctx.check_device_errors()
    ctx.close()


# ------------------------------------------------------------- elementwise ops

@pytest.mark.parametrize("n", [1, 1000, 65537])
def test_reconstruct_reshare_mul_and(pg, ctx, n):
    import torch

    a, b = orc.random_views(n, U64, 40), orc.random_views(n, U64, 41)
    comm = orc.Comm()
    rec = pg.reconstruct(ctx, dev(pg, a))
    ctx.sync()
    assert np.array_equal(rec.cpu().numpy().view(U64), orc.reconstruct(a, comm))
    c3 = rnd((3, n), U64, 42)
    out = pg.empty_shares(n)
    pg.reshare(ctx, torch.from_numpy(c3.view(np.int64)).cuda(), out)
    assert np.array_equal(host(pg, out), orc.reshare(c3, comm))
    da = dev(pg, a)
    pg.mul_(ctx, da, dev(pg, b))
    assert np.array_equal(host(pg, da), orc.mul(a, b, comm))
    da = dev(pg, a)
    pg.and_(ctx, da, dev(pg, b))
    assert np.array_equal(host(pg, da), orc.and_(a, b, comm))
    ctx.sync()
    comm_equal(ctx, comm)


@pytest.mark.parametrize("d", [1, 2, 1 << 13, 1 << 26, 1 << 62, 3, 1000003, 0])
def test_divide_public_scalar(pg, ctx, d):
    n = 4099
    a = orc.random_views(n, U64, 50)
    want = orc.divide_public(a, d)
    da = dev(pg, a)
    pg.dividePublic(ctx, da, d)
    ctx.sync()
    assert np.array_equal(host(pg, da), want)


def test_divide_public_vector(pg, ctx):
    import torch

    n = 5000
    a = orc.random_views(n, U64, 51)
    pows = np.random.default_rng(52).integers(0, 40, size=n)
    d = (np.ones(n, dtype=U64) << pows.astype(U64)).astype(U64)
    d[::7] = 12345  # non-power-of-two denominators take the double path
    want = orc.divide_public(a, d)
    da = dev(pg, a)
    pg.dividePublic(ctx, da, torch.from_numpy(d.view(np.int64)).cuda())
    ctx.sync()
    assert np.array_equal(host(pg, da), want)


def test_divide_public_u32(pg, ctx):
    n = 3001
    a = orc.random_views(n, U32, 53)
    want = orc.divide_public(a, 1 << 10)
    da = dev(pg, a)
    pg.dividePublic(ctx, da, 1 << 10)
    ctx.sync()
    assert np.array_equal(host(pg, da, "u32"), want)


# ------------------------------------------------------------- dReLU / ReLU

@pytest.mark.parametrize("udt,ring", [(U8, "u8"), (U64, "u64")])
@pytest.mark.parametrize("n", [1, 34, 4097])
@pytest.mark.parametrize("kind", ["random", "fixed"])
def test_drelu(pg, ctx, udt, ring, n, kind):
    x = orc.random_views(n, U64, 60) if kind == "random" else small_fixed_views(n, 61)
    comm = orc.Comm()
    want = orc.drelu(x, udtype=udt, comm=comm)
    out = pg.empty_shares(n, ring)
    pg.dReLU(ctx, dev(pg, x), out)
    ctx.sync()
    assert np.array_equal(host(pg, out, ring), want)
    comm_equal(ctx, comm)


@pytest.mark.parametrize("udt,ring", [(U8, "u8"), (U64, "u64")])
@pytest.mark.parametrize("kind", ["random", "fixed", "public"])
def test_relu(pg, ctx, udt, ring, kind):
    n = 3333
    if kind == "random":
        x = orc.random_views(n, U64, 70)
    elif kind == "fixed":
        x = small_fixed_views(n, 71)
    else:  # setPublic with the PARTY_B fall-through
        x = orc.set_public(np.random.default_rng(72).normal(0, 3, n))
    comm = orc.Comm()
    want, dwant = orc.relu(x, udtype=udt, comm=comm)
    out, dout = pg.empty_shares(n), pg.empty_shares(n, ring)
    pg.ReLU(ctx, dev(pg, x), out, dout)
    ctx.sync()
    assert np.array_equal(host(pg, out), want)
    assert np.array_equal(host(pg, dout, ring), dwant)
    comm_equal(ctx, comm)


def test_relu_u32(pg, ctx):
    n = 2000
    x = orc.random_views(n, U32, 73)
    want, dwant = orc.relu(x, udtype=U8)
    out, dout = pg.empty_shares(n, "u32"), pg.empty_shares(n, "u8")
    pg.ReLU(ctx, dev(pg, x), out, dout)
    ctx.sync()
    assert np.array_equal(host(pg, out, "u32"), want)
    assert np.array_equal(host(pg, dout, "u8"), dwant)


def test_relu_golden(pg, ctx, golden):
    a = golden[0]["RELU"]["arrays"]
    x = orc.from_list(a["input"])
    out, dout = pg.empty_shares(x.shape[2]), pg.empty_shares(x.shape[2], "u64")
    pg.ReLU(ctx, dev(pg, x), out, dout)
    ctx.sync()
    rec = orc.reconstruct(host(pg, out))
    assert np.allclose(orc.decode(rec[0]), a["expected"], atol=1e-3)


@pytest.mark.parametrize("udt,ring", [(U8, "u8"), (U64, "u64")])
def test_select_share(pg, ctx, udt, ring):
    n = 2500
    x, y = orc.random_views(n, U64, 80), orc.random_views(n, U64, 81)
    # arbitrary small bit-share values, including ones whose reveal is not 0/1
    b = np.random.default_rng(82).integers(0, 4, size=(3, 2, n)).astype(udt)
    comm = orc.Comm()
    want = orc.select_share(x, y, b, comm)
    z = pg.empty_shares(n)
    pg.selectShare(ctx, dev(pg, x), dev(pg, y), dev(pg, b), z)
    ctx.sync()
    assert np.array_equal(host(pg, z), want)
    comm_equal(ctx, comm)


# ----------------------------------------------------------------- maxpool

@pytest.mark.parametrize("k", [4, 16])
@pytest.mark.parametrize("udt,ring", [(U8, "u8"), (U64, "u64")])
def test_maxpool_rows(pg, ctx, k, udt, ring):
    rows = 777
    x = small_fixed_views(rows * k, 90)
    comm = orc.Comm()
    want, dwant = orc.maxpool(x, k, udtype=udt, comm=comm)
    out, dout = pg.empty_shares(rows), pg.empty_shares(rows * k, ring)
    pg.maxpool(ctx, dev(pg, x), out, dout, k)
    ctx.sync()
    assert np.array_equal(host(pg, out), want)
    assert np.array_equal(host(pg, dout, ring), dwant)
    comm_equal(ctx, comm)


@pytest.mark.parametrize("H,W,C,pool,stride,batch", [(24, 24, 20, 2, 2, 4), (8, 8, 50, 2, 2, 3), (9, 9, 2, 3, 2, 5),
                                                     (4, 4, 3, 2, 1, 2), (6, 5, 2, 2, 2, 2)])
def test_maxpool_layer(pg, ctx, H, W, C, pool, stride, batch):
    x = small_fixed_views(batch * H * W * C, 91)
    comm = orc.Comm()
    want, dwant = orc.maxpool_layer(x, H, W, C, pool, stride, batch, comm=comm)
    out, dout = pg.empty_shares(want.shape[2]), pg.empty_shares(dwant.shape[2], "u8")
    pg.maxpool_layer(ctx, dev(pg, x), out, dout, H, W, C, pool, stride, batch)
    ctx.sync()
    assert np.array_equal(host(pg, out), want)
    assert np.array_equal(host(pg, dout, "u8"), dwant)
    comm_equal(ctx, comm)


def test_maxpool_layer_mnist_fixture(pg, ctx, golden):
    L = golden[1]
    x = orc.set_public(L["maxpool_mnist_input"])
    out, dout = pg.empty_shares(128 * 2 * 16), pg.empty_shares(128 * 2 * 16 * 9, "u8")
    pg.maxpool_layer(ctx, dev(pg, x), out, dout, 9, 9, 2, 3, 2, 128)
    ctx.sync()
    want, dwant = orc.maxpool_layer(x, 9, 9, 2, 3, 2, 128)
    assert np.array_equal(host(pg, out), want)
    assert np.array_equal(host(pg, dout, "u8"), dwant)
    rec = orc.reconstruct(host(pg, out))
    assert np.max(np.abs(orc.decode(rec[0]) - L["maxpool_mnist_output"])) <= 1e-3


# ------------------------------------------------------------------- glue ops

def test_glue_kernels(pg, ctx, golden):
    import torch

    kat = golden[0]
    c = kat["Maxpool_Im2Row"]
    p = c["params"]
    im = np.array([int(v) for v in c["arrays"]["im"]], dtype=U64)
    want = orc.maxpool_im2row(im, p["H"], p["W"], p["f"], p["Din"], p["batch"], p["stride"], p["pad"], p["pad_val"])
    out = torch.empty(want.size, dtype=torch.int64, device="cuda")
    pg.gpu.maxpool_im2row(ctx, torch.from_numpy(im.view(np.int64)).cuda(), out, p["H"], p["W"], p["f"], p["Din"],
                          p["batch"], p["stride"], p["pad"], p["pad_val"])
    a = rnd(600, U64, 100)
    bits = torch.empty(600 * 64, dtype=torch.int64, device="cuda")
    pg.gpu.bitexpand(ctx, torch.from_numpy(a.view(np.int64)).cuda(), bits)
    m = rnd(12 * 7, U64, 101)
    tm = torch.from_numpy(m.view(np.int64)).cuda()
    vec = rnd(12, U64, 102)
    pg.gpu.elementVectorAdd(ctx, tm, torch.from_numpy(vec.view(np.int64)).cuda(), False, 12, 7)
    red = torch.zeros(7, dtype=torch.int64, device="cuda")
    pg.gpu.reduceSum(ctx, tm, red, True, 12, 7)
    ctx.sync()
    assert np.array_equal(out.cpu().numpy().view(U64), want)
    assert np.array_equal(bits.cpu().numpy().view(U64), orc.bitexpand(a))
    m2 = orc.element_vector_add(m, vec, False, 12, 7)
    assert np.array_equal(tm.cpu().numpy().view(U64), m2)
    assert np.array_equal(red.cpu().numpy().view(U64), orc.reduce_sum(m2, np.zeros(7, U64), True, 12, 7))


def test_invalid_arguments_return_status(pg, ctx):
    import torch

    a = pg.empty_shares(10)
    with pytest.raises(pg.PiranhaError):
        pg.maxpool(ctx, a, pg.empty_shares(2), pg.empty_shares(10, "u8"), 5)  # k must be 4 or 16
    with pytest.raises(pg.PiranhaError):
        pg.convolution(ctx, a, a, a, 0, 1, 2, 2, 5, 1, 1, 1, 0, 26)  # filter larger than padded image
    # the context stays usable after an error
    out = pg.empty_shares(10)
    pg.ReLU(ctx, pg.zeros_shares(10), out, pg.empty_shares(10, "u8"))
    ctx.sync()
    assert torch.count_nonzero(out).item() == 0


def test_empty_inputs(pg, ctx):
    """Zero-length inputs: every elementwise protocol step returns without a
    launch, its messages empty and its rounds counted as the oracle counts them
    (the reference sends its empty vectors). Empty CUDA tensors have null data
    pointers, which a zero length allows."""
    import torch

    e, e8 = np.zeros((3, 2, 0), U64), np.zeros((3, 2, 0), U8)
    comm = orc.Comm()
    a, b = pg.empty_shares(0), pg.empty_shares(0)
    assert pg.reconstruct(ctx, a).shape == (3, 0)
    orc.reconstruct(e, comm)
    pg.reshare(ctx, torch.empty((3, 0), dtype=torch.int64, device="cuda"), pg.empty_shares(0))
    orc.reshare(np.zeros((3, 0), U64), comm)
    pg.mul_(ctx, a, b)
    orc.mul(e, e, comm)
    pg.and_(ctx, a, b)
    orc.and_(e, e, comm)
    pg.and_(ctx, pg.empty_shares(0, "u8"), pg.empty_shares(0, "u8"))
    orc.and_(e, e, comm)  # one round, no bytes, whatever the ring
    pg.dividePublic(ctx, a, 3)
    orc.divide_public(e.copy(), 3, comm)
    pg.dividePublic(ctx, a, torch.empty(0, dtype=torch.int64, device="cuda"))
    orc.divide_public(e.copy(), 3, comm)
    pg.dReLU(ctx, a, pg.empty_shares(0, "u8"))
    orc.drelu(e, comm=comm)
    pg.ReLU(ctx, a, pg.empty_shares(0), pg.empty_shares(0, "u8"))
    orc.relu(e, comm=comm)
    pg.selectShare(ctx, a, b, pg.empty_shares(0, "u8"), pg.empty_shares(0))
    orc.select_share(e, e, e8, comm)
    for op in (pg.OP_ADD, pg.OP_XOR):
        pg.local_(ctx, op, a, b)
    pg.local_(ctx, pg.OP_MUL, a, 5)
    # maxpool of no rows is a no-op (the reference divides by the row count)
    pg.maxpool(ctx, a, pg.empty_shares(0), pg.empty_shares(0, "u8"), 4)
    ctx.sync()
    ctx.check_device_errors()
    comm_equal(ctx, comm)
    assert ctx.comm()["rounds"] > 20


# ------------------------------------------------------------ local operators

@pytest.mark.parametrize("op,kind", [("add", "scalar"), ("sub", "scalar"), ("mul", "scalar"), ("shr", "scalar"),
                                     ("add", "public"), ("sub", "public"), ("mul", "public"), ("xor", "public"),
                                     ("and", "public"), ("shr", "public"), ("shl", "public"),
                                     ("add", "shares"), ("sub", "shares"), ("xor", "shares")])
def test_rss_local(pg, ctx, op, kind):
    import torch

    n = 5003
    a = orc.random_views(n, U64, 60)
    rng = np.random.default_rng(61)
    if kind == "scalar":
        rhs_np = int(rng.integers(0, 70)) if op == "shr" else int(rng.integers(0, 2**63))
        rhs_dev = rhs_np
    elif kind == "public":
        rhs_np = rng.integers(0, 70, n, dtype=U64) if op in ("shr", "shl") else \
            rng.integers(0, 2**64 - 1, n, dtype=U64, endpoint=True)
        rhs_dev = torch.from_numpy(rhs_np.view(np.int64)).cuda()
    else:
        rhs_np = orc.random_views(n, U64, 62)
        rhs_dev = dev(pg, rhs_np)
    ops = {"add": pg.OP_ADD, "sub": pg.OP_SUB, "mul": pg.OP_MUL, "xor": pg.OP_XOR, "and": pg.OP_AND,
           "shr": pg.OP_SHR, "shl": pg.OP_SHL}
    da = dev(pg, a)
    pg.local_(ctx, ops[op], da, rhs_dev)
    ctx.sync()
    assert np.array_equal(host(pg, da), orc.rss_local(op, a, rhs_np))
    assert ctx.comm()["rounds"] == 0


def test_rss_local_unsupported(pg, ctx):
    a = dev(pg, orc.random_views(10, U64, 63))
    for op in (pg.OP_MUL, pg.OP_AND):  # protocol steps, not local operators
        with pytest.raises(pg.PiranhaError):
            pg.local_(ctx, op, a, a)
    with pytest.raises(pg.PiranhaError):
        pg.local_(ctx, pg.OP_XOR, a, 5)
