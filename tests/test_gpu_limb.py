"""The 8-bit-limb tensor-core form (tcgen05) against the CPU oracle, bit for bit.

Covers the single-MMA self test (descriptor and tensor-memory layout), the
fused share-GEMM and implicit-GEMM conv at several shapes (including split-K
and tile-ragged edges), the digit-magnitude worst case (every product at
2^14, so every fp32 accumulator reaches exactly 2^24 per chunk), and a full
VGG16 forward in the limb form.
"""
import ctypes

import numpy as np
import pytest

import oracle as orc
from oracle import netref

pytestmark = pytest.mark.gpu

U64 = np.uint64


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
    # no timing-based choices here: every call runs the limb kernel, with the
    # heuristic split-K (the tuner has its own tests below)
    c = pg.Context(0, form=pg.FORM_LIMB_TC)
    c.set_autotune(False)
    yield c
    c.check_device_errors()
    c.close()


def test_tc_selftest(pg, ctx):
    import torch

    rng = np.random.default_rng(1)
    A = rng.integers(-128, 128, size=(128, 16)).astype(np.float16)
    B = rng.integers(-128, 128, size=(64, 16)).astype(np.float16)
    ta = torch.from_numpy(A.view(np.int16)).cuda()
    tb = torch.from_numpy(B.view(np.int16)).cuda()
    D = torch.zeros((128, 64), dtype=torch.float32, device="cuda")
    st = pg.lib().pg_tc_selftest(ctx.handle, ctypes.c_void_p(ta.data_ptr()), ctypes.c_void_p(tb.data_ptr()),
                                 ctypes.c_void_p(D.data_ptr()))
    ctx._check(st)
    ctx.check_device_errors()
    want = A.astype(np.float64) @ B.astype(np.float64).T
    assert np.array_equal(D.cpu().numpy().astype(np.float64), want)


@pytest.mark.parametrize("M,N,K,tA,tB,tC", [
    (128, 64, 16, 1, 1, 1),     # one tile, one stage
    (128, 128, 512, 1, 1, 1),   # FC-like
    (200, 70, 144, 1, 0, 1),    # ragged tiles, B column-major
    (64, 256, 256, 0, 1, 0),    # A column-major, C column-major
    (32, 32, 2048, 1, 1, 1),    # split-K over many chunks
    (128, 10, 784, 1, 1, 1),    # SecureML-like output layer
    (300, 20, 16, 1, 1, 1),     # M not a multiple of 32: zero rows pad the last line
    (256, 128, 512, 1, 1, 1),   # two row and two column tiles with split-K
])
def test_limb_matmul(pg, ctx, M, N, K, tA, tB, tC):
    a, b = orc.random_views(M * K, U64, 3), orc.random_views(K * N, U64, 4)
    comm = orc.Comm()
    want = orc.matmul(a, b, M, N, K, tA, tB, tC, 26, comm)
    c = pg.empty_shares(M * N)
    pg.matmul(ctx, pg.to_device(a), pg.to_device(b), c, M, N, K, tA, tB, tC, 26)
    ctx.check_device_errors()
    assert np.array_equal(pg.to_host(c), want)
    cc = ctx.comm()
    assert cc["tx"] == comm.tx and cc["rounds"] == comm.rounds


def test_limb_matmul_odd_k(pg, ctx):
    M, N, K = 20, 30, 25  # K not a multiple of 16: zero digits pad the contraction
    a, b = orc.random_views(M * K, U64, 5), orc.random_views(K * N, U64, 6)
    want = orc.matmul(a, b, M, N, K, 1, 1, 1, 20)
    c = pg.empty_shares(M * N)
    pg.matmul(ctx, pg.to_device(a), pg.to_device(b), c, M, N, K, 1, 1, 1, 20)
    ctx.sync()
    assert np.array_equal(pg.to_host(c), want)


@pytest.mark.parametrize("fill", [0, (1 << 64) - 1, 0x8080808080808080, 0x7F7F7F7F7F7F7F7F, 0x7F7F7F7F7F7F7F80])
def test_limb_digit_extremes(pg, ctx, fill):
    """Constant operands put every digit at an extreme: 0x7F..7F80 has all digits -128, so every
    product is 2^14 and each accumulator reaches exactly 2^24 per chunk."""
    M, N, K = 128, 64, 1024
    a = np.full((3, 2, M * K), fill, dtype=U64)
    b = np.full((3, 2, K * N), fill, dtype=U64)
    want = orc.matmul(a, b, M, N, K, 1, 1, 1, 13)
    c = pg.empty_shares(M * N)
    pg.matmul(ctx, pg.to_device(a), pg.to_device(b), c, M, N, K, 1, 1, 1, 13)
    ctx.check_device_errors()
    assert np.array_equal(pg.to_host(c), want)


@pytest.mark.parametrize("batch,H,W,f,Din,Dout,stride,pad", [
    (2, 8, 8, 3, 16, 64, 1, 1),
    (3, 5, 5, 3, 32, 70, 2, 1),
    (2, 4, 4, 3, 64, 128, 1, 1),
    (1, 2, 2, 3, 128, 64, 1, 1),
    (2, 6, 6, 1, 16, 16, 1, 0),
    (2, 8, 8, 3, 3, 64, 1, 1),      # Din = 3: im2col image, K = 27 padded to 32
    (9, 4, 4, 3, 16, 16, 1, 1),     # whole-image tiles, the last one ragged
    (1, 4, 4, 3, 16, 16, 1, 2),     # padding wider than the kernel reach: im2col image
    (2, 12, 12, 5, 20, 50, 1, 0),   # LeNet-like 5x5, Din = 20
    (1, 32, 32, 3, 64, 64, 1, 1),   # one VGG row tile: 4 rows x 32 columns
    (1, 5, 40, 3, 16, 16, 1, 1),    # wider than one 32-pixel line: tiles along w
    (1, 3, 70, 1, 16, 8, 1, 0),     # ragged last w tile
    (2, 16, 16, 3, 64, 128, 1, 1),  # two N tiles, four row tiles of 8 x 16 pixels
    (4, 32, 32, 3, 64, 64, 1, 1),   # 32 row tiles of 4 x 32 pixels
])
def test_limb_conv(pg, ctx, batch, H, W, f, Din, Dout, stride, pad):
    A = orc.random_views(batch * H * W * Din, U64, 7)
    B = orc.random_views(Dout * f * f * Din, U64, 8)
    want = orc.convolution(A, B, orc.FPROP, batch, H, W, f, Din, Dout, stride, pad, 26)
    C = pg.empty_shares(want.shape[2])
    pg.convolution(ctx, pg.to_device(A), pg.to_device(B), C, orc.FPROP, batch, H, W, f, Din, Dout, stride, pad, 26)
    ctx.check_device_errors()
    assert np.array_equal(pg.to_host(C), want)


@pytest.mark.parametrize("op", [orc.DGRAD, orc.WGRAD])
@pytest.mark.parametrize("batch,H,W,f,Din,Dout,stride,pad", [
    (3, 28, 28, 5, 1, 20, 1, 0),    # LeNet conv 1: one input channel
    (4, 12, 12, 5, 20, 50, 1, 0),   # LeNet conv 2: odd channel counts
    (2, 8, 8, 3, 64, 64, 1, 1),     # VGG-like, padded
    (2, 9, 7, 3, 5, 7, 2, 1),       # strided, ragged
    (1, 5, 5, 5, 3, 2, 1, 2),       # filter as wide as the padding allows
])
def test_limb_conv_backward(pg, ctx, op, batch, H, W, f, Din, Dout, stride, pad):
    """Input gradient (dY x W into column products, then col2im and one
    truncation) and weight gradient (the forward input's transposed im2col x
    dY) against the oracle's dgrad / wgrad convolutions."""
    P, Q = (H + 2 * pad - f) // stride + 1, (W + 2 * pad - f) // stride + 1
    A = orc.random_views(batch * P * Q * Dout, U64, 17)
    nb = Dout * f * f * Din if op == orc.DGRAD else batch * H * W * Din
    B = orc.random_views(nb, U64, 18)
    comm = orc.Comm()
    want = orc.convolution(A, B, op, batch, H, W, f, Din, Dout, stride, pad, 26, comm)
    C = pg.empty_shares(want.shape[2])
    pg.convolution(ctx, pg.to_device(A), pg.to_device(B), C, op, batch, H, W, f, Din, Dout, stride, pad, 26)
    ctx.check_device_errors()
    assert np.array_equal(pg.to_host(C), want)
    got = ctx.comm()
    assert got["tx"] == comm.tx and got["rx"] == comm.rx and got["rounds"] == comm.rounds


def test_limb_vgg16_forward(pg):
    from tests.test_gpu_network import run_net

    layers = netref.vgg16_layers()
    params = netref.kaiming_uniform_params(layers, 21)
    batch = 2
    rng = np.random.default_rng(22)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 3072)), seed=23)
    want, want_outs = netref.forward(layers, params, x, batch, keep=True)
    got, got_outs, _ = run_net(pg, layers, params, x, batch, capture=True, form=pg.FORM_LIMB_TC)
    for i, (g, w) in enumerate(zip(got_outs, want_outs)):
        assert np.array_equal(g, w), f"layer {i} {layers[i]}"
    assert np.array_equal(got, want)


@pytest.mark.parametrize("M,N,K", [(128, 64, 4096), (256, 200, 1000), (2, 10, 784)])
def test_limb_split_autotune(pg, M, N, K):
    """The split-K autotuner (timed candidates, cached per shape) and the
    heuristic split give the same bits as the oracle."""
    A = orc.random_views(M * K, U64, 41)
    B = orc.random_views(K * N, U64, 42)
    want = orc.matmul(A, B, M, N, K, 1, 1, 1, 26)
    for tune in (True, False):
        c = pg.Context(0, form=pg.FORM_LIMB_TC)
        c.set_autotune(tune)
        for _ in range(2):  # the second call uses the cached choice
            C = pg.empty_shares(M * N)
            pg.matmul(c, pg.to_device(A), pg.to_device(B), C, M, N, K, 1, 1, 1, 26)
            c.check_device_errors()
            assert np.array_equal(pg.to_host(C), want)
        c.close()


def test_alloc_shares(pg, ctx):
    import torch

    vp = ctypes.c_void_p
    out = (vp * 6)()
    ctx._check(pg.lib().pg_alloc_shares(ctx.handle, 6, 1000, 8, out))
    ptrs = [out[i] for i in range(6)]
    assert all(p % 256 == 0 for p in ptrs) and len(set(ptrs)) == 6
    ctx.sync()

    class _A:
        def __init__(self, p):
            self.__cuda_array_interface__ = {"shape": (1000,), "typestr": "<i8", "data": (p, False), "version": 3}

    for p in ptrs:
        assert int(torch.as_tensor(_A(p), device="cuda").abs().sum()) == 0
    ctx._check(pg.lib().pg_free_shares(ctx.handle, vp(ptrs[0])))


def test_tune_cache_round_trip(pg, tmp_path):
    """Tuned split-K choices saved to a file and loaded into another context,
    which then reuses them (same bits)."""
    M, N, K = 128, 64, 2048
    A = orc.random_views(M * K, U64, 51)
    B = orc.random_views(K * N, U64, 52)
    want = orc.matmul(A, B, M, N, K, 1, 1, 1, 26)
    path = str(tmp_path / "tune.txt")
    c1 = pg.Context(0, form=pg.FORM_LIMB_TC)
    C = pg.empty_shares(M * N)
    pg.matmul(c1, pg.to_device(A), pg.to_device(B), C, M, N, K, 1, 1, 1, 26)
    c1.tune_save(path)
    c1.close()
    lines = open(path).read().split("\n")
    assert lines[0].startswith("pg-tune ") and len([x for x in lines[1:] if x.strip()]) >= 1
    c2 = pg.Context(0, form=pg.FORM_LIMB_TC)
    c2.tune_load(path)
    C2 = pg.empty_shares(M * N)
    pg.matmul(c2, pg.to_device(A), pg.to_device(B), C2, M, N, K, 1, 1, 1, 26)
    c2.check_device_errors()
    assert np.array_equal(pg.to_host(C2), want) and np.array_equal(pg.to_host(C), want)
    with open(path, "w") as f:
        f.write("pg-tune 1\n")
    with pytest.raises(pg.PiranhaError):
        c2.tune_load(path)
    c2.close()


def test_form_pick_same_bits(pg, tmp_path):
    """With autotuning on, a standalone call runs in whichever form timed
    faster for its shape (cached in the tuning file as sform/...): the bits
    are those of the oracle either way."""
    cases = [("conv", (orc.WGRAD, 4, 28, 28, 5, 1, 20, 1, 0)), ("conv", (orc.DGRAD, 4, 12, 12, 5, 20, 50, 1, 0)),
             ("mm", (64, 10, 256))]
    c = pg.Context(0, form=pg.FORM_LIMB_TC)
    for kind, args in cases:
        if kind == "conv":
            op, batch, H, W, f, Din, Dout, stride, pad = args
            P, Q = (H + 2 * pad - f) // stride + 1, (W + 2 * pad - f) // stride + 1
            A = orc.random_views(batch * P * Q * Dout, U64, 91)
            nb = Dout * f * f * Din if op == orc.DGRAD else batch * H * W * Din
            B = orc.random_views(nb, U64, 92)
            want = orc.convolution(A, B, op, batch, H, W, f, Din, Dout, stride, pad, 26)
            for _ in range(2):
                C = pg.empty_shares(want.shape[2])
                pg.convolution(c, pg.to_device(A), pg.to_device(B), C, op, batch, H, W, f, Din, Dout, stride, pad, 26)
                c.check_device_errors()
                assert np.array_equal(pg.to_host(C), want)
        else:
            M, N, K = args
            A, B = orc.random_views(M * K, U64, 93), orc.random_views(K * N, U64, 94)
            want = orc.matmul(A, B, M, N, K, 1, 1, 1, 26)
            for _ in range(2):
                C = pg.empty_shares(M * N)
                pg.matmul(c, pg.to_device(A), pg.to_device(B), C, M, N, K, 1, 1, 1, 26)
                c.check_device_errors()
                assert np.array_equal(pg.to_host(C), want)
    path = str(tmp_path / "t.txt")
    c.tune_save(path)
    assert sum(1 for line in open(path) if line.startswith("sform/")) == 3
    c.close()
