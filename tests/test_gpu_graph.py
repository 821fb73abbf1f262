"""Stream capture of call sequences (pg_graph_begin / end / launch): a
captured 2PC and 4PC FC + ReLU forward replays to the eager result with the
eager counters, a graph stays valid after the context's scratch grows, and
capture on the legacy default stream is refused with a status.
"""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

U32, U64 = np.uint32, np.uint64


@pytest.fixture(scope="module")
def pg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    pg.lib()
    return pg


def _dev(a):
    import torch

    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(np.int32 if a.dtype == U32 else np.int64)).cuda()


def _host(t):
    a = t.cpu().numpy()
    return a.view(U32 if a.dtype == np.int32 else U64)


@pytest.mark.parametrize("parties", [2, 4])
def test_capture_fc_relu_forward(pg, parties):
    import torch

    from piranha_gb300 import encode as enc

    proto = pg.tpc if parties == 2 else pg.fpc
    setp = enc.tpc_set_public if parties == 2 else enc.fpc_set_public
    rng = np.random.default_rng(parties)
    batch, din, dout, fp = 16, 40, 24, 10
    x = _dev(setp(rng.uniform(-1, 1, batch * din), "u32", fp))
    w = _dev(setp(rng.uniform(-1, 1, din * dout) / 8, "u32", fp))
    b = _dev(setp(np.full(dout, 0.01), "u32", fp))
    stream = torch.cuda.Stream()
    ctx = pg.Context(0, stream=stream)
    o1, o2 = proto.empty(batch * dout, "u32"), proto.empty(batch * dout, "u32")
    d = proto.zeros(batch * dout, "u8")

    def forward():
        proto.fc_forward(ctx, x, w, b, o1, batch, din, dout, fp)
        proto.ReLU(ctx, o1, o2, d)

    c0 = ctx.comm(parties)
    forward()
    ctx.sync()
    c1 = ctx.comm(parties)
    want_o2, want_d = _host(o2).copy(), d.cpu().numpy().copy()
    o2.zero_()
    d.zero_()
    l0 = ctx.kernel_launches()
    with ctx.capture() as g:
        forward()
    # capture does no work and counts nothing
    assert ctx.comm(parties) == c1 and ctx.kernel_launches() == l0
    assert not _host(o2).any()
    for _ in range(2):
        g.launch()
    ctx.sync()
    assert np.array_equal(_host(o2), want_o2)
    assert np.array_equal(d.cpu().numpy(), want_d)
    c2 = ctx.comm(parties)
    for k in ("tx", "rx"):
        assert [c - bb for c, bb in zip(c2[k], c1[k])] == [2 * (bb - a) for bb, a in zip(c1[k], c0[k])]
    assert c2["rounds"] - c1["rounds"] == 2 * (c1["rounds"] - c0["rounds"])
    assert ctx.kernel_launches() > l0
    g.close()
    ctx.close()


def test_graph_survives_scratch_growth(pg):
    """A graph keeps the scratch buffer it was captured with: growing the
    context's scratch afterwards retires that buffer instead of freeing it."""
    import torch

    stream = torch.cuda.Stream()
    ctx = pg.Context(0, stream=stream)
    rng = np.random.default_rng(7)

    def case(batch, H, W, f, Din, Dout, seed):
        A = np.stack([rng.integers(0, 2**64 - 1, batch * H * W * Din, dtype=U64, endpoint=True) for _ in range(2)])
        B = np.stack([rng.integers(0, 2**64 - 1, Dout * f * f * Din, dtype=U64, endpoint=True) for _ in range(2)])
        P, Q = H - f + 3, W - f + 3
        return A, B, pg.tpc.empty(batch * P * Q * Dout), (batch, H, W, f, Din, Dout, 1, 1)

    A, B, C, geo = case(2, 6, 6, 3, 4, 5, 1)
    want = orc.tpc_convolution(A, B, orc.FPROP, *geo, 20)
    a_d, b_d = _dev(A), _dev(B)
    pg.tpc.convolution(ctx, a_d, b_d, C, orc.FPROP, *geo, 20)  # sizes the scratch
    with ctx.capture() as g:
        pg.tpc.convolution(ctx, a_d, b_d, C, orc.FPROP, *geo, 20)
    A2, B2, C2, geo2 = case(4, 16, 16, 3, 16, 32, 2)
    pg.tpc.convolution(ctx, _dev(A2), _dev(B2), C2, orc.FPROP, *geo2, 20)  # grows the scratch
    C.zero_()
    g.launch()
    ctx.sync()
    assert np.array_equal(_host(C), want)
    g.close()
    ctx.close()


def test_capture_needs_a_stream(pg):
    import torch

    ctx = pg.Context(0, stream=torch.cuda.default_stream())
    with pytest.raises(pg.PiranhaError):
        with ctx.capture():
            pass
    ctx.close()
