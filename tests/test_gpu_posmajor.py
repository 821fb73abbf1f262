"""Position-major tiles of the limb convolution (same convolutions of at most
1024 output positions per image, batch a multiple of 128): a tile is one output
pixel of 128 images and runs only the taps that fall inside the input. Every
share against the oracle, bit for bit, at the shapes of VGG16's small layers
and at ragged ones (non-square images, 5x5 filters, output channels that are
not a multiple of the 64-column tile, two image blocks), with the heuristic
split-K and with the tuner; and the network forward whose ReLU writes the
batch-innermost digit image these tiles read."""
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


SHAPES = [
    # batch, H, W, Din, Dout, f, pad
    (128, 2, 2, 16, 64, 3, 1),
    (128, 4, 4, 32, 128, 3, 1),
    (128, 8, 8, 16, 64, 3, 1),
    (128, 5, 3, 16, 64, 3, 1),
    (128, 4, 4, 16, 64, 5, 2),
    (128, 3, 3, 16, 72, 3, 1),
    (256, 2, 2, 32, 64, 3, 1),
    (128, 1, 1, 16, 64, 3, 1),
]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("autotune", [False, True])
def test_posmajor_conv_equals_oracle(pg, shape, autotune):
    batch, H, W, Din, Dout, f, pad = shape
    x = orc.random_views(batch * H * W * Din, U64, 100 + H * 7 + W)
    w = orc.random_views(Dout * f * f * Din, U64, 200 + Dout)
    want = orc.convolution(x, w, orc.FPROP, batch, H, W, f, Din, Dout, 1, pad, 26)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    ctx.set_autotune(autotune)
    out = pg.empty_shares(want.shape[2])
    pg.convolution(ctx, pg.to_device(x), pg.to_device(w), out, pg.FPROP, batch, H, W, f, Din, Dout, 1, pad, 26)
    ctx.check_device_errors()
    assert np.array_equal(pg.to_host(out), want)
    ctx.close()


def test_posmajor_network_forward_equals_oracle(pg):
    """A VGG-like tail at batch 128 (ReLU fused with the batch-innermost digit
    image of the next convolution), every layer against the oracle."""
    from tests.test_gpu_network import run_net

    layers = [("cnn", 8, 8, 16, 32, 3, 1, 1), ("relu", 8 * 8 * 32), ("cnn", 8, 8, 32, 64, 3, 1, 1),
              ("maxpool", 8, 8, 64, 2, 2), ("relu", 4 * 4 * 64), ("cnn", 4, 4, 64, 64, 3, 1, 1),
              ("relu", 4 * 4 * 64), ("cnn", 4, 4, 64, 128, 3, 1, 1), ("maxpool", 4, 4, 128, 2, 2),
              ("relu", 2 * 2 * 128), ("cnn", 2, 2, 128, 64, 3, 1, 1), ("relu", 2 * 2 * 64)]
    params = netref.kaiming_uniform_params(layers, 41)
    batch = 128
    rng = np.random.default_rng(42)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 8 * 8 * 16)), seed=43)
    _, want = netref.forward(layers, params, x, batch, keep=True)
    for capture in (False, True):
        _, outs, _ = run_net(pg, layers, params, x, batch, capture=capture, form=pg.FORM_LIMB_TC, autotune=True)
        for i, (g, wv) in enumerate(zip(outs, want)):
            assert np.array_equal(g, wv), f"layer {i} {layers[i]} (capture={capture})"


def _small_vgg_tail():
    return [("cnn", 8, 8, 16, 32, 3, 1, 1), ("relu", 8 * 8 * 32), ("cnn", 8, 8, 32, 64, 3, 1, 1),
            ("maxpool", 8, 8, 64, 2, 2), ("relu", 4 * 4 * 64), ("cnn", 4, 4, 64, 64, 3, 1, 1),
            ("relu", 4 * 4 * 64), ("cnn", 4, 4, 64, 128, 3, 1, 1), ("maxpool", 4, 4, 128, 2, 2),
            ("relu", 2 * 2 * 128), ("cnn", 2, 2, 128, 64, 3, 1, 1), ("relu", 2 * 2 * 64)]


def _forward(pg, ctx, layers, params, x, batch):
    from tests.test_gpu_network import gather

    net = pg.Network(ctx, layers, batch)
    for i, prm in enumerate(params):
        if prm is not None:
            net.set_params(i, pg.to_device(prm[0]), pg.to_device(prm[1]) if prm[1] is not None else None)
    out = pg.empty_shares(net.out_n)
    net.forward(pg.to_device(x), out)
    ctx.sync()
    outs = [gather(pg, *net.layer_output_ptrs(i)) for i in range(len(layers))]
    plans = [net.layer_plan(i) for i in range(len(layers))]
    net.close()
    return outs, plans


def test_tile_choice_rectangle_from_the_tuning_cache(pg, tmp_path):
    """The set-up tuner times position-major against rectangle tiles per
    convolution and caches the choice with the split-K choices; a tuning file
    that records rectangles for every layer makes the network run them, with
    the same bits."""
    layers = _small_vgg_tail()
    params = netref.kaiming_uniform_params(layers, 51)
    batch = 128
    rng = np.random.default_rng(52)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 8 * 8 * 16)), seed=53)
    _, want = netref.forward(layers, params, x, batch, keep=True)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    ctx.set_autotune(True)
    outs, plans = _forward(pg, ctx, layers, params, x, batch)
    for i, (g, w) in enumerate(zip(outs, want)):
        assert np.array_equal(g, w), f"layer {i}"
    convs = [i for i, L in enumerate(layers) if L[0] == "cnn"]
    assert all(plans[i]["form"] in (1, 2) for i in convs)
    path = tmp_path / "tune.txt"
    ctx.tune_save(str(path))
    ctx.close()
    lines = path.read_text().splitlines()
    tiles = [ln for ln in lines if ln.startswith("tile/")]
    assert len(tiles) == len(convs)
    edited = [(ln.split()[0] + " 1 1") if ln.startswith("tile/") else ln for ln in lines]
    path.write_text("\n".join(edited) + "\n")
    ctx2 = pg.Context(0, form=pg.FORM_LIMB_TC)
    ctx2.set_autotune(True)
    ctx2.tune_load(str(path))
    outs2, plans2 = _forward(pg, ctx2, layers, params, x, batch)
    ctx2.check_device_errors()
    ctx2.close()
    for i in convs:
        assert plans2[i]["form"] != 1 or plans2[i]["posmajor"] == 0, (i, plans2[i])
    for i, (g, w) in enumerate(zip(outs2, want)):
        assert np.array_equal(g, w), f"layer {i} (rectangle tiles)"
