"""The implicit weight gradient of the limb form (stride 1, a multiple of 16
images): rows (filter tap, input channel) from one digit image of the forward
input, each tap a shift of the image's pixel coordinate, K over the output
pixels whose tap lands inside the input (16 images per stage), the packed
operand the output gradient. Every share of dW against the oracle's
convolution with the CUTLASS Wgrad problem semantics, at LeNet's and VGG16's
shapes and ragged ones (one input channel, channels not a multiple of 8,
more than one 128-channel tile, 2x2 images), with the heuristic split and
with the tuner; a stride-2 case keeps the explicit gather."""
import numpy as np
import pytest

import oracle as orc

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
    # batch, H, W, Din, Dout, f, stride, pad
    (16, 28, 28, 1, 20, 5, 1, 0),     # LeNet conv 1
    (32, 12, 12, 20, 50, 5, 1, 0),    # LeNet conv 2
    (16, 8, 8, 16, 32, 3, 1, 1),
    (16, 4, 4, 136, 64, 3, 1, 1),
    (16, 2, 2, 64, 64, 3, 1, 1),
    (48, 5, 3, 24, 70, 3, 1, 1),
    (16, 8, 8, 16, 16, 3, 2, 1),      # stride 2: explicit gather
]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("autotune", [False, True])
def test_wgrad_equals_oracle(pg, shape, autotune):
    batch, H, W, Din, Dout, f, stride, pad = shape
    P, Q = (H + 2 * pad - f) // stride + 1, (W + 2 * pad - f) // stride + 1
    dy = orc.random_views(batch * P * Q * Dout, U64, 300 + Din)
    x = orc.random_views(batch * H * W * Din, U64, 400 + Dout)
    want = orc.convolution(dy, x, orc.WGRAD, batch, H, W, f, Din, Dout, stride, pad, 26)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    ctx.set_autotune(autotune)  # on: the form and the split-K by timing, as the training step runs it
    out = pg.empty_shares(Dout * f * f * Din)
    pg.convolution(ctx, pg.to_device(dy), pg.to_device(x), out, pg.WGRAD, batch, H, W, f, Din, Dout, stride, pad,
                   26)
    ctx.check_device_errors()
    assert np.array_equal(pg.to_host(out), want)
    ctx.close()
