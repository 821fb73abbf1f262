"""Average pool layer (AveragepoolLayer.cu) on the GPU against the oracle, bit
for bit: forward, backward, and networks that use it (the reference's own
VGG16 with its five averagepool layers; a training step through one)."""
import numpy as np
import pytest

import oracle as orc
from oracle import netref
from tests.test_gpu_network import run_net
from tests.test_gpu_train import check_against_oracle, make_net, one_hot_labels, oracle_step

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    pg.lib()
    return pg


@pytest.mark.parametrize("H,W,C,pool,stride,batch", [(8, 8, 4, 2, 2, 3), (9, 9, 2, 3, 3, 2), (2, 2, 2, 2, 1, 2),
                                                     (32, 32, 64, 2, 2, 2)])
def test_avgpool_forward_backward(pg, H, W, C, pool, stride, batch):
    x = orc.random_views(batch * H * W * C, seed=1)
    comm = orc.Comm()
    want = orc.avgpool_layer(x, H, W, C, pool, stride, batch, comm)
    ctx = pg.Context(0)
    out = pg.empty_shares(want.shape[2])
    pg.avgpool_layer(ctx, pg.to_device(x), out, H, W, C, pool, stride, batch)
    ctx.sync()
    assert np.array_equal(pg.to_host(out), want)
    got = ctx.comm()
    assert got["tx"] == comm.tx and got["rounds"] == comm.rounds
    delta = orc.random_views(want.shape[2], seed=2)
    dwant = orc.avgpool_layer_backward(delta, H, W, C, pool, batch)
    din = pg.empty_shares(batch * H * W * C)
    pg.avgpool_backward(ctx, pg.to_device(delta), din, H, W, C, pool, stride, batch)
    ctx.sync()
    assert np.array_equal(pg.to_host(din), dwant)
    ctx.close()


@pytest.mark.parametrize("form", [0, 1])
def test_vgg16_averagepool_forward_batch2(pg, form):
    """The reference's own files/models/vgg16-cifar10.json, averagepool layers kept."""
    layers = netref.vgg16_layers(maxpool=False)
    params = netref.kaiming_uniform_params(layers, 5)
    batch = 2
    rng = np.random.default_rng(6)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 3072)), seed=7)
    want, want_outs = netref.forward(layers, params, x, batch, keep=True)
    got, got_outs, _ = run_net(pg, layers, params, x, batch, capture=True, form=form)
    for i, (g, w) in enumerate(zip(got_outs, want_outs)):
        assert np.array_equal(g, w), f"layer {i} {layers[i]}"
    assert np.array_equal(got, want)


def test_training_step_through_averagepool(pg):
    layers = [("cnn", 8, 8, 1, 4, 3, 1, 1), ("avgpool", 8, 8, 4, 2, 2), ("relu", 64), ("fc", 64, 10), ("relu", 10)]
    params = netref.kaiming_uniform_params(layers, 8)
    batch = 8
    rng = np.random.default_rng(9)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 64)), seed=10)
    labels = one_hot_labels(batch, 10, 11)
    outs, new_params, deltas, softmax = oracle_step(layers, params, x, labels, batch, 5)
    ctx = pg.Context(0)
    net = make_net(pg, ctx, layers, params, batch)
    net.train_step(pg.to_device(x), pg.to_device(labels), 5)
    ctx.sync()
    check_against_oracle(pg, net, layers, outs, new_params, deltas, softmax)
    net.close()
    ctx.close()
