"""Training-step parity: the GPU executor's forward + backward + SGD update
against the oracle's restatement, bit for bit — every layer's outputs, every
gradient passed between layers, the softmax gradient, and every updated
weight and bias share — plus the message counters."""
import numpy as np
import pytest

import oracle as orc
from oracle import netref
from tests.test_gpu_network import _wrap_device, gather

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    pg.lib()
    return pg


def one_hot_labels(batch, classes, seed):
    rng = np.random.default_rng(seed)
    y = np.zeros((batch, classes))
    y[np.arange(batch), rng.integers(0, classes, batch)] = 1.0
    return orc.set_public(y.ravel())


def make_net(pg, ctx, layers, params, batch):
    net = pg.Network(ctx, layers, batch)
    for i, prm in enumerate(params):
        if prm is not None:
            net.set_params(i, pg.to_device(prm[0]), pg.to_device(prm[1]) if prm[1] is not None else None)
    return net


def fill(ptrs, views):
    """Copy (3, 2, n) views into a contiguous [6][n] device block."""
    import torch

    n = views.shape[2]
    dst = _wrap_device(ptrs[0], 6 * n)
    dst.copy_(torch.from_numpy(np.ascontiguousarray(views).reshape(-1).view(np.int64)).cuda())
    torch.cuda.synchronize()


def check_against_oracle(pg, net, layers, want_outs, want_params, want_deltas, want_softmax):
    for i in range(len(layers)):
        optrs, n = net.layer_output_ptrs(i)
        assert np.array_equal(gather(pg, optrs, n), want_outs[i]), f"output of layer {i} {layers[i]}"
    dptrs, n = net.layer_delta_ptrs(-1)
    assert np.array_equal(gather(pg, dptrs, n), want_softmax), "softmax gradient"
    for i in range(len(layers)):
        dptrs, n = net.layer_delta_ptrs(i)
        assert np.array_equal(gather(pg, dptrs, n), want_deltas[i]), f"gradient out of layer {i} {layers[i]}"
        if want_params[i] is not None:
            w, wn, b, bn = net.layer_param_ptrs(i)
            assert np.array_equal(gather(pg, w, wn), want_params[i][0]), f"weights of layer {i}"
            if want_params[i][1] is not None:
                assert np.array_equal(gather(pg, b, bn), want_params[i][1]), f"bias of layer {i}"


def oracle_step(layers, params, x, labels, batch, log_lr, comm=None):
    bits = []
    _, outs = netref.forward(layers, params, x, batch, keep=True, bits=bits, comm=comm)
    softmax = orc.reveal_softmax_grad(outs[-1], labels, batch)
    new_params, deltas = netref.backward(layers, params, x, outs, bits, labels, batch, log_lr=log_lr, comm=comm)
    return outs, new_params, deltas, softmax


@pytest.mark.parametrize("form", ["u64", "tc"])
def test_secureml_fixture_training_step(pg, golden, form):
    """One SGD iteration of the SecureML net on the reference's training
    fixture (learning rate 2^-9), every share against the oracle."""
    L = golden[1]
    layers = netref.secureml_layers()
    params = []
    for li in (0, 2, 4):
        params += [(orc.set_public(L[f"secureml_weight{li}"]), orc.set_public(L[f"secureml_bias{li}"])), None]
    x = orc.set_public(L["secureml_input"])
    labels = orc.set_public(L["secureml_labels"])
    comm = orc.Comm()
    outs, new_params, deltas, softmax = oracle_step(layers, params, x, labels, 128, 9)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC if form == "tc" else pg.FORM_U64)
    ctx.set_autotune(False)  # every share-GEMM / conv then runs in the form under test
    net = make_net(pg, ctx, layers, params, 128)
    ctx.reset_comm()
    net.train_step(pg.to_device(x), pg.to_device(labels), 9)
    ctx.sync()
    check_against_oracle(pg, net, layers, outs, new_params, deltas, softmax)
    ctx.check_device_errors()
    net.close()
    ctx.close()


def test_training_step_counters(pg):
    layers = netref.secureml_layers()
    params = netref.kaiming_uniform_params(layers, 3)
    batch = 16
    rng = np.random.default_rng(4)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 784)), seed=5)
    labels = one_hot_labels(batch, 10, 6)
    # the forward's FC layers are accounted by netref.forward itself
    comm = orc.Comm()
    oracle_step(layers, params, x, labels, batch, 5, comm)
    ctx = pg.Context(0)
    net = make_net(pg, ctx, layers, params, batch)
    ctx.reset_comm()
    net.train_step(pg.to_device(x), pg.to_device(labels), 5)
    ctx.sync()
    got = ctx.comm()
    assert got["tx"] == comm.tx and got["rx"] == comm.rx and got["rounds"] == comm.rounds, (got, comm.tx, comm.rounds)
    net.close()
    ctx.close()


@pytest.mark.parametrize("form", ["u64", "tc"])
def test_lenet_training_step(pg, form):
    """LeNet (files/models/lenet.json: conv-maxpool-relu x2, FC-relu-FC-relu)
    at batch 8, log learning rate 5, random input shares."""
    layers = netref.lenet_layers()
    params = netref.kaiming_uniform_params(layers, 11)
    batch = 8
    rng = np.random.default_rng(12)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 784)), seed=13)
    labels = one_hot_labels(batch, 10, 14)
    outs, new_params, deltas, softmax = oracle_step(layers, params, x, labels, batch, 5)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC if form == "tc" else pg.FORM_U64)
    ctx.set_autotune(False)  # every share-GEMM / conv then runs in the form under test
    net = make_net(pg, ctx, layers, params, batch)
    net.train_step(pg.to_device(x), pg.to_device(labels), 5)
    ctx.sync()
    check_against_oracle(pg, net, layers, outs, new_params, deltas, softmax)
    ctx.check_device_errors()
    net.close()
    ctx.close()


@pytest.mark.parametrize("form", ["u64", "tc"])
def test_lenet_training_captured_two_steps(pg, form):
    """The captured training step: the capture's eager warm-up leaves the
    parameters as they were, and two graph replays are two SGD iterations."""
    layers = netref.lenet_layers()
    params = netref.kaiming_uniform_params(layers, 21)
    batch = 4
    rng = np.random.default_rng(22)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 784)), seed=23)
    labels = one_hot_labels(batch, 10, 24)
    _, p1, _, _ = oracle_step(layers, params, x, labels, batch, 6)
    outs2, p2, deltas2, softmax2 = oracle_step(layers, p1, x, labels, batch, 6)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC if form == "tc" else pg.FORM_U64)
    ctx.set_autotune(False)  # every share-GEMM / conv then runs in the form under test
    net = make_net(pg, ctx, layers, params, batch)
    net.train_step(pg.to_device(x), pg.to_device(labels), 6)  # sets up the training buffers eagerly
    for i, prm in enumerate(params):  # back to the initial parameters
        if prm is not None:
            net.set_params(i, pg.to_device(prm[0]), pg.to_device(prm[1]) if prm[1] is not None else None)
    fill(net.input_buffers(), x)
    fill(net.label_buffers(), labels)
    net.capture_train(6)
    net.train_resident()
    net.train_resident()
    ctx.sync()
    check_against_oracle(pg, net, layers, outs2, p2, deltas2, softmax2)
    net.close()
    ctx.close()


def test_train_host_buffers(pg):
    """pg_net_train_host: pinned host input and labels in, the forward's output
    shares out, the parameters updated on the device."""
    import torch

    layers = netref.secureml_layers()
    params = netref.kaiming_uniform_params(layers, 31)
    batch = 32
    rng = np.random.default_rng(32)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 784)), seed=33)
    labels = one_hot_labels(batch, 10, 34)
    outs, new_params, _, _ = oracle_step(layers, params, x, labels, batch, 7)
    ctx = pg.Context(0)
    net = make_net(pg, ctx, layers, params, batch)
    xin = torch.from_numpy(np.ascontiguousarray(x).reshape(-1).view(np.int64)).pin_memory()
    lin = torch.from_numpy(np.ascontiguousarray(labels).reshape(-1).view(np.int64)).pin_memory()
    out = torch.empty(6 * net.out_n, dtype=torch.int64).pin_memory()
    net.train_host(xin.data_ptr(), lin.data_ptr(), out.data_ptr(), 7)
    ctx.sync()
    assert np.array_equal(out.numpy().view(np.uint64).reshape(3, 2, -1), outs[-1])
    for i, prm in enumerate(new_params):
        if prm is not None:
            w, wn, b, bn = net.layer_param_ptrs(i)
            assert np.array_equal(gather(pg, w, wn), prm[0])
            assert np.array_equal(gather(pg, b, bn), prm[1])
    net.close()
    ctx.close()


def _model(name):
    import json
    import os

    models = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "models.json")))
    return models


@pytest.mark.parametrize("name", ["minionn", "sarda", "lenet-norelu-avgpool"])
@pytest.mark.parametrize("form", ["u64", "tc"])
def test_reference_model_files_training_step(pg, name, form):
    """Training steps of networks read from the reference's model files
    (MiniONN, Sarda's 2x2 stride-2 convolution, LeNet with 2x2/2 average
    pools) at batch 4: every output, gradient and updated parameter share
    equals the oracle's."""
    models = _model(name)
    layers = [tuple(L) for L in models[name]["layers"]]
    params = netref.kaiming_uniform_params(layers, 61)
    batch = 4
    rng = np.random.default_rng(62)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * models[name]["meta"]["input_size"])), seed=63)
    labels = one_hot_labels(batch, 10, 64)
    outs, new_params, deltas, softmax = oracle_step(layers, params, x, labels, batch, 5)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC if form == "tc" else pg.FORM_U64)
    ctx.set_autotune(False)
    net = make_net(pg, ctx, layers, params, batch)
    net.train_step(pg.to_device(x), pg.to_device(labels), 5)
    ctx.sync()
    check_against_oracle(pg, net, layers, outs, new_params, deltas, softmax)
    ctx.check_device_errors()
    net.close()
    ctx.close()


def test_alexnet_training_refused_on_overlapping_average_pool(pg):
    """AlexNet's first average pool overlaps (3x3, stride 2: 16 windows x 9 >
    100 inputs). The reference's averagepool backward expands each delta into
    pool^2 slots as for a pool that tiles the image and would write past its
    input-gradient buffer; the library refuses the step with a status (before
    any launch) and so does the oracle, while the forward runs."""
    models = _model("alexnet-cifar10")
    layers = [tuple(L) for L in models["alexnet-cifar10"]["layers"]]
    params = netref.kaiming_uniform_params(layers, 81)
    batch = 2
    rng = np.random.default_rng(82)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 3072)), seed=83)
    labels = one_hot_labels(batch, 10, 84)
    with pytest.raises(ValueError, match="overlapping"):
        oracle_step(layers, params, x, labels, batch, 5)
    ctx = pg.Context(0, form=pg.FORM_U64)
    ctx.set_autotune(False)
    net = make_net(pg, ctx, layers, params, batch)
    with pytest.raises(pg.PiranhaError, match="overlapping"):
        net.train_step(pg.to_device(x), pg.to_device(labels), 5)
    ctx.sync()
    ctx.check_device_errors()
    net.close()
    # the context is still usable: a fresh network's forward equals the oracle's
    net = make_net(pg, ctx, layers, params, batch)
    out = pg.empty_shares(net.out_n)
    net.forward(pg.to_device(x), out)
    ctx.sync()
    assert np.array_equal(pg.to_host(out).reshape(3, 2, -1), netref.forward(layers, params, x, batch))
    net.close()
    ctx.close()


def test_training_step_flipped_input_gradient(pg, tmp_path):
    """A training step whose convolutions' input gradients run as convolutions
    of dY with the flipped filter (forced through tuning-cache entries), on
    position-major tiles at 128 images: bit-exact against the oracle."""
    import torch

    layers = [("cnn", 8, 8, 16, 32, 3, 1, 1), ("relu", 2048), ("cnn", 8, 8, 32, 32, 3, 1, 1), ("relu", 2048),
              ("fc", 2048, 10), ("relu", 10)]
    params = netref.kaiming_uniform_params(layers, 71)
    batch = 128
    rng = np.random.default_rng(72)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 8 * 8 * 16)), seed=73)
    labels = one_hot_labels(batch, 10, 74)
    outs, new_params, deltas, softmax = oracle_step(layers, params, x, labels, batch, 5)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    cache = tmp_path / "tune.txt"
    cache.write_text(f"pg-tune {sms}\nsform/conv/1/128/8/8/3/16/32/1/1 3 1\nsform/conv/1/128/8/8/3/32/32/1/1 3 1\n")
    ctx.tune_load(str(cache))
    ctx.set_autotune(False)
    net = make_net(pg, ctx, layers, params, batch)
    net.train_step(pg.to_device(x), pg.to_device(labels), 5)
    ctx.sync()
    check_against_oracle(pg, net, layers, outs, new_params, deltas, softmax)
    ctx.check_device_errors()
    net.close()
    ctx.close()



def test_inference_forward_keeps_relu_outputs_as_digit_images(pg):
    """Before the training buffers exist a forward is an inference forward: a
    ReLU that feeds a limb-form convolution keeps its output only as that
    convolution's digit image, and reading the layer rebuilds the six shares
    from the image. Every reading follows the last forward that ran: the
    captured inference graph, an eager training step (which writes every
    layer output), then the inference graph again with the updated weights.
    A backward right after an inference forward is refused."""
    layers = [("cnn", 8, 8, 16, 16, 3, 1, 1), ("relu", 1024), ("cnn", 8, 8, 16, 16, 3, 1, 1),
              ("maxpool", 8, 8, 16, 2, 2), ("relu", 256), ("cnn", 4, 4, 16, 32, 3, 1, 1), ("relu", 512),
              ("fc", 512, 10), ("relu", 10)]
    params = netref.kaiming_uniform_params(layers, 61)
    batch = 16
    rng = np.random.default_rng(62)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 1024)), seed=63)
    labels = one_hot_labels(batch, 10, 64)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    ctx.set_autotune(False)  # every convolution in the limb form, so that the ReLUs write digit images
    net = make_net(pg, ctx, layers, params, batch)
    net.capture()
    fill(net.input_buffers(), x)

    def check_forward(prm, what):
        _, want = netref.forward(layers, prm, x, batch, keep=True)
        for i in range(len(layers)):
            optrs, n = net.layer_output_ptrs(i)
            assert np.array_equal(gather(pg, optrs, n), want[i]), f"{what}: output of layer {i} {layers[i]}"

    net.forward_resident()
    ctx.sync()
    check_forward(params, "inference graph")
    with pytest.raises(pg.PiranhaError):
        net.backward(pg.to_device(x), pg.to_device(labels), 5)
    outs, new_params, deltas, softmax = oracle_step(layers, params, x, labels, batch, 5)
    net.train_step(pg.to_device(x), pg.to_device(labels), 5)
    ctx.sync()
    check_against_oracle(pg, net, layers, outs, new_params, deltas, softmax)
    net.forward_resident()
    ctx.sync()
    check_forward(new_params, "inference graph after the training step")
    ctx.check_device_errors()
    net.close()
    ctx.close()
