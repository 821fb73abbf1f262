"""Network-level parity: the GPU executor against the oracle, layer by layer, bit for bit."""
import numpy as np
import pytest

import oracle as orc
from oracle import netref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    pg.lib()
    return pg


def _wrap_device(ptr, n):
    """A torch view of n int64 elements of existing device memory."""
    import torch

    class _A:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<i8", "data": (ptr, False), "version": 3}

    return torch.as_tensor(_A(), device="cuda")


def run_net(pg, layers, params, x, batch, capture=False, form=0, autotune=False):
    # autotune off by default: every FC / CNN layer of a limb-form network then
    # runs the limb kernels (timing could pick the u64 form for small layers)
    ctx = pg.Context(0, form=form)
    ctx.set_autotune(autotune)
    net = pg.Network(ctx, layers, batch)
    for i, prm in enumerate(params):
        if prm is not None:
            net.set_params(i, pg.to_device(prm[0]), pg.to_device(prm[1]) if prm[1] is not None else None)
    if capture:
        net.capture()
        # the network's input buffers are one contiguous [6][n] block
        ptrs = net.input_buffers()
        dst = _wrap_device(ptrs[0], 6 * net.in_n)
        dst.copy_(pg.to_device(x).reshape(-1))
        import torch

        torch.cuda.synchronize()
        net.forward_resident()
        ctx.sync()
        optrs, n = net.layer_output_ptrs(len(layers) - 1)
        res = gather(pg, optrs, n)
    else:
        out = pg.empty_shares(net.out_n)
        net.forward(pg.to_device(x), out)
        ctx.sync()
        res = pg.to_host(out)
    outs = []
    for i in range(len(layers)):
        optrs, n = net.layer_output_ptrs(i)
        outs.append(gather(pg, optrs, n))
    comm = ctx.comm()
    net.close()
    ctx.close()
    return res, outs, comm


def gather(pg, ptrs, n):
    out = np.empty((3, 2, n), dtype=np.uint64)
    for k, ptr in enumerate(ptrs):
        t = _wrap_device(ptr, n)
        out[k // 2, k % 2] = t.cpu().numpy().view(np.uint64)
    return out


def test_secureml_fixture_forward(pg, golden):
    L = golden[1]
    layers = netref.secureml_layers()
    params = []
    for li in (0, 2, 4):
        params.append((orc.set_public(L[f"secureml_weight{li}"]), orc.set_public(L[f"secureml_bias{li}"])))
        params.append(None)
    x = orc.set_public(L["secureml_input"])
    comm = orc.Comm()
    want, want_outs = netref.forward(layers, params, x, 128, comm=comm, keep=True)
    got, got_outs, gcomm = run_net(pg, layers, params, x, 128)
    for i, (g, w) in enumerate(zip(got_outs, want_outs)):
        assert np.array_equal(g, w), f"layer {i}"
    assert np.array_equal(got, want)
    # the reference's own fixture values, decoded at party A (eps 1e-3)
    for i, o in enumerate(got_outs):
        rec = orc.reconstruct(o)[0]
        assert np.max(np.abs(orc.decode(rec) - L[f"secureml_output{i}"])) <= 1e-3
    assert gcomm["tx"] == comm.tx and gcomm["rounds"] == comm.rounds


def test_lenet_forward_random_shares(pg):
    layers = netref.lenet_layers()
    params = netref.kaiming_uniform_params(layers, 7)
    batch = 4
    rng = np.random.default_rng(8)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 784)), seed=9)
    want, want_outs = netref.forward(layers, params, x, batch, keep=True)
    got, got_outs, _ = run_net(pg, layers, params, x, batch)
    for i, (g, w) in enumerate(zip(got_outs, want_outs)):
        assert np.array_equal(g, w), f"layer {i} {layers[i]}"


def test_vgg16_forward_batch2(pg):
    layers = netref.vgg16_layers()
    params = netref.kaiming_uniform_params(layers, 11)
    batch = 2
    rng = np.random.default_rng(12)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 3072)), seed=13)
    want = netref.forward(layers, params, x, batch)
    got, got_outs, _ = run_net(pg, layers, params, x, batch)
    assert np.array_equal(got, want)
    got2, _, _ = run_net(pg, layers, params, x, batch, capture=True)
    assert np.array_equal(got2, want)


def test_capture_with_layer_timing_on_side_stream(pg):
    """The bench path: a non-default stream, per-layer events recorded inside the graph."""
    import torch

    layers = netref.secureml_layers()
    params = netref.kaiming_uniform_params(layers, 31)
    batch = 16
    x = orc.share_random(orc.encode(np.random.default_rng(32).uniform(0, 1, batch * 784)), seed=33)
    want = netref.forward(layers, params, x, batch)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        for form in (pg.FORM_U64, pg.FORM_LIMB_TC):
            ctx = pg.Context(0, stream=stream, form=form)
            net = pg.Network(ctx, layers, batch)
            for i, prm in enumerate(params):
                if prm is not None:
                    net.set_params(i, pg.to_device(prm[0]), pg.to_device(prm[1]))
            net.enable_timing(True)
            net.capture()
            ptrs = net.input_buffers()
            _wrap_device(ptrs[0], 6 * net.in_n).copy_(pg.to_device(x).reshape(-1))
            net.forward_resident()
            ctx.sync()
            times = net.layer_times_ms()
            assert len(times) == len(layers) and all(t >= 0 for t in times) and sum(times) > 0
            optrs, n = net.layer_output_ptrs(len(layers) - 1)
            assert np.array_equal(gather(pg, optrs, n), want)
            ctx.check_device_errors()
            net.close()
            ctx.close()


@pytest.mark.parametrize("capture", [False, True])
def test_lenet_forward_limb_form(pg, capture):
    """LeNet in the limb tensor-core form: im2col-image convs (Din = 1 and 20),
    FC layers with bias and split-K, weights packed once by the network."""
    layers = netref.lenet_layers()
    params = netref.kaiming_uniform_params(layers, 17)
    batch = 4
    rng = np.random.default_rng(18)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 784)), seed=19)
    want, want_outs = netref.forward(layers, params, x, batch, keep=True)
    got, got_outs, _ = run_net(pg, layers, params, x, batch, capture=capture, form=pg.FORM_LIMB_TC)
    for i, (g, w) in enumerate(zip(got_outs, want_outs)):
        assert np.array_equal(g, w), f"layer {i} {layers[i]}"
    assert np.array_equal(got, want)


def test_secureml_fixture_forward_limb_form(pg, golden):
    L = golden[1]
    layers = netref.secureml_layers()
    params = []
    for li in (0, 2, 4):
        params.append((orc.set_public(L[f"secureml_weight{li}"]), orc.set_public(L[f"secureml_bias{li}"])))
        params.append(None)
    x = orc.set_public(L["secureml_input"])
    comm = orc.Comm()
    want, want_outs = netref.forward(layers, params, x, 128, comm=comm, keep=True)
    got, got_outs, gcomm = run_net(pg, layers, params, x, 128, form=pg.FORM_LIMB_TC)
    for i, (g, w) in enumerate(zip(got_outs, want_outs)):
        assert np.array_equal(g, w), f"layer {i}"
    assert gcomm["tx"] == comm.tx and gcomm["rounds"] == comm.rounds


def test_limb_weights_repacked_after_capture(pg):
    """set_params after capture repacks the layer, and the replayed graph uses the new weights."""
    import torch

    layers = netref.secureml_layers()
    p1 = netref.kaiming_uniform_params(layers, 41)
    p2 = netref.kaiming_uniform_params(layers, 42)
    batch = 8
    x = orc.share_random(orc.encode(np.random.default_rng(43).uniform(0, 1, batch * 784)), seed=44)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    ctx.set_autotune(False)  # every layer in the limb form, so that its packed weights are what is tested
    net = pg.Network(ctx, layers, batch)
    for i, prm in enumerate(p1):
        if prm is not None:
            net.set_params(i, pg.to_device(prm[0]), pg.to_device(prm[1]))
    net.capture()
    ptrs = net.input_buffers()
    _wrap_device(ptrs[0], 6 * net.in_n).copy_(pg.to_device(x).reshape(-1))
    torch.cuda.synchronize()
    for params in (p1, p2):
        for i, prm in enumerate(params):
            if prm is not None:
                net.set_params(i, pg.to_device(prm[0]), pg.to_device(prm[1]))
        net.forward_resident()
        ctx.sync()
        optrs, n = net.layer_output_ptrs(len(layers) - 1)
        assert np.array_equal(gather(pg, optrs, n), netref.forward(layers, params, x, batch))
    ctx.check_device_errors()
    net.close()
    ctx.close()


@pytest.mark.parametrize("name", ["alexnet-cifar10", "minionn", "sarda", "lenet-norelu-avgpool"])
@pytest.mark.parametrize("limb", [False, True])
def test_reference_model_files_forward(pg, name, limb):
    """Networks read from the reference's own model files (11x11 stride-4
    and 5x5 convolutions, 3x3/2 and 2x2/1 average pools, 1x1 images, a
    stride-2 2x2 convolution): every layer's shares equal the oracle's, in
    the u64 and the limb form."""
    import json
    import os

    models = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "models.json")))
    layers = [tuple(L) for L in models[name]["layers"]]
    params = netref.kaiming_uniform_params(layers, 51)
    batch = 2
    rng = np.random.default_rng(52)
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * models[name]["meta"]["input_size"])), seed=53)
    want, want_outs = netref.forward(layers, params, x, batch, keep=True)
    got, got_outs, _ = run_net(pg, layers, params, x, batch, form=pg.FORM_LIMB_TC if limb else pg.FORM_U64)
    for i, (g, w) in enumerate(zip(got_outs, want_outs)):
        assert np.array_equal(g, w), f"layer {i} {layers[i]}"
    assert np.array_equal(got, want)



@pytest.mark.parametrize("replicated_bias", [False, True])
def test_fc_fed_by_a_biased_fc(pg, replicated_bias):
    """An FC layer whose input comes straight from a biased FC layer. With
    the reference's setPublic bias (its PARTY_B fall-through leaves party B
    holding (0, b), not a replicated sharing) the first layer's output is not
    replicated, and the second layer's digit image keeps all six share
    buffers; with a replicated bias it stores each share once. Both equal the
    oracle's per-party computation, share for share."""
    rng = np.random.default_rng(61)
    layers = [("fc", 256, 128), ("fc", 128, 64), ("relu", 64), ("fc", 64, 32)]
    params = []
    for L in layers:
        if L[0] != "fc":
            params.append(None)
            continue
        w = rng.uniform(-1, 1, L[1] * L[2]) * np.sqrt(6.0 / L[1])
        b = orc.set_public(rng.uniform(-0.1, 0.1, L[2]), ref_compat=not replicated_bias)
        params.append((orc.set_public(w), b))
    batch = 128
    x = orc.share_random(orc.encode(rng.uniform(0, 1, batch * 256)), seed=62)
    want, want_outs = netref.forward(layers, params, x, batch, keep=True)
    got, got_outs, _ = run_net(pg, layers, params, x, batch, form=pg.FORM_LIMB_TC)
    for i, (g, w) in enumerate(zip(got_outs, want_outs)):
        assert np.array_equal(g, w), f"layer {i} {layers[i]}"
    assert np.array_equal(got, want)


def test_input_replication_checked_on_the_device_per_replay(pg):
    """The first layer's digit image stores each share once when the
    network's input is a replicated sharing, and all six otherwise: the
    check runs on the device in every forward, so one captured graph serves
    both kinds of input. VGG16's first convolution (the im2col image) at
    batch 2, replayed with a replicated input, a six-independent-buffer
    input, then the replicated one again; every layer equals the oracle."""
    import torch

    layers = netref.vgg16_layers()
    params = netref.kaiming_uniform_params(layers, 71)
    batch = 2
    rng = np.random.default_rng(72)
    n_in = batch * 3072
    rep = orc.share_random(orc.encode(rng.uniform(0, 1, n_in)), seed=73)
    indep = rng.integers(0, 2**63, size=(3, 2, n_in), dtype=np.uint64)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    ctx.set_autotune(False)
    net = pg.Network(ctx, layers, batch)
    for i, prm in enumerate(params):
        if prm is not None:
            net.set_params(i, pg.to_device(prm[0]), pg.to_device(prm[1]) if prm[1] is not None else None)
    net.capture()
    ptrs = net.input_buffers()
    dst = _wrap_device(ptrs[0], 6 * net.in_n)
    for x in (rep, indep, rep):
        dst.copy_(pg.to_device(x).reshape(-1))
        torch.cuda.synchronize()
        net.forward_resident()
        ctx.sync()
        want, want_outs = netref.forward(layers, params, x, batch, keep=True)
        for i in range(len(layers)):
            optrs, n = net.layer_output_ptrs(i)
            assert np.array_equal(gather(pg, optrs, n), want_outs[i]), f"layer {i} {layers[i]}"
    ctx.check_device_errors()
    net.close()
    ctx.close()


@pytest.mark.parametrize("form", ["u64", "tc"])
def test_host_forwards_back_to_back_after_capture(pg, form):
    """pg_net_forward_host after pg_net_capture: each call's input goes to
    one of two input buffer sets on a copy stream while the previous call's
    replay runs. Three calls with three different inputs, queued without a
    synchronisation between them, then a device-resident replay and two
    more host calls: every output equals the oracle's for its own input."""
    import torch

    layers = netref.lenet_layers()
    params = netref.kaiming_uniform_params(layers, 81)
    batch = 8
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC if form == "tc" else pg.FORM_U64)
    ctx.set_autotune(False)
    net = pg.Network(ctx, layers, batch)
    for i, prm in enumerate(params):
        if prm is not None:
            net.set_params(i, pg.to_device(prm[0]), pg.to_device(prm[1]) if prm[1] is not None else None)
    net.capture()
    rng = np.random.default_rng(82)
    xs = [orc.share_random(orc.encode(rng.uniform(0, 1, batch * 784)), seed=83 + k) for k in range(5)]
    ins = [torch.from_numpy(x.reshape(-1).view(np.int64)).pin_memory() for x in xs]
    outs = [torch.empty(6 * net.out_n, dtype=torch.int64).pin_memory() for _ in range(5)]
    for k in range(3):
        net.forward_host(ins[k].data_ptr(), outs[k].data_ptr())
    # a replay of whatever the first buffer set holds, then two more host
    # calls (the second one's copy into the first set waits for that replay)
    net.forward_resident()
    net.forward_host(ins[3].data_ptr(), outs[3].data_ptr())
    net.forward_host(ins[4].data_ptr(), outs[4].data_ptr())
    ctx.sync()
    for k in range(5):
        want = netref.forward(layers, params, xs[k], batch)
        got = outs[k].numpy().view(np.uint64).reshape(3, 2, -1)
        assert np.array_equal(got, want), f"call {k}"
    ctx.check_device_errors()
    net.close()
    ctx.close()
