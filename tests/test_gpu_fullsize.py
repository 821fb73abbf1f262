"""Parity at the benchmark configurations' full sizes.

* VGG16 (maxpool) 3PC inference at batch 128 and one LeNet training step at
  batch 128: every layer's six output shares (and, for training, the softmax
  gradient, every gradient passed between layers and every updated weight
  and bias share) hash to the SHA-256 digests of the oracle's run of the same
  inputs, stored in tests/golden/fullsize.json by tests/golden/make_fullsize.py;
  the message counters are compared too. Both forms, with the tuner on as the
  benchmark runs them.
* The request stream's bucket path: a request of b images served on the
  captured network of a larger batch bucket, whose other rows hold an earlier
  request's data, gives the oracle's result for its b images; and requests
  packed into one replay (piranha_gb300.stream) each get their own result.
* Share-GEMMs with truncation at 512^3, 4096^3, 8192^3 and non-cubic shapes:
  both forms agree on every share, and sampled rows equal the oracle's
  product of those rows.
"""
import json
import os

import numpy as np
import pytest

import oracle as orc
from oracle import netref
from tests.golden import seeded
from tests.test_gpu_network import _wrap_device, gather, run_net

pytestmark = pytest.mark.gpu

U64 = np.uint64
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def pg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    pg.lib()
    return pg


@pytest.fixture(scope="module")
def fixtures():
    return json.load(open(os.path.join(HERE, "golden", "fullsize.json")))


def _form(pg, name):
    return pg.FORM_LIMB_TC if name == "tc" else pg.FORM_U64


@pytest.mark.parametrize("form", ["tc", "u64"])
def test_vgg16_batch128_equals_oracle_digests(pg, fixtures, form):
    fx = fixtures["vgg16_b128"]
    layers = netref.vgg16_layers(maxpool=True)
    params = seeded.kaiming_uniform(layers, fx["seeds"]["weights"])
    batch = fx["batch"]
    x = seeded.images(fx["seeds"]["images"], batch * 3072)
    assert seeded.digest(x) == fx["input"], "inputs differ from the fixture's"
    assert [None if p is None else seeded.digest(p[0]) for p in params] == fx["params"]
    _, outs, comm = run_net(pg, layers, params, x, batch, capture=True, form=_form(pg, form), autotune=True)
    for i, o in enumerate(outs):
        assert seeded.digest(o) == fx["layers"][i], f"layer {i} {layers[i]}"
    assert {"tx": comm["tx"], "rx": comm["rx"], "rounds": comm["rounds"]} == fx["comm"]


@pytest.mark.parametrize("form", ["tc", "u64"])
def test_lenet_training_batch128_equals_oracle_digests(pg, fixtures, form):
    from tests.test_gpu_train import make_net

    fx = fixtures["lenet_train_b128"]
    layers = netref.lenet_layers()
    params = seeded.kaiming_uniform(layers, fx["seeds"]["weights"])
    batch = fx["batch"]
    x = seeded.images(fx["seeds"]["images"], batch * 784)
    labels = seeded.labels(fx["seeds"]["labels"], batch)
    assert seeded.digest(x) == fx["input"] and seeded.digest(labels) == fx["labels"]
    ctx = pg.Context(0, form=_form(pg, form))
    ctx.set_autotune(True)
    net = make_net(pg, ctx, layers, params, batch)
    ctx.reset_comm()
    net.train_step(pg.to_device(x), pg.to_device(labels), fx["log_lr"])
    ctx.sync()
    ctx.check_device_errors()
    for i in range(len(layers)):
        optrs, n = net.layer_output_ptrs(i)
        assert seeded.digest(gather(pg, optrs, n)) == fx["outputs"][i], f"output of layer {i} {layers[i]}"
    dptrs, n = net.layer_delta_ptrs(-1)
    assert seeded.digest(gather(pg, dptrs, n)) == fx["softmax"], "softmax gradient"
    for i in range(len(layers)):
        dptrs, n = net.layer_delta_ptrs(i)
        assert seeded.digest(gather(pg, dptrs, n)) == fx["deltas"][i], f"gradient out of layer {i} {layers[i]}"
        if fx["params"][i] is not None:
            w, wn, b, bn = net.layer_param_ptrs(i)
            assert seeded.digest(gather(pg, w, wn)) == fx["params"][i][0], f"weights of layer {i}"
            if fx["params"][i][1] is not None:
                assert seeded.digest(gather(pg, b, bn)) == fx["params"][i][1], f"bias of layer {i}"
    comm = ctx.comm()
    assert {"tx": comm["tx"], "rx": comm["rx"], "rounds": comm["rounds"]} == fx["comm"]
    net.close()
    ctx.close()


@pytest.mark.parametrize("model,requests", [
    ("secureml", [(64, 64), (37, 40), (1, 1), (5, 8)]),
    ("vgg16", [(3, 4), (1, 2)]),
])
def test_stream_bucket_path_equals_oracle(pg, model, requests):
    """Each (b, bucket): the request's b images go into the first rows of the
    bucket network's input, whose remaining rows hold an earlier request's
    images, as the benchmark's request stream serves them."""
    import torch

    layers = netref.vgg16_layers(maxpool=True) if model == "vgg16" else netref.secureml_layers()
    params = seeded.kaiming_uniform(layers, 77)
    n_img = 3072 if model == "vgg16" else 784
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    ctx.set_autotune(True)
    for r, (b, bucket) in enumerate(requests):
        net = pg.Network(ctx, layers, bucket)
        for i, prm in enumerate(params):
            if prm is not None:
                net.set_params(i, pg.to_device(prm[0]), pg.to_device(prm[1]) if prm[1] is not None else None)
        net.capture()
        inb = _wrap_device(net.input_buffers()[0], 6 * net.in_n).view(6, net.in_n)
        earlier = seeded.images(500 + r, bucket * n_img)
        inb.copy_(pg.to_device(earlier).reshape(6, -1))
        net.forward_resident()
        x = seeded.images(600 + r, b * n_img)
        inb[:, : b * n_img].copy_(pg.to_device(x).reshape(6, -1))
        net.forward_resident()
        ctx.sync()
        optrs, on = net.layer_output_ptrs(len(layers) - 1)
        got = gather(pg, optrs, on)[..., : b * 10]
        want = netref.forward(layers, params, x, b)
        assert np.array_equal(got, want), f"request {r}: b={b} on the {bucket}-image network"
        net.close()
    ctx.check_device_errors()
    ctx.close()
    torch.cuda.synchronize()


@pytest.mark.parametrize("M,N,K", [(512, 512, 512), (4096, 4096, 4096), (8192, 8192, 8192), (1024, 8192, 2048),
                                   (8192, 512, 4096), (3000, 1000, 777)])
def test_gemm_forms_agree_and_sampled_rows_equal_oracle(pg, M, N, K):
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(M * 31 + N * 7 + K)
    A = torch.randint(-2**63, 2**63 - 1, (3, 2, M * K), dtype=torch.int64, device="cuda", generator=g)
    B = torch.randint(-2**63, 2**63 - 1, (3, 2, K * N), dtype=torch.int64, device="cuda", generator=g)
    out = {}
    for form in (pg.FORM_LIMB_TC, pg.FORM_U64):
        ctx = pg.Context(0, form=form)
        ctx.set_autotune(False)  # the form under test for every shape
        C = pg.empty_shares(M * N)
        pg.matmul(ctx, A, B, C, M, N, K, 1, 1, 1, 26)
        ctx.check_device_errors()
        out[form] = C
        ctx.close()
    assert torch.equal(out[pg.FORM_LIMB_TC], out[pg.FORM_U64])
    rows = sorted({0, 1, M // 2, M - 1})
    a_rows = pg.to_host(A.view(3, 2, M, K)[:, :, rows, :].reshape(3, 2, -1).contiguous())
    want = orc.matmul(a_rows, pg.to_host(B), len(rows), N, K, 1, 1, 1, 26).reshape(3, 2, len(rows), N)
    got = pg.to_host(out[pg.FORM_LIMB_TC].view(3, 2, M, N)[:, :, rows, :].contiguous())
    assert np.array_equal(got, want)


def test_stream_packed_replays_equal_oracle(pg):
    """Requests of one model packed into one replay (StreamServer): each
    request's output rows equal the oracle's result for that request alone."""
    import torch

    from piranha_gb300 import stream as st

    models = {"secureml": netref.secureml_layers(), "vgg16": netref.vgg16_layers(maxpool=True)}
    params = {m: seeded.kaiming_uniform(L, 91 if m == "vgg16" else 92) for m, L in models.items()}
    n_in = {"secureml": 784, "vgg16": 3072}
    reqs = [("secureml", 5), ("vgg16", 2), ("secureml", 17), ("secureml", 9), ("vgg16", 3), ("secureml", 64)]
    packs = st.plan_packs(reqs, cap=128, lookahead=16)
    assert [p.requests for p in packs] == [[0, 2, 3, 5], [1, 4]]
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    server = st.StreamServer(pg, ctx, {m: (models[m], params[m]) for m in models})
    for rnd in range(2):
        xs = [seeded.images(700 + 10 * rnd + r, b * n_in[m]) for r, (m, b) in enumerate(reqs)]
        ins = [pg.to_device(x).reshape(6, -1) for x in xs]
        outs = [torch.empty((6, b * 10), dtype=torch.int64, device="cuda") for _, b in reqs]
        for p in packs:
            server.serve(p, ins, outs)
        ctx.sync()
        for r, (m, b) in enumerate(reqs):
            want = netref.forward(models[m], params[m], xs[r], b)
            assert np.array_equal(pg.to_host(outs[r]).reshape(3, 2, -1), want), f"round {rnd} request {r}"
    ctx.check_device_errors()
    server.close()
    ctx.close()


def test_stream_pack_on_a_larger_bucket_equals_oracle(pg):
    """A pack served on a larger bucket than the smallest that holds it (what
    StreamServer.tune_buckets does when the larger network replays faster)
    gives each request the oracle's result; tune_buckets never picks a
    bucket smaller than the pack."""
    import torch

    from piranha_gb300 import stream as st

    layers = netref.secureml_layers()
    params = seeded.kaiming_uniform(layers, 93)
    reqs = [("secureml", 5), ("secureml", 17), ("secureml", 9), ("secureml", 100)]
    packs = st.plan_packs(reqs, cap=128, lookahead=16)
    assert [(p.requests, p.bucket) for p in packs] == [([0, 1, 2], 32), ([3], 112)]
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    server = st.StreamServer(pg, ctx, {"secureml": (layers, params)})
    tuned = server.tune_buckets(packs)
    assert all(t.bucket >= t.images and t.bucket in (32, 112) for t in tuned)
    moved = [st.Pack(p.model, p.requests, p.images, 112) for p in packs]
    xs = [seeded.images(800 + r, b * 784) for r, (_, b) in enumerate(reqs)]
    ins = [pg.to_device(x).reshape(6, -1) for x in xs]
    for plan in (tuned, moved):
        outs = [torch.empty((6, b * 10), dtype=torch.int64, device="cuda") for _, b in reqs]
        for p in plan:
            server.serve(p, ins, outs)
        ctx.sync()
        for r, (_, b) in enumerate(reqs):
            want = netref.forward(layers, params, xs[r], b)
            assert np.array_equal(pg.to_host(outs[r]).reshape(3, 2, -1), want), f"request {r}"
    ctx.check_device_errors()
    server.close()
    ctx.close()
