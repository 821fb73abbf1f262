"""The reference's model configurations (files/models/*.json) as layer
tuples for ``piranha_gb300.Network``, and seeded synthetic parameters.

Layer tuples: ("fc", din, dout), ("cnn", H, W, Din, Dout, f, stride, pad),
("relu", n_per_image), ("maxpool", H, W, C, pool, stride),
("avgpool", H, W, C, pool, stride).
"""
from __future__ import annotations

import numpy as np

from . import encode as _enc


def secureml():
    """files/models/secureml.json: 784-128-128-10 with ReLU after every FC."""
    return [("fc", 784, 128), ("relu", 128), ("fc", 128, 128), ("relu", 128), ("fc", 128, 10), ("relu", 10)]


def lenet():
    """files/models/lenet.json (maxpool variant)."""
    return [("cnn", 28, 28, 1, 20, 5, 1, 0), ("maxpool", 24, 24, 20, 2, 2), ("relu", 2880),
            ("cnn", 12, 12, 20, 50, 5, 1, 0), ("maxpool", 8, 8, 50, 2, 2), ("relu", 800),
            ("fc", 800, 500), ("relu", 500), ("fc", 500, 10), ("relu", 10)]


def vgg16(maxpool: bool = True):
    """files/models/vgg16-cifar10.json; maxpool=True replaces each of its five
    2x2/2 averagepool layers by a maxpool (the secure-inference benchmark's
    network), maxpool=False keeps them."""
    pool = "maxpool" if maxpool else "avgpool"
    L = []
    hw, c = 32, 3
    for width, reps in [(64, 2), (128, 2), (256, 3), (512, 3), (512, 3)]:
        for r in range(reps):
            L.append(("cnn", hw, hw, c, width, 3, 1, 1))
            c = width
            if r < reps - 1:
                L.append(("relu", hw * hw * c))
        L.append((pool, hw, hw, c, 2, 2))
        hw //= 2
        L.append(("relu", hw * hw * c))
    L += [("fc", 512, 256), ("relu", 256), ("fc", 256, 256), ("relu", 256), ("fc", 256, 10), ("relu", 10)]
    return L


def from_model(doc: dict):
    """Layer tuples of a model in the reference's model-file format (the JSON
    of files/models/*.json: {"batch_size", "input_size", "num_classes",
    "model": [{"layer": ...}, ...]}), read field by field as the reference's
    loader reads them (src/util/model.cu:43-118: input_hw = (height, width),
    only the first filter_hw / pool_hw entry). Returns (layers, meta) with meta
    = {"name", "dataset", "batch_size", "input_size", "num_classes"}. Layer
    normalisation ("ln") and residual blocks ("res") are outside this
    library's layers and raise ValueError."""
    layers = []
    for i, l in enumerate(doc["model"]):
        kind = l["layer"]
        if kind == "fc":
            layers.append(("fc", int(l["input_dim"]), int(l["output_dim"])))
        elif kind == "relu":
            layers.append(("relu", int(l["input_dim"])))
        elif kind == "cnn":
            H, W = (int(v) for v in l["input_hw"])
            layers.append(("cnn", H, W, int(l["in_channels"]), int(l["out_channels"]), int(l["filter_hw"][0]),
                           int(l["stride"]), int(l["padding"])))
        elif kind in ("maxpool", "averagepool"):
            H, W = (int(v) for v in l["input_hw"])
            layers.append(("maxpool" if kind == "maxpool" else "avgpool", H, W, int(l["in_channels"]),
                           int(l["pool_hw"][0]), int(l["stride"])))
        else:
            raise ValueError(f"layer {i}: {kind!r} is not one of this library's layers "
                             "(fc, relu, cnn, maxpool, averagepool)")
    meta = {k: doc.get(k) for k in ("name", "dataset", "batch_size", "input_size", "num_classes")}
    return layers, meta


def load_model(path: str):
    """from_model of a model file (the reference's files/models/*.json format)."""
    import json

    with open(path) as f:
        return from_model(json.load(f))


def to_model(layers, batch_size: int = 128, name: str = "", dataset: str = "", num_classes: int = 10) -> dict:
    """The reference's model-file dict of layer tuples (the inverse of from_model)."""
    out = []
    for L in layers:
        if L[0] == "fc":
            out.append({"layer": "fc", "input_dim": L[1], "output_dim": L[2]})
        elif L[0] == "relu":
            out.append({"layer": "relu", "input_dim": L[1]})
        elif L[0] == "cnn":
            out.append({"layer": "cnn", "input_hw": [L[1], L[2]], "in_channels": L[3], "out_channels": L[4],
                        "filter_hw": [L[5], L[5]], "stride": L[6], "padding": L[7]})
        else:
            out.append({"layer": "maxpool" if L[0] == "maxpool" else "averagepool", "input_hw": [L[1], L[2]],
                        "in_channels": L[3], "pool_hw": [L[4], L[4]], "stride": L[5]})
    return {"name": name, "dataset": dataset, "batch_size": batch_size, "input_size": input_size(layers),
            "num_classes": num_classes, "model": out}


def input_size(layers):
    L = layers[0]
    if L[0] == "fc":
        return L[1]
    if L[0] == "cnn":
        return L[1] * L[2] * L[3]
    if L[0] == "relu":
        return L[1]
    return L[1] * L[2] * L[3]


NN_SEED = 343934585  # nn_seed of the reference's config.json


def reference_normal(n: int, seed: int, std_dev: float) -> np.ndarray:
    """n draws of the reference's weight generator (std::default_random_engine
    + std::normal_distribution<double>), computed by the library's host code."""
    import ctypes

    from . import lib

    out = np.empty(n, dtype=np.float64)
    st = lib().pg_reference_init_normal(out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n, int(seed),
                                        float(std_dev))
    if st != 0:
        raise ValueError(f"pg_reference_init_normal status {st}")
    return out


def reference_init(layers, seed: int = NN_SEED, fp: int = 26, ring: str = "u64"):
    """The reference's own initialisation (FCLayer.cu:31-47, CNNLayer.cu:36-50):
    layer i draws from std::default_random_engine(seed + i) a normal with
    standard deviation sqrt(2 / fan_in); FC biases 0.01; all loaded with
    setPublic. None for layers without parameters."""
    params = []
    for i, L in enumerate(layers):
        if L[0] == "fc":
            din, dout = L[1], L[2]
            w = reference_normal(din * dout, seed + i, float(np.sqrt(2.0 / din)))
            params.append((_enc.set_public(w, ring, fp), _enc.set_public(np.full(dout, 0.01), ring, fp)))
        elif L[0] == "cnn":
            Din, Dout, f = L[3], L[4], L[5]
            w = reference_normal(Dout * f * f * Din, seed + i, float(np.sqrt(2.0 / (f * f * Din))))
            params.append((_enc.set_public(w, ring, fp), None))
        else:
            params.append(None)
    return params


def kaiming_uniform(layers, seed: int, fp: int = 26, ring: str = "u64"):
    """Seeded Kaiming-uniform weights (bound sqrt(6 / fan_in)), FC bias 0.01,
    loaded with setPublic; None for layers without parameters."""
    rng = np.random.default_rng(seed)
    params = []
    for L in layers:
        if L[0] == "fc":
            din, dout = L[1], L[2]
            w = rng.uniform(-1, 1, din * dout) * np.sqrt(6.0 / din)
            params.append((_enc.set_public(w, ring, fp), _enc.set_public(np.full(dout, 0.01), ring, fp)))
        elif L[0] == "cnn":
            Din, Dout, f = L[3], L[4], L[5]
            w = rng.uniform(-1, 1, Dout * f * f * Din) * np.sqrt(6.0 / (f * f * Din))
            params.append((_enc.set_public(w, ring, fp), None))
        else:
            params.append(None)
    return params
