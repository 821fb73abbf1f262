"""The reference's model files (files/models/*.json, parsed into
tests/golden/models.json by tests/golden/make_models.py): this library's
network builders equal them layer for layer, every supported file round-trips
through nets.to_model / nets.from_model, and layers outside the library's
layer set (layer normalisation, residual blocks) are refused by name."""
import json
import os

import pytest

from piranha_gb300 import nets

MODELS = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "models.json")))


def _layers(name):
    return [tuple(L) for L in MODELS[name]["layers"]]


def test_builders_equal_the_reference_model_files():
    assert _layers("lenet") == nets.lenet()
    assert _layers("secureml") == nets.secureml()
    assert _layers("vgg16-cifar10") == nets.vgg16(maxpool=False)
    assert MODELS["vgg16-cifar10"]["meta"]["batch_size"] == 128


def test_model_files_round_trip():
    done = 0
    for name, m in MODELS.items():
        if "layers" not in m:
            continue
        L = _layers(name)
        back, meta = nets.from_model(nets.to_model(L, batch_size=m["meta"]["batch_size"]))
        assert back == L, name
        assert nets.input_size(L) == m["meta"]["input_size"], name
        done += 1
    assert done >= 10


def test_layers_outside_the_library_are_refused():
    for kind in ("ln", "res"):
        with pytest.raises(ValueError, match=repr(kind)):
            nets.from_model({"model": [{"layer": "fc", "input_dim": 4, "output_dim": 4}, {"layer": kind}]})
    assert "unsupported" in MODELS["resnet18-cifar10"]
    assert "unsupported" in MODELS["lenet-ln-norelu"]
