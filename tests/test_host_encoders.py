"""The package's host-side share constructors and model definitions against
the oracle's restatement of the reference (CPU only)."""
import numpy as np
import pytest

import oracle as orc
from piranha_gb300 import encode as enc
from piranha_gb300 import nets
from tests import netref


@pytest.mark.parametrize("ring,dt", [("u64", np.uint64), ("u32", np.uint32)])
def test_encode_matches_oracle(ring, dt):
    rng = np.random.default_rng(1)
    fp = 26 if ring == "u64" else 10
    v = np.concatenate([rng.normal(0, 50, 5000), [0.0, -0.0, 1e-12, -1e-12, -3.5, 3.5, -1.0 / (1 << fp)]])
    assert np.array_equal(enc.encode(v, ring, fp), orc.encode(v, dt, fp))


def test_set_public_and_from_list_match_oracle():
    v = np.random.default_rng(2).normal(0, 3, 777)
    assert np.array_equal(enc.set_public(v), orc.set_public(v))
    assert np.array_equal(enc.from_list(v), orc.from_list(v))
    assert np.array_equal(enc.from_list(np.arange(-5, 5), to_fixed=False), orc.from_list(np.arange(-5, 5), to_fixed=False))
    assert np.array_equal(enc.tpc_set_public(v, "u32", 10), orc.tpc_from_list(v, np.uint32, 10))
    assert np.array_equal(enc.fpc_set_public(v), orc.fpc_from_list(v))


def test_share_random_matches_oracle():
    s = orc.encode(np.random.default_rng(3).normal(0, 1, 999))
    assert np.array_equal(enc.share_random(s, seed=7), orc.share_random(s, seed=7))
    rec = orc.reconstruct(enc.share_random(s, seed=8))
    assert all(np.array_equal(rec[p], s) for p in range(3))


@pytest.mark.parametrize("name", ["secureml", "lenet", "vgg16"])
def test_model_layers_and_params_match_test_reference(name):
    layers = getattr(nets, name)()
    assert layers == getattr(netref, f"{name}_layers")()
    ours = nets.kaiming_uniform(layers, 11)
    theirs = netref.kaiming_uniform_params(layers, 11)
    for a, b in zip(ours, theirs):
        assert (a is None) == (b is None)
        if a is not None:
            assert np.array_equal(a[0], b[0])
            assert (a[1] is None) == (b[1] is None)
            if a[1] is not None:
                assert np.array_equal(a[1], b[1])
