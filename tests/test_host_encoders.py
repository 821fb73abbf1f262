"""The package's host-side share constructors and model definitions against
the oracle's restatement of the reference (CPU only)."""
import numpy as np
import pytest

import oracle as orc
from piranha_gb300 import encode as enc
from piranha_gb300 import nets
from oracle import netref


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


# The reference's weight generator, restated from the published algorithms of
# the C++ standard library it runs on (libstdc++): minstd_rand0 (Park-Miller,
# a = 16807, m = 2^31 - 1) as std::default_random_engine,
# generate_canonical<double, 53> over two draws, and normal_distribution's
# Marsaglia polar method, which returns the second variate of a pair first and
# keeps the other for the next call.
class _MinstdRand0:
    M = 2147483647

    def __init__(self, seed):
        self.x = seed % self.M or 1

    def __call__(self):
        self.x = (16807 * self.x) % self.M
        return self.x


def _canonical(g):
    r = float(2147483646)  # max - min + 1 with min = 1, max = m - 1
    s = float(g() - 1) + float(g() - 1) * r
    v = s / (r * r)
    return v if v < 1.0 else np.nextafter(1.0, 0.0)


def _normal_stream(seed, std_dev, n):
    import math

    g = _MinstdRand0(seed)
    out, saved = [], None
    while len(out) < n:
        if saved is not None:
            out.append(saved * std_dev)
            saved = None
            continue
        while True:
            x = 2.0 * _canonical(g) - 1.0
            y = 2.0 * _canonical(g) - 1.0
            r2 = x * x + y * y
            if 0.0 < r2 <= 1.0:
                break
        mult = math.sqrt(-2.0 * math.log(r2) / r2)
        saved = x * mult
        out.append(y * mult * std_dev)
    return np.array(out)


@pytest.mark.parametrize("seed,std", [(nets.NN_SEED, float(np.sqrt(2.0 / 784))), (nets.NN_SEED + 4, 0.05), (1, 1.0)])
def test_reference_init_normal_is_the_published_generator(seed, std):
    got = nets.reference_normal(1001, seed, std)
    want = _normal_stream(seed, std, 1001)
    assert np.array_equal(got, want)


def test_reference_init_layers():
    layers = nets.secureml()
    params = nets.reference_init(layers)
    assert [p is None for p in params] == [False, True, False, True, False, True]
    w0 = nets.reference_normal(784 * 128, nets.NN_SEED + 0, float(np.sqrt(2.0 / 784)))
    assert np.array_equal(params[0][0], enc.set_public(w0))
    assert np.array_equal(params[2][1], enc.set_public(np.full(128, 0.01)))
    lp = nets.reference_init(nets.lenet())
    assert lp[0][1] is None and lp[0][0].shape == (3, 2, 20 * 25)


def test_aes_key_from_file(tmp_path):
    f = tmp_path / "key"
    f.write_bytes(b"short key\n")
    assert enc.aes_key_from_file(f) == b"short key\n" + bytes(22)
    f.write_bytes(b"k" * 40)
    assert enc.aes_key_from_file(f) == b"k" * 32
    f.write_bytes(b"abc\0def")
    assert enc.aes_key_from_file(f) == b"abc" + bytes(29)
