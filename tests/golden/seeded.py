"""Seeded synthetic inputs for the full-size parity fixtures.

The fixtures in ``fullsize.json`` hold SHA-256 digests of oracle outputs, so
the test inputs must be reproduced bit for bit on any machine and any numpy
version. Everything here is derived from SplitMix64 (Steele, Lea and Flood,
"Fast splittable pseudorandom number generators", OOPSLA 2014) in plain
numpy integer arithmetic, with no dependence on numpy's own generators.
"""
from __future__ import annotations

import hashlib

import numpy as np

import oracle as orc

U64 = np.uint64
_GOLDEN = U64(0x9E3779B97F4A7C15)


def splitmix64(seed: int, n: int) -> np.ndarray:
    """The first n outputs of SplitMix64 started from state ``seed``."""
    with np.errstate(over="ignore"):
        z = U64(seed % (1 << 64)) + np.arange(1, n + 1, dtype=U64) * _GOLDEN
        z = (z ^ (z >> U64(30))) * U64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> U64(27))) * U64(0x94D049BB133111EB)
        return z ^ (z >> U64(31))


def uniform01(seed: int, n: int) -> np.ndarray:
    """n doubles in [0, 1): the top 53 bits of each SplitMix64 output."""
    return (splitmix64(seed, n) >> U64(11)).astype(np.float64) * (2.0 ** -53)


def share(secret: np.ndarray, seed: int) -> np.ndarray:
    """A consistent 3-party replicated sharing (3, 2, n) of u64 ring values:
    x1, x2 from SplitMix64 streams seed and seed + 1, x0 = secret - x1 - x2;
    party p holds (x_p, x_{p+1})."""
    s = np.asarray(secret, dtype=U64).ravel()
    x1 = splitmix64(seed, s.size)
    x2 = splitmix64(seed + 1, s.size)
    with np.errstate(over="ignore"):
        x0 = s - x1 - x2
    sh = (x0, x1, x2)
    out = np.empty((3, 2, s.size), dtype=U64)
    for p in range(3):
        out[p, 0] = sh[p]
        out[p, 1] = sh[(p + 1) % 3]
    return out


def images(seed: int, n_values: int) -> np.ndarray:
    """Synthetic image values uniform in [0, 1), fixed-point encoded with 26
    fractional bits and shared with masks from streams seed + 1, seed + 2."""
    return share(orc.encode(uniform01(seed, n_values)), seed + 1)


def kaiming_uniform(layers, seed: int, fp: int = 26):
    """Kaiming-uniform weights w = (2u - 1) sqrt(6 / fan_in) (layer i from
    stream seed + i), FC bias 0.01, loaded with setPublic; None for layers
    without parameters."""
    params = []
    for i, L in enumerate(layers):
        if L[0] == "fc":
            din, dout = L[1], L[2]
            w = (2.0 * uniform01(seed + i, din * dout) - 1.0) * np.sqrt(6.0 / din)
            params.append((orc.set_public(w, fp=fp), orc.set_public(np.full(dout, 0.01), fp=fp)))
        elif L[0] == "cnn":
            Din, Dout, f = L[3], L[4], L[5]
            w = (2.0 * uniform01(seed + i, Dout * f * f * Din) - 1.0) * np.sqrt(6.0 / (f * f * Din))
            params.append((orc.set_public(w, fp=fp), None))
        else:
            params.append(None)
    return params


def labels(seed: int, batch: int, classes: int = 10) -> np.ndarray:
    """One-hot labels, class = SplitMix64 output mod classes, loaded with setPublic."""
    y = np.zeros((batch, classes))
    y[np.arange(batch), (splitmix64(seed, batch) % U64(classes)).astype(np.int64)] = 1.0
    return orc.set_public(y.ravel())


def digest(a: np.ndarray) -> str:
    """SHA-256 of an array's bytes in C order (little-endian ring elements)."""
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
