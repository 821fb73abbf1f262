"""Host-side constructors of share tensors, with the reference's semantics.

These are the host halves of the reference's Share classes: fixed-point
encoding (``src/util/util.cuh:28-33``), ``setPublic`` and the
initializer-list constructors of RSS (``src/mpc/RSS.inl:123-142``,
``:389-414``), TPC (``src/mpc/TPC.inl:109-123``) and FPC
(``src/mpc/FPC.inl:127-155``), and seeded random sharings for synthetic
inputs. They build numpy arrays in the layouts the C ABI takes:
RSS ``(3, 2, n)``, TPC ``(2, n)``, FPC ``(4, 3, n)``.
"""
from __future__ import annotations

import numpy as np

_DT = {"u64": np.uint64, "u32": np.uint32}
_ST = {"u64": np.int64, "u32": np.int32}


def encode(vals, ring: str = "u64", fp: int = 26) -> np.ndarray:
    """(T)(f * (1 << FP)) with a negative value going through the signed type
    (truncation toward zero), as the reference's hosts computed it."""
    v = np.asarray(vals, dtype=np.float64).ravel() * float(1 << fp)
    return np.trunc(v).astype(np.int64).astype(_ST[ring]).view(_DT[ring])


def decode(x, fp: int = 26) -> np.ndarray:
    x = np.asarray(x)
    return x.view(np.int64 if x.dtype == np.uint64 else np.int32).astype(np.float64) / float(1 << fp)


def set_public(vals, ring: str = "u64", fp: int = 26) -> np.ndarray:
    """RSSBase::setPublic (RSS.inl:123-142): party A's shareA and party C's
    shareB hold the values; the missing ``break`` after case PARTY_B makes
    party B's shareB hold them as well."""
    x = encode(vals, ring, fp)
    out = np.zeros((3, 2, x.size), dtype=_DT[ring])
    out[0, 0] = x
    out[1, 1] = x
    out[2, 1] = x
    return out


def from_list(vals, ring: str = "u64", fp: int = 26, to_fixed: bool = True) -> np.ndarray:
    """The RSS initializer-list constructor (RSS.inl:389-414): no fall-through."""
    x = encode(vals, ring, fp) if to_fixed else np.asarray(vals, dtype=np.float64).astype(np.int64).astype(
        _ST[ring]).view(_DT[ring])
    out = np.zeros((3, 2, x.size), dtype=_DT[ring])
    out[0, 0] = x
    out[2, 1] = x
    return out


def share_random(secret, ring: str = "u64", seed: int = 0) -> np.ndarray:
    """A consistent 3-party replicated sharing of ring values: party p holds
    (x_p, x_{p+1}) with x_1, x_2 seeded uniform and x_0 = secret - x_1 - x_2."""
    dt = _DT[ring]
    s = np.asarray(secret, dtype=dt).ravel()
    rng = np.random.default_rng(seed)
    x1 = rng.integers(0, np.iinfo(dt).max, size=s.size, dtype=dt, endpoint=True)
    x2 = rng.integers(0, np.iinfo(dt).max, size=s.size, dtype=dt, endpoint=True)
    with np.errstate(over="ignore"):
        x0 = s - x1 - x2
    sh = [x0, x1, x2]
    out = np.empty((3, 2, s.size), dtype=dt)
    for p in range(3):
        out[p, 0] = sh[p]
        out[p, 1] = sh[(p + 1) % 3]
    return out


def tpc_set_public(vals, ring: str = "u64", fp: int = 26) -> np.ndarray:
    """TPC setPublic / initializer list (TPC.inl:109-123, :341-363): party A holds the values."""
    x = encode(vals, ring, fp)
    out = np.zeros((2, x.size), dtype=_DT[ring])
    out[0] = x
    return out


def fpc_set_public(vals, ring: str = "u64", fp: int = 26) -> np.ndarray:
    """FPC setPublic (FPC.inl:127-155): component x0, held by party B as
    shareC, party C as shareB and party D as shareA."""
    x = encode(vals, ring, fp)
    out = np.zeros((4, 3, x.size), dtype=_DT[ring])
    out[1, 2] = x
    out[2, 1] = x
    out[3, 0] = x
    return out


def one_hot(classes_per_row, n_classes: int) -> np.ndarray:
    """One-hot label rows as doubles (the reference's label files)."""
    y = np.zeros((len(classes_per_row), n_classes))
    y[np.arange(len(classes_per_row)), np.asarray(classes_per_row)] = 1.0
    return y.ravel()


def aes_key_from_file(path) -> bytes:
    """The 32-byte AES-256 key of a reference key file (AESObject::AESObject,
    src/mpc/AESObject.cpp:9-34): the file's text up to its first NUL,
    zero-padded (or cut) to 32 bytes."""
    data = open(path, "rb").read()
    data = data.split(b"\0", 1)[0]
    return (data + bytes(32))[:32]
