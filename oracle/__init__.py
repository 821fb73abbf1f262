"""CPU oracle for Piranha's party-local share arithmetic (test infrastructure).

This package is the checker. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import it; the ``piranha_gb300`` product
never does. The arithmetic lives in ``oracle.hpp`` (C++17, restating
``src/mpc/RSS.inl`` and the ``src/gpu`` kernels of Piranha); this module only
builds ``_build/liboracle.so`` on demand and wraps its C entry points for numpy.

Array conventions
-----------------
* an RSS tensor of n elements is a numpy array of shape ``(3, 2, n)``:
  ``[party A/B/C][shareA/shareB][element]``;
* per-party public data (the output of ``reconstruct``) has shape ``(3, n)``;
* a TPC tensor has shape ``(2, n)`` and an FPC tensor ``(4, 3, n)``
  (``[party A..D][shareA/shareB/shareC][element]``);
* ``Comm`` accumulates the bytes each party sends/receives and the rounds
  (``Comm(4)`` reports all four parties).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None

FP_DEFAULT = 26

FPROP, DGRAD, WGRAD = 0, 1, 2

_SUF = {np.uint64: "u64", np.uint32: "u32", np.uint8: "u8"}
_CT = {np.uint64: ctypes.c_uint64, np.uint32: ctypes.c_uint32, np.uint8: ctypes.c_uint8}


def build() -> str:
    """Compile the oracle with its Makefile (idempotent); return the .so path."""
    srcs = [os.path.join(_HERE, f) for f in ("capi.cpp", "oracle.hpp", "aes.hpp")]
    if os.path.exists(_LIB_PATH) and all(os.path.getmtime(_LIB_PATH) >= os.path.getmtime(s) for s in srcs):
        return _LIB_PATH
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            _lib = ctypes.CDLL(build())
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Comm:
    """Per-party byte counters and the round counter (one round per protocol step)."""

    def __init__(self, parties=3):
        self.parties = parties
        self.buf = np.zeros(9, dtype=np.uint64)

    @property
    def tx(self):
        return [int(x) for x in self.buf[:self.parties]]

    @property
    def rx(self):
        return [int(x) for x in self.buf[4:4 + self.parties]]

    @property
    def rounds(self):
        return int(self.buf[8])

    def ptr(self):
        return _p(self.buf)


def _ring(dtype):
    dt = np.dtype(dtype).type
    if dt not in (np.uint64, np.uint32):
        raise TypeError("ring must be uint64 or uint32")
    return dt, _SUF[dt]


def _views(a, dtype, n=None):
    a = np.ascontiguousarray(a, dtype=dtype)
    if a.ndim != 3 or a.shape[:2] != (3, 2) or (n is not None and a.shape[2] != n):
        raise ValueError(f"expected RSS views of shape (3, 2, {n}), got {a.shape}")
    return a


# ------------------------------------------------------------------ encoding

def encode(vals, dtype=np.uint64, fp=FP_DEFAULT):
    dt, suf = _ring(dtype)
    v = np.ascontiguousarray(vals, dtype=np.float64).ravel()
    out = np.empty(v.size, dtype=dt)
    getattr(lib(), f"or_encode_{suf}")(_p(v), ctypes.c_size_t(v.size), _p(out), fp)
    return out


def decode(x, fp=FP_DEFAULT):
    x = np.asarray(x)
    s = x.view(np.int64 if x.dtype == np.uint64 else np.int32)
    return s.astype(np.float64) / float(1 << fp)


def set_public(vals, dtype=np.uint64, fp=FP_DEFAULT, ref_compat=True):
    """RSSBase::setPublic (RSS.inl:123-142); ref_compat keeps the PARTY_B fall-through."""
    dt, suf = _ring(dtype)
    v = np.ascontiguousarray(vals, dtype=np.float64).ravel()
    out = np.zeros((3, 2, v.size), dtype=dt)
    getattr(lib(), f"or_rss_set_public_{suf}")(_p(v), ctypes.c_size_t(v.size), _p(out), fp, int(ref_compat))
    return out


def from_list(vals, dtype=np.uint64, fp=FP_DEFAULT, to_fixed=True):
    """The RSS initializer-list constructor (RSS.inl:389-414)."""
    dt, suf = _ring(dtype)
    v = np.ascontiguousarray(vals, dtype=np.float64).ravel()
    out = np.zeros((3, 2, v.size), dtype=dt)
    getattr(lib(), f"or_rss_from_list_{suf}")(_p(v), ctypes.c_size_t(v.size), _p(out), fp, int(to_fixed))
    return out


def share_random(secret, dtype=np.uint64, seed=0):
    """A consistent 3-party RSS sharing of ring values with seeded random masks."""
    dt, _ = _ring(dtype)
    secret = np.asarray(secret, dtype=dt).ravel()
    rng = np.random.default_rng(seed)
    info = np.iinfo(dt)
    x1 = rng.integers(0, info.max, size=secret.size, dtype=dt, endpoint=True)
    x2 = rng.integers(0, info.max, size=secret.size, dtype=dt, endpoint=True)
    with np.errstate(over="ignore"):
        x0 = secret - x1 - x2
    sh = [x0, x1, x2]
    out = np.empty((3, 2, secret.size), dtype=dt)
    for p in range(3):
        out[p, 0] = sh[p]
        out[p, 1] = sh[(p + 1) % 3]
    return out


def random_views(n, dtype=np.uint64, seed=0):
    """Independent uniform ring values in all six share slots (arbitrary party views)."""
    dt, _ = _ring(dtype)
    rng = np.random.default_rng(seed)
    return rng.integers(0, np.iinfo(dt).max, size=(3, 2, n), dtype=dt, endpoint=True)


# ------------------------------------------------------------------ protocol

def reconstruct(a, comm=None):
    dt, suf = _ring(np.asarray(a).dtype)
    a = _views(a, dt)
    n = a.shape[2]
    out = np.empty((3, n), dtype=dt)
    comm = comm or Comm()
    getattr(lib(), f"or_rss_reconstruct_{suf}")(_p(a), ctypes.c_size_t(n), _p(out), comm.ptr())
    return out


def reshare(c, comm=None):
    dt, suf = _ring(np.asarray(c).dtype)
    c = np.ascontiguousarray(c, dtype=dt)
    n = c.shape[1]
    out = np.empty((3, 2, n), dtype=dt)
    comm = comm or Comm()
    getattr(lib(), f"or_rss_reshare_{suf}")(_p(c), ctypes.c_size_t(n), _p(out), comm.ptr())
    return out


def matmul(a, b, M, N, K, tA, tB, tC, trunc, comm=None):
    """RSS matmul (RSS.inl:482-540): localMatMul + dividePublic3out3."""
    dt, suf = _ring(np.asarray(a).dtype)
    a = _views(a, dt, M * K)
    b = _views(b, dt, K * N)
    c = np.empty((3, 2, M * N), dtype=dt)
    comm = comm or Comm()
    getattr(lib(), f"or_rss_matmul_{suf}")(_p(a), _p(b), _p(c), M, N, K, int(tA), int(tB), int(tC), trunc,
                                           comm.ptr())
    return c


def conv_out_size(op, batch, H, W, f, Din, Dout, stride, pad):
    P = (H + 2 * pad - f) // stride + 1
    Q = (W + 2 * pad - f) // stride + 1
    if op == FPROP:
        return batch * P * Q * Dout
    if op == DGRAD:
        return batch * H * W * Din
    return Dout * f * f * Din


def convolution(a, b, op, batch, H, W, f, Din, Dout, stride, pad, trunc, comm=None):
    """RSS convolution (RSS.inl:706-803)."""
    dt, suf = _ring(np.asarray(a).dtype)
    a = _views(a, dt)
    b = _views(b, dt)
    n_out = conv_out_size(op, batch, H, W, f, Din, Dout, stride, pad)
    c = np.empty((3, 2, n_out), dtype=dt)
    comm = comm or Comm()
    getattr(lib(), f"or_rss_conv_{suf}")(_p(a), ctypes.c_size_t(a.shape[2]), _p(b), ctypes.c_size_t(b.shape[2]),
                                         _p(c), op, batch, H, W, f, Din, Dout, stride, pad, trunc, comm.ptr())
    return c


def divide_public(a, d, comm=None):
    """dividePublic (RSS.inl:423-455); d is a scalar or a per-element array."""
    dt, suf = _ring(np.asarray(a).dtype)
    a = _views(a, dt).copy()
    n = a.shape[2]
    dv = np.ascontiguousarray(np.atleast_1d(np.asarray(d, dtype=dt)))
    vec = dv.size > 1 or (np.ndim(d) > 0)
    if vec and dv.size != n:
        raise ValueError("denominator vector size mismatch")
    comm = comm or Comm()
    getattr(lib(), f"or_rss_divide_public_{suf}")(_p(a), ctypes.c_size_t(n), _p(dv), int(vec), comm.ptr())
    return a


def divide_3of3(z, d, comm=None):
    dt, suf = _ring(np.asarray(z).dtype)
    z = np.ascontiguousarray(z, dtype=dt)
    n = z.shape[1]
    out = np.zeros((3, 2, n), dtype=dt)
    comm = comm or Comm()
    getattr(lib(), f"or_rss_divide_3of3_{suf}")(_p(z), ctypes.c_size_t(n), _CT[dt](int(d)), _p(out), comm.ptr())
    return out


def mul(a, b, comm=None):
    dt, suf = _ring(np.asarray(a).dtype)
    a = _views(a, dt).copy()
    b = _views(b, dt, a.shape[2])
    comm = comm or Comm()
    getattr(lib(), f"or_rss_mul_{suf}")(_p(a), _p(b), ctypes.c_size_t(a.shape[2]), comm.ptr())
    return a


def and_(a, b, comm=None):
    dt, suf = _ring(np.asarray(a).dtype)
    a = _views(a, dt).copy()
    b = _views(b, dt, a.shape[2])
    comm = comm or Comm()
    getattr(lib(), f"or_rss_and_{suf}")(_p(a), _p(b), ctypes.c_size_t(a.shape[2]), comm.ptr())
    return a


def _bits_suffix(dt, udt):
    return f"{_SUF[dt]}_{_SUF[np.dtype(udt).type]}"


def drelu(x, udtype=np.uint8, comm=None):
    dt, _ = _ring(np.asarray(x).dtype)
    x = _views(x, dt)
    n = x.shape[2]
    out = np.empty((3, 2, n), dtype=udtype)
    comm = comm or Comm()
    getattr(lib(), f"or_rss_drelu_{_bits_suffix(dt, udtype)}")(_p(x), ctypes.c_size_t(n), _p(out), comm.ptr())
    return out


def relu(x, udtype=np.uint8, comm=None):
    dt, _ = _ring(np.asarray(x).dtype)
    x = _views(x, dt)
    n = x.shape[2]
    out = np.empty((3, 2, n), dtype=dt)
    dout = np.empty((3, 2, n), dtype=udtype)
    comm = comm or Comm()
    getattr(lib(), f"or_rss_relu_{_bits_suffix(dt, udtype)}")(_p(x), ctypes.c_size_t(n), _p(out), _p(dout),
                                                              comm.ptr())
    return out, dout


def select_share(x, y, b, comm=None):
    dt, _ = _ring(np.asarray(x).dtype)
    x = _views(x, dt)
    n = x.shape[2]
    y = _views(y, dt, n)
    b = np.ascontiguousarray(b)
    z = np.empty((3, 2, n), dtype=dt)
    comm = comm or Comm()
    getattr(lib(), f"or_rss_select_share_{_bits_suffix(dt, b.dtype)}")(_p(x), _p(y), _p(b), _p(z),
                                                                       ctypes.c_size_t(n), comm.ptr())
    return z


def maxpool(x, k, udtype=np.uint8, comm=None):
    """RSS maxpool tournament (RSS.inl:868-1017) over rows of k (padded) values."""
    dt, _ = _ring(np.asarray(x).dtype)
    x = _views(x, dt)
    n = x.shape[2]
    out = np.empty((3, 2, n // k), dtype=dt)
    dout = np.empty((3, 2, n), dtype=udtype)
    comm = comm or Comm()
    getattr(lib(), f"or_rss_maxpool_{_bits_suffix(dt, udtype)}")(_p(x), ctypes.c_size_t(n), _p(out), _p(dout), k,
                                                                 comm.ptr())
    return out, dout


def maxpool_layer(x, H, W, C, pool, stride, batch, fp=FP_DEFAULT, udtype=np.uint8, comm=None):
    """MaxpoolLayer::forward (MaxpoolLayer.cu:52-131) for RSS."""
    dt, _ = _ring(np.asarray(x).dtype)
    x = _views(x, dt, batch * H * W * C)
    oh = (H - pool) // stride + 1
    ow = (W - pool) // stride + 1
    out = np.empty((3, 2, batch * oh * ow * C), dtype=dt)
    dout = np.empty((3, 2, batch * oh * ow * C * pool * pool), dtype=udtype)
    comm = comm or Comm()
    getattr(lib(), f"or_maxpool_layer_{_bits_suffix(dt, udtype)}")(_p(x), _p(out), _p(dout), H, W, C, pool,
                                                                   stride, batch, fp, comm.ptr())
    return out, dout


# -------------------------------------------------------- single-array kernels

def gemm(M, N, K, A, tA, B, tB, tC, dtype=np.uint64):
    dt, suf = _ring(dtype)
    A = np.ascontiguousarray(A, dtype=dt)
    B = np.ascontiguousarray(B, dtype=dt)
    C = np.empty(M * N, dtype=dt)
    getattr(lib(), f"or_gemm_{suf}")(M, N, K, _p(A), int(tA), _p(B), int(tB), _p(C), int(tC))
    return C


def conv(op, N, H, W, C, K, R, S, pad, stride, a, b, dtype=np.uint64):
    dt, suf = _ring(dtype)
    a = np.ascontiguousarray(a, dtype=dt)
    b = np.ascontiguousarray(b, dtype=dt)
    P = (H + 2 * pad - R) // stride + 1
    Q = (W + 2 * pad - S) // stride + 1
    n_out = {FPROP: N * P * Q * K, DGRAD: N * H * W * C, WGRAD: K * R * S * C}[op]
    out = np.empty(n_out, dtype=dt)
    getattr(lib(), f"or_conv_{suf}")(op, N, H, W, C, K, R, S, pad, stride, _p(a), _p(b), _p(out))
    return out


def maxpool_im2row(im, H, W, f, Din, batch, stride, pad, pad_val, dtype=np.uint64):
    dt, suf = _ring(dtype)
    im = np.ascontiguousarray(im, dtype=dt)
    fn = getattr(lib(), f"or_maxpool_im2row_{suf}")
    fn.restype = ctypes.c_size_t
    n = fn(_p(im), None, ctypes.c_size_t(0), H, W, f, Din, batch, stride, pad, _CT[dt](int(pad_val) % (1 << 64)))
    out = np.empty(n, dtype=dt)
    fn(_p(im), _p(out), ctypes.c_size_t(n), H, W, f, Din, batch, stride, pad, _CT[dt](int(pad_val) % (1 << 64)))
    return out


def element_vector_add(a, b, rowwise, rows, cols, dtype=np.uint64):
    dt, suf = _ring(dtype)
    a = np.ascontiguousarray(a, dtype=dt).copy()
    b = np.ascontiguousarray(b, dtype=dt)
    getattr(lib(), f"or_element_vector_add_{suf}")(_p(a), _p(b), int(rowwise), rows, cols)
    return a


def reduce_sum(a, b, reduce_rows, rows, cols, dtype=np.uint64):
    dt, suf = _ring(dtype)
    a = np.ascontiguousarray(a, dtype=dt)
    b = np.ascontiguousarray(b, dtype=dt).copy()
    getattr(lib(), f"or_reduce_sum_{suf}")(_p(a), _p(b), int(reduce_rows), rows, cols)
    return b


def bitexpand(a, dtype=np.uint64):
    dt, suf = _ring(dtype)
    a = np.ascontiguousarray(a, dtype=dt)
    bits = np.empty(a.size * np.dtype(dt).itemsize * 8, dtype=dt)
    getattr(lib(), f"or_bitexpand_{suf}")(_p(a), ctypes.c_size_t(a.size), _p(bits))
    return bits


def expand_compare(b, nb, out_n):
    b = np.ascontiguousarray(b, dtype=np.uint8)
    nb = np.ascontiguousarray(nb, dtype=np.uint8)
    out = np.empty(out_n, dtype=np.uint8)
    lib().or_expand_compare_u8(_p(b), _p(nb), ctypes.c_size_t(b.size), _p(out), ctypes.c_size_t(out_n))
    return out


def div_public_values(x, d, dtype=np.uint64):
    """The ring division functor alone (functors.cuh:33-45,94-105)."""
    dt, suf = _ring(dtype)
    x = np.ascontiguousarray(x, dtype=dt).ravel()
    dv = np.ascontiguousarray(np.atleast_1d(np.asarray(d, dtype=dt)))
    out = np.empty_like(x)
    getattr(lib(), f"or_div_public_scalar_{suf}")(_p(x), ctypes.c_size_t(x.size), _p(dv), int(dv.size > 1), _p(out))
    return out


# ------------------------------------------------------- training step (RSS)

def vector_expand(a, f):
    """vectorExpand (matrix.cuh:129-139)."""
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.empty(a.size * f, dtype=np.uint64)
    lib().or_vector_expand_u64(_p(a), ctypes.c_size_t(a.size), _p(b), ctypes.c_size_t(f))
    return b


def maxpool_row2im(rows, out, image_height, image_width, f, Din, batch, stride):
    """maxpool_row2im (convolution.cuh:111-152): adds into a copy of out."""
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    out = np.ascontiguousarray(out, dtype=np.uint64).copy()
    lib().or_maxpool_row2im_u64(_p(rows), _p(out), image_height, image_width, f, Din, batch, stride)
    return out


def avgpool_layer(x, H, W, C, pool, stride, batch, comm=None):
    """AveragepoolLayer::forward (AveragepoolLayer.cu:58-81) for RSS."""
    x = _views(x, np.uint64, batch * H * W * C)
    oh, ow = (H - pool) // stride + 1, (W - pool) // stride + 1
    out = np.empty((3, 2, batch * oh * ow * C), dtype=np.uint64)
    comm = comm or Comm()
    lib().or_avgpool_layer_forward_u64(_p(x), _p(out), H, W, C, pool, stride, batch, comm.ptr())
    return out


def avgpool_layer_backward(delta, H, W, C, pool, batch, comm=None):
    """AveragepoolLayer::backward (AveragepoolLayer.cu:88-117)."""
    delta = _views(delta, np.uint64)
    out = np.empty((3, 2, batch * H * W * C), dtype=np.uint64)
    comm = comm or Comm()
    if lib().or_avgpool_layer_backward_u64(_p(delta), ctypes.c_size_t(delta.shape[2]), _p(out), H, W, C, pool,
                                           batch, comm.ptr()):
        raise ValueError(f"averagepool backward: {delta.shape[2]} deltas x pool {pool}^2 exceed the "
                         f"{batch * H * W * C}-element input gradient (overlapping pools)")
    return out


def relu_layer_backward(delta, relu_prime, comm=None):
    """ReLULayer::backward (ReLULayer.cu:90-124)."""
    delta = _views(delta, np.uint64)
    n = delta.shape[2]
    b = np.ascontiguousarray(relu_prime, dtype=np.uint8)
    out = np.empty((3, 2, n), dtype=np.uint64)
    comm = comm or Comm()
    lib().or_relu_layer_backward_u64_u8(_p(delta), ctypes.c_size_t(n), _p(b), _p(out), comm.ptr())
    return out


def maxpool_layer_backward(delta, max_prime, H, W, C, pool, stride, batch, comm=None):
    """MaxpoolLayer::backward (MaxpoolLayer.cu:133-185)."""
    delta = _views(delta, np.uint64)
    n = delta.shape[2]
    mp = np.ascontiguousarray(max_prime, dtype=np.uint8)
    if mp.shape != (3, 2, n * pool * pool):
        raise ValueError("maxPrime must have shape (3, 2, n * pool^2)")
    out = np.empty((3, 2, batch * H * W * C), dtype=np.uint64)
    comm = comm or Comm()
    lib().or_maxpool_layer_backward_u64_u8(_p(delta), ctypes.c_size_t(n), _p(mp), _p(out), H, W, C, pool, stride,
                                           batch, comm.ptr())
    return out


def fc_layer_backward(delta, fwd_in, w, b, batch, din, dout, fp, lr, comm=None):
    """FCLayer::backward (FCLayer.cu:132-217): returns (deltas, new w, new b)."""
    delta = _views(delta, np.uint64, batch * dout)
    fwd_in = _views(fwd_in, np.uint64, batch * din)
    w = _views(w, np.uint64, din * dout).copy()
    b = _views(b, np.uint64, dout).copy()
    out = np.empty((3, 2, batch * din), dtype=np.uint64)
    comm = comm or Comm()
    lib().or_fc_layer_backward_u64(_p(delta), _p(fwd_in), _p(w), _p(b), _p(out), batch, din, dout, fp, lr,
                                   comm.ptr())
    return out, w, b


def cnn_layer_backward(delta, fwd_in, w, batch, H, W, Din, Dout, f, stride, pad, fp, lr, comm=None):
    """CNNLayer::backward (CNNLayer.cu:114-193): returns (deltas, new w)."""
    delta = _views(delta, np.uint64)
    fwd_in = _views(fwd_in, np.uint64, batch * H * W * Din)
    w = _views(w, np.uint64, Dout * f * f * Din).copy()
    out = np.empty((3, 2, batch * H * W * Din), dtype=np.uint64)
    comm = comm or Comm()
    lib().or_cnn_layer_backward_u64(_p(delta), _p(fwd_in), _p(w), _p(out), batch, H, W, Din, Dout, f, stride, pad,
                                    fp, lr, comm.ptr())
    return out, w


def reveal_softmax_grad(act, labels, batch, fp=FP_DEFAULT, comm=None):
    """NeuralNetwork::_reveal_softmax_grad (NeuralNetwork.cu:207-267)."""
    act = _views(act, np.uint64)
    n = act.shape[2]
    labels = _views(labels, np.uint64, n)
    out = np.empty((3, 2, n), dtype=np.uint64)
    comm = comm or Comm()
    lib().or_reveal_softmax_grad_u64(_p(act), _p(labels), ctypes.c_size_t(n), batch, fp, _p(out), comm.ptr())
    return out


# ------------------------------------------------------------------- TPC
# A TPC tensor of n elements is a numpy array of shape (2, n): [party A/B][element]
# (src/mpc/TPC.h: one additive share per party).

def _tviews(a, dtype, n=None):
    a = np.ascontiguousarray(a, dtype=dtype)
    if a.ndim != 2 or a.shape[0] != 2 or (n is not None and a.shape[1] != n):
        raise ValueError(f"expected TPC shares of shape (2, {n}), got {a.shape}")
    return a


def tpc_from_list(vals, dtype=np.uint64, fp=FP_DEFAULT, to_fixed=True):
    """setPublic / initializer list (TPC.inl:109-123, :341-363): party A holds the values."""
    dt, suf = _ring(dtype)
    v = np.ascontiguousarray(vals, dtype=np.float64).ravel()
    out = np.empty((2, v.size), dtype=dt)
    getattr(lib(), f"or_tpc_from_list_{suf}")(_p(v), ctypes.c_size_t(v.size), fp, int(to_fixed), _p(out))
    return out


def tpc_share_random(secret, dtype=np.uint64, seed=0):
    """A valid 2-party sharing of `secret` with a seeded random mask for party B."""
    dt, _ = _ring(dtype)
    s = np.ascontiguousarray(secret, dtype=dt).ravel()
    rng = np.random.default_rng(seed)
    mask = rng.integers(0, np.iinfo(dt).max, size=s.size, dtype=dt, endpoint=True)
    return np.stack([(s - mask).astype(dt), mask])


def tpc_reconstruct(a, comm=None):
    """reconstruct (TPC.inl:552-572): both parties get share A + share B (uint64/uint32/uint8)."""
    dt = np.asarray(a).dtype.type
    suf = _SUF[dt]
    a = _tviews(a, dt)
    n = a.shape[1]
    out = np.empty((2, n), dtype=dt)
    comm = comm or Comm()
    getattr(lib(), f"or_tpc_reconstruct_{suf}")(_p(a), ctypes.c_size_t(n), _p(out), comm.ptr())
    return out


def tpc_matmul(a, b, M, N, K, tA, tB, tC, trunc, comm=None):
    """TPC matmul (TPC.inl:575-583): localMatMul with the matrix triple, then dividePublic."""
    dt, suf = _ring(np.asarray(a).dtype)
    a = _tviews(a, dt, M * K)
    b = _tviews(b, dt, K * N)
    c = np.empty((2, M * N), dtype=dt)
    comm = comm or Comm()
    getattr(lib(), f"or_tpc_matmul_{suf}")(_p(a), _p(b), _p(c), M, N, K, int(tA), int(tB), int(tC), trunc,
                                           comm.ptr())
    return c


def tpc_convolution(a, b, op, batch, H, W, f, Din, Dout, stride, pad, trunc, comm=None):
    """TPC convolution (TPC.inl:789-827)."""
    dt, suf = _ring(np.asarray(a).dtype)
    a = _tviews(a, dt)
    b = _tviews(b, dt)
    n_out = conv_out_size(op, batch, H, W, f, Din, Dout, stride, pad)
    c = np.empty((2, n_out), dtype=dt)
    comm = comm or Comm()
    getattr(lib(), f"or_tpc_conv_{suf}")(_p(a), ctypes.c_size_t(a.shape[1]), _p(b), ctypes.c_size_t(b.shape[1]),
                                         _p(c), op, batch, H, W, f, Din, Dout, stride, pad, trunc, comm.ptr())
    return c


def tpc_divide_public(a, d, comm=None):
    dt, suf = _ring(np.asarray(a).dtype)
    a = _tviews(a, dt).copy()
    n = a.shape[1]
    dv = np.ascontiguousarray(np.atleast_1d(np.asarray(d, dtype=dt)))
    vec = dv.size > 1 or (np.ndim(d) > 0)
    if vec and dv.size != n:
        raise ValueError("denominator vector size mismatch")
    comm = comm or Comm()
    getattr(lib(), f"or_tpc_divide_public_{suf}")(_p(a), ctypes.c_size_t(n), _p(dv), int(vec), comm.ptr())
    return a


def tpc_mul(a, b, comm=None):
    dt, suf = _ring(np.asarray(a).dtype)
    a = _tviews(a, dt).copy()
    b = _tviews(b, dt, a.shape[1])
    comm = comm or Comm()
    getattr(lib(), f"or_tpc_mul_{suf}")(_p(a), _p(b), ctypes.c_size_t(a.shape[1]), comm.ptr())
    return a


def tpc_drelu(x, udtype=np.uint8, comm=None):
    dt, _ = _ring(np.asarray(x).dtype)
    x = _tviews(x, dt)
    n = x.shape[1]
    out = np.empty((2, n), dtype=udtype)
    comm = comm or Comm()
    getattr(lib(), f"or_tpc_drelu_{_bits_suffix(dt, udtype)}")(_p(x), ctypes.c_size_t(n), _p(out), comm.ptr())
    return out


def tpc_relu(x, udtype=np.uint8, comm=None):
    dt, _ = _ring(np.asarray(x).dtype)
    x = _tviews(x, dt)
    n = x.shape[1]
    out = np.empty((2, n), dtype=dt)
    dout = np.empty((2, n), dtype=udtype)
    comm = comm or Comm()
    getattr(lib(), f"or_tpc_relu_{_bits_suffix(dt, udtype)}")(_p(x), ctypes.c_size_t(n), _p(out), _p(dout),
                                                              comm.ptr())
    return out, dout


def tpc_select_share(x, y, b, comm=None):
    dt, _ = _ring(np.asarray(x).dtype)
    x = _tviews(x, dt)
    n = x.shape[1]
    y = _tviews(y, dt, n)
    b = np.ascontiguousarray(b)
    z = np.empty((2, n), dtype=dt)
    comm = comm or Comm()
    getattr(lib(), f"or_tpc_select_share_{_bits_suffix(dt, b.dtype)}")(_p(x), _p(y), _p(b), ctypes.c_size_t(n),
                                                                       _p(z), comm.ptr())
    return z


def tpc_maxpool(x, k, udtype=np.uint8, comm=None):
    """TPC maxpool tournament (TPC.inl:887-1058) over rows of k (padded) values."""
    dt, _ = _ring(np.asarray(x).dtype)
    x = _tviews(x, dt)
    n = x.shape[1]
    out = np.empty((2, n // k), dtype=dt)
    dout = np.empty((2, n), dtype=udtype)
    comm = comm or Comm()
    getattr(lib(), f"or_tpc_maxpool_{_bits_suffix(dt, udtype)}")(_p(x), ctypes.c_size_t(n), k, _p(out), _p(dout),
                                                                 comm.ptr())
    return out, dout


# ------------------------------------------------------------------- FPC
# An FPC tensor of n elements is a numpy array of shape (4, 3, n):
# [party A/B/C/D][shareA/shareB/shareC][element]; party p's share k holds the
# component x_{(p+1+k) mod 4} of x = x0 + x1 + x2 + x3 (src/mpc/FPC.inl:948-953).

def _fviews(a, dtype, n=None):
    a = np.ascontiguousarray(a, dtype=dtype)
    if a.ndim != 3 or a.shape[:2] != (4, 3) or (n is not None and a.shape[2] != n):
        raise ValueError(f"expected FPC views of shape (4, 3, {n}), got {a.shape}")
    return a


def fpc_from_list(vals, dtype=np.uint64, fp=FP_DEFAULT, to_fixed=True):
    """setPublic / initializer list (FPC.inl:127-155, :528-565): component x0 holds the values."""
    dt = np.dtype(dtype).type
    v = np.ascontiguousarray(vals, dtype=np.float64).ravel()
    out = np.empty((4, 3, v.size), dtype=dt)
    getattr(lib(), f"or_fpc_from_list_{_SUF[dt]}")(_p(v), ctypes.c_size_t(v.size), fp, int(to_fixed), _p(out))
    return out


def fpc_share_random(secret, dtype=np.uint64, seed=0):
    """A consistent 4-party replicated sharing of `secret` with seeded random x1, x2, x3."""
    dt = np.dtype(dtype).type
    s = np.ascontiguousarray(secret, dtype=dt).ravel()
    rng = np.random.default_rng(seed)
    comp = [None] + [rng.integers(0, np.iinfo(dt).max, size=s.size, dtype=dt, endpoint=True) for _ in range(3)]
    comp[0] = (s - comp[1] - comp[2] - comp[3]).astype(dt)
    out = np.empty((4, 3, s.size), dtype=dt)
    for p in range(4):
        for k in range(3):
            out[p, k] = comp[(p + 1 + k) % 4]
    return out


def fpc_reconstruct(a, comm=None):
    """reconstruct (FPC.inl:611-634): own three shares plus the previous party's shareA."""
    dt = np.asarray(a).dtype.type
    a = _fviews(a, dt)
    n = a.shape[2]
    out = np.empty((4, n), dtype=dt)
    comm = comm or Comm(4)
    getattr(lib(), f"or_fpc_reconstruct_{_SUF[dt]}")(_p(a), ctypes.c_size_t(n), _p(out), comm.ptr())
    return out


def fpc_matmul(a, b, M, N, K, tA, tB, tC, trunc, comm=None):
    """FPC matmul (FPC.inl:636-670): local products, six reshares, dividePublic."""
    dt, suf = _ring(np.asarray(a).dtype)
    a = _fviews(a, dt, M * K)
    b = _fviews(b, dt, K * N)
    c = np.empty((4, 3, M * N), dtype=dt)
    comm = comm or Comm(4)
    getattr(lib(), f"or_fpc_matmul_{suf}")(_p(a), _p(b), _p(c), M, N, K, int(tA), int(tB), int(tC), trunc,
                                           comm.ptr())
    return c


def fpc_convolution(a, b, op, batch, H, W, f, Din, Dout, stride, pad, trunc, comm=None):
    """FPC convolution (FPC.inl:862-925)."""
    dt, suf = _ring(np.asarray(a).dtype)
    a = _fviews(a, dt)
    b = _fviews(b, dt)
    n_out = conv_out_size(op, batch, H, W, f, Din, Dout, stride, pad)
    c = np.empty((4, 3, n_out), dtype=dt)
    comm = comm or Comm(4)
    getattr(lib(), f"or_fpc_conv_{suf}")(_p(a), ctypes.c_size_t(a.shape[2]), _p(b), ctypes.c_size_t(b.shape[2]),
                                         _p(c), op, batch, H, W, f, Din, Dout, stride, pad, trunc, comm.ptr())
    return c


def fpc_divide_public(a, d, comm=None):
    dt, suf = _ring(np.asarray(a).dtype)
    a = _fviews(a, dt).copy()
    n = a.shape[2]
    dv = np.ascontiguousarray(np.atleast_1d(np.asarray(d, dtype=dt)))
    vec = dv.size > 1 or (np.ndim(d) > 0)
    if vec and dv.size != n:
        raise ValueError("denominator vector size mismatch")
    comm = comm or Comm(4)
    getattr(lib(), f"or_fpc_divide_public_{suf}")(_p(a), ctypes.c_size_t(n), _p(dv), int(vec), comm.ptr())
    return a


def fpc_mul(a, b, comm=None):
    dt, suf = _ring(np.asarray(a).dtype)
    a = _fviews(a, dt).copy()
    b = _fviews(b, dt, a.shape[2])
    comm = comm or Comm(4)
    getattr(lib(), f"or_fpc_mul_{suf}")(_p(a), _p(b), ctypes.c_size_t(a.shape[2]), comm.ptr())
    return a


def fpc_and(a, b, comm=None):
    dt = np.asarray(a).dtype.type
    a = _fviews(a, dt).copy()
    b = _fviews(b, dt, a.shape[2])
    comm = comm or Comm(4)
    getattr(lib(), f"or_fpc_and_{_SUF[dt]}")(_p(a), _p(b), ctypes.c_size_t(a.shape[2]), comm.ptr())
    return a


def fpc_drelu(x, udtype=np.uint8, comm=None):
    dt, _ = _ring(np.asarray(x).dtype)
    x = _fviews(x, dt)
    n = x.shape[2]
    out = np.empty((4, 3, n), dtype=udtype)
    comm = comm or Comm(4)
    getattr(lib(), f"or_fpc_drelu_{_bits_suffix(dt, udtype)}")(_p(x), ctypes.c_size_t(n), _p(out), comm.ptr())
    return out


def fpc_relu(x, udtype=np.uint8, comm=None):
    dt, _ = _ring(np.asarray(x).dtype)
    x = _fviews(x, dt)
    n = x.shape[2]
    out = np.empty((4, 3, n), dtype=dt)
    dout = np.empty((4, 3, n), dtype=udtype)
    comm = comm or Comm(4)
    getattr(lib(), f"or_fpc_relu_{_bits_suffix(dt, udtype)}")(_p(x), ctypes.c_size_t(n), _p(out), _p(dout),
                                                              comm.ptr())
    return out, dout


def fpc_select_share(x, y, b, comm=None):
    dt, _ = _ring(np.asarray(x).dtype)
    x = _fviews(x, dt)
    n = x.shape[2]
    y = _fviews(y, dt, n)
    b = np.ascontiguousarray(b)
    z = np.empty((4, 3, n), dtype=dt)
    comm = comm or Comm(4)
    getattr(lib(), f"or_fpc_select_share_{_bits_suffix(dt, b.dtype)}")(_p(x), _p(y), _p(b), ctypes.c_size_t(n),
                                                                       _p(z), comm.ptr())
    return z


def fpc_maxpool(x, k, udtype=np.uint8, comm=None):
    """FPC maxpool tournament (FPC.inl:1005-1177) over rows of k (padded) values."""
    dt, _ = _ring(np.asarray(x).dtype)
    x = _fviews(x, dt)
    n = x.shape[2]
    out = np.empty((4, 3, n // k), dtype=dt)
    dout = np.empty((4, 3, n), dtype=udtype)
    comm = comm or Comm(4)
    getattr(lib(), f"or_fpc_maxpool_{_bits_suffix(dt, udtype)}")(_p(x), ctypes.c_size_t(n), k, _p(out), _p(dout),
                                                                 comm.ptr())
    return out, dout


# ---------------------------------------------------------------- generator

def aes256_encrypt(key: bytes, block: bytes) -> bytes:
    """One AES-256 block (FIPS-197), restated byte by byte."""
    assert len(key) == 32 and len(block) == 16
    out = ctypes.create_string_buffer(16)
    lib().or_aes256_encrypt(key, block, out)
    return out.raw


def prg_fill_u64(key: bytes, counter: int, n: int) -> np.ndarray:
    """AESObject's uint64 stream from block `counter` (src/mpc/AESObject.cpp:40-91)."""
    assert len(key) == 32
    out = np.zeros(n, dtype=np.uint64)
    lib().or_prg_fill_u64(key, ctypes.c_uint64(counter), _p(out), ctypes.c_size_t(n))
    return out


def prg_masks(keys, counter: int, n: int, xor: bool = False, bits: bool = False) -> np.ndarray:
    """The resharing masks alpha_p = G(key p) - G(key p-1) (or XOR; low bit for
    bit shares) of n elements from block `counter`, as (3, n)."""
    g = [prg_fill_u64(k, counter, n) for k in keys]
    out = np.zeros((3, n), dtype=np.uint64)
    with np.errstate(over="ignore"):
        for p in range(3):
            q = (p + 2) % 3
            out[p] = (g[p] ^ g[q]) if xor else (g[p] - g[q])
    if bits:
        out &= np.uint64(1)
    return out


# ---------------------------------------------------------- local operators

def _local(op, a, rhs, pub_rows):
    a = np.array(a, dtype=np.uint64, copy=True)
    shape = a.shape
    n = shape[-1]
    flat = a.reshape(-1, n)
    if isinstance(rhs, (int, np.integer)):
        kind, r = "scalar", np.full(n, int(rhs) % (1 << 64), dtype=np.uint64)
    elif np.asarray(rhs).ndim == 1:
        kind, r = "public", np.asarray(rhs, dtype=np.uint64)
    else:
        kind, r = "shares", np.asarray(rhs, dtype=np.uint64).reshape(-1, n)
    with np.errstate(over="ignore"):
        for k in range(flat.shape[0]):
            x = flat[k]
            y = r[k] if kind == "shares" else r
            if op in ("add", "sub", "xor") and kind != "shares" and k not in pub_rows:
                continue
            if op == "add":
                x = x + y
            elif op == "sub":
                x = x - y
            elif op == "xor":
                x = x ^ y
            elif op == "mul":
                x = x * y
            elif op == "and":
                x = x & y
            elif op == "shr":
                sx = x.view(np.int64)
                x = np.where(y >= 64, np.where(sx < 0, np.uint64(2**64 - 1), np.uint64(0)),
                             (sx >> np.minimum(y, 63).astype(np.int64)).view(np.uint64))
            elif op == "shl":
                x = np.where(y >= 64, np.uint64(0), x << np.minimum(y, np.uint64(63)))
            flat[k] = x
    return flat.reshape(shape)


def rss_local(op, a, rhs):
    """RSSBase's local operators (src/mpc/RSS.inl:168-345) on (3, 2, n) uint64
    views: rhs an int (public scalar), an (n,) array (public DeviceData) or
    (3, 2, n) shares. Public + - ^ go to party A's shareA and party C's shareB;
    * & and shifts to every share; shares + - ^ share by share. >> is the
    arithmetic shift of functors.cuh:48-70; shifts of 64 or more saturate."""
    return _local(op, a, rhs, {0, 5})


def tpc_local(op, a, rhs):
    """TPCBase's local operators (src/mpc/TPC.inl:146-240) on (2, n) views:
    public + - ^ at party A's share."""
    return _local(op, a, rhs, {0})


def fpc_local(op, a, rhs):
    """FPCBase's local operators (src/mpc/FPC.inl:187-300) on (4, 3, n) views:
    public + - ^ in the x0 component (party B's shareC, party C's shareB,
    party D's shareA)."""
    return _local(op, a, rhs, {5, 7, 9})
