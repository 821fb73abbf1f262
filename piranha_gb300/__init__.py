"""piranha_gb300 — GB300-native party-local secret-share arithmetic (Piranha's hot path).

The compute lives in ``libpiranha_gb300.so`` (hand-written sm_103a CUDA behind
the C ABI of ``include/piranha_gb300.h``). This module is the Python host
mirror of the reference's operator surface (``src/mpc/RSS.h:105-145``,
``src/gpu/gemm.cuh``, ``src/gpu/conv.cuh``): the same operation names and
argument meanings, operating on all three simulated parties at once.

Share tensors are torch CUDA tensors of shape ``(3, 2, n)`` —
``[party A/B/C][shareA/shareB][element]`` — holding ring elements
(uint64 stored as ``torch.int64`` bit patterns, uint32 as ``torch.int32``,
bit shares as ``torch.uint8``). PyTorch only provides device memory and
streams here; every operation below is one or more launches of this
library's own kernels. There is no CPU fallback: if the library cannot be
built or loaded, importing the ops raises.
"""
from __future__ import annotations

import ctypes
import os
import threading
import weakref

import numpy as np

from . import build as _build

PG_OK = 0
FORM_U64, FORM_LIMB_TC = 0, 1
RATE_TC_F16, RATE_TC_F8, RATE_MMA_S8, RATE_MMA_F16 = 0, 1, 2, 3
FPROP, DGRAD, WGRAD = 0, 1, 2
LAYER_FC, LAYER_CNN, LAYER_RELU, LAYER_MAXPOOL, LAYER_AVGPOOL = 1, 2, 3, 4, 5
OP_ADD, OP_SUB, OP_MUL, OP_XOR, OP_AND, OP_SHR, OP_SHL, OP_DIV, OP_SET = range(9)
RHS_SCALAR, RHS_PUBLIC, RHS_SHARES = range(3)
FLOAT_PRECISION = 26

_lib = None
_lock = threading.Lock()


class PiranhaError(RuntimeError):
    pass


_P6 = ctypes.c_void_p * 6
_P3 = ctypes.c_void_p * 3
_P2 = ctypes.c_void_p * 2
_P4 = ctypes.c_void_p * 4
_P12 = ctypes.c_void_p * 12


def _declare(lib):
    vp, i, sz, u64, u32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_uint32
    sig = {
        "pg_ctx_create": [ctypes.POINTER(vp), i],
        "pg_ctx_destroy": [vp],
        "pg_ctx_set_stream": [vp, vp],
        "pg_ctx_set_form": [vp, i],
        "pg_ctx_get_form": [vp],
        "pg_sync": [vp],
        "pg_comm_get": [vp, vp],
        "pg_comm_reset": [vp],
        "pg_gemm_u64": [vp, i, i, i, vp, i, vp, i, vp, i],
        "pg_gemm_u32": [vp, i, i, i, vp, i, vp, i, vp, i],
        "pg_conv_u64": [vp, i, i, i, i, i, i, i, i, i, i, vp, vp, vp],
        "pg_rss_matmul_u64": [vp, _P6, _P6, _P6, i, i, i, i, i, i, i],
        "pg_rss_matmul_u32": [vp, _P6, _P6, _P6, i, i, i, i, i, i, i],
        "pg_rss_fc_forward_u64": [vp, _P6, _P6, vp, _P6, i, i, i, i],
        "pg_rss_conv_u64": [vp, _P6, _P6, _P6, i, i, i, i, i, i, i, i, i, i],
        "pg_rss_divide_public_u64": [vp, _P6, sz, u64],
        "pg_rss_divide_public_vec_u64": [vp, _P6, sz, vp],
        "pg_rss_divide_public_u32": [vp, _P6, sz, u32],
        "pg_rss_reconstruct_u64": [vp, _P6, sz, _P3],
        "pg_rss_reconstruct_u8": [vp, _P6, sz, _P3],
        "pg_rss_reshare_u64": [vp, _P3, sz, _P6],
        "pg_rss_mul_u64": [vp, _P6, _P6, sz],
        "pg_rss_and_u64": [vp, _P6, _P6, sz],
        "pg_rss_and_u8": [vp, _P6, _P6, sz],
        "pg_rss_drelu_u64_u8": [vp, _P6, sz, _P6],
        "pg_rss_drelu_u64_u64": [vp, _P6, sz, _P6],
        "pg_rss_relu_u64_u8": [vp, _P6, sz, _P6, _P6],
        "pg_rss_relu_u64_u64": [vp, _P6, sz, _P6, _P6],
        "pg_rss_relu_u32_u8": [vp, _P6, sz, _P6, _P6],
        "pg_rss_select_share_u64_u8": [vp, _P6, _P6, _P6, _P6, sz],
        "pg_rss_select_share_u64_u64": [vp, _P6, _P6, _P6, _P6, sz],
        "pg_rss_maxpool_u64_u8": [vp, _P6, sz, i, _P6, _P6],
        "pg_rss_maxpool_u64_u64": [vp, _P6, sz, i, _P6, _P6],
        "pg_rss_maxpool_layer_u64_u8": [vp, _P6, _P6, _P6, i, i, i, i, i, i, i],
        "pg_rss_avgpool_layer_u64": [vp, _P6, _P6, i, i, i, i, i, i],
        "pg_rss_avgpool_backward_u64": [vp, _P6, _P6, i, i, i, i, i, i],
        "pg_element_vector_add_u64": [vp, vp, vp, i, i, i],
        "pg_reduce_sum_u64": [vp, vp, vp, i, i, i],
        "pg_truncate_cols_u8": [vp, vp, vp, sz, i, i],
        "pg_bitexpand_u64": [vp, vp, sz, vp],
        "pg_expand_compare_u8": [vp, vp, vp, sz, vp, sz],
        "pg_maxpool_im2row_u64": [vp, vp, vp, i, i, i, i, i, i, i, u64],
        "pg_net_create": [vp, ctypes.POINTER(vp), vp, i, i, i],
        "pg_net_destroy": [vp],
        "pg_net_set_params": [vp, i, _P6, vp],
        "pg_net_forward": [vp, _P6, _P6],
        "pg_net_forward_host": [vp, vp, vp],
        "pg_net_forward_resident": [vp],
        "pg_net_capture": [vp],
        "pg_net_input_shares": [vp, _P6],
        "pg_net_layer_output": [vp, i, _P6, ctypes.POINTER(sz)],
        "pg_net_enable_timing": [vp, i],
        "pg_net_train_setup": [vp],
        "pg_net_train_step": [vp, _P6, _P6, i],
        "pg_net_backward": [vp, _P6, _P6, i],
        "pg_net_label_shares": [vp, _P6],
        "pg_net_capture_train": [vp, i],
        "pg_net_train_resident": [vp],
        "pg_net_train_host": [vp, vp, vp, vp, i],
        "pg_net_layer_delta": [vp, i, _P6, ctypes.POINTER(sz)],
        "pg_net_layer_params": [vp, i, _P6, _P6, ctypes.POINTER(sz), ctypes.POINTER(sz)],
        "pg_device_errors": [vp, ctypes.POINTER(i)],
        "pg_tc_selftest": [vp, vp, vp, vp],
        "pg_tensor_rate": [vp, i, i, vp],
        "pg_device_op_u64": [vp, i, vp, sz, i, u64, vp],
        "pg_ctx_set_wait_limit": [vp, u64, i],
        "pg_net_layer_plan": [vp, i, vp],
        "pg_party_create": [ctypes.POINTER(vp), i, i, vp, i, i],
        "pg_party_destroy": [vp],
        "pg_party_send": [vp, i, vp, sz],
        "pg_party_recv": [vp, i, vp, sz],
        "pg_party_exchange": [vp, vp, i, vp, sz, i, vp, sz],
        "pg_party_counters": [vp, vp],
        "pg_party_check": [vp],
        "pg_party_inject": [vp, i, i],
        "pg_party_rss_reconstruct_u64": [vp, vp, vp, sz, vp],
        "pg_party_rss_reshare_u64": [vp, vp, vp, sz, vp],
        "pg_party_rss_matmul_u64": [vp, vp, vp, vp, vp, i, i, i, i, i, i, i],
        "pg_net_layer_times": [vp, vp],
        "pg_tpc_matmul_u64": [vp, _P2, _P2, _P2, i, i, i, i, i, i, i],
        "pg_tpc_matmul_u32": [vp, _P2, _P2, _P2, i, i, i, i, i, i, i],
        "pg_tpc_fc_forward_u64": [vp, _P2, _P2, vp, _P2, i, i, i, i],
        "pg_tpc_fc_forward_u32": [vp, _P2, _P2, vp, _P2, i, i, i, i],
        "pg_tpc_conv_u64": [vp, _P2, _P2, _P2, i, i, i, i, i, i, i, i, i, i],
        "pg_tpc_divide_public_u64": [vp, _P2, sz, u64],
        "pg_tpc_divide_public_vec_u64": [vp, _P2, sz, vp],
        "pg_tpc_divide_public_u32": [vp, _P2, sz, u32],
        "pg_tpc_reconstruct_u64": [vp, _P2, sz, _P2],
        "pg_tpc_reconstruct_u32": [vp, _P2, sz, _P2],
        "pg_tpc_reconstruct_u8": [vp, _P2, sz, _P2],
        "pg_tpc_mul_u64": [vp, _P2, _P2, sz],
        "pg_tpc_drelu_u64_u8": [vp, _P2, sz, _P2],
        "pg_tpc_drelu_u32_u8": [vp, _P2, sz, _P2],
        "pg_tpc_relu_u64_u8": [vp, _P2, sz, _P2, _P2],
        "pg_tpc_relu_u32_u8": [vp, _P2, sz, _P2, _P2],
        "pg_tpc_select_share_u64_u8": [vp, _P2, _P2, _P2, _P2, sz],
        "pg_tpc_maxpool_u64_u8": [vp, _P2, sz, i, _P2, _P2],
        "pg_fpc_matmul_u64": [vp, _P12, _P12, _P12, i, i, i, i, i, i, i],
        "pg_fpc_matmul_u32": [vp, _P12, _P12, _P12, i, i, i, i, i, i, i],
        "pg_fpc_fc_forward_u64": [vp, _P12, _P12, vp, _P12, i, i, i, i],
        "pg_fpc_fc_forward_u32": [vp, _P12, _P12, vp, _P12, i, i, i, i],
        "pg_fpc_conv_u64": [vp, _P12, _P12, _P12, i, i, i, i, i, i, i, i, i, i],
        "pg_fpc_divide_public_u64": [vp, _P12, sz, u64],
        "pg_fpc_divide_public_vec_u64": [vp, _P12, sz, vp],
        "pg_fpc_divide_public_u32": [vp, _P12, sz, u32],
        "pg_fpc_reconstruct_u64": [vp, _P12, sz, _P4],
        "pg_fpc_reconstruct_u32": [vp, _P12, sz, _P4],
        "pg_fpc_reconstruct_u8": [vp, _P12, sz, _P4],
        "pg_fpc_mul_u64": [vp, _P12, _P12, sz],
        "pg_fpc_and_u8": [vp, _P12, _P12, sz],
        "pg_fpc_drelu_u64_u8": [vp, _P12, sz, _P12],
        "pg_fpc_drelu_u32_u8": [vp, _P12, sz, _P12],
        "pg_fpc_relu_u64_u8": [vp, _P12, sz, _P12, _P12],
        "pg_fpc_relu_u32_u8": [vp, _P12, sz, _P12, _P12],
        "pg_fpc_select_share_u64_u8": [vp, _P12, _P12, _P12, _P12, sz],
        "pg_fpc_maxpool_u64_u8": [vp, _P12, sz, i, _P12, _P12],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    lib.pg_last_error.argtypes = [vp]
    lib.pg_last_error.restype = ctypes.c_char_p
    lib.pg_party_last_error.argtypes = [vp]
    lib.pg_party_last_error.restype = ctypes.c_char_p
    lib.pg_kernel_launches.argtypes = [vp]
    lib.pg_kernel_launches.restype = ctypes.c_uint64
    lib.pg_reference_init_normal.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_size_t, ctypes.c_int,
                                             ctypes.c_double]
    lib.pg_ctx_set_autotune.argtypes = [vp, ctypes.c_int]
    lib.pg_rss_local_u64.argtypes = [vp, ctypes.c_int, vp, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint64, vp, vp]
    lib.pg_tpc_local_u64.argtypes = [vp, ctypes.c_int, vp, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint64, vp, vp]
    lib.pg_fpc_local_u64.argtypes = [vp, ctypes.c_int, vp, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint64, vp, vp]
    lib.pg_prg_fill_u64.argtypes = [vp, ctypes.c_char_p, ctypes.c_uint64, vp, ctypes.c_size_t]
    lib.pg_prg_set_keys.argtypes = [vp, ctypes.c_char_p, ctypes.c_uint64]
    lib.pg_prg_counter.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64)]
    lib.pg_tune_load.argtypes = [vp, ctypes.c_char_p]
    lib.pg_tune_save.argtypes = [vp, ctypes.c_char_p]
    lib.pg_alloc_shares.argtypes = [vp, ctypes.c_int, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(vp)]
    lib.pg_free_shares.argtypes = [vp, vp]
    lib.pg_graph_begin.argtypes = [vp]
    lib.pg_graph_end.argtypes = [vp, ctypes.POINTER(vp)]
    lib.pg_graph_launch.argtypes = [vp, vp]
    lib.pg_graph_destroy.argtypes = [vp]
    lib.pg_ctx_get_stream.argtypes = [vp]
    lib.pg_ctx_get_stream.restype = vp
    lib.pg_net_input_size.argtypes = [vp]
    lib.pg_net_input_size.restype = sz
    lib.pg_net_output_size.argtypes = [vp]
    lib.pg_net_output_size.restype = sz


def lib():
    """Load (building first when stale) the CUDA library. Raises on failure."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            _lib = ctypes.CDLL(path)
            _declare(_lib)
    return _lib


def library_path() -> str:
    return _build.LIB


# ------------------------------------------------------------------ context

class Graph:
    """pg_graph: a captured sequence of calls, replayed by launch()."""

    def __init__(self, ctx: "Context"):
        self.ctx = ctx
        self._h = None

    def launch(self):
        if self._h is None:
            raise PiranhaError("graph was not captured")
        self.ctx._check(lib().pg_graph_launch(self.ctx.handle, self._h))

    def close(self):
        if self._h is not None:
            lib().pg_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Capture:
    def __init__(self, ctx: "Context"):
        self.ctx = ctx
        self.graph = Graph(ctx)

    def __enter__(self) -> Graph:
        self.ctx._check(lib().pg_graph_begin(self.ctx.handle))
        return self.graph

    def __exit__(self, et, ev, tb):
        h = ctypes.c_void_p()
        st = lib().pg_graph_end(self.ctx.handle, ctypes.byref(h))
        if et is not None:
            if h.value:
                lib().pg_graph_destroy(h)
            return False
        self.ctx._check(st)
        self.graph._h = h
        return False


class Context:
    """pg_ctx: stream, implementation form and per-party comm counters."""

    def __init__(self, device: int = 0, stream=None, form: int = FORM_LIMB_TC):
        import torch

        self.torch = torch
        self.device = device
        self._children = weakref.WeakSet()  # networks created on this context
        torch.cuda.set_device(device)
        self._h = ctypes.c_void_p()
        self._check(lib().pg_ctx_create(ctypes.byref(self._h), device))
        # default: torch's current stream, so that torch's allocator and
        # uploads are ordered with this library's kernels
        self.stream = stream if stream is not None else torch.cuda.current_stream(device)
        lib().pg_ctx_set_stream(self._h, ctypes.c_void_p(self.stream.cuda_stream))
        self.set_form(form)

    @property
    def handle(self):
        return self._h

    def _check(self, st):
        if st != PG_OK:
            msg = lib().pg_last_error(self._h).decode() if getattr(self, "_h", None) else ""
            raise PiranhaError(f"piranha_gb300 status {st}: {msg}")

    def set_form(self, form: int):
        self._check(lib().pg_ctx_set_form(self._h, form))

    @property
    def form(self):
        return lib().pg_ctx_get_form(self._h)

    def sync(self):
        self._check(lib().pg_sync(self._h))

    def set_autotune(self, on: bool):
        """Split-K of the limb-form GEMMs by timing (default on) or by the heuristic."""
        self._check(lib().pg_ctx_set_autotune(self._h, 1 if on else 0))

    def tune_load(self, path: str):
        self._check(lib().pg_tune_load(self._h, os.fsencode(path)))

    def tune_save(self, path: str):
        self._check(lib().pg_tune_save(self._h, os.fsencode(path)))

    def prg_fill(self, key: bytes, counter: int, out):
        """The reference generator's uint64 stream from `counter` into a CUDA int64 tensor."""
        if len(key) != 32:
            raise ValueError("AES-256 key of 32 bytes")
        self._check(lib().pg_prg_fill_u64(self._h, key, counter, ctypes.c_void_p(out.data_ptr()), out.numel()))
        return out

    def set_prg_keys(self, keys, counter: int = 0):
        """Live resharing masks from three 32-byte pairwise keys (None: off)."""
        if keys is None:
            self._check(lib().pg_prg_set_keys(self._h, None, 0))
            return
        blob = b"".join(keys)
        if len(keys) != 3 or len(blob) != 96:
            raise ValueError("three 32-byte keys")
        self._check(lib().pg_prg_set_keys(self._h, blob, counter))

    def prg_counter(self) -> int:
        v = ctypes.c_uint64()
        self._check(lib().pg_prg_counter(self._h, ctypes.byref(v)))
        return v.value

    def capture(self) -> _Capture:
        """``with ctx.capture() as g: ...`` records every call on this
        context's stream (which must not be the legacy default stream) into a
        CUDA graph; ``g.launch()`` replays it. Run the calls eagerly once
        first so that the context's scratch is sized."""
        return _Capture(self)

    def set_wait_limit(self, wait_ns: int = 0, withhold_stage: int = -1):
        """Bound on the limb kernels' device-side waits (0: the default 2 s) and
        the diagnostic K stage whose copies the producer withholds (-1: none)."""
        self._check(lib().pg_ctx_set_wait_limit(self._h, int(wait_ns), int(withhold_stage)))

    def tensor_rate(self, form: int, iters: int = 200000) -> dict:
        """Sustained rate of one tensor-core instruction form (RATE_TC_F16,
        RATE_TC_F8, RATE_MMA_S8, RATE_MMA_F16) on this context's device."""
        out = (ctypes.c_double * 3)()
        self._check(lib().pg_tensor_rate(self._h, form, iters, out))
        return {"tops": out[0], "cycles_per_inst": out[1], "ms": out[2]}

    def comm(self, parties=3):
        buf = (ctypes.c_uint64 * 9)()
        self._check(lib().pg_comm_get(self._h, buf))
        return {"tx": list(buf[0:parties]), "rx": list(buf[4:4 + parties]), "rounds": buf[8]}

    def reset_comm(self):
        self._check(lib().pg_comm_reset(self._h))

    def check_device_errors(self):
        """Synchronize and raise if a bounded device-side wait gave up."""
        code = ctypes.c_int(0)
        self._check(lib().pg_device_errors(self._h, ctypes.byref(code)))

    def kernel_launches(self) -> int:
        return int(lib().pg_kernel_launches(self._h))

    def close(self):
        if getattr(self, "_h", None):
            for child in list(self._children):
                child.close()
            self.stream.synchronize()
            lib().pg_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------- share tensors

def _torch():
    import torch

    return torch


_TDT = {"u64": "int64", "u32": "int32", "u8": "uint8"}


def empty_shares(n: int, ring: str = "u64", device="cuda"):
    torch = _torch()
    return torch.empty((3, 2, n), dtype=getattr(torch, _TDT[ring]), device=device)


def zeros_shares(n: int, ring: str = "u64", device="cuda"):
    torch = _torch()
    return torch.zeros((3, 2, n), dtype=getattr(torch, _TDT[ring]), device=device)


def to_device(views: np.ndarray, device="cuda"):
    """numpy (3, 2, n) uint64/uint32/uint8 -> torch device tensor (bit-identical)."""
    torch = _torch()
    v = np.ascontiguousarray(views)
    view_as = {np.dtype(np.uint64): np.int64, np.dtype(np.uint32): np.int32, np.dtype(np.uint8): np.uint8}
    return torch.from_numpy(v.view(view_as[v.dtype])).to(device)


def to_host(t, ring: str = "u64") -> np.ndarray:
    a = t.detach().cpu().numpy()
    return a.view({"u64": np.uint64, "u32": np.uint32, "u8": np.uint8}[ring])


def _p6(t):
    if t.dim() != 3 or t.shape[0] != 3 or t.shape[1] != 2 or not t.is_cuda:
        raise PiranhaError("expected a CUDA share tensor of shape (3, 2, n)")
    if not t.is_contiguous():
        raise PiranhaError("share tensor must be contiguous")
    return _P6(*[t[p, s].data_ptr() for p in range(3) for s in range(2)])


def _p3(t):
    return _P3(*[t[p].data_ptr() for p in range(3)])


def _ring(t):
    torch = _torch()
    return {torch.int64: "u64", torch.int32: "u32", torch.uint8: "u8"}[t.dtype]


# --------------------------------------------------------- RSS protocol ops
# Names and argument meanings follow src/mpc/RSS.h:105-145.

def matmul(ctx: Context, a, b, c, M, N, K, transpose_a, transpose_b, transpose_c, truncation):
    """RSS matmul (RSS.inl:482-540): c = trunc(a @ b) as shares of all parties."""
    fn = lib().pg_rss_matmul_u64 if _ring(a) == "u64" else lib().pg_rss_matmul_u32
    ctx._check(fn(ctx.handle, _p6(a), _p6(b), _p6(c), M, N, K, int(transpose_a), int(transpose_b), int(transpose_c),
                  int(truncation)))
    return c


def fc_forward(ctx: Context, x, w, bias, out, batch, din, dout, fp=FLOAT_PRECISION):
    """FCLayer::forward (FCLayer.cu:78-130): matmul + per-share bias add."""
    bp = ctypes.cast(_p6(bias), ctypes.c_void_p) if bias is not None else None
    ctx._check(lib().pg_rss_fc_forward_u64(ctx.handle, _p6(x), _p6(w), bp, _p6(out), batch, din, dout, fp))
    return out


def convolution(ctx: Context, A, B, C, op, batchSize, imageHeight, imageWidth, filterSize, Din, Dout, stride,
                padding, truncation):
    """RSS convolution (RSS.inl:706-803)."""
    ctx._check(lib().pg_rss_conv_u64(ctx.handle, _p6(A), _p6(B), _p6(C), op, batchSize, imageHeight, imageWidth,
                                     filterSize, Din, Dout, stride, padding, truncation))
    return C


def dividePublic(ctx: Context, a, denominator):
    """dividePublic (RSS.inl:423-455), scalar or per-element device vector, in place."""
    n = a.shape[2]
    torch = _torch()
    if isinstance(denominator, torch.Tensor):
        ctx._check(lib().pg_rss_divide_public_vec_u64(ctx.handle, _p6(a), n, ctypes.c_void_p(denominator.data_ptr())))
    elif _ring(a) == "u32":
        ctx._check(lib().pg_rss_divide_public_u32(ctx.handle, _p6(a), n, int(denominator) & 0xFFFFFFFF))
    else:
        ctx._check(lib().pg_rss_divide_public_u64(ctx.handle, _p6(a), n, int(denominator) & 0xFFFFFFFFFFFFFFFF))
    return a


def reconstruct(ctx: Context, a, out=None):
    """reconstruct (RSS.inl:458-479): returns (3, n) — the value each party reveals."""
    torch = _torch()
    n = a.shape[2]
    if out is None:
        out = torch.empty((3, n), dtype=a.dtype, device=a.device)
    fn = lib().pg_rss_reconstruct_u8 if _ring(a) == "u8" else lib().pg_rss_reconstruct_u64
    ctx._check(fn(ctx.handle, _p6(a), n, _p3(out)))
    return out


def reshare(ctx: Context, c, out):
    ctx._check(lib().pg_rss_reshare_u64(ctx.handle, _p3(c), c.shape[1], _p6(out)))
    return out


def device_op_(ctx: Context, op: int, a, rhs):
    """DeviceData<uint64_t>'s own operators (DeviceData.h:131-277,
    functors.cuh) in place on one CUDA int64 tensor a: rhs an int (scalar) or
    a tensor of a's size. op is one of OP_ADD, OP_SUB, OP_MUL, OP_DIV (through
    double), OP_XOR, OP_AND, OP_SHR (arithmetic), OP_SHL, or OP_SET (fill)."""
    torch = _torch()
    if isinstance(rhs, torch.Tensor):
        if rhs.numel() != a.numel():
            raise PiranhaError("device_op_: sizes differ")
        st = lib().pg_device_op_u64(ctx.handle, op, ctypes.c_void_p(a.data_ptr()), a.numel(), RHS_PUBLIC, 0,
                                    ctypes.c_void_p(rhs.data_ptr()))
    else:
        st = lib().pg_device_op_u64(ctx.handle, op, ctypes.c_void_p(a.data_ptr()), a.numel(), RHS_SCALAR,
                                    int(rhs) % (1 << 64), None)
    ctx._check(st)
    return a


def local_(ctx: Context, op: int, a, rhs):
    """RSSBase's local operators (RSS.inl:168-345), in place on a (3, 2, n)
    uint64 shares: rhs an int (public scalar), a CUDA (n,) tensor (public
    vector, DeviceData) or (3, 2, n) shares. op is one of OP_ADD, OP_SUB,
    OP_MUL, OP_XOR, OP_AND, OP_SHR (arithmetic), OP_SHL."""
    n = a.shape[2]
    torch = _torch()
    if isinstance(rhs, torch.Tensor) and rhs.dim() == 3:
        st = lib().pg_rss_local_u64(ctx.handle, op, _p6(a), n, RHS_SHARES, 0, None, _p6(rhs))
    elif isinstance(rhs, torch.Tensor):
        st = lib().pg_rss_local_u64(ctx.handle, op, _p6(a), n, RHS_PUBLIC, 0, ctypes.c_void_p(rhs.data_ptr()), None)
    else:
        st = lib().pg_rss_local_u64(ctx.handle, op, _p6(a), n, RHS_SCALAR, int(rhs) % (1 << 64), None, None)
    ctx._check(st)
    return a


def mul_(ctx: Context, a, b):
    """RSS *= RSS (RSS.inl:284-320), in place on a."""
    ctx._check(lib().pg_rss_mul_u64(ctx.handle, _p6(a), _p6(b), a.shape[2]))
    return a


def and_(ctx: Context, a, b):
    """RSS &= RSS (RSS.inl:331-345), in place on a."""
    fn = lib().pg_rss_and_u8 if _ring(a) == "u8" else lib().pg_rss_and_u64
    ctx._check(fn(ctx.handle, _p6(a), _p6(b), a.shape[2]))
    return a


def dReLU(ctx: Context, input, result):
    """dReLU (RSS.inl:807-852); result is uint8 or uint64 bit shares."""
    fn = lib().pg_rss_drelu_u64_u8 if _ring(result) == "u8" else lib().pg_rss_drelu_u64_u64
    ctx._check(fn(ctx.handle, _p6(input), input.shape[2], _p6(result)))
    return result


def ReLU(ctx: Context, input, result, dresult):
    """ReLU (RSS.inl:855-865)."""
    if _ring(input) == "u32":
        fn = lib().pg_rss_relu_u32_u8
    else:
        fn = lib().pg_rss_relu_u64_u8 if _ring(dresult) == "u8" else lib().pg_rss_relu_u64_u64
    ctx._check(fn(ctx.handle, _p6(input), input.shape[2], _p6(result), _p6(dresult)))
    return result, dresult


def selectShare(ctx: Context, x, y, b, z):
    """selectShare (RSS.inl:543-569): z = b ? y : x."""
    fn = lib().pg_rss_select_share_u64_u8 if _ring(b) == "u8" else lib().pg_rss_select_share_u64_u64
    ctx._check(fn(ctx.handle, _p6(x), _p6(y), _p6(b), _p6(z), x.shape[2]))
    return z


def maxpool(ctx: Context, input, result, dresult, k):
    """maxpool (RSS.inl:868-1017) over rows of k (4 or 16) contiguous values."""
    fn = lib().pg_rss_maxpool_u64_u8 if _ring(dresult) == "u8" else lib().pg_rss_maxpool_u64_u64
    ctx._check(fn(ctx.handle, _p6(input), input.shape[2], k, _p6(result), _p6(dresult)))
    return result, dresult


def avgpool_layer(ctx: Context, input, out, H, W, C, pool, stride, batch):
    """AveragepoolLayer::forward (AveragepoolLayer.cu:58-81)."""
    ctx._check(lib().pg_rss_avgpool_layer_u64(ctx.handle, _p6(input), _p6(out), H, W, C, pool, stride, batch))
    return out


def avgpool_backward(ctx: Context, delta, deltas, H, W, C, pool, stride, batch):
    """AveragepoolLayer::backward (AveragepoolLayer.cu:88-117)."""
    ctx._check(lib().pg_rss_avgpool_backward_u64(ctx.handle, _p6(delta), _p6(deltas), H, W, C, pool, stride, batch))
    return deltas


def maxpool_layer(ctx: Context, input, out, maxprime, H, W, C, pool, stride, batch, fp=FLOAT_PRECISION):
    """MaxpoolLayer::forward (MaxpoolLayer.cu:52-131)."""
    ctx._check(lib().pg_rss_maxpool_layer_u64_u8(ctx.handle, _p6(input), _p6(out), _p6(maxprime), H, W, C, pool,
                                                  stride, batch, fp))
    return out, maxprime


# --------------------------------------------------------------- gpu:: ops

class tpc:
    """The 2-party protocol (src/mpc/TPC.h): a TPC tensor of n elements is a
    CUDA tensor of shape (2, n), [party A, party B], whose value is the sum.
    Names and argument meanings follow TPC.h's free functions."""

    @staticmethod
    def empty(n: int, ring: str = "u64", device="cuda"):
        torch = _torch()
        return torch.empty((2, n), dtype=getattr(torch, _TDT[ring]), device=device)

    @staticmethod
    def zeros(n: int, ring: str = "u64", device="cuda"):
        torch = _torch()
        return torch.zeros((2, n), dtype=getattr(torch, _TDT[ring]), device=device)

    @staticmethod
    def _p2(t):
        if t.dim() != 2 or t.shape[0] != 2 or not t.is_cuda:
            raise PiranhaError("expected a CUDA TPC tensor of shape (2, n)")
        if not t.is_contiguous():
            raise PiranhaError("TPC tensor must be contiguous")
        return _P2(t[0].data_ptr(), t[1].data_ptr())

    @staticmethod
    def matmul(ctx: Context, a, b, c, M, N, K, transpose_a, transpose_b, transpose_c, truncation):
        """matmul (TPC.inl:575-583)."""
        fn = lib().pg_tpc_matmul_u64 if _ring(a) == "u64" else lib().pg_tpc_matmul_u32
        ctx._check(fn(ctx.handle, tpc._p2(a), tpc._p2(b), tpc._p2(c), M, N, K, int(transpose_a), int(transpose_b),
                      int(transpose_c), int(truncation)))
        return c

    @staticmethod
    def fc_forward(ctx: Context, x, w, bias, out, batch, din, dout, fp=FLOAT_PRECISION):
        """FCLayer::forward (FCLayer.cu:78-130) for TPC: matmul + per-party bias shares."""
        fn = lib().pg_tpc_fc_forward_u64 if _ring(x) == "u64" else lib().pg_tpc_fc_forward_u32
        bp = ctypes.cast(tpc._p2(bias), ctypes.c_void_p) if bias is not None else None
        ctx._check(fn(ctx.handle, tpc._p2(x), tpc._p2(w), bp, tpc._p2(out), batch, din, dout, fp))
        return out

    @staticmethod
    def convolution(ctx: Context, A, B, C, op, batchSize, imageHeight, imageWidth, filterSize, Din, Dout, stride,
                    padding, truncation):
        """convolution (TPC.inl:789-827)."""
        ctx._check(lib().pg_tpc_conv_u64(ctx.handle, tpc._p2(A), tpc._p2(B), tpc._p2(C), int(op), batchSize,
                                         imageHeight, imageWidth, filterSize, Din, Dout, stride, padding,
                                         int(truncation)))
        return C

    @staticmethod
    def dividePublic(ctx: Context, a, denominator):
        """dividePublic (TPC.inl:371-401); the denominator is a scalar or a CUDA tensor."""
        torch = _torch()
        n = a.shape[1]
        if isinstance(denominator, torch.Tensor):
            ctx._check(lib().pg_tpc_divide_public_vec_u64(ctx.handle, tpc._p2(a), n,
                                                          ctypes.c_void_p(denominator.data_ptr())))
        elif _ring(a) == "u64":
            ctx._check(lib().pg_tpc_divide_public_u64(ctx.handle, tpc._p2(a), n, int(denominator)))
        else:
            ctx._check(lib().pg_tpc_divide_public_u32(ctx.handle, tpc._p2(a), n, int(denominator)))
        return a

    @staticmethod
    def reconstruct(ctx: Context, a, out):
        """reconstruct (TPC.inl:552-572): out has shape (2, n), one row per party."""
        fn = getattr(lib(), f"pg_tpc_reconstruct_{_ring(a)}")
        ctx._check(fn(ctx.handle, tpc._p2(a), a.shape[1], tpc._p2(out)))
        return out

    @staticmethod
    def local_(ctx: Context, op: int, a, rhs):
        """TPCBase's local operators (TPC.inl:146-240) in place on (2, n) uint64
        shares; rhs as for piranha_gb300.local_ ((2, n) for shares)."""
        n = a.shape[1]
        torch = _torch()
        if isinstance(rhs, torch.Tensor) and rhs.dim() == 2:
            st = lib().pg_tpc_local_u64(ctx.handle, op, tpc._p2(a), n, RHS_SHARES, 0, None, tpc._p2(rhs))
        elif isinstance(rhs, torch.Tensor):
            st = lib().pg_tpc_local_u64(ctx.handle, op, tpc._p2(a), n, RHS_PUBLIC, 0, ctypes.c_void_p(rhs.data_ptr()),
                                        None)
        else:
            st = lib().pg_tpc_local_u64(ctx.handle, op, tpc._p2(a), n, RHS_SCALAR, int(rhs) % (1 << 64), None, None)
        ctx._check(st)
        return a

    @staticmethod
    def mul_(ctx: Context, a, b):
        """TPC *= TPC (TPC.inl:242-272), in place on a."""
        ctx._check(lib().pg_tpc_mul_u64(ctx.handle, tpc._p2(a), tpc._p2(b), a.shape[1]))
        return a

    @staticmethod
    def dReLU(ctx: Context, input, result):
        """dReLU (TPC.inl:829-868): uint8 bit shares."""
        fn = lib().pg_tpc_drelu_u64_u8 if _ring(input) == "u64" else lib().pg_tpc_drelu_u32_u8
        ctx._check(fn(ctx.handle, tpc._p2(input), input.shape[1], tpc._p2(result)))
        return result

    @staticmethod
    def ReLU(ctx: Context, input, result, dresult):
        """ReLU (TPC.inl:871-884)."""
        fn = lib().pg_tpc_relu_u64_u8 if _ring(input) == "u64" else lib().pg_tpc_relu_u32_u8
        ctx._check(fn(ctx.handle, tpc._p2(input), input.shape[1], tpc._p2(result), tpc._p2(dresult)))
        return result, dresult

    @staticmethod
    def selectShare(ctx: Context, x, y, b, z):
        """selectShare (TPC.inl:586-610): z = b ? y : x."""
        ctx._check(lib().pg_tpc_select_share_u64_u8(ctx.handle, tpc._p2(x), tpc._p2(y), tpc._p2(b), tpc._p2(z),
                                                    x.shape[1]))
        return z

    @staticmethod
    def maxpool(ctx: Context, input, result, dresult, k):
        """maxpool (TPC.inl:887-1058) over rows of k values."""
        ctx._check(lib().pg_tpc_maxpool_u64_u8(ctx.handle, tpc._p2(input), input.shape[1], int(k), tpc._p2(result),
                                               tpc._p2(dresult)))
        return result, dresult


class fpc:
    """The 4-party protocol (src/mpc/FPC.h): an FPC tensor of n elements is a
    CUDA tensor of shape (4, 3, n), [party A..D][shareA/shareB/shareC], party
    p's share k holding component x_{(p+1+k) mod 4} of x = x0 + x1 + x2 + x3.
    Names and argument meanings follow FPC.h's free functions."""

    @staticmethod
    def empty(n: int, ring: str = "u64", device="cuda"):
        torch = _torch()
        return torch.empty((4, 3, n), dtype=getattr(torch, _TDT[ring]), device=device)

    @staticmethod
    def zeros(n: int, ring: str = "u64", device="cuda"):
        torch = _torch()
        return torch.zeros((4, 3, n), dtype=getattr(torch, _TDT[ring]), device=device)

    @staticmethod
    def _p12(t):
        if t.dim() != 3 or tuple(t.shape[:2]) != (4, 3) or not t.is_cuda:
            raise PiranhaError("expected a CUDA FPC tensor of shape (4, 3, n)")
        if not t.is_contiguous():
            raise PiranhaError("FPC tensor must be contiguous")
        return _P12(*[t[p, k].data_ptr() for p in range(4) for k in range(3)])

    @staticmethod
    def _p4(t):
        if t.dim() != 2 or t.shape[0] != 4 or not t.is_cuda or not t.is_contiguous():
            raise PiranhaError("expected a contiguous CUDA tensor of shape (4, n)")
        return _P4(*[t[p].data_ptr() for p in range(4)])

    @staticmethod
    def matmul(ctx: Context, a, b, c, M, N, K, transpose_a, transpose_b, transpose_c, truncation):
        """matmul (FPC.inl:636-670)."""
        fn = lib().pg_fpc_matmul_u64 if _ring(a) == "u64" else lib().pg_fpc_matmul_u32
        ctx._check(fn(ctx.handle, fpc._p12(a), fpc._p12(b), fpc._p12(c), M, N, K, int(transpose_a),
                      int(transpose_b), int(transpose_c), int(truncation)))
        return c

    @staticmethod
    def fc_forward(ctx: Context, x, w, bias, out, batch, din, dout, fp=FLOAT_PRECISION):
        """FCLayer::forward (FCLayer.cu:78-130) for FPC: matmul + bias shares."""
        fn = lib().pg_fpc_fc_forward_u64 if _ring(x) == "u64" else lib().pg_fpc_fc_forward_u32
        bp = ctypes.cast(fpc._p12(bias), ctypes.c_void_p) if bias is not None else None
        ctx._check(fn(ctx.handle, fpc._p12(x), fpc._p12(w), bp, fpc._p12(out), batch, din, dout, fp))
        return out

    @staticmethod
    def convolution(ctx: Context, A, B, C, op, batchSize, imageHeight, imageWidth, filterSize, Din, Dout, stride,
                    padding, truncation):
        """convolution (FPC.inl:862-925)."""
        ctx._check(lib().pg_fpc_conv_u64(ctx.handle, fpc._p12(A), fpc._p12(B), fpc._p12(C), int(op), batchSize,
                                         imageHeight, imageWidth, filterSize, Din, Dout, stride, padding,
                                         int(truncation)))
        return C

    @staticmethod
    def dividePublic(ctx: Context, a, denominator):
        """dividePublic (FPC.inl:576-608); the denominator is a scalar or a CUDA tensor."""
        torch = _torch()
        n = a.shape[2]
        if isinstance(denominator, torch.Tensor):
            ctx._check(lib().pg_fpc_divide_public_vec_u64(ctx.handle, fpc._p12(a), n,
                                                          ctypes.c_void_p(denominator.data_ptr())))
        elif _ring(a) == "u64":
            ctx._check(lib().pg_fpc_divide_public_u64(ctx.handle, fpc._p12(a), n, int(denominator)))
        else:
            ctx._check(lib().pg_fpc_divide_public_u32(ctx.handle, fpc._p12(a), n, int(denominator)))
        return a

    @staticmethod
    def reconstruct(ctx: Context, a, out):
        """reconstruct (FPC.inl:611-634): out has shape (4, n), one row per party."""
        fn = getattr(lib(), f"pg_fpc_reconstruct_{_ring(a)}")
        ctx._check(fn(ctx.handle, fpc._p12(a), a.shape[2], fpc._p4(out)))
        return out

    @staticmethod
    def local_(ctx: Context, op: int, a, rhs):
        """FPCBase's local operators (FPC.inl:187-300) in place on (4, 3, n) uint64
        shares; rhs as for piranha_gb300.local_ ((4, 3, n) for shares)."""
        n = a.shape[2]
        torch = _torch()
        if isinstance(rhs, torch.Tensor) and rhs.dim() == 3:
            st = lib().pg_fpc_local_u64(ctx.handle, op, fpc._p12(a), n, RHS_SHARES, 0, None, fpc._p12(rhs))
        elif isinstance(rhs, torch.Tensor):
            st = lib().pg_fpc_local_u64(ctx.handle, op, fpc._p12(a), n, RHS_PUBLIC, 0, ctypes.c_void_p(rhs.data_ptr()),
                                        None)
        else:
            st = lib().pg_fpc_local_u64(ctx.handle, op, fpc._p12(a), n, RHS_SCALAR, int(rhs) % (1 << 64), None, None)
        ctx._check(st)
        return a

    @staticmethod
    def mul_(ctx: Context, a, b):
        """FPC *= FPC (FPC.inl:322-364), in place on a."""
        ctx._check(lib().pg_fpc_mul_u64(ctx.handle, fpc._p12(a), fpc._p12(b), a.shape[2]))
        return a

    @staticmethod
    def and_(ctx: Context, a, b):
        """FPC &= FPC on uint8 bit shares (FPC.inl:375-399), in place on a."""
        ctx._check(lib().pg_fpc_and_u8(ctx.handle, fpc._p12(a), fpc._p12(b), a.shape[2]))
        return a

    @staticmethod
    def dReLU(ctx: Context, input, result):
        """dReLU (FPC.inl:930-990): uint8 bit shares."""
        fn = lib().pg_fpc_drelu_u64_u8 if _ring(input) == "u64" else lib().pg_fpc_drelu_u32_u8
        ctx._check(fn(ctx.handle, fpc._p12(input), input.shape[2], fpc._p12(result)))
        return result

    @staticmethod
    def ReLU(ctx: Context, input, result, dresult):
        """ReLU (FPC.inl:992-1003)."""
        fn = lib().pg_fpc_relu_u64_u8 if _ring(input) == "u64" else lib().pg_fpc_relu_u32_u8
        ctx._check(fn(ctx.handle, fpc._p12(input), input.shape[2], fpc._p12(result), fpc._p12(dresult)))
        return result, dresult

    @staticmethod
    def selectShare(ctx: Context, x, y, b, z):
        """selectShare (FPC.inl:672-711): z = b ? y : x."""
        ctx._check(lib().pg_fpc_select_share_u64_u8(ctx.handle, fpc._p12(x), fpc._p12(y), fpc._p12(b),
                                                    fpc._p12(z), x.shape[2]))
        return z

    @staticmethod
    def maxpool(ctx: Context, input, result, dresult, k):
        """maxpool (FPC.inl:1005-1177) over rows of k values (k a power of two)."""
        ctx._check(lib().pg_fpc_maxpool_u64_u8(ctx.handle, fpc._p12(input), input.shape[2], int(k),
                                               fpc._p12(result), fpc._p12(dresult)))
        return result, dresult


class gpu:
    """Single-array kernels of src/gpu (gemm.cuh, conv.cuh, matrix.cuh, bitwise.cuh, convolution.cuh)."""

    @staticmethod
    def gemm(ctx: Context, M, N, K, A, transpose_a, B, transpose_b, C, transpose_c):
        fn = lib().pg_gemm_u64 if A.dtype == _torch().int64 else lib().pg_gemm_u32
        ctx._check(fn(ctx.handle, M, N, K, ctypes.c_void_p(A.data_ptr()), int(transpose_a),
                      ctypes.c_void_p(B.data_ptr()), int(transpose_b), ctypes.c_void_p(C.data_ptr()),
                      int(transpose_c)))
        return C

    @staticmethod
    def conv(ctx: Context, op, N, H, W, C, K, R, S, pad, stride, a, b, out):
        ctx._check(lib().pg_conv_u64(ctx.handle, op, N, H, W, C, K, R, S, pad, stride, ctypes.c_void_p(a.data_ptr()),
                                     ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(out.data_ptr())))
        return out

    @staticmethod
    def elementVectorAdd(ctx: Context, a, b, rowwise, rows, cols):
        ctx._check(lib().pg_element_vector_add_u64(ctx.handle, ctypes.c_void_p(a.data_ptr()),
                                                   ctypes.c_void_p(b.data_ptr()), int(rowwise), rows, cols))
        return a

    @staticmethod
    def reduceSum(ctx: Context, a, b, reduceRows, rows, cols):
        ctx._check(lib().pg_reduce_sum_u64(ctx.handle, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                                           int(reduceRows), rows, cols))
        return b

    @staticmethod
    def truncate_cols(ctx: Context, a, b, rows, start_cols, end_cols):
        ctx._check(lib().pg_truncate_cols_u8(ctx.handle, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                                             rows, start_cols, end_cols))
        return b

    @staticmethod
    def bitexpand(ctx: Context, a, bits):
        ctx._check(lib().pg_bitexpand_u64(ctx.handle, ctypes.c_void_p(a.data_ptr()), a.numel(),
                                          ctypes.c_void_p(bits.data_ptr())))
        return bits

    @staticmethod
    def expandCompare(ctx: Context, b, nb, out):
        ctx._check(lib().pg_expand_compare_u8(ctx.handle, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(nb.data_ptr()),
                                              b.numel(), ctypes.c_void_p(out.data_ptr()), out.numel()))
        return out

    @staticmethod
    def maxpool_im2row(ctx: Context, im, out, imageHeight, imageWidth, filterSize, Din, batchSize, stride, padding,
                       pad_val):
        ctx._check(lib().pg_maxpool_im2row_u64(ctx.handle, ctypes.c_void_p(im.data_ptr()),
                                               ctypes.c_void_p(out.data_ptr()), imageHeight, imageWidth, filterSize,
                                               Din, batchSize, stride, padding, int(pad_val) % (1 << 64)))
        return out


# ------------------------------------------------------------------ network

class Network:
    """Secure-inference and training executor (NeuralNetwork::forward and
    ::backward, NeuralNetwork.cu:109-148).

    ``layers`` is a list of tuples: ("fc", din, dout), ("cnn", H, W, Din, Dout, f, stride, pad),
    ("relu", n_per_image), ("maxpool", H, W, C, pool, stride), ("avgpool", H, W, C, pool, stride).
    """

    _CODES = {"fc": LAYER_FC, "cnn": LAYER_CNN, "relu": LAYER_RELU, "maxpool": LAYER_MAXPOOL,
              "avgpool": LAYER_AVGPOOL}

    def __init__(self, ctx: Context, layers, batch: int, fp: int = FLOAT_PRECISION):
        self.ctx = ctx
        self.layers = list(layers)
        self.batch = batch
        spec = np.zeros((len(self.layers), 8), dtype=np.int32)
        for i, L in enumerate(self.layers):
            spec[i, 0] = self._CODES[L[0]]
            spec[i, 1:1 + len(L) - 1] = L[1:]
        self._spec = spec
        self._h = ctypes.c_void_p()
        ctx._check(lib().pg_net_create(ctx.handle, ctypes.byref(self._h), spec.ctypes.data_as(ctypes.c_void_p),
                                       len(self.layers), batch, fp))
        ctx._children.add(self)
        self.in_n = int(lib().pg_net_input_size(self._h))
        self.out_n = int(lib().pg_net_output_size(self._h))

    def set_params(self, layer: int, w, bias=None):
        bp = ctypes.cast(_p6(bias), ctypes.c_void_p) if bias is not None else None
        self.ctx._check(lib().pg_net_set_params(self._h, layer, _p6(w), bp))

    def forward(self, x, out):
        self.ctx._check(lib().pg_net_forward(self._h, _p6(x), _p6(out)))
        return out

    def capture(self):
        self.ctx._check(lib().pg_net_capture(self._h))

    def forward_resident(self):
        self.ctx._check(lib().pg_net_forward_resident(self._h))

    def input_buffers(self):
        arr = _P6()
        self.ctx._check(lib().pg_net_input_shares(self._h, arr))
        return [int(x) for x in arr]

    def forward_host(self, in_host_ptr: int, out_host_ptr: int):
        self.ctx._check(lib().pg_net_forward_host(self._h, ctypes.c_void_p(in_host_ptr), ctypes.c_void_p(out_host_ptr)))

    def enable_timing(self, on: bool = True):
        self.ctx._check(lib().pg_net_enable_timing(self._h, int(on)))

    def layer_times_ms(self):
        buf = (ctypes.c_float * len(self.layers))()
        self.ctx._check(lib().pg_net_layer_times(self._h, buf))
        return list(buf)

    def layer_output_ptrs(self, layer: int):
        arr = _P6()
        n = ctypes.c_size_t()
        self.ctx._check(lib().pg_net_layer_output(self._h, layer, arr, ctypes.byref(n)))
        return [int(x) for x in arr], int(n.value)

    def layer_plan(self, layer: int) -> dict:
        """How FC / CNN layer `layer` runs (after the first forward): form
        (1 limb, 2 u64, 0 other layers), position-major tiles, split-K, tiles."""
        arr = (ctypes.c_int * 4)()
        self.ctx._check(lib().pg_net_layer_plan(self._h, layer, arr))
        return {"form": arr[0], "posmajor": arr[1], "split": arr[2], "tiles": arr[3]}

    # ---------------------------------------------------------- training
    # One SGD iteration = forward + NeuralNetwork::backward (NeuralNetwork.cu:136-148).

    def train_step(self, x, labels, log_lr: int = 5):
        """Forward on x, then the backward pass and parameter updates with
        learning rate 2^-log_lr; labels are (3, 2, out_n) RSS shares."""
        self.ctx._check(lib().pg_net_train_step(self._h, _p6(x), _p6(labels), int(log_lr)))

    def backward(self, x, labels, log_lr: int = 5):
        """The backward pass after a forward on x."""
        self.ctx._check(lib().pg_net_backward(self._h, _p6(x), _p6(labels), int(log_lr)))

    def label_buffers(self):
        arr = _P6()
        self.ctx._check(lib().pg_net_label_shares(self._h, arr))
        return [int(x) for x in arr]

    def capture_train(self, log_lr: int = 5):
        self.ctx._check(lib().pg_net_capture_train(self._h, int(log_lr)))

    def train_resident(self):
        self.ctx._check(lib().pg_net_train_resident(self._h))

    def train_host(self, in_host_ptr: int, labels_host_ptr: int, out_host_ptr: int, log_lr: int = 5):
        self.ctx._check(lib().pg_net_train_host(self._h, ctypes.c_void_p(in_host_ptr), ctypes.c_void_p(labels_host_ptr),
                                                ctypes.c_void_p(out_host_ptr), int(log_lr)))

    def layer_delta_ptrs(self, layer: int):
        """Layer i's backward output (layer -1: the softmax gradient)."""
        arr = _P6()
        n = ctypes.c_size_t()
        self.ctx._check(lib().pg_net_layer_delta(self._h, layer, arr, ctypes.byref(n)))
        return [int(x) for x in arr], int(n.value)

    def layer_param_ptrs(self, layer: int):
        w, b = _P6(), _P6()
        wn, bn = ctypes.c_size_t(), ctypes.c_size_t()
        self.ctx._check(lib().pg_net_layer_params(self._h, layer, w, b, ctypes.byref(wn), ctypes.byref(bn)))
        return [int(x or 0) for x in w], int(wn.value), [int(x or 0) for x in b], int(bn.value)

    def close(self):
        # a network must be destroyed before its context (Context.close does this first)
        if getattr(self, "_h", None) and getattr(self.ctx, "_h", None):
            self.ctx.stream.synchronize()
            lib().pg_net_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
