"""Failure detection on the GPU without a fault: a bounded device-side wait
that runs out. The limb GEMM's producer withholds the copies of one K stage
(a diagnostic of the context), so the MMA warps' wait for that stage's data
runs out after the context's short wait limit; the kernel then records a
timeout in the device error word, stops issuing, waits (bounded) for its own
copies and MMAs, frees its tensor memory and returns. pg_device_errors must
report PG_ERR_TIMEOUT, and the same context must then compute a normal
share-GEMM bit for bit. Nothing here traps, faults or hangs the GPU: every
wait has a limit of about a millisecond."""
import ctypes
import time

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

U64 = np.uint64
PG_ERR_TIMEOUT = 5


@pytest.fixture(scope="module")
def pg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    pg.lib()
    return pg


def _errors(pg, ctx):
    code = ctypes.c_int(0)
    st = pg.lib().pg_device_errors(ctx.handle, ctypes.byref(code))
    return st, code.value


@pytest.mark.parametrize("M,N,K,withhold", [(128, 64, 64, 0), (256, 128, 512, 5), (64, 128, 2048, 3)])
def test_withheld_stage_times_out_and_context_recovers(pg, M, N, K, withhold):
    a = orc.random_views(M * K, U64, 1)
    b = orc.random_views(K * N, U64, 2)
    want = orc.matmul(a, b, M, N, K, 1, 1, 1, 26)
    ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
    ctx.set_autotune(False)  # the limb kernel, with the heuristic split-K
    da, db = pg.to_device(a), pg.to_device(b)
    out = pg.empty_shares(M * N)
    ctx.set_wait_limit(1_000_000, withhold)  # 1 ms
    t0 = time.perf_counter()
    pg.matmul(ctx, da, db, out, M, N, K, 1, 1, 1, 26)
    ctx.sync()
    elapsed = time.perf_counter() - t0
    st, code = _errors(pg, ctx)
    assert st == PG_ERR_TIMEOUT and code != 0, (st, hex(code))
    assert elapsed < 1.0
    # the error word was cleared by the read; the context works again
    ctx.set_wait_limit(0, -1)
    out2 = pg.empty_shares(M * N)
    pg.matmul(ctx, da, db, out2, M, N, K, 1, 1, 1, 26)
    ctx.sync()
    assert _errors(pg, ctx) == (0, 0)
    assert np.array_equal(pg.to_host(out2), want)
    ctx.close()


def test_wait_limit_rejects_bad_stage(pg):
    ctx = pg.Context(0)
    with pytest.raises(pg.PiranhaError):
        ctx.set_wait_limit(1000, -2)
    ctx.close()
