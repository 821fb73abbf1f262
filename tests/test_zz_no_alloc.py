"""pg_rss_matmul_u64_noalloc (the limb-form share-GEMM whose scratch is one
fixed device array) against pg_rss_matmul_u64, bit for bit, through the C ABI.

The file name sorts last, so in a full run these calls come after every other
test has used the library in the same process; it passes on its own as well.
One test runs the calls in a child process whose CUDA allocation functions
are wrapped by a small counting library (LD_PRELOAD), so that an allocation
freed again inside a call is seen too.
"""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

U64 = np.uint64
P6 = ctypes.c_void_p * 6
PG_ERR_SIZE = 2


@pytest.fixture(scope="module")
def pg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    fn = pg.lib().pg_rss_matmul_u64_noalloc
    fn.argtypes = [ctypes.c_void_p, P6, P6, P6] + [ctypes.c_int] * 7
    fn.restype = ctypes.c_int
    return pg


@pytest.fixture()
def ctx(pg):
    c = pg.Context(0, form=pg.FORM_LIMB_TC)
    yield c
    c.check_device_errors()
    c.close()


def _p6(t):
    return P6(*[t[p, s].data_ptr() for p in range(3) for s in range(2)])


def _noalloc(pg, ctx, a, b, c, M, N, K, tA, tB, tC, trunc):
    return pg.lib().pg_rss_matmul_u64_noalloc(ctx.handle, _p6(a), _p6(b), _p6(c), M, N, K, tA, tB, tC, trunc)


CASES = [
    (256, 192, 512, 1, 1, 1, 26),   # several tiles, one K' slice per tile
    (64, 128, 1024, 1, 0, 1, 20),   # few tiles: split-K with partial sums
]


def test_noalloc_matches_regular_two_calls(pg, ctx):
    import torch

    ins, want = [], []
    for i, (M, N, K, tA, tB, tC, t) in enumerate(CASES):
        a = orc.random_views(M * K, U64, 100 + i)
        b = orc.random_views(K * N, U64, 200 + i)
        da, db = pg.to_device(a), pg.to_device(b)
        ref = pg.empty_shares(M * N)
        pg.matmul(ctx, da, db, ref, M, N, K, tA, tB, tC, t)
        ins.append((da, db))
        want.append(pg.to_host(ref))
        if i == 0:
            assert np.array_equal(want[0], orc.matmul(a, b, M, N, K, tA, tB, tC, t))
    outs = [pg.empty_shares(M * N) for (M, N, *_) in CASES]
    # set-up call (the first on this device in a fresh process): loads the
    # module that holds the fixed scratch
    (M, N, K, tA, tB, tC, t), (da, db) = CASES[0], ins[0]
    ctx._check(_noalloc(pg, ctx, da, db, outs[0], M, N, K, tA, tB, tC, t))
    ctx.sync()
    comm0 = ctx.comm()
    free0 = torch.cuda.mem_get_info()[0]
    # two calls in a row on one stream: the second reuses the scratch the first just used
    for (M, N, K, tA, tB, tC, t), (da, db), out in zip(CASES, ins, outs):
        ctx._check(_noalloc(pg, ctx, da, db, out, M, N, K, tA, tB, tC, t))
    ctx.check_device_errors()
    for got, w in zip(outs, want):
        assert np.array_equal(pg.to_host(got), w)
    comm1 = ctx.comm()
    per = [2 * M * N * 8 for (M, N, *_) in CASES]
    assert [x - y for x, y in zip(comm1["tx"], comm0["tx"])] == [sum(per)] * 3
    assert comm1["rounds"] - comm0["rounds"] == 2
    # after the set-up of the first call, a call reserves no device memory
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_repeat_is_stable(pg, ctx):
    M, N, K, tA, tB, tC, t = CASES[1]
    a, b = orc.random_views(M * K, U64, 7), orc.random_views(K * N, U64, 8)
    want = orc.matmul(a, b, M, N, K, tA, tB, tC, t)
    da, db = pg.to_device(a), pg.to_device(b)
    for _ in range(2):
        out = pg.zeros_shares(M * N)
        ctx._check(_noalloc(pg, ctx, da, db, out, M, N, K, tA, tB, tC, t))
        ctx.check_device_errors()
        assert np.array_equal(pg.to_host(out), want)


def test_noalloc_refuses_what_does_not_fit(pg, ctx):
    # sizes are checked before any device memory is touched, so small buffers do
    d = pg.zeros_shares(16)
    st = _noalloc(pg, ctx, d, d, d, 4096, 4096, 4096, 1, 1, 1, 26)
    assert st == PG_ERR_SIZE
    msg = pg.lib().pg_last_error(ctx.handle)
    msg = msg.decode() if isinstance(msg, bytes) else str(msg)
    assert "fixed scratch" in msg


def test_noalloc_any_k(pg, ctx):
    # K not a multiple of 16: zero digits pad the contraction
    M, N, K = 40, 24, 25
    a, b = orc.random_views(M * K, U64, 11), orc.random_views(K * N, U64, 12)
    out = pg.zeros_shares(M * N)
    ctx._check(_noalloc(pg, ctx, pg.to_device(a), pg.to_device(b), out, M, N, K, 1, 1, 1, 20))
    ctx.check_device_errors()
    assert np.array_equal(pg.to_host(out), orc.matmul(a, b, M, N, K, 1, 1, 1, 20))


_COUNTER_C = r"""
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stddef.h>
static long n_calls;
long pg_test_alloc_calls(void) { return __atomic_load_n(&n_calls, __ATOMIC_SEQ_CST); }
void pg_test_alloc_reset(void) { __atomic_store_n(&n_calls, 0, __ATOMIC_SEQ_CST); }
#define COUNT() __atomic_add_fetch(&n_calls, 1, __ATOMIC_SEQ_CST)
#define REAL(name, type) static type real; if (!real) real = (type)dlsym(RTLD_NEXT, name)
typedef int (*f_pp_sz)(void **, size_t);
typedef int (*f_p)(void *);
typedef int (*f_pp_sz_s)(void **, size_t, void *);
typedef int (*f_p_s)(void *, void *);
typedef int (*f_pp_sz_u)(void **, size_t, unsigned);
typedef int (*f_pitch)(void **, size_t *, size_t, size_t);
int cudaMalloc(void **p, size_t n) { REAL("cudaMalloc", f_pp_sz); COUNT(); return real(p, n); }
int cudaFree(void *p) { REAL("cudaFree", f_p); COUNT(); return real(p); }
int cudaMallocAsync(void **p, size_t n, void *s) { REAL("cudaMallocAsync", f_pp_sz_s); COUNT(); return real(p, n, s); }
int cudaFreeAsync(void *p, void *s) { REAL("cudaFreeAsync", f_p_s); COUNT(); return real(p, s); }
int cudaMallocHost(void **p, size_t n) { REAL("cudaMallocHost", f_pp_sz); COUNT(); return real(p, n); }
int cudaFreeHost(void *p) { REAL("cudaFreeHost", f_p); COUNT(); return real(p); }
int cudaHostAlloc(void **p, size_t n, unsigned f) { REAL("cudaHostAlloc", f_pp_sz_u); COUNT(); return real(p, n, f); }
int cudaMallocManaged(void **p, size_t n, unsigned f) { REAL("cudaMallocManaged", f_pp_sz_u); COUNT(); return real(p, n, f); }
int cudaMallocPitch(void **p, size_t *pitch, size_t w, size_t h) { REAL("cudaMallocPitch", f_pitch); COUNT(); return real(p, pitch, w, h); }
"""

_CHILD = r"""
import ctypes, json, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[2])
import piranha_gb300 as pg
counter = ctypes.CDLL(sys.argv[1])
P6 = ctypes.c_void_p * 6
fn = pg.lib().pg_rss_matmul_u64_noalloc
fn.argtypes = [ctypes.c_void_p, P6, P6, P6] + [ctypes.c_int] * 7
p6 = lambda t: P6(*[t[p, s].data_ptr() for p in range(3) for s in range(2)])
cases = [(256, 192, 512, 1, 1, 1, 26), (64, 128, 1024, 1, 0, 1, 20)]
g = torch.Generator(device="cuda")
g.manual_seed(5)
ins = [(torch.randint(-2**63, 2**63 - 1, (3, 2, M * K), dtype=torch.int64, device="cuda", generator=g),
        torch.randint(-2**63, 2**63 - 1, (3, 2, K * N), dtype=torch.int64, device="cuda", generator=g))
       for (M, N, K, *_) in cases]
outs = [pg.empty_shares(M * N) for (M, N, *_) in cases]
ctx = pg.Context(0, form=pg.FORM_LIMB_TC)
want = []
for (M, N, K, tA, tB, tC, t), (a, b) in zip(cases, ins):
    w = pg.empty_shares(M * N)
    pg.matmul(ctx, a, b, w, M, N, K, tA, tB, tC, t)
    want.append(w)
(M, N, K, tA, tB, tC, t), (a, b) = cases[0], ins[0]
ctx._check(fn(ctx.handle, p6(a), p6(b), p6(outs[0]), M, N, K, tA, tB, tC, t))  # set-up call
ctx.sync()
ctx2 = pg.Context(0, form=pg.FORM_LIMB_TC)
ctx2.set_autotune(False)
w2 = pg.empty_shares(96 * 80)
a2 = ins[0][0][..., : 96 * 512].contiguous()
b2 = ins[0][1][..., : 512 * 80].contiguous()
torch.cuda.synchronize()
counter.pg_test_alloc_reset()
for (M, N, K, tA, tB, tC, t), (a, b), o in zip(cases, ins, outs):
    ctx._check(fn(ctx.handle, p6(a), p6(b), p6(o), M, N, K, tA, tB, tC, t))
ctx.sync()
noalloc_calls = counter.pg_test_alloc_calls()
counter.pg_test_alloc_reset()
# the detector itself: a regular call on a fresh context grows its scratch
pg.matmul(ctx2, a2, b2, w2, 96, 80, 512, 1, 1, 1, 26)
ctx2.sync()
regular_calls = counter.pg_test_alloc_calls()
ctx.check_device_errors()
equal = all(torch.equal(o, w) for o, w in zip(outs, want))
print(json.dumps({"noalloc": noalloc_calls, "regular": regular_calls, "equal": equal}))
"""


def test_noalloc_calls_no_allocation_function(pg, tmp_path):
    """Two calls in a row (after the set-up call) reach no CUDA allocation or
    free function at all, while a regular call on a fresh context does."""
    import shutil

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler for the allocation counter")
    src = tmp_path / "count_alloc.c"
    src.write_text(_COUNTER_C)
    so = tmp_path / "libcount_alloc.so"
    subprocess.run([cc, "-shared", "-fPIC", "-O1", "-o", str(so), str(src), "-ldl"], check=True)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, LD_PRELOAD=str(so))
    r = subprocess.run([sys.executable, "-c", _CHILD, str(so), root], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["equal"], res
    assert res["regular"] > 0, res  # the counter sees the regular path's scratch growth
    assert res["noalloc"] == 0, res
