"""DeviceData<uint64_t>'s own elementwise operators (pg_device_op_u64) on one
device array, against numpy's ring arithmetic and the oracle's restatement of
the reference's division through double (functors.cuh:33-45,94-105)."""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

U64 = np.uint64


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    ctx = pg.Context(0)
    yield pg, torch, ctx
    ctx.close()


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()


def _host(t):
    return t.cpu().numpy().view(U64)


def _ref(op, a, r):
    with np.errstate(over="ignore"):
        if op == "add":
            return a + r
        if op == "sub":
            return a - r
        if op == "mul":
            return a * r
        if op == "xor":
            return a ^ r
        if op == "and":
            return a & r
        if op == "shr":
            s = np.minimum(r, U64(63)).astype(np.int64)
            return (a.view(np.int64) >> s).view(U64)
        if op == "shl":
            return np.where(r >= 64, U64(0), a << np.minimum(r, U64(63)))
    raise ValueError(op)


@pytest.mark.parametrize("op", ["add", "sub", "mul", "xor", "and", "shr", "shl"])
@pytest.mark.parametrize("vector", [False, True])
def test_device_data_operators(env, op, vector):
    pg, torch, ctx = env
    code = {"add": pg.OP_ADD, "sub": pg.OP_SUB, "mul": pg.OP_MUL, "xor": pg.OP_XOR, "and": pg.OP_AND,
            "shr": pg.OP_SHR, "shl": pg.OP_SHL}[op]
    rng = np.random.default_rng(3)
    n = 1000
    a = rng.integers(0, 2**64 - 1, n, dtype=U64, endpoint=True)
    if op in ("shr", "shl"):
        r = rng.integers(0, 70, n).astype(U64) if vector else U64(13)
    else:
        r = rng.integers(0, 2**64 - 1, n, dtype=U64, endpoint=True) if vector else U64(0x9E3779B97F4A7C15)
    t = _dev(torch, a)
    pg.device_op_(ctx, code, t, _dev(torch, r) if vector else int(r))
    ctx.sync()
    assert np.array_equal(_host(t), _ref(op, a, r))


@pytest.mark.parametrize("vector", [False, True])
def test_device_data_division_through_double(env, vector):
    pg, torch, ctx = env
    rng = np.random.default_rng(4)
    n = 2000
    a = rng.integers(0, 2**64 - 1, n, dtype=U64, endpoint=True)
    a[:4] = [0, 1, U64(2**63), U64(2**63 - 1)]
    if vector:
        d = (U64(1) << rng.integers(0, 40, n).astype(U64))
        d[::3] = rng.integers(1, 10**6, d[::3].size).astype(U64)  # general denominators too
    else:
        d = U64(1 << 26)
    t = _dev(torch, a)
    pg.device_op_(ctx, pg.OP_DIV, t, _dev(torch, d) if vector else int(d))
    ctx.sync()
    assert np.array_equal(_host(t), orc.div_public_values(a, d))


def test_device_data_fill_and_refusals(env):
    pg, torch, ctx = env
    t = torch.zeros(777, dtype=torch.int64, device="cuda")
    pg.device_op_(ctx, pg.OP_SET, t, 2**64 - 5)
    ctx.sync()
    assert np.all(_host(t) == U64(2**64 - 5))
    with pytest.raises(pg.PiranhaError):
        pg.device_op_(ctx, pg.OP_SET, t, t)  # fill takes a scalar
    with pytest.raises(pg.PiranhaError):
        pg.device_op_(ctx, 42, t, 1)
