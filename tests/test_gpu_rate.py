"""The tensor-core rate probe (pg_tensor_rate): every instruction form runs to
completion with a positive rate, and the exact fp16 tcgen05 form the limb
GEMM uses outruns the only INT8 tensor form sm_103a offers (mma.sync s8)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    c = pg.Context(0)
    yield c
    c.close()


def test_tensor_rates(ctx):
    import piranha_gb300 as pg

    rates = {}
    for name, form in (("tc_f16", pg.RATE_TC_F16), ("tc_f8", pg.RATE_TC_F8), ("mma_s8", pg.RATE_MMA_S8),
                       ("mma_f16", pg.RATE_MMA_F16)):
        r = ctx.tensor_rate(form, 20000)
        assert r["tops"] > 0 and r["cycles_per_inst"] > 0 and r["ms"] > 0, (name, r)
        rates[name] = r["tops"]
    ctx.check_device_errors()
    print("tensor rates (TOP/s):", rates)
    assert rates["tc_f16"] > rates["mma_s8"]


def test_tensor_rate_rejects_bad_arguments(ctx):
    import piranha_gb300 as pg

    for form, iters in ((7, 10), (pg.RATE_TC_F16, 0), (pg.RATE_MMA_S8, -1)):
        with pytest.raises(pg.PiranhaError):
            ctx.tensor_rate(form, iters)
