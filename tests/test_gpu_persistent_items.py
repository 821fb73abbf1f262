"""The limb kernel's persistent grid with many work items per CTA.

One CTA per SM walks a list of items (output tiles and their K' slices);
the items of a CTA run back to back, with the stage ring, the chunk counts
and the issue lag carried across them, and every item but the CTA's last
stores its output straight from the epilogue registers. The parity tests
mostly run problems of fewer items than the GPU has SMs, one item per CTA;
here they run again in a child process whose grid is capped at a few CTAs
(PG_CTAS), so that every CTA walks many items, in every form of the kernel:
GEMM layouts (row- and column-major outputs, bias, split-K), convolutions
(rectangle and position-major tiles, channel padding), input gradients
(flipped filter, column GEMM), weight gradients (implicit, explicit), the
network forward and the training step, all against the oracle."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("ctas", [3, 7])
def test_limb_forms_with_many_items_per_cta(ctas):
    pytest.importorskip("torch")
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    env = dict(os.environ, PG_CTAS=str(ctas))
    cmd = [sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider", "-m", "gpu",
           os.path.join(HERE, "test_gpu_limb.py"), os.path.join(HERE, "test_gpu_wgrad.py"),
           os.path.join(HERE, "test_gpu_posmajor.py"),
           os.path.join(HERE, "test_gpu_network.py") + "::test_lenet_forward_limb_form",
           os.path.join(HERE, "test_gpu_network.py") + "::test_fc_fed_by_a_biased_fc",
           "-k", "not vgg16_forward"]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=1500)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    # the training step: weight gradients, input gradients, FC GEMMs with column-major outputs
    cmd = [sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider", "-m", "gpu",
           os.path.join(HERE, "test_gpu_train.py"), "-k", "tc and not captured"]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=1500)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
