"""Generate tests/golden/fullsize.json: SHA-256 digests of the oracle's
results on the benchmark configurations at their full sizes.

    python tests/golden/make_fullsize.py            # about 5 minutes on 8 cores

* ``vgg16_b128``: 3PC VGG16 (files/models/vgg16-cifar10.json with each 2x2/2
  averagepool replaced by a maxpool) secure inference on 128 synthetic 32x32x3
  images, every layer's six output shares, and the message counters;
* ``lenet_train_b128``: one 3PC LeNet (files/models/lenet.json) training step
  at batch 128, log learning rate 5: every layer's output, the revealed
  softmax gradient, every gradient passed between layers, every updated
  weight and bias share, and the counters.

The inputs come from ``seeded.py`` (SplitMix64 streams), so the GPU tests
rebuild them bit for bit on any machine; their digests are stored too, so a
mismatch of the inputs is reported as such. The oracle is the CPU restatement
of the reference's arithmetic (``oracle/``).
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import oracle as orc  # noqa: E402
from oracle import netref  # noqa: E402
from tests.golden import seeded  # noqa: E402

VGG_SEEDS = {"images": 1, "weights": 1000}
LENET_SEEDS = {"images": 11, "labels": 14, "weights": 1100}
LENET_LOG_LR = 5


def comm_dict(c: orc.Comm) -> dict:
    return {"tx": c.tx, "rx": c.rx, "rounds": c.rounds}


def vgg16_case(batch: int = 128) -> dict:
    layers = netref.vgg16_layers(maxpool=True)
    params = seeded.kaiming_uniform(layers, VGG_SEEDS["weights"])
    x = seeded.images(VGG_SEEDS["images"], batch * 3072)
    comm = orc.Comm()
    t = time.time()
    _, outs = netref.forward(layers, params, x, batch, comm=comm, keep=True)
    print(f"vgg16 b{batch}: {time.time() - t:.1f} s", file=sys.stderr)
    return {
        "batch": batch,
        "seeds": VGG_SEEDS,
        "input": seeded.digest(x),
        "params": [None if p is None else seeded.digest(p[0]) for p in params],
        "layers": [seeded.digest(o) for o in outs],
        "comm": comm_dict(comm),
    }


def lenet_train_case(batch: int = 128) -> dict:
    layers = netref.lenet_layers()
    params = seeded.kaiming_uniform(layers, LENET_SEEDS["weights"])
    x = seeded.images(LENET_SEEDS["images"], batch * 784)
    labels = seeded.labels(LENET_SEEDS["labels"], batch)
    comm = orc.Comm()
    t = time.time()
    bits = []
    _, outs = netref.forward(layers, params, x, batch, keep=True, bits=bits, comm=comm)
    softmax = orc.reveal_softmax_grad(outs[-1], labels, batch)
    new_params, deltas = netref.backward(layers, params, x, outs, bits, labels, batch, log_lr=LENET_LOG_LR,
                                         comm=comm)
    print(f"lenet train b{batch}: {time.time() - t:.1f} s", file=sys.stderr)
    return {
        "batch": batch,
        "seeds": LENET_SEEDS,
        "log_lr": LENET_LOG_LR,
        "input": seeded.digest(x),
        "labels": seeded.digest(labels),
        "outputs": [seeded.digest(o) for o in outs],
        "softmax": seeded.digest(softmax),
        "deltas": [seeded.digest(d) for d in deltas],
        "params": [None if p is None else [seeded.digest(p[0]), None if p[1] is None else seeded.digest(p[1])]
                   for p in new_params],
        "comm": comm_dict(comm),
    }


def main() -> None:
    out = {
        "generator": "tests/golden/make_fullsize.py (oracle/, inputs from tests/golden/seeded.py)",
        "lenet_train_b128": lenet_train_case(),
        "vgg16_b128": vgg16_case(),
    }
    path = os.path.join(HERE, "fullsize.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print("wrote", path, file=sys.stderr)


if __name__ == "__main__":
    main()
