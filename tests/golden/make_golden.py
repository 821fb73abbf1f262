"""Regenerate the golden fixtures in this directory from the Piranha sources.

Run with the Piranha source tree as the first argument (or in the
environment variable PIRANHA_SRC):

    python tests/golden/make_golden.py /path/to/piranha

It reads Piranha's own known-answer tests as text (src/test/GPU.cu,
src/test/Func.cu, src/test/Layer.cu) and its layer fixtures (files/test/*),
and writes:

* kat.json     — the literal arrays of the GPU.cu / Func.cu / Layer.cu cases,
                 extracted from the test bodies, keyed by test name; the call
                 parameters of each case are recorded next to them with the
                 line they come from;
* layers.npz   — the fixture-driven layer tests (FC MNIST, SecureML forward
                 chain, ReLU MNIST, maxpool MNIST, CNN MNIST, the FC /
                 maxpool / CNN MNIST backward cases, and the SecureML
                 training step) as float64 arrays.

Nothing under tests/ reads the reference tree at test time; only this
generator does.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PIRANHA_SRC", "")

_SAFE = re.compile(r"^[0-9a-fA-FxX\s\.\+\-\*/<>\(\)e]+$")


def _eval_item(tok: str, env: dict) -> float:
    tok = tok.strip()
    for k, v in env.items():
        tok = re.sub(rf"\b{k}\b", f"({v})", tok)
    if not _SAFE.match(tok):
        raise ValueError(f"unsupported literal {tok!r}")
    return float(eval(tok, {"__builtins__": {}}, {}))


def _body(src: str, macro_name: str) -> tuple[str, int]:
    m = re.search(r"(TYPED_TEST|TEST)\(\w+,\s*" + re.escape(macro_name) + r"\)\s*\{", src)
    if not m:
        raise KeyError(macro_name)
    i = m.end()
    depth = 1
    while depth:
        depth += {"{": 1, "}": -1}.get(src[i], 0)
        i += 1
    line = src.count("\n", 0, m.start()) + 1
    return src[m.end():i - 1], line


def _arrays(body: str, env: dict | None = None) -> dict:
    env = env or {}
    out = {}
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)  # block comments
    body = re.sub(r"//[^\n]*", "", body)  # line comments (commented-out variants)
    pat = re.compile(r"(?:DeviceData<[^>]+>|Share|LAYER_TEST_SHARE<T>|std::vector<double>|RSS<uint8_t>)\s*"
                     r"(\w+)\s*(?:=\s*)?(?:\(\s*)?\{([^}]*)\}", re.S)
    for m in pat.finditer(body):
        name, items = m.group(1), m.group(2)
        items = re.sub(r"//[^\n]*", "", items)
        vals = [_eval_item(t, env) for t in items.split(",") if t.strip()]
        out.setdefault(name, vals)
        # re-assignment `expected = {...}` later in the body
    for m in re.finditer(r"\n\s*(\w+)\s*=\s*\{([^}]*)\};", body):
        name, items = m.group(1), m.group(2)
        vals = [_eval_item(t, env) for t in items.split(",") if t.strip()]
        out[name + "@2"] = vals
    return out


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "src", "test")):
        sys.exit("usage: make_golden.py /path/to/piranha (or set PIRANHA_SRC)")
    gpu = open(os.path.join(REF, "src/test/GPU.cu")).read()
    func = open(os.path.join(REF, "src/test/Func.cu")).read()
    layer = open(os.path.join(REF, "src/test/Layer.cu")).read()
    fp = 26
    neg = -10 * (1 << fp)
    kat = {"_source": "Piranha src/test/{GPU,Func,Layer}.cu, extracted by make_golden.py", "cases": {}}

    def add(src, fname, test, params, env=None):
        body, line = _body(src, test)
        kat["cases"][test] = {"file": fname, "line": line, "params": params, "arrays": _arrays(body, env)}

    # GPU.cu known answers (u64). Parameters are the literal call arguments.
    add(gpu, "src/test/GPU.cu", "CutlassGemm", {"calls": [[2, 4, 3, 0, 0, 0]]})
    add(gpu, "src/test/GPU.cu", "CutlassGemmTranspose",
        {"calls": [[2, 2, 3, 0, 1, 0], [3, 3, 2, 1, 0, 0], [3, 1, 2, 1, 1, 0]]})
    add(gpu, "src/test/GPU.cu", "CutlassGemmTranspose2", {"calls": [[3, 4, 2, 1, 1, 1]]})
    add(gpu, "src/test/GPU.cu", "CutlassConvFprop", {"N": 1, "H": 3, "W": 3, "C": 1, "K": 1, "R": 3, "pad": 1, "stride": 1})
    add(gpu, "src/test/GPU.cu", "CutlassConvDgrad", {"N": 1, "H": 3, "W": 3, "C": 1, "K": 1, "R": 3, "pad": 1, "stride": 1})
    add(gpu, "src/test/GPU.cu", "CutlassConvDgrad2", {"N": 2, "H": 5, "W": 5, "C": 4, "K": 10, "R": 3, "pad": 1, "stride": 2})
    add(gpu, "src/test/GPU.cu", "CutlassConvWgrad", {"N": 1, "H": 3, "W": 3, "C": 1, "K": 1, "R": 3, "pad": 1, "stride": 1})
    add(gpu, "src/test/GPU.cu", "CutlassConvWgrad2", {"N": 2, "H": 5, "W": 5, "C": 4, "K": 10, "R": 3, "pad": 1, "stride": 2})
    add(gpu, "src/test/GPU.cu", "ElementwiseVectorAdd", {"rows": 2, "cols": 3})
    add(gpu, "src/test/GPU.cu", "ReduceSum", {"reduceRows": 1, "rows": 2, "cols": 4})
    add(gpu, "src/test/GPU.cu", "BitExpand64", {})
    add(gpu, "src/test/GPU.cu", "ExpandCompare", {})
    s64min3 = -(2 ** 63) // 3 + (1 if (-(2 ** 63)) % 3 else 0)  # C++ truncating division
    add(gpu, "src/test/GPU.cu", "Maxpool_Im2Row",
        {"H": 4, "W": 4, "f": 3, "Din": 2, "batch": 1, "stride": 1, "pad": 0, "pad_val": s64min3},
        env={"pad": float(s64min3)})
    add(gpu, "src/test/GPU.cu", "StridePad", {})

    # Func.cu protocol known answers (values decoded with eps = 1e-3, util.cuh:19).
    for t, p in [("Reconstruct", {}),
                 ("MatMul", {"M": 2, "N": 4, "K": 3, "tA": 0, "tB": 0, "tC": 0}),
                 ("MatMul2", {"M": 4, "N": 3, "K": 4, "tA": 1, "tB": 1, "tC": 1}),
                 ("Mult", {"fixed": False}),
                 ("Truncate", {"d": 1 << 3}),
                 ("Truncate2", {"d": 1 << 21}),
                 ("TruncateVec", {}),
                 ("SelectShare", {}),
                 ("Convolution", {"batch": 2, "H": 3, "W": 3, "f": 3, "Din": 1, "Dout": 1, "stride": 1, "pad": 1}),
                 ("DRELU", {}), ("DRELU2", {}), ("DRELU3", {}), ("RELU", {}),
                 ("Maxpool", {"k": 4}), ("Maxpool2", {"k": 16})]:
        add(func, "src/test/Func.cu", t, p, env={"negative": float(neg)})

    # Layer.cu inline cases
    add(layer, "src/test/Layer.cu", "FCForwardBasic", {"inputDim": 4, "batch": 4, "outputDim": 3})
    add(layer, "src/test/Layer.cu", "ReLUForwardBasic", {})
    add(layer, "src/test/Layer.cu", "MaxpoolForwardBasic", {"H": 2, "W": 2, "C": 2, "pool": 2, "stride": 1, "batch": 2})
    for t, p in [("CNNForwardBasic", {"H": 3, "W": 3, "Din": 1, "Dout": 1, "f": 3, "stride": 1, "pad": 1, "batch": 2}),
                 ("CNNForwardStride", {"H": 3, "W": 3, "Din": 1, "Dout": 1, "f": 3, "stride": 2, "pad": 1, "batch": 1}),
                 ("CNNForwardInputChannels", {"H": 3, "W": 3, "Din": 2, "Dout": 1, "f": 3, "stride": 2, "pad": 1, "batch": 2}),
                 ("CNNForwardAllDims", {"H": 3, "W": 3, "Din": 2, "Dout": 2, "f": 3, "stride": 2, "pad": 1, "batch": 2})]:
        add(layer, "src/test/Layer.cu", t, p)

    # Layer.cu backward inline cases
    add(layer, "src/test/Layer.cu", "ReLUBackwardBasic", {"batch": 1})
    add(layer, "src/test/Layer.cu", "MaxpoolBackwardBasic", {"H": 2, "W": 2, "C": 2, "pool": 2, "stride": 1, "batch": 2})
    add(layer, "src/test/Layer.cu", "AveragepoolForwardBasic", {"H": 2, "W": 2, "C": 2, "pool": 2, "stride": 1, "batch": 2})
    add(layer, "src/test/Layer.cu", "AveragepoolBackwardBasic", {"H": 2, "W": 2, "C": 2, "pool": 2, "stride": 1, "batch": 2})
    add(layer, "src/test/Layer.cu", "CNNBackwardBasic",
        {"H": 3, "W": 3, "Din": 2, "Dout": 3, "f": 3, "stride": 2, "pad": 1, "batch": 2})

    with open(os.path.join(HERE, "kat.json"), "w") as f:
        json.dump(kat, f, indent=0, sort_keys=True)

    def load(rel, n=None):
        vals = np.array(open(os.path.join(REF, "files/test", rel)).read().split(), dtype=np.float64)
        return vals if n is None else vals[:n]

    arrays = {
        # FCForwardMNIST (Layer.cu:52-84): 16 -> 10, batch 128
        "fc_mnist_input": load("test_fclayer_input", 128 * 16),
        "fc_mnist_weight": load("test_fclayer_weight", 16 * 10),
        "fc_mnist_bias": load("test_fclayer_bias", 10),
        "fc_mnist_output": load("test_fclayer_output", 128 * 10),
        # ReLUForwardMNIST (Layer.cu:205-236): 128 x 128
        "relu_mnist_input": load("test_relulayer_input", 128 * 128),
        "relu_mnist_output": load("test_relulayer_output", 128 * 128),
        # MaxpoolForwardMNIST (Layer.cu:299-339): 9x9x2, pool 3, stride 2, batch 128
        "maxpool_mnist_input": load("test_maxpoollayer_input", 128 * 2 * 81),
        "maxpool_mnist_output": load("test_maxpoollayer_output", 128 * 2 * 16),
        # CNNForwardMNIST (Layer.cu:670-713): 9x9x2 -> 3, f 3, stride 2, pad 1, batch 128
        "cnn_mnist_input": load("test_convlayer_input", 128 * 81 * 2),
        "cnn_mnist_weight": load("test_convlayer_weight", 3 * 9 * 2),
        "cnn_mnist_output": load("test_convlayer_output", 128 * 25 * 3),
    }
    # FCBackwardMNIST (Layer.cu:118-180): 16 -> 10, batch 128, log_learning_rate 6
    arrays["fc_bw_gradin"] = load("test_fclayer_gradin", 128 * 10)
    arrays["fc_bw_gradout"] = load("test_fclayer_gradout", 128 * 16)
    arrays["fc_bw_newweight"] = load("test_fclayer_newweight", 16 * 10)
    arrays["fc_bw_newbias"] = load("test_fclayer_newbias", 10)
    arrays["fc_bw_gradweight"] = load("test_fclayer_gradweight", 16 * 10)
    arrays["fc_bw_gradbias"] = load("test_fclayer_gradbias", 10)
    # MaxpoolBackwardMNIST (Layer.cu:379-417): 9x9x2, pool 3, stride 2, batch 128
    arrays["maxpool_bw_gradin"] = load("test_maxpoollayer_gradin", 128 * 2 * 16)
    arrays["maxpool_bw_gradout"] = load("test_maxpoollayer_gradout", 128 * 2 * 81)
    # CNNBackwardMNIST (Layer.cu:772-836): 9x9x2 -> 3, f 3, stride 2, pad 1, batch 128
    arrays["cnn_bw_gradin"] = load("test_convlayer_gradin", 128 * 25 * 3)
    arrays["cnn_bw_gradout"] = load("test_convlayer_gradout", 128 * 81 * 2)
    arrays["cnn_bw_newweight"] = load("test_convlayer_newweight", 3 * 9 * 2)
    arrays["cnn_bw_gradweight"] = load("test_convlayer_gradweight", 3 * 9 * 2)
    # SecureML forward chain (Layer.cu:86-116 and files/test/secureml/*)
    arrays["secureml_input"] = load("secureml/input", 128 * 784)
    for i, (din, dout) in zip((0, 2, 4), ((784, 128), (128, 128), (128, 10))):
        arrays[f"secureml_weight{i}"] = load(f"secureml/weight{i}", din * dout)
        arrays[f"secureml_bias{i}"] = load(f"secureml/bias{i}", dout)
    for i in range(6):
        n = 128 * (10 if i >= 4 else 128)
        arrays[f"secureml_output{i}"] = load(f"secureml/outputlayer{i}", n)
    # SecureML training step (files/test/secureml/*): labels, every layer's
    # incoming gradient, and the updated parameters (a 4096-value slice of the
    # 784 x 128 layer-0 weights keeps the fixture small)
    arrays["secureml_labels"] = load("secureml/labels", 128 * 10)
    for i in range(6):
        n = 128 * (10 if i >= 4 else 128)
        arrays[f"secureml_gradin{i}"] = load(f"secureml/gradin_layer{i}", n)
    arrays["secureml_newweight0_head"] = load("secureml/newweight_layer0", 4096)
    for i, (din, dout) in zip((2, 4), ((128, 128), (128, 10))):
        arrays[f"secureml_newweight{i}"] = load(f"secureml/newweight_layer{i}", din * dout)
    for i, dout in zip((0, 2, 4), (128, 128, 10)):
        arrays[f"secureml_newbias{i}"] = load(f"secureml/newbias_layer{i}", dout)
    np.savez_compressed(os.path.join(HERE, "layers.npz"), **arrays)
    print("wrote", sorted(kat["cases"]), "and", sorted(arrays))


if __name__ == "__main__":
    main()
