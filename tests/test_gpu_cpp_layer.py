"""The C++ share-class layer (include/piranha_gb300.hpp) from C++.

tests/cpp/func_kat.cpp is compiled against the header and the library, and
runs the reference's protocol known answers (src/test/Func.cu: Reconstruct,
MatMul, MatMul2, Mult, Truncate, Truncate2, TruncateVec, SelectShare,
Convolution, DRELU, DRELU2, DRELU3, RELU, Maxpool, Maxpool2; src/test/GPU.cu:
CutlassGemm, CutlassConvFprop) the way those tests call RSS<T>, DeviceData<T>
and the free functions. The revealed results must be the reference's
expected values (within its epsilon, 1e-3, or exactly for bits and plain ring
values), and every share of every result must equal the oracle's.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
U64 = np.uint64
EPS = 1e-3  # src/util/util.cuh:19

FUNC_CASES = ["Reconstruct", "MatMul", "MatMul2", "Mult", "Truncate", "Truncate2", "TruncateVec", "SelectShare",
              "Convolution", "DRELU", "DRELU2", "DRELU3", "RELU", "Maxpool", "Maxpool2"]
GPU_CASES = ["CutlassGemm", "CutlassConvFprop"]


@pytest.fixture(scope="module")
def binary(tmp_path_factory):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import piranha_gb300 as pg

    libpath = pg.library_path()
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    out = str(tmp_path_factory.mktemp("cpp") / "func_kat")
    libdir = os.path.dirname(libpath)
    cudalib = next((d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"),
                                os.path.join(cuda, "targets", "sbsa-linux", "lib"))
                    if os.path.exists(os.path.join(d, "libcudart.so"))), os.path.join(cuda, "lib64"))
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "cpp", "func_kat.cpp"), "-o", out, "-L" + libdir, "-lpiranha_gb300",
           "-L" + cudalib, "-lcudart", "-Wl,-rpath," + libdir, "-Wl,-rpath," + cudalib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _case_text(name, case):
    lines = [f"case {name}"]
    for k, v in case["arrays"].items():
        if k in ("expected", "dexpected"):
            continue
        lines.append(f"arr {k} {len(v)} " + " ".join(repr(float(x)) for x in v))
    params = dict(case["params"])
    if name == "CutlassGemm":
        M, N, K, tA, tB, tC = params.pop("calls")[0]
        params.update(M=M, N=N, K=K, tA=tA, tB=tB, tC=tC)
    for k, v in params.items():
        if isinstance(v, bool):
            v = int(v)
        lines.append(f"param {k} {int(v)}")
    lines.append("run")
    return "\n".join(lines) + "\n"


@pytest.fixture(scope="module")
def results(binary, golden):
    kat = golden[0]
    text = "".join(_case_text(n, kat[n]) for n in FUNC_CASES + GPU_CASES)
    r = subprocess.run([binary], input=text, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    out = {}
    for line in r.stdout.splitlines():
        parts = line.split()
        if parts[0] == "error":
            pytest.fail(line)
        tag, case, key, n = parts[0], parts[1], parts[2], int(parts[3])
        vals = parts[4:]
        if tag == "out":
            out[(case, "out", key)] = np.array([float(x) for x in vals])
        elif tag == "shares":
            out[(case, "shares", key)] = np.array([int(x) for x in vals], dtype=U64).reshape(3, 2, n)
        else:
            out[(case, "plain", key)] = np.array([int(x) for x in vals], dtype=U64)
    return out


@pytest.mark.parametrize("name", FUNC_CASES)
def test_reference_known_answers_through_cpp(results, golden, name):
    case = golden[0][name]
    got = results[(name, "out", "result")]
    want = np.array(case["arrays"]["expected"], dtype=np.float64)
    assert got.shape == want.shape and np.all(np.abs(got - want) <= EPS), (got, want)
    if "dexpected" in case["arrays"]:
        dgot = results[(name, "out", "dresult")]
        assert np.array_equal(dgot, np.array(case["arrays"]["dexpected"], dtype=np.float64))


def _oracle_shares(name, case):
    a = case["arrays"]
    p = case["params"]
    L = orc.from_list
    if name in ("MatMul", "MatMul2"):
        return "c", orc.matmul(L(a["a"]), L(a["b"]), p["M"], p["N"], p["K"], p["tA"], p["tB"], p["tC"], 26)
    if name == "Mult":
        return "b", orc.mul(L(a["b"], to_fixed=False), L(a["a"], to_fixed=False))
    if name in ("Truncate", "Truncate2"):
        return "a", orc.divide_public(L(a["a"]), p["d"])
    if name == "TruncateVec":
        d = np.left_shift(np.ones(len(a["pows"]), dtype=U64), np.array(a["pows"], dtype=U64))
        return "a", orc.divide_public(L(a["a"]), d)
    if name == "SelectShare":
        return "z", orc.select_share(L(a["x"]), L(a["y"]), L(a["b"], to_fixed=False))
    if name == "Convolution":
        return "out", orc.convolution(L(a["im"]), L(a["filters"]), orc.FPROP, p["batch"], p["H"], p["W"], p["f"],
                                      p["Din"], p["Dout"], p["stride"], p["pad"], 26)
    if name in ("DRELU", "DRELU2", "DRELU3"):
        x = L(a["input"])
        if name == "DRELU3":
            neg = np.uint64((-10 * (1 << 26)) % (1 << 64))
            add = np.array([0, 0, 0, 0, 0, neg, neg, neg], dtype=U64)
            with np.errstate(over="ignore"):
                x = x + add[None, None, :]
        return "result", orc.drelu(x, U64)
    if name == "RELU":
        return "result", orc.relu(L(a["input"]), U64)[0]
    if name == "Maxpool":
        return "result", orc.maxpool(L(a["input"]), p["k"], U64)[0]
    if name == "Maxpool2":
        x = L(a["input"])
        pools = np.stack([np.stack([orc.maxpool_im2row(x[q, s], 3, 3, 3, 1, 1, 1, 0, -10) for s in range(2)])
                          for q in range(3)])
        return "result", orc.maxpool(pools, 16)[0]
    return None, None


@pytest.mark.parametrize("name", [n for n in FUNC_CASES if n != "Reconstruct"])
def test_cpp_shares_equal_oracle(results, golden, name):
    key, want = _oracle_shares(name, golden[0][name])
    assert np.array_equal(results[(name, "shares", key)], want)


def test_cpp_gpu_kernels_known_answers(results, golden):
    kat = golden[0]
    g = kat["CutlassGemm"]
    assert np.array_equal(results[("CutlassGemm", "plain", "c")],
                          np.array(g["arrays"]["expected"], dtype=np.float64).astype(np.int64).astype(U64))
    c = kat["CutlassConvFprop"]
    assert np.array_equal(results[("CutlassConvFprop", "plain", "out")],
                          np.array(c["arrays"]["expected"], dtype=np.float64).astype(np.int64).astype(U64))
