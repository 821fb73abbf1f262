"""Pin the CPU oracle against Piranha's own known-answer tests and fixtures.

The cases come from src/test/GPU.cu, src/test/Func.cu and src/test/Layer.cu
(extracted into tests/golden by make_golden.py). Ring-level kernels (GEMM,
conv, bitexpand, im2row, ...) must match exactly. Protocol-level cases are
compared the way the reference compares them: the value revealed at a party,
decoded from fixed point, within eps = 1e-3 (util.cuh:19), or exactly for the
integer (convertFixed=false) checks. Reveals are taken at party A and C; with
the setPublic fall-through (RSS.inl:129-141) party B's view of a public-loaded
tensor is inconsistent, so the reference's own assertions only hold at A and C
for those cases.
"""
import numpy as np
import pytest

import oracle as orc

FP = 26
EPS = 1e-3
U64 = np.uint64


def u64(vals):
    return np.array([int(v) % (1 << 64) for v in vals], dtype=U64)


def s64(x):
    return np.asarray(x, dtype=U64).view(np.int64)


def reveal(views, party=0):
    return orc.reconstruct(views)[party]


# ------------------------------------------------------------- GPU.cu cases

def test_gemm_kats(golden):
    kat, _ = golden
    c = kat["CutlassGemm"]
    a, b = c["arrays"]["a"], c["arrays"]["b"]
    M, N, K, tA, tB, tC = c["params"]["calls"][0]
    assert list(orc.gemm(M, N, K, u64(a), tA, u64(b), tB, tC)) == list(u64(c["arrays"]["expected"]))

    c = kat["CutlassGemmTranspose"]
    a, d = u64(c["arrays"]["a"]), u64(c["arrays"]["d"])
    outs = ["expected", "expected2", "expected3"]
    rhs = [a, a, d]
    for (M, N, K, tA, tB, tC), o, r in zip(c["params"]["calls"], outs, rhs):
        assert list(orc.gemm(M, N, K, a, tA, r, tB, tC)) == list(u64(c["arrays"][o]))

    c = kat["CutlassGemmTranspose2"]
    M, N, K, tA, tB, tC = c["params"]["calls"][0]
    got = orc.gemm(M, N, K, u64(c["arrays"]["a"]), tA, u64(c["arrays"]["b"]), tB, tC)
    assert list(got) == list(u64(c["arrays"]["expected"]))


@pytest.mark.parametrize("name,op,a,b", [
    ("CutlassConvFprop", orc.FPROP, "im", "f"),
    ("CutlassConvDgrad", orc.DGRAD, "delta", "f"),
    ("CutlassConvDgrad2", orc.DGRAD, "delta", "filters"),
    ("CutlassConvWgrad", orc.WGRAD, "delta", "im"),
    ("CutlassConvWgrad2", orc.WGRAD, "delta", "input"),
])
def test_conv_kats(golden, name, op, a, b):
    kat, _ = golden
    c = kat[name]
    p = c["params"]
    got = orc.conv(op, p["N"], p["H"], p["W"], p["C"], p["K"], p["R"], p["R"], p["pad"], p["stride"],
                   u64(c["arrays"][a]), u64(c["arrays"][b]))
    assert list(got) == list(u64(c["arrays"]["expected"]))


def test_element_vector_add_and_reduce(golden):
    kat, _ = golden
    c = kat["ElementwiseVectorAdd"]
    a = orc.element_vector_add(u64(c["arrays"]["a"]), u64(c["arrays"]["row_b"]), True, 2, 3)
    assert list(a) == list(u64(c["arrays"]["expected"]))
    a = orc.element_vector_add(a, u64(c["arrays"]["col_b"]), False, 2, 3)
    assert list(a) == list(u64(c["arrays"]["expected@2"]))
    c = kat["ReduceSum"]
    b = orc.reduce_sum(u64(c["arrays"]["a"]), u64(c["arrays"]["b"]), True, 2, 4)
    assert list(b) == list(u64(c["arrays"]["expected"]))


def test_bitexpand_kat(golden):
    kat, _ = golden
    c = kat["BitExpand64"]
    assert list(orc.bitexpand(u64(c["arrays"]["a"]))) == list(u64(c["arrays"]["expected"]))


def test_expand_compare_kat(golden):
    kat, _ = golden
    c = kat["ExpandCompare"]
    b = np.array(c["arrays"]["b"], dtype=np.uint8)
    nb = np.array(c["arrays"]["negb"], dtype=np.uint8)
    # RSS<uint8_t>(list, false): party A shareA / party C shareB hold the values
    outs = np.zeros((3, 2, 8), dtype=np.uint8)
    zero = np.zeros(4, dtype=np.uint8)
    for p, s in ((0, 0), (2, 1)):
        outs[p, s] = orc.expand_compare(b, nb, 8)
    for p, s in ((0, 1), (1, 0), (1, 1), (2, 0)):
        outs[p, s] = orc.expand_compare(zero, zero, 8)
    rec = (outs[0, 0].astype(int) + outs[0, 1] + outs[2, 0]) % 256
    assert list(rec) == [int(v) for v in c["arrays"]["expected"]]


def test_maxpool_im2row_kat(golden):
    kat, _ = golden
    c = kat["Maxpool_Im2Row"]
    p = c["params"]
    got = orc.maxpool_im2row(u64(c["arrays"]["im"]), p["H"], p["W"], p["f"], p["Din"], p["batch"], p["stride"],
                             p["pad"], p["pad_val"])
    # the reference compares (double)(int64) values (util.cuh:55-70,317-328)
    assert np.array_equal(s64(got).astype(np.float64), np.array(c["arrays"]["expected"]))


# ------------------------------------------------------------ Func.cu cases

def enc_list(vals, fixed=True):
    return orc.from_list(vals, U64, FP, to_fixed=fixed)


def assert_reveal(views, expected, fixed=True, parties=(0, 1, 2)):
    rec = orc.reconstruct(views)
    for p in parties:
        got = orc.decode(rec[p], FP) if fixed else s64(rec[p]).astype(np.float64)
        assert np.max(np.abs(got - np.asarray(expected, dtype=np.float64))) <= EPS, (p, got, expected)


def test_func_reconstruct(golden):
    c = golden[0]["Reconstruct"]["arrays"]
    assert_reveal(enc_list(c["a"]), c["expected"])


@pytest.mark.parametrize("name", ["MatMul", "MatMul2"])
def test_func_matmul(golden, name):
    c = golden[0][name]
    p, a = c["params"], c["arrays"]
    comm = orc.Comm()
    out = orc.matmul(enc_list(a["a"]), enc_list(a["b"]), p["M"], p["N"], p["K"], p["tA"], p["tB"], p["tC"], FP, comm)
    assert_reveal(out, a["expected"])
    mn = p["M"] * p["N"]
    assert comm.rounds == 1 and comm.tx == [2 * mn * 8] * 3 and comm.rx == [2 * mn * 8] * 3


def test_func_mult(golden):
    a = golden[0]["Mult"]["arrays"]
    out = orc.mul(enc_list(a["b"], False), enc_list(a["a"], False))
    assert_reveal(out, a["expected"], fixed=False)


@pytest.mark.parametrize("name", ["Truncate", "Truncate2"])
def test_func_truncate(golden, name):
    c = golden[0][name]
    out = orc.divide_public(enc_list(c["arrays"]["a"]), c["params"]["d"])
    assert_reveal(out, c["arrays"]["expected"])


def test_func_truncate_vec(golden):
    a = golden[0]["TruncateVec"]["arrays"]
    d = np.array([1 << int(x) for x in a["pows"]], dtype=U64)
    assert_reveal(orc.divide_public(enc_list(a["a"]), d), a["expected"])


def test_func_select_share(golden):
    a = golden[0]["SelectShare"]["arrays"]
    z = orc.select_share(enc_list(a["x"]), enc_list(a["y"]), enc_list(a["b"], False))
    assert_reveal(z, a["expected"])


def test_func_convolution(golden):
    c = golden[0]["Convolution"]
    p, a = c["params"], c["arrays"]
    out = orc.convolution(enc_list(a["im"]), enc_list(a["filters"]), orc.FPROP, p["batch"], p["H"], p["W"], p["f"],
                          p["Din"], p["Dout"], p["stride"], p["pad"], FP)
    assert_reveal(out, a["expected"])


@pytest.mark.parametrize("name", ["DRELU", "DRELU2"])
def test_func_drelu(golden, name):
    a = golden[0][name]["arrays"]
    comm = orc.Comm()
    res = orc.drelu(enc_list(a["input"]), udtype=U64, comm=comm)
    assert_reveal(res, a["expected"], fixed=False)
    n = len(a["input"])
    assert comm.rounds == 13  # 1 reveal + 6 carry levels x 2 AND-reshares
    assert comm.tx == [n * 8 + 2 * n * (32 + 16 + 8 + 4 + 2 + 1) * 8] * 3  # u64 bit words


def test_func_drelu3(golden):
    a = golden[0]["DRELU3"]["arrays"]
    x = enc_list(a["input"])
    add = u64(a["add"])
    x = (x + add[None, None, :]).astype(U64)  # every share of every party += add
    res = orc.drelu(x, udtype=U64)
    assert_reveal(res, a["expected"], fixed=False)


def test_func_relu(golden):
    a = golden[0]["RELU"]["arrays"]
    comm = orc.Comm()
    out, dout = orc.relu(enc_list(a["input"]), udtype=U64, comm=comm)
    assert_reveal(out, a["expected"])
    assert_reveal(dout, a["dexpected"], fixed=False)
    assert comm.rounds == 15


def test_func_maxpool(golden):
    a = golden[0]["Maxpool"]["arrays"]
    out, dout = orc.maxpool(enc_list(a["input"]), 4, udtype=U64)
    assert_reveal(out, a["expected"])
    assert_reveal(dout, a["dexpected"], fixed=False)


def test_func_maxpool2(golden):
    a = golden[0]["Maxpool2"]["arrays"]
    x = enc_list(a["input"])
    pools = np.stack([np.stack([orc.maxpool_im2row(x[p, s], 3, 3, 3, 1, 1, 1, 0, -10) for s in range(2)])
                      for p in range(3)])
    out, dexp = orc.maxpool(pools, 16, udtype=U64)
    dres = dexp[:, :, :9]  # truncate_cols(16 -> 9) for the single pool row
    assert_reveal(out, a["expected"])
    assert_reveal(dres, a["dexpected"], fixed=False)


# ---------------------------------------------- Func.cu cases, TPC (2PC)
# The reference's Func tests are typed over RSS, TPC, FPC and OPC
# (src/test/Func.cu:11), so the same expected values pin the TPC restatement.

def tenc(vals, fixed=True):
    return orc.tpc_from_list(vals, U64, FP, to_fixed=fixed)


def assert_reveal_tpc(shares, expected, fixed=True):
    rec = orc.tpc_reconstruct(shares)
    for p in (0, 1):
        got = orc.decode(rec[p], FP) if fixed else s64(rec[p].astype(U64)).astype(np.float64)
        assert np.max(np.abs(got - np.asarray(expected, dtype=np.float64))) <= EPS, (p, got, expected)


def test_tpc_func_reconstruct(golden):
    c = golden[0]["Reconstruct"]["arrays"]
    assert_reveal_tpc(tenc(c["a"]), c["expected"])


@pytest.mark.parametrize("name", ["MatMul", "MatMul2"])
def test_tpc_func_matmul(golden, name):
    c = golden[0][name]
    p, a = c["params"], c["arrays"]
    comm = orc.Comm()
    out = orc.tpc_matmul(tenc(a["a"]), tenc(a["b"]), p["M"], p["N"], p["K"], p["tA"], p["tB"], p["tC"], FP, comm)
    assert_reveal_tpc(out, a["expected"])
    # reveal e (M x K) and f (K x N), then the truncation's reveal (M x N)
    n = p["M"] * p["K"] + p["K"] * p["N"] + p["M"] * p["N"]
    assert comm.rounds == 3 and comm.tx[:2] == [n * 8] * 2


def test_tpc_func_mult(golden):
    a = golden[0]["Mult"]["arrays"]
    assert_reveal_tpc(orc.tpc_mul(tenc(a["b"], False), tenc(a["a"], False)), a["expected"], fixed=False)


@pytest.mark.parametrize("name", ["Truncate", "Truncate2"])
def test_tpc_func_truncate(golden, name):
    c = golden[0][name]
    assert_reveal_tpc(orc.tpc_divide_public(tenc(c["arrays"]["a"]), c["params"]["d"]), c["arrays"]["expected"])


def test_tpc_func_truncate_vec(golden):
    a = golden[0]["TruncateVec"]["arrays"]
    d = np.array([1 << int(x) for x in a["pows"]], dtype=U64)
    assert_reveal_tpc(orc.tpc_divide_public(tenc(a["a"]), d), a["expected"])


def test_tpc_func_select_share(golden):
    a = golden[0]["SelectShare"]["arrays"]
    z = orc.tpc_select_share(tenc(a["x"]), tenc(a["y"]), tenc(a["b"], False))
    assert_reveal_tpc(z, a["expected"])


@pytest.mark.parametrize("name", ["DRELU", "DRELU2"])
def test_tpc_func_drelu(golden, name):
    a = golden[0][name]["arrays"]
    comm = orc.Comm()
    res = orc.tpc_drelu(tenc(a["input"]), udtype=U64, comm=comm)
    assert_reveal_tpc(res, a["expected"], fixed=False)
    assert comm.rounds == 25  # 1 reveal + 6 carry levels x 2 ANDs x 2 reveals


def test_tpc_func_drelu3(golden):
    a = golden[0]["DRELU3"]["arrays"]
    x = tenc(a["input"])
    x = (x + u64(a["add"])[None, :]).astype(U64)  # the one share of each party += add
    assert_reveal_tpc(orc.tpc_drelu(x, udtype=U64), a["expected"], fixed=False)


def test_tpc_func_relu(golden):
    a = golden[0]["RELU"]["arrays"]
    out, dout = orc.tpc_relu(tenc(a["input"]), udtype=U64)
    assert_reveal_tpc(out, a["expected"])
    assert_reveal_tpc(dout, a["dexpected"], fixed=False)


def test_tpc_func_maxpool(golden):
    a = golden[0]["Maxpool"]["arrays"]
    out, dout = orc.tpc_maxpool(tenc(a["input"]), 4, udtype=U64)
    assert_reveal_tpc(out, a["expected"])
    assert_reveal_tpc(dout, a["dexpected"], fixed=False)


def test_tpc_func_convolution(golden):
    c = golden[0]["Convolution"]
    p, a = c["params"], c["arrays"]
    out = orc.tpc_convolution(tenc(a["im"]), tenc(a["filters"]), orc.FPROP, p["batch"], p["H"], p["W"], p["f"],
                              p["Din"], p["Dout"], p["stride"], p["pad"], FP)
    assert_reveal_tpc(out, a["expected"])


# ---------------------------------------------- Func.cu cases, FPC (4PC)
# The same typed Func vectors pin the 4-party restatement; every party's
# reveal (own three shares plus the previous party's shareA) must match.

def fenc(vals, fixed=True):
    return orc.fpc_from_list(vals, U64, FP, to_fixed=fixed)


def assert_reveal_fpc(shares, expected, fixed=True):
    rec = orc.fpc_reconstruct(shares)
    for p in range(4):
        got = orc.decode(rec[p], FP) if fixed else s64(rec[p].astype(U64)).astype(np.float64)
        assert np.max(np.abs(got - np.asarray(expected, dtype=np.float64))) <= EPS, (p, got, expected)


def test_fpc_func_reconstruct(golden):
    c = golden[0]["Reconstruct"]["arrays"]
    comm = orc.Comm(4)
    rec = orc.fpc_reconstruct(fenc(c["a"]), comm)
    for p in range(4):
        assert np.max(np.abs(orc.decode(rec[p], FP) - np.asarray(c["expected"]))) <= EPS
    n = len(c["a"])
    assert comm.rounds == 1 and comm.tx == [n * 8] * 4 and comm.rx == [n * 8] * 4


@pytest.mark.parametrize("name", ["MatMul", "MatMul2"])
def test_fpc_func_matmul(golden, name):
    c = golden[0][name]
    p, a = c["params"], c["arrays"]
    comm = orc.Comm(4)
    out = orc.fpc_matmul(fenc(a["a"]), fenc(a["b"]), p["M"], p["N"], p["K"], p["tA"], p["tB"], p["tC"], FP, comm)
    assert_reveal_fpc(out, a["expected"])
    # six reshares (sender I -> receiver G, M x N each), then the truncation's reveal
    mn = p["M"] * p["N"]
    assert comm.rounds == 7
    assert comm.tx == [3 * mn * 8 + mn * 8, 2 * mn * 8 + mn * 8, mn * 8 + mn * 8, mn * 8]
    assert comm.rx == [mn * 8 + mn * 8, 2 * mn * 8 + mn * 8, 2 * mn * 8 + mn * 8, mn * 8 + mn * 8]


def test_fpc_func_mult(golden):
    a = golden[0]["Mult"]["arrays"]
    assert_reveal_fpc(orc.fpc_mul(fenc(a["b"], False), fenc(a["a"], False)), a["expected"], fixed=False)


@pytest.mark.parametrize("name", ["Truncate", "Truncate2"])
def test_fpc_func_truncate(golden, name):
    c = golden[0][name]
    assert_reveal_fpc(orc.fpc_divide_public(fenc(c["arrays"]["a"]), c["params"]["d"]), c["arrays"]["expected"])


def test_fpc_func_truncate_vec(golden):
    a = golden[0]["TruncateVec"]["arrays"]
    d = np.array([1 << int(x) for x in a["pows"]], dtype=U64)
    assert_reveal_fpc(orc.fpc_divide_public(fenc(a["a"]), d), a["expected"])


def test_fpc_func_select_share(golden):
    a = golden[0]["SelectShare"]["arrays"]
    z = orc.fpc_select_share(fenc(a["x"]), fenc(a["y"]), fenc(a["b"], False))
    assert_reveal_fpc(z, a["expected"])


@pytest.mark.parametrize("name", ["DRELU", "DRELU2"])
def test_fpc_func_drelu(golden, name):
    a = golden[0][name]["arrays"]
    comm = orc.Comm(4)
    res = orc.fpc_drelu(fenc(a["input"]), udtype=U64, comm=comm)
    assert_reveal_fpc(res, a["expected"], fixed=False)
    assert comm.rounds == 73  # 1 reveal + 6 carry levels x 2 ANDs x 6 reshares


def test_fpc_func_drelu3(golden):
    a = golden[0]["DRELU3"]["arrays"]
    x = fenc(a["input"])
    x = (x + u64(a["add"])[None, None, :]).astype(U64)  # every share of every party += add
    assert_reveal_fpc(orc.fpc_drelu(x, udtype=U64), a["expected"], fixed=False)


def test_fpc_func_relu(golden):
    a = golden[0]["RELU"]["arrays"]
    out, dout = orc.fpc_relu(fenc(a["input"]), udtype=U64)
    assert_reveal_fpc(out, a["expected"])
    assert_reveal_fpc(dout, a["dexpected"], fixed=False)


def test_fpc_func_maxpool(golden):
    a = golden[0]["Maxpool"]["arrays"]
    out, dout = orc.fpc_maxpool(fenc(a["input"]), 4, udtype=U64)
    assert_reveal_fpc(out, a["expected"])
    assert_reveal_fpc(dout, a["dexpected"], fixed=False)


def test_fpc_func_convolution(golden):
    c = golden[0]["Convolution"]
    p, a = c["params"], c["arrays"]
    out = orc.fpc_convolution(fenc(a["im"]), fenc(a["filters"]), orc.FPROP, p["batch"], p["H"], p["W"], p["f"],
                              p["Din"], p["Dout"], p["stride"], p["pad"], FP)
    assert_reveal_fpc(out, a["expected"])


def test_fpc_random_sharing_product_is_not_the_product():
    """A quirk the restatement keeps: reshareFPC's PRG masks are zero and party
    J adds its own cross term where I and G add I's (FPC.inl:1184-1259), so a
    product of two fully random 4-party sharings does not reveal x*y, while
    the same values loaded through setPublic (x0 only) do."""
    M, N, K = 4, 3, 5
    rng = np.random.default_rng(3)
    xv, wv = rng.normal(0, 1, M * K), rng.normal(0, 1, K * N)
    ref = orc.decode(orc.gemm(M, N, K, orc.encode(xv), 1, orc.encode(wv), 1, 1), 2 * FP)
    pub = orc.fpc_reconstruct(orc.fpc_matmul(fenc(xv), fenc(wv), M, N, K, 1, 1, 1, FP))
    assert all(np.max(np.abs(orc.decode(pub[p], FP) - ref)) < EPS for p in range(4))
    a, b = orc.fpc_share_random(orc.encode(xv), seed=4), orc.fpc_share_random(orc.encode(wv), seed=5)
    rnd = orc.fpc_reconstruct(orc.fpc_matmul(a, b, M, N, K, 1, 1, 1, FP))
    assert any(np.max(np.abs(orc.decode(rnd[p], FP) - ref)) > 1.0 for p in range(4))


def test_fpc_share_random_reconstructs():
    rng = np.random.default_rng(5)
    v = rng.integers(0, 1 << 63, 100, dtype=U64)
    rec = orc.fpc_reconstruct(orc.fpc_share_random(v, seed=6))
    assert all(np.array_equal(rec[p], v) for p in range(4))


# ----------------------------------------------------------- Layer.cu cases

def test_layer_relu_basic(golden):
    a = golden[0]["ReLUForwardBasic"]["arrays"]
    out, _ = orc.relu(enc_list(a["input"]))
    assert_reveal(out, a["expected"])


def test_layer_maxpool_basic(golden):
    c = golden[0]["MaxpoolForwardBasic"]
    p, a = c["params"], c["arrays"]
    out, _ = orc.maxpool_layer(enc_list(a["inputImage"]), p["H"], p["W"], p["C"], p["pool"], p["stride"], p["batch"])
    assert_reveal(out, a["expected"])


@pytest.mark.parametrize("name", ["CNNForwardBasic", "CNNForwardStride", "CNNForwardInputChannels",
                                  "CNNForwardAllDims"])
def test_layer_cnn_inline(golden, name):
    c = golden[0][name]
    p, a = c["params"], c["arrays"]
    out = orc.convolution(enc_list(a["im"]), enc_list(a["filter"]), orc.FPROP, p["batch"], p["H"], p["W"], p["f"],
                          p["Din"], p["Dout"], p["stride"], p["pad"], FP)
    assert_reveal(out, a["expected"])


def fc_forward(x, w, b, batch, din, dout):
    """FCLayer::forward (FCLayer.cu:78-130): matmul(tA=tB=tC=1) + per-share bias add."""
    act = orc.matmul(x, w, batch, dout, din, 1, 1, 1, FP)
    for p in range(3):
        for s in range(2):
            act[p, s] = orc.element_vector_add(act[p, s], b[p, s], False, dout, batch)
    return act


def test_layer_fc_mnist(golden):
    L = golden[1]
    x = orc.set_public(L["fc_mnist_input"])
    w = orc.set_public(L["fc_mnist_weight"])
    b = orc.set_public(L["fc_mnist_bias"])
    act = fc_forward(x, w, b, 128, 16, 10)
    assert_reveal(act, L["fc_mnist_output"], parties=(0, 2))


def test_layer_relu_mnist(golden):
    L = golden[1]
    out, _ = orc.relu(orc.set_public(L["relu_mnist_input"]))
    assert_reveal(out, L["relu_mnist_output"], parties=(0, 2))


def test_layer_maxpool_mnist(golden):
    L = golden[1]
    out, _ = orc.maxpool_layer(orc.set_public(L["maxpool_mnist_input"]), 9, 9, 2, 3, 2, 128)
    assert_reveal(out, L["maxpool_mnist_output"], parties=(0, 2))


def test_layer_cnn_mnist(golden):
    L = golden[1]
    out = orc.convolution(orc.set_public(L["cnn_mnist_input"]), orc.set_public(L["cnn_mnist_weight"]), orc.FPROP,
                          128, 9, 9, 3, 2, 3, 2, 1, FP)
    assert_reveal(out, L["cnn_mnist_output"], parties=(0, 2))


def test_layer_secureml_chain(golden):
    """SecureML forward (files/test/secureml): FC-ReLU-FC-ReLU-FC-ReLU, every intermediate output."""
    L = golden[1]
    x = orc.set_public(L["secureml_input"])
    dims = [(784, 128), (128, 128), (128, 10)]
    outs = []
    for li, (din, dout) in zip((0, 2, 4), dims):
        w = orc.set_public(L[f"secureml_weight{li}"])
        b = orc.set_public(L[f"secureml_bias{li}"])
        x = fc_forward(x, w, b, 128, din, dout)
        outs.append(x)
        x, _ = orc.relu(x)
        outs.append(x)
    for i, o in enumerate(outs):
        assert_reveal(o, L[f"secureml_output{i}"], parties=(0,))


# ------------------------------------------------ Layer.cu backward cases

def test_layer_relu_backward_basic(golden):
    a = golden[0]["ReLUBackwardBasic"]["arrays"]
    _, d = orc.relu(enc_list(a["input"]))
    assert_reveal(orc.relu_layer_backward(enc_list(a["delta"]), d), a["expected"])


def test_layer_maxpool_backward_basic(golden):
    c = golden[0]["MaxpoolBackwardBasic"]
    p, a = c["params"], c["arrays"]
    geo = (p["H"], p["W"], p["C"], p["pool"], p["stride"], p["batch"])
    _, mp = orc.maxpool_layer(enc_list(a["inputImage"]), *geo)
    assert_reveal(orc.maxpool_layer_backward(enc_list(a["gradin"]), mp, *geo), a["expected"])


def test_layer_avgpool_forward_basic(golden):
    c = golden[0]["AveragepoolForwardBasic"]
    p, a = c["params"], c["arrays"]
    out = orc.avgpool_layer(enc_list(a["inputImage"]), p["H"], p["W"], p["C"], p["pool"], p["stride"], p["batch"])
    assert_reveal(out, a["expected"])


def test_layer_avgpool_backward_basic(golden):
    c = golden[0]["AveragepoolBackwardBasic"]
    p, a = c["params"], c["arrays"]
    comm = orc.Comm()
    d = orc.avgpool_layer_backward(enc_list(a["gradin"]), p["H"], p["W"], p["C"], p["pool"], p["batch"], comm)
    assert_reveal(d, a["expected"])
    assert comm.rounds == 1 and comm.tx == [16 * 8] * 3  # the dividePublic of the 16 input gradients


def test_layer_cnn_backward_basic(golden):
    c = golden[0]["CNNBackwardBasic"]
    p, a = c["params"], c["arrays"]
    w, x = enc_list(a["weights"]), enc_list(a["input"])
    act = orc.convolution(x, w, orc.FPROP, p["batch"], p["H"], p["W"], p["f"], p["Din"], p["Dout"], p["stride"],
                          p["pad"], FP)
    assert_reveal(act, a["expected_activations"])
    d, _ = orc.cnn_layer_backward(enc_list(a["gradin"]), x, w, p["batch"], p["H"], p["W"], p["Din"], p["Dout"], p["f"],
                                  p["stride"], p["pad"], FP, 5)
    assert_reveal(d, a["gradout"])


def test_layer_fc_backward_mnist(golden):
    """FCBackwardMNIST (Layer.cu:118-180), log_learning_rate 6: the input
    gradient, the updated weights and the updated biases (the bias gradient
    goes through the reference's reduceSum(delta, db, false, outputDim,
    batchSize), restated as is)."""
    L = golden[1]
    comm = orc.Comm()
    d, w, b = orc.fc_layer_backward(orc.set_public(L["fc_bw_gradin"]), orc.set_public(L["fc_mnist_input"]),
                                    orc.set_public(L["fc_mnist_weight"]), orc.set_public(L["fc_mnist_bias"]),
                                    128, 16, 10, FP, 6, comm)
    assert_reveal(d, L["fc_bw_gradout"], parties=(0, 2))
    assert_reveal(w, L["fc_bw_newweight"], parties=(0, 2))
    assert_reveal(b, L["fc_bw_newbias"], parties=(0, 2))
    # delta matmul (128 x 16), dW matmul (10 x 16), db dividePublic (10)
    assert comm.rounds == 3 and comm.tx == [(2 * 128 * 16 + 2 * 16 * 10 + 10) * 8] * 3


def test_layer_maxpool_backward_mnist(golden):
    L = golden[1]
    _, mp = orc.maxpool_layer(orc.set_public(L["maxpool_mnist_input"]), 9, 9, 2, 3, 2, 128)
    d = orc.maxpool_layer_backward(orc.set_public(L["maxpool_bw_gradin"]), mp, 9, 9, 2, 3, 2, 128)
    assert_reveal(d, L["maxpool_bw_gradout"], parties=(0, 2))


@pytest.mark.parametrize("log_lr", [5, 6])
def test_layer_cnn_backward_mnist(golden, log_lr):
    """CNNBackwardMNIST (Layer.cu:772-836). The test leaves log_learning_rate
    at whatever the suite set before it (6 after FCBackwardMNIST, 5 alone);
    the new weights match within eps for both."""
    L = golden[1]
    d, w = orc.cnn_layer_backward(orc.set_public(L["cnn_bw_gradin"]), orc.set_public(L["cnn_mnist_input"]),
                                  orc.set_public(L["cnn_mnist_weight"]), 128, 9, 9, 2, 3, 3, 2, 1, FP, log_lr)
    assert_reveal(d, L["cnn_bw_gradout"], parties=(0, 2))
    assert_reveal(w, L["cnn_bw_newweight"], parties=(0, 2))


def test_secureml_training_step(golden):
    """One SecureML training iteration (files/test/secureml): forward, the
    revealed softmax gradient (NeuralNetwork.cu:207-267), every layer's
    backward; each layer's incoming gradient and the updated weights and
    biases match the fixtures, whose update used learning rate 2^-9."""
    from oracle import netref

    L = golden[1]
    layers = netref.secureml_layers()
    params = []
    for li in (0, 2, 4):
        params += [(orc.set_public(L[f"secureml_weight{li}"]), orc.set_public(L[f"secureml_bias{li}"])), None]
    x = orc.set_public(L["secureml_input"])
    labels = orc.set_public(L["secureml_labels"])
    _, outs, newp, deltas = netref.train_step(layers, params, x, labels, 128, FP, 9)
    for i in range(6):
        assert_reveal(outs[i], L[f"secureml_output{i}"], parties=(0, 2))
    softmax_delta = orc.reveal_softmax_grad(outs[-1], labels, 128, FP)
    assert_reveal(softmax_delta, L["secureml_gradin5"], parties=(0, 2))
    for i in range(5):
        assert_reveal(deltas[i + 1], L[f"secureml_gradin{i}"], parties=(0, 2))
    w0 = orc.decode(orc.reconstruct(newp[0][0])[0], FP)[:4096]
    assert np.max(np.abs(w0 - L["secureml_newweight0_head"])) <= EPS
    for li in (2, 4):
        assert_reveal(newp[li][0], L[f"secureml_newweight{li}"], parties=(0, 2))
    for li in (0, 2, 4):
        assert_reveal(newp[li][1], L[f"secureml_newbias{li}"], parties=(0, 2))


# --------------------------------------------------------- ring semantics

def test_division_semantics():
    """functors.cuh:33-45: truncation toward zero of the rounded double."""
    x = np.array([7, (-7) % (1 << 64), (1 << 60) + 1, (1 << 63) - 1, 1 << 63], dtype=U64)
    got = s64(orc.div_public_values(x, 2))
    exp = [3, -3, 1 << 59, 1 << 62, -(1 << 62)]
    assert list(got) == exp
    # |x| > 2^53: the int64 -> double rounding is visible
    x = np.array([(1 << 54) + 3], dtype=U64)
    assert int(s64(orc.div_public_values(x, 1))[0]) == (1 << 54) + 4
    # d = 1 and x rounding up to 2^63 saturates like cvt.rzi.s64.f64
    x = np.array([(1 << 63) - 1], dtype=U64)
    assert int(s64(orc.div_public_values(x, 1))[0]) == (1 << 63) - 1


def test_encode_negative_two_complement():
    got = orc.encode([-1.5, 2.25, -0.0000001], U64, FP)
    assert list(s64(got)) == [-(3 << 25), 9 << 24, int(-0.0000001 * (1 << 26))]
