"""The C ABI on the CPU: libpiranha_gb300.so loads, exports every function
that include/piranha_gb300.h declares, agrees with the Python mirror on
names and constants, and answers a missing context with a status code.
No call here reaches a kernel.
"""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "piranha_gb300.h")


def _header_text():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return re.sub(r"//[^\n]*", " ", src)


def declared_functions():
    names = re.findall(r"\b(pg_\w+)\s*\(", _header_text())
    # drop names that appear only as arguments of other declarations (none expected)
    return sorted(set(names))


def declared_constants():
    return {m.group(1): m.group(2) for m in re.finditer(r"#define\s+(PG_\w+)\s+(\S.*)", _header_text())}


@pytest.fixture(scope="module")
def pg():
    import piranha_gb300 as pg

    pg.lib()  # builds the library first when it is missing or stale
    return pg


def test_header_declares_the_surface():
    names = declared_functions()
    for must in ("pg_ctx_create", "pg_rss_matmul_u64", "pg_rss_conv_u64", "pg_rss_relu_u64_u8",
                 "pg_rss_maxpool_u64_u8", "pg_rss_divide_public_u64", "pg_gemm_u64", "pg_net_forward_host"):
        assert must in names
    assert len(names) >= 55


def test_library_exports_every_declared_function(pg):
    lib = ctypes.CDLL(pg.library_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared in the header but not exported: {missing}"


def test_python_mirror_binds_only_declared_functions(pg):
    lib = pg.lib()
    declared = set(declared_functions())
    bound = {n for n in dir(lib) if n.startswith("pg_")} | {
        n for n in vars(lib) if n.startswith("pg_")}
    assert bound <= declared, sorted(bound - declared)


def test_constants_match_python_mirror(pg):
    consts = declared_constants()
    assert int(consts["PG_OK"]) == 0
    assert int(consts["PG_FORM_U64"]) == pg.FORM_U64
    assert int(consts["PG_FORM_LIMB_TC"]) == pg.FORM_LIMB_TC
    for name in ("OP_ADD", "OP_SUB", "OP_MUL", "OP_XOR", "OP_AND", "OP_SHR", "OP_SHL", "RHS_SCALAR", "RHS_PUBLIC",
                 "RHS_SHARES"):
        assert int(consts["PG_" + name]) == getattr(pg, name)
    for name in ("PG_CONV_FPROP", "PG_CONV_DGRAD", "PG_CONV_WGRAD"):
        assert int(consts[name]) in (0, 1, 2)


def test_null_context_is_an_error_status(pg):
    lib = pg.lib()
    assert lib.pg_sync(None) == 1
    assert lib.pg_comm_reset(None) == 1
    assert lib.pg_ctx_get_form(None) == -1
    assert lib.pg_kernel_launches(None) == 0
    assert lib.pg_last_error(None) == b"null context"
    P6 = ctypes.c_void_p * 6
    z = P6()
    assert lib.pg_rss_matmul_u64(None, z, z, z, 1, 1, 16, 1, 1, 1, 0) == 1
    f = lib.pg_rss_matmul_u64_noalloc
    f.argtypes = [ctypes.c_void_p, P6, P6, P6] + [ctypes.c_int] * 7
    assert f(None, z, z, z, 1, 1, 16, 1, 1, 1, 0) == 1


def test_context_without_device_fails_cleanly(pg):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    out = ctypes.c_void_p(1)
    st = pg.lib().pg_ctx_create(ctypes.byref(out), 0)
    assert st == 3  # PG_ERR_CUDA
    assert not out.value
