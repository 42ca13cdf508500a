"""CPU tests of the C ABI: the library loads, exports every symbol the header
declares, and rejects bad arguments on the host before touching a device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gffm.h")


@pytest.fixture(scope="module")
def lib():
    import gffm
    gffm.build()
    return gffm.load_library()


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"GFFM_API\s+[\w\s\*]*?\b(gffm_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gffm_matmul_limb_f64" in syms and "gffm_matmul_plain_f64" in syms
    assert len(syms) >= 20


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert missing == []


def test_python_binding_covers_header():
    from gffm import _lib
    assert sorted(_lib.SIGNATURES) == declared_symbols()


def test_version_and_stripe_bound(lib):
    assert lib.gffm_version().startswith(b"gffm-gb300")
    out = ctypes.c_int64(0)
    assert lib.gffm_find_max_stripe_ops(53, 67108859, ctypes.byref(out)) == 0 and out.value == 1
    assert lib.gffm_find_max_stripe_ops(53, 65521, ctypes.byref(out)) == 0 and out.value == 2098175
    assert lib.gffm_find_max_stripe_ops(53, 33554393, ctypes.byref(out)) == 0 and out.value == 7


def test_host_side_argument_errors(lib):
    # negative size / bad modulus are refused before any device work
    st = lib.gffm_matmul_limb_f64(-1, 4, 4, None, 4, None, 4, None, 4, 7, None, 0, None)
    assert st == 1
    st = lib.gffm_matmul_limb_f64(4, 4, 4, None, 4, None, 4, None, 4, 2 ** 26, None, 0, None)
    assert st == 3 and b"2^26" in lib.gffm_last_error_string()
    st = lib.gffm_matmul_plain_f64(4, 4, 4, None, 4, None, 4, None, 4, 2 ** 30, 0, None)
    assert st == 4 and b"cannot perform a single multiplication" in lib.gffm_last_error_string()
    st = lib.gffm_matmul_plain_f32(4, 4, 4, None, 4, None, 4, None, 4, 2 ** 13, 0, None)
    assert st == 4
    st = lib.gffm_matmul_plain_f64(4, 4, 4, None, 2, None, 4, None, 4, 7, 0, None)
    assert st == 1
    ws = ctypes.c_size_t(0)
    assert lib.gffm_matmul_limb_workspace_size(8192, 8192, 8192, 67108859, ctypes.byref(ws)) == 0
    # default form at 8192^3 mod p26: Karatsuba, six digit planes per operand
    assert ws.value == 6 * (8192 + 8192) * 8192 * 2
    # the schoolbook form asked for explicitly: four digit planes per operand
    class Tuning(ctypes.Structure):
        _fields_ = [(f, ctypes.c_int32) for f in ("digit_bits", "max_ctas", "tile_n", "form")]
    assert lib.gffm_matmul_limb_tuned_workspace_size(8192, 8192, 8192, 67108859, ctypes.byref(Tuning(0, 0, 0, 1)),
                                                     ctypes.byref(ws)) == 0
    assert ws.value == 4 * (8192 + 8192) * 8192 * 2
    # below 1024 of k the default is the schoolbook
    assert lib.gffm_matmul_limb_workspace_size(1000, 1000, 1000, 67108859, ctypes.byref(ws)) == 0
    assert ws.value == 4 * (1024 + 1024) * 1024 * 2
    # an explicit Karatsuba form for a modulus it does not cover is refused
    assert lib.gffm_matmul_limb_tuned_workspace_size(64, 64, 64, 65521, ctypes.byref(Tuning(0, 0, 0, 2)),
                                                     ctypes.byref(ws)) == 10


def test_host_gemm_workspace_and_argument_errors(lib):
    """gffm_matmul_host_*: the workspace holds staging copies of A, B and C and the
    digit planes of A's and B's blocks; bad sizes and moduli are refused on the host."""
    ws = ctypes.c_size_t(0)
    assert lib.gffm_matmul_host_workspace_size(8192, 8192, 8192, 67108859, ctypes.byref(ws)) == 0
    staging = 3 * 8192 * 8192 * 8
    digits = 2 * 6 * 8192 * 8192 * 2          # 6 fp16 planes per residue (the Karatsuba form) at this modulus
    assert staging + digits <= ws.value <= staging + digits + 64 * 1024
    assert lib.gffm_matmul_host_workspace_size(0, 5, 5, 7, ctypes.byref(ws)) == 0 and ws.value == 0
    assert lib.gffm_matmul_host_f64(-1, 4, 4, None, 4, None, 4, None, 4, 7, None, 0, None) == 1
    assert lib.gffm_matmul_host_f64(4, 4, 4, None, 4, None, 4, None, 4, 2 ** 26, None, 0, None) == 3
    assert lib.gffm_matmul_host_f64(4, 4, 4, None, 3, None, 4, None, 4, 7, None, 0, None) == 1


def test_tuning_structs_match_header():
    """ctypes layouts of gffm_limb_tuning, gffm_tune_entry, gffm_batch_tuning and gffm_batch_desc."""
    import ctypes
    from gffm import autotune, batched, cumod
    assert ctypes.sizeof(cumod.LimbTuning) == 16
    assert ctypes.sizeof(autotune._Entry) == 48
    assert ctypes.sizeof(batched.Tuning) == 20
    assert ctypes.sizeof(batched._Desc) == 17 * 8


def test_limbs_for_thresholds():
    from gffm import cumod
    assert [cumod.limbs_for(N) for N in (2, 127, 128, 16255, 16256, 2080639, 2080640, 2 ** 26 - 1)] == \
        [1, 1, 2, 2, 3, 3, 4, 4]
    assert [cumod.limbs_for(N, 8) for N in (2, 255, 256, 65279, 65280, 16711423, 16711424, 2 ** 26 - 1)] == \
        [1, 1, 2, 2, 3, 3, 4, 4]


def test_fixed_primes_of_the_batched_workload():
    from gffm import batched
    assert batched.fixed_primes() == [
        1021, 1447, 2039, 2887, 4093, 5791, 8191, 11579, 16381, 23167, 32749, 46337, 65521, 92681, 131071, 185363,
        262139, 370723, 524287, 741431, 1048573, 1482907, 2097143, 2965819, 4194301, 5931641, 8388593, 11863279,
        16777213, 23726561, 33554393, 47453111]
