"""CPU tests of the C ABI: the library loads, exports every declared symbol,
validates arguments before touching a GPU, and the C++ drop-in header
compiles and links against it with the reference's signatures."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(kmx):
    from kronmult_gb300 import _lib

    L = kmx.lib()
    names = _lib.exported_symbols()
    assert len(names) >= 19
    for name in names:
        assert hasattr(L, name), name


def test_version_and_status_strings(kmx):
    L = kmx.lib()
    assert b"sm_103a" in L.kmx_version()
    assert L.kmx_status_string(3) == b"KMX_ERR_WORKSPACE"


@pytest.mark.parametrize("d,n,expect", [(0, 4, 1), (7, 4, 1), (3, 0, 1), (3, -2, 1)])
def test_invalid_shape_rejected_without_gpu(kmx, d, n, expect):
    L = kmx.lib()
    assert L.kmx_kronmult_batched_f64(d, n, 8, 8, 8, 0, 4, None) == expect
    assert L.kmx_kronmult_xbatched_f64(d, n, 8, 0, 8, 8, 0, 4, 0, None) == expect


def test_null_pointers_and_empty_batch(kmx):
    L = kmx.lib()
    assert L.kmx_kronmult_batched_f64(3, 4, 0, 8, 8, 0, 4, None) == 2
    assert L.kmx_kronmult_pbatched_f64(3, 4, 8, 0, 8, 0, 4, None) == 2
    assert L.kmx_kronmult_xbatched_f64(3, 4, 8, 0, 0, 8, 0, 4, 0, None) == 2
    # batchCount == 0 is a no-op, even with NULL arrays
    assert L.kmx_kronmult_batched_f64(3, 4, 0, 0, 0, 0, 0, None) == 0
    assert L.kmx_kronmult_xbatched_f32(6, 4, 0, 0, 0, 0, 0, 0, 0, None) == 0


def test_lda_smaller_than_n_rejected(kmx):
    L = kmx.lib()
    assert L.kmx_kronmult_xbatched_f64(3, 4, 8, 3, 8, 8, 0, 2, 0, None) == 1
    assert L.kmx_kronmult_xbatched_f64(3, 4, 8, 4, 8, 8, 0, 0, 0, None) == 0


def test_vbatched_bad_shape_rejected(kmx):
    L = kmx.lib()
    m = (C.c_int * 3)(2, 0, 2)
    n = (C.c_int * 3)(2, 2, 2)
    assert L.kmx_kronmult_vbatched_f64(3, m, n, 8, 8, 8, 0, 0, 2, None) == 1


def test_kron_flops_matches_reference_formula(kmx):
    for d in range(1, 7):
        for n in (1, 2, 3, 4, 8):
            assert kmx.kron_flops(d, n) == 2.0 * d * n ** (d + 1)
    # rectangular: kroncommon.hpp:204-234 recursion
    assert kmx.kron_flops(2, [3, 2], [4, 5]) == 2.0 * 5 * 4 * 3 + 3 * (2.0 * 2 * 5)


def test_default_options_roundtrip(kmx):
    from kronmult_gb300 import _lib

    L = kmx.lib()
    old = _lib.Options()
    L.kmx_get_default_options(C.byref(old))
    try:
        kmx.set_default_form("plain")
        cur = _lib.Options()
        L.kmx_get_default_options(C.byref(cur))
        assert cur.form == 1 and cur.accumulate == 0
    finally:
        L.kmx_set_default_options(C.byref(old))


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_cpp_dropin_header_compiles_and_links(kmx, tmp_path):
    """A translation unit written against the reference's host API (names,
    argument order, default subbatchCount, the kgemm batched API) builds against our header and
    library without edits."""
    src = tmp_path / "user.cpp"
    src.write_text(r'''
#include "kronmult_gb300.hpp"
void user(int n, double* A, double** pA, double** pX, double** pY, double** pW, double* X,
          double* Y, double* W, float* Af, float** pAf, float** pXf, float** pYf, float** pWf,
          int batch) {
  kronmult6_batched(n, A, X, Y, W, batch);
  kronmult4_pbatched(n, A, pX, pY, pW, batch);
  kronmult6_xbatched(n, pA, n + 3, pX, pY, pW, batch);
  kronmult3_xbatched(n, pAf, n, pXf, pYf, pWf, batch, 8);
  kronmult2_vbatched<double>(2, 3, 4, 5, pA, pX, pY, W, 1 << 20, batch);
  kronmult6_vbatched<float>(1, 2, 2, 1, 1, 1, 2, 2, 3, 3, 2, 2, pAf, pXf, pYf, Af, 1 << 20, batch);
  int* ld = nullptr;
  kgemm_nn_batched(4, 1024, 4, 1.3, pA, ld, pX, ld, 1.2, pY, ld, batch);
  kgemm_nt_batched(1024, 4, 4, 1.0, pXf, ld, pAf, ld, 0.0f, pWf, ld, batch);
}
int main() { return 0; }
''')
    exe = tmp_path / "user"
    lib_dir = os.path.join(ROOT, "kronmult_gb300")
    subprocess.run(["g++", "-std=c++14", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe), f"-L{lib_dir}", "-lkronmult_gb300",
                    f"-Wl,-rpath,{lib_dir}"], check=True)
    assert exe.exists()


def test_kgemm_argument_checks_without_gpu(kmx):
    L = kmx.lib()
    for fn in (L.kmx_kgemm_nn_batched_f64, L.kmx_kgemm_nt_batched_f64,
               L.kmx_kgemm_nn_batched_f32, L.kmx_kgemm_nt_batched_f32):
        assert fn(-1, 4, 4, 1.0, 8, 8, 8, 8, 0.0, 8, 8, 2, None) == 1  # negative size
        assert fn(4, 4, 4, 1.0, 8, 8, 8, 8, 0.0, 8, 8, -1, None) == 1  # negative batch
        assert fn(4, 4, 4, 1.0, 8, 8, 8, 8, 0.0, 0, 8, 2, None) == 2   # no C array
        assert fn(4, 4, 4, 1.0, 0, 8, 8, 8, 0.0, 8, 8, 2, None) == 2   # no A array with kk > 0
        assert fn(4, 4, 4, 1.0, 8, 8, 8, 0, 0.0, 8, 8, 2, None) == 2   # no ldB array
        assert fn(4, 4, 4, 1.0, 0, 0, 0, 0, 0.0, 0, 0, 0, None) == 0   # empty batch
        assert fn(0, 4, 4, 1.0, 0, 0, 0, 0, 0.0, 0, 0, 3, None) == 0   # empty matrices


def test_xbatched_build_argument_checks_without_gpu(kmx):
    L = kmx.lib()
    for fn in (L.kmx_xbatched_build_f64, L.kmx_xbatched_build_f32):
        ok = [3, 8, 16, 4, 8, 8, 64, 8, 8, 64, 8, 8, 8, 8, 10, 0, 0, 0, 8, 8, 8, None]
        bad_d = list(ok)
        bad_d[0] = 7
        assert fn(*bad_d) == 1
        neg_stride = list(ok)
        neg_stride[2] = -1
        assert fn(*neg_stride) == 1
        null_idx = list(ok)
        null_idx[12] = 0
        assert fn(*null_idx) == 2
        sort_no_ws = list(ok)
        sort_no_ws[15] = 1
        assert fn(*sort_no_ws) == 3
        empty = list(ok)
        empty[14] = 0
        empty[1] = 0
        assert fn(*empty) == 0
    assert L.kmx_xbatched_build_workspace_bytes(1000) >= 4 * 4 * 1000


def test_vmixed_argument_checks_without_gpu(kmx):
    L = kmx.lib()
    good = (C.c_int * 13)(2, 3, 4, 1, 1, 1, 1, 4, 5, 1, 1, 1, 1)
    bad_d = (C.c_int * 13)(7, 3, 4, 1, 1, 1, 1, 4, 5, 1, 1, 1, 1)
    bad_m = (C.c_int * 13)(2, 3, 0, 1, 1, 1, 1, 4, 5, 1, 1, 1, 1)
    for fn in (L.kmx_kronmult_vmixed_f64, L.kmx_kronmult_vmixed_f32):
        assert fn(4, 8, 8, 8, 8, 8, 0, 0, good, 0, None, None) == 1   # no classes
        assert fn(4, 8, 8, 8, 8, 8, 0, 0, good, 65, None, None) == 1  # too many classes
        assert fn(4, 8, 8, 8, 8, 8, 0, 0, bad_d, 1, None, None) == 1  # d outside 1..6
        assert fn(4, 8, 8, 8, 8, 8, 0, 0, bad_m, 1, None, None) == 1  # a zero extent
        assert fn(-1, 8, 8, 8, 8, 8, 0, 0, good, 1, None, None) == 1  # negative count
        assert fn(4, 0, 8, 8, 8, 8, 0, 0, good, 1, None, None) == 2   # no class ids
        assert fn(0, 0, 0, 0, 0, 0, 0, 0, good, 1, None, None) == 0   # empty call


def test_grad_ex_and_mixed_accumulate_checks_without_gpu(kmx):
    from kronmult_gb300 import _lib

    L = kmx.lib()
    bad_form = _lib.options(7)  # no such form
    assert L.kmx_kronmult_batched_grad_f64_ex(3, 4, 8, 8, 8, 0, 8, 8, 0, 0, 2, C.byref(bad_form),
                                              None) == 1
    assert L.kmx_kronmult_batched_grad_f64_ex(0, 4, 8, 8, 8, 0, 8, 8, 0, 0, 2, None, None) == 1
    assert L.kmx_kronmult_batched_grad_f64_ex(3, 4, 0, 8, 8, 0, 8, 8, 0, 0, 2, None, None) == 2
    assert L.kmx_kronmult_batched_grad_f64_ex(3, 4, 8, 8, 8, 0, 8, 8, 0, 0, 0, None, None) == 0
    bad_acc = _lib.options("auto", 5)  # no such accumulation mode
    good = (C.c_int * 13)(2, 3, 4, 1, 1, 1, 1, 4, 5, 1, 1, 1, 1)
    assert L.kmx_kronmult_vmixed_f64(4, 8, 8, 8, 8, 8, 0, 0, good, 1, C.byref(bad_acc), None) == 1
    sq = (C.c_int * 2)(3, 4)
    assert L.kmx_kronmult_mixed_f64(4, 8, 8, 8, 8, 8, 0, 0, sq, 1, C.byref(bad_acc), None) == 1
