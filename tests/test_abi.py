"""CPU tests of the C ABI boundary: the library loads, exports every declared symbol, and
validates arguments (LAPACK INFO-style negative indices) before touching the GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from paraht_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "paraht.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(paraht_\w+)\s*\(", src, flags=re.M)))


def test_library_loads_and_exports_every_declared_symbol():
    L = _lib.lib()
    names = declared_symbols()
    assert len(names) >= 15
    for name in names:
        assert hasattr(L, name), name
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)
    assert L.paraht_version() == 100
    assert L.paraht_strerror(-1002) == b"allocation failed"


def _args(n=10, lda=None, r=4, p=2, nq=2):
    A = np.zeros((max(n, 1), max(n, 1)), order="F")
    lda = lda if lda is not None else max(n, 1)
    ptr = A.ctypes.data
    return A, [n, ptr, lda, ptr, lda, ptr, lda, ptr, lda, r, p, nq, 0]


@pytest.mark.parametrize("field,value,expected", [
    (0, -1, -1),    # n
    (2, 0, -3),     # lda < n
    (4, 3, -5),     # ldb
    (6, 3, -7),     # ldq
    (8, 3, -9),     # ldz
    (9, 0, -10),    # r < 1
    (9, 65, -10),   # r > 64
    (10, 1, -11),   # p < 2
    (11, 0, -12),   # nq < 1
    (11, 5, -12),   # nq > r (outside the reference's valid domain)
])
def test_reduce_argument_errors(field, value, expected):
    A, args = _args()
    args[field] = value
    assert _lib.lib().paraht_reduce(*args) == expected


def test_null_pointer_and_stage_entry_errors():
    L = _lib.lib()
    A, args = _args()
    args[1] = None
    assert L.paraht_reduce(*args) == -2
    A, args = _args()
    # ab2rht: (n, A, lda, B, ldb, Q, ldq, Z, ldz, nb, p, time_components)
    assert L.paraht_ab2rht(*(args[:9] + [4, 1, 0])) == -11
    # rht2ht: (..., r, nq, time_components)
    assert L.paraht_rht2ht(*(args[:9] + [4, 9, 0])) == -11
    assert L.paraht_reduce(*([0] + args[1:])) == 0  # n = 0: quick return


def test_givens_entry_rejects_before_the_gpu():
    L = _lib.lib()
    A, args = _args()
    # rht2ht_givens: (n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq)
    assert L.paraht_rht2ht_givens(*(args[:9] + [4, 9])) == -11  # nq > r, outside the reference's valid domain
    assert L.paraht_rht2ht_givens(*(args[:9] + [40, 8])) == -1005  # r > 32: PARAHT_ERR_NOT_SUPPORTED
    assert L.paraht_rht2ht_givens(*([0] + args[1:9] + [4, 4])) == 0  # n = 0: quick return


def test_batch_plan_entry_points_reject_bad_handles():
    L = _lib.lib()
    assert L.paraht_batch_plan_create(None, 0, None, None, None, None, None, None, None, None, None, None, None,
                                      None, 0, None) == -16  # no place for the plan handle
    plan = C.c_void_p()
    assert L.paraht_batch_plan_create(None, 0, None, None, None, None, None, None, None, None, None, None, None,
                                      None, 0, C.byref(plan)) == -1007  # no context
    assert plan.value is None
    assert L.paraht_batch_plan_launch(None, None) == -1007
    assert L.paraht_batch_plan_destroy(None) == -1007


def test_context_entry_points_reject_bad_context():
    L = _lib.lib()
    A, args = _args()
    assert L.paraht_reduce_d(None, *args) == -1007
    assert L.paraht_ctx_destroy(None) == -1007
    buf = (C.c_double * 8)()
    assert L.paraht_ctx_phase_times(None, buf, 8) == -1007


def test_python_wrapper_raises_with_argument_index():
    import paraht_gb300 as ph

    n = 8
    A = np.zeros((n, n), order="F")
    with pytest.raises(ph.ParahtError) as e:
        ph.ab2rht_simple(n, A, n, A, n, A, n, A, n, 4, 1, False)
    assert e.value.status == -11
    with pytest.raises(TypeError):
        ph.ab2rht_simple(n, np.zeros((n, n)), n, A, n, A, n, A, n, 4, 2, False)  # C order rejected


@pytest.mark.parametrize("args,expected", [
    ((b"X", b"I", 10, 1, 10), -1),   # compq
    ((b"I", b"?", 10, 1, 10), -2),   # compz
    ((b"I", b"I", -1, 1, 10), -3),   # n
    ((b"I", b"I", 10, 0, 10), -4),   # ilo < 1
    ((b"I", b"I", 10, 5, 3), -5),    # ihi < ilo - 1
    ((b"I", b"I", 10, 1, 11), -5),   # ihi > n
])
def test_gghd3_argument_errors_before_any_gpu_work(args, expected):
    A = np.zeros((10, 10), order="F")
    p = A.ctypes.data
    rc = _lib.lib().paraht_gghd3(*args, p, 10, p, 10, p, 10, p, 10, 4, 2, 2, 0)
    assert rc == expected


def test_gghd3_leading_dimension_and_parameter_errors():
    A = np.zeros((10, 10), order="F")
    p = A.ctypes.data
    L = _lib.lib()
    assert L.paraht_gghd3(b"I", b"I", 10, 1, 10, p, 9, p, 10, p, 10, p, 10, 4, 2, 2, 0) == -7
    assert L.paraht_gghd3(b"N", b"I", 10, 1, 10, p, 10, p, 10, None, 1, p, 10, 4, 2, 2, 0) != -11  # Q unused
    assert L.paraht_gghd3(b"V", b"I", 10, 1, 10, p, 10, p, 10, p, 5, p, 10, 4, 2, 2, 0) == -11
    assert L.paraht_gghd3(b"I", b"I", 10, 1, 10, p, 10, p, 10, p, 10, p, 10, 4, 1, 2, 0) == -15
    assert L.paraht_gghd3(b"I", b"I", 10, 1, 10, p, 10, p, 10, p, 10, p, 10, 4, 2, 5, 0) == -16


def _header_arg_counts():
    """Number of parameters of every function the header declares."""
    with open(os.path.join(os.path.dirname(__file__), "..", "include", "paraht.h")) as f:
        src = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
    out = {}
    for name, params in re.findall(r"\b(paraht_\w+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        params = params.strip()
        out[name] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_fortran_interfaces_match_the_header():
    """The Fortran module (paraht_gb300/fortran/paraht_gb300.f90, not compiled here: no Fortran
    compiler in the image) binds each C entry by name with as many dummy arguments as the header's
    prototype has parameters, and only entries the library exports."""
    path = os.path.join(os.path.dirname(__file__), "..", "paraht_gb300", "fortran", "paraht_gb300.f90")
    with open(path) as f:
        src = re.sub(r"!.*", "", f.read())
    src = src.replace("&\n", " ")
    binds = re.findall(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\(\s*C\s*,\s*name\s*=\s*\"(\w+)\"\s*\)", src, flags=re.I)
    assert len(binds) >= 6
    counts = _header_arg_counts()
    L = _lib.lib()
    for fname, args, cname in binds:
        assert fname.lower() == cname.lower()
        assert cname in counts, cname
        assert len([a for a in args.split(",") if a.strip()]) == counts[cname], cname
        assert hasattr(L, cname), cname


def test_header_is_plain_c_and_links(tmp_path):
    """include/paraht.h is valid C99 on its own, and a C program built against it links with
    libparaht.so and calls it (no GPU needed for the calls made: version, strerror, argument
    rejection)."""
    import shutil
    import subprocess

    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc missing")
    _lib.lib()  # the library is built and current
    src = tmp_path / "caller.c"
    src.write_text(
        '#include "paraht.h"\n#include <stdio.h>\n'
        "int main(void) {\n"
        "  int n = 4, ld = 4, info = 0;\n"
        "  if (paraht_version() != 100) return 1;\n"
        "  if (paraht_hgeqz_eigs(-1, &n, 0, &ld, 0, &ld, 0, 0, 0, &info) != -2) return 2;\n"
        "  if (paraht_reduce_d(0, 4, 0, 4, 0, 4, 0, 4, 0, 4, 2, 2, 2, 0) != PARAHT_ERR_BAD_CTX) return 3;\n"
        '  printf("%s\\n", paraht_strerror(PARAHT_ERR_ALLOC));\n'
        "  return 0;\n}\n")
    exe = tmp_path / "caller"
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"), str(src),
                        "-o", str(exe), "-L", libdir, "-lparaht", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "allocation failed", (r.returncode, r.stdout, r.stderr)
