"""CPU-side checks of the C-ABI library: it builds, loads, exports every
symbol include/grmp.h declares, and its host-only tables agree bit for bit
with the oracle's.  No kernel is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "grmp.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b(grmp_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib(G):
    import grmp_gb300.build as b
    b.build()
    from grmp_gb300 import _lib
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    from grmp_gb300 import _lib
    names = header_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), f"{n} declared in grmp.h but not exported"
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"


def test_version(lib):
    assert lib.grmp_version() >= 10000


@pytest.mark.parametrize("dim,fe,order", [(2, 1, 0), (2, 2, 2), (2, 2, 4), (2, 2, 7), (3, 2, 2), (3, 2, 4),
                                          (3, 1, 2), (2, 1, 3), (2, 2, 8), (2, 1, 13), (3, 2, 6), (3, 1, 9),
                                          (3, 2, 5)])
def test_reference_tables_bitwise_equal_oracle(lib, O, dim, fe, order):
    """Quadrature points/weights and ForwardDiff-ordered basis derivative
    tables of the library (host code) equal the oracle's to the last bit."""
    nq = ctypes.c_int()
    nb = ctypes.c_int()
    rc = lib.grmp_reference_tables(dim, fe, order, ctypes.byref(nq), ctypes.byref(nb), None, None, None, None)
    assert rc == 0
    x = np.zeros(3 * nq.value)
    w = np.zeros(nq.value)
    v = np.zeros(nq.value * nb.value)
    d = np.zeros(nq.value * nb.value * dim)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    rc = lib.grmp_reference_tables(dim, fe, order, ctypes.byref(nq), ctypes.byref(nb), dp(x), dp(w), dp(v), dp(d))
    assert rc == 0
    ox, ow, _ = O.qrule(dim, order)
    ov, od = O.basis_tables(fe, dim, ox)
    assert np.array_equal(x.reshape(-1, 3), ox)
    assert np.array_equal(w, ow)
    assert np.array_equal(v.reshape(ov.shape), ov)
    assert np.array_equal(d.reshape(od.shape), od)


def test_no_device_is_reported_not_faked(lib):
    """Without a visible GPU the library refuses to create a context
    (GRMP_ERR_NO_DEVICE) instead of falling back to the CPU."""
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is visible")
    h = ctypes.c_void_p()
    assert lib.grmp_create_context(0, 0, ctypes.byref(h)) == 9


def test_invalid_handles_rejected(lib):
    assert lib.grmp_destroy_context(None) == 1
    assert lib.grmp_matrix_destroy(None) == 1
    assert lib.grmp_vector_fill(None, 0.0) == 1
    p = __import__("grmp_gb300")._lib.SolveParams()
    assert lib.grmp_solve_params_default(ctypes.byref(p)) == 0
    assert p.reltol == 1e-12 and p.abstol == 1e-12


def test_build_compiles_every_source():
    """Every translation unit under csrc/ is in the build list (a file left
    out would not exist on a machine that builds from source)."""
    import grmp_gb300.build as b
    csrc = os.path.join(ROOT, "gradientrobustmultiphysics.jl_gb300", "csrc")
    tus = sorted(f for f in os.listdir(csrc) if f.endswith((".cu", ".cpp")))
    assert sorted(b.SOURCES) == tus


def test_header_is_plain_c(tmp_path):
    """include/grmp.h is a C-ABI header: it compiles as strict C99 (what an
    FFI generator or a C caller sees), not only as C++."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "h.c"
    src.write_text('#include "grmp.h"\nint main(void) { return grmp_version() > 0 ? 0 : 1; }\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only",
                        "-I" + os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
