"""The C-ABI library loads and exports every entry point include/tagi_gb300.h
declares; host-only entry points behave.  No GPU compute here."""
import ctypes
import os
import re
import subprocess

import numpy as np

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "tagi_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:void|int|long long|const char \*|double)\s*\*?\s*(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_dropins():
    names = declared_functions()
    for n in ("BaryTreeInterface", "modifiedGramSchmidt_singleWavefunction",
              "InterpolateBetweenTwoMeshes", "tagi_plan_create", "tagi_plan_convolve"):
        assert n in names


def test_library_exports_every_declared_symbol(native):
    lib = ctypes.CDLL(native.LIB_PATH)
    for n in declared_functions():
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_python_binding_covers_header(native):
    assert set(declared_functions()) == set(native.SIGNATURES)


def test_host_only_entry_points(native):
    L = native.lib()
    assert L.tagi_version() >= 100
    t, d, sl, tl = ctypes.c_double(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert L.tagi_beta_parameters(1.0, ctypes.byref(t), ctypes.byref(d), ctypes.byref(sl),
                                  ctypes.byref(tl)) == 0
    assert d.value == 10 and abs(t.value - 0.35) < 1e-12
    assert L.tagi_beta_parameters(0.0, ctypes.byref(t), ctypes.byref(d), ctypes.byref(sl),
                                  ctypes.byref(tl)) == 0
    assert d.value == 1
    old = L.tagi_get_precision()
    assert L.tagi_set_precision(7) == native.TAGI_ERR_ARG
    assert b"precision" in L.tagi_last_error_message()
    assert L.tagi_set_precision(0) == 0 and L.tagi_get_precision() == 0
    L.tagi_set_precision(old)
    L.tagi_clear_error()
    assert L.tagi_last_error() == 0


def test_orbital_group_choice(native):
    """Automatic orbitals per item by the measured group cost model, groups of 16 up to degree 7."""
    L = native.lib()
    og = ctypes.c_int()

    def choose(norb, degree=7, requested=0, kernel=2, precision=native.PREC_MIXED):
        native.check(L.tagi_orbitals_per_item(kernel, precision, norb, requested, degree, ctypes.byref(og)))
        return og.value

    assert choose(32) == 16 and choose(16) == 16 and choose(28) == 16
    assert choose(21) == 16 and choose(17) == 16 and choose(24) == 16 and choose(9) == 16
    assert choose(8) == 8 and choose(7) == 8 and choose(6) == 16 and choose(5) == 16 and choose(4) == 4
    assert choose(32, degree=9) == 8 and choose(5, degree=9) == 8 and choose(3) == 1
    assert choose(32, requested=8) == 8 and choose(3, requested=16) == 16
    assert choose(32, precision=native.PREC_FP64) == 1 and choose(32, kernel=1) == 1
    assert L.tagi_orbitals_per_item(2, 0, 32, 12, 7, ctypes.byref(og)) == native.TAGI_ERR_ARG
    L.tagi_clear_error()


def test_argument_errors_before_any_device_work(native):
    """Unsupported options are refused on the host with a status, never exit()."""
    L = native.lib()
    z = np.zeros(4)
    p = native.dptr(z)
    kp = np.array([1.0])
    common = [4, 4, p, p, p, p, p, p, p, p, p, p]
    # HERMITE (2) and CLUSTER_CLUSTER (3) are unsupported; kernel 5 (ATAN) too.
    for kernel, approx, ctype in ((2, 2, 1), (2, 1, 3), (5, 1, 1)):
        rc = L.tagi_BaryTreeInterface_ex(*common, kernel, 1, native.dptr(kp), 2, approx, ctype, 0.7, 7,
                                         10, 10, 1.0, -1.0, 0, 1)
        assert rc == native.TAGI_ERR_UNSUPPORTED
    bad_k = np.array([-1.0])
    rc = L.tagi_BaryTreeInterface_ex(*common, 2, 1, native.dptr(bad_k), 2, 1, 1, 0.7, 7, 10, 10, 1.0,
                                     -1.0, 0, 1)
    assert rc == native.TAGI_ERR_ARG


def declared_arities():
    """{name: parameter count} from include/tagi_gb300.h."""
    src = open(os.path.join(ROOT, "include", "tagi_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for m in re.finditer(r"^\s*(?:void|int|long long|const char \*|double)\s*\*?\s*(\w+)\s*\(([^)]*)\)\s*;",
                         src, flags=re.M | re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_binding_arities_match_header(native):
    """Every ctypes signature has as many parameters as the header declares."""
    ar = declared_arities()
    assert set(ar) == set(native.SIGNATURES)
    bad = {n: (ar[n], len(native.SIGNATURES[n][1])) for n in ar if ar[n] != len(native.SIGNATURES[n][1])}
    assert not bad, bad


def test_mesh_entry_points_refuse_bad_arguments_on_the_host(native):
    """tagi_mesh_refine / tagi_mesh_points validate before touching the device."""
    L = native.lib()
    base = np.array([[-1.0, 1.0, -1.0, 1.0, -1.0, 1.0]])
    atoms = np.array([[0.1, 0.2, 0.3]])
    n, nc, nf = ctypes.c_int(-7), ctypes.c_longlong(0), ctypes.c_longlong(0)
    null8 = [None] * 8

    def refine(numBase=1, order=3, level=-2.0, minDepth=0, maxDepth=16, h=1.0, numCells=True):
        return L.tagi_mesh_refine(native.dptr(base), numBase, native.dptr(atoms), 1, order, h, 4.0, 1.0, level,
                                  minDepth, maxDepth, *null8, 0, ctypes.byref(n) if numCells else None,
                                  ctypes.byref(nc), ctypes.byref(nf), None)

    assert refine(numCells=False) == native.TAGI_ERR_ARG
    assert refine(numBase=0) == native.TAGI_ERR_ARG and n.value == 0
    assert refine(numBase=1 << 17) == native.TAGI_ERR_ARG
    assert refine(order=16) == native.TAGI_ERR_UNSUPPORTED
    assert refine(level=-5.0) == native.TAGI_ERR_UNSUPPORTED
    assert b"children" in L.tagi_last_error_message()
    assert refine(maxDepth=17) == native.TAGI_ERR_ARG
    assert refine(minDepth=-1) == native.TAGI_ERR_ARG
    assert refine(h=float("nan")) == native.TAGI_ERR_ARG
    c = np.zeros(4)
    cp = native.dptr(c)
    dp = ctypes.POINTER(ctypes.c_double)
    u = np.zeros(4)

    def points(numCells=1, order=3, ncoarse=64, tables=(None, None), fine=False, nfine=0):
        f = [cp] * 4 if fine else [None] * 4
        return L.tagi_mesh_points(cp, cp, cp, cp, cp, cp, None, numCells, order, tables[0], tables[1],
                                  cp, cp, cp, cp, ncoarse, *f, nfine, None)

    assert points(numCells=-1) == native.TAGI_ERR_ARG
    assert points(order=16) == native.TAGI_ERR_UNSUPPORTED
    assert points(ncoarse=63) == native.TAGI_ERR_ARG
    assert points(numCells=0, ncoarse=0) == native.TAGI_OK
    assert points(fine=True) == native.TAGI_ERR_ARG          # fine arrays without ptsPerCellFine
    assert points(tables=(u.ctypes.data_as(dp), None)) == native.TAGI_ERR_ARG
    L.tagi_clear_error()
