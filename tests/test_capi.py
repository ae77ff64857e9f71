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
