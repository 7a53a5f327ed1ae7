"""The C-ABI library builds, loads and exports every entry point that
include/*.h declares (no device work: runs on a machine without a GPU)."""
import ctypes
import os
import re
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
PKG = os.path.join(ROOT, "vibe-model_gb300")


def declared_symbols():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(vibe_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    sys.path.insert(0, PKG)
    import build
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    assert len(declared_symbols()) >= 30


def test_reference_abi_names_present():
    """The six entry points of the reference's c_kernels.h:54-117."""
    names = declared_symbols()
    for n in ["vibe_tridiagonal_solve_f64", "vibe_weno5_reconstruct_f64", "vibe_bilinear_f64",
              "vibe_cfl_scan_f64", "vibe_neumaier_sum_f64", "vibe_advect_scalar_flux_f64"]:
        assert n in names


def test_product_imports_no_oracle():
    """Product sources never reference the oracle or the tests."""
    for d, _, files in os.walk(PKG):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                text = open(os.path.join(d, f)).read()
                assert "oracle" not in text.lower() or f == "build.py", f
