"""CPU: the C-ABI library loads and exports every entry point include/egx.h
declares (no compute calls here: there may be no GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(egx_\w+)\s*\(", src))
    return names


def test_header_declares_expected_surface():
    names = declared_symbols()
    for required in ("egx_green_build", "egx_op_prepare", "egx_op_apply", "egx_fft2d", "egx_fgmres_solve",
                     "egx_set_precond"):
        assert required in names


def test_library_exports_every_declared_symbol():
    from extreme_gb300 import egx
    lib = ctypes.CDLL(egx.LIB_PATH)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(egx.EXPORTS) <= declared_symbols()


def test_library_is_sm103a_only():
    """The fatbin is built for sm_103a alone (build flags, not binary inspection)."""
    from extreme_gb300 import _build
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
