"""ctypes access to the reference's own native math, compiled by
``oracle/Makefile`` into ``oracle/_ref/libntv_math_ref.so``.

TEST INFRASTRUCTURE ONLY: known-answer checks of the oracle restatement
against the reference's C code (``Native/Native.Matrix/*.c``). The library is
built from the reference sources (it is not part of this repository), so the
helpers here return ``None`` from :func:`load` when it has not been built.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libntv_math_ref.so")


class NativeEnvelop(C.Structure):
    """``NativeEnvelop`` (``Native/Native.Matrix/green_scalar.c:13-28``)."""
    _fields_ = [("n", C.c_int), ("r", C.c_int), ("s", C.c_int), ("t", C.c_int), ("b", C.c_int),
                ("dt", C.c_double), ("db1", C.c_double), ("r1", C.c_double), ("r2", C.c_double),
                ("s1", C.c_double), ("s2", C.c_double)]


class Complex16(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


_lib = None


def load():
    global _lib
    if _lib is None and os.path.exists(LIB_PATH):
        lib = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        lib.CalcEta.argtypes = [C.c_int, vp, vp, Complex16]
        lib.CalcExp.argtypes = [C.c_int, vp, C.c_double, vp]
        lib.CalcDotProduct.argtypes = [vp, vp, C.c_int, C.c_int]
        lib.CalcDotProduct.restype = Complex16
        for name in ("CalculateT", "CalculateR", "CalculateCTop", "CalculateCBot",
                     "CalculateDTop", "CalculateDBot"):
            getattr(lib, name).argtypes = [C.POINTER(NativeEnvelop), vp, vp]
        lib.FullZgemv.argtypes = [C.c_int, C.c_int] + [vp] * 8
        lib.Zrotg.argtypes = [Complex16, Complex16, vp, vp]
        lib.Zrot.argtypes = [C.c_int, vp, C.c_int, vp, C.c_int, C.c_double, Complex16]
        lib.SimplifiedZtrsv.argtypes = [C.c_int, vp, C.c_int, vp]
        lib.CalculateDotProductConjugatedLeft.argtypes = [C.c_long, vp, vp, vp]
        lib.ZgemvNotTrans.argtypes = [C.c_int, C.c_int, Complex16, vp, vp, Complex16, vp]
        lib.Dznrm2.argtypes = [C.c_int, vp]
        lib.Dznrm2.restype = C.c_double
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def calc_eta(lambdas, value):
    lib = load()
    lam = np.ascontiguousarray(lambdas, np.float64)
    out = np.empty(lam.size, np.complex128)
    lib.CalcEta(lam.size, _p(lam), _p(out), Complex16(value.real, value.imag))
    return out


def calc_exp(eta, factor):
    lib = load()
    e = np.ascontiguousarray(eta, np.complex128)
    out = np.empty_like(e)
    lib.CalcExp(e.size, _p(e), float(factor), _p(out))
    return out


def exp_sum(name, eta, r, s, t, b, dt, db1, r1, r2, s1, s2):
    """One of CalculateT/R/CTop/CBot/DTop/DBot over eta[L, n]."""
    lib = load()
    e = np.ascontiguousarray(eta, np.complex128)
    n = e.shape[1]
    ne = NativeEnvelop(n, r, s, t, b, dt, db1, r1, r2, s1, s2)
    out = np.empty(n, np.complex128)
    getattr(lib, name)(C.byref(ne), _p(e), _p(out))
    return out


def hankel_dot(rev_hank, fk, shift):
    lib = load()
    h = np.ascontiguousarray(rev_hank, np.float64)
    f = np.ascontiguousarray(fk, np.complex128)
    r = lib.CalcDotProduct(_p(h), _p(f), h.size, shift)
    return complex(r.re, r.im)


def full_zgemv(nz, xx, xy, xz, yy, yz, zz, src):
    """Reference block contraction over ``length`` spectral points
    (``Native/Native.Matrix/full_zgemv.c:93-150``)."""
    lib = load()
    arrs = [np.ascontiguousarray(a, np.complex128) for a in (xx, xy, xz, yy, yz, zz, src)]
    length = arrs[-1].size // (3 * nz)
    dst = np.zeros_like(arrs[-1])
    lib.FullZgemv(nz, length, *[_p(a) for a in arrs], _p(dst))
    return dst


def zrotg(a, b):
    lib = load()
    c = C.c_double()
    s = Complex16()
    lib.Zrotg(Complex16(a.real, a.imag), Complex16(b.real, b.imag), C.byref(c), C.byref(s))
    return c.value, complex(s.re, s.im)
