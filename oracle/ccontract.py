"""ctypes access to the oracle's C restatement of the Green block contraction
(``oracle/contract.c``, built by ``make -C oracle port`` into
``oracle/_lib/liboracle.so``).

TEST INFRASTRUCTURE ONLY: the multi-threaded CPU baseline of the benchmark
and a cross-check of :func:`oracle.operator.contract`. Follows
``Extreme.Cartesian/Forward/AtoA/ConvolutionOperator.cs:274-327``.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liboracle.so")
_lib = None


def load():
    """Load the library, building it with gcc first if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            subprocess.run(["make", "-s", "-C", _HERE, "port"], check=True)
        lib = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        lib.oracle_contract.argtypes = [C.c_long, C.c_int] + [vp] * 8 + [C.c_int]
        lib.oracle_contract.restype = None
        lib.oracle_max_threads.restype = C.c_int
        _lib = lib
    return _lib


def max_threads():
    return int(load().oracle_max_threads())


def contract(G, buf, nz, nthreads=0, out=None):
    """Same contract as :func:`oracle.operator.contract`: G maps component ->
    [..., block] complex128 (packed symmetric for xx/xy/yy/zz, [nz*nz] for
    xz/yz), buf is [..., 3, nz]; returns a new array like buf (or fills
    ``out``, a contiguous complex128 array of buf's shape)."""
    lib = load()
    lead = buf.shape[:-2]
    npts = int(np.prod(lead)) if lead else 1
    comps = [np.ascontiguousarray(G[c], np.complex128) for c in ("xx", "xy", "yy", "zz", "xz", "yz")]
    x = np.ascontiguousarray(buf, np.complex128)
    if out is None:
        out = np.empty_like(x)
    assert out.shape == x.shape and out.dtype == np.complex128 and out.flags.c_contiguous
    lib.oracle_contract(npts, nz, *[c.ctypes.data for c in comps], x.ctypes.data, out.ctypes.data, nthreads)
    return out
