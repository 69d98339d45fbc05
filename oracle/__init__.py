"""CPU oracle of the reference's integral-equation forward solve.

TEST INFRASTRUCTURE ONLY. This package restates, in numpy complex128, the
algorithm of prisae/extreme (extrEMe) for the IE forward-solve hot path: the
layered-earth Green tensor (Hankel-filtered scalars, face integration,
mirroring, 2-D FFT), the CIE convolution operator, restarted FGMRES with an
inner GMRES preconditioner, and the MT plane-wave pipeline around the solve.
Every function cites the reference file:line it follows.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline
leg may import it, and only as the checker or the timed CPU baseline. The
product package (``extreme_gb300``) never imports it.

Parity pins: the scalar kernels and the Green-block contraction are checked
against the reference's own C code (``Native/Native.Matrix/*.c``) compiled
with ``oracle/Makefile`` into ``oracle/_ref/`` with a project-written
reference BLAS shim (``oracle/ref_blas_shim.c``). FFTW and OpenBLAS are not
vendored by the reference, so the FFT and BLAS-2 steps rest on their published
definitions (numpy.fft / plain loops).
"""
