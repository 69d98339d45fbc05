"""Oracle (TEST INFRASTRUCTURE ONLY, see ``oracle/__init__.py``): the
complex128 CIE operator apply and one Gram-Schmidt pass of an Arnoldi step,
run on all host cores -- the CPU baseline of the benchmark.

The arithmetic is that of :func:`oracle.operator.apply`
(``Extreme.Cartesian/Forward/AtoA/ConvolutionOperator.cs:45-327``): ``r x``
and the forward factors into the zero-padded ``[2Nx][2Ny][3Nz]`` buffer
(``PrepareForForwardFft``), forward 2-D FFT (FFTW sign -1, unnormalised),
the per-point block contraction over all ``4 Nx Ny`` spectral points
(``ApplyGreenTensorAlongZ``: packed symmetric blocks as ``zspmv``, the
``xz``/``yz`` blocks as ``zgemv``, every point stored, as the reference
stores it), backward FFT, extraction with the backward factors and the last
step. The FFTs run in ``scipy.fft`` with ``workers`` threads (FFTW's role,
``FftWrap``), the contraction in the threaded C restatement
(``oracle/contract.c``).

``icgs_pass`` is one classical Gram-Schmidt pass of ``GmresSolver``
(``Extreme.Fgmres/Gmres.cs:297-313``): ``h = V^H w``, ``w -= V h``,
``||w||`` -- the per-step vector work of FGMRES at basis size ``j + 1``.
"""
import numpy as np

from . import ccontract
from . import operator as _op


class ThreadedOperator:
    """Prepared complex128 operator of one omega-model on the host cores."""

    def __init__(self, G, om, op_type, threads=0):
        self.G = {c: np.ascontiguousarray(v, np.complex128) for c, v in G.items()}
        self.om = om
        self.op_type = op_type
        self.threads = threads or ccontract.max_threads()
        self.r, self.fwd, self.bwd = _op.prepare(om, op_type)
        m = om.model
        self.buf = np.zeros((2 * m.nx, 2 * m.ny, 3, m.nz), np.complex128)
        self.res = np.empty_like(self.buf)
        self.n_applies = 0

    def __call__(self, x):
        self.n_applies += 1
        import scipy.fft as sfft
        m = self.om.model
        nx, ny, nz = m.nx, m.ny, m.nz
        w = self.threads
        xv = x.reshape(nx, ny, 3, nz)
        rx = self.r[:, :, None, :] * xv
        buf = self.buf
        buf[:] = 0
        buf[:nx, :ny] = self.fwd[None, None, None, :] * rx
        spec = sfft.fft2(buf, axes=(0, 1), workers=w, overwrite_x=True)
        ccontract.contract(self.G, spec, nz, w, out=self.res)
        back = sfft.ifft2(self.res, axes=(0, 1), workers=w, overwrite_x=True, norm="forward")
        y = self.bwd[None, None, None, :] * back[:nx, :ny]
        if self.op_type == _op.OP_A:
            y = (xv - y) - rx
        else:
            y = y + rx
        return y.reshape(-1)


def icgs_pass(V, j, w):
    """One classical Gram-Schmidt pass against the first j + 1 columns of V
    ([n, m] complex128): returns (h, ||w||) and updates w in place."""
    basis = V[:, :j + 1]
    h = basis.conj().T @ w
    w -= basis @ h
    return h, float(np.sqrt(np.vdot(w, w).real))
