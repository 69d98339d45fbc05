"""Oracle (TEST INFRASTRUCTURE ONLY, see ``oracle/__init__.py``): the CIE convolution operator, numpy complex128.

Restates ``Extreme.Cartesian/Forward/AtoA/ConvolutionOperator.cs``:

* ``PrepareOperator`` (``:64-143``): ``r = (zeta - zeta0)/(zeta + conj zeta0)``
  (type A) or ``sqrt(Re zeta0)/(zeta + conj zeta0)`` (type Chi0); forward
  factors ``sqrt(Re zeta0_k)``; backward factors
  ``2 sqrt(Re zeta0_k) / (dz_k * 4 Nx Ny)``;
* ``Apply`` (``:162-327``): ``rx = r*x`` -> scale and zero-pad into the
  ``[2Nx][2Ny][3Nz]`` buffer -> forward FFT (FFTW sign -1, batch 3Nz
  interleaved) -> per-spectral-point block contraction -> backward FFT
  (sign +1, unnormalised) -> extract and scale -> last step
  (``y = x - y - rx`` for A, ``y = y + rx`` for Chi0).

Vector layout (``Core/AnomalyCurrent.cs``, ``Core/LayerAccessor.cs:45-47``):
index ``((i*Ny + j)*3 + c)*Nz + k``.
"""
import numpy as np

OP_A = 0
OP_CHI0 = 1


def unpack_symm(packed, nz):
    """Packed upper storage ``[rc + tr*(tr+1)/2]`` (``zspmv`` 'U',
    ``Model/TranceiverUtils.cs:65-74``) -> full symmetric [.., nz, nz]."""
    p = packed.shape[:-1]
    full = np.empty(p + (nz, nz), packed.dtype)
    idx = 0
    for tr in range(nz):
        for rc in range(tr + 1):
            full[..., rc, tr] = packed[..., idx]
            full[..., tr, rc] = packed[..., idx]
            idx += 1
    return full


def prepare(om, op_type):
    """(r[nx,ny,nz], fwd[nz], bwd[nz])."""
    m = om.model
    z0 = om.zeta0
    conj = np.conj(z0)
    sq = np.sqrt(z0.real).astype(np.complex128)
    if op_type == OP_CHI0:
        r = sq[None, None, :] / (om.zeta + conj[None, None, :])
    else:
        r = (om.zeta - z0[None, None, :]) / (om.zeta + conj[None, None, :])
    fwd = np.sqrt(z0.real).astype(np.complex128)
    norm = 1.0 / (float(m.nx) * float(m.ny) * 4)
    bwd = (2 * np.sqrt(z0.real)) / m.layer_thickness * norm
    return r, fwd, bwd.astype(np.complex128)


def unpack_blocks(G, nz):
    """The six components of G as full [.., nz, nz] blocks (xx, xy, yy, zz
    unpacked from the packed upper storage; xz, yz reshaped)."""
    return (unpack_symm(G["xx"], nz), unpack_symm(G["xy"], nz), unpack_symm(G["yy"], nz),
            unpack_symm(G["zz"], nz), G["xz"].reshape(G["xz"].shape[:-1] + (nz, nz)),
            G["yz"].reshape(G["yz"].shape[:-1] + (nz, nz)))


def contract(G, buf, nz, blocks=None):
    """``ApplyGreenTensorAlongZ`` (``ConvolutionOperator.cs:274-327``) on
    buf[..., 3, nz]; G in the reference layout c -> [.., block] (or its
    ``unpack_blocks`` in ``blocks``)."""
    sxx, sxy, syy, szz, axz, ayz = blocks if blocks is not None else unpack_blocks(G, nz)
    x = buf[..., 0, :, None]
    y = buf[..., 1, :, None]
    z = buf[..., 2, :, None]
    out = np.empty_like(buf)
    out[..., 0, :] = (sxx @ x + sxy @ y + axz @ z)[..., 0]
    out[..., 1, :] = (sxy @ x + syy @ y + ayz @ z)[..., 0]
    axz_t = np.swapaxes(axz, -1, -2)
    ayz_t = np.swapaxes(ayz, -1, -2)
    out[..., 2, :] = (-(axz_t @ x) - (ayz_t @ y) + szz @ z)[..., 0]
    return out


def apply(G, om, x, op_type, prepared=None, blocks=None, chunk=None):
    """One operator application ``y = K x`` on a flat vector. ``chunk``: the
    contraction runs over that many rows of the first spectral axis at a
    time (bounds the unpacked blocks' memory at large sizes; same values)."""
    m = om.model
    nx, ny, nz = m.nx, m.ny, m.nz
    r, fwd, bwd = prepared if prepared is not None else prepare(om, op_type)
    xv = x.reshape(nx, ny, 3, nz)
    rx = r[:, :, None, :] * xv
    buf = np.zeros((2 * nx, 2 * ny, 3, nz), np.complex128)
    buf[:nx, :ny] = fwd[None, None, None, :] * rx
    spec = np.fft.fft2(buf, axes=(0, 1))
    if chunk is None or blocks is not None:
        res = contract(G, spec, nz, blocks)
    else:
        res = np.empty_like(spec)
        for i0 in range(0, 2 * nx, chunk):
            sl = slice(i0, min(2 * nx, i0 + chunk))
            res[sl] = contract({c: v[sl] for c, v in G.items()}, spec[sl], nz)
    back = np.fft.ifft2(res, axes=(0, 1)) * (4 * nx * ny)
    y = bwd[None, None, None, :] * back[:nx, :ny]
    if op_type == OP_A:
        y = (xv - y) - rx
    else:
        y = y + rx
    return y.reshape(-1)


class Operator:
    """Prepared operator (``PrepareOperator`` once, ``Apply`` many times)."""

    def __init__(self, G, om, op_type):
        self.G, self.om, self.op_type = G, om, op_type
        self.prepared = prepare(om, op_type)
        self.blocks = unpack_blocks(G, om.model.nz)  # unpacked once, the same values every apply
        self.n_applies = 0

    def __call__(self, x):
        self.n_applies += 1
        return apply(self.G, self.om, x, self.op_type, self.prepared, self.blocks)
