"""Oracle (test infrastructure only): the learned preconditioner's spectral
network in numpy FP64 -- forward, loss, analytic backward -- with the flat
parameter layout of ``extreme_gb300/csrc/egx_learn.cu`` (each block padded to
a multiple of 4 floats: P, bP, per layer Wm, Wp, Dz, b, then Q, bQ), so that
the GPU's BF16 gradients can be checked against it. The backward pass here is
itself checked against central finite differences (``tests/test_oracle_net.py``).

Network, per sample on the nx x ny x nz anomaly mesh (depth is a spatial
axis), channels last:
  X0[x, y, z] = [Re v_x, Re v_y, Re v_z, Im v_x, Im v_y, Im v_z] / rms(v),
                logsig[x, y, z]                           (7 channels)
  H0 = X0 P + bP                                          (7 -> width)
  H_{l+1} = act(S_l(H_l) + H_l Wp_l + Dz_l H_l + b_l), act = GELU (tanh
            form) for l < L-1, identity for the last layer, where
            S_l(H)[z] = Bx (Wm_l . (Bx^T H[z] By)) By^T: per depth, 16 x 16
            retained lateral modes in a real Fourier basis, a width x width
            channel mixing per mode (shared by every depth);
            (Dz_l H)[x, y, z] = sum_z' Dz_l[z, z'] H[x, y, z']: depth mixing
  Out = H_L Q + bQ                                        (width -> 6)
  z = v + rms(v) (Out_Re + i Out_Im)
  loss = mean_b |Out_b - T_b|^2 / |T_b|^2,  T = (z* - v)/rms(v)
"""
import numpy as np

KM = 16


def basis(n):
    """Real Fourier basis [n, 16]: cos k = 0..7, sin k = 1..8, unit columns
    (a column that vanishes on the grid stays zero)."""
    x = np.arange(n)
    cols = []
    for i in range(KM):
        c = np.cos(2 * np.pi * i * x / n) if i < 8 else np.sin(2 * np.pi * (i - 7) * x / n)
        nrm = np.linalg.norm(c)
        cols.append(c / nrm if nrm > 1e-9 else np.zeros(n))
    return np.stack(cols, 1)


def _pad4(k):
    return (k + 3) // 4 * 4


def layout(nz, width, layers):
    """{name: (offset, shape)} and the total size."""
    W = width
    out, off = {}, 0

    def take(name, shape):
        nonlocal off
        out[name] = (off, shape)
        off += _pad4(int(np.prod(shape)))
    take("P", (7, W))
    take("bP", (W,))
    for l in range(layers):
        take("Wm%d" % l, (KM * KM, W, W))
        take("Wp%d" % l, (W, W))
        take("Dz%d" % l, (nz, nz))
        take("b%d" % l, (W,))
    take("Q", (W, 6))
    take("bQ", (6,))
    return out, off


def unpack(flat, nz, width, layers):
    lay, _ = layout(nz, width, layers)
    return {k: np.asarray(flat[o:o + int(np.prod(s))], np.float64).reshape(s) for k, (o, s) in lay.items()}


def pack(grads, nz, width, layers):
    lay, size = layout(nz, width, layers)
    flat = np.zeros(size)
    for k, (o, s) in lay.items():
        flat[o:o + int(np.prod(s))] = grads[k].ravel()
    return flat


_C = np.sqrt(2 / np.pi)


def gelu(x):
    return 0.5 * x * (1 + np.tanh(_C * (x + 0.044715 * x ** 3)))


def gelu_d(x):
    th = np.tanh(_C * (x + 0.044715 * x ** 3))
    return 0.5 * (1 + th) + 0.5 * x * (1 - th ** 2) * _C * (1 + 3 * 0.044715 * x ** 2)


def _logsig(logsig, B, nx, ny, nz):
    ls = np.asarray(logsig, np.float64)
    if ls.ndim == 3:  # one model for every sample
        ls = ls[None]
    return np.stack([ls[b % ls.shape[0]] for b in range(B)])


def encode(v, logsig, nx, ny, nz):
    """v [B, N] complex (anomaly layout ((x ny + y) 3 + c) nz + z) ->
    X0 [B, nx, ny, nz, 7], rms [B], 1/rms [B]. logsig: [nx, ny, nz] or
    [models, nx, ny, nz] (sample b uses model b % models)."""
    B = v.shape[0]
    rms = np.sqrt(np.mean(np.abs(v) ** 2, axis=1))
    inv = np.where(rms > 0, 1 / np.where(rms > 0, rms, 1), 0)
    vv = (v * inv[:, None]).reshape(B, nx, ny, 3, nz).transpose(0, 1, 2, 4, 3)  # [B, x, y, z, c]
    ls = _logsig(logsig, B, nx, ny, nz)[..., None]
    return np.concatenate([vv.real, vv.imag, ls], -1), rms, inv


def target(t, inv, nx, ny, nz):
    """t [B, N] -> T [B, nx, ny, nz, 6] = [Re | Im] of t / rms(v)."""
    B = t.shape[0]
    tt = (t * inv[:, None]).reshape(B, nx, ny, 3, nz).transpose(0, 1, 2, 4, 3)
    return np.concatenate([tt.real, tt.imag], -1)


def forward(p, X0, layers, Bx, By):
    cache = {"X0": X0, "H": [], "Pre": [], "U": []}
    H = X0 @ p["P"] + p["bP"]
    for l in range(layers):
        cache["H"].append(H)
        U = np.einsum("bxyzc,xi,yj->bijzc", H, Bx, By)
        cache["U"].append(U)
        Wm = p["Wm%d" % l].reshape(KM, KM, *p["Wm%d" % l].shape[1:])
        V = np.einsum("bijzc,ijcd->bijzd", U, Wm)
        S = np.einsum("bijzd,xi,yj->bxyzd", V, Bx, By)
        Y = np.einsum("zw,bxywc->bxyzc", p["Dz%d" % l], H)
        pre = S + H @ p["Wp%d" % l] + Y + p["b%d" % l]
        cache["Pre"].append(pre)
        H = gelu(pre) if l < layers - 1 else pre
    cache["HL"] = H
    return H @ p["Q"] + p["bQ"], cache


def loss_grad(flat, v, t, logsig, nx, ny, nz, width, layers):
    """(loss, flat gradient) for residuals v and targets t (complex [B, N])."""
    p = unpack(flat, nz, width, layers)
    Bx, By = basis(nx), basis(ny)
    X0, rms, inv = encode(v, logsig, nx, ny, nz)
    B = v.shape[0]
    T = target(t, inv, nx, ny, nz)
    out, c = forward(p, X0, layers, Bx, By)
    e2 = ((out - T) ** 2).sum((1, 2, 3, 4))
    t2 = (T ** 2).sum((1, 2, 3, 4))
    loss = float(np.mean(np.where(t2 > 0, e2 / np.where(t2 > 0, t2, 1), 0)))
    dout = 2 * (out - T) / (B * np.where(t2 > 0, t2, 1))[:, None, None, None, None]
    g = {"Q": np.einsum("bxyzc,bxyzo->co", c["HL"], dout), "bQ": dout.sum((0, 1, 2, 3))}
    dH = dout @ p["Q"].T
    for l in range(layers - 1, -1, -1):
        dpre = dH * gelu_d(c["Pre"][l]) if l < layers - 1 else dH
        Hl = c["H"][l]
        g["b%d" % l] = dpre.sum((0, 1, 2, 3))
        g["Wp%d" % l] = np.einsum("bxyzc,bxyzd->cd", Hl, dpre)
        g["Dz%d" % l] = np.einsum("bxyzc,bxywc->zw", dpre, Hl)
        dHprev = dpre @ p["Wp%d" % l].T + np.einsum("zw,bxyzc->bxywc", p["Dz%d" % l], dpre)
        dV = np.einsum("bxyzd,xi,yj->bijzd", dpre, Bx, By)
        g["Wm%d" % l] = np.einsum("bijzc,bijzd->ijcd", c["U"][l], dV).reshape(KM * KM, width, width)
        Wm = p["Wm%d" % l].reshape(KM, KM, width, width)
        dU = np.einsum("bijzd,ijcd->bijzc", dV, Wm)
        dHprev = dHprev + np.einsum("bijzc,xi,yj->bxyzc", dU, Bx, By)
        dH = dHprev
    g["P"] = np.einsum("bxyzk,bxyzc->kc", c["X0"], dH)
    g["bP"] = dH.sum((0, 1, 2, 3))
    return loss, pack(g, nz, width, layers)


def apply(flat, v, logsig, nx, ny, nz, width, layers):
    """z = v + rms (Out_Re + i Out_Im) for v [B, N]."""
    p = unpack(flat, nz, width, layers)
    X0, rms, _ = encode(v, logsig, nx, ny, nz)
    out, _ = forward(p, X0, layers, basis(nx), basis(ny))
    B = v.shape[0]
    corr = (out[..., :3] + 1j * out[..., 3:]).transpose(0, 1, 2, 4, 3)  # [B, x, y, c, z]
    return v + rms[:, None] * corr.reshape(B, -1)
