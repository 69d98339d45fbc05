"""ctypes binding of ``libegx.so`` (the C ABI declared in ``include/egx.h``).

This is the Python face of the drop-in boundary: the same entry points a C#
P/Invoke layer binds. The library must be built
(``python -m extreme_gb300._build``); there is no fallback when it is missing.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libegx.so")

OK = 0
ERR_INVALID, ERR_OOM, ERR_CUDA, ERR_NOT_CONVERGED, ERR_TIMEOUT, ERR_STATE, ERR_MODEL = range(1, 8)
OP_A, OP_CHI0 = 0, 1
HOST, DEVICE = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
PRECOND_GMRES, PRECOND_CALLBACK, PRECOND_NONE, PRECOND_LEARNED = 0, 1, 2, 3

# Every symbol the header declares (checked by the ABI test).
EXPORTS = [
    "egx_create", "egx_destroy", "egx_last_error", "egx_version", "egx_device_allocations", "egx_set_stream",
    "egx_launch_count", "egx_set_graphs", "egx_graph_stats", "egx_tune_apply", "egx_apply_variant",
    "egx_green_build", "egx_green_upload", "egx_green_download", "egx_green_free",
    "egx_op_prepare", "egx_op_apply", "egx_op_apply_ds", "egx_op_apply_c64", "egx_fft2d",
    "egx_fgmres_solve", "egx_mixed_solve", "egx_set_precond", "egx_dot_products", "egx_dot_products_static",
    "egx_normal_field", "egx_plane_wave", "egx_solve_sources", "egx_profile", "egx_profile_kinds",
    "egx_profile_read",
    "egx_level_fields", "egx_level_cache", "egx_set_level_precision", "egx_mt_responses", "egx_mt_responses_dev",
    "egx_wait_selftest",
    "egx_net_create", "egx_net_free", "egx_net_size", "egx_net_params", "egx_net_set_model", "egx_net_set_models", "egx_net_loss_grad",
    "egx_net_adam", "egx_net_use_tcgen05", "egx_net_apply", "egx_learned_stats", "egx_learned_inject_nonfinite",
]

# kernel kinds of egx_profile_read
K_FWD_Y, K_FWD_X, K_CONTRACT, K_BWD_X, K_BWD_Y, K_GS_DOTS, K_GS_UPDATE = range(7)
K_C64 = 8
K_GREEN_LAYERS, K_GREEN_KERNELS, K_GREEN_HANKEL, K_GREEN_CELLS, K_GREEN_FFT = range(16, 21)
KERNEL_NAMES = {K_FWD_Y: "fwd_y", K_FWD_X: "fwd_x", K_CONTRACT: "contract", K_BWD_X: "bwd_x", K_BWD_Y: "bwd_y",
                K_GS_DOTS: "gs_dots", K_GS_UPDATE: "gs_update", K_GREEN_LAYERS: "green_layers",
                K_GREEN_KERNELS: "green_kernels", K_GREEN_HANKEL: "green_hankel", K_GREEN_CELLS: "green_cells",
                K_GREEN_FFT: "green_fft"}


class EgxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("egx error %d: %s" % (code, msg))
        self.code = code


class Model(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("dx", C.c_double), ("dy", C.c_double),
                ("layer_depth", C.POINTER(C.c_double)), ("layer_thickness", C.POINTER(C.c_double)),
                ("n_bg", C.c_int), ("zero_air_level", C.c_double),
                ("bg_thickness", C.POINTER(C.c_double)), ("bg_sigma", C.POINTER(C.c_double))]


class GmresParams(C.Structure):
    _fields_ = [("m_out", C.c_int), ("m_in", C.c_int), ("tol", C.c_double), ("max_restarts", C.c_int),
                ("precond", C.c_int), ("check_true", C.c_int)]


class MixedParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_outer", C.c_int), ("m_out", C.c_int), ("m_in", C.c_int),
                ("inner_tol", C.c_double), ("inner_restarts", C.c_int), ("batch", C.c_int)]


class SourceParams(C.Structure):
    _fields_ = [("precision", C.c_int), ("fgmres", GmresParams), ("mixed", MixedParams)]


class Result(C.Structure):
    _fields_ = [("converged", C.c_int), ("iterations", C.c_int), ("arnoldi_be", C.c_double),
                ("true_be", C.c_double), ("n_applies", C.c_int), ("n_refinements", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


PRECOND_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_long, C.c_int)

_lib = None


def load(path=None):
    """Load libegx.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libegx.so is not built (%s); run `python -m extreme_gb300._build`" % path)
    lib = C.CDLL(path)
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    lib.egx_create.argtypes = [i, C.POINTER(vp)]
    lib.egx_destroy.argtypes = [vp]
    lib.egx_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    lib.egx_set_stream.argtypes = [vp, vp]
    lib.egx_launch_count.argtypes = [vp]
    lib.egx_launch_count.restype = C.c_long
    lib.egx_set_graphs.argtypes = [vp, i]
    lib.egx_tune_apply.argtypes = [vp, i, i, vp]
    lib.egx_apply_variant.argtypes = [vp, i, i]
    lib.egx_graph_stats.argtypes = [vp, C.POINTER(C.c_long), C.POINTER(C.c_long)]
    lib.egx_device_allocations.argtypes = []
    lib.egx_device_allocations.restype = C.c_long
    lib.egx_green_build.argtypes = [vp, C.POINTER(Model), d, i, i, C.POINTER(vp)]
    lib.egx_green_upload.argtypes = [vp, i, i, i, C.POINTER(vp), i, C.POINTER(vp)]
    lib.egx_green_download.argtypes = [vp, vp, C.POINTER(vp)]
    lib.egx_green_free.argtypes = [vp, vp]
    lib.egx_op_prepare.argtypes = [vp, vp, vp, vp, vp, i]
    lib.egx_op_apply.argtypes = [vp, vp, vp, i, i]
    lib.egx_op_apply_c64.argtypes = [vp, vp, vp, i, i]
    lib.egx_op_apply_ds.argtypes = [vp, vp, vp, i, i]
    lib.egx_fft2d.argtypes = [vp, vp, i, i, i, i, i]
    lib.egx_fgmres_solve.argtypes = [vp, vp, vp, C.POINTER(GmresParams), C.POINTER(Result), i]
    lib.egx_mixed_solve.argtypes = [vp, vp, vp, C.POINTER(MixedParams), C.POINTER(Result), i]
    lib.egx_set_precond.argtypes = [vp, i, PRECOND_FN, vp]
    lib.egx_dot_products.argtypes = [vp, vp, i, vp, C.c_long, vp, i]
    lib.egx_dot_products_static.argtypes = [vp, vp, i, vp, C.c_long, vp]
    lib.egx_normal_field.argtypes = [C.POINTER(Model), d, vp]
    lib.egx_plane_wave.argtypes = [C.POINTER(Model), d, d, vp, vp]
    lib.egx_solve_sources.argtypes = [vp, vp, vp, vp, vp, vp, vp, i, C.POINTER(SourceParams), vp, vp,
                                      C.POINTER(Result), i]
    lib.egx_level_fields.argtypes = [vp, C.POINTER(Model), d, i, d, d, d, vp, i, vp, vp, i]
    lib.egx_mt_responses.argtypes = [vp, vp, vp, vp, C.c_long, d, vp, vp, vp]
    lib.egx_mt_responses_dev.argtypes = [vp, vp, vp, C.c_long, d, vp, vp, vp, vp, vp]
    lib.egx_level_cache.argtypes = [vp, i, C.POINTER(C.c_long), C.POINTER(C.c_long)]
    lib.egx_set_level_precision.argtypes = [vp, i]
    lib.egx_wait_selftest.argtypes = [vp, d]
    lib.egx_net_create.argtypes = [vp, i, i, i, i, i, C.c_uint, C.POINTER(vp)]
    lib.egx_net_free.argtypes = [vp, vp]
    lib.egx_net_size.argtypes = [vp]
    lib.egx_net_size.restype = C.c_long
    lib.egx_net_params.argtypes = [vp, vp, vp, i]
    lib.egx_net_set_model.argtypes = [vp, vp, vp]
    lib.egx_net_set_models.argtypes = [vp, vp, vp, i]
    lib.egx_net_loss_grad.argtypes = [vp, vp, vp, vp, i, C.POINTER(C.c_float), vp, i]
    lib.egx_net_adam.argtypes = [vp, vp, C.c_float]
    lib.egx_net_use_tcgen05.argtypes = [vp, vp, i]
    lib.egx_net_apply.argtypes = [vp, vp, vp, vp, i, i]
    lib.egx_learned_stats.argtypes = [vp, C.POINTER(C.c_long), C.POINTER(C.c_long)]
    lib.egx_learned_inject_nonfinite.argtypes = [vp, i]
    lib.egx_profile.argtypes = [vp, i]
    lib.egx_profile_kinds.argtypes = [vp, C.c_uint]
    lib.egx_profile_read.argtypes = [vp, i, C.POINTER(C.c_long), C.POINTER(C.c_double)]
    _lib = lib
    return lib


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


def _c128(a):
    a = np.ascontiguousarray(a, np.complex128)
    return a


GREEN_COMPONENTS = ("xx", "xy", "yy", "zz", "xz", "yz")


class Context:
    """An ``egx_ctx``: one device, one stream."""

    def __init__(self, device=0):
        self.lib = load()
        h = C.c_void_p()
        self._check(self.lib.egx_create(device, C.byref(h)), None)
        self.h = h
        self._cb = None

    def _check(self, rc, h="self"):
        if rc != OK:
            msg = ""
            hh = self.h if h == "self" else h
            if hh is not None:
                buf = C.create_string_buffer(1024)
                self.lib.egx_last_error(hh, buf, 1024)
                msg = buf.value.decode()
            raise EgxError(rc, msg)

    def close(self):
        if getattr(self, "h", None) is not None:
            self.lib.egx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def launch_count(self):
        return int(self.lib.egx_launch_count(self.h))

    def set_graphs(self, enable):
        """Capture the inner GMRES cycle as a CUDA graph and replay it (egx_set_graphs)."""
        self._check(self.lib.egx_set_graphs(self.h, int(bool(enable))))

    def tune_apply(self, nrhs=2, reps=5):
        """egx_tune_apply: times every (FFT tile, contraction kernel) variant
        of the complex64 apply; keeps the fastest. Returns (tile, variant,
        {(tile, variant): ms})."""
        ms = np.zeros(9)
        self._check(self.lib.egx_tune_apply(self.h, nrhs, reps, _ptr(ms)))
        table = {(t, v): float(ms[3 * t + v]) for t in range(3) for v in range(3) if ms[3 * t + v] >= 0}
        best = min(table, key=table.get)
        return best[0], best[1], table

    def apply_variant(self, fft_tile=0, contract_variant=0):
        self._check(self.lib.egx_apply_variant(self.h, fft_tile, contract_variant))

    def graph_stats(self):
        r, nn = C.c_long(), C.c_long()
        self._check(self.lib.egx_graph_stats(self.h, C.byref(r), C.byref(nn)))
        return r.value, nn.value

    @staticmethod
    def device_allocations():
        """Device allocations (cudaMalloc calls) the library has made in this process."""
        return int(load().egx_device_allocations())

    def set_stream(self, stream_handle):
        self._check(self.lib.egx_set_stream(self.h, C.c_void_p(stream_handle)))

    # -- Green tensor -----------------------------------------------------
    def green_upload(self, G, nx, ny, nz, precision=PREC_FP64):
        """G: dict c -> [2nx, 2ny, block] complex128 in the reference layout."""
        arrs = [_c128(G[c]) for c in GREEN_COMPONENTS]
        ptrs = (C.c_void_p * 6)(*[a.ctypes.data for a in arrs])
        h = C.c_void_p()
        self._check(self.lib.egx_green_upload(self.h, nx, ny, nz, ptrs, precision, C.byref(h)))
        return GreenTensor(self, h, nx, ny, nz)

    def green_build(self, model, omega, n_hankels=10, precision=PREC_FP64):
        m = model_struct(model)
        h = C.c_void_p()
        self._check(self.lib.egx_green_build(self.h, C.byref(m.s), float(omega), int(n_hankels), precision,
                                             C.byref(h)))
        return GreenTensor(self, h, model.nx, model.ny, model.nz)

    # -- operator ---------------------------------------------------------
    def op_prepare(self, green, zeta, zeta0, dz, op_type):
        z = _c128(zeta)
        z0 = _c128(zeta0)
        dz = np.ascontiguousarray(dz, np.float64)
        self._check(self.lib.egx_op_prepare(self.h, green.h, _ptr(z), _ptr(z0), _ptr(dz), op_type))

    def op_apply(self, x, nrhs=1, out=None):
        """Host arrays (complex128)."""
        x = _c128(x)
        y = np.empty_like(x) if out is None else out
        self._check(self.lib.egx_op_apply(self.h, _ptr(x), _ptr(y), nrhs, HOST))
        return y

    def op_apply_dev(self, x_ptr, y_ptr, nrhs=1):
        self._check(self.lib.egx_op_apply(self.h, C.c_void_p(x_ptr), C.c_void_p(y_ptr), nrhs, DEVICE))

    def op_apply_ds(self, x, nrhs=1):
        """Host arrays (complex128); the contraction in double-FP32."""
        x = _c128(x)
        y = np.empty_like(x)
        self._check(self.lib.egx_op_apply_ds(self.h, _ptr(x), _ptr(y), nrhs, HOST))
        return y

    def op_apply_c64(self, x, nrhs=1):
        x = np.ascontiguousarray(x, np.complex64)
        y = np.empty_like(x)
        self._check(self.lib.egx_op_apply_c64(self.h, _ptr(x), _ptr(y), nrhs, HOST))
        return y

    def fft2d(self, buf, sign):
        """In-place on a host array [n0, n1, howmany] complex128."""
        assert buf.dtype == np.complex128 and buf.flags.c_contiguous and buf.ndim == 3
        n0, n1, hm = buf.shape
        self._check(self.lib.egx_fft2d(self.h, _ptr(buf), n0, n1, hm, sign, HOST))
        return buf

    # -- solver -----------------------------------------------------------
    def fgmres_solve(self, b, x0, m_out=20, m_in=10, tol=1e-8, max_restarts=100, precond=PRECOND_GMRES,
                     check_true=True, raise_on_nonconv=False):
        b = _c128(b)
        x = _c128(x0).copy()
        p = GmresParams(m_out, m_in, tol, max_restarts, precond, int(check_true))
        r = Result()
        rc = self.lib.egx_fgmres_solve(self.h, _ptr(b), _ptr(x), C.byref(p), C.byref(r), HOST)
        if rc != OK and not (rc == ERR_NOT_CONVERGED and not raise_on_nonconv):
            self._check(rc)
        return x, r.as_dict()

    def fgmres_solve_dev(self, b_ptr, x_ptr, m_out=20, m_in=10, tol=1e-8, max_restarts=100,
                         precond=PRECOND_GMRES, check_true=True):
        p = GmresParams(m_out, m_in, tol, max_restarts, precond, int(check_true))
        r = Result()
        rc = self.lib.egx_fgmres_solve(self.h, C.c_void_p(b_ptr), C.c_void_p(x_ptr), C.byref(p), C.byref(r), DEVICE)
        if rc not in (OK, ERR_NOT_CONVERGED):
            self._check(rc)
        return r.as_dict()

    def mixed_solve(self, b, x0, tol=1e-6, max_outer=10, m_out=30, m_in=10, inner_tol=5e-7, inner_restarts=20):
        b = _c128(b)
        x = _c128(x0).copy()
        p = MixedParams(tol, max_outer, m_out, m_in, inner_tol, inner_restarts, 0)
        r = Result()
        rc = self.lib.egx_mixed_solve(self.h, _ptr(b), _ptr(x), C.byref(p), C.byref(r), HOST)
        if rc not in (OK, ERR_NOT_CONVERGED):
            self._check(rc)
        return x, r.as_dict()

    def mixed_solve_dev(self, b_ptr, x_ptr, tol=1e-6, max_outer=10, m_out=30, m_in=10, inner_tol=5e-7,
                        inner_restarts=20):
        p = MixedParams(tol, max_outer, m_out, m_in, inner_tol, inner_restarts, 0)
        r = Result()
        rc = self.lib.egx_mixed_solve(self.h, C.c_void_p(b_ptr), C.c_void_p(x_ptr), C.byref(p), C.byref(r), DEVICE)
        if rc not in (OK, ERR_NOT_CONVERGED):
            self._check(rc)
        return r.as_dict()

    def dot_products(self, V, w):
        """DotProductRequest: conj(V[:, k]) . w for every column of V [n, ncols]."""
        Vt = np.ascontiguousarray(np.asarray(V, np.complex128).T)
        w = _c128(w)
        out = np.empty(Vt.shape[0], np.complex128)
        self._check(self.lib.egx_dot_products(self.h, _ptr(Vt), Vt.shape[0], _ptr(w), w.size, _ptr(out), HOST))
        return out

    def dot_products_static(self, V_ptr, ncols, w_ptr, n, out_ptr):
        """egx_dot_products_static on device pointers: V holds ncols vectors
        of n complex128 one after another, out receives ncols complex128.
        Allocates no device memory (a fixed static scratch, <= 64 columns)."""
        self._check(self.lib.egx_dot_products_static(self.h, C.c_void_p(V_ptr), ncols, C.c_void_p(w_ptr), n,
                                                     C.c_void_p(out_ptr)))

    def solve_sources(self, green, zeta, zeta0, dz, e0, pols, precision=PREC_FP64, fgmres=None, mixed=None,
                      want_chi=False, where=HOST, dev_ptrs=None, out=None):
        """SolveForOneSource up to jQ for each (e0[i], pols[i]).

        Host mode: zeta [nx,ny,nz], zeta0 [nz], e0 [nsrc, nz] complex128 arrays;
        returns (jq [nsrc, N], chi or None, [result dicts]); out: a
        C-contiguous complex128 host array of nsrc * N entries for jq (e.g.
        page-locked).
        Device mode: dev_ptrs = dict(zeta=, zeta0=, e0=, jq=, chi=) device pointers."""
        nsrc = len(pols)
        pol = np.ascontiguousarray(pols, np.int32)
        dz = np.ascontiguousarray(dz, np.float64)
        fg = fgmres or {}
        mx = mixed or {}
        p = SourceParams(precision,
                         GmresParams(fg.get("m_out", 15), fg.get("m_in", 10), fg.get("tol", 1e-8),
                                     fg.get("max_restarts", 100), fg.get("precond", PRECOND_GMRES),
                                     int(fg.get("check_true", True))),
                         MixedParams(mx.get("tol", 1e-6), mx.get("max_outer", 10), mx.get("m_out", 30),
                                     mx.get("m_in", 10), mx.get("inner_tol", 5e-7), mx.get("inner_restarts", 20),
                                     int(mx.get("batch", True))))
        res = (Result * nsrc)()
        if where == DEVICE:
            d = dev_ptrs
            rc = self.lib.egx_solve_sources(self.h, green.h, C.c_void_p(d["zeta"]), C.c_void_p(d["zeta0"]), _ptr(dz),
                                            C.c_void_p(d["e0"]), _ptr(pol), nsrc, C.byref(p),
                                            C.c_void_p(d.get("chi") or 0), C.c_void_p(d["jq"]), res, DEVICE)
            if rc not in (OK, ERR_NOT_CONVERGED):
                self._check(rc)
            return [r.as_dict() for r in res]
        z = _c128(zeta)
        z0 = _c128(zeta0)
        e = _c128(e0).reshape(nsrc, -1)
        n = z.size * 3
        if out is not None:
            jq = out
            if jq.dtype != np.complex128 or not jq.flags.c_contiguous or jq.size != nsrc * n:
                raise ValueError("out must be a C-contiguous complex128 array of %d entries" % (nsrc * n))
            jq = jq.reshape(nsrc, n)
        else:
            jq = np.empty((nsrc, n), np.complex128)
        chi = np.empty((nsrc, n), np.complex128) if want_chi else None
        rc = self.lib.egx_solve_sources(self.h, green.h, _ptr(z), _ptr(z0), _ptr(dz), _ptr(e), _ptr(pol), nsrc,
                                        C.byref(p), _ptr(chi) if want_chi else None, _ptr(jq), res, HOST)
        if rc not in (OK, ERR_NOT_CONVERGED):
            self._check(rc)
        return jq, chi, [r.as_dict() for r in res]

    def wait_selftest(self, limit_ms=100.0):
        """egx_wait_selftest: the status code (EGX_ERR_TIMEOUT expected) and
        the library's message."""
        rc = self.lib.egx_wait_selftest(self.h, float(limit_ms))
        buf = C.create_string_buffer(1024)
        self.lib.egx_last_error(self.h, buf, 1024)
        return rc, buf.value.decode()

    def level_cache(self, capacity=-1):
        """Set the level-tensor cache capacity (0..4; -1 keeps it) and return
        (hits, builds) since the context was created (egx_level_cache)."""
        hits, builds = C.c_long(), C.c_long()
        self._check(self.lib.egx_level_cache(self.h, int(capacity), C.byref(hits), C.byref(builds)))
        return hits.value, builds.value

    def set_level_precision(self, precision):
        """PREC_FP64 (default) or PREC_MIXED (complex64 lateral FFT of the
        level tensors) for the level tensors built from now on."""
        self._check(self.lib.egx_set_level_precision(self.h, int(precision)))

    def level_fields(self, model, omega, jq, z=0.0, shift_x=0.0, shift_y=0.0, n_hankels=10, precision=PREC_FP64,
                     out=None):
        """Anomalous E and H at the observation level z for jq [nsrc, N]
        (host arrays): returns (e, h), each [nsrc, nx, ny, 3] complex128.
        precision: of the level tensors (egx_set_level_precision). out: an
        (e, h) pair of C-contiguous complex128 host arrays of that shape to
        write into (e.g. page-locked buffers)."""
        self.set_level_precision(precision)
        jq = _c128(jq).reshape(-1, model.nx * model.ny * 3 * model.nz)
        nsrc = jq.shape[0]
        if out is not None:
            e, h = out
            shape = (nsrc, model.nx, model.ny, 3)
            for a in (e, h):
                if a.dtype != np.complex128 or not a.flags.c_contiguous or a.shape != shape:
                    raise ValueError("out arrays must be C-contiguous complex128 of shape %s" % (shape,))
        else:
            e = np.empty((nsrc, model.nx, model.ny, 3), np.complex128)
            h = np.empty_like(e)
        ms = model_struct(model)
        self._check(self.lib.egx_level_fields(self.h, C.byref(ms.s), omega, n_hankels, z, shift_x, shift_y,
                                              _ptr(jq), nsrc, _ptr(e), _ptr(h), HOST))
        return e, h

    def level_fields_dev(self, model, omega, jq_ptr, nsrc, e_ptr, h_ptr, z=0.0, shift_x=0.0, shift_y=0.0,
                         n_hankels=10, precision=PREC_FP64):
        """egx_level_fields on device pointers (jq [nsrc][N], e/h [nsrc][nx][ny][3])."""
        self.set_level_precision(precision)
        ms = model_struct(model)
        self._check(self.lib.egx_level_fields(self.h, C.byref(ms.s), omega, n_hankels, z, shift_x, shift_y,
                                              C.c_void_p(jq_ptr), nsrc, C.c_void_p(e_ptr), C.c_void_p(h_ptr),
                                              DEVICE))

    def mt_responses_dev(self, e_ptr, h_ptr, n, omega, e_normal, h_normal, z_ptr, rho_ptr, ph_ptr):
        """egx_mt_responses_dev: impedance [n][2][2] complex, apparent
        resistivity and phase [n][2][2] into device arrays, from the anomalous
        fields [2][n][3] on the device and the plane wave's (E, H) at the
        level."""
        en = np.array([complex(e_normal).real, complex(e_normal).imag])
        hn = np.array([complex(h_normal).real, complex(h_normal).imag])
        self._check(self.lib.egx_mt_responses_dev(self.h, C.c_void_p(e_ptr), C.c_void_p(h_ptr), int(n), float(omega),
                                                  _ptr(en), _ptr(hn), C.c_void_p(z_ptr), C.c_void_p(rho_ptr),
                                                  C.c_void_p(ph_ptr)))

    def profile(self, enable=True, kinds=None):
        """Per-kernel event timing on (the kinds listed, default all) or off."""
        mask = 0xFFFFFFFF if kinds is None else sum(1 << k for k in kinds)
        self._check(self.lib.egx_profile_kinds(self.h, mask))
        self._check(self.lib.egx_profile(self.h, int(enable)))

    def profile_read(self, kind):
        n = C.c_long()
        ms = C.c_double()
        self._check(self.lib.egx_profile_read(self.h, kind, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def set_learned(self, net):
        """Mixed inner solves with the network as their flexible
        preconditioner (a bounded attempt, then the GMRES preconditioner as
        the fallback); net=None goes back to the GMRES preconditioner."""
        if net is None:
            self.set_precond(PRECOND_GMRES)
        else:
            self._check(self.lib.egx_set_precond(self.h, PRECOND_LEARNED, PRECOND_FN(), net.h))

    def learned_stats(self):
        uses, fb = C.c_long(), C.c_long()
        self._check(self.lib.egx_learned_stats(self.h, C.byref(uses), C.byref(fb)))
        return uses.value, fb.value

    def learned_inject_nonfinite(self, count):
        """Test hook: the next `count` learned-preconditioner outputs get a
        NaN written over their first entry from the host."""
        self._check(self.lib.egx_learned_inject_nonfinite(self.h, int(count)))

    def set_precond(self, kind, fn=None):
        """fn(src_ptr, dst_ptr, n, precision) -> None, device pointers."""
        if kind == PRECOND_CALLBACK:
            def tramp(user, src, dst, n, prec):
                try:
                    fn(src, dst, n, prec)
                    return 0
                except Exception:
                    return 1
            self._cb = PRECOND_FN(tramp)
            self._check(self.lib.egx_set_precond(self.h, kind, self._cb, None))
        else:
            self._cb = None
            self._check(self.lib.egx_set_precond(self.h, kind, PRECOND_FN(), None))


class SpectralNet:
    """The learned preconditioner's network (egx_net_*): z = v + rms(v) N(v/rms(v))
    for complex64 vectors in the anomaly layout, batches [B, N]."""

    def __init__(self, ctx, nx, ny, nz, width=32, layers=4, seed=0):
        self.ctx, self.nx, self.ny, self.nz = ctx, nx, ny, nz
        h = C.c_void_p()
        ctx._check(ctx.lib.egx_net_create(ctx.h, nx, ny, nz, width, layers, seed, C.byref(h)))
        self.h = h
        self.n = nx * ny * 3 * nz

    @property
    def size(self):
        return self.ctx.lib.egx_net_size(self.h)

    def params(self, values=None):
        """Read (values None) or write the flat FP32 parameter vector."""
        if values is None:
            out = np.empty(self.size, np.float32)
            self.ctx._check(self.ctx.lib.egx_net_params(self.ctx.h, self.h, _ptr(out), 0))
            return out
        v = np.ascontiguousarray(values, np.float32)
        assert v.size == self.size
        self.ctx._check(self.ctx.lib.egx_net_params(self.ctx.h, self.h, _ptr(v), 1))

    def set_model(self, logsig):
        """log10(omega mu0 sigma dx dy) per anomaly cell, [nx, ny, nz], or
        [count, nx, ny, nz] for a batch whose sample b uses model b % count."""
        ls = np.ascontiguousarray(logsig, np.float32)
        if ls.ndim == 3:
            assert ls.shape == (self.nx, self.ny, self.nz)
            self.ctx._check(self.ctx.lib.egx_net_set_model(self.ctx.h, self.h, _ptr(ls)))
        else:
            assert ls.shape[1:] == (self.nx, self.ny, self.nz)
            self.ctx._check(self.ctx.lib.egx_net_set_models(self.ctx.h, self.h, _ptr(ls), ls.shape[0]))

    def loss_grad(self, v, t, want_grad=False):
        """Loss (and the flat gradient) for residuals v and target corrections
        t = z* - v, host complex arrays [B, N]."""
        v = np.ascontiguousarray(v, np.complex64).reshape(-1, self.n)
        t = np.ascontiguousarray(t, np.complex64).reshape(-1, self.n)
        loss = C.c_float()
        g = np.empty(self.size, np.float32) if want_grad else None
        self.ctx._check(self.ctx.lib.egx_net_loss_grad(self.ctx.h, self.h, _ptr(v), _ptr(t), v.shape[0],
                                                       C.byref(loss), _ptr(g) if g is not None else None, HOST))
        return (loss.value, g) if want_grad else loss.value

    def loss_grad_dev(self, v_ptr, t_ptr, batch):
        loss = C.c_float()
        self.ctx._check(self.ctx.lib.egx_net_loss_grad(self.ctx.h, self.h, C.c_void_p(v_ptr), C.c_void_p(t_ptr),
                                                       batch, C.byref(loss), None, DEVICE))
        return loss.value

    def use_tcgen05(self, enable):
        """Pointwise GEMMs on the tcgen05 kernel (default) or the mma.sync one."""
        self.ctx._check(self.ctx.lib.egx_net_use_tcgen05(self.ctx.h, self.h, int(bool(enable))))

    def adam(self, lr):
        self.ctx._check(self.ctx.lib.egx_net_adam(self.ctx.h, self.h, float(lr)))

    def apply(self, v):
        v = np.ascontiguousarray(v, np.complex64).reshape(-1, self.n)
        z = np.empty_like(v)
        self.ctx._check(self.ctx.lib.egx_net_apply(self.ctx.h, self.h, _ptr(v), _ptr(z), v.shape[0], HOST))
        return z

    def free(self):
        if self.h is not None and self.ctx.h is not None:
            self.ctx.lib.egx_net_free(self.ctx.h, self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class GreenTensor:
    def __init__(self, ctx, h, nx, ny, nz):
        self.ctx, self.h, self.nx, self.ny, self.nz = ctx, h, nx, ny, nz

    def download(self):
        nx, ny, nz = self.nx, self.ny, self.nz
        S = nz * (nz + 1) // 2
        A = nz * nz
        out = {}
        for c in GREEN_COMPONENTS:
            blk = A if c in ("xz", "yz") else S
            out[c] = np.empty((2 * nx, 2 * ny, blk), np.complex128)
        ptrs = (C.c_void_p * 6)(*[out[c].ctypes.data for c in GREEN_COMPONENTS])
        self.ctx._check(self.ctx.lib.egx_green_download(self.ctx.h, self.h, ptrs))
        return out

    def free(self):
        if self.h is not None and self.ctx.h is not None:
            self.ctx.lib.egx_green_free(self.ctx.h, self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def normal_field(model, omega):
    """Thickness-averaged plane-wave E0 on each anomaly layer ([nz] complex)."""
    lib = load()
    m = model_struct(model)
    out = np.empty(model.nz, np.complex128)
    rc = lib.egx_normal_field(C.byref(m.s), float(omega), _ptr(out))
    if rc != OK:
        raise EgxError(rc, "normal field")
    return out


def plane_wave(model, omega, depth):
    """(E, H) of the 1-D plane wave at a flat depth."""
    lib = load()
    m = model_struct(model)
    e = np.empty(1, np.complex128)
    h = np.empty(1, np.complex128)
    rc = lib.egx_plane_wave(C.byref(m.s), float(omega), float(depth), _ptr(e), _ptr(h))
    if rc != OK:
        raise EgxError(rc, "plane wave")
    return complex(e[0]), complex(h[0])


class _ModelStruct:
    pass


def model_struct(model):
    """egx_model view of a :class:`extreme_gb300.model.CartesianModel`
    (keeps the arrays alive)."""
    ms = _ModelStruct()
    ms.depth = np.ascontiguousarray(model.layer_depth, np.float64)
    ms.thick = np.ascontiguousarray(model.layer_thickness, np.float64)
    ms.bg_t = np.ascontiguousarray(model.section.thickness, np.float64)
    ms.bg_s = np.ascontiguousarray(model.section.sigma, np.float64)
    dp = C.POINTER(C.c_double)
    ms.s = Model(model.nx, model.ny, model.nz, float(model.dx), float(model.dy),
                 ms.depth.ctypes.data_as(dp), ms.thick.ctypes.data_as(dp), len(ms.bg_t),
                 float(model.section.zero_air_level), ms.bg_t.ctypes.data_as(dp), ms.bg_s.ctypes.data_as(dp))
    return ms


def mt_responses(e1, e2, h1, h2, omega):
    """Impedance [n, 2, 2], apparent resistivity [n, 2, 2] (Ohm m) and phase
    [n, 2, 2] (degrees) from the total fields [n, 3] of polarisation X (e1, h1)
    and Y (e2, h2) (egx_mt_responses)."""
    lib = load()
    arrs = [_c128(a).reshape(-1, 3) for a in (e1, e2, h1, h2)]
    n = arrs[0].shape[0]
    z = np.empty((n, 2, 2), np.complex128)
    rho = np.empty((n, 2, 2))
    ph = np.empty((n, 2, 2))
    rc = lib.egx_mt_responses(*[_ptr(a) for a in arrs], n, omega, _ptr(z), _ptr(rho), _ptr(ph))
    if rc != OK:
        raise EgxError(rc, "egx_mt_responses: bad arguments")
    return z, rho, ph
