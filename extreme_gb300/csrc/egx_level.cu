// Fields at an observation level and the MT responses.
//
// egx_level_fields builds the anomaly-to-observation-level tensors of E and H
// on the device, in FP64 or, for the mixed form, with double-FP32 face sums
// and complex64 FFTs and storage (build_level_green, egx_green.cu;
// AtoOLevelGreenTensorCalculator.cs:21-126) and convolves them with jQ
// (ToOCalculator.CalculateAnomalyField, ToOCalculator.cs:21-125):
//   k_level_pad + 2-D DFT   jQ into the zero-padded [2nx][2ny][3nz] buffer
//                           (PrepareForForwardFft, Plan3Nz forward);
//   k_level_contract        per spectral point the sum over the anomaly layers
//                           (ZgemvAtoO, Native/Native.Matrix/full_zgemv.c:22-26)
//                           in the component pattern of ApplyGreenTensorAlongZForE/H;
//   inverse 2-D DFT + k_level_extract   3 columns, scaled by 1/(4 nx ny),
//                           rows i < nx, j < ny (Plan3 backward, Zscal, ExtractData).
// egx_mt_responses is host arithmetic on the two polarisations' total fields
// (ResponseFunctionsCalculator.cs:36-51, PlainTextExporter.cs:322-420);
// egx_mt_responses_dev does the same on the device from the anomalous fields
// that egx_level_fields_dev writes, adding the plane wave's normal field.
#include <cmath>
#include <complex>

#include "egx_ctx.cuh"
#include "egx_ds.cuh"

using namespace egx;

namespace {

// the mixed form's jQ, rounded to complex64 into the padded buffer
__global__ void k_level_pad32(const double2 *__restrict__ jq, int nx, int ny, int per, float2 *__restrict__ buf) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)nx * ny * per) return;
    const long cell = idx / per;
    const int b = (int)(idx - cell * per);
    const int i = (int)(cell / ny), j = (int)(cell - (long)i * ny);
    const double2 v = jq[idx];
    buf[((long)i * 2 * ny + j) * per + b] = make_float2((float)v.x, (float)v.y);
}

// (s, c) += a b for floats a, b: the product error-free (FMA), the sum
// compensated (TwoSum)
__device__ __forceinline__ void ds_mac(float &s, float &c, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z)), e));
    s = t;
}

struct DsC {
    float rs = 0.f, rc = 0.f, is = 0.f, ic = 0.f;
    // += sign * g * x
    __device__ __forceinline__ void mac(float2 g, float2 x, float sign) {
        ds_mac(rs, rc, sign * g.x, x.x);
        ds_mac(rs, rc, -sign * g.y, x.y);
        ds_mac(is, ic, sign * g.x, x.y);
        ds_mac(is, ic, sign * g.y, x.x);
    }
    __device__ __forceinline__ double2 value() const {
        return make_double2((double)rs + (double)rc, (double)is + (double)ic);
    }
};

// k_level_contract for the mixed form: complex64 spectra and level tensors,
// products and sums exact to ~47 bits (Dot2), the result in complex128
__global__ void k_level_contract_ds(const float2 *__restrict__ X, const float2 *__restrict__ G, long P, int nz,
                                    int kind, double2 *__restrict__ out) {
    const long p = (long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= P) return;
    const float2 *x = X + p * 3 * nz;
    const size_t cs = (size_t)P * nz;
    const float2 *g = G + p * nz;
    DsC ax, ay, az;
    for (int k = lane; k < nz; k += 32) {
        const float2 sx = x[k], sy = x[nz + k], sz = x[2 * nz + k];
        auto gc = [&](int c) { return g[c * cs + k]; };
        if (kind == 0) {
            ax.mac(gc(0), sx, 1.f);
            ax.mac(gc(3), sy, 1.f);
            ax.mac(gc(4), sz, 1.f);
            ay.mac(gc(3), sx, 1.f);
            ay.mac(gc(1), sy, 1.f);
            ay.mac(gc(5), sz, 1.f);
            az.mac(gc(6), sx, 1.f);
            az.mac(gc(7), sy, 1.f);
            az.mac(gc(2), sz, 1.f);
        } else {
            ax.mac(gc(0), sx, -1.f);
            ax.mac(gc(2), sy, -1.f);
            ax.mac(gc(3), sz, -1.f);
            ay.mac(gc(1), sx, 1.f);
            ay.mac(gc(0), sy, 1.f);
            ay.mac(gc(4), sz, 1.f);
            az.mac(gc(5), sx, -1.f);
            az.mac(gc(6), sy, 1.f);
        }
    }
    double2 v[3] = {ax.value(), ay.value(), az.value()};
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            v[c].x += __shfl_xor_sync(0xffffffffu, v[c].x, o);
            v[c].y += __shfl_xor_sync(0xffffffffu, v[c].y, o);
        }
    if (lane == 0) {
        out[p * 3] = v[0];
        out[p * 3 + 1] = v[1];
        out[p * 3 + 2] = v[2];
    }
}

__global__ void k_level_pad(const double2 *__restrict__ jq, int nx, int ny, int per, double2 *__restrict__ buf) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)nx * ny * per) return;
    const long cell = idx / per;
    const int b = (int)(idx - cell * per);
    const int i = (int)(cell / ny), j = (int)(cell - (long)i * ny);
    buf[((long)i * 2 * ny + j) * per + b] = jq[idx];
}

__device__ __forceinline__ void acc_mul(double2 &a, double2 g, double2 s, double sign) {
    a.x += sign * (g.x * s.x - g.y * s.y);
    a.y += sign * (g.x * s.y + g.y * s.x);
}

// one warp per spectral point p: out[p][3] from X[p][3nz] and G[c][p][nz]
// (E components xx yy zz xy xz yz zx zy, H components xx yx xy xz yz zx zy)
__global__ void k_level_contract(const double2 *__restrict__ X, const double2 *__restrict__ G, long P, int nz,
                                 int kind, double2 *__restrict__ out) {
    const long p = (long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= P) return;
    const double2 *x = X + p * 3 * nz;
    const size_t cs = (size_t)P * nz;
    const double2 *g = G + p * nz;
    double2 ax = make_double2(0, 0), ay = ax, az = ax;
    for (int k = lane; k < nz; k += 32) {
        const double2 sx = x[k], sy = x[nz + k], sz = x[2 * nz + k];
        auto gc = [&](int c) { return g[c * cs + k]; };
        if (kind == 0) {
            acc_mul(ax, gc(0), sx, 1);
            acc_mul(ax, gc(3), sy, 1);
            acc_mul(ax, gc(4), sz, 1);
            acc_mul(ay, gc(3), sx, 1);
            acc_mul(ay, gc(1), sy, 1);
            acc_mul(ay, gc(5), sz, 1);
            acc_mul(az, gc(6), sx, 1);
            acc_mul(az, gc(7), sy, 1);
            acc_mul(az, gc(2), sz, 1);
        } else {
            acc_mul(ax, gc(0), sx, -1);
            acc_mul(ax, gc(2), sy, -1);
            acc_mul(ax, gc(3), sz, -1);
            acc_mul(ay, gc(1), sx, 1);
            acc_mul(ay, gc(0), sy, 1);
            acc_mul(ay, gc(4), sz, 1);
            acc_mul(az, gc(5), sx, -1);
            acc_mul(az, gc(6), sy, 1);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        ax.x += __shfl_xor_sync(0xffffffffu, ax.x, o);
        ax.y += __shfl_xor_sync(0xffffffffu, ax.y, o);
        ay.x += __shfl_xor_sync(0xffffffffu, ay.x, o);
        ay.y += __shfl_xor_sync(0xffffffffu, ay.y, o);
        az.x += __shfl_xor_sync(0xffffffffu, az.x, o);
        az.y += __shfl_xor_sync(0xffffffffu, az.y, o);
    }
    if (lane == 0) {
        out[p * 3] = ax;
        out[p * 3 + 1] = ay;
        out[p * 3 + 2] = az;
    }
}

__global__ void k_level_extract(const double2 *__restrict__ out3, int nx, int ny, double scale,
                                double2 *__restrict__ field) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)nx * ny * 3) return;
    const long cell = idx / 3;
    const int c = (int)(idx - cell * 3);
    const int i = (int)(cell / ny), j = (int)(cell - (long)i * ny);
    const double2 v = out3[((long)i * 2 * ny + j) * 3 + c];
    field[idx] = make_double2(scale * v.x, scale * v.y);
}

// per site: total fields of polarisation X (E + (en, 0, 0), H + (0, hn, 0))
// and Y (E + (0, en, 0), H + (-hn, 0, 0)) from the anomalous fields [2][n][3],
// Z = E H^-1 (2 x 2, complex128), rho = |Z|^2 / (omega mu0), phase in degrees
__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__global__ void k_mt_responses(const double2 *__restrict__ e, const double2 *__restrict__ h, long n, double omega,
                               double2 en, double2 hn, double2 *__restrict__ z, double *__restrict__ rho,
                               double *__restrict__ phase) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double2 *e1 = e + 3 * k, *e2 = e + 3 * (n + k), *h1 = h + 3 * k, *h2 = h + 3 * (n + k);
    const double2 f11x = make_double2(e1[0].x + en.x, e1[0].y + en.y), f11y = e1[1];
    const double2 f12x = e2[0], f12y = make_double2(e2[1].x + en.x, e2[1].y + en.y);
    const double2 f21x = h1[0], f21y = make_double2(h1[1].x + hn.x, h1[1].y + hn.y);
    const double2 f22x = make_double2(h2[0].x - hn.x, h2[0].y - hn.y), f22y = h2[1];
    const double2 a = cmul2(f21x, f22y), b = cmul2(f22x, f21y);
    const double2 det = make_double2(a.x - b.x, a.y - b.y);
    const double dd = det.x * det.x + det.y * det.y;
    const double2 inv = make_double2(det.x / dd, -det.y / dd);
    const double2 hi11 = cmul2(f22y, inv), hi22 = cmul2(f21x, inv);
    const double2 hi12 = cmul2(make_double2(-f22x.x, -f22x.y), inv), hi21 = cmul2(make_double2(-f21y.x, -f21y.y), inv);
    double2 zz[4];
    {
        const double2 p = cmul2(f11x, hi11), q = cmul2(f12x, hi21);
        zz[0] = make_double2(p.x + q.x, p.y + q.y);
    }
    {
        const double2 p = cmul2(f11x, hi12), q = cmul2(f12x, hi22);
        zz[1] = make_double2(p.x + q.x, p.y + q.y);
    }
    {
        const double2 p = cmul2(f11y, hi11), q = cmul2(f12y, hi21);
        zz[2] = make_double2(p.x + q.x, p.y + q.y);
    }
    {
        const double2 p = cmul2(f11y, hi12), q = cmul2(f12y, hi22);
        zz[3] = make_double2(p.x + q.x, p.y + q.y);
    }
    const double mu0 = 4.0e-7 * 3.14159265358979323846;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        z[4 * k + c] = zz[c];
        rho[4 * k + c] = (zz[c].x * zz[c].x + zz[c].y * zz[c].y) / (omega * mu0);
        phase[4 * k + c] = atan2(zz[c].y, zz[c].x) * (180.0 / 3.14159265358979323846);
    }
}

}  // namespace

extern "C" {

int egx_set_level_precision(egx_ctx *ctx, int precision) {
    if (!ctx) return EGX_ERR_INVALID;
    if (precision != EGX_PREC_FP64 && precision != EGX_PREC_MIXED)
        return fail(ctx, EGX_ERR_INVALID, "unknown level precision");
    ctx->lvl_prec = precision;
    return EGX_OK;
}

int egx_level_fields(egx_ctx *ctx, const egx_model *model, double omega, int n_hankels, double z, double shift_x,
                     double shift_y, const double *jq, int nsrc, double *e, double *h, int where) {
    if (!ctx) return EGX_ERR_INVALID;
    try {
        EGX_CHECK(model && jq && e && h && nsrc >= 1, EGX_ERR_INVALID, "bad level-field arguments");
        EGX_CHECK(model->layer_depth && model->layer_thickness && model->bg_thickness && model->bg_sigma,
                  EGX_ERR_INVALID, "null model arrays");
        EGX_CHECK(omega > 0, EGX_ERR_INVALID, "omega must be positive");
        set_device(ctx);
        const GreenModel gm = green_model(model, omega);
        const int nx = gm.nx, ny = gm.ny, nz = gm.nz, n0 = 2 * nx, n1 = 2 * ny, per = 3 * nz;
        cudaStream_t s = ctx->stream;
        ensure_twiddles(ctx, n0, n1);
        // level tensors: reuse a cached pair or build into the least recently used slot
        std::vector<double> key = {(double)nx, (double)ny, (double)nz, model->dx, model->dy, omega,
                                   (double)n_hankels, z, shift_x, shift_y, (double)model->n_bg, model->zero_air_level,
                                   (double)ctx->lvl_prec};
        key.insert(key.end(), model->layer_depth, model->layer_depth + nz);
        key.insert(key.end(), model->layer_thickness, model->layer_thickness + nz);
        key.insert(key.end(), model->bg_thickness, model->bg_thickness + model->n_bg);
        key.insert(key.end(), model->bg_sigma, model->bg_sigma + model->n_bg);
        const int cap = std::max(1, ctx->lvl_capacity);
        int slot = -1;
        if (ctx->lvl_capacity > 0)
            for (int i = 0; i < cap; i++)
                if (ctx->lvl_cache[i].key == key) slot = i;
        if (slot >= 0) {
            ctx->lvl_hits++;
        } else {
            slot = 0;
            for (int i = 1; i < cap; i++)
                if (ctx->lvl_cache[i].used < ctx->lvl_cache[slot].used) slot = i;
            egx_ctx::LevelEntry &L = ctx->lvl_cache[slot];
            L.key.clear();  // not valid until both tensors are built
            const bool fft32 = ctx->lvl_prec == EGX_PREC_MIXED;
            build_level_green(gm, n_hankels, z, shift_x, shift_y, 0, s, L.g[0], &ctx->launches, ctx->gws, fft32);
            build_level_green(gm, n_hankels, z, shift_x, shift_y, 1, s, L.g[1], &ctx->launches, ctx->gws, fft32);
            if (ctx->lvl_capacity > 0) L.key = key;
            ctx->lvl_builds++;
        }
        egx_ctx::LevelEntry &lv = ctx->lvl_cache[slot];
        lv.used = ++ctx->lvl_clock;
        const long N = (long)nx * ny * per, P = (long)n0 * n1, F = (long)nx * ny * 3;
        ctx->lvl_x.ensure((size_t)P * per * sizeof(double2));
        ctx->lvl_out.ensure((size_t)P * 3 * sizeof(double2));
        if (where != EGX_DEVICE) {
            ctx->lvl_in.ensure((size_t)N * sizeof(double2));
            ctx->lvl_field.ensure((size_t)F * sizeof(double2));
        }
        double2 *X = ctx->lvl_x.as<double2>(), *O = ctx->lvl_out.as<double2>();
        const double2 *tw0 = ctx->tw0_64.as<double2>(), *tw1 = ctx->tw1_64.as<double2>();
        const float2 *tw0_32 = ctx->tw0_32.as<float2>(), *tw1_32 = ctx->tw1_32.as<float2>();
        const bool mixed = ctx->lvl_prec == EGX_PREC_MIXED;
        for (int i = 0; i < nsrc; i++) {
            const double2 *src;
            if (where == EGX_DEVICE) {
                src = reinterpret_cast<const double2 *>(jq) + (size_t)i * N;
            } else {
                EGX_CUDA(cudaMemcpyAsync(ctx->lvl_in.p, jq + 2 * (size_t)i * N, N * sizeof(double2),
                                         cudaMemcpyHostToDevice, s));
                src = ctx->lvl_in.as<double2>();
            }
            if (mixed) {
                // the mixed form: jQ's spectrum in complex64 against the
                // complex64 level tensors
                float2 *X32 = ctx->lvl_x.as<float2>();
                k_level_pad32<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(src, nx, ny, per, X32);
                EGX_CUDA(cudaGetLastError());
                fft_lines<float>(X32, nx, (long)n1 * per, per, per, ny, n1, ctx->p1, tw1_32, -1, s, &ctx->launches);
                fft_lines<float>(X32, n1, per, (long)n1 * per, per, nx, n0, ctx->p0, tw0_32, -1, s, &ctx->launches);
            } else {
                k_level_pad<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(src, nx, ny, per, X);
                EGX_CUDA(cudaGetLastError());
                // forward DFT: y over the nx data rows (ny loaded), then x over all columns (nx loaded)
                fft_lines<double>(X, nx, (long)n1 * per, per, per, ny, n1, ctx->p1, tw1, -1, s, &ctx->launches);
                fft_lines<double>(X, n1, per, (long)n1 * per, per, nx, n0, ctx->p0, tw0, -1, s, &ctx->launches);
            }
            for (int kind = 0; kind < 2; kind++) {
                if (mixed)
                    k_level_contract_ds<<<(unsigned)((P + 7) / 8), 256, 0, s>>>(
                        ctx->lvl_x.as<float2>(), lv.g[kind].as<float2>(), P, nz, kind, O);
                else
                    k_level_contract<<<(unsigned)((P + 7) / 8), 256, 0, s>>>(X, lv.g[kind].as<double2>(), P, nz,
                                                                             kind, O);
                EGX_CUDA(cudaGetLastError());
                // inverse DFT of the 3 columns: x keeping rows < nx, then y keeping j < ny
                fft_lines<double>(O, n1, 3, (long)n1 * 3, 3, n0, nx, ctx->p0, tw0, +1, s, &ctx->launches);
                fft_lines<double>(O, nx, (long)n1 * 3, 3, 3, n1, ny, ctx->p1, tw1, +1, s, &ctx->launches);
                double *dst_host = (kind == 0 ? e : h) + 2 * (size_t)i * F;
                double2 *dst = where == EGX_DEVICE ? reinterpret_cast<double2 *>(dst_host) : ctx->lvl_field.as<double2>();
                k_level_extract<<<(unsigned)((F + 255) / 256), 256, 0, s>>>(O, nx, ny, 1.0 / (4.0 * nx * ny), dst);
                EGX_CUDA(cudaGetLastError());
                if (where != EGX_DEVICE)
                    EGX_CUDA(cudaMemcpyAsync(dst_host, dst, F * sizeof(double2), cudaMemcpyDeviceToHost, s));
                ctx->launches += 2;
            }
            ctx->launches += 1;
            EGX_CUDA(cudaStreamSynchronize(s));
        }
        check_device_error(ctx);
    } catch (const egx::Error &err) {
        return fail(ctx, err.code, err.what());
    } catch (const std::exception &err) {
        return fail(ctx, EGX_ERR_INVALID, err.what());
    }
    return EGX_OK;
}

int egx_level_cache(egx_ctx *ctx, int capacity, long *hits, long *builds) {
    if (!ctx) return EGX_ERR_INVALID;
    if (capacity > egx_ctx::kLevelSlots) return fail(ctx, EGX_ERR_INVALID, "level cache holds at most 4 levels");
    if (capacity >= 0) {
        try {
            set_device(ctx);
        } catch (const egx::Error &err) {
            return fail(ctx, err.code, err.what());
        }
        for (auto &L : ctx->lvl_cache) L.key.clear();
        for (int i = std::max(1, capacity); i < egx_ctx::kLevelSlots; i++) {
            ctx->lvl_cache[i].g[0].release();
            ctx->lvl_cache[i].g[1].release();
        }
        ctx->lvl_capacity = capacity;
    }
    if (hits) *hits = ctx->lvl_hits;
    if (builds) *builds = ctx->lvl_builds;
    return EGX_OK;
}

int egx_mt_responses_dev(egx_ctx *ctx, const double *e, const double *h, long n, double omega,
                         const double e_normal[2], const double h_normal[2], double *z, double *rho, double *phase) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(e && h && e_normal && h_normal && z && rho && phase && n >= 1 && omega > 0, EGX_ERR_INVALID,
                  "bad response arguments");
        set_device(ctx);
        const unsigned blocks = (unsigned)((n + 255) / 256);
        k_mt_responses<<<blocks, 256, 0, ctx->stream>>>(
            reinterpret_cast<const double2 *>(e), reinterpret_cast<const double2 *>(h), n, omega,
            make_double2(e_normal[0], e_normal[1]), make_double2(h_normal[0], h_normal[1]),
            reinterpret_cast<double2 *>(z), rho, phase);
        EGX_CUDA(cudaGetLastError());
        ++ctx->launches;
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int egx_mt_responses(const double *e1, const double *e2, const double *h1, const double *h2, long n, double omega,
                     double *z, double *rho, double *phase) {
    if (!e1 || !e2 || !h1 || !h2 || !z || !rho || !phase || n < 1 || !(omega > 0)) return EGX_ERR_INVALID;
    typedef std::complex<double> cd;
    const double mu0 = 4.0 * M_PI * 1.0e-7;
    auto at = [](const double *v, long k, int c) { return cd(v[2 * (3 * k + c)], v[2 * (3 * k + c) + 1]); };
    for (long k = 0; k < n; k++) {
        const cd f11x = at(e1, k, 0), f11y = at(e1, k, 1), f12x = at(e2, k, 0), f12y = at(e2, k, 1);
        const cd f21x = at(h1, k, 0), f21y = at(h1, k, 1), f22x = at(h2, k, 0), f22y = at(h2, k, 1);
        const cd det = f21x * f22y - f22x * f21y;
        const cd hi11 = f22y / det, hi12 = -f22x / det, hi21 = -f21y / det, hi22 = f21x / det;
        const cd zz[4] = {f11x * hi11 + f12x * hi21, f11x * hi12 + f12x * hi22, f11y * hi11 + f12y * hi21,
                          f11y * hi12 + f12y * hi22};
        for (int c = 0; c < 4; c++) {
            z[2 * (4 * k + c)] = zz[c].real();
            z[2 * (4 * k + c) + 1] = zz[c].imag();
            rho[4 * k + c] = std::norm(zz[c]) / (omega * mu0);
            phase[4 * k + c] = std::arg(zz[c]) * (180.0 / M_PI);
        }
    }
    return EGX_OK;
}

}  // extern "C"
