// MT source field and the CIE pipeline around the solve.
//
// Host: the 1-D plane-wave field at lambda = 0
// (Extreme.Cartesian.Magnetotellurics/PlaneWaveCalculator.cs:11-83 with the
// single-lambda recursions of Green/Scalar/Impl/PlanCalculator.cs:173-314).
// Device: jS = (zeta - zeta0) E0, chi0 = K_chi0 jS, the solve of A chi = chi0
// (complex128 FGMRES from x0 = chi0 as the reference; the mixed solve from zero),
// Es = (2 sqrt(Re zeta0) chi - jS)/(zeta + conj zeta0) and
// jQ = Es (zeta - zeta0) + jS (Forward/ForwardSolver.cs:186-436).
#include <cmath>
#include <complex>
#include <vector>

#include "egx_ctx.cuh"

using namespace egx;
typedef std::complex<double> cd;

namespace {

constexpr double kMu0 = 4.0 * M_PI * 1.0e-7;
constexpr double kEps0 = 1.0 / (kMu0 * 299792458.0 * 299792458.0);

struct PlaneWave {
    std::vector<double> tops;
    std::vector<cd> zeta, q;
    std::vector<std::vector<cd>> A;
    int rc, tr;
};

int corr_layer(const std::vector<double> &tops, const std::vector<double> &thick, double depth) {
    double prev = tops[0];
    for (size_t k = 0; k < thick.size(); k++) {
        double d1 = prev, d2 = prev + thick[k];
        if (depth >= d1 && depth < d2) return (int)k;
        prev = d2;
    }
    throw Error(EGX_ERR_MODEL, "depth is not within the 1-D section");
}

// PlaneWaveCalculator.PrepareContainer at lambda = 0.
PlaneWave plane_wave_container(const egx_model *m, double omega, double rc_depth) {
    PlaneWave pw;
    const int L = m->n_bg;
    EGX_CHECK(L >= 3, EGX_ERR_INVALID, "background needs at least 3 layers");
    std::vector<double> thick(m->bg_thickness, m->bg_thickness + L);
    pw.tops.resize(L + 1);
    pw.tops[0] = m->zero_air_level;
    for (int k = 0; k < L; k++) pw.tops[k + 1] = pw.tops[k] + thick[k];
    pw.zeta.resize(L);
    for (int k = 0; k < L; k++) pw.zeta[k] = cd(m->bg_sigma[k], -omega * kEps0);
    const cd iom(0.0, omega);
    std::vector<cd> eta(L), ex(L), p(L, 0.0);
    pw.q.assign(L, 0.0);
    for (int k = 0; k < L; k++) {
        eta[k] = std::sqrt(cd(0.0, 0.0) - iom * pw.zeta[k] * kMu0);
        ex[k] = std::exp(-2.0 * eta[k] * thick[k]);
    }
    const int n = L - 1;
    cd part = eta[n] / eta[n - 1];
    pw.q[n - 1] = (1.0 - part) / (1.0 + part);
    for (int k = n - 1; k > 1; k--) {
        cd qexp = pw.q[k] * ex[k];
        part = (eta[k] / eta[k - 1]) * ((qexp - 1.0) / (qexp + 1.0));
        pw.q[k - 1] = (1.0 + part) / (1.0 - part);
    }
    p[1] = (eta[1] - eta[0]) / (eta[1] + eta[0]);
    for (int k = 1; k < L - 1; k++) {
        cd pexp = p[k] * ex[k];
        part = (eta[k] / eta[k + 1]) * ((pexp - 1.0) / (pexp + 1.0));
        p[k + 1] = (1.0 + part) / (1.0 - part);
    }
    pw.tr = corr_layer(pw.tops, thick, 0.0);
    pw.rc = corr_layer(pw.tops, thick, rc_depth);
    EGX_CHECK(pw.rc + 1 < L && pw.tr + 1 < L, EGX_ERR_MODEL, "plane-wave depth inside the lower half-space");
    const int s = std::max(pw.rc, pw.tr), r = std::min(pw.rc, pw.tr);
    pw.A.assign(L, std::vector<cd>(L, 0.0));
    for (int nn = s; nn >= r; nn--) {
        cd prev = 1.0 / (eta[nn] * (1.0 - p[nn] * pw.q[nn] * ex[nn]));
        pw.A[nn][nn] = prev;
        for (int k = nn - 1; k >= r; k--) {
            cd f = ((1.0 + p[k + 1]) / (1.0 + p[k] * ex[k])) * std::exp((eta[k + 1] - eta[k]) * pw.tops[k + 1]);
            prev = f * prev;
            pw.A[k][nn] = prev;
            pw.A[nn][k] = prev;
        }
    }
    return pw;
}

// PlaneWaveCalculator.CalculateFieldE (PlaneWaveCalculator.cs:11-40)
cd field_e(const egx_model *m, double omega, double zr, double thick) {
    PlaneWave pw = plane_wave_container(m, omega, zr);
    const cd kkr = cd(0.0, 1.0) * omega * kMu0 * pw.zeta[pw.rc];
    const cd ikr = cd(0.0, 1.0) * std::sqrt(kkr);
    const cd kk1 = cd(0.0, 1.0) * omega * kMu0 * pw.zeta[pw.tr];
    const cd ik1 = cd(0.0, 1.0) * std::sqrt(kk1);
    const double dr1 = pw.tops[pw.rc + 1], d2 = pw.tops[pw.tr + 1];
    const cd a = pw.A[pw.rc][pw.tr] / pw.A[pw.tr][pw.tr];
    cd upper;
    if (thick == 0) {
        upper = std::exp(ikr * zr) + pw.q[pw.rc] * std::exp(ikr * (2 * dr1 - zr));
    } else {
        double z1 = zr - thick / 2, z2 = zr + thick / 2;
        cd u1 = std::exp(ikr * z1) - pw.q[pw.rc] * std::exp(ikr * (2 * dr1 - z1));
        cd u2 = std::exp(ikr * z2) - pw.q[pw.rc] * std::exp(ikr * (2 * dr1 - z2));
        upper = (u2 - u1) / (z2 - z1) / ikr;
    }
    const cd lower = 1.0 + pw.q[pw.tr] * std::exp(ik1 * (2 * d2));
    return a * (upper / lower);
}

// PlaneWaveCalculator.CalculateFieldH (PlaneWaveCalculator.cs:42-64)
cd field_h(const egx_model *m, double omega, double zr) {
    PlaneWave pw = plane_wave_container(m, omega, zr);
    const cd kkr = cd(0.0, 1.0) * omega * kMu0 * pw.zeta[pw.rc];
    const cd ikr = cd(0.0, 1.0) * std::sqrt(kkr);
    const cd kk1 = cd(0.0, 1.0) * omega * kMu0 * pw.zeta[pw.tr];
    const cd ik1 = cd(0.0, 1.0) * std::sqrt(kk1);
    const double dr1 = pw.tops[pw.rc + 1], d2 = pw.tops[pw.tr + 1];
    const cd a = pw.A[pw.rc][pw.tr] / pw.A[pw.tr][pw.tr];
    const cd upper = std::exp(ikr * zr) - pw.q[pw.rc] * std::exp(ikr * (2 * dr1 - zr));
    const cd lower = 1.0 + pw.q[pw.tr] * std::exp(ik1 * (2 * d2));
    return (std::sqrt(kkr) / (omega * kMu0)) * a * (upper / lower);
}

// jS[(cell*3 + c)*nz + k] = (zeta - zeta0_k) * E0_k for c == pol, else 0
// (ForwardSolver.CalculateScatteredCurrentFromBackgroundField, ForwardSolver.cs:223-237).
__global__ void k_js(const double2 *__restrict__ zeta, const double2 *__restrict__ zeta0,
                     const double2 *__restrict__ e0, int pol, int nz, long ncell, double2 *__restrict__ js) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ncell * 3 * nz) return;
    int k = (int)(idx % nz);
    long rest = idx / nz;
    int c = (int)(rest % 3);
    long cell = rest / 3;
    double2 out = make_double2(0, 0);
    if (c == pol) {
        double2 z = zeta[cell * nz + k], z0 = zeta0[k];
        out = cmul<double>(make_double2(z.x - z0.x, z.y - z0.y), e0[k]);
    }
    js[idx] = out;
}

// Es and jQ (ForwardSolver.CalculateScatteredFieldFromChi / CalculateJqFromScatteredField,
// ForwardSolver.cs:391-436). In place: chi and jq may be the same vector
// (each thread reads its element before writing it).
__global__ void k_post(const double2 *__restrict__ zeta, const double2 *__restrict__ zeta0, const double2 *chi,
                       const double2 *__restrict__ js, int nz, long ncell, double2 *jq) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ncell * 3 * nz) return;
    int k = (int)(idx % nz);
    long cell = idx / nz / 3;
    double2 z = zeta[cell * nz + k], z0 = zeta0[k];
    double sq = sqrt(z0.x);
    double2 num = make_double2(2 * sq * chi[idx].x - js[idx].x, 2 * sq * chi[idx].y - js[idx].y);
    double2 es = cdiv<double>(num, make_double2(z.x + z0.x, z.y - z0.y));
    double2 q = cmul<double>(es, make_double2(z.x - z0.x, z.y - z0.y));
    jq[idx] = make_double2(q.x + js[idx].x, q.y + js[idx].y);
}

}  // namespace

extern "C" {

int egx_normal_field(const egx_model *model, double omega, double *e0) {
    if (!model || !e0 || !model->layer_depth || !model->layer_thickness || !model->bg_thickness ||
        !model->bg_sigma)
        return EGX_ERR_INVALID;
    try {
        cd *out = reinterpret_cast<cd *>(e0);
        for (int k = 0; k < model->nz; k++) {
            double mid = model->layer_depth[k] + model->layer_thickness[k] / 2;
            out[k] = field_e(model, omega, mid, model->layer_thickness[k]);
        }
    } catch (const egx::Error &e) {
        return e.code;
    }
    return EGX_OK;
}

int egx_plane_wave(const egx_model *model, double omega, double depth, double *e, double *h) {
    if (!model || !e || !h || !model->bg_thickness || !model->bg_sigma) return EGX_ERR_INVALID;
    try {
        *reinterpret_cast<cd *>(e) = field_e(model, omega, depth, 0.0);
        *reinterpret_cast<cd *>(h) = field_h(model, omega, depth);
    } catch (const egx::Error &ex) {
        return ex.code;
    }
    return EGX_OK;
}

int egx_solve_sources(egx_ctx *ctx, egx_green *g, const double *zeta, const double *zeta0, const double *dz,
                      const double *e0, const int *pol, int nsrc, const egx_source_params *p, double *chi,
                      double *jq, egx_result *res, int where) {
    if (!ctx) return EGX_ERR_INVALID;
    int status = EGX_OK;
    try {
        EGX_CHECK(g && zeta && zeta0 && dz && e0 && pol && p && jq && res && nsrc >= 1, EGX_ERR_INVALID,
                  "bad source-solve arguments");
        EGX_CHECK(p->precision == EGX_PREC_FP64 || p->precision == EGX_PREC_MIXED, EGX_ERR_INVALID,
                  "unknown precision");
        set_device(ctx);
        const cudaStream_t s = ctx->stream;
        upload_model(ctx, g, zeta, zeta0, where);
        const int nz = g->nz;
        const long ncell = (long)g->nx * g->ny;
        const long n = ncell * 3 * nz;
        ctx->js.ensure((size_t)nsrc * n * sizeof(double2));
        ctx->chi0.ensure((size_t)nsrc * n * sizeof(double2));
        ctx->src_io.ensure((size_t)nsrc * (n + nz) * sizeof(double2));
        double2 *js = ctx->js.as<double2>(), *chi0 = ctx->chi0.as<double2>();
        double2 *e0d = ctx->src_io.as<double2>();            // [nsrc][nz]
        double2 *xs = ctx->src_io.as<double2>() + (size_t)nsrc * nz;  // [nsrc][n] solution / jq
        EGX_CUDA(cudaMemcpyAsync(e0d, e0, (size_t)nsrc * nz * sizeof(double2),
                                 where == EGX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
        for (int i = 0; i < nsrc; i++) {
            EGX_CHECK(pol[i] == 0 || pol[i] == 1, EGX_ERR_INVALID, "polarization must be 0 (x) or 1 (y)");
            k_js<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(ctx->zeta.as<double2>(), ctx->zeta0.as<double2>(),
                                                             e0d + (size_t)i * nz, pol[i], nz, ncell, js + i * n);
        }
        ctx->launches += nsrc;
        // chi0 = K_chi0 jS for all sources in one apply; the mixed form applies
        // it in complex64 (its error, ~1e-7, stays far below the 1e-6 target;
        // the refinement's residual against this chi0 is still complex128)
        prepare_device(ctx, g, dz, EGX_OP_CHI0);
        if (p->precision == EGX_PREC_MIXED && ctx->prepared32) {
            ctx->xin32.ensure((size_t)nsrc * n * sizeof(float2));
            ctx->yout32.ensure((size_t)nsrc * n * sizeof(float2));
            float2 *js32 = ctx->xin32.as<float2>(), *chi32 = ctx->yout32.as<float2>();
            convert_d2f(js, js32, (long)nsrc * n, 1.0, s);
            apply_dev<float>(ctx, js32, chi32, nsrc);
            EGX_CUDA(cudaMemsetAsync(chi0, 0, (size_t)nsrc * n * sizeof(double2), s));
            convert_f2d_add(chi32, chi0, (long)nsrc * n, 1.0, s);
            ctx->launches += 2;
        } else {
            apply_dev<double>(ctx, js, chi0, nsrc);
        }
        prepare_device(ctx, g, dz, EGX_OP_A);
        const bool stacked = p->precision == EGX_PREC_MIXED && p->mixed.batch && nsrc > 1;
        if (stacked) {
            // all sources as one stacked system from zero: every operator
            // apply covers every source
            EGX_CUDA(cudaMemsetAsync(xs, 0, (size_t)nsrc * n * sizeof(double2), s));
            int applies = 0, refinements = 0;
            std::vector<double> tbe(nsrc, -1.0);
            GmresResult r = mixed_dev(ctx, chi0, xs, p->mixed, &applies, &refinements, tbe.data(), nsrc);
            for (int i = 0; i < nsrc; i++) {
                res[i].converged = tbe[i] < p->mixed.tol;
                res[i].iterations = r.iterations;
                res[i].arnoldi_be = r.arnoldi_be;
                res[i].true_be = tbe[i];
                res[i].n_applies = applies + 1;  // applies of the operator to this source, + chi0
                res[i].n_refinements = refinements;
            }
            if (!r.converged) status = fail(ctx, EGX_ERR_NOT_CONVERGED, "source solve did not converge");
        }
        for (int i = 0; i < nsrc; i++) {
            double2 *x = xs + (size_t)i * n;
            if (!stacked) {
                int applies = 0, refinements = 0;
                double tbe = -1;
                GmresResult r;
                if (p->precision == EGX_PREC_FP64) {
                    // the reference starts FGMRES from chi0 (ForwardSolver.cs:300-306)
                    EGX_CUDA(cudaMemcpyAsync(x, chi0 + i * n, n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
                    r = fgmres_dev(ctx, chi0 + i * n, x, p->fgmres, &applies);
                    tbe = r.true_be;
                } else {
                    // the refinement starts from zero: its first residual is chi0
                    // itself, which saves a complex128 apply
                    EGX_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double2), s));
                    r = mixed_dev(ctx, chi0 + i * n, x, p->mixed, &applies, &refinements, &tbe);
                }
                res[i].converged = r.converged;
                res[i].iterations = r.iterations;
                res[i].arnoldi_be = r.arnoldi_be;
                res[i].true_be = tbe;
                res[i].n_applies = applies + 1;  // + the chi0 apply
                res[i].n_refinements = refinements;
                if (!r.converged) status = fail(ctx, EGX_ERR_NOT_CONVERGED, "source solve did not converge");
            }
            if (chi)
                EGX_CUDA(cudaMemcpyAsync(chi + 2 * (size_t)i * n, x, n * sizeof(double2),
                                         where == EGX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
            k_post<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(ctx->zeta.as<double2>(), ctx->zeta0.as<double2>(), x,
                                                               js + i * n, nz, ncell, x);
            ctx->launches++;
            EGX_CUDA(cudaMemcpyAsync(jq + 2 * (size_t)i * n, x, n * sizeof(double2),
                                     where == EGX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
        }
        EGX_CUDA(cudaGetLastError());
        EGX_CUDA(cudaStreamSynchronize(s));
        check_device_error(ctx);
    } catch (const egx::Error &e) {
        return fail(ctx, e.code, e.what());
    } catch (const std::exception &e) {
        return fail(ctx, EGX_ERR_INVALID, e.what());
    }
    return status;
}

}  // extern "C"
