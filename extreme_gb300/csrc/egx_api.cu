// extern "C" entry points of libegx.so (declared in include/egx.h): context,
// Green tensor handles, operator, FFT, solvers, profiling.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>

#include "egx_ctx.cuh"
#include "egx_learn.cuh"
#include "egx_wait.cuh"

using namespace egx;
typedef std::complex<double> cd;

namespace egx {

int fail(egx_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}

void set_device(egx_ctx *ctx) { EGX_CUDA(cudaSetDevice(ctx->device)); }

void check_device_error(egx_ctx *ctx) {
    int flag = 0;
    EGX_CUDA(cudaMemcpyAsync(&flag, ctx->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    EGX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (flag) {
        EGX_CUDA(cudaMemsetAsync(ctx->errflag.p, 0, sizeof(int), ctx->stream));
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        throw Error(flag, "a device wait timed out (shared-memory pipeline did not complete)");
    }
}

long nvec(const egx_ctx *ctx) { return (long)ctx->nx * ctx->ny * 3 * ctx->nz; }

namespace {

template <typename T>
void upload_twiddles(DevBuf &dst, int n, cudaStream_t s) {
    std::vector<double> t = twiddles(n);
    if (sizeof(T) == sizeof(double)) {
        dst.ensure(t.size() * sizeof(double));
        EGX_CUDA(cudaMemcpyAsync(dst.p, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    } else {
        std::vector<float> f(t.begin(), t.end());
        dst.ensure(f.size() * sizeof(float));
        EGX_CUDA(cudaMemcpyAsync(dst.p, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice, s));
        EGX_CUDA(cudaStreamSynchronize(s));
        return;
    }
    EGX_CUDA(cudaStreamSynchronize(s));
}


// r = (zeta - zeta0)/(zeta + conj zeta0) (A) or sqrt(Re zeta0)/(zeta + conj zeta0)
// (Chi0) (ConvolutionOperator.PrepareRFunction, ConvolutionOperator.cs:113-143).
__global__ void k_prepare_r(const double2 *__restrict__ zeta, const double2 *__restrict__ zeta0, int nz, long ncell,
                            int type, double2 *__restrict__ r64, float2 *__restrict__ r32) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ncell * nz) return;
    int k = (int)(idx % nz);
    double2 z = zeta[idx], z0 = zeta0[k];
    double2 den = make_double2(z.x + z0.x, z.y - z0.y);
    double2 num = type == EGX_OP_CHI0 ? make_double2(sqrt(z0.x), 0.0) : make_double2(z.x - z0.x, z.y - z0.y);
    double2 r = cdiv<double>(num, den);
    r64[idx] = r;
    if (r32) r32[idx] = make_float2((float)r.x, (float)r.y);
}

void gather_quadrant(int nx, int ny, int nz, const double *const comps[6], std::vector<cd> &q) {
    GreenDims gd{nx, ny, nz};
    const int S = gd.S(), A = gd.A(), Bs = gd.Bs(), lda = gd.lda();
    q.assign((size_t)gd.Q() * Bs, cd(0, 0));
    const int ref_blk[6] = {S, S, S, S, nz * nz, nz * nz};
    const int off[6] = {0, S, 2 * S, 3 * S, 4 * S, 4 * S + A};
    for (int a = 0; a <= nx; a++)
        for (int b = 0; b <= ny; b++) {
            long qi = (long)a * (ny + 1) + b;
            long pt = (long)a * 2 * ny + b;
            for (int c = 0; c < 6; c++) {
                const cd *src = reinterpret_cast<const cd *>(comps[c]) + pt * ref_blk[c];
                if (c < 4) {
                    std::memcpy(&q[qi * Bs + off[c]], src, sizeof(cd) * S);
                } else {
                    for (int rc = 0; rc < nz; rc++)
                        std::memcpy(&q[qi * Bs + off[c] + rc * lda], src + rc * nz, sizeof(cd) * nz);
                }
            }
        }
}

// Forget the captured inner-cycle graph (egx_set_graphs).
void drop_graph(egx_ctx *ctx) {
    if (ctx->pc_exec) cudaGraphExecDestroy(ctx->pc_exec);
    ctx->pc_exec = nullptr;
    ctx->pc_key.clear();
}

template <typename T>
GmresResult run_fgmres(egx_ctx *ctx, const C<T> *b, C<T> *x, int m_out, int m_in, double tol, int max_restarts,
                       bool check_true, int precond_kind, int *n_applies, int nrhs = 1) {
    // nrhs > 1: one stacked system of nrhs blocks [nrhs][nvec], each Krylov
    // step one nrhs-vector operator apply
    const long n = nvec(ctx) * nrhs;
    const bool dbl = sizeof(T) == sizeof(double);
    char keybuf[160];
    snprintf(keybuf, sizeof keybuf, "%ld/%d/%d/%d/%d/%d", n, m_out, m_in, max_restarts, (int)check_true,
             precond_kind);
    std::unique_ptr<Gmres<T>> *outer, *inner;
    std::string *key;
    if (dbl) {
        outer = reinterpret_cast<std::unique_ptr<Gmres<T>> *>(&ctx->outer64);
        inner = reinterpret_cast<std::unique_ptr<Gmres<T>> *>(&ctx->inner64);
        key = &ctx->key64;
    } else if (precond_kind == EGX_PRECOND_LEARNED) {
        outer = reinterpret_cast<std::unique_ptr<Gmres<T>> *>(&ctx->outer32l);
        inner = reinterpret_cast<std::unique_ptr<Gmres<T>> *>(&ctx->inner32l);
        key = &ctx->key32l;
    } else {
        outer = reinterpret_cast<std::unique_ptr<Gmres<T>> *>(&ctx->outer32);
        inner = reinterpret_cast<std::unique_ptr<Gmres<T>> *>(&ctx->inner32);
        key = &ctx->key32;
    }
    if (*key != keybuf) {
        if (*outer) ctx->launches += (*outer)->kernel_launches;
        if (*inner) ctx->launches += (*inner)->kernel_launches;
        drop_graph(ctx);  // a captured inner cycle refers to the old solvers' buffers
        outer->reset();
        inner->reset();
        outer->reset(new Gmres<T>(n, m_out, tol, max_restarts, check_true, ctx->stream));
        if (precond_kind == EGX_PRECOND_GMRES) {
            inner->reset(new Gmres<T>(n, m_in, tol, 1, false, ctx->stream));
            // the inner cycle is enqueued whole: its steps never wait for the host
            (*inner)->enqueue_only = true;
        }
        *key = keybuf;
    }
    // Krylov control on the device (default) or, with EGX_KRYLOV_HOST=1 in
    // the environment, the host-driven driver that reads every Gram-Schmidt
    // pass back (the same arithmetic; kept for comparison)
    const char *host_env = getenv("EGX_KRYLOV_HOST");
    const bool host_krylov = host_env && host_env[0] == '1';
    (*outer)->device_control = !host_krylov;
    if (*inner) (*inner)->device_control = !host_krylov;
    // the inner GMRES runs one cycle to the outer tolerance
    // (FlexibleGmresWithGmresPreconditioner.cs:35-44)
    (*outer)->set_tol(tol);
    if (*inner) (*inner)->set_tol(tol);
    int applies = 0;
    auto apply = [ctx, &applies, nrhs](const C<T> *in, C<T> *out) {
        apply_dev<T>(ctx, in, out, nrhs);
        applies++;
    };
    // a device-controlled inner cycle counts its applies on the device (only
    // those that ran while its cycle was live)
    auto apply_inner = [ctx, &applies, nrhs, host_krylov](const C<T> *in, C<T> *out) {
        apply_dev<T>(ctx, in, out, nrhs);
        if (host_krylov) applies++;
    };
    (*outer)->apply = apply;
    (*outer)->timers = &ctx->timers;
    if (precond_kind == EGX_PRECOND_GMRES) {
        (*inner)->apply = apply_inner;
        (*inner)->timers = &ctx->timers;
        Gmres<T> *in = inner->get();
        if (ctx->use_graphs && !host_krylov && !ctx->timers.on) {
            // the inner cycle as one CUDA graph: its input and output staged
            // in fixed buffers, captured once per operator and tolerance
            // (the graph bakes in every pointer and scalar of the cycle)
            const size_t vb = (size_t)n * sizeof(C<T>);
            ctx->pc_in.ensure(vb);
            ctx->pc_out.ensure(vb);
            (*outer)->precond = [ctx, in, vb, tol, nrhs](const C<T> *src, C<T> *dst) {
                C<T> *pin = ctx->pc_in.as<C<T>>(), *pout = ctx->pc_out.as<C<T>>();
                char key[512];
                snprintf(key, sizeof key, "%p/%p/%p/%p/%p/%p/%p/%p/%p/%p/%p/%d/%d/%.17g/%zu/%d/%d", (void *)in, ctx->g,
                         ctx->g->g32.p, ctx->g->g64.p, ctx->r32.p, ctx->r64.p, ctx->buf32.p, ctx->buf64.p,
                         ctx->tw0_32.p, (void *)pin, (void *)pout, ctx->type, nrhs, tol, vb, ctx->fft_tile,
                         ctx->contract_variant);
                EGX_CUDA(cudaMemcpyAsync(pin, src, vb, cudaMemcpyDeviceToDevice, ctx->stream));
                if (ctx->pc_key != key || !ctx->pc_exec) {
                    if (ctx->pc_exec) EGX_CUDA(cudaGraphExecDestroy(ctx->pc_exec));
                    ctx->pc_exec = nullptr;
                    ctx->pc_key.clear();
                    cudaGraph_t graph = nullptr;
                    const long k0 = in->kernel_launches;
                    EGX_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
                    try {
                        in->solve(pin, pin, pout);
                    } catch (...) {
                        cudaStreamEndCapture(ctx->stream, &graph);
                        if (graph) cudaGraphDestroy(graph);
                        throw;
                    }
                    EGX_CUDA(cudaStreamEndCapture(ctx->stream, &graph));
                    const cudaError_t e = cudaGraphInstantiate(&ctx->pc_exec, graph, 0);
                    cudaGraphDestroy(graph);
                    EGX_CUDA(e);
                    ctx->pc_nodes = in->kernel_launches - k0;
                    in->kernel_launches = k0;
                    ctx->pc_key = key;
                }
                EGX_CUDA(cudaGraphLaunch(ctx->pc_exec, ctx->stream));
                ctx->launches += ctx->pc_nodes;
                ctx->pc_replays++;
                EGX_CUDA(cudaMemcpyAsync(dst, pout, vb, cudaMemcpyDeviceToDevice, ctx->stream));
            };
        } else {
            (*outer)->precond = [in](const C<T> *src, C<T> *dst) { in->solve(src, src, dst); };
        }
    } else if (precond_kind == EGX_PRECOND_LEARNED) {
        EGX_CHECK(!dbl && ctx->precond_user, EGX_ERR_STATE, "learned preconditioner without a network");
        // the network is the flexible right preconditioner, z_j = N(v_j), in
        // place of the inner GMRES(m_in) cycle
        // (FlexibleGmresWithGmresPreconditioner.cs:35-57)
        egx_net *net = static_cast<egx_net *>(ctx->precond_user);
        EGX_CHECK(net_length(net) == nvec(ctx), EGX_ERR_INVALID, "learned preconditioner built for another grid");
        (*outer)->precond = [ctx, net, nrhs](const C<T> *src, C<T> *dst) {
            net_apply(net, reinterpret_cast<const float2 *>(src), reinterpret_cast<float2 *>(dst), nrhs, ctx->stream,
                      &ctx->launches);
            if (ctx->learned_inject > 0) {
                // test hook (egx_learned_inject_nonfinite): the host overwrites
                // the network's first output entry with NaN
                static const float2 kNonFinite = make_float2(__builtin_nanf(""), __builtin_nanf(""));
                ctx->learned_inject--;
                EGX_CUDA(cudaMemcpyAsync(dst, &kNonFinite, sizeof(float2), cudaMemcpyHostToDevice, ctx->stream));
            }
        };
    } else if (precond_kind == EGX_PRECOND_CALLBACK) {
        egx_precond_fn fn = ctx->precond_fn;
        void *user = ctx->precond_user;
        cudaStream_t s = ctx->stream;
        const int prec = dbl ? EGX_PREC_FP64 : EGX_PREC_MIXED;
        (*outer)->precond = [fn, user, n, s, prec](const C<T> *src, C<T> *dst) {
            EGX_CUDA(cudaStreamSynchronize(s));
            int rc = fn(user, src, dst, n, prec);
            if (rc != 0) throw Error(EGX_ERR_INVALID, "preconditioner callback failed");
        };
    } else {
        (*outer)->precond = nullptr;
    }
    // the inner cycle is enqueued whole: its applies after a stop are
    // speculative and are not counted (the reference never runs them)
    Gmres<T> *in = inner->get();
    const bool spec = in && in->device_control && in->enqueue_only;
    if (spec) in->reset_apply_counts();
    GmresResult r = (*outer)->solve(b, x, x);
    if (spec) applies += (int)in->live_applies();
    *n_applies = applies;
    return r;
}

}  // namespace

GreenModel green_model(const egx_model *model, double omega) {
    GreenModel gm;
    gm.nx = model->nx;
    gm.ny = model->ny;
    gm.nz = model->nz;
    gm.dx = model->dx;
    gm.dy = model->dy;
    gm.depth.assign(model->layer_depth, model->layer_depth + model->nz);
    gm.thick.assign(model->layer_thickness, model->layer_thickness + model->nz);
    gm.bg_thick.assign(model->bg_thickness, model->bg_thickness + model->n_bg);
    gm.bg_sigma.assign(model->bg_sigma, model->bg_sigma + model->n_bg);
    gm.zero_air_level = model->zero_air_level;
    gm.omega = omega;
    return gm;
}

void ensure_twiddles(egx_ctx *ctx, int n0, int n1) {
    if (ctx->tw_n0 == n0 && ctx->tw_n1 == n1) return;
    ctx->p0 = make_fft_plan(n0);
    ctx->p1 = make_fft_plan(n1);
    upload_twiddles<double>(ctx->tw0_64, n0, ctx->stream);
    upload_twiddles<double>(ctx->tw1_64, n1, ctx->stream);
    upload_twiddles<float>(ctx->tw0_32, n0, ctx->stream);
    upload_twiddles<float>(ctx->tw1_32, n1, ctx->stream);
    ctx->tw_n0 = n0;
    ctx->tw_n1 = n1;
}

void upload_model(egx_ctx *ctx, egx_green *g, const double *zeta, const double *zeta0, int where) {
    const long ncell = (long)g->nx * g->ny;
    ctx->zeta.ensure(ncell * g->nz * sizeof(double2));
    ctx->zeta0.ensure(g->nz * sizeof(double2));
    cudaMemcpyKind kind = where == EGX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    EGX_CUDA(cudaMemcpyAsync(ctx->zeta.p, zeta, ncell * g->nz * sizeof(double2), kind, ctx->stream));
    EGX_CUDA(cudaMemcpyAsync(ctx->zeta0.p, zeta0, g->nz * sizeof(double2), kind, ctx->stream));
}

void prepare_device(egx_ctx *ctx, egx_green *g, const double *dz, int type) {
    EGX_CHECK(type == EGX_OP_A || type == EGX_OP_CHI0, EGX_ERR_INVALID, "unknown operator type");
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    std::vector<cd> z0(nz);
    EGX_CUDA(cudaMemcpyAsync(z0.data(), ctx->zeta0.p, nz * sizeof(cd), cudaMemcpyDeviceToHost, ctx->stream));
    EGX_CUDA(cudaStreamSynchronize(ctx->stream));
    // PrepareForwardFactors / PrepareBackwardFactors (ConvolutionOperator.cs:90-111)
    std::vector<cd> fwd(nz), bwd(nz);
    const cd norm(1.0 / ((double)nx * (double)ny * 4), 0);
    for (int k = 0; k < nz; k++) {
        EGX_CHECK(dz[k] > 0, EGX_ERR_INVALID, "layer thickness must be positive");
        fwd[k] = cd(std::sqrt(z0[k].real()), 0);
        cd sc(2 * std::sqrt(z0[k].real()), 0);
        sc /= dz[k];
        sc *= norm;
        bwd[k] = sc;
    }
    const long ncell = (long)nx * ny;
    ctx->r64.ensure(ncell * nz * sizeof(double2));
    ctx->fwd64.ensure(nz * sizeof(double2));
    ctx->bwd64.ensure(nz * sizeof(double2));
    EGX_CUDA(cudaMemcpyAsync(ctx->fwd64.p, fwd.data(), nz * sizeof(cd), cudaMemcpyHostToDevice, ctx->stream));
    EGX_CUDA(cudaMemcpyAsync(ctx->bwd64.p, bwd.data(), nz * sizeof(cd), cudaMemcpyHostToDevice, ctx->stream));
    float2 *r32 = nullptr;
    if (g->has32) {
        ctx->r32.ensure(ncell * nz * sizeof(float2));
        ctx->fwd32.ensure(nz * sizeof(float2));
        ctx->bwd32.ensure(nz * sizeof(float2));
        r32 = ctx->r32.as<float2>();
    }
    long n = ncell * nz;
    k_prepare_r<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(ctx->zeta.as<double2>(), ctx->zeta0.as<double2>(),
                                                                      nz, ncell, type, ctx->r64.as<double2>(), r32);
    ctx->launches++;
    if (g->has32) {
        convert_d2f(ctx->fwd64.as<double2>(), ctx->fwd32.as<float2>(), nz, 1.0, ctx->stream);
        convert_d2f(ctx->bwd64.as<double2>(), ctx->bwd32.as<float2>(), nz, 1.0, ctx->stream);
        ctx->launches += 2;
    }
    EGX_CUDA(cudaGetLastError());
    ctx->prepared32 = g->has32;
    ensure_twiddles(ctx, 2 * nx, 2 * ny);
    ctx->g = g;
    ctx->type = type;
    ctx->nx = nx;
    ctx->ny = ny;
    ctx->nz = nz;
}

template <typename T>
void apply_dev(egx_ctx *ctx, const C<T> *x, C<T> *y, int nrhs, bool ds) {
    EGX_CHECK(ctx->g && ctx->type >= 0, EGX_ERR_STATE, "operator is not prepared (PrepareOperator not called)");
    OpDims d{ctx->nx, ctx->ny, ctx->nz, nrhs, nrhs * 3 * ctx->nz, nvec(ctx)};
    d.ds = ds ? 1 : 0;
    if (sizeof(T) == sizeof(float)) {  // the apply tuner's choices (egx_tune_apply)
        d.fft_tile = ctx->fft_tile;
        d.contract_variant = ctx->contract_variant;
    }
    size_t bufbytes = (size_t)4 * ctx->nx * ctx->ny * d.B * sizeof(C<T>);
    const bool dbl = sizeof(T) == sizeof(double);
    DevBuf &buf = dbl ? ctx->buf64 : ctx->buf32;
    buf.ensure(bufbytes);
    OperatorData<T> op;
    if (dbl) {
        op.r = (const C<T> *)ctx->r64.p;
        op.fwd = (const C<T> *)ctx->fwd64.p;
        op.bwd = (const C<T> *)ctx->bwd64.p;
    } else {
        EGX_CHECK(ctx->g->has32 && ctx->prepared32, EGX_ERR_STATE, "complex64 operator is not available");
        op.r = (const C<T> *)ctx->r32.p;
        op.fwd = (const C<T> *)ctx->fwd32.p;
        op.bwd = (const C<T> *)ctx->bwd32.p;
    }
    op.type = ctx->type;
    const C<T> *G = dbl ? (const C<T> *)ctx->g->g64.p : (const C<T> *)ctx->g->g32.p;
    const C<T> *tw0 = dbl ? (const C<T> *)ctx->tw0_64.p : (const C<T> *)ctx->tw0_32.p;
    const C<T> *tw1 = dbl ? (const C<T> *)ctx->tw1_64.p : (const C<T> *)ctx->tw1_32.p;
    operator_apply<T>(d, op, G, x, y, buf.as<C<T>>(), tw0, tw1, ctx->p0, ctx->p1, ctx->stream, &ctx->launches,
                      &ctx->timers, ctx->errflag.as<int>());
}
template void apply_dev<double>(egx_ctx *, const C<double> *, C<double> *, int, bool);
template void apply_dev<float>(egx_ctx *, const C<float> *, C<float> *, int, bool);

GmresResult fgmres_dev(egx_ctx *ctx, const double2 *b, double2 *x, const egx_gmres_params &p, int *applies) {
    EGX_CHECK(p.m_out >= 1 && p.m_in >= 1 && p.max_restarts >= 1 && p.tol > 0, EGX_ERR_INVALID,
              "bad GMRES parameters");
    int kind = p.precond;
    if (kind == EGX_PRECOND_GMRES && ctx->precond_kind == EGX_PRECOND_CALLBACK) kind = EGX_PRECOND_CALLBACK;
    if (ctx->precond_kind == EGX_PRECOND_NONE) kind = EGX_PRECOND_NONE;
    return run_fgmres<double>(ctx, b, x, p.m_out, p.m_in, p.tol, p.max_restarts, p.check_true != 0, kind, applies);
}

// Outer FP64 iterative refinement: r = b - A x (complex128 apply), inner
// complex64 FGMRES on A d = r/||r||, x += ||r|| d, until ||r||/||b|| < tol.
// The inner relative tolerance of a refinement at true residual be is
// max(inner_tol, min(0.5, kInnerSafety * tol / be)).
//
// nrhs > 1 solves the nrhs systems A x_i = b_i ([nrhs][nvec] blocks) as one
// stacked block-diagonal system: each block's residual is scaled to unit norm
// before the inner solve, the inner tolerance is divided by sqrt(nrhs) (a
// stacked residual below itol * sqrt(nrhs) bounds every block's by the same),
// every apply is one nrhs-vector apply, and the refinement stops when every
// block's own complex128 residual is below tol. true_be[i] per block.
// Failure-detection check: a barrier that nothing completes, waited on
// through the bounded wait of the TMA-fed kernels.
__global__ void k_wait_probe(uint64_t limit_ns, int *err) {
    __shared__ __align__(8) uint64_t bar;
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const bool done = mbar_wait_ns(b, 0, limit_ns);  // phase 0 never completes
    if (__syncthreads_or(!done) && threadIdx.x == 0) atomicExch(err, EGX_ERR_TIMEOUT);
}

static const double kInnerSafety = 0.3;
GmresResult mixed_dev(egx_ctx *ctx, const double2 *b, double2 *x, const egx_mixed_params &p, int *applies,
                      int *refinements, double *true_be, int nrhs) {
    EGX_CHECK(p.m_out >= 1 && p.m_in >= 1 && p.max_outer >= 1 && p.tol > 0 && p.inner_tol > 0 &&
                  p.inner_restarts >= 1 && nrhs >= 1,
              EGX_ERR_INVALID, "bad mixed-solve parameters");
    EGX_CHECK(ctx->g->has32 && ctx->prepared32, EGX_ERR_STATE,
              "mixed solve needs a Green tensor built or uploaded with EGX_PREC_MIXED");
    const long n = nvec(ctx), N = n * nrhs;
    ctx->mix_r.ensure(N * sizeof(double2));
    ctx->mix_t.ensure(N * sizeof(double2));
    ctx->mix_r32.ensure(N * sizeof(float2));
    ctx->mix_d32.ensure(N * sizeof(float2));
    ctx->nrm_part.ensure(2048 * sizeof(double));
    ctx->nrm_out.ensure(sizeof(double));
    double2 *r = ctx->mix_r.as<double2>(), *t = ctx->mix_t.as<double2>();
    float2 *r32 = ctx->mix_r32.as<float2>(), *d32 = ctx->mix_d32.as<float2>();
    auto norm64 = [&](const double2 *v, long len) {
        VecOps<double>::norm2(v, len, ctx->nrm_out.as<double>(), ctx->nrm_part.as<double>(), 1024, ctx->stream);
        ctx->launches += 2;
        double h;
        EGX_CUDA(cudaMemcpyAsync(&h, ctx->nrm_out.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        return std::sqrt(h);
    };
    std::vector<double> bn(nrhs), rn(nrhs), be(nrhs);
    // max over the blocks with a nonzero right-hand side (a zero block has x = 0)
    auto residuals = [&](const double2 *rv) {
        double m = 0;
        for (int i = 0; i < nrhs; i++) {
            rn[i] = bn[i] > 0 ? norm64(rv + i * n, n) : 0.0;
            be[i] = bn[i] > 0 ? rn[i] / bn[i] : 0.0;
            m = std::max(m, be[i]);
        }
        return m;
    };
    int applies64 = 0, applies32 = 0;
    GmresResult out;
    bool any = false;
    for (int i = 0; i < nrhs; i++) {
        bn[i] = norm64(b + i * n, n);
        if (bn[i] == 0) VecOps<double>::zero(x + i * n, n, ctx->stream);
        any = any || bn[i] > 0;
    }
    if (!any) {
        out.converged = true;
        *applies = 0;
        *refinements = 0;
        for (int i = 0; i < nrhs; i++) true_be[i] = 0;
        return out;
    }
    // r = b - A x; a zero initial guess needs no complex128 apply
    double bemax;
    if (norm64(x, N) == 0) {
        EGX_CUDA(cudaMemcpyAsync(r, b, N * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream));
        bemax = residuals(r);
    } else {
        apply_dev<double>(ctx, x, t, nrhs, true);
        applies64++;
        VecOps<double>::sub(b, t, r, N, ctx->stream);
        ctx->launches++;
        bemax = residuals(r);
    }
    int k = 0;
    bool conv = bemax < p.tol;
    while (!conv && k < p.max_outer) {
        for (int i = 0; i < nrhs; i++) convert_d2f(r + i * n, r32 + i * n, n, rn[i] > 0 ? 1.0 / rn[i] : 0.0, ctx->stream);
        VecOps<float>::zero(d32, N, ctx->stream);
        ctx->launches += 1 + nrhs;
        int a32 = 0;
        // ask the inner solve only for the reduction still needed (with a
        // safety factor), never for less than inner_tol
        double itol = std::max(p.inner_tol, std::min(0.5, kInnerSafety * p.tol / bemax)) / std::sqrt((double)nrhs);
        GmresResult ir;
        bool done = false;
        if (ctx->precond_kind == EGX_PRECOND_LEARNED) {
            // the network as the flexible preconditioner, at most four
            // FGMRES cycles; then the GMRES-preconditioned solve from zero
            // (the fallback)
            ctx->learned_uses++;
            ir = run_fgmres<float>(ctx, r32, d32, p.m_out, p.m_in, itol, std::min(p.inner_restarts, 4), false,
                                   EGX_PRECOND_LEARNED, &a32, nrhs);
            done = ir.converged;
            if (!done) {
                ctx->learned_fallbacks++;
                applies32 += a32;
                out.iterations += ir.iterations;
                VecOps<float>::zero(d32, N, ctx->stream);
                ctx->launches++;
            }
        }
        if (!done)
            ir = run_fgmres<float>(ctx, r32, d32, p.m_out, p.m_in, itol, p.inner_restarts, false,
                                   ctx->precond_kind == EGX_PRECOND_NONE ? EGX_PRECOND_NONE : EGX_PRECOND_GMRES, &a32,
                                   nrhs);
        applies32 += a32;
        out.iterations += ir.iterations;
        out.arnoldi_be = ir.arnoldi_be;
        for (int i = 0; i < nrhs; i++) convert_f2d_add(d32 + i * n, x + i * n, n, rn[i], ctx->stream);
        apply_dev<double>(ctx, x, t, nrhs, true);
        applies64++;
        VecOps<double>::sub(b, t, r, N, ctx->stream);
        ctx->launches += 1 + nrhs;
        bemax = residuals(r);
        k++;
        conv = bemax < p.tol;
    }
    out.converged = conv;
    out.true_be = bemax;
    *applies = applies64 + applies32;
    *refinements = k;
    for (int i = 0; i < nrhs; i++) true_be[i] = be[i];
    return out;
}

}  // namespace egx

extern "C" {

int egx_version(void) { return 1; }

long egx_device_allocations(void) { return egx::device_allocations().load(); }

int egx_create(int device, egx_ctx **out) {
    if (!out) return EGX_ERR_INVALID;
    *out = nullptr;
    auto *ctx = new egx_ctx();
    ctx->device = device;
    try {
        set_device(ctx);
        EGX_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->own_stream = true;
        ctx->errflag.ensure(sizeof(int));
        EGX_CUDA(cudaMemset(ctx->errflag.p, 0, sizeof(int)));
    } catch (const egx::Error &e) {
        delete ctx;
        return e.code;
    }
    *out = ctx;
    return EGX_OK;
}

int egx_destroy(egx_ctx *ctx) {
    if (!ctx) return EGX_ERR_INVALID;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->timers.flush();
    drop_graph(ctx);
    ctx->outer64.reset();
    ctx->inner64.reset();
    ctx->outer32.reset();
    ctx->inner32.reset();
    ctx->outer32l.reset();
    ctx->inner32l.reset();
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return EGX_OK;
}

int egx_last_error(egx_ctx *ctx, char *buf, size_t len) {
    if (!ctx || !buf || len == 0) return EGX_ERR_INVALID;
    std::strncpy(buf, ctx->err.c_str(), len - 1);
    buf[len - 1] = 0;
    return EGX_OK;
}

int egx_set_stream(egx_ctx *ctx, void *stream) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        set_device(ctx);
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->timers.flush();
        if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
        ctx->stream = (cudaStream_t)stream;
        ctx->own_stream = false;
        // the solvers keep the stream they were made with
        drop_graph(ctx);
        ctx->outer64.reset();
        ctx->inner64.reset();
        ctx->outer32.reset();
        ctx->inner32.reset();
        ctx->outer32l.reset();
        ctx->inner32l.reset();
        ctx->key64.clear();
        ctx->key32.clear();
        ctx->key32l.clear();
    });
}

int egx_set_graphs(egx_ctx *ctx, int enable) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        set_device(ctx);
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        drop_graph(ctx);
        ctx->use_graphs = enable ? 1 : 0;
    });
}

int egx_tune_apply(egx_ctx *ctx, int nrhs, int reps, double *ms_out) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(nrhs >= 1 && nrhs <= 16 && reps >= 1 && reps <= 100, EGX_ERR_INVALID, "bad tuning arguments");
        EGX_CHECK(ctx->g && ctx->type >= 0 && ctx->prepared32, EGX_ERR_STATE,
                  "tuning needs an operator prepared with a complex64 Green tensor");
        set_device(ctx);
        const long n = nvec(ctx) * nrhs;
        DevBuf xb, yb;
        xb.ensure(n * sizeof(float2));
        yb.ensure(n * sizeof(float2));
        EGX_CUDA(cudaMemsetAsync(xb.p, 0, n * sizeof(float2), ctx->stream));
        const bool was_on = ctx->timers.on;
        ctx->timers.on = false;
        cudaEvent_t a, b;
        EGX_CUDA(cudaEventCreate(&a));
        EGX_CUDA(cudaEventCreate(&b));
        double best = 1e300;
        int bt = 0, bv = 0;
        // three contraction kernels to choose from in either Green layout:
        // packed (tensor-core, TMA-staged CUDA-core, generic) or sub-block
        // for nz in 16, 32, 48 (built-in FP16 split by role, TF32 split,
        // FP16 split in lockstep)
        const int nvar = 3;
        for (int tile = 0; tile < 3; tile++)
            for (int var = 0; var < nvar; var++) {
                ctx->fft_tile = tile;
                ctx->contract_variant = var;
                apply_dev<float>(ctx, xb.as<float2>(), yb.as<float2>(), nrhs);  // untimed first run
                EGX_CUDA(cudaEventRecord(a, ctx->stream));
                for (int r = 0; r < reps; r++) apply_dev<float>(ctx, xb.as<float2>(), yb.as<float2>(), nrhs);
                EGX_CUDA(cudaEventRecord(b, ctx->stream));
                EGX_CUDA(cudaEventSynchronize(b));
                float ms = 0;
                EGX_CUDA(cudaEventElapsedTime(&ms, a, b));
                const double per = ms / reps;
                if (ms_out) ms_out[tile * 3 + var] = per;
                if (per < best) {
                    best = per;
                    bt = tile;
                    bv = var;
                }
            }
        if (ms_out)
            for (int var = nvar; var < 3; var++)
                for (int tile = 0; tile < 3; tile++) ms_out[tile * 3 + var] = -1;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        ctx->fft_tile = bt;
        ctx->contract_variant = bv;
        ctx->timers.on = was_on;
        check_device_error(ctx);
    });
}

int egx_apply_variant(egx_ctx *ctx, int fft_tile, int contract_variant) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(fft_tile >= 0 && fft_tile <= 2 && contract_variant >= 0 && contract_variant <= 2, EGX_ERR_INVALID,
                  "fft_tile and contract_variant must be in 0..2");
        ctx->fft_tile = fft_tile;
        ctx->contract_variant = contract_variant;
    });
}

int egx_graph_stats(egx_ctx *ctx, long *replays, long *nodes) {
    if (!ctx) return EGX_ERR_INVALID;
    if (replays) *replays = ctx->pc_replays;
    if (nodes) *nodes = ctx->pc_nodes;
    return EGX_OK;
}

long egx_launch_count(egx_ctx *ctx) {
    if (!ctx) return -1;
    long n = ctx->launches;
    if (ctx->outer64) n += ctx->outer64->kernel_launches;
    if (ctx->inner64) n += ctx->inner64->kernel_launches;
    if (ctx->outer32) n += ctx->outer32->kernel_launches;
    if (ctx->inner32) n += ctx->inner32->kernel_launches;
    return n;
}

int egx_profile(egx_ctx *ctx, int enable) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        set_device(ctx);
        ctx->timers.reset();
        ctx->timers.on = enable != 0;
    });
}

int egx_profile_kinds(egx_ctx *ctx, unsigned mask) {
    if (!ctx) return EGX_ERR_INVALID;
    ctx->timers.mask = mask;
    return EGX_OK;
}

int egx_profile_read(egx_ctx *ctx, int kind, long *launches, double *total_ms) {
    if (!ctx || !launches || !total_ms || kind < 0 || kind >= Timers::kKinds) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        set_device(ctx);
        ctx->timers.flush();
        *launches = ctx->timers.count[kind];
        *total_ms = ctx->timers.total_ms[kind];
    });
}

int egx_green_build(egx_ctx *ctx, const egx_model *model, double omega, int n_hankels, int precision,
                    egx_green **out) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(model && out, EGX_ERR_INVALID, "null model or output");
        EGX_CHECK(model->layer_depth && model->layer_thickness && model->bg_thickness && model->bg_sigma,
                  EGX_ERR_INVALID, "null model arrays");
        EGX_CHECK(omega > 0, EGX_ERR_INVALID, "omega must be positive");
        set_device(ctx);
        GreenModel gm = green_model(model, omega);
        auto g = std::unique_ptr<egx_green>(new egx_green());
        g->nx = gm.nx;
        g->ny = gm.ny;
        g->nz = gm.nz;
        GreenBuildStats st;
        g->g64.swap(ctx->spare64);  // storage of the last freed tensor, if any
        // the mixed form transforms the FP64 face integrals laterally in complex64
        build_green(gm, n_hankels, ctx->stream, g->g64, &st, &ctx->launches, &ctx->timers, &ctx->gws,
                    precision == EGX_PREC_MIXED);
        if (precision == EGX_PREC_MIXED) {
            GreenDims gd{gm.nx, gm.ny, gm.nz};
            g->g32.swap(ctx->spare32);
            g->g32.ensure(green_c64_entries(gd) * sizeof(float2));
            green_to_c64(g->g64.as<double2>(), g->g32.as<float2>(), gd, ctx->stream, &ctx->launches);
            g->has32 = true;
        }
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->last_build = st;
        *out = g.release();
    });
}

int egx_green_upload(egx_ctx *ctx, int nx, int ny, int nz, const double *const comps[6], int precision,
                     egx_green **out) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(out && comps && nx > 0 && ny > 0 && nz > 0, EGX_ERR_INVALID, "bad Green tensor arguments");
        for (int c = 0; c < 6; c++) EGX_CHECK(comps[c], EGX_ERR_INVALID, "null Green tensor component");
        set_device(ctx);
        std::vector<cd> q;
        gather_quadrant(nx, ny, nz, comps, q);
        auto g = std::unique_ptr<egx_green>(new egx_green());
        g->nx = nx;
        g->ny = ny;
        g->nz = nz;
        g->g64.ensure(q.size() * sizeof(cd));
        EGX_CUDA(cudaMemcpyAsync(g->g64.p, q.data(), q.size() * sizeof(cd), cudaMemcpyHostToDevice, ctx->stream));
        if (precision == EGX_PREC_MIXED) {
            GreenDims gd{nx, ny, nz};
            g->g32.ensure(green_c64_entries(gd) * sizeof(float2));
            green_to_c64(g->g64.as<double2>(), g->g32.as<float2>(), gd, ctx->stream, &ctx->launches);
            g->has32 = true;
        }
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        *out = g.release();
    });
}

int egx_green_download(egx_ctx *ctx, const egx_green *g, double *const comps[6]) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(g && comps, EGX_ERR_INVALID, "bad arguments");
        set_device(ctx);
        GreenDims gd{g->nx, g->ny, g->nz};
        const int S = gd.S(), A = gd.A(), Bs = gd.Bs(), lda = gd.lda(), nz = g->nz;
        const size_t qn = (size_t)gd.Q() * Bs;
        std::unique_ptr<cd[]> qbuf(static_cast<cd *>(::operator new[](qn * sizeof(cd))));
        cd *q = qbuf.get();
        EGX_CUDA(cudaMemcpyAsync(q, g->g64.p, qn * sizeof(cd), cudaMemcpyDeviceToHost, ctx->stream));
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        const int blk[6] = {S, S, S, S, nz * nz, nz * nz};
        const int off[6] = {0, S, 2 * S, 3 * S, 4 * S, 4 * S + A};
        // parity (x, y) of xx, xy, yy, zz, xz, yz
        const int px[6] = {1, -1, 1, 1, -1, 1}, py[6] = {1, -1, 1, 1, 1, -1};
        const int n0 = 2 * g->nx, n1 = 2 * g->ny;
        // rows kx split over host threads (the reference layout of a large
        // tensor is tens of GB)
        auto rows = [&](int k0, int k1) {
          for (int kx = k0; kx < k1; kx++)
            for (int ky = 0; ky < n1; ky++) {
                int a = kx <= g->nx ? kx : n0 - kx;
                int b = ky <= g->ny ? ky : n1 - ky;
                bool mx = kx > g->nx, my = ky > g->ny;
                long qi = (long)a * (g->ny + 1) + b;
                long pt = (long)kx * n1 + ky;
                for (int c = 0; c < 6; c++) {
                    double sg = (mx ? px[c] : 1) * (my ? py[c] : 1);
                    cd *dst = reinterpret_cast<cd *>(comps[c]) + pt * blk[c];
                    const cd *src = &q[qi * Bs + off[c]];
                    if (c < 4) {
                        for (int t = 0; t < blk[c]; t++) dst[t] = sg * src[t];
                    } else {
                        for (int rc = 0; rc < nz; rc++)
                            for (int tr = 0; tr < nz; tr++) dst[rc * nz + tr] = sg * src[rc * lda + tr];
                    }
                }
            }
        };
        const long work = (long)n0 * n1 * Bs;
        const int nt = work < (1L << 22) ? 1 : std::max(1, std::min(n0, (int)std::thread::hardware_concurrency()));
        if (nt == 1) {
            rows(0, n0);
        } else {
            std::vector<std::thread> pool;
            for (int t = 0; t < nt; t++) pool.emplace_back(rows, (int)((long)n0 * t / nt), (int)((long)n0 * (t + 1) / nt));
            for (auto &th : pool) th.join();
        }
    });
}

int egx_green_free(egx_ctx *ctx, egx_green *g) {
    if (!ctx || !g) return EGX_ERR_INVALID;
    if (ctx->g == g) {
        ctx->g = nullptr;
        ctx->type = -1;
    }
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    // keep the storage for the next build in this context (a build usually
    // follows, one frequency after another); egx_destroy releases it
    if (!ctx->spare64.p) ctx->spare64.swap(g->g64);
    if (!ctx->spare32.p) ctx->spare32.swap(g->g32);
    delete g;
    return EGX_OK;
}

int egx_op_prepare(egx_ctx *ctx, egx_green *g, const double *zeta, const double *zeta0, const double *dz, int type) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(g, EGX_ERR_INVALID, "greenTensor is null");
        EGX_CHECK(zeta && zeta0 && dz, EGX_ERR_INVALID, "null model arrays");
        set_device(ctx);
        upload_model(ctx, g, zeta, zeta0, EGX_HOST);
        prepare_device(ctx, g, dz, type);
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int egx_op_apply(egx_ctx *ctx, const double *x, double *y, int nrhs, int where) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(x && y && nrhs >= 1, EGX_ERR_INVALID, "bad apply arguments");
        set_device(ctx);
        EGX_CHECK(ctx->g, EGX_ERR_STATE, "operator is not prepared");
        long n = nvec(ctx) * nrhs;
        if (where == EGX_DEVICE) {
            apply_dev<double>(ctx, (const double2 *)x, (double2 *)y, nrhs);
        } else {
            ctx->xin.ensure(n * sizeof(double2));
            ctx->yout.ensure(n * sizeof(double2));
            EGX_CUDA(cudaMemcpyAsync(ctx->xin.p, x, n * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
            apply_dev<double>(ctx, ctx->xin.as<double2>(), ctx->yout.as<double2>(), nrhs);
            EGX_CUDA(cudaMemcpyAsync(y, ctx->yout.p, n * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
        }
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        check_device_error(ctx);
    });
}

int egx_op_apply_ds(egx_ctx *ctx, const double *x, double *y, int nrhs, int where) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(x && y && nrhs >= 1, EGX_ERR_INVALID, "bad apply arguments");
        set_device(ctx);
        EGX_CHECK(ctx->g, EGX_ERR_STATE, "operator is not prepared");
        long n = nvec(ctx) * nrhs;
        if (where == EGX_DEVICE) {
            apply_dev<double>(ctx, (const double2 *)x, (double2 *)y, nrhs, true);
        } else {
            ctx->xin.ensure(n * sizeof(double2));
            ctx->yout.ensure(n * sizeof(double2));
            EGX_CUDA(cudaMemcpyAsync(ctx->xin.p, x, n * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
            apply_dev<double>(ctx, ctx->xin.as<double2>(), ctx->yout.as<double2>(), nrhs, true);
            EGX_CUDA(cudaMemcpyAsync(y, ctx->yout.p, n * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
        }
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        check_device_error(ctx);
    });
}

int egx_op_apply_c64(egx_ctx *ctx, const float *x, float *y, int nrhs, int where) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(x && y && nrhs >= 1, EGX_ERR_INVALID, "bad apply arguments");
        set_device(ctx);
        EGX_CHECK(ctx->g, EGX_ERR_STATE, "operator is not prepared");
        long n = nvec(ctx) * nrhs;
        if (where == EGX_DEVICE) {
            apply_dev<float>(ctx, (const float2 *)x, (float2 *)y, nrhs);
        } else {
            ctx->xin32.ensure(n * sizeof(float2));
            ctx->yout32.ensure(n * sizeof(float2));
            EGX_CUDA(cudaMemcpyAsync(ctx->xin32.p, x, n * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream));
            apply_dev<float>(ctx, ctx->xin32.as<float2>(), ctx->yout32.as<float2>(), nrhs);
            EGX_CUDA(cudaMemcpyAsync(y, ctx->yout32.p, n * sizeof(float2), cudaMemcpyDeviceToHost, ctx->stream));
        }
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        check_device_error(ctx);
    });
}

int egx_fft2d(egx_ctx *ctx, double *buf, int n0, int n1, int howmany, int sign, int where) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(buf && n0 > 0 && n1 > 0 && howmany > 0, EGX_ERR_INVALID, "bad FFT arguments");
        EGX_CHECK(sign == -1 || sign == 1, EGX_ERR_INVALID, "sign must be -1 or +1");
        set_device(ctx);
        FftPlan p0 = make_fft_plan(n0), p1 = make_fft_plan(n1);
        DevBuf t0, t1;
        upload_twiddles<double>(t0, n0, ctx->stream);
        upload_twiddles<double>(t1, n1, ctx->stream);
        long n = (long)n0 * n1 * howmany;
        double2 *dbuf;
        if (where == EGX_DEVICE) {
            dbuf = (double2 *)buf;
        } else {
            ctx->fftbuf.ensure(n * sizeof(double2));
            dbuf = ctx->fftbuf.as<double2>();
            EGX_CUDA(cudaMemcpyAsync(dbuf, buf, n * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
        }
        fft2d<double>(dbuf, n0, n1, howmany, sign, t0.as<double2>(), t1.as<double2>(), p0, p1, ctx->stream,
                      &ctx->launches);
        if (where != EGX_DEVICE)
            EGX_CUDA(cudaMemcpyAsync(buf, dbuf, n * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int egx_set_precond(egx_ctx *ctx, int kind, egx_precond_fn fn, void *user) {
    if (!ctx) return EGX_ERR_INVALID;
    if (kind != EGX_PRECOND_GMRES && kind != EGX_PRECOND_CALLBACK && kind != EGX_PRECOND_NONE &&
        kind != EGX_PRECOND_LEARNED)
        return fail(ctx, EGX_ERR_INVALID, "unknown preconditioner kind");
    if (kind == EGX_PRECOND_CALLBACK && !fn) return fail(ctx, EGX_ERR_INVALID, "callback preconditioner without fn");
    if (kind == EGX_PRECOND_LEARNED && !user) return fail(ctx, EGX_ERR_INVALID, "learned preconditioner without net");
    ctx->precond_kind = kind;
    ctx->precond_fn = fn;
    ctx->precond_user = user;
    return EGX_OK;
}

int egx_fgmres_solve(egx_ctx *ctx, const double *b, double *x, const egx_gmres_params *p, egx_result *res,
                     int where) {
    if (!ctx) return EGX_ERR_INVALID;
    int status = EGX_OK;
    try {
        EGX_CHECK(b && x && p && res, EGX_ERR_INVALID, "bad solve arguments");
        set_device(ctx);
        EGX_CHECK(ctx->g && ctx->type >= 0, EGX_ERR_STATE, "operator is not prepared");
        const long n = nvec(ctx);
        const double2 *db;
        double2 *dx;
        if (where == EGX_DEVICE) {
            db = (const double2 *)b;
            dx = (double2 *)x;
        } else {
            ctx->xin.ensure(2 * n * sizeof(double2));
            db = ctx->xin.as<double2>();
            dx = ctx->xin.as<double2>() + n;
            EGX_CUDA(cudaMemcpyAsync((void *)db, b, n * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
            EGX_CUDA(cudaMemcpyAsync(dx, x, n * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
        }
        int applies = 0;
        GmresResult r = fgmres_dev(ctx, db, dx, *p, &applies);
        if (where != EGX_DEVICE)
            EGX_CUDA(cudaMemcpyAsync(x, dx, n * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        check_device_error(ctx);
        res->converged = r.converged;
        res->iterations = r.iterations;
        res->arnoldi_be = r.arnoldi_be;
        res->true_be = r.true_be;
        res->n_applies = applies;
        res->n_refinements = 0;
        if (!r.converged) status = fail(ctx, EGX_ERR_NOT_CONVERGED, "FGMRES did not converge");
    } catch (const egx::Error &e) {
        return fail(ctx, e.code, e.what());
    } catch (const std::exception &e) {
        return fail(ctx, EGX_ERR_INVALID, e.what());
    }
    return status;
}

int egx_mixed_solve(egx_ctx *ctx, const double *b, double *x, const egx_mixed_params *p, egx_result *res,
                    int where) {
    if (!ctx) return EGX_ERR_INVALID;
    int status = EGX_OK;
    try {
        EGX_CHECK(b && x && p && res, EGX_ERR_INVALID, "bad solve arguments");
        set_device(ctx);
        EGX_CHECK(ctx->g && ctx->type >= 0, EGX_ERR_STATE, "operator is not prepared");
        const long n = nvec(ctx);
        const double2 *db;
        double2 *dx;
        if (where == EGX_DEVICE) {
            db = (const double2 *)b;
            dx = (double2 *)x;
        } else {
            ctx->xin.ensure(2 * n * sizeof(double2));
            db = ctx->xin.as<double2>();
            dx = ctx->xin.as<double2>() + n;
            EGX_CUDA(cudaMemcpyAsync((void *)db, b, n * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
            EGX_CUDA(cudaMemcpyAsync(dx, x, n * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
        }
        int applies = 0, refinements = 0;
        double tbe = -1;
        GmresResult r = mixed_dev(ctx, db, dx, *p, &applies, &refinements, &tbe);
        if (where != EGX_DEVICE)
            EGX_CUDA(cudaMemcpyAsync(x, dx, n * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        check_device_error(ctx);
        res->converged = r.converged;
        res->iterations = r.iterations;
        res->arnoldi_be = r.arnoldi_be;
        res->true_be = tbe;
        res->n_applies = applies;
        res->n_refinements = refinements;
        if (!r.converged) status = fail(ctx, EGX_ERR_NOT_CONVERGED, "mixed-precision refinement did not converge");
    } catch (const egx::Error &e) {
        return fail(ctx, e.code, e.what());
    } catch (const std::exception &e) {
        return fail(ctx, EGX_ERR_INVALID, e.what());
    }
    return status;
}

int egx_learned_inject_nonfinite(egx_ctx *ctx, int count) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(count >= 0, EGX_ERR_INVALID, "injection count must be >= 0");
        ctx->learned_inject = count;
    });
}

int egx_learned_stats(egx_ctx *ctx, long *uses, long *fallbacks) {
    if (!ctx) return EGX_ERR_INVALID;
    if (uses) *uses = ctx->learned_uses;
    if (fallbacks) *fallbacks = ctx->learned_fallbacks;
    return EGX_OK;
}

int egx_wait_selftest(egx_ctx *ctx, double limit_ms) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(limit_ms >= 1 && limit_ms <= 2000, EGX_ERR_INVALID, "limit_ms must be in [1, 2000]");
        set_device(ctx);
        k_wait_probe<<<1, 32, 0, ctx->stream>>>((uint64_t)(limit_ms * 1e6), ctx->errflag.as<int>());
        ctx->launches++;
        EGX_CUDA(cudaGetLastError());
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
        check_device_error(ctx);  // EGX_ERR_TIMEOUT when the wait gave up; clears the flag
    });
}

int egx_dot_products(egx_ctx *ctx, const double *V, int ncols, const double *w, long n, double *out, int where) {
    if (!ctx) return EGX_ERR_INVALID;
    EGX_GUARD(ctx, {
        EGX_CHECK(V && w && out && ncols >= 1 && ncols <= 64 && n >= 1, EGX_ERR_INVALID,
                  "bad dot-product arguments");
        set_device(ctx);
        const double2 *dV, *dw;
        if (where == EGX_DEVICE) {
            EGX_CHECK(aligned16(V) && aligned16(w) && aligned16(out), EGX_ERR_INVALID,
                      "egx_dot_products: device V, w and out must be 16-byte aligned");
            dV = (const double2 *)V;
            dw = (const double2 *)w;
        } else {
            ctx->xin.ensure((size_t)(ncols + 1) * n * sizeof(double2));
            double2 *stage = ctx->xin.as<double2>();
            EGX_CUDA(cudaMemcpyAsync(stage, V, (size_t)ncols * n * sizeof(double2), cudaMemcpyHostToDevice,
                                     ctx->stream));
            EGX_CUDA(cudaMemcpyAsync(stage + (size_t)ncols * n, w, n * sizeof(double2), cudaMemcpyHostToDevice,
                                     ctx->stream));
            dV = stage;
            dw = stage + (size_t)ncols * n;
        }
        int nblocks = (int)std::min<long>(1024, (n + 255) / 256);
        ctx->nrm_part.ensure((size_t)nblocks * 64 * sizeof(double2));
        ctx->yout.ensure(64 * sizeof(double2));
        VecOps<double>::multi_dot(dV, ncols, dw, n, ctx->yout.as<double2>(), ctx->nrm_part.as<double2>(), nblocks,
                                  ctx->stream);
        ctx->launches += 2;
        cudaMemcpyKind k = where == EGX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        EGX_CUDA(cudaMemcpyAsync(out, ctx->yout.p, ncols * sizeof(double2), k, ctx->stream));
        EGX_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

}  // extern "C"
