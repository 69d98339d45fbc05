// The egx_ctx / egx_green objects behind the C ABI and the per-kernel timers.
#pragma once

#include <complex>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "egx_green.cuh"
#include "egx_krylov.cuh"
#include "egx_operator.cuh"

struct egx_green {
    int nx = 0, ny = 0, nz = 0;
    egx::DevBuf g64;  // quadrant, complex128
    egx::DevBuf g32;  // quadrant, complex64 (mixed precision)
    bool has32 = false;
};

struct egx_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    long launches = 0;
    egx::Timers timers;
    // Green-tensor build workspace, and the storage of the last freed tensor
    // (reused by the next build of the same size; released by egx_destroy)
    egx::GreenWorkspace gws;
    egx::DevBuf spare64, spare32;

    // prepared operator
    egx_green *g = nullptr;
    int type = -1;
    int nx = 0, ny = 0, nz = 0;
    egx::DevBuf zeta, zeta0;                 // device copies of the model (complex128)
    egx::DevBuf r64, fwd64, bwd64, r32, fwd32, bwd32;
    bool prepared32 = false;
    egx::DevBuf buf64, buf32;
    int tw_n0 = 0, tw_n1 = 0;
    egx::DevBuf tw0_64, tw1_64, tw0_32, tw1_32;
    egx::FftPlan p0{}, p1{};
    // host staging
    egx::DevBuf xin, yout, xin32, yout32, src_io;
    // solvers (cached workspaces)
    std::unique_ptr<egx::Gmres<double>> outer64, inner64;
    std::unique_ptr<egx::Gmres<float>> outer32, inner32;
    std::string key64, key32;
    // inner solves with the learned preconditioner keep their own workspace
    std::unique_ptr<egx::Gmres<float>> outer32l, inner32l;
    std::string key32l;
    long learned_uses = 0, learned_fallbacks = 0;
    int learned_inject = 0;  // test hook: learned outputs still to be overwritten with NaN
    // preconditioner plug
    int precond_kind = EGX_PRECOND_GMRES;
    egx_precond_fn precond_fn = nullptr;
    void *precond_user = nullptr;
    egx::DevBuf fftbuf;
    // egx_set_graphs: the inner GMRES cycle of the flexible preconditioner
    // captured as one CUDA graph (staging buffers, the executable graph and
    // the key of everything it bakes in)
    int use_graphs = 0;
    int fft_tile = 0, contract_variant = 0;  // egx_tune_apply / egx_apply_variant
    egx::DevBuf pc_in, pc_out;
    cudaGraphExec_t pc_exec = nullptr;
    std::string pc_key;
    long pc_nodes = 0, pc_replays = 0;
    egx::DevBuf nrm_part, nrm_out, mix_r, mix_t, mix_r32, mix_d32;
    egx::DevBuf js, chi0;
    egx::DevBuf errflag;  // device int: EGX_ERR_TIMEOUT from a bounded wait
    egx::GreenBuildStats last_build;
    // observation level: transformed sources, 3-column results
    egx::DevBuf lvl_x, lvl_out, lvl_in, lvl_field;
    // E and H level tensors of the most recently used levels, keyed by all
    // they depend on (geometry, background, omega, filter length, level);
    // the anomaly conductivity is not part of them
    struct LevelEntry {
        std::vector<double> key;
        egx::DevBuf g[2];
        unsigned long long used = 0;
    };
    static constexpr int kLevelSlots = 4;
    LevelEntry lvl_cache[kLevelSlots];
    int lvl_capacity = kLevelSlots;
    unsigned long long lvl_clock = 0;
    long lvl_hits = 0, lvl_builds = 0;
    int lvl_prec = EGX_PREC_FP64;  // EGX_PREC_MIXED: complex64 lateral FFT of the level tensors
};

// Body of a C entry point: returns EGX_OK, or the status of the exception
// with its message kept for egx_last_error (exceptions never cross the ABI).
#define EGX_GUARD(ctx, ...)                                             \
    try {                                                               \
        __VA_ARGS__;                                                    \
        return EGX_OK;                                                  \
    } catch (const egx::Error &e) {                                     \
        return fail((ctx), e.code, e.what());                           \
    } catch (const std::exception &e) {                                 \
        return fail((ctx), EGX_ERR_INVALID, e.what());                  \
    }

namespace egx {

// Operator/solver helpers shared by egx_api.cu and egx_mt.cu.
void set_device(egx_ctx *ctx);
long nvec(const egx_ctx *ctx);
// PrepareOperator from the device copies of zeta/zeta0 already held in ctx.
void prepare_device(egx_ctx *ctx, egx_green *g, const double *dz_host, int type);
// Upload zeta [nx][ny][nz] and zeta0 [nz] (host or device pointers).
void upload_model(egx_ctx *ctx, egx_green *g, const double *zeta, const double *zeta0, int where);
// ds: a complex128 apply whose block contraction runs in double-FP32
// arithmetic (the mixed form's refinement residual)
template <typename T> void apply_dev(egx_ctx *ctx, const C<T> *x, C<T> *y, int nrhs, bool ds = false);
GmresResult fgmres_dev(egx_ctx *ctx, const double2 *b, double2 *x, const egx_gmres_params &p, int *applies);
GmresResult mixed_dev(egx_ctx *ctx, const double2 *b, double2 *x, const egx_mixed_params &p, int *applies,
                      int *refinements, double *true_be, int nrhs = 1);
int fail(egx_ctx *ctx, int code, const std::string &msg);
// egx_model -> the build's model at angular frequency omega
GreenModel green_model(const egx_model *model, double omega);
// FFT plans and twiddles of lengths n0 (x) and n1 (y) in ctx
void ensure_twiddles(egx_ctx *ctx, int n0, int n1);
// Throws EGX_ERR_TIMEOUT (and clears the flag) if a kernel gave up a bounded
// wait; call after a stream synchronisation.
void check_device_error(egx_ctx *ctx);

}  // namespace egx
