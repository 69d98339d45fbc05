/*
 * egx.h -- C ABI of the GB300-native integral-equation (IE) forward solve.
 *
 * This library replaces, behind plain C entry points, the four C# surfaces of
 * the reference's IE hot path (prisae/extreme):
 *
 *   Green tensor  Extreme.Cartesian/Green/Tensor/GreenTensor.cs:14-209 and
 *                 Extreme.Cartesian/Forward/AtoA/AtoAGreenTensorCalculatorComponent.cs:69-279
 *   operator      Extreme.Cartesian/Forward/AtoA/ConvolutionOperator.cs:45-143
 *                 (PrepareOperator / Apply, the mat-vec callback of FlexibleGmresSolver)
 *   2-D FFT       Extreme.Cartesian/Fft/FftW/FftWTransform.cs:218-225 (FftWrap plan_many_dft)
 *   solver        Extreme.Cartesian/Forward/AnomalyCurrentFgmresSolver.cs:59-85 and
 *                 Extreme.Fgmres/FlexibleGmresWithGmresPreconditioner.cs:105-139
 *
 * Conventions
 *   - complex numbers are interleaved (re, im) doubles, as System.Numerics.Complex
 *     and the reference's complex16;
 *   - anomaly vectors use the reference's AnomalyCurrent layout, index
 *     ((i*ny + j)*3 + c)*nz + k (Extreme.Cartesian/Core/LayerAccessor.cs:45-47);
 *     nrhs vectors are stored one after the other;
 *   - every entry point returns an egx_status; errors never cross the ABI as
 *     exceptions; egx_last_error() gives the message of the last failure;
 *   - host buffers are owned by the caller and copied on the context stream;
 *     calls complete synchronously. A context is not thread-safe.
 */
#ifndef EGX_H
#define EGX_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    EGX_OK = 0,
    EGX_ERR_INVALID = 1,       /* bad argument (ArgumentNullException / ArgumentOutOfRange) */
    EGX_ERR_OOM = 2,           /* device allocation failed */
    EGX_ERR_CUDA = 3,          /* CUDA runtime error */
    EGX_ERR_NOT_CONVERGED = 4, /* FGMRES ran out of restarts (ResultInfo.NonConverged) */
    EGX_ERR_TIMEOUT = 5,       /* a bounded device wait gave up */
    EGX_ERR_STATE = 6,         /* call order (e.g. apply before prepare, InvalidOperationException) */
    EGX_ERR_MODEL = 7          /* anomaly layer not inside one background layer (ModelUtils.cs:160-185) */
} egx_status;

enum { EGX_OP_A = 0, EGX_OP_CHI0 = 1 };             /* OperatorType.cs */
enum { EGX_HOST = 0, EGX_DEVICE = 1 };              /* where the vectors live */
enum { EGX_PREC_FP64 = 0, EGX_PREC_MIXED = 1 };     /* storage/arithmetic of the operator */
enum { EGX_PRECOND_GMRES = 0, EGX_PRECOND_CALLBACK = 1, EGX_PRECOND_NONE = 2, EGX_PRECOND_LEARNED = 3 };
enum { EGX_FFT_FORWARD = -1, EGX_FFT_BACKWARD = 1 }; /* FFTW sign convention */

typedef struct egx_ctx egx_ctx;
typedef struct egx_green egx_green;
typedef struct egx_net egx_net;

/* Cartesian model at one frequency's geometry (CartesianModel, Section1D). */
typedef struct {
    int nx, ny, nz;
    double dx, dy;                  /* lateral cell sizes, m */
    const double *layer_depth;      /* [nz] top of each anomaly layer, m */
    const double *layer_thickness;  /* [nz] */
    int n_bg;                       /* background layers incl. both half-spaces */
    double zero_air_level;          /* depth of the top of layer 0 */
    const double *bg_thickness;     /* [n_bg]; first and last are 0 */
    const double *bg_sigma;         /* [n_bg] conductivity, S/m */
} egx_model;

/* GmresParams + ForwardSettings (Extreme.Fgmres/GmresParams.cs:151-170,
 * Extreme.Cartesian/Forward/Project/ForwardSettings.cs:8-12). */
typedef struct {
    int m_out;            /* OuterBufferLength */
    int m_in;             /* InnerBufferLength */
    double tol;           /* Residual */
    int max_restarts;     /* MaxRepeatsNumber */
    int precond;          /* EGX_PRECOND_* */
    int check_true;       /* 1: final true-residual check (CheckWithWarning), 0: Arnoldi only */
} egx_gmres_params;

/* Mixed-precision solve: inner FGMRES in complex64 inside an FP64
 * iterative-refinement loop (no reference counterpart; it wraps the same
 * operator and returns the same result record). */
typedef struct {
    double tol;           /* target relative true residual of the outer loop */
    int max_outer;        /* refinement steps */
    int m_out, m_in;      /* inner FGMRES buffers */
    double inner_tol;     /* tightest relative tolerance asked of an inner solve;
                             a refinement at true residual be asks only for
                             max(inner_tol, min(0.5, 0.3 * tol / be)) */
    int inner_restarts;
    int batch;            /* egx_solve_sources with several sources: 1 solves
                             them as one stacked block-diagonal system (every
                             operator apply covers all sources, each source
                             still checked against tol on its own residual);
                             0 solves them one after the other */
} egx_mixed_params;

/* ResultInfo (Extreme.Fgmres/ResultInfo.cs) plus counters. */
typedef struct {
    int converged;
    int iterations;       /* outer Arnoldi steps */
    double arnoldi_be;    /* |g_{j+1}| / ||b|| */
    double true_be;       /* ||b - A x|| / ||b|| (-1 if not computed) */
    int n_applies;        /* operator applications */
    int n_refinements;    /* mixed solve only */
} egx_result;

/* Right-preconditioner callback (RightPreconditionerRequest,
 * Extreme.Fgmres/FlexibleGmresSolver.cs:19-29): dst = M(src); device pointers
 * of n complex values in the operator's precision. Return 0 on success. */
typedef int (*egx_precond_fn)(void *user, const void *src, void *dst, long n, int precision);

/* ---- context ----------------------------------------------------------- */
int egx_create(int device, egx_ctx **out);
int egx_destroy(egx_ctx *ctx);
int egx_last_error(egx_ctx *ctx, char *buf, size_t len);
int egx_version(void);
/* Device allocations (cudaMalloc calls) this library has made in the
 * process so far; a diagnostic for callers that must know whether a call
 * allocates. No counterpart in the reference. */
long egx_device_allocations(void);
/* Use an external CUDA stream (cudaStream_t) for all work of this context. */
int egx_set_stream(egx_ctx *ctx, void *stream);
/* Execution of the flexible preconditioner (no reference counterpart; the
 * arithmetic is unchanged). The Arnoldi decisions of every solve run on the
 * device; with enable != 0 the inner GMRES cycle of each outer FGMRES step
 * is additionally captured once as a CUDA graph (per prepared operator,
 * tolerance and buffer set) and replayed, one launch instead of a few
 * hundred -- for many small solves, where launching is the cost. Ignored
 * while per-kernel timing (egx_profile) is on. Default off. */
int egx_set_graphs(egx_ctx *ctx, int enable);
/* Replays of the captured inner cycle since the context was created and the
 * kernel nodes of the last capture. */
int egx_graph_stats(egx_ctx *ctx, long *replays, long *nodes);
/* Apply autotuner (no reference counterpart): on the prepared operator
 * (complex64 Green tensor), times `reps` complex64 applies of nrhs vectors
 * for every kernel variant -- the FFT passes' column tile (0 built-in per
 * pass, 1 64-byte, 2 128-byte) x the contraction kernel: for the packed
 * Green layout 0 built-in order, 1 TMA-staged CUDA-core, 2 generic; for the
 * sub-block layout of nz in {16, 32, 48} 0 built-in (FP16 split, warps by
 * role), 1 TF32 split, 2 FP16 split in lockstep -- keeps the fastest for the
 * context's later complex64 applies, and writes the mean ms per apply to
 * ms_out[tile * 3 + variant] (9 doubles; may be NULL). The results agree to
 * complex64 rounding whatever the choice. */
int egx_tune_apply(egx_ctx *ctx, int nrhs, int reps, double *ms_out);
/* Set the variants by hand (same ranges). */
int egx_apply_variant(egx_ctx *ctx, int fft_tile, int contract_variant);
/* Count of this library's kernel launches since the context was created. */
long egx_launch_count(egx_ctx *ctx);

/* ---- Green tensor (GreenTensor, AtoAGreenTensorCalculatorComponent) ----- */
/* Build the anomaly-to-anomaly tensor on the device
 * (AtoAGreenTensorCalculatorComponent.CalculateGreenTensor,
 * AtoAGreenTensorCalculatorComponent.cs:69-89). EGX_PREC_FP64: all in FP64,
 * complex128 storage. EGX_PREC_MIXED: layer recursions, Hankel sums and face
 * integrals in FP64, the 2-D lateral FFT in complex64 (when 2nx and 2ny are
 * in {64, 128, 256, 512}; else FP64), stored as complex64 (for the inner
 * solves) and widened to complex128 (for the refinement's residual); within
 * ~1e-7 of the FP64 tensor. */
int egx_green_build(egx_ctx *ctx, const egx_model *model, double omega, int n_hankels,
                    int precision, egx_green **out);
/* Upload a spectral tensor given in the reference layout: comps[6] =
 * xx, xy, yy, zz (packed rc + tr*(tr+1)/2, Nz(Nz+1)/2 entries per point) and
 * xz, yz (rc*Nz + tr, Nz*Nz entries), each [2nx][2ny][block] complex. */
int egx_green_upload(egx_ctx *ctx, int nx, int ny, int nz, const double *const comps[6],
                     int precision, egx_green **out);
/* Download the complex128 spectral tensor in the reference layout. */
int egx_green_download(egx_ctx *ctx, const egx_green *g, double *const comps[6]);
/* Free a tensor. The context keeps its device storage for the next
 * egx_green_build (one frequency after another reuses it); egx_destroy
 * releases it. */
int egx_green_free(egx_ctx *ctx, egx_green *g);

/* ---- operator (ConvolutionOperator) ------------------------------------ */
/* PrepareOperator (ConvolutionOperator.cs:64-143). zeta: [nx][ny][nz]
 * complex anomaly conductivities, zeta0: [nz] complex background of each
 * anomaly layer, dz: [nz] layer thicknesses. type: EGX_OP_A or EGX_OP_CHI0. */
int egx_op_prepare(egx_ctx *ctx, egx_green *g, const double *zeta, const double *zeta0,
                   const double *dz, int type);
/* Apply (ConvolutionOperator.cs:45-62,162-327): y = K x for nrhs vectors. */
int egx_op_apply(egx_ctx *ctx, const double *x, double *y, int nrhs, int where);
/* Same in complex64 (interleaved floats) with the complex64 tensor. */
int egx_op_apply_c64(egx_ctx *ctx, const float *x, float *y, int nrhs, int where);
/* The complex128 apply with its block contraction in double-FP32
 * arithmetic (Dot2 on float pairs, ~47 significant bits, no complex128 FMA):
 * the apply the mixed form uses for its refinement residuals. Same
 * arguments as egx_op_apply; nz <= 53 and 4 nrhs 3 nz float4 of staged
 * vectors <= 96 KiB, else the complex128 contraction runs. */
int egx_op_apply_ds(egx_ctx *ctx, const double *x, double *y, int nrhs, int where);

/* ---- FFT (FftWrap plan_many_dft rank 2) -------------------------------- */
/* In-place unnormalised 2-D DFT over (n0, n1) of `howmany` interleaved
 * sequences: element (i, j, b) at (i*n1 + j)*howmany + b. sign -1 forward. */
int egx_fft2d(egx_ctx *ctx, double *buf, int n0, int n1, int howmany, int sign, int where);

/* ---- solver (AnomalyCurrentFgmresSolver / FGMRES with GMRES precond) ---- */
/* Solve A x = b with x holding the initial guess on entry
 * (AnomalyCurrentFgmresSolver.Solve, FlexibleGmresWithGmresPreconditioner). */
int egx_fgmres_solve(egx_ctx *ctx, const double *b, double *x, const egx_gmres_params *p,
                     egx_result *res, int where);
/* Mixed-precision form of the same solve. */
int egx_mixed_solve(egx_ctx *ctx, const double *b, double *x, const egx_mixed_params *p,
                    egx_result *res, int where);
/* RightPreconditionerRequest plug point: kind EGX_PRECOND_CALLBACK routes
 * z_j = M(v_j) of the outer FGMRES to fn(user, ...). */
int egx_set_precond(egx_ctx *ctx, int kind, egx_precond_fn fn, void *user);

/* ---- learned flexible preconditioner (the RightPreconditionerRequest plug
 * point, FlexibleGmresSolver.cs:24-36; no reference counterpart otherwise) --
 * A spectral network z = N(v) = v + rms(v) Out(v / rms(v), log sigma) on the
 * nx x ny x nz anomaly mesh, depth a spatial axis: 7 input channels per cell
 * (Re and Im of the three residual components, log10(omega mu0 sigma dx dy)),
 * a lift to `width` channels, `layers` layers each of a per-depth lateral
 * spectral convolution (16 x 16 retained modes in a real Fourier basis, a
 * width x width mixing per mode), a pointwise width x width map and an
 * nz x nz depth mixing, GELU between layers, a projection to 6 channels
 * (Re and Im of the correction) that starts at zero: an untrained network
 * is the identity. BF16 tensor-core GEMMs with FP32 accumulation for the
 * forward and backward passes, Adam. Vectors are complex64 [batch][N] in the
 * anomaly layout; batch <= 64. */
int egx_net_create(egx_ctx *ctx, int nx, int ny, int nz, int width, int layers, unsigned seed, egx_net **out);
int egx_net_free(egx_ctx *ctx, egx_net *net);
long egx_net_size(const egx_net *net);                               /* parameters */
int egx_net_params(egx_ctx *ctx, egx_net *net, float *host, int set);  /* set = 0 read, 1 write */
/* log-conductivity channel, [nx][ny][nz] host floats */
int egx_net_set_model(egx_ctx *ctx, egx_net *net, const float *logsig);
/* `count` log-conductivity models [count][nx][ny][nz] (1..64): sample b of
 * the next calls uses model b % count (training batches drawn from several
 * solves) */
int egx_net_set_models(egx_ctx *ctx, egx_net *net, const float *logsig, int count);
/* loss = mean_b |N(v_b/rms_b) - t_b/rms_b|^2 / |t_b/rms_b|^2 for targets t = z* - v;
 * gradients kept for egx_net_adam and copied to grad (n_params floats) if not NULL */
int egx_net_loss_grad(egx_ctx *ctx, egx_net *net, const float *v, const float *t, int batch, float *loss, float *grad,
                      int where);
int egx_net_adam(egx_ctx *ctx, egx_net *net, float lr);
/* The network's pointwise GEMMs (lift, per-layer width x width map,
 * projection, and their backward products; width <= 32) run on a tcgen05
 * kernel (enable = 1, the default: BF16 operands staged in shared memory,
 * FP32 accumulator in tensor memory) or on the warp-level mma.sync kernel
 * that the spectral and weight-gradient GEMMs use (enable = 0). */
int egx_net_use_tcgen05(egx_ctx *ctx, egx_net *net, int enable);
int egx_net_apply(egx_ctx *ctx, egx_net *net, const float *v, float *z, int batch, int where);
/* With egx_set_precond(ctx, EGX_PRECOND_LEARNED, NULL, net) each inner
 * complex64 FGMRES of the mixed form uses the network as its flexible right
 * preconditioner, z_j = N(v_j), in place of the reference's inner GMRES(m_in)
 * cycle (FlexibleGmresWithGmresPreconditioner.cs:35-57); the network must be
 * built for the solve's grid (EGX_ERR_INVALID otherwise). An inner solve that
 * does not reach its tolerance within min(inner_restarts, 4) cycles is redone
 * with the GMRES preconditioner (the fallback), and the refinement's
 * complex128 residual judges the result. uses/fallbacks count the inner
 * solves since the context was created. EGX_PRECOND_NONE makes the mixed
 * form's inner FGMRES unpreconditioned. */
int egx_learned_stats(egx_ctx *ctx, long *uses, long *fallbacks);
/* Failure-injection hook for tests (no reference counterpart): the next
 * `count` applications of the learned preconditioner have the first entry of
 * the network's output overwritten with NaN by a host-to-device copy (no
 * device-side fault injection), so that the inner solve fails and the
 * fallback to the GMRES preconditioner runs. A GMRES cycle that meets a
 * non-finite norm stops at once as not converged. count 0 disarms it. */
int egx_learned_inject_nonfinite(egx_ctx *ctx, int count);

/* Failure-detection check (no reference counterpart): one kernel waits,
 * through the bounded wait that every TMA-fed kernel uses, on a shared-memory
 * barrier that nothing completes, and gives up after limit_ms (1..2000).
 * Returns EGX_ERR_TIMEOUT (message from egx_last_error) with the context
 * still usable; EGX_OK would mean that the wait did not give up. */
int egx_wait_selftest(egx_ctx *ctx, double limit_ms);

/* DotProductRequest (AnomalyCurrentFgmresSolver.cs:115-130): out[k] =
 * conj(V[:, k])^T w for k < ncols, V column-major with leading dimension n.
 * With EGX_DEVICE, V, w and out must be 16-byte aligned. */
int egx_dot_products(egx_ctx *ctx, const double *V, int ncols, const double *w, long n, double *out, int where);

/* egx_dot_products on device pointers (V, w, out in device memory) that
 * allocates nothing -- for callers that cannot allocate device memory where
 * they call it, such as a host whose device memory belongs to its own pool
 * allocator, or a host function that a host-driven Krylov loop calls between
 * its launches. No counterpart in the reference. The partial sums live in
 * one static device array of 128 KiB that every call on a device shares: at
 * most 64 columns per call (more is EGX_ERR_INVALID, see egx_last_error);
 * calls that overlap on the GPU race. V, w and out must be 16-byte aligned
 * (else EGX_ERR_INVALID, nothing launched). The first call on a device looks
 * the array up (cudaGetSymbolAddress). Every call synchronises the context's
 * stream: it must not be made while that stream is being captured, nor from
 * a CUDA host callback (cudaLaunchHostFunc). */
int egx_dot_products_static(egx_ctx *ctx, const double *V, int ncols, const double *w, long n, double *out);

/* ---- MT source and the CIE pipeline around the solve ------------------- */
/* Thickness-averaged 1-D plane-wave field on each anomaly layer
 * (Mt3DForwardSolver.CalculateNormalFieldFromSource, Mt3DForwardSolver.cs:251-275;
 * PlaneWaveCalculator.CalculateFieldE, PlaneWaveCalculator.cs:11-40). e0: [nz] complex. */
int egx_normal_field(const egx_model *model, double omega, double *e0);
/* Plane-wave E and H at a flat depth (PlaneWaveCalculator.CalculateFieldE/H,
 * PlaneWaveCalculator.cs:11-64). e, h: one complex each. */
int egx_plane_wave(const egx_model *model, double omega, double depth, double *e, double *h);

typedef struct {
    int precision;              /* EGX_PREC_FP64: complex128 FGMRES; EGX_PREC_MIXED: mixed solve */
    egx_gmres_params fgmres;    /* used with EGX_PREC_FP64 */
    egx_mixed_params mixed;     /* used with EGX_PREC_MIXED */
} egx_source_params;

/* ForwardSolverGenerics.SolveForOneSource up to jQ for nsrc sources
 * (Forward/ForwardSolverGenerics.cs:30-50, Forward/ForwardSolver.cs:186-436):
 * jS = (zeta - zeta0) E0, chi0 = K_chi0 jS, solve A chi = chi0 (EGX_PREC_FP64
 * from x0 = chi0 as the reference, EGX_PREC_MIXED from zero),
 * Es = (2 sqrt(Re zeta0) chi - jS)/(zeta + conj zeta0), jQ = Es (zeta - zeta0) + jS.
 * e0: [nsrc][nz] complex normal field per layer, pol: [nsrc] component
 * (0 = x, 1 = y); chi (may be NULL), jq: [nsrc][N]; res: [nsrc]. */
int egx_solve_sources(egx_ctx *ctx, egx_green *g, const double *zeta, const double *zeta0, const double *dz,
                      const double *e0, const int *pol, int nsrc, const egx_source_params *p, double *chi,
                      double *jq, egx_result *res, int where);

/* ---- fields at an observation level and MT responses --------------------- */
/* Anomalous E and H at the observation level z (with its lateral shift) of
 * nsrc current distributions jq [nsrc][N] (AtoOCalculator.CalculateAnomalyFieldE/H,
 * AtoOCalculator.cs:68-176; ToOCalculator.CalculateAnomalyField,
 * ToOCalculator.cs:21-125). The level tensors of E and H are built in FP64 on
 * the device (AtoOLevelGreenTensorCalculator.cs:21-126). e, h: [nsrc][nx][ny][3]
 * complex, anomalous part only (the normal field is egx_plane_wave at z). */
int egx_level_fields(egx_ctx *ctx, const egx_model *model, double omega, int n_hankels, double z, double shift_x,
                     double shift_y, const double *jq, int nsrc, double *e, double *h, int where);
/* Level-tensor cache of a context (the level part of TensorCache,
 * Extreme.Cartesian/Forward/TensorCache.cs:8-35): egx_level_fields keeps the
 * E and H level tensors of the last `capacity` levels (0..4, default 4),
 * keyed by everything they depend on -- lateral geometry, anomaly layers,
 * background section, omega, filter length, z and shifts, not the anomaly
 * conductivity -- and reuses them when a later call matches. Each cached
 * level holds 15 complex128 arrays of [2nx][2ny][nz] (3 GB at 256x256x48).
 * capacity 0 rebuilds every call; a negative capacity leaves the setting;
 * setting it drops the cached levels. hits, builds (may be NULL): counts of
 * reused and built levels since the context was created. */
int egx_level_cache(egx_ctx *ctx, int capacity, long *hits, long *builds);
/* Precision of egx_level_fields from now on (part of the level cache's
 * key): EGX_PREC_FP64 (default, the reference's arithmetic) or
 * EGX_PREC_MIXED: face sums in double-FP32 rounded to complex64, level
 * tensors kept in complex64 (2-D FFT and storage, half the cache memory),
 * jQ's spectrum in complex64, layer sums as Dot2 into complex128 (fields
 * within ~1e-6 of the FP64 build; the mixed form's solve is 1e-6-accurate). */
int egx_set_level_precision(egx_ctx *ctx, int precision);
/* Impedance, apparent resistivity and phase at n sites from the total fields
 * of polarisation X (e1, h1) and Y (e2, h2), each [n][3] complex, host arrays
 * (ResponseFunctionsCalculator.CalculateTensor, ResponseFunctionsCalculator.cs:36-51;
 * PlainTextExporter.cs:360-420): z [n][4] complex (xx, xy, yx, yy),
 * rho [n][4] in Ohm m, phase [n][4] in degrees. */
int egx_mt_responses(const double *e1, const double *e2, const double *h1, const double *h2, long n, double omega,
                     double *z, double *rho, double *phase);
/* The same responses on the device, on ctx's stream, from the anomalous
 * fields that egx_level_fields_dev writes: e, h device arrays [2][n][3]
 * complex (polarisations X, Y), to which the plane wave's normal field at
 * the level is added (e_normal, h_normal: one complex value each; X:
 * E + (en, 0, 0), H + (0, hn, 0); Y: E + (0, en, 0), H + (-hn, 0, 0), as
 * Mt3DForwardSolver.cs:297-337 combines them). z [n][4] complex, rho [n][4],
 * phase [n][4]: device arrays. Synchronises the stream before returning. */
int egx_mt_responses_dev(egx_ctx *ctx, const double *e, const double *h, long n, double omega,
                         const double e_normal[2], const double h_normal[2], double *z, double *rho, double *phase);

/* ---- per-kernel device time ---------------------------------------------- */
/* Instrumented kernels; add EGX_K_C64 for the complex64 variants. */
enum {
    EGX_K_FWD_Y = 0, EGX_K_FWD_X = 1, EGX_K_CONTRACT = 2, EGX_K_BWD_X = 3, EGX_K_BWD_Y = 4,
    EGX_K_GS_DOTS = 5, EGX_K_GS_UPDATE = 6, EGX_K_C64 = 8,
    EGX_K_GREEN_LAYERS = 16, EGX_K_GREEN_KERNELS = 17, EGX_K_GREEN_HANKEL = 18, EGX_K_GREEN_CELLS = 19,
    EGX_K_GREEN_FFT = 20
};
/* enable != 0 records CUDA events around every instrumented launch (of the
 * kinds selected by egx_profile_kinds); resets the sums. */
int egx_profile(egx_ctx *ctx, int enable);
/* Bit k of mask selects kind k (default: all); fewer kinds, fewer event
 * records on the host's path between launches. */
int egx_profile_kinds(egx_ctx *ctx, unsigned mask);
/* Launches and summed device milliseconds of one kernel kind since enable. */
int egx_profile_read(egx_ctx *ctx, int kind, long *launches, double *total_ms);

#ifdef __cplusplus
}
#endif
#endif /* EGX_H */
