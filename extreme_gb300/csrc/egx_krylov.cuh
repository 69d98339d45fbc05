// Restarted GMRES / flexible GMRES on device vectors, mirroring
// Extreme.Fgmres/Gmres.cs step by step (Solve :77-143, PrepareRestart :145-175,
// FinalActions :177-230, KrylovSubspaceConstruction :233-295, iterative
// classical Gram-Schmidt :297-313) with the Hessenberg/Givens work on the host
// and every O(N) vector operation in device kernels.
#pragma once

#include <complex>
#include <functional>

#include "egx_common.cuh"

namespace egx {

// Vector kernels. `live` (device int, may be null): when it points at 0 the
// launched kernel returns at once -- the predicated work of a Krylov cycle
// that the host enqueued ahead of the device's decision to stop.
template <typename T>
struct VecOps {
    // dots[k] = sum_r conj(V[r, k]) w[r] for k < ncols (V column-major, ld = n)
    static void multi_dot(const C<T> *V, int ncols, const C<T> *w, long n, double2 *dots_dev, double2 *partials,
                          int nblocks, cudaStream_t s, const int *live = nullptr);
    // w -= V[:, :ncols] * dots ; norm2_dev = ||w||^2
    static void update_norm(const C<T> *V, int ncols, const double2 *dots_dev, C<T> *w, long n, double *norm2_dev,
                            double *partials, int nblocks, cudaStream_t s, const int *live = nullptr);
    // ||x||^2 into norm2_dev
    static void norm2(const C<T> *x, long n, double *norm2_dev, double *partials, int nblocks, cudaStream_t s,
                      const int *live = nullptr);
    // y = alpha * x (alpha real)
    static void scale(const C<T> *x, double alpha, C<T> *y, long n, cudaStream_t s);
    // y = x / d (d real)
    static void divide(const C<T> *x, double d, C<T> *y, long n, cudaStream_t s);
    // y = x / *d_dev (device scalar), when live
    static void divide_dev(const C<T> *x, const double *d_dev, C<T> *y, long n, cudaStream_t s, const int *live);
    // y = a - b
    static void sub(const C<T> *a, const C<T> *b, C<T> *y, long n, cudaStream_t s, const int *live = nullptr);
    // y += x
    static void add(const C<T> *x, C<T> *y, long n, cudaStream_t s, const int *live = nullptr);
    // out = V[:, :ncols] * coef (coef device); ncols_dev (device, may be null)
    // overrides ncols, and 0 columns launch nothing that writes
    static void gemv(const C<T> *V, int ncols, const double2 *coef, C<T> *out, long n, cudaStream_t s,
                     const int *ncols_dev = nullptr);
    static void copy(const C<T> *x, C<T> *y, long n, cudaStream_t s);
    static void zero(C<T> *x, long n, cudaStream_t s);
};

// Conversions between complex128 and complex64 vectors.
void convert_d2f(const double2 *x, float2 *y, long n, double scale, cudaStream_t s);
void convert_f2d_add(const float2 *x, double2 *y, long n, double scale, cudaStream_t s);

struct GmresResult {
    bool converged = false;
    double arnoldi_be = -1;
    double true_be = -1;
    int iterations = 0;
};

// Device state of a device-controlled solve (Gmres::solve with
// device_control): the scalars the reference's GmresSolver keeps in its
// fields, updated by one-thread control kernels between the vector kernels.
struct GmState {
    double bn, beta, bea, dnormw, dloo, true_be;
    int active;      // the current cycle continues
    int reorth;      // another classical Gram-Schmidt pass is needed
    int jh;          // steps of the current cycle
    int iterations;  // steps of the solve
    int flags;       // kGmZero | kGmExact | kGmNonFinite
    int ncols;       // columns of the last solution update
};
enum { kGmZero = 1, kGmExact = 2, kGmNonFinite = 4 };

// A GmresSolver with device workspace. apply(x, y): y = A x on device
// vectors. precond(src, dst): dst = M(src); empty -> classic solver.
template <typename T>
class Gmres {
  public:
    typedef std::function<void(const C<T> *, C<T> *)> Fn;
    Gmres(long n, int m, double tol, int max_restarts, bool check_true, cudaStream_t s);
    ~Gmres();
    Gmres(const Gmres &) = delete;
    Gmres &operator=(const Gmres &) = delete;
    // Solve(rightHandSide, initialGuess, result); result may alias
    // initialGuess; rhs may alias initialGuess (the inner preconditioner).
    GmresResult solve(const C<T> *rhs, const C<T> *x0, C<T> *result);
    // the tolerance of the next solve (the workspace does not depend on it)
    void set_tol(double tol) { tol_ = tol; }
    Fn apply;
    Fn precond;
    long kernel_launches = 0;
    Timers *timers = nullptr;
    // Device control: the Arnoldi decisions (Gram-Schmidt passes, Givens
    // rotations, stopping test, triangular solve) run in one-thread kernels
    // on the device. With enqueue_only the whole solve (one cycle) is
    // enqueued without any host wait -- the inner GMRES cycle of the
    // flexible preconditioner: steps after the device's stop are skipped by
    // their kernels, and the operator applies among them run speculatively
    // and are not counted; otherwise the host reads the device state once
    // per Arnoldi step (and at the start and end of a cycle) to decide what
    // to enqueue next.
    bool device_control = true;
    bool enqueue_only = false;
    // Operator applies of enqueue-only solves that ran while their cycle was
    // live (counted on the device, so also across CUDA-graph replays of a
    // captured solve); reset_apply_counts zeroes the count.
    long live_applies();
    void reset_apply_counts();

  private:
    double norm(const C<T> *x);
    void construct(int jh, C<T> *result);
    double final_actions(int jh, const C<T> *rhs, C<T> *result);
    double arnoldi(double bn, int &jh);
    GmresResult solve_host(const C<T> *rhs, const C<T> *x0, C<T> *result);
    GmresResult solve_device(const C<T> *rhs, const C<T> *x0, C<T> *result);
    void apply_counted(const C<T> *x, C<T> *y, const int *live);
    void dc_norm(const C<T> *x, const int *live);
    void dc_step(int j);
    void dc_construct(C<T> *result);
    void dc_residual(const C<T> *rhs, const C<T> *x, bool first);
    GmState read_state();
    long long *napp_dev_ = nullptr;  // live applies of enqueue-only solves
    GmState *st_ = nullptr;    // device state
    GmState *hst_ = nullptr;   // pinned copy for the host
    double2 *Hd_ = nullptr;    // device Hessenberg + rhs column, (m+1) x (m+1) column-major
    double *csd_ = nullptr;    // Givens cosines
    double2 *snd_ = nullptr;   // Givens sines

    long n_;
    int m_;
    int iterations_done_ = 0;
    double bn_ = 0;
    double tol_;
    int max_restarts_;
    bool check_true_;
    cudaStream_t s_;
    int nblocks_;
    C<T> *V_ = nullptr, *Z_ = nullptr, *w_ = nullptr, *r0_ = nullptr, *xcur_ = nullptr;
    double2 *dots_ = nullptr, *coef_ = nullptr, *partials_ = nullptr;
    double *norm_dev_ = nullptr;
    double *host_ = nullptr;  // pinned: dots + norm
    std::vector<std::complex<double>> H_;
    std::vector<double> cs_;
    std::vector<std::complex<double>> sn_;
    std::complex<double> &h(int i, int j) { return H_[(size_t)j * (m_ + 1) + i]; }
};

}  // namespace egx
