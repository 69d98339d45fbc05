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

template <typename T>
struct VecOps {
    // dots[k] = sum_r conj(V[r, k]) w[r] for k < ncols (V column-major, ld = n)
    static void multi_dot(const C<T> *V, int ncols, const C<T> *w, long n, double2 *dots_dev, double2 *partials,
                          int nblocks, cudaStream_t s);
    // w -= V[:, :ncols] * dots ; norm2_dev = ||w||^2
    static void update_norm(const C<T> *V, int ncols, const double2 *dots_dev, C<T> *w, long n, double *norm2_dev,
                            double *partials, int nblocks, cudaStream_t s);
    // ||x||^2 into norm2_dev
    static void norm2(const C<T> *x, long n, double *norm2_dev, double *partials, int nblocks, cudaStream_t s);
    // y = alpha * x (alpha real)
    static void scale(const C<T> *x, double alpha, C<T> *y, long n, cudaStream_t s);
    // y = x / d (d real)
    static void divide(const C<T> *x, double d, C<T> *y, long n, cudaStream_t s);
    // y = a - b
    static void sub(const C<T> *a, const C<T> *b, C<T> *y, long n, cudaStream_t s);
    // y += x
    static void add(const C<T> *x, C<T> *y, long n, cudaStream_t s);
    // out = V[:, :ncols] * coef (coef device)
    static void gemv(const C<T> *V, int ncols, const double2 *coef, C<T> *out, long n, cudaStream_t s);
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
    std::function<void(int, double)> on_iteration;
    long kernel_launches = 0;
    Timers *timers = nullptr;

  private:
    double norm(const C<T> *x);
    void construct(int jh, C<T> *result);
    double final_actions(int jh, const C<T> *rhs, C<T> *result);
    double arnoldi(double bn, int &jh);

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
