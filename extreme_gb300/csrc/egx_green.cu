// Anomaly-to-anomaly Green tensor, FP64, on the device.
//
// Host: radius plan and lambdas (ScalarPlansCreater.cs:102-176, ScalarPlan.cs:460-481),
// merge of the plan items (InnerResultsCombiner.cs:19-61), transceiver lists
// (TranceiverUtils.cs:55-74), knots and face integral factors
// (GreenTensorCalculator.cs:166-437, IntegralFactors.cs:17-30), gathered per
// cell into sparse weight lists.
// Device, per tensor half (asym: xz, yz; symm: xx, xy, yy, zz):
//   k_layers   per lambda: eta, exp, P/Q reflection recursions of both modes
//              (PlanCalculatorFast.cs:203-318, green_scalar.c:30-41);
//   k_kernels  per (transceiver, lambda): exponential sums, propagators and
//              the kernels U1..U5 with their pre-Hankel normalisation
//              (VolumeToVolumeCalculatorUFast.cs:34-337, green_scalar.c:86-386,
//              ScalarMathUtils.cs:243-263);
//   k_hankel   the 431-tap digital filter and the post normalisation
//              (HankelCoefficients.cs:103-118, ScalarMathUtils.cs:189-207);
//   k_segments linear pieces per radius interval (ScalarSegments.cs:86-128);
//   k_cells    per (cell, block entry): signed sum of face integrals, written
//              with the parity mirroring into the 2Nx x 2Ny grid
//              (GreenTensorCalculator.cs:460-552, GreenTensorFftPopulator.cs:221-273);
//   FFT        y then x (only the ky <= Ny columns, kx <= Nx rows kept);
//   k_extract  the (Nx+1)(Ny+1) quadrant into the operator's block layout.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <mutex>
#include <set>

#include "egx_ds.cuh"
#include "egx_green.cuh"
#include "egx_operator.cuh"
#include "hankel_ndec40.inc"

namespace egx {

namespace {

constexpr double kMu0 = 4.0 * M_PI * 1.0e-7;
constexpr double kEps0 = 1.0 / (kMu0 * 299792458.0 * 299792458.0);
constexpr int kTaps = 431;
constexpr int kL2 = 130;
constexpr int kMaxLayers = 32;

__constant__ double c_h0[kTaps];
__constant__ double c_h1[kTaps];

typedef std::complex<double> cd;

// ---------------------------------------------------------------- device math
__device__ __forceinline__ double2 dmk(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ double2 dadd(double2 a, double2 b) { return dmk(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 dsub(double2 a, double2 b) { return dmk(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 dmul(double2 a, double2 b) { return dmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 dscal(double s, double2 a) { return dmk(s * a.x, s * a.y); }
__device__ __forceinline__ double2 dneg(double2 a) { return dmk(-a.x, -a.y); }
__device__ __forceinline__ double2 ddiv(double2 a, double2 b) { return cdiv<double>(a, b); }
__device__ __forceinline__ double2 drecip(double2 b) { return cdiv<double>(dmk(1.0, 0.0), b); }
__device__ __forceinline__ double2 dexp(double2 z) {
    double s, c;
    sincos(z.y, &s, &c);
    double e = exp(z.x);
    return dmk(e * c, e * s);
}
// Principal square root; the sign of a zero imaginary part selects the
// branch on the negative real axis (C99 csqrt).
__device__ __forceinline__ double2 dsqrt(double2 z) {
    double x = z.x, y = z.y;
    if (x == 0.0 && y == 0.0) return dmk(0.0, y);
    double t = sqrt((fabs(x) + hypot(x, y)) * 0.5);
    if (x >= 0.0) return dmk(t, y / (2.0 * t));
    return dmk(fabs(y) / (2.0 * t), copysign(t, y));
}

struct LayerArgs {
    int L;
    double omega;
    double2 zeta[kMaxLayers];
    double2 alpha_s[kMaxLayers];
    double2 beta_s[kMaxLayers];
    double thick[kMaxLayers];
    double tops[kMaxLayers + 1];
};

// Per lambda: eta, exp, P1, Q1, Ps, Qs over all layers. Arrays [6][L][nl]
// (of the ten that k_chain_factors completes).
__global__ void k_layers(const double *__restrict__ lam, int nl, const LayerArgs a, double2 *__restrict__ out) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nl) return;
    const int L = a.L;
    double2 eta[kMaxLayers], ex[kMaxLayers];
    const double l = lam[m];
    for (int k = 0; k < L; k++) {
        // value = (i*omega) * zeta * mu0, then lambda^2 - value with -Im(value)
        double2 io = dmk(0.0, a.omega);
        double2 v = dmul(io, a.zeta[k]);
        v = dmk(v.x * kMu0, v.y * kMu0);
        eta[k] = dsqrt(dmk(l * l - v.x, -v.y));
        ex[k] = dexp(dscal(-2.0 * a.thick[k], eta[k]));
    }
    double2 *Eta = out, *Ex = out + (long)L * nl, *P1 = out + 2L * L * nl, *Q1 = out + 3L * L * nl;
    double2 *Ps = out + 4L * L * nl, *Qs = out + 5L * L * nl;
    for (int k = 0; k < L; k++) {
        Eta[(long)k * nl + m] = eta[k];
        Ex[(long)k * nl + m] = ex[k];
    }
    for (int mode = 0; mode < 2; mode++) {
        double2 p[kMaxLayers], q[kMaxLayers];
        for (int k = 0; k < L; k++) p[k] = q[k] = dmk(0, 0);
        if (mode == 0) p[1] = ddiv(dsub(eta[1], eta[0]), dadd(eta[1], eta[0]));
        else {
            double2 a0 = dmul(a.zeta[0], eta[1]), a1 = dmul(a.zeta[1], eta[0]);
            p[1] = ddiv(dsub(a0, a1), dadd(a0, a1));
        }
        for (int k = 1; k < L - 1; k++) {
            double2 pexp = dmul(p[k], ex[k]);
            double2 ae = ddiv(eta[k], eta[k + 1]);
            if (mode == 1) ae = dmul(a.alpha_s[k], ae);
            double2 part = dmul(ae, ddiv(dsub(pexp, dmk(1, 0)), dadd(pexp, dmk(1, 0))));
            p[k + 1] = ddiv(dadd(dmk(1, 0), part), dsub(dmk(1, 0), part));
        }
        const int n = L - 1;
        {
            double2 be = ddiv(eta[n], eta[n - 1]);
            if (mode == 1) be = dmul(a.beta_s[n], be);
            q[n - 1] = ddiv(dsub(dmk(1, 0), be), dadd(dmk(1, 0), be));
        }
        for (int k = n - 1; k > 1; k--) {
            double2 qexp = dmul(q[k], ex[k]);
            double2 be = ddiv(eta[k], eta[k - 1]);
            if (mode == 1) be = dmul(a.beta_s[k], be);
            double2 part = dmul(be, ddiv(dsub(qexp, dmk(1, 0)), dadd(qexp, dmk(1, 0))));
            q[k - 1] = ddiv(dadd(dmk(1, 0), part), dsub(dmk(1, 0), part));
        }
        double2 *P = mode == 0 ? P1 : Ps, *Q = mode == 0 ? Q1 : Qs;
        for (int k = 0; k < L; k++) {
            P[(long)k * nl + m] = p[k];
            Q[(long)k * nl + m] = q[k];
        }
    }
}

struct Trans {
    double r1, r2, s1, s2;
    int r, s;      // background layers of receiver / transmitter
    int kase;      // 0 match, 1 receiver below, 2 receiver above
};

// The propagator chains' per-layer pieces, which depend on the layer and
// lambda only (not on the transmitter pair): per mode (P1/Q1, Ps/Qs) the
// head H[b] = 1 / (eta_b (1 - P_b Q_b X_b)) and the factors
// F[k] = (1 + P_{k+1}) / (1 + P_k X_k) exp(z_{k+1} (eta_{k+1} - eta_k)),
// so that a pair's chain A[t, b] = F[t] (... (F[b-1] H[b])) is a few complex
// products. Arrays [mode][L][nl] after the six of k_layers: F at 6L nl, H at
// 8L nl.
__global__ void k_chain_factors(int nl, const LayerArgs a, double2 *__restrict__ lay) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nl) return;
    const int L = a.L;
    const double2 *Eta = lay, *Ex = lay + (long)L * nl;
    auto E = [&](int k) { return Eta[(long)k * nl + m]; };
    for (int mode = 0; mode < 2; mode++) {
        const double2 *P = lay + (2L + 2 * mode) * L * nl, *Q = lay + (3L + 2 * mode) * L * nl;
        double2 *F = lay + (6L + mode) * L * nl, *H = lay + (8L + mode) * L * nl;
        for (int b = 0; b < L; b++)
            H[(long)b * nl + m] = drecip(dmul(E(b), dsub(dmk(1, 0), dmul(dmul(P[(long)b * nl + m], Q[(long)b * nl + m]),
                                                                       Ex[(long)b * nl + m]))));
        for (int k = 0; k + 1 < L; k++) {
            const double2 num = dadd(dmk(1, 0), P[(long)(k + 1) * nl + m]);
            const double2 den = dadd(dmk(1, 0), dmul(P[(long)k * nl + m], Ex[(long)k * nl + m]));
            F[(long)k * nl + m] = dmul(ddiv(num, den), dexp(dscal(a.tops[k + 1], dsub(E(k + 1), E(k)))));
        }
    }
}

// which kernels: bit0 U1, bit1 U2, bit2 U3, bit3 U4, bit4 U5; outputs packed
// in that order, each [ntrans][nl_total] at column offset `col0`.
__global__ void k_kernels(const double *__restrict__ lam, int nl, const double2 *__restrict__ lay, const LayerArgs a,
                          const Trans *__restrict__ trans, int ntrans, int which, double2 *__restrict__ U,
                          long nl_total, long col0) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)ntrans * nl) return;
    const int tr = (int)(idx / nl);
    const int m = (int)(idx - (long)tr * nl);
    const Trans T0 = trans[tr];
    const int L = a.L;
    const double2 *Eta = lay, *P1 = lay + 2L * L * nl, *Q1 = lay + 3L * L * nl;
    const double2 *Ps = lay + 4L * L * nl, *Qs = lay + 5L * L * nl;
#define E(k) Eta[(long)(k) * nl + m]
    const int r = T0.r, s = T0.s, t = min(r, s), b = max(r, s);
    const double dt = a.tops[t], db1 = a.tops[b + 1];
    const double r1 = T0.r1, r2 = T0.r2, s1 = T0.s1, s2 = T0.s2;
    const double2 er = E(r), es = E(s), et = E(t), eb = E(b);
    const double l = lam[m];
    auto lin3 = [](double c1, double2 v1, double c2, double2 v2, double c3, double2 v3) {
        double2 acc = dscal(c1, v1);
        acc = dadd(acc, dscal(c2, v2));
        return dadd(acc, dscal(c3, v3));
    };
    auto lin2 = [](double c1, double2 v1, double c2, double2 v2) { return dadd(dscal(c1, v1), dscal(c2, v2)); };
    // CalculateT / CalculateR and the C, D sums. Each is a signed sum of four
    // exponentials of the form e^G (e^a - e^b)(e^c - e^d) over the receiver
    // interval [r1, r2] and the source interval [s1, s2], so it equals its
    // first term times fr fs, fr = 1 - e^{-(r2 - r1) er}, fs = 1 - e^{-(s2 - s1) es}:
    // six complex exponentials instead of sixteen. With r1 <= r2, s1 <= s2
    // and Re eta >= 0 the factors have modulus <= 2 and the leading exponent
    // is the four-term form's first one, so nothing overflows that did not.
    double2 Tt, Rr, C = dmk(0, 0), D = dmk(0, 0);
    const double2 F = lin2(-2 * db1, eb, 2 * dt, et);
    if (r1 <= r2 && s1 <= s2) {
        const double2 fsr = dmul(dsub(dmk(1, 0), dexp(dscal(-(r2 - r1), er))),
                                 dsub(dmk(1, 0), dexp(dscal(-(s2 - s1), es))));
        Tt = dmul(dexp(lin3(-r1, er, -s1, es, 2 * dt, et)), fsr);
        Rr = dmul(dexp(lin3(-2 * db1, eb, s2, es, r2, er)), fsr);
        if (T0.kase == 2) {  // receiver above: CTop, DTop
            C = dmul(dexp(lin2(-s1, es, r2, er)), fsr);
            D = dmul(dexp(dadd(dadd(F, dscal(s2, es)), dscal(-r1, er))), fsr);
        } else if (T0.kase == 1) {  // receiver below: CBot, DBot
            C = dmul(dexp(lin2(-r1, er, s2, es)), fsr);
            D = dmul(dexp(dadd(dadd(F, dscal(-s1, es)), dscal(r2, er))), fsr);
        }
    } else {
        Tt = dexp(lin3(-r1, er, -s1, es, 2 * dt, et));
        Tt = dsub(Tt, dexp(lin3(-r1, er, -s2, es, 2 * dt, et)));
        Tt = dsub(Tt, dexp(lin3(-r2, er, -s1, es, 2 * dt, et)));
        Tt = dadd(Tt, dexp(lin3(-r2, er, -s2, es, 2 * dt, et)));
        Rr = dexp(lin3(-2 * db1, eb, s2, es, r2, er));
        Rr = dsub(Rr, dexp(lin3(-2 * db1, eb, s1, es, r2, er)));
        Rr = dsub(Rr, dexp(lin3(-2 * db1, eb, s2, es, r1, er)));
        Rr = dadd(Rr, dexp(lin3(-2 * db1, eb, s1, es, r1, er)));
        if (T0.kase == 2) {
            C = dexp(lin2(-s1, es, r2, er));
            C = dsub(C, dexp(lin2(-s2, es, r2, er)));
            C = dsub(C, dexp(lin2(-s1, es, r1, er)));
            C = dadd(C, dexp(lin2(-s2, es, r1, er)));
            D = dexp(dadd(dadd(F, dscal(s2, es)), dscal(-r1, er)));
            D = dsub(D, dexp(dadd(dadd(F, dscal(s1, es)), dscal(-r1, er))));
            D = dsub(D, dexp(dadd(dadd(F, dscal(s2, es)), dscal(-r2, er))));
            D = dadd(D, dexp(dadd(dadd(F, dscal(s1, es)), dscal(-r2, er))));
        } else if (T0.kase == 1) {
            C = dexp(lin2(-r1, er, s2, es));
            C = dsub(C, dexp(lin2(-r1, er, s1, es)));
            C = dsub(C, dexp(lin2(-r2, er, s2, es)));
            C = dadd(C, dexp(lin2(-r2, er, s1, es)));
            D = dexp(dadd(dadd(F, dscal(-s1, es)), dscal(r2, er)));
            D = dsub(D, dexp(dadd(dadd(F, dscal(-s2, es)), dscal(r2, er))));
            D = dsub(D, dexp(dadd(dadd(F, dscal(-s1, es)), dscal(r1, er))));
            D = dadd(D, dexp(dadd(dadd(F, dscal(-s2, es)), dscal(r1, er))));
        }
    }
    // propagator chain A[t, b] of a mode from the per-layer pieces of
    // k_chain_factors
    auto chain = [&](int mode) {
        const double2 *F = lay + (6L + mode) * L * nl, *H = lay + (8L + mode) * L * nl;
        double2 A = H[(long)b * nl + m];
        for (int k = b - 1; k >= t; k--) A = dmul(F[(long)k * nl + m], A);
        return A;
    };
    auto psi1 = [&](const double2 *P, const double2 *Q) {
        double2 pt = P[(long)t * nl + m], qb = Q[(long)b * nl + m];
        if (T0.kase == 0) {
            const int n = r;
            const double tau = r2 - r1;
            const double dn1 = a.tops[n + 1] - a.tops[n];
            double2 en = E(n);
            double2 part1 = dsub(dscal(tau, en), dsub(dmk(1, 0), dexp(dscal(-tau, en))));
            double2 pq = dmul(P[(long)n * nl + m], Q[(long)n * nl + m]);
            double2 e1 = dexp(dscal(-2 * dn1, en));
            double2 e2 = dexp(dadd(dscal(-2 * dn1, en), dscal(tau, en)));
            double2 part2 = dmul(pq, dsub(dmul(dadd(dscal(tau, en), dmk(1, 0)), e1), e2));
            return dscal(2.0, dsub(part1, part2));
        }
        return dadd(C, dmul(dmul(pt, qb), D));
    };
    auto psi3 = [&](const double2 *P, const double2 *Q) {
        if (T0.kase == 0) return dmk(0, 0);
        double2 pqd = dmul(dmul(P[(long)t * nl + m], Q[(long)b * nl + m]), D);
        if (T0.kase == 1) return dadd(dneg(C), pqd);
        return dsub(C, pqd);
    };
    auto special = [&](const double2 *P, const double2 *Q, double psign, double psisign, double2 psi) {
        double2 v = dmul(dscal(psign, P[(long)t * nl + m]), Tt);
        v = dadd(v, dmul(Q[(long)b * nl + m], Rr));
        return dadd(v, dscal(psisign, psi));
    };
    const double2 annf = drecip(dmul(er, es));
    const double2 zr2 = dscal(2.0, a.zeta[r]);
    long out = 0;
    double2 *Ub = U + (long)tr * nl_total + col0 + m;
    const long ustride = (long)ntrans * nl_total;
    if (which & 1) {
        double2 ann = chain(0);
        double2 u = dmul(dmul(ann, annf), special(P1, Q1, 1, 1, psi1(P1, Q1)));
        u = dmul(u, dmk(0.0, a.omega * kMu0 * 0.5));
        Ub[ustride * out++] = u;
    }
    double2 anns = chain(1);
    if (r > s) anns = dmul(ddiv(a.zeta[r], a.zeta[s]), anns);
    if (which & 2) {
        double2 u = dmul(anns, special(Ps, Qs, 1, -1, psi1(Ps, Qs)));
        Ub[ustride * out++] = ddiv(u, zr2);
    }
    if (which & 4) {
        double2 u = dmul(dmul(anns, drecip(es)), special(Ps, Qs, -1, 1, psi3(Ps, Qs)));
        Ub[ustride * out++] = dmul(u, ddiv(dmk(l, 0), zr2));
    }
    if (which & 8) {
        double2 u = dmul(dmul(anns, drecip(er)), special(Ps, Qs, -1, -1, psi3(Ps, Qs)));
        Ub[ustride * out++] = dmul(u, ddiv(dmk(-l, 0), zr2));
    }
    if (which & 16) {
        double2 u;
        if (T0.kase == 0) {
            const int n = r;
            const double tau = r2 - r1;
            const double ln = a.thick[n];
            double2 en = E(n);
            double2 kk = dmk(-a.omega * kMu0 * a.zeta[n].y, a.omega * kMu0 * a.zeta[n].x);
            double2 pq = dmul(Ps[(long)n * nl + m], Qs[(long)n * nl + m]);
            double2 part1 = dneg(dsub(dmk(1, 0), dexp(dscal(-tau, en))));
            double2 part2 = dmul(pq, dsub(dexp(dscal(-(2 * ln - tau), en)), dexp(dscal(-2 * ln, en))));
            double2 part3 = dmul(dmul(dscal(1.0 / (l * l), kk), dsub(dmk(1, 0), dmul(pq, dexp(dscal(-2 * ln, en))))),
                                 dscal(tau, en));
            double2 psi5 = dscal(2.0, dadd(dadd(part1, part2), part3));
            double2 sp = dadd(dadd(dmul(Ps[(long)t * nl + m], Tt), dmul(Qs[(long)b * nl + m], Rr)), psi5);
            u = dmul(dmul(anns, annf), sp);
        } else {
            u = dmul(dmul(anns, annf), special(Ps, Qs, 1, 1, psi1(Ps, Qs)));
        }
        Ub[ustride * out++] = dmul(u, ddiv(dmk(l * l, 0), zr2));
    }
#undef E
}

// I[u][trans][g] = norm * sum_j h[430 - j] * U[u][trans][col0 + i + j]
__global__ void k_hankel(const double2 *__restrict__ U, int nu, int ntrans, long nl_total, long col0, int nrho,
                         const double *__restrict__ rho, const int *__restrict__ gidx, const int *__restrict__ use_h0,
                         const int *__restrict__ negate, double2 *__restrict__ I, int nrad, double den_scale) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)nu * ntrans * nrho) return;
    int i = (int)(idx % nrho);
    long rest = idx / nrho;
    int tr = (int)(rest % ntrans);
    int u = (int)(rest / ntrans);
    const double2 *f = U + ((long)u * ntrans + tr) * nl_total + col0 + i;
    const double *h = use_h0[u] ? c_h0 : c_h1;
    double sx = 0, sy = 0;
    for (int j = 0; j < kTaps; j++) {
        double hj = h[kTaps - 1 - j];
        double2 v = f[j];
        sx += v.x * hj;
        sy += v.y * hj;
    }
    double den = den_scale * rho[i];   // 2 pi (E scalars) or 4 pi (H scalars)
    if (negate[u]) {
        sx = -sx;
        sy = -sy;
    }
    I[((long)u * ntrans + tr) * nrad + gidx[i]] = dmk(sx / den, sy / den);
}

// IA/IB[u][seg][trans]; with IA32/IB32 also as float pairs {re h, re l,
// im h, im l} for the double-FP32 face sums
__global__ void k_segments(const double2 *__restrict__ I, int nu, int ntrans, int nrad, const double *__restrict__ radii,
                           double2 *__restrict__ IA, double2 *__restrict__ IB, float4 *__restrict__ IA32,
                           float4 *__restrict__ IB32) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nseg = nrad - 1;
    if (idx >= (long)nu * nseg * ntrans) return;
    int tr = (int)(idx % ntrans);
    long rest = idx / ntrans;
    int sg = (int)(rest % nseg);
    int u = (int)(rest / nseg);
    const double2 *v = I + ((long)u * ntrans + tr) * nrad;
    double sr = radii[sg], ur = radii[sg + 1];
    double div = ur - sr;
    double2 a = dmk((v[sg + 1].x - v[sg].x) / div, (v[sg + 1].y - v[sg].y) / div);
    double2 bb = dsub(v[sg], dmul(a, dmk(sr, 0)));
    long o = ((long)u * nseg + sg) * ntrans + tr;
    IA[o] = a;
    IB[o] = bb;
    if (IA32) {
        float4 fa, fb;
        ds_split(a.x, fa.x, fa.y);
        ds_split(a.y, fa.z, fa.w);
        ds_split(bb.x, fb.x, fb.y);
        ds_split(bb.y, fb.z, fb.w);
        IA32[o] = fa;
        IB32[o] = fb;
    }
}

struct Term {
    int seg;
    int src;
    double wa, wb;
};

template <typename O> __device__ __forceinline__ O cell_out(double2 v);
template <> __device__ __forceinline__ double2 cell_out<double2>(double2 v) { return v; }

// Real-space value of each quadrant cell for block entries [t0, t0+tc),
// written with the parity mirroring into buf[2nx][2ny][tc] (or only the
// quadrant when compact), as complex128 or rounded to complex64.
template <typename O>
__global__ void k_cells(const int *__restrict__ rowptr, const Term *__restrict__ terms, const double2 *__restrict__ IA,
                        const double2 *__restrict__ IB, int ntrans, int nseg, int nx, int ny, int t0, int tc, int xs,
                        int ys, int compact, O *__restrict__ buf) {
    const int cell = blockIdx.x;
    const int i = cell / ny, j = cell - (cell / ny) * ny;
    const int t = blockIdx.y * blockDim.x + threadIdx.x;
    if (t >= tc) return;
    double2 acc = dmk(0, 0);
    for (int e = rowptr[cell]; e < rowptr[cell + 1]; e++) {
        const Term tm = terms[e];
        long o = ((long)tm.src * nseg + tm.seg) * ntrans + t0 + t;
        double2 a = IA[o], b = IB[o];
        acc.x = fma(tm.wa, a.x, acc.x);
        acc.y = fma(tm.wa, a.y, acc.y);
        acc.x = fma(tm.wb, b.x, acc.x);
        acc.y = fma(tm.wb, b.y, acc.y);
    }
    if (compact) {
        // quadrant buffer [nx+1][ny+1][tc]: the mirror images are made by
        // the FFT's loads (fft_lines_sym)
        buf[((long)i * (ny + 1) + j) * tc + t] = cell_out<O>(acc);
        return;
    }
    const int n0 = 2 * nx, n1 = 2 * ny;
    buf[((long)i * n1 + j) * tc + t] = cell_out<O>(acc);
    if (i >= 1 && j >= 1) {
        buf[((long)(n0 - i) * n1 + j) * tc + t] = cell_out<O>(dscal((double)xs, acc));
        buf[((long)i * n1 + (n1 - j)) * tc + t] = cell_out<O>(dscal((double)ys, acc));
        buf[((long)(n0 - i) * n1 + (n1 - j)) * tc + t] = cell_out<O>(dscal((double)(xs * ys), acc));
    } else if (i >= 1) {
        buf[((long)(n0 - i) * n1) * tc + t] = cell_out<O>(dscal((double)xs, acc));
    } else if (j >= 1) {
        buf[((long)(n1 - j)) * tc + t] = cell_out<O>(dscal((double)ys, acc));
    }
}

// k_cells for the mixed form: the same face sums as Dot2 on float pairs
// (double-FP32, the FP32 pipes), rounded to complex64. The block's cell
// terms are split into shared memory once per chunk.
constexpr int kCellChunk = 128;
__global__ void __launch_bounds__(128) k_cells_ds(const int *__restrict__ rowptr, const Term *__restrict__ terms,
                                                  const float4 *__restrict__ IA, const float4 *__restrict__ IB,
                                                  int ntrans, int nseg, int nx, int ny, int t0, int tc, int xs,
                                                  int ys, int compact, float2 *__restrict__ buf) {
    __shared__ float4 sw[kCellChunk];
    __shared__ long so[kCellChunk];
    const int cell = blockIdx.x;
    const int i = cell / ny, j = cell - (cell / ny) * ny;
    const int t = blockIdx.y * blockDim.x + threadIdx.x;
    float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
    const int e0 = rowptr[cell], e1 = rowptr[cell + 1];
    for (int c0 = e0; c0 < e1; c0 += kCellChunk) {
        const int cnt = min(kCellChunk, e1 - c0);
        __syncthreads();
        if ((int)threadIdx.x < cnt) {
            const Term tm = terms[c0 + threadIdx.x];
            float4 w;
            ds_split(tm.wa, w.x, w.y);
            ds_split(tm.wb, w.z, w.w);
            sw[threadIdx.x] = w;
            so[threadIdx.x] = ((long)tm.src * nseg + tm.seg) * ntrans + t0;
        }
        __syncthreads();
        if (t < tc) {
            for (int e = 0; e < cnt; e++) {
                const float4 w = sw[e];
                const float4 a = IA[so[e] + t], b = IB[so[e] + t];
                ds_dot2(sr, cr, w.x, w.y, a.x, a.y);
                ds_dot2(sr, cr, w.z, w.w, b.x, b.y);
                ds_dot2(si, ci, w.x, w.y, a.z, a.w);
                ds_dot2(si, ci, w.z, w.w, b.z, b.w);
            }
        }
    }
    if (t >= tc) return;
    const float2 v = make_float2(__fadd_rn(sr, cr), __fadd_rn(si, ci));
    if (compact) {
        buf[((long)i * (ny + 1) + j) * tc + t] = v;
        return;
    }
    const int n0 = 2 * nx, n1 = 2 * ny;
    const float fx = (float)xs, fy = (float)ys;
    buf[((long)i * n1 + j) * tc + t] = v;
    if (i >= 1 && j >= 1) {
        buf[((long)(n0 - i) * n1 + j) * tc + t] = make_float2(fx * v.x, fx * v.y);
        buf[((long)i * n1 + (n1 - j)) * tc + t] = make_float2(fy * v.x, fy * v.y);
        buf[((long)(n0 - i) * n1 + (n1 - j)) * tc + t] = make_float2(fx * fy * v.x, fx * fy * v.y);
    } else if (i >= 1) {
        buf[((long)(n0 - i) * n1) * tc + t] = make_float2(fx * v.x, fx * v.y);
    } else if (j >= 1) {
        buf[((long)(n1 - j)) * tc + t] = make_float2(fy * v.x, fy * v.y);
    }
}

// quad block entry of reference entry tt: packed symmetric entries keep
// their index, xz/yz entries rc*nz + tr move to rc*(nz+1) + tr.
template <typename I>
__global__ void k_extract(const I *__restrict__ buf, int nx, int ny, int row, int tc, int Bs, int off, int t0,
                          int nz, int asym, double2 *__restrict__ quad) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    long total = (long)(nx + 1) * (ny + 1) * tc;
    if (idx >= total) return;
    int t = (int)(idx % tc);
    long q = idx / tc;
    int a = (int)(q / (ny + 1)), b = (int)(q - (long)a * (ny + 1));
    int tt = t0 + t;
    int dst = asym ? (tt / nz) * (nz + 1) + tt % nz : tt;
    const I v = buf[((long)a * row + b) * tc + t];
    quad[q * Bs + off + dst] = make_double2((double)v.x, (double)v.y);
}

// ---------------------------------------------------------------- host plan
double rho_step() {
    float e = 1.0f / 40.0f;
    return (double)(float)std::pow(10.0, (double)e);
}

std::vector<double> rho_from_min(double mn, double mx, double step) {
    std::vector<double> out;
    double r = mn;
    while (r <= mx) {
        out.push_back(r);
        r *= step;
    }
    out.push_back(r);
    return out;
}

std::vector<double> rho_from_max(double mn, double mx, double step) {
    std::vector<double> out;
    double r = mx;
    while (r >= mn) {
        out.push_back(r);
        r /= step;
    }
    out.push_back(r);
    std::reverse(out.begin(), out.end());
    return out;
}

std::vector<double> lambdas_for(const std::vector<double> &rho, double step) {
    int n = kTaps + (int)rho.size();
    std::vector<double> k(n);
    k[kL2] = 1.0 / rho[0];
    for (int i = kL2 + 1; i < n; i++) k[i] = k[i - 1] / step;
    for (int i = kL2 - 1; i >= 0; i--) k[i] = k[i + 1] * step;
    return k;
}

struct Knot {
    int idx;
    double r;
};

Knot make_knot(const std::vector<double> &radii, double x, double y) {
    double r = std::sqrt(x * x + y * y);
    int idx = (int)(std::upper_bound(radii.begin(), radii.end(), r) - radii.begin()) - 1;
    if (idx == (int)radii.size() - 1) idx--;
    if (idx < 0) idx = 0;
    return Knot{idx, r};
}

struct Factors {
    double d1a, d1b, d2a, d2b, d3a, d3b;
};

Factors integral_factors(double s, double u, double rs, double ru, double v) {
    Factors f;
    if (v == 0) {
        f.d1a = (u * ru - s * rs) / 2;
        f.d2a = 0;
        f.d2b = 0;
    } else {
        double lg = std::log((u + ru) / (s + rs));
        f.d1a = (u * ru - s * rs + v * v * lg) / 2;
        f.d2a = -(u - s) * v;
        f.d2b = -(v * lg);
    }
    f.d1b = u - s;
    f.d3a = -(u * u - s * s) / 2;
    f.d3b = -(ru - rs);
    return f;
}

struct SegF {
    int seg;
    Factors f;
};

void integrate(const std::vector<double> &radii, Knot left, Knot right, double s, double u, double v,
               std::vector<SegF> &out) {
    out.clear();
    if (left.idx == right.idx) {
        out.push_back({left.idx, integral_factors(s, u, left.r, right.r, v)});
        return;
    }
    double r1 = left.r, r2 = radii[left.idx + 1];
    double sj = s, uj = std::sqrt(r2 * r2 - v * v);
    out.push_back({left.idx, integral_factors(sj, uj, r1, r2, v)});
    for (int i = left.idx + 1; i < right.idx; i++) {
        r1 = r2;
        r2 = radii[i + 1];
        sj = uj;
        uj = std::sqrt(r2 * r2 - v * v);
        out.push_back({i, integral_factors(sj, uj, r1, r2, v)});
    }
    sj = uj;
    uj = u;
    r1 = r2;
    r2 = right.r;
    out.push_back({right.idx, integral_factors(sj, uj, r1, r2, v)});
}

// component index: 0 xx, 1 xy, 2 yy, 3 zz, 4 xz, 5 yz
// QSigns (QSign.cs:254-257) in that order
const int kQX[6] = {1, -1, -1, -1, 1, 1};
const int kQY[6] = {-1, -1, 1, -1, 1, 1};
const int kQXS[6] = {1, 1, -1, -1, -1, 1};
const int kQYS[6] = {-1, 1, 1, -1, 1, -1};
// (factor 1/2/3, source scalar) per direction (AddToQBuffAlong{X,Y}Electric);
// source: 1 I1, 2 I2, 3 I3, 5 I5; 0 = component not filled in that direction
const int kFacX[6] = {2, 3, 2, 2, 0, 1}, kSrcX[6] = {1, 2, 2, 5, 0, 3};
const int kFacY[6] = {2, 3, 2, 2, 1, 0}, kSrcY[6] = {2, 1, 1, 5, 3, 0};

double fac_a(const Factors &f, int k) { return k == 1 ? f.d1a : (k == 2 ? f.d2a : f.d3a); }
double fac_b(const Factors &f, int k) { return k == 1 ? f.d1b : (k == 2 ? f.d2b : f.d3b); }

// Per-cell term lists of one component.
void cell_terms(const GreenModel &m, const std::vector<double> &radii, int comp, const int *src_slot,
                std::vector<int> &rowptr, std::vector<Term> &terms) {
    const int nx = m.nx, ny = m.ny;
    const double dx = m.dx, dy = m.dy;
    std::vector<Knot> kn((size_t)(nx + 1) * (ny + 1));
    for (int i = 0; i <= nx; i++)
        for (int j = 0; j <= ny; j++) kn[(size_t)i * (ny + 1) + j] = make_knot(radii, dx * (i - 0.5), dy * (j - 0.5));
    std::vector<Knot> zx(ny + 1), zy(nx + 1);
    for (int j = 0; j <= ny; j++) zx[j] = make_knot(radii, 0.0, dy * (j - 0.5));
    for (int i = 0; i <= nx; i++) zy[i] = make_knot(radii, dx * (i - 0.5), 0.0);
    auto K = [&](int i, int j) { return kn[(size_t)i * (ny + 1) + j]; };
    std::vector<std::vector<Term>> per((size_t)nx * ny);
    std::vector<SegF> parts;
    auto add = [&](int dir, bool symm, int i, int j, int sign) {
        const int fac = dir == 0 ? kFacX[comp] : kFacY[comp];
        const int src = dir == 0 ? kSrcX[comp] : kSrcY[comp];
        const int q = dir == 0 ? (symm ? kQXS[comp] : kQX[comp]) : (symm ? kQYS[comp] : kQY[comp]);
        const double w = (double)(sign * q);
        auto &lst = per[(size_t)i * ny + j];
        for (const SegF &p : parts) lst.push_back(Term{p.seg, src_slot[src], w * fac_a(p.f, fac), w * fac_b(p.f, fac)});
    };
    auto fill_x = [&](bool symm, int i, int j) {
        if (j == 0) add(0, symm, i, 0, -1);
        else if (j == ny) add(0, symm, i, ny - 1, 1);
        else {
            add(0, symm, i, j - 1, 1);
            add(0, symm, i, j, -1);
        }
    };
    auto fill_y = [&](bool symm, int i, int j) {
        if (i == 0) add(1, symm, 0, j, -1);
        else if (i == nx) add(1, symm, nx - 1, j, 1);
        else {
            add(1, symm, i - 1, j, 1);
            add(1, symm, i, j, -1);
        }
    };
    if (kFacX[comp]) {
        for (int j = 0; j <= ny; j++) {
            double y = dy * (j - 0.5);
            for (int i = 0; i < nx; i++) {
                double x1 = dx * (i - 0.5), x2 = dx * (i + 0.5);
                if (x1 > 0 && x2 > 0) {
                    integrate(radii, K(i, j), K(i + 1, j), x1, x2, y, parts);
                    fill_x(false, i, j);
                } else if (x1 < 0 && x2 < 0) {
                    integrate(radii, K(i + 1, j), K(i, j), -x2, -x1, y, parts);
                    fill_x(true, i, j);
                } else {
                    integrate(radii, zx[j], K(i, j), 0.0, -x1, y, parts);
                    fill_x(true, i, j);
                    integrate(radii, zx[j], K(i + 1, j), 0.0, x2, y, parts);
                    fill_x(false, i, j);
                }
            }
        }
    }
    if (kFacY[comp]) {
        for (int i = 0; i <= nx; i++) {
            double x = dx * (i - 0.5);
            for (int j = 0; j < ny; j++) {
                double y1 = dy * (j - 0.5), y2 = dy * (j + 0.5);
                if (y1 > 0 && y2 > 0) {
                    integrate(radii, K(i, j), K(i, j + 1), y1, y2, x, parts);
                    fill_y(false, i, j);
                } else if (y1 < 0 && y2 < 0) {
                    integrate(radii, K(i, j + 1), K(i, j), -y2, -y1, x, parts);
                    fill_y(true, i, j);
                } else {
                    integrate(radii, zy[i], K(i, j), 0.0, -y1, x, parts);
                    fill_y(true, i, j);
                    integrate(radii, zy[i], K(i, j + 1), 0.0, y2, x, parts);
                    fill_y(false, i, j);
                }
            }
        }
    }
    rowptr.assign((size_t)nx * ny + 1, 0);
    terms.clear();
    for (size_t c = 0; c < per.size(); c++) {
        rowptr[c] = (int)terms.size();
        terms.insert(terms.end(), per[c].begin(), per[c].end());
    }
    rowptr[per.size()] = (int)terms.size();
}

int layer_of(const std::vector<double> &tops, const std::vector<double> &thick, double depth) {
    double prev = tops[0];
    for (size_t k = 0; k < thick.size(); k++) {
        double d1 = prev, d2 = prev + thick[k];
        if (depth >= d1 && depth < d2) return (int)k;
        prev = d2;
    }
    throw Error(EGX_ERR_MODEL, "anomaly is not within the 1-D section");
}

template <typename X>
X *dev_upload(DevBuf &b, const std::vector<X> &v, cudaStream_t s) {
    b.ensure(std::max<size_t>(1, v.size()) * sizeof(X));
    if (!v.empty()) EGX_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(X), cudaMemcpyHostToDevice, s));
    return b.as<X>();
}

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// ---------------------------------------------------------------- observation level
// Volume-to-point kernels U of one mode (VolumeToPointCalculatorU.cs:21-352):
// the receiver is the point zw = T0.r1, the transmitter the layer [s1, s2].
struct VtpTerms {
    double2 T, R, psi15, psi34, psi5;
};

__device__ VtpTerms vtp_terms(const double2 *Eta, const double2 *P, const double2 *Q, long nl, int m, const LayerArgs &a,
                              const Trans &T0, double lam) {
#define E(k) Eta[(long)(k) * nl + m]
    const int r = T0.r, s = T0.s, t = min(r, s), b = max(r, s);
    const double zw = T0.r1, z1 = T0.s1, z2 = T0.s2;
    const double dt = a.tops[t], db1 = a.tops[b + 1];
    const double2 er = E(r), es = E(s), et = E(t), eb = E(b);
    auto ex3 = [](double c1, double2 v1, double c2, double2 v2, double c3, double2 v3) {
        return dexp(dadd(dadd(dscal(c1, v1), dscal(c2, v2)), dscal(c3, v3)));
    };
    VtpTerms o;
    // CalculateT / CalculateR with (z1, z2, r, s)
    o.T = dsub(ex3(-zw, er, -z1, es, 2 * dt, et), ex3(-zw, er, -z2, es, 2 * dt, et));
    o.R = dsub(ex3(-2 * db1, eb, z2, es, zw, er), ex3(-2 * db1, eb, z1, es, zw, er));
    const double2 pt = P[(long)t * nl + m], qb = Q[(long)b * nl + m];
    const double2 F = dadd(dscal(-2 * db1, eb), dscal(2 * dt, et));
    if (T0.kase == 0) {
        // CalcPsi1RcAndTrMatch / CalcPsi3And4RcAndTrMatch / CalcPsi5RcAndTrMatch, n = r = s
        const int n = r;
        const double2 en = E(n);
        const double2 Fn = dadd(dscal(-2 * a.tops[n + 1], en), dscal(2 * a.tops[n], en));
        auto ctop = [&](double x1, double x2) { return dsub(dexp(dscal(zw - x1, en)), dexp(dscal(zw - x2, en))); };
        auto cbot = [&](double x1, double x2) { return dsub(dexp(dscal(x2 - zw, en)), dexp(dscal(x1 - zw, en))); };
        auto dtop = [&](double x1, double x2) {
            return dsub(dexp(dadd(Fn, dscal(x2 - zw, en))), dexp(dadd(Fn, dscal(x1 - zw, en))));
        };
        auto dbot = [&](double x1, double x2) {
            return dsub(dexp(dadd(Fn, dscal(zw - x1, en))), dexp(dadd(Fn, dscal(zw - x2, en))));
        };
        const double2 pq = dmul(P[(long)n * nl + m], Q[(long)n * nl + m]);
        o.psi15 = dadd(dadd(ctop(zw, z2), cbot(z1, zw)), dmul(pq, dadd(dtop(zw, z2), dbot(z1, zw))));
        o.psi34 = dadd(dsub(ctop(zw, z2), cbot(z1, zw)), dmul(pq, dadd(dneg(dtop(zw, z2)), dtop(z1, zw))));
        const double ln = a.thick[n];
        const double2 kk = dmk(-a.omega * kMu0 * a.zeta[n].y, a.omega * kMu0 * a.zeta[n].x);
        double2 v = dmul(pq, dadd(dexp(dscal(-(2 * ln - (z2 - zw)), en)), dexp(dscal(-(2 * ln - (zw - z1)), en))));
        v = dsub(v, dadd(dexp(dscal(-(z2 - zw), en)), dexp(dscal(-(zw - z1), en))));
        const double2 w = dsub(dmk(1, 0), dmul(pq, dexp(dscal(-2 * ln, en))));
        o.psi5 = dadd(v, dscal(2.0 / (lam * lam), dmul(kk, w)));
    } else if (T0.kase == 2) {
        // receiver above: CTop, DTop with (z1, z2, r, s)
        const double2 C = dsub(dexp(dadd(dscal(-z1, es), dscal(zw, er))), dexp(dadd(dscal(-z2, es), dscal(zw, er))));
        const double2 D = dsub(dexp(dadd(F, dadd(dscal(z2, es), dscal(-zw, er)))),
                               dexp(dadd(F, dadd(dscal(z1, es), dscal(-zw, er)))));
        const double2 pqd = dmul(dmul(pt, qb), D);
        o.psi15 = dadd(C, pqd);
        o.psi34 = dsub(C, pqd);
        o.psi5 = o.psi15;
    } else {
        // receiver below: CBot, DBot with (z1, z2, r, s)
        const double2 C = dsub(dexp(dadd(dscal(-zw, er), dscal(z2, es))), dexp(dadd(dscal(-zw, er), dscal(z1, es))));
        const double2 D = dsub(dexp(dadd(F, dadd(dscal(-z1, es), dscal(zw, er)))),
                               dexp(dadd(F, dadd(dscal(-z2, es), dscal(zw, er)))));
        const double2 pqd = dmul(dmul(pt, qb), D);
        o.psi15 = dadd(C, pqd);
        o.psi34 = dadd(dneg(C), pqd);
        o.psi5 = o.psi15;
    }
#undef E
    return o;
}

// Per (transceiver, lambda): the pre-Hankel kernels of the level scalars
// (PlanCalculator.CalculateForE/H, PlanCalculator.cs:60-140, with
// NormalizeBeforeHankelForE/H, ScalarMathUtils.cs:171-263).
//   E (kind 0): slots I1..I5 = U1(1) i omega mu0/2, U2(s)/2zr, U3(s) lam/2zr,
//               -U4(s) lam/2zr, U5(s) lam^2/2zr;
//   H (kind 1): slots I1..I4 = U3(1), U4(s), U1(s) lam, U1(1) lam
// ("1": the P1/Q1/A1 mode, "s": the sigma mode).
__global__ void k_kernels_vtp(const double *__restrict__ lam, int nl, const double2 *__restrict__ lay,
                              const LayerArgs a, const Trans *__restrict__ trans, int ntrans, int kind,
                              double2 *__restrict__ U, long nl_total, long col0) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)ntrans * nl) return;
    const int tr = (int)(idx / nl);
    const int m = (int)(idx - (long)tr * nl);
    const Trans T0 = trans[tr];
    const int L = a.L;
    const double2 *Eta = lay, *P1 = lay + 2L * L * nl, *Q1 = lay + 3L * L * nl;
    const double2 *Ps = lay + 4L * L * nl, *Qs = lay + 5L * L * nl;
    const int r = T0.r, s = T0.s, t = min(r, s), b = max(r, s);
    const double l = lam[m];
    auto E = [&](int k) { return Eta[(long)k * nl + m]; };
    auto chain = [&](int mode) {  // k_chain_factors' pieces, as in k_kernels
        const double2 *F = lay + (6L + mode) * L * nl, *H = lay + (8L + mode) * L * nl;
        double2 A = H[(long)b * nl + m];
        for (int k = b - 1; k >= t; k--) A = dmul(F[(long)k * nl + m], A);
        return A;
    };
    const double2 er = E(r), es = E(s);
    const double2 a1 = chain(0);
    double2 as = chain(1);
    if (r > s) as = dmul(ddiv(a.zeta[r], a.zeta[s]), as);
    const VtpTerms v1 = vtp_terms(Eta, P1, Q1, nl, m, a, T0, l);
    const VtpTerms vs = vtp_terms(Eta, Ps, Qs, nl, m, a, T0, l);
    auto pre = [&](const double2 *P, const double2 *Q, const VtpTerms &v, double psign) {
        return dadd(dmul(dscal(psign, P[(long)t * nl + m]), v.T), dmul(Q[(long)b * nl + m], v.R));
    };
    auto u1 = [&](const double2 *P, const double2 *Q, const VtpTerms &v, double2 A) {
        return dmul(ddiv(A, es), dadd(pre(P, Q, v, 1), v.psi15));
    };
    auto u3 = [&](const double2 *P, const double2 *Q, const VtpTerms &v, double2 A) {
        return dmul(dmul(A, ddiv(er, es)), dadd(pre(P, Q, v, -1), v.psi34));
    };
    auto u4 = [&](const double2 *P, const double2 *Q, const VtpTerms &v, double2 A) {
        return dmul(A, dsub(pre(P, Q, v, -1), v.psi34));
    };
    double2 *Ub = U + (long)tr * nl_total + col0 + m;
    const long us = (long)ntrans * nl_total;
    if (kind == 0) {
        const double2 zr2 = dscal(2.0, a.zeta[r]);
        Ub[0] = dmul(u1(P1, Q1, v1, a1), dmk(0.0, a.omega * kMu0 * 0.5));
        Ub[us] = ddiv(dmul(dmul(as, er), dsub(pre(Ps, Qs, vs, 1), vs.psi15)), zr2);
        Ub[2 * us] = dmul(u3(Ps, Qs, vs, as), ddiv(dmk(l, 0), zr2));
        Ub[3 * us] = dmul(u4(Ps, Qs, vs, as), ddiv(dmk(-l, 0), zr2));
        const double2 u5 = dmul(ddiv(as, es), dadd(pre(Ps, Qs, vs, 1), vs.psi5));
        Ub[4 * us] = dmul(u5, ddiv(dmk(l * l, 0), zr2));
    } else {
        Ub[0] = u3(P1, Q1, v1, a1);
        Ub[us] = u4(Ps, Qs, vs, as);
        Ub[2 * us] = dscal(l, u1(Ps, Qs, vs, as));
        Ub[3 * us] = dscal(l, u1(P1, Q1, v1, a1));
    }
}

// Zero radius of the first plan item (ScalarMathUtils.CalculateZeroRhoFor{E,H},
// ScalarMathUtils.cs:33-87): I3 and I4 extrapolated from the item's second
// and third radii, the others 0. I[u][trans][nrad], radius 0 at index 0.
__global__ void k_zero_rho(double2 *__restrict__ I, int nu, int ntrans, int nrad, int g1, int g2, double a2) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nu * ntrans) return;
    const int u = idx / ntrans;
    double2 *v = I + (long)idx * nrad;
    if (u == 2 || u == 3) {
        const double2 f1 = v[g1], f2 = v[g2];
        v[0] = dmk((f1.x * a2 - f2.x) / (a2 - 1), (f1.y * a2 - f2.y) / (a2 - 1));
    } else {
        v[0] = dmk(0, 0);
    }
}

// Level tensor value of every cell of the full 2nx x 2ny offset grid for
// transmitter layers [0, nt): buf[cell][nt] (cells without terms stay 0).
template <typename O>
__global__ void k_cells_level(const int *__restrict__ rowptr, const Term *__restrict__ terms,
                              const double2 *__restrict__ IA, const double2 *__restrict__ IB, int ntrans, int nseg,
                              int ncell, O *__restrict__ buf) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)ncell * ntrans) return;
    const int cell = (int)(idx / ntrans), t = (int)(idx - (long)cell * ntrans);
    double2 acc = dmk(0, 0);
    for (int e = rowptr[cell]; e < rowptr[cell + 1]; e++) {
        const Term tm = terms[e];
        const long o = ((long)tm.src * nseg + tm.seg) * ntrans + t;
        const double2 a = IA[o], b = IB[o];
        acc.x = fma(tm.wa, a.x, fma(tm.wb, b.x, acc.x));
        acc.y = fma(tm.wa, a.y, fma(tm.wb, b.y, acc.y));
    }
    buf[idx] = cell_out<O>(acc);
}

// k_cells_level for the mixed form: Dot2 on float pairs, rounded to complex64
__global__ void k_cells_level_ds(const int *__restrict__ rowptr, const Term *__restrict__ terms,
                                 const float4 *__restrict__ IA, const float4 *__restrict__ IB, int ntrans, int nseg,
                                 int ncell, float2 *__restrict__ buf) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)ncell * ntrans) return;
    const int cell = (int)(idx / ntrans), t = (int)(idx - (long)cell * ntrans);
    float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
    for (int e = rowptr[cell]; e < rowptr[cell + 1]; e++) {
        const Term tm = terms[e];
        const long o = ((long)tm.src * nseg + tm.seg) * ntrans + t;
        float wah, wal, wbh, wbl;
        ds_split(tm.wa, wah, wal);
        ds_split(tm.wb, wbh, wbl);
        const float4 a = IA[o], b = IB[o];
        ds_dot2(sr, cr, wah, wal, a.x, a.y);
        ds_dot2(sr, cr, wbh, wbl, b.x, b.y);
        ds_dot2(si, ci, wah, wal, a.z, a.w);
        ds_dot2(si, ci, wbh, wbl, b.z, b.w);
    }
    buf[idx] = make_float2(__fadd_rn(sr, cr), __fadd_rn(si, ci));
}


// Component tables of the level tensors, in the order of level_components:
// E: xx yy zz xy xz yz zx zy; H: xx yx xy xz yz zx zy. QSigns (QSign.cs:31-39)
// and (integral factor, scalar) of AddToQBuffAlong{X,Y}{Electric,Magnetic}
// (GreenTensorCalculator.cs:505-552); 0 = not filled in that direction.
const int kLvQX[2][8] = {{1, -1, -1, -1, 1, 1, 1, 1}, {-1, 1, -1, 1, 1, 1, 1, 0}};
const int kLvQY[2][8] = {{-1, 1, -1, -1, 1, 1, 1, 1}, {-1, -1, 1, 1, 1, 1, 1, 0}};
const int kLvQXS[2][8] = {{1, -1, -1, 1, -1, 1, -1, 1}, {1, 1, -1, 1, -1, 1, -1, 0}};
const int kLvQYS[2][8] = {{-1, 1, -1, 1, 1, -1, 1, -1}, {1, -1, 1, 1, 1, -1, 1, 0}};
const int kLvFacX[2][8] = {{2, 2, 2, 3, 0, 1, 0, 1}, {3, 2, 2, 1, 0, 1, 0, 0}};
const int kLvSrcX[2][8] = {{1, 2, 5, 2, 0, 3, 0, 4}, {2, 1, 2, 3, 0, 4, 0, 0}};
const int kLvFacY[2][8] = {{2, 2, 2, 3, 1, 0, 1, 0}, {3, 2, 2, 0, 1, 0, 1, 0}};
const int kLvSrcY[2][8] = {{2, 1, 5, 1, 3, 0, 4, 0}, {1, 2, 1, 0, 3, 0, 4, 0}};

// Term lists of all components of a level tensor over the full offset grid
// (AtoOLevelGreenTensorCalculator.cs:82-126 with GreenTensorCalculator.cs:166-437):
// knots at x = dx (i - 1/2) + shift_x, i in [-nx+1, nx], y likewise; cell
// (i, j) is row ((i < 0 ? 2nx + i : i) * 2ny + (j < 0 ? 2ny + j : j)). The
// face integrations are made once and shared by the components.
void level_terms(const GreenModel &m, const std::vector<double> &radii, double shx, double shy, int kind, int ncomp,
                 std::vector<std::vector<int>> &rowptr, std::vector<std::vector<Term>> &terms) {
    const int nx = m.nx, ny = m.ny, lx = -nx + 1, rx = nx, ly = -ny + 1, ry = ny;
    const double dx = m.dx, dy = m.dy;
    auto X = [&](int i) { return dx * (i - 0.5) + shx; };
    auto Y = [&](int j) { return dy * (j - 0.5) + shy; };
    const int w = ry - ly + 1;
    std::vector<Knot> kn((size_t)(rx - lx + 1) * w);
    for (int i = lx; i <= rx; i++)
        for (int j = ly; j <= ry; j++) kn[(size_t)(i - lx) * w + (j - ly)] = make_knot(radii, X(i), Y(j));
    std::vector<Knot> zx(w), zy(rx - lx + 1);
    for (int j = ly; j <= ry; j++) zx[j - ly] = make_knot(radii, 0.0, Y(j));
    for (int i = lx; i <= rx; i++) zy[i - lx] = make_knot(radii, X(i), 0.0);
    auto K = [&](int i, int j) { return kn[(size_t)(i - lx) * w + (j - ly)]; };
    auto row = [&](int i, int j) { return (int)((i < 0 ? 2 * nx + i : i) * (2 * ny) + (j < 0 ? 2 * ny + j : j)); };
    // events: one face integration (parts [p0, p0 + np)) added to 1 or 2 cells
    struct Ev {
        int dir, symm, ncell, cell[2], sign[2], p0, np;
    };
    std::vector<Ev> evs;
    std::vector<SegF> all, parts;
    auto push = [&](int dir, bool symm, int i, int j) {
        Ev e{dir, symm ? 1 : 0, 0, {0, 0}, {0, 0}, (int)all.size(), (int)parts.size()};
        const int lo = dir == 0 ? ly : lx, hi = dir == 0 ? ry : rx, v = dir == 0 ? j : i;
        auto cell = [&](int a, int b) { return dir == 0 ? row(i, b) : row(a, j); };
        if (v == lo) {
            e.cell[0] = dir == 0 ? cell(0, lo) : cell(lo, 0);
            e.sign[0] = -1;
            e.ncell = 1;
        } else if (v == hi) {
            e.cell[0] = dir == 0 ? cell(0, hi - 1) : cell(hi - 1, 0);
            e.sign[0] = 1;
            e.ncell = 1;
        } else {
            e.cell[0] = dir == 0 ? cell(0, v - 1) : cell(v - 1, 0);
            e.sign[0] = 1;
            e.cell[1] = dir == 0 ? cell(0, v) : cell(v, 0);
            e.sign[1] = -1;
            e.ncell = 2;
        }
        all.insert(all.end(), parts.begin(), parts.end());
        evs.push_back(e);
    };
    for (int j = ly; j <= ry; j++) {
        const double y = Y(j);
        for (int i = lx; i < rx; i++) {
            const double x1 = X(i), x2 = X(i + 1);
            if (x1 > 0 && x2 > 0) {
                integrate(radii, K(i, j), K(i + 1, j), x1, x2, y, parts);
                push(0, false, i, j);
            } else if (x1 < 0 && x2 < 0) {
                integrate(radii, K(i + 1, j), K(i, j), -x2, -x1, y, parts);
                push(0, true, i, j);
            } else {
                integrate(radii, zx[j - ly], K(i, j), 0.0, -x1, y, parts);
                push(0, true, i, j);
                integrate(radii, zx[j - ly], K(i + 1, j), 0.0, x2, y, parts);
                push(0, false, i, j);
            }
        }
    }
    for (int i = lx; i <= rx; i++) {
        const double x = X(i);
        for (int j = ly; j < ry; j++) {
            const double y1 = Y(j), y2 = Y(j + 1);
            if (y1 > 0 && y2 > 0) {
                integrate(radii, K(i, j), K(i, j + 1), y1, y2, x, parts);
                push(1, false, i, j);
            } else if (y1 < 0 && y2 < 0) {
                integrate(radii, K(i, j + 1), K(i, j), -y2, -y1, x, parts);
                push(1, true, i, j);
            } else {
                integrate(radii, zy[i - lx], K(i, j), 0.0, -y1, x, parts);
                push(1, true, i, j);
                integrate(radii, zy[i - lx], K(i, j + 1), 0.0, y2, x, parts);
                push(1, false, i, j);
            }
        }
    }
    const int ncell = 4 * nx * ny;
    rowptr.assign(ncomp, {});
    terms.assign(ncomp, {});
    for (int c = 0; c < ncomp; c++) {
        std::vector<int> &rp = rowptr[c];
        rp.assign(ncell + 1, 0);
        for (const Ev &e : evs) {
            if ((e.dir == 0 ? kLvFacX[kind][c] : kLvFacY[kind][c]) == 0) continue;
            for (int k = 0; k < e.ncell; k++) rp[e.cell[k] + 1] += e.np;
        }
        for (int r = 0; r < ncell; r++) rp[r + 1] += rp[r];
        std::vector<int> fill(rp.begin(), rp.end() - 1);
        std::vector<Term> &tl = terms[c];
        tl.resize(rp[ncell]);
        for (const Ev &e : evs) {
            const int fac = e.dir == 0 ? kLvFacX[kind][c] : kLvFacY[kind][c];
            if (fac == 0) continue;
            const int src = e.dir == 0 ? kLvSrcX[kind][c] : kLvSrcY[kind][c];
            const int q = e.dir == 0 ? (e.symm ? kLvQXS[kind][c] : kLvQX[kind][c])
                                     : (e.symm ? kLvQYS[kind][c] : kLvQY[kind][c]);
            for (int k = 0; k < e.ncell; k++) {
                const double wgt = (double)(e.sign[k] * q);
                for (int pi = 0; pi < e.np; pi++) {
                    const SegF &p = all[e.p0 + pi];
                    tl[fill[e.cell[k]]++] = Term{p.seg, src - 1, wgt * fac_a(p.f, fac), wgt * fac_b(p.f, fac)};
                }
            }
        }
    }
}

// ScalarPlansCreater.FindRhoMin(numberOfCells, cellSize, shift) for the
// anomaly at the origin (ScalarPlansCreater.cs:240-262), in integer
// micrometres as the reference's decimal arithmetic is exact.
double level_rho_min_1d(int n, double cell, double shift) {
    auto um = [](double v) { return std::llround(v * 1e6); };
    const long long c = um(cell), sh = um(shift);
    const long long a_start = -c / 2, a_end = c * n - c / 2;
    const long long y_start = sh - c / 2, y_end = y_start + c * n;
    auto between = [](long long v, long long lo, long long hi) { return v >= lo && v <= hi; };
    if (between(y_start, a_start, a_end) || between(y_end, a_start, a_end)) {
        const long long rem = std::llabs(a_start - y_start) % c;
        if (rem == 0) return (double)(c / 2) * 1e-6;
        return (double)std::llabs(c / 2 - rem) * 1e-6;
    }
    const long long lc = 0, rc = c * (n - 1);
    const long long v = std::min(std::min(std::llabs(y_start - lc), std::llabs(y_start - rc)),
                                 std::min(std::llabs(y_end - lc), std::llabs(y_end - rc)));
    return (double)v * 1e-6;
}

// FindRhoMaxByFourPoints (ScalarPlansCreater.cs:220-233)
double level_rho_max4(const GreenModel &m, double sx, double sy, double x0, double y0) {
    const double x1 = sx - m.dx / 2, y1 = sy - m.dy / 2, x2 = x1 + m.dx * m.nx, y2 = y1 + m.dy * m.ny;
    auto d = [](double a, double b) { return std::sqrt(a * a + b * b); };
    return std::max(std::max(d(x1 - x0, y1 - y0), d(x2 - x0, y1 - y0)), std::max(d(x2 - x0, y2 - y0), d(x1 - x0, y2 - y0)));
}

}  // namespace

// ModelUtils.FindCorrespondingBackgroundLayerIndex (ModelUtils.cs:27-50)
// sums depths and thicknesses in C# decimal; integer micrometres keep those
// sums exact here for every length given to 1e-6 m.
std::vector<int> background_indices(const GreenModel &m) {
    auto um = [](double v) { return std::llround(v * 1e6); };
    std::vector<int> out(m.nz);
    for (int k = 0; k < m.nz; k++) {
        const long long start = um(m.depth[k]), end = um(m.depth[k]) + um(m.thick[k]);
        long long ss = um(m.zero_air_level);
        int found = -1;
        for (size_t i = 0; i < m.bg_thick.size(); i++) {
            const long long es = ss + um(m.bg_thick[i]);
            if (start >= ss && end <= es) {
                found = (int)i;
                break;
            }
            ss = es;
        }
        if (found < 0)
            throw Error(EGX_ERR_MODEL, "anomaly layer " + std::to_string(k) + " is not inside one background layer");
        out[k] = found;
    }
    return out;
}


// The filter taps in constant memory, once per device (contexts on other
// host threads may build at the same time).
static void load_hankel_taps() {
    static std::mutex mu;
    static std::set<int> loaded;
    int dev = 0;
    EGX_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (loaded.count(dev)) return;
    EGX_CUDA(cudaMemcpyToSymbol(c_h0, kHankelJ0, sizeof(kHankelJ0)));
    EGX_CUDA(cudaMemcpyToSymbol(c_h1, kHankelJ1, sizeof(kHankelJ1)));
    loaded.insert(dev);
}

void build_green(const GreenModel &m, int n_hankels, cudaStream_t s, DevBuf &quad, GreenBuildStats *stats,
                 long *launches, Timers *tm, GreenWorkspace *ws, bool lateral_fft32) {
    auto t_start = std::chrono::steady_clock::now();
    EGX_CHECK(m.nx > 0 && m.ny > 0 && m.nz > 0 && m.dx > 0 && m.dy > 0, EGX_ERR_INVALID, "bad model dimensions");
    const int L = (int)m.bg_thick.size();
    EGX_CHECK(L >= 3 && L <= kMaxLayers, EGX_ERR_INVALID, "background must have 3.." + std::to_string(kMaxLayers) +
                                                              " layers including both half-spaces");
    background_indices(m);
    load_hankel_taps();
    // ---- background
    LayerArgs la{};
    la.L = L;
    la.omega = m.omega;
    std::vector<double> tops(L + 1);
    tops[0] = m.zero_air_level;
    for (int k = 0; k < L; k++) tops[k + 1] = tops[k] + m.bg_thick[k];
    std::vector<cd> zb(L);
    for (int k = 0; k < L; k++) {
        zb[k] = cd(m.bg_sigma[k], -m.omega * kEps0);
        la.zeta[k] = make_double2(zb[k].real(), zb[k].imag());
        la.thick[k] = m.bg_thick[k];
        la.tops[k] = tops[k];
    }
    la.tops[L] = tops[L];
    for (int k = 0; k < L - 1; k++) {
        cd v = zb[k + 1] / zb[k];
        la.alpha_s[k] = make_double2(v.real(), v.imag());
    }
    for (int k = 1; k < L; k++) {
        cd v = zb[k - 1] / zb[k];
        la.beta_s[k] = make_double2(v.real(), v.imag());
    }
    // ---- plan
    const double step = rho_step();
    const double half1 = m.dx / 2.0, half2 = m.dy / 2.0;
    const double rho_min = std::min(half1, half2);
    const double mxx = m.nx * m.dx - half1, mxy = m.ny * m.dy - half2;
    const double rho_max = std::sqrt(mxx * mxx + mxy * mxy);
    const int nh = std::abs(n_hankels);
    EGX_CHECK(nh >= 1, EGX_ERR_INVALID, "NumberOfHankels must be non-zero");
    std::vector<std::vector<double>> items;
    items.push_back(rho_from_min(rho_min, rho_max, step));
    const double r2 = items[0].back(), r1 = items[0][items[0].size() - 2];
    const double lin = (r2 - r1) / nh;
    for (int i = 1; i < nh; i++) items.push_back(rho_from_max(rho_min, r2 - i * lin, step));
    // merge
    struct RI {
        double r;
        int item, idx;
    };
    std::vector<RI> all;
    for (int it = 0; it < (int)items.size(); it++)
        for (int j = 0; j < (int)items[it].size(); j++) all.push_back({items[it][j], it, j});
    std::stable_sort(all.begin(), all.end(), [](const RI &a, const RI &b) { return a.r < b.r; });
    std::vector<double> radii(all.size());
    std::vector<std::vector<int>> gidx(items.size());
    for (size_t it = 0; it < items.size(); it++) gidx[it].resize(items[it].size());
    for (size_t g = 0; g < all.size(); g++) {
        radii[g] = all[g].r;
        gidx[all[g].item][all[g].idx] = (int)g;
        if (g > 0) EGX_CHECK(radii[g] != radii[g - 1], EGX_ERR_INVALID, "duplicate radii across plan items");
    }
    const int nrad = (int)radii.size();
    std::vector<std::vector<double>> lams;
    std::vector<long> col0;
    long nl_total = 0;
    for (auto &rho : items) {
        lams.push_back(lambdas_for(rho, step));
        col0.push_back(nl_total);
        nl_total += (long)lams.back().size();
    }
    if (stats) {
        stats->n_items = (int)items.size();
        stats->n_radii = nrad;
        stats->n_lambda = nl_total;
    }
    // ---- transceivers
    std::vector<double> bthick(m.bg_thick.begin(), m.bg_thick.end());
    auto make_trans = [&](int rc, int tr) {
        Trans t;
        t.r1 = m.depth[rc];
        t.r2 = m.depth[rc] + m.thick[rc];
        t.s1 = m.depth[tr];
        t.s2 = m.depth[tr] + m.thick[tr];
        double zwork = t.r1 + (t.r2 - t.r1) / 2;
        t.r = layer_of(tops, bthick, zwork);
        t.s = layer_of(tops, bthick, t.s1 + (t.s2 - t.s1) / 2);
        EGX_CHECK(t.r + 1 < L && t.s + 1 < L, EGX_ERR_MODEL, "anomaly layer inside the lower half-space");
        if (zwork > t.s1 && zwork < t.s2) t.kase = 0;
        else if (zwork >= t.s2) t.kase = 1;
        else t.kase = 2;
        return t;
    };
    std::vector<Trans> asym, symm;
    for (int rc = 0; rc < m.nz; rc++)
        for (int tr = 0; tr < m.nz; tr++) asym.push_back(make_trans(rc, tr));
    for (int tr = 0; tr < m.nz; tr++)
        for (int rc = 0; rc <= tr; rc++) symm.push_back(make_trans(rc, tr));

    GreenDims gd{m.nx, m.ny, m.nz};
    const int Bs = gd.Bs();
    quad.ensure((size_t)gd.Q() * Bs * sizeof(double2));
    EGX_CUDA(cudaMemsetAsync(quad.p, 0, (size_t)gd.Q() * Bs * sizeof(double2), s));  // row padding stays zero

    GreenWorkspace local_ws;
    GreenWorkspace &w = ws ? *ws : local_ws;
    DevBuf &d_lam = w.d_lam, &d_lay = w.d_lay, &d_trans = w.d_trans, &d_U = w.d_U, &d_I = w.d_I, &d_rho = w.d_rho,
           &d_gidx = w.d_gidx, &d_flags = w.d_flags, &d_neg = w.d_neg, &d_radii = w.d_radii, &d_IA = w.d_IA,
           &d_IB = w.d_IB, &d_buf = w.d_buf;
    {
        std::vector<double> key = {(double)m.nx, (double)m.ny, m.dx, m.dy};
        key.insert(key.end(), radii.begin(), radii.end());
        if (key != w.key) {
            for (bool &c : w.cached) c = false;
            w.key = key;
        }
    }
    FftPlan p0 = make_fft_plan(2 * m.nx), p1 = make_fft_plan(2 * m.ny);
    DevBuf &tw0 = w.tw0, &tw1 = w.tw1;
    {
        std::vector<double> t0 = twiddles(2 * m.nx), t1 = twiddles(2 * m.ny);
        dev_upload(tw0, t0, s);
        dev_upload(tw1, t1, s);
        if (lateral_fft32) {
            dev_upload(w.tw0_32, std::vector<float>(t0.begin(), t0.end()), s);
            dev_upload(w.tw1_32, std::vector<float>(t1.begin(), t1.end()), s);
        }
    }
    double *radii_dev = dev_upload(d_radii, radii, s);

    // the two halves: asym (U3 -> xz, yz), symm (U1, U2, U5 -> xx, xy, yy, zz)
    for (int half = 0; half < 2; half++) {
        auto t_half = std::chrono::steady_clock::now();
        const std::vector<Trans> &tl = half == 0 ? asym : symm;
        const int ntrans = (int)tl.size();
        const int which = half == 0 ? 4 : (1 | 2 | 16);
        const int nu = half == 0 ? 1 : 3;
        std::vector<int> use_h0 = half == 0 ? std::vector<int>{1} : std::vector<int>{0, 0, 0};
        std::vector<int> negate = half == 0 ? std::vector<int>{0} : std::vector<int>{1, 0, 0};
        Trans *dtrans = dev_upload(d_trans, tl, s);
        d_U.ensure((size_t)nu * ntrans * nl_total * sizeof(double2));
        d_I.ensure((size_t)nu * ntrans * nrad * sizeof(double2));
        int *dflags = dev_upload(d_flags, use_h0, s);
        int *dneg = dev_upload(d_neg, negate, s);
        for (size_t it = 0; it < items.size(); it++) {
            const int nl = (int)lams[it].size();
            double *dl = dev_upload(d_lam, lams[it], s);
            d_lay.ensure((size_t)10 * L * nl * sizeof(double2));
            int ev = tm ? tm->begin(EGX_K_GREEN_LAYERS, s) : -1;
            k_layers<<<(nl + 127) / 128, 128, 0, s>>>(dl, nl, la, d_lay.as<double2>());
            k_chain_factors<<<(nl + 127) / 128, 128, 0, s>>>(nl, la, d_lay.as<double2>());
            if (launches) *launches += 1;
            if (tm) tm->end(ev, s);
            long nthreads = (long)ntrans * nl;
            ev = tm ? tm->begin(EGX_K_GREEN_KERNELS, s) : -1;
            k_kernels<<<(unsigned)((nthreads + 127) / 128), 128, 0, s>>>(dl, nl, d_lay.as<double2>(), la, dtrans,
                                                                          ntrans, which, d_U.as<double2>(), nl_total,
                                                                          col0[it]);
            if (tm) tm->end(ev, s);
            const int nrho = (int)items[it].size();
            double *drho = dev_upload(d_rho, items[it], s);
            int *dg = dev_upload(d_gidx, gidx[it], s);
            long nh_threads = (long)nu * ntrans * nrho;
            ev = tm ? tm->begin(EGX_K_GREEN_HANKEL, s) : -1;
            k_hankel<<<(unsigned)((nh_threads + 127) / 128), 128, 0, s>>>(d_U.as<double2>(), nu, ntrans, nl_total,
                                                                           col0[it], nrho, drho, dg, dflags, dneg,
                                                                           d_I.as<double2>(), nrad, 2.0 * M_PI);
            if (tm) tm->end(ev, s);
            // the per-item uploads above reuse buffers: finish before the next item
            EGX_CUDA(cudaStreamSynchronize(s));
            if (launches) *launches += 3;
        }
        const int nseg = nrad - 1;
        d_IA.ensure((size_t)nu * nseg * ntrans * sizeof(double2));
        d_IB.ensure((size_t)nu * nseg * ntrans * sizeof(double2));
        // the mixed form's face sums run in double-FP32 on float pairs
        const bool face_ds = lateral_fft32 && fft_lines_sym_ok(2 * m.nx) && fft_lines_sym_ok(2 * m.ny);
        if (face_ds) {
            w.d_IA32.ensure((size_t)nu * nseg * ntrans * sizeof(float4));
            w.d_IB32.ensure((size_t)nu * nseg * ntrans * sizeof(float4));
        }
        {
            long n = (long)nu * nseg * ntrans;
            k_segments<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
                d_I.as<double2>(), nu, ntrans, nrad, radii_dev, d_IA.as<double2>(), d_IB.as<double2>(),
                face_ds ? w.d_IA32.as<float4>() : nullptr, face_ds ? w.d_IB32.as<float4>() : nullptr);
            if (launches) *launches += 1;
        }
        EGX_CUDA(cudaGetLastError());
        EGX_CUDA(cudaStreamSynchronize(s));
        if (stats) stats->ms_scalars += ms_since(t_half);
        // source slot of each scalar in the IA/IB arrays of this half
        int slot[6] = {0, 0, 1, 0, 0, 2};  // I1 -> 0, I2 -> 1, I5 -> 2 (symm); I3 -> 0 (asym)
        const int comps_asym[2] = {4, 5}, comps_symm[4] = {0, 1, 2, 3};
        const int *comps = half == 0 ? comps_asym : comps_symm;
        const int ncomp = half == 0 ? 2 : 4;
        // one FFT column per transceiver: nz*nz for xz/yz, nz(nz+1)/2 for the
        // packed components (k_extract pads the xz/yz rows on the way out)
        const int blk = ntrans;
        EGX_CHECK(ntrans == (half == 0 ? m.nz * m.nz : gd.S()), EGX_ERR_INVALID, "transceiver count mismatch");
        const int S = gd.S(), A = gd.A();
        const int offs[6] = {0, S, 2 * S, 3 * S, 4 * S, 4 * S + A};
        const int px[6] = {1, -1, 1, 1, -1, 1}, py[6] = {1, -1, 1, 1, 1, -1};
        // compact: the real-space quadrant only, its mirror images generated
        // by the FFT's loads (half the y lines, a quarter of the memory);
        // otherwise the full 2nx x 2ny grid populated by mirroring
        const int n0 = 2 * m.nx, n1 = 2 * m.ny;
        const bool compact = fft_lines_sym_ok(n0) && fft_lines_sym_ok(n1);
        const bool fft32 = lateral_fft32 && compact;
        const long cells4 = compact ? (long)(m.nx + 1) * (m.ny + 1) : 4L * m.nx * m.ny;
        const int row = compact ? m.ny + 1 : n1;
        int tc = (int)std::min<long>(blk, std::max<long>(1, (long)(1.5e9 / (cells4 * sizeof(double2)))));
        if (fft32)
            w.d_buf32.ensure((size_t)cells4 * tc * sizeof(float2));
        else
            d_buf.ensure((size_t)cells4 * tc * sizeof(double2));
        for (int ci = 0; ci < ncomp; ci++) {
            const int c = comps[ci];
            auto t_int = std::chrono::steady_clock::now();
            if (!w.cached[c]) {
                // the term lists depend on the lateral mesh and radii only:
                // made once and reused for every frequency of the model
                std::vector<int> rowptr;
                std::vector<Term> terms;
                cell_terms(m, radii, c, slot, rowptr, terms);
                dev_upload(w.rowptr[c], rowptr, s);
                dev_upload(w.terms[c], terms, s);
                EGX_CUDA(cudaStreamSynchronize(s));
                w.nterms[c] = (long)terms.size();
                w.cached[c] = true;
            }
            if (stats) stats->face_terms += w.nterms[c];
            const int *drow = w.rowptr[c].as<int>();
            const Term *dterm = w.terms[c].as<Term>();
            for (int t0 = 0; t0 < blk; t0 += tc) {
                const int tcc = std::min(tc, blk - t0);
                if (!compact) EGX_CUDA(cudaMemsetAsync(d_buf.p, 0, (size_t)cells4 * tcc * sizeof(double2), s));
                dim3 grid(m.nx * m.ny, (tcc + 127) / 128);
                int ev = tm ? tm->begin(EGX_K_GREEN_CELLS, s) : -1;
                if (fft32)
                    k_cells_ds<<<grid, 128, 0, s>>>(drow, dterm, w.d_IA32.as<float4>(), w.d_IB32.as<float4>(),
                                                    ntrans, nseg, m.nx, m.ny, t0, tcc, px[c], py[c], 1,
                                                    w.d_buf32.as<float2>());
                else
                    k_cells<double2><<<grid, 128, 0, s>>>(drow, dterm, d_IA.as<double2>(), d_IB.as<double2>(), ntrans,
                                                          nseg, m.nx, m.ny, t0, tcc, px[c], py[c], compact ? 1 : 0,
                                                          d_buf.as<double2>());
                if (tm) tm->end(ev, s);
                EGX_CUDA(cudaGetLastError());
                ev = tm ? tm->begin(EGX_K_GREEN_FFT, s) : -1;
                if (fft32) {
                    // as below, in complex64
                    fft_lines_sym<float>(w.d_buf32.as<float2>(), m.nx, (long)row * tcc, tcc, tcc, py[c], m.ny + 1, n1,
                                         w.tw1_32.as<float2>(), -1, s, launches);
                    fft_lines_sym<float>(w.d_buf32.as<float2>(), m.ny + 1, tcc, (long)row * tcc, tcc, px[c], m.nx + 1,
                                         n0, w.tw0_32.as<float2>(), -1, s, launches);
                } else if (compact) {
                    // y along the nx computed rows, ky <= ny kept; then x along
                    // ky <= ny, kx <= nx kept (row nx of the input is zero)
                    fft_lines_sym<double>(d_buf.as<double2>(), m.nx, (long)row * tcc, tcc, tcc, py[c], m.ny + 1, n1,
                                          tw1.as<double2>(), -1, s, launches);
                    fft_lines_sym<double>(d_buf.as<double2>(), m.ny + 1, tcc, (long)row * tcc, tcc, px[c], m.nx + 1,
                                          n0, tw0.as<double2>(), -1, s, launches);
                } else {
                    // y along all 2nx rows; x along ky <= ny, kx <= nx kept
                    fft_lines<double>(d_buf.as<double2>(), n0, (long)n1 * tcc, tcc, tcc, n1, n1, p1,
                                      tw1.as<double2>(), -1, s, launches);
                    fft_lines<double>(d_buf.as<double2>(), m.ny + 1, tcc, (long)n1 * tcc, tcc, n0, m.nx + 1, p0,
                                      tw0.as<double2>(), -1, s, launches);
                }
                if (tm) tm->end(ev, s);
                long n = (long)(m.nx + 1) * (m.ny + 1) * tcc;
                if (fft32)
                    k_extract<float2><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
                        w.d_buf32.as<float2>(), m.nx, m.ny, row, tcc, Bs, offs[c], t0, m.nz, c >= 4 ? 1 : 0,
                        quad.as<double2>());
                else
                    k_extract<double2><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
                        d_buf.as<double2>(), m.nx, m.ny, row, tcc, Bs, offs[c], t0, m.nz, c >= 4 ? 1 : 0,
                        quad.as<double2>());
                EGX_CUDA(cudaGetLastError());
                if (launches) *launches += 2;
            }
            EGX_CUDA(cudaStreamSynchronize(s));
            if (stats) stats->ms_integrate += ms_since(t_int);
        }
    }
    (void)t_start;
}

int level_components(int kind) { return kind == 0 ? 8 : 7; }

void build_level_green(const GreenModel &m, int n_hankels, double z, double shx, double shy, int kind, cudaStream_t s,
                       DevBuf &out, long *launches, GreenWorkspace &w, bool fft32) {
    EGX_CHECK(m.nx > 0 && m.ny > 0 && m.nz > 0 && m.dx > 0 && m.dy > 0, EGX_ERR_INVALID, "bad model dimensions");
    EGX_CHECK(kind == 0 || kind == 1, EGX_ERR_INVALID, "level tensor kind must be 0 (E) or 1 (H)");
    const int L = (int)m.bg_thick.size();
    EGX_CHECK(L >= 3 && L <= kMaxLayers, EGX_ERR_INVALID, "background must have 3.." + std::to_string(kMaxLayers) +
                                                              " layers including both half-spaces");
    load_hankel_taps();
    // ---- background (as build_green)
    LayerArgs la{};
    la.L = L;
    la.omega = m.omega;
    std::vector<double> tops(L + 1);
    tops[0] = m.zero_air_level;
    for (int k = 0; k < L; k++) tops[k + 1] = tops[k] + m.bg_thick[k];
    std::vector<cd> zb(L);
    for (int k = 0; k < L; k++) {
        zb[k] = cd(m.bg_sigma[k], -m.omega * kEps0);
        la.zeta[k] = make_double2(zb[k].real(), zb[k].imag());
        la.thick[k] = m.bg_thick[k];
        la.tops[k] = tops[k];
    }
    la.tops[L] = tops[L];
    for (int k = 0; k < L - 1; k++) {
        cd v = zb[k + 1] / zb[k];
        la.alpha_s[k] = make_double2(v.real(), v.imag());
    }
    for (int k = 1; k < L; k++) {
        cd v = zb[k - 1] / zb[k];
        la.beta_s[k] = make_double2(v.real(), v.imag());
    }
    // ---- plan (CreateForAnomalyToObservationLevels, ScalarPlansCreater.cs:51-66)
    const double step = rho_step();
    double rho_min = std::min(level_rho_min_1d(m.nx, m.dx, shx), level_rho_min_1d(m.ny, m.dy, shy));
    const double ex = m.dx * (m.nx - 1), ey = m.dy * (m.ny - 1);
    const double rho_max = std::max(std::max(level_rho_max4(m, shx, shy, 0, 0), level_rho_max4(m, shx, shy, 0, ey)),
                                    std::max(level_rho_max4(m, shx, shy, ex, ey), level_rho_max4(m, shx, shy, ex, 0)));
    const bool add_zero = rho_min <= 0;
    if (add_zero) rho_min = std::min(m.dx, m.dy) * 0.001;
    const int nh = std::abs(n_hankels);
    EGX_CHECK(nh >= 1, EGX_ERR_INVALID, "NumberOfHankels must be non-zero");
    std::vector<std::vector<double>> items;
    items.push_back(rho_from_min(rho_min, rho_max, step));
    {
        const double r2 = items[0].back(), r1 = items[0][items[0].size() - 2], lin = (r2 - r1) / nh;
        for (int i = 1; i < nh; i++) items.push_back(rho_from_max(rho_min, r2 - i * lin, step));
    }
    struct RI {
        double r;
        int item, idx;
    };
    std::vector<RI> all;
    if (add_zero) all.push_back({0.0, 0, -1});
    for (int it = 0; it < (int)items.size(); it++)
        for (int j = 0; j < (int)items[it].size(); j++) all.push_back({items[it][j], it, j});
    std::stable_sort(all.begin(), all.end(), [](const RI &a, const RI &b) { return a.r < b.r; });
    std::vector<double> radii(all.size());
    std::vector<std::vector<int>> gidx(items.size());
    for (size_t it = 0; it < items.size(); it++) gidx[it].resize(items[it].size());
    for (size_t g = 0; g < all.size(); g++) {
        radii[g] = all[g].r;
        if (all[g].idx >= 0) gidx[all[g].item][all[g].idx] = (int)g;
        if (g > 0) EGX_CHECK(radii[g] != radii[g - 1], EGX_ERR_INVALID, "duplicate radii across plan items");
    }
    const int nrad = (int)radii.size();
    std::vector<std::vector<double>> lams;
    std::vector<long> col0;
    long nl_total = 0;
    for (auto &rho : items) {
        lams.push_back(lambdas_for(rho, step));
        col0.push_back(nl_total);
        nl_total += (long)lams.back().size();
    }
    // ---- transceivers: the level point above/below/inside each anomaly layer
    std::vector<double> bthick(m.bg_thick.begin(), m.bg_thick.end());
    std::vector<Trans> tl;
    for (int k = 0; k < m.nz; k++) {
        Trans t;
        t.r1 = t.r2 = z;
        t.s1 = m.depth[k];
        t.s2 = m.depth[k] + m.thick[k];
        t.r = layer_of(tops, bthick, z);
        t.s = layer_of(tops, bthick, t.s1 + (t.s2 - t.s1) / 2);
        EGX_CHECK(t.r + 1 < L && t.s + 1 < L, EGX_ERR_MODEL, "level or anomaly layer inside the lower half-space");
        t.kase = (z > t.s1 && z < t.s2) ? 0 : (z >= t.s2 ? 1 : 2);
        tl.push_back(t);
    }
    const int ntrans = m.nz;
    const int nu = kind == 0 ? 5 : 4;
    // Hankel order and signs (CalculateHankelForE/H, NormalizeAfterHankelForE/H)
    const std::vector<int> use_h0 = kind == 0 ? std::vector<int>{0, 0, 1, 1, 0} : std::vector<int>{0, 0, 1, 1};
    const std::vector<int> negate = kind == 0 ? std::vector<int>{1, 0, 0, 0, 0} : std::vector<int>{1, 1, 1, 0};
    const double den = kind == 0 ? 2.0 * M_PI : 4.0 * M_PI;
    Trans *dtrans = dev_upload(w.d_trans, tl, s);
    int *dflags = dev_upload(w.d_flags, use_h0, s);
    int *dneg = dev_upload(w.d_neg, negate, s);
    double *radii_dev = dev_upload(w.d_radii, radii, s);
    w.d_U.ensure((size_t)nu * ntrans * nl_total * sizeof(double2));
    w.d_I.ensure((size_t)nu * ntrans * nrad * sizeof(double2));
    for (size_t it = 0; it < items.size(); it++) {
        const int nl = (int)lams[it].size();
        double *dl = dev_upload(w.d_lam, lams[it], s);
        w.d_lay.ensure((size_t)10 * L * nl * sizeof(double2));
        k_layers<<<(nl + 127) / 128, 128, 0, s>>>(dl, nl, la, w.d_lay.as<double2>());
        k_chain_factors<<<(nl + 127) / 128, 128, 0, s>>>(nl, la, w.d_lay.as<double2>());
        if (launches) *launches += 1;
        const long nthreads = (long)ntrans * nl;
        k_kernels_vtp<<<(unsigned)((nthreads + 127) / 128), 128, 0, s>>>(
            dl, nl, w.d_lay.as<double2>(), la, dtrans, ntrans, kind, w.d_U.as<double2>(), nl_total, col0[it]);
        const int nrho = (int)items[it].size();
        double *drho = dev_upload(w.d_rho, items[it], s);
        int *dg = dev_upload(w.d_gidx, gidx[it], s);
        const long nh_threads = (long)nu * ntrans * nrho;
        k_hankel<<<(unsigned)((nh_threads + 127) / 128), 128, 0, s>>>(w.d_U.as<double2>(), nu, ntrans, nl_total,
                                                                       col0[it], nrho, drho, dg, dflags, dneg,
                                                                       w.d_I.as<double2>(), nrad, den);
        EGX_CUDA(cudaStreamSynchronize(s));  // per-item uploads reuse buffers
        if (launches) *launches += 3;
    }
    if (add_zero) {
        const double a2 = step * step;
        k_zero_rho<<<(nu * ntrans + 127) / 128, 128, 0, s>>>(w.d_I.as<double2>(), nu, ntrans, nrad, gidx[0][1],
                                                             gidx[0][2], a2);
        if (launches) *launches += 1;
    }
    const int nseg = nrad - 1;
    w.d_IA.ensure((size_t)nu * nseg * ntrans * sizeof(double2));
    w.d_IB.ensure((size_t)nu * nseg * ntrans * sizeof(double2));
    if (fft32) {
        w.d_IA32.ensure((size_t)nu * nseg * ntrans * sizeof(float4));
        w.d_IB32.ensure((size_t)nu * nseg * ntrans * sizeof(float4));
    }
    {
        const long n = (long)nu * nseg * ntrans;
        k_segments<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
            w.d_I.as<double2>(), nu, ntrans, nrad, radii_dev, w.d_IA.as<double2>(), w.d_IB.as<double2>(),
            fft32 ? w.d_IA32.as<float4>() : nullptr, fft32 ? w.d_IB32.as<float4>() : nullptr);
        if (launches) *launches += 1;
    }
    EGX_CUDA(cudaGetLastError());
    // ---- face integration (term lists cached per geometry, shift and radii)
    const int ncomp = level_components(kind);
    {
        std::vector<double> key = {(double)m.nx, (double)m.ny, m.dx, m.dy, shx, shy};
        key.insert(key.end(), radii.begin(), radii.end());
        if (key != w.lkey[kind]) {
            std::vector<std::vector<int>> rp;
            std::vector<std::vector<Term>> tt;
            level_terms(m, radii, shx, shy, kind, ncomp, rp, tt);
            for (int c = 0; c < ncomp; c++) {
                dev_upload(w.lrow[kind][c], rp[c], s);
                dev_upload(w.lterm[kind][c], tt[c], s);
            }
            EGX_CUDA(cudaStreamSynchronize(s));
            w.lkey[kind] = key;
        }
    }
    const long ncell = 4L * m.nx * m.ny;
    const size_t comp_elems = (size_t)ncell * m.nz;
    out.ensure((size_t)ncomp * comp_elems * (fft32 ? sizeof(float2) : sizeof(double2)));
    const int n0 = 2 * m.nx, n1 = 2 * m.ny;
    FftPlan p0 = make_fft_plan(n0), p1 = make_fft_plan(n1);
    {
        std::vector<double> t0 = twiddles(n0), t1 = twiddles(n1);
        if (fft32) {
            dev_upload(w.tw0_32, std::vector<float>(t0.begin(), t0.end()), s);
            dev_upload(w.tw1_32, std::vector<float>(t1.begin(), t1.end()), s);
        } else {
            dev_upload(w.tw0, t0, s);
            dev_upload(w.tw1, t1, s);
        }
    }
    for (int c = 0; c < ncomp; c++) {
        const long n = ncell * m.nz;
        const int *rp = w.lrow[kind][c].as<int>();
        const Term *tt = w.lterm[kind][c].as<Term>();
        if (fft32) {
            // face sums in double-FP32 rounded to complex64 as written, the
            // 2-D FFT in complex64, the tensor kept in complex64
            float2 *g32 = out.as<float2>() + (size_t)c * comp_elems;
            k_cells_level_ds<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
                rp, tt, w.d_IA32.as<float4>(), w.d_IB32.as<float4>(), ntrans, nseg, (int)ncell, g32);
            EGX_CUDA(cudaGetLastError());
            fft_lines<float>(g32, n0, (long)n1 * m.nz, m.nz, m.nz, n1, n1, p1, w.tw1_32.as<float2>(), -1, s, launches);
            fft_lines<float>(g32, n1, m.nz, (long)n1 * m.nz, m.nz, n0, n0, p0, w.tw0_32.as<float2>(), -1, s, launches);
            if (launches) *launches += 1;
            continue;
        }
        double2 *g = out.as<double2>() + (size_t)c * comp_elems;
        k_cells_level<double2><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(rp, tt, w.d_IA.as<double2>(),
                                                                           w.d_IB.as<double2>(), ntrans, nseg,
                                                                           (int)ncell, g);
        EGX_CUDA(cudaGetLastError());
        // PerformGreenTensorFft: the full 2-D transform of every layer column
        fft_lines<double>(g, n0, (long)n1 * m.nz, m.nz, m.nz, n1, n1, p1, w.tw1.as<double2>(), -1, s, launches);
        fft_lines<double>(g, n1, m.nz, (long)n1 * m.nz, m.nz, n0, n0, p0, w.tw0.as<double2>(), -1, s, launches);
        if (launches) *launches += 1;
    }
    EGX_CUDA(cudaStreamSynchronize(s));
}

}  // namespace egx
