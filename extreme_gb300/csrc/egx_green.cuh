// Anomaly-to-anomaly Green tensor build on the device, FP64
// (Extreme.Cartesian/Forward/AtoA/AtoAGreenTensorCalculatorComponent.cs:82-279).
#pragma once

#include <vector>

#include "egx_fft.cuh"

namespace egx {

// Host description of the model geometry needed by the build.
struct GreenModel {
    int nx, ny, nz;
    double dx, dy;
    std::vector<double> depth, thick;    // anomaly layers [nz]
    std::vector<double> bg_thick;        // background [L]
    std::vector<double> bg_sigma;        // background [L]
    double zero_air_level;
    double omega;
};

struct GreenBuildStats {
    int n_items = 0;
    int n_radii = 0;
    long n_lambda = 0;
    long face_terms = 0;
    double ms_scalars = 0, ms_integrate = 0, ms_fft = 0;
};

// Device workspace of build_green that a context keeps across builds: the
// scratch buffers, and per component the face-integration term lists (CSR),
// which depend only on the lateral mesh and the radii -- not on frequency.
struct GreenWorkspace {
    DevBuf d_lam, d_lay, d_trans, d_U, d_I, d_rho, d_gidx, d_flags, d_neg, d_radii, d_IA, d_IB, d_buf, tw0, tw1;
    DevBuf d_buf32, tw0_32, tw1_32;  // the complex64 lateral FFT of the mixed form
    DevBuf d_IA32, d_IB32;           // its face-sum coefficients as float pairs
    std::vector<double> key;  // nx, ny, dx, dy and the radii of the cached term lists
    DevBuf rowptr[6], terms[6];
    long nterms[6] = {};
    bool cached[6] = {};
    // observation-level tensors (E: kind 0, H: kind 1): term lists per component,
    // keyed by the lateral mesh, the level's shift and the radii
    std::vector<double> lkey[2];
    DevBuf lrow[2][8], lterm[2][8];
};

// Components of a level tensor: E (kind 0) xx yy zz xy xz yz zx zy, H (kind 1)
// xx yx xy xz yz zx zy.
int level_components(int kind);

// Build the spectral anomaly-to-observation-level tensor of one kind at depth
// z with the level's lateral shift, in FP64 on the device
// (AtoOLevelGreenTensorCalculator.cs:21-126, AtoOCalculator.cs:120-176):
// out = [component][2nx][2ny][nz] complex128. With fft32 (the mixed form's
// level tensors) the face sums run in double-FP32, are rounded to complex64,
// and the 2-D FFT and `out` are complex64.
void build_level_green(const GreenModel &m, int n_hankels, double z, double shift_x, double shift_y, int kind,
                       cudaStream_t s, DevBuf &out, long *launches, GreenWorkspace &ws, bool fft32 = false);

// Build the spectral tensor into `quad` (device, complex128, layout of
// GreenDims: quadrant points x [xx|xy|yy|zz|xz|yz] blocks). The layer
// recursions, Hankel sums, segment and face integrals run in FP64; with
// `lateral_fft32` (and 2nx, 2ny in {64, 128, 256, 512}) the face integrals
// are rounded to complex64 and the 2-D lateral FFT runs in complex64, its
// result widened into `quad`.
void build_green(const GreenModel &m, int n_hankels, cudaStream_t s, DevBuf &quad, GreenBuildStats *stats,
                 long *launches, Timers *timers = nullptr, GreenWorkspace *ws = nullptr, bool lateral_fft32 = false);

// Index of the background layer holding each anomaly layer; throws
// EGX_ERR_MODEL when a layer straddles an interface (ModelUtils.cs:160-185).
std::vector<int> background_indices(const GreenModel &m);

}  // namespace egx
