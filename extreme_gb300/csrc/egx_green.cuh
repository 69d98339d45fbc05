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

// Build the spectral tensor into `quad` (device, complex128, layout of
// GreenDims: quadrant points x [xx|xy|yy|zz|xz|yz] blocks).
void build_green(const GreenModel &m, int n_hankels, cudaStream_t s, DevBuf &quad, GreenBuildStats *stats,
                 long *launches, Timers *timers = nullptr);

// Index of the background layer holding each anomaly layer; throws
// EGX_ERR_MODEL when a layer straddles an interface (ModelUtils.cs:160-185).
std::vector<int> background_indices(const GreenModel &m);

}  // namespace egx
