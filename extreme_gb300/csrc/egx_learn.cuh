// Learned flexible preconditioner: a spectral network on the lateral grid
// (declarations shared by egx_learn.cu and the solver in egx_api.cu).
#pragma once

#include "egx_common.cuh"

struct egx_net;

namespace egx {

// z = v + rms(v) N(v / rms(v)) for `batch` complex64 vectors [batch][N] on
// the device (N = nx ny 3 nz in the anomaly layout), on stream s. Uses the
// log-conductivity set by egx_net_set_model.
void net_apply(egx_net *net, const float2 *v, float2 *z, int batch, cudaStream_t s, long *launches);

// nx ny 3 nz: the vector length the network was built for
long net_length(const egx_net *net);

}  // namespace egx
