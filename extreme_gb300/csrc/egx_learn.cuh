// Learned flexible preconditioner: a spectral network on the anomaly mesh
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

// Pointwise GEMM on the tcgen05 tensor cores (egx_learn_tc.cu): C[m, n] =
// sum_k A[m, k] B[k b_k + n b_n] (+ C[m, n] with accumulate), A row-major
// [M x K], C row-major [M x N], K and N in 1..32, BF16 operands, FP32
// accumulation; err receives EGX_ERR_TIMEOUT if a bounded wait expires.
bool pw_gemm_tc_fits(int K, int N);
void pw_gemm_tc(const float *A, int M, int K, const float *B, long b_k, long b_n, int N, float *C, bool accumulate,
                int *err, cudaStream_t s);

}  // namespace egx
