// generic_kernels.h -- host launchers of the nvcc-built kernels.
#pragma once
#include <cuda_runtime.h>

#include "pk_args.h"

namespace pk {

cudaError_t launch_gen_fwd(const FwdArgs<double>& a, bool kahan, cudaStream_t st);
cudaError_t launch_gen_fwd(const FwdArgs<float>& a, bool kahan, cudaStream_t st);
cudaError_t launch_gen_adj(const AdjArgs<double>& a, cudaStream_t st);
cudaError_t launch_gen_adj(const AdjArgs<float>& a, cudaStream_t st);
cudaError_t launch_gen_refgrad(const RefGradArgs<double>& a, cudaStream_t st);
cudaError_t launch_gen_refgrad(const RefGradArgs<float>& a, cudaStream_t st);

// [B][k] double (host order) -> [k][B] in the compute precision, and back.
cudaError_t launch_to_interleaved(const double* src, void* dst, int B, int k, bool f32, cudaStream_t st);
cudaError_t launch_from_interleaved(const void* src, double* dst, int B, int k, bool f32, cudaStream_t st,
                                    double scale = 1.0);
// Measured FMA throughput of this GPU (FLOP/s, FMA = 2) in FP32 or FP64.
cudaError_t measure_fma_peak(bool f32, double* flops_per_s);
// Serving pools: src[m][k] double -> dst[k][C] columns slots[i]; the inverse
// gather (scaled); per-slot scalar scatters.
cudaError_t launch_scatter_cols(const double* src, void* dst, const int* slots, int m, int k, long long C, bool f32,
                                cudaStream_t st);
cudaError_t launch_gather_cols(const void* src, double* dst, const int* slots, int m, int k, long long C, bool f32,
                               double scale, cudaStream_t st);
cudaError_t launch_scatter_u32(const unsigned* src, unsigned* dst, const int* slots, int m, cudaStream_t st);
cudaError_t launch_scatter_i32(const int* src, int* dst, const int* slots, int m, cudaStream_t st);
cudaError_t launch_scatter_i64(const long long* src, long long* dst, const int* slots, int m, cudaStream_t st);
// [B][k] double -> [B][2k] double: high parts (v rounded to FP32) then low
// parts (v minus its high part), the extended-state mode's value split.
cudaError_t launch_split_hi_lo(const double* src, double* dst, int B, int k, cudaStream_t st);
// [k][B] FP32 high and low parts -> [B][k] double hi + lo (scaled).
cudaError_t launch_from_interleaved_pair(const float* hi, const float* lo, double* dst, int B, int k, double scale,
                                         cudaStream_t st);
// element-wise double -> compute precision
cudaError_t launch_convert(const double* src, void* dst, long long n, bool f32, cudaStream_t st);

}  // namespace pk
