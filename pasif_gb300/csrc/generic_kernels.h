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
// element-wise double -> compute precision
cudaError_t launch_convert(const double* src, void* dst, long long n, bool f32, cudaStream_t st);

}  // namespace pk
