// jit.h -- pattern-specialised kernels compiled at run time with NVRTC.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "pattern.h"

namespace pasif {

// Per-parameter specialisation: a value shared by every instance of a batch
// (after rounding to the compute precision) is baked into the code as an
// exact hexadecimal literal; the others are loaded per instance.
struct Literals {
    std::vector<unsigned char> is_lit;   // size P
    std::vector<double> value;           // size P (meaningful where is_lit)
};

struct FwdKernelKey {
    bool f32 = false;
    bool kahan = false;
    unsigned long long max_mask = 0;
    unsigned long long sq_mask = 0;
    bool traj = false;
    int block = 128;
    int window = 0;                 // forcing window (0 = sample and hold)
    std::vector<double> wn, wc;     // its weights in the compute precision
};

struct JitKernel {
    cudaKernel_t fn = nullptr;
    int block = 128;
    int regs = 0;
    int local_bytes = 0;
};

// Source of the forward kernel for a pattern (exposed for tests and docs).
std::string fwd_source(const Pattern& pat, const Literals& lit, const FwdKernelKey& key);

// Compile (or fetch from the process-wide cache) the forward kernel.
// Returns false and sets err on failure.
bool get_fwd_kernel(const Pattern& pat, const Literals& lit, const FwdKernelKey& key,
                    JitKernel* out, std::string* err);

// Source and cached kernel of the exact adjoint (AdjArgs) for a pattern.
std::string adj_source(const Pattern& pat, const Literals& lit, bool f32, unsigned long long sq_mask);
bool get_adj_kernel(const Pattern& pat, const Literals& lit, bool f32, unsigned long long sq_mask, JitKernel* out,
                    std::string* err);
// Serving-pool chunk kernel (PoolArgs): values always loaded, no literals.
std::string pool_source(const Pattern& pat, const FwdKernelKey& key);
bool get_pool_kernel(const Pattern& pat, const FwdKernelKey& key, JitKernel* out, std::string* err);
// Compile a source without loading it (no GPU needed); report = compiler log.
bool compile_report(const std::string& src, std::string* report, std::string* err);

// Compile the forward kernel without loading it (no GPU needed) and return
// the compiler's resource report (registers, spills).
bool fwd_compile_report(const Pattern& pat, const Literals& lit, const FwdKernelKey& key, std::string* report,
                        std::string* err);

// Largest state size the register-resident specialisation accepts.
constexpr int kJitMaxN = 128;

}  // namespace pasif
