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
    // Extended-state mode: the same for the low parts of the FP64 values
    // (v - (float)v, rounded to FP32); a term whose low part is the literal 0
    // drops out of the low-part right-hand side.
    std::vector<unsigned char> is_lit_lo;
    std::vector<double> value_lo;
};

struct FwdKernelKey {
    bool f32 = false;
    bool kahan = false;
    unsigned long long max_mask = 0;
    unsigned long long sq_mask = 0;
    int traj = 0;                   // 1: states every traj_every steps; 2: adjoint trajectory (state + stage inputs)
    int block = 128;
    int window = 0;                 // forcing window (0 = sample and hold)
    std::vector<double> wn, wc;     // its weights in the compute precision
    int slices = 0;                 // >= 2: warp-sliced kernel with that many warps per 32 systems
    bool ext = false;               // extended-state mode (FP32 stages, double-float state, low parts of the values)
    bool fast = false;              // PASIF_PLAN_FAST: shared products, folded RK sum (not the oracle's bits)
};

struct JitKernel {
    cudaKernel_t fn = nullptr;
    int block = 128;                // threads per block
    int per_block = 128;            // systems per block (32 for warp-sliced kernels)
    int smem = 0;                   // dynamic shared memory bytes
    int regs = 0;
    int local_bytes = 0;
};

// Warps per 32 systems of the warp-sliced kernels for a pattern: 0 (thread
// per system) where that layout is faster (small systems in FP32), unless
// `force`.  B: systems per launch (0: unknown, taken as large).
int ws_slices(const Pattern& pat, bool f32, bool force, int B = 0, bool ext = false);
// Same for the exact adjoint (sliced from smaller systems).
int ws_slices_adjoint(const Pattern& pat, bool f32, bool force, bool ext = false);
// Warps for n components (2..16).
int ws_split(int n, bool f32, bool force, bool adjoint, bool ext = false);

// Source of the forward kernel for a pattern (exposed for tests and docs).
std::string fwd_source(const Pattern& pat, const Literals& lit, const FwdKernelKey& key);

// Compile (or fetch from the process-wide cache) the forward kernel.
// Returns false and sets err on failure.
bool get_fwd_kernel(const Pattern& pat, const Literals& lit, const FwdKernelKey& key,
                    JitKernel* out, std::string* err);

// Source and cached kernel of the exact adjoint (AdjArgs) for a pattern.
// (slices >= 2: warp-sliced, with the forward passes' Kahan mode compiled in)
std::string adj_source(const Pattern& pat, const Literals& lit, bool f32, unsigned long long sq_mask, int slices = 0,
                       bool kahan = false, bool ext = false);
bool get_adj_kernel(const Pattern& pat, const Literals& lit, bool f32, bool kahan, unsigned long long sq_mask, int slices,
                    JitKernel* out, std::string* err, bool ext = false);
// Serving-pool chunk kernel (PoolArgs): values always loaded, no literals.
std::string pool_source(const Pattern& pat, const FwdKernelKey& key);
bool get_pool_kernel(const Pattern& pat, const FwdKernelKey& key, JitKernel* out, std::string* err);
// Compile a source without loading it (no GPU needed); report = compiler log.
bool compile_report(const std::string& src, std::string* report, std::string* err);

// Compile the forward kernel without loading it (no GPU needed) and return
// the compiler's resource report (registers, spills).
bool fwd_compile_report(const Pattern& pat, const Literals& lit, const FwdKernelKey& key, std::string* report,
                        std::string* err);

// Largest state size the register-resident specialisation accepts (thread
// per system, and warp-sliced).
constexpr int kJitMaxN = 128;
constexpr int kWsMaxN = 256;

}  // namespace pasif
