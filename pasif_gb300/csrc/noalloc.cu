// noalloc.cu -- a forward solve that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code that runs inside another
// framework's memory pool or under a strict memory budget, code that must not
// synchronise the device (cudaMalloc/cudaFree may), and applications that
// reserve all device memory up front and hand out slices of it.  For them,
// pasif_forward_noalloc runs the generic (pattern-interpreting) FP64 forward
// kernel with its work space -- the pattern, the instance values and state in
// the kernel's [k][n_sys] layout, the kernel's per-instance work vectors and a
// checked copy of the excitation indices -- in one fixed-size array that
// lives in the library's own device memory (a file-scope __device__ array).
// The caller passes inputs and outputs in device memory; nothing is
// allocated, on the device or on the host heap, and nothing waits for the
// device: the pattern travels as kernel arguments (no pageable-memory copy)
// and the excitation indices, which are device data, are checked on the
// device.
//
// Limits and rules:
//   * the array holds kNoallocBytes = 32 MiB on every GPU that loads the
//     library, for as long as the process lives: a 256-byte status block,
//     the pattern area (1 MiB - 256 B, <= 262080 integers), then
//     8 * n_sys * (P + 7 n) + 4 * n_sys bytes of work space (<= 31 MiB);
//     larger requests are rejected with PASIF_ERR_INVALID;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (a host-side name is not a device address); make
//     that first call before any stream capture;
//   * every call shares the one array and leaves its last contents there:
//     calls whose GPU work overlaps (different streams, threads) race.  The
//     status block is cleared at the start of every call's GPU work.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/pasif_gb300.h"
#include "generic_kernels.h"
#include "pk_args.h"

// Sets the thread-local message returned by pasif_last_error (capi.cpp).
void pasif_internal_set_error(const std::string& msg);

namespace {

constexpr size_t kNoallocBytes = 32u << 20;
constexpr size_t kStatusBytes = 256;
constexpr size_t kPatternBytes = 1u << 20;   // status block + pattern area
constexpr int kMaxDevices = 64;
constexpr int kChunkInts = 1000;            // pattern integers per upload launch (4 KB of arguments)

__device__ __align__(256) unsigned char pk_noalloc_scratch[kNoallocBytes];

// Status block at the start of the array: written by the last call's GPU work.
struct NoallocStatus {
    int bad;         // systems whose excitation index was outside [0, n_exc)
    int first_bad;   // lowest such system (n_sys when none)
};

std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Device address of pk_noalloc_scratch on the current device (set-up once
// per device).
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, pk_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

int fail(int code, const std::string& msg) {
    pasif_internal_set_error(msg);
    return code;
}

bool pow2(int w) { return w > 0 && !(w & (w - 1)); }

// Up to kChunkInts pattern integers passed by value (kernel arguments are
// copied when the launch is queued: no host buffer has to outlive the call).
struct IntChunk {
    int v[kChunkInts];
};

__global__ void put_ints(int* dst, IntChunk c, int count) {
    for (int i = threadIdx.x; i < count; i += blockDim.x) dst[i] = c.v[i];
}

// Appends to the flat pattern the per-destination term lists the generic
// kernels read (d_ptr[n+1] | term[P], same encoding as Pattern::flat) by a
// counting sort: count per destination, prefix sum, then place the terms in
// parameter order (K, Gamma, Lambda, Psi, F), which keeps every list in
// canonical order.  One thread, O(n + P); cur[n] follows the term list.
// Also clears the status block (the first kernel of a call to touch it).
__global__ void build_term_lists(int* d, int n, int kn, int gn, int ln, int pn, int fn, NoallocStatus* status,
                                 int n_sys) {
    status->bad = 0;
    status->first_bad = n_sys;
    const int* kp = d;
    const int* gi = d + (n + 1) + kn;
    const int* li = gi + 3 * gn;
    const int* pi = li + 4 * ln;
    const int* fi = pi + 5 * pn;
    int* dp = d + (n + 1) + kn + 3 * gn + 4 * ln + 5 * pn + fn;
    int* tl = dp + n + 1;
    int* cur = tl + kn + gn + ln + pn + fn;
    for (int i = 0; i <= n; ++i) dp[i] = 0;
    for (int i = 0; i < n; ++i) dp[i + 1] += kp[i + 1] - kp[i];
    for (int e = 0; e < gn; ++e) dp[gi[3 * e] + 1]++;
    for (int e = 0; e < ln; ++e) dp[li[4 * e] + 1]++;
    for (int e = 0; e < pn; ++e) dp[pi[5 * e] + 1]++;
    for (int e = 0; e < fn; ++e) dp[fi[e] + 1]++;
    for (int i = 0; i < n; ++i) dp[i + 1] += dp[i];
    for (int i = 0; i < n; ++i) cur[i] = dp[i];
    for (int i = 0; i < n; ++i)
        for (int q = kp[i]; q < kp[i + 1]; ++q) tl[cur[i]++] = q;
    int base = kn;
    for (int e = 0; e < gn; ++e) tl[cur[gi[3 * e]]++] = (1 << 28) | (base + e);
    base += gn;
    for (int e = 0; e < ln; ++e) tl[cur[li[4 * e]]++] = (2 << 28) | (base + e);
    base += ln;
    for (int e = 0; e < pn; ++e) tl[cur[pi[5 * e]]++] = (3 << 28) | (base + e);
    base += pn;
    for (int e = 0; e < fn; ++e) tl[cur[fi[e]]++] = (4 << 28) | (base + e);
}

// Checked copy of the caller's excitation indices: an index outside
// [0, n_exc) is counted in the status block and replaced by 0, so that the
// forward kernel never reads outside the signal table.
__global__ void check_exc(const int* exc, int n_sys, int n_exc, int* out, NoallocStatus* status) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_sys) return;
    const int e = exc[b];
    const bool ok = e >= 0 && e < n_exc;
    out[b] = ok ? e : 0;
    if (!ok) {
        atomicAdd(&status->bad, 1);
        atomicMin(&status->first_bad, b);
    }
}

// The final state of a system with an out-of-range excitation index is NaN.
__global__ void poison_bad(const int* exc, int n_sys, int n_exc, int n, double* state_out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_sys) return;
    const int e = exc[b];
    if (e >= 0 && e < n_exc) return;
    for (int i = 0; i < n; ++i) state_out[(long long)b * n + i] = __longlong_as_double(0x7ff8000000000000LL);
}

// Queues the pattern integers of `src` (count of them) at dst + off through
// put_ints launches, batching consecutive parts into one chunk.
struct IntUploader {
    int* dst;
    cudaStream_t st;
    IntChunk chunk;
    int fill = 0;
    long long base = 0;   // destination offset of chunk.v[0]
    cudaError_t err = cudaSuccess;

    void add(const int* src, long long count) {
        for (long long i = 0; i < count && err == cudaSuccess; ++i) {
            chunk.v[fill++] = src[i];
            if (fill == kChunkInts) flush();
        }
    }
    void flush() {
        if (fill == 0 || err != cudaSuccess) return;
        put_ints<<<1, 256, 0, st>>>(dst + base, chunk, fill);
        err = cudaGetLastError();
        base += fill;
        fill = 0;
    }
};

}  // namespace

extern "C" int pasif_forward_noalloc(const pasif_pattern* pat, int n_sys, const double* values, const double* x0,
                                     const int* exc_index, const double* signals, int n_exc, int len, int window,
                                     const double* im, double h, int step0, int nsteps, double* state_out,
                                     void* stream) {
    if (!pat || pat->n < 0 || pat->k_nnz < 0 || pat->g_nnz < 0 || pat->l_nnz < 0 || pat->p_nnz < 0 ||
        pat->f_nnz < 0)
        return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: bad pattern");
    if (!pat->k_ptr || (pat->k_nnz && !pat->k_col) || (pat->g_nnz && !pat->g_idx) || (pat->l_nnz && !pat->l_idx) ||
        (pat->p_nnz && !pat->p_idx) || (pat->f_nnz && !pat->f_idx))
        return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: null pattern array");
    const int n = pat->n;
    const int n_sp = pat->n_sp > 0 ? pat->n_sp : n;
    const long long P = (long long)pat->k_nnz + pat->g_nnz + pat->l_nnz + pat->p_nnz + pat->f_nnz;
    const long long pat_ints = (n + 1LL) + pat->k_nnz + 3LL * pat->g_nnz + 4LL * pat->l_nnz + 5LL * pat->p_nnz +
                               pat->f_nnz + (n + 1LL) + P + n;   // + term lists and their cursors
    if (n_sys < 0 || nsteps < 0 || step0 < 0) return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: negative size");
    if (n_exc < 1 || len < 1 || !signals) return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: empty signal table");
    if (window < 0 || (window > 0 && (!pow2(window) || !im)))
        return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: window must be 0 or a power of two with weights");
    if (!(h > 0.0) || !std::isfinite(h)) return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: bad time step");
    if ((size_t)pat_ints * sizeof(int) > kPatternBytes - kStatusBytes)
        return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: pattern larger than the 1 MiB pattern area");
    const double need = 8.0 * (double)n_sys * (double)(P + 7LL * n) + 4.0 * (double)n_sys;
    if (need > (double)(kNoallocBytes - kPatternBytes))
        return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: 8*n_sys*(P+7n) + 4*n_sys = " +
                                           std::to_string((long long)need) +
                                           " bytes exceeds the 31 MiB static work space; split the batch");
    if (n_sys == 0) return PASIF_OK;
    if (!x0 || !exc_index || !state_out || (P > 0 && !values))
        return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: null input or output");
    // pattern checks (host arrays), as the allocating entry points make them
    for (int i = 0; i < n; ++i)
        if (pat->k_ptr[i + 1] < pat->k_ptr[i]) return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: bad CSR");
    if (pat->k_ptr[0] != 0 || pat->k_ptr[n] != pat->k_nnz) return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: bad CSR");
    for (int q = 0; q < pat->k_nnz; ++q)
        if (pat->k_col[q] < 0 || pat->k_col[q] >= n) return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: bad index");
    // tensor entries: destination and source in [0, n), setpoint indices in [0, n_sp)
    const int* lists[3] = {pat->g_idx, pat->l_idx, pat->p_idx};
    const int widths[3] = {3, 4, 5};
    const int counts[3] = {pat->g_nnz, pat->l_nnz, pat->p_nnz};
    for (int l = 0; l < 3; ++l)
        for (long long e = 0; e < counts[l]; ++e)
            for (int k = 0; k < widths[l]; ++k) {
                const int v = lists[l][e * widths[l] + k];
                if (v < 0 || v >= (k < 2 ? n : n_sp)) return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: bad index");
            }
    for (int q = 0; q < pat->f_nnz; ++q)
        if (pat->f_idx[q] < 0 || pat->f_idx[q] >= n) return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc: bad index");
    cudaStream_t st = (cudaStream_t)stream;
    void* base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) return fail(PASIF_ERR_CUDA, std::string("pasif_forward_noalloc: symbol address: ") + cudaGetErrorString(e));
    NoallocStatus* d_status = static_cast<NoallocStatus*>(base);
    int* d_pat = reinterpret_cast<int*>(static_cast<unsigned char*>(base) + kStatusBytes);
    double* d_vals = reinterpret_cast<double*>(static_cast<unsigned char*>(base) + kPatternBytes);
    double* d_state = d_vals + (size_t)P * n_sys;
    double* d_work = d_state + (size_t)n * n_sys;
    int* d_exc = reinterpret_cast<int*>(d_work + (size_t)6 * n * n_sys);
    // pattern: k_ptr | k_col | g | l | p | f (the generic kernels' layout), as kernel arguments
    IntUploader up;
    up.dst = d_pat;
    up.st = st;
    up.add(pat->k_ptr, n + 1LL);
    up.add(pat->k_col, pat->k_nnz);
    up.add(pat->g_idx, 3LL * pat->g_nnz);
    up.add(pat->l_idx, 4LL * pat->l_nnz);
    up.add(pat->p_idx, 5LL * pat->p_nnz);
    up.add(pat->f_idx, pat->f_nnz);
    up.flush();
    e = up.err;
    // per-destination term lists (d_ptr | terms) built on the device; status cleared
    if (e == cudaSuccess) {
        build_term_lists<<<1, 1, 0, st>>>(d_pat, n, pat->k_nnz, pat->g_nnz, pat->l_nnz, pat->p_nnz, pat->f_nnz,
                                          d_status, n_sys);
        e = cudaGetLastError();
    }
    const int grid = (n_sys + 255) / 256;
    if (e == cudaSuccess) {
        check_exc<<<grid, 256, 0, st>>>(exc_index, n_sys, n_exc, d_exc, d_status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = pk::launch_to_interleaved(values, d_vals, n_sys, (int)P, false, st);
    if (e == cudaSuccess) e = pk::launch_to_interleaved(x0, d_state, n_sys, n, false, st);
    if (e != cudaSuccess) return fail(PASIF_ERR_CUDA, std::string("pasif_forward_noalloc: ") + cudaGetErrorString(e));
    pk::FwdArgs<double> a;
    memset(&a, 0, sizeof(a));
    a.vals = d_vals;
    a.state = d_state;
    a.exc_index = d_exc;
    a.scratch = d_work;
    a.traj_every = 1;
    a.frc.x = signals;
    a.frc.im = window ? im : nullptr;
    a.frc.total = (long long)n_exc * len;
    a.frc.len = (unsigned)len;
    a.frc.w = (unsigned)window;
    a.frc.lw = 0;
    while (window > 0 && (1u << a.frc.lw) < (unsigned)window) a.frc.lw++;
    a.gp.data = d_pat;
    a.gp.n = n;
    a.gp.n_sp = n_sp;
    a.gp.k_nnz = pat->k_nnz;
    a.gp.g_nnz = pat->g_nnz;
    a.gp.l_nnz = pat->l_nnz;
    a.gp.p_nnz = pat->p_nnz;
    a.gp.f_nnz = pat->f_nnz;
    a.gp.P = (int)P;
    a.h = h;
    a.h2 = h / 2.0;
    a.h6 = h / 6.0;
    a.B = n_sys;
    a.step0 = (unsigned)step0;
    a.nsteps = nsteps;
    e = pk::launch_gen_fwd(a, false, st);
    if (e == cudaSuccess) e = pk::launch_from_interleaved(d_state, state_out, n_sys, n, false, st, 1.0);
    if (e == cudaSuccess) {
        poison_bad<<<grid, 256, 0, st>>>(exc_index, n_sys, n_exc, n, state_out);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return fail(PASIF_ERR_CUDA, std::string("pasif_forward_noalloc: ") + cudaGetErrorString(e));
    return PASIF_OK;
}

extern "C" int pasif_forward_noalloc_status(int* n_bad, int* first_bad, void* stream) {
    if (!n_bad) return fail(PASIF_ERR_INVALID, "pasif_forward_noalloc_status: null output");
    void* base = nullptr;
    cudaError_t e = scratch_address(&base);
    NoallocStatus s = {0, 0};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&s, base, sizeof(s), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess)
        return fail(PASIF_ERR_CUDA, std::string("pasif_forward_noalloc_status: ") + cudaGetErrorString(e));
    *n_bad = s.bad;
    if (first_bad) *first_bad = s.first_bad;
    return PASIF_OK;
}
