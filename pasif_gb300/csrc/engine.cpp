// engine.cpp -- host side of the batched RK4 engine (plans, signal tables,
// device-resident batches, kernel selection and launch).
#include "engine.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "generic_kernels.h"

namespace pasif {

std::string cuda_err(const char* what, cudaError_t e) {
    return std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
}

#define PK_CUDA(call, what)                          \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) {                     \
            *err = cuda_err(what, e_);               \
            return e_ == cudaErrorMemoryAllocation ? 4 : 2; \
        }                                            \
    } while (0)

DevBuf::~DevBuf() { release(); }

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

cudaError_t DevBuf::ensure(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    else p = nullptr;
    return e;
}

static bool is_pow2(unsigned w) { return w && !(w & (w - 1)); }

static cudaMemcpyKind kind_in(int memory) { return memory == kDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice; }

// Copy a double array (host or device) into a device buffer converted to the
// compute precision.
static int upload_conv(const double* src, long long n, bool f32, int memory, DevBuf& dst, DevBuf& stage,
                       cudaStream_t st, std::string* err) {
    const size_t rs = f32 ? sizeof(float) : sizeof(double);
    PK_CUDA(dst.ensure((size_t)(n > 0 ? n : 1) * rs), "cudaMalloc");
    if (n == 0) return 0;
    if (!f32) {
        PK_CUDA(cudaMemcpyAsync(dst.p, src, (size_t)n * sizeof(double), kind_in(memory), st), "cudaMemcpyAsync");
        return 0;
    }
    const double* dsrc = src;
    if (memory == kHost) {
        PK_CUDA(stage.ensure((size_t)n * sizeof(double)), "cudaMalloc");
        PK_CUDA(cudaMemcpyAsync(stage.p, src, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st),
                "cudaMemcpyAsync");
        dsrc = stage.as<double>();
    }
    PK_CUDA(pk::launch_convert(dsrc, dst.p, n, true, st), "convert kernel");
    return 0;
}

// [B][k] double (host or device) -> [k][B] compute precision.
static int upload_interleaved(const double* src, int B, int k, bool f32, int memory, DevBuf& dst,
                              DevBuf& stage, cudaStream_t st, std::string* err) {
    const size_t rs = f32 ? sizeof(float) : sizeof(double);
    const long long total = (long long)B * k;
    PK_CUDA(dst.ensure((size_t)(total > 0 ? total : 1) * rs), "cudaMalloc");
    if (total == 0) return 0;
    const double* dsrc = src;
    if (memory == kHost) {
        PK_CUDA(stage.ensure((size_t)total * sizeof(double)), "cudaMalloc");
        PK_CUDA(cudaMemcpyAsync(stage.p, src, (size_t)total * sizeof(double), cudaMemcpyHostToDevice, st),
                "cudaMemcpyAsync");
        dsrc = stage.as<double>();
    }
    PK_CUDA(pk::launch_to_interleaved(dsrc, dst.p, B, k, f32, st), "layout kernel");
    return 0;
}

// [B][k] double (host or device) -> [2k][B] FP32: the high parts (v rounded
// to FP32) of the k values, then their low parts (v minus its high part,
// rounded to FP32); the extended-state mode's layout of values and x0.
static int upload_split(const double* src, int B, int k, int memory, DevBuf& dst, DevBuf& split, DevBuf& stage,
                        cudaStream_t st, std::string* err) {
    const long long total = (long long)B * k;
    PK_CUDA(dst.ensure((size_t)(total > 0 ? 2 * total : 1) * sizeof(float)), "cudaMalloc");
    if (total == 0) return 0;
    const double* dsrc = src;
    if (memory == kHost) {
        PK_CUDA(stage.ensure((size_t)total * sizeof(double)), "cudaMalloc");
        PK_CUDA(cudaMemcpyAsync(stage.p, src, (size_t)total * sizeof(double), cudaMemcpyHostToDevice, st),
                "cudaMemcpyAsync");
        dsrc = stage.as<double>();
    }
    PK_CUDA(split.ensure((size_t)total * 2 * sizeof(double)), "cudaMalloc");
    PK_CUDA(pk::launch_split_hi_lo(dsrc, split.as<double>(), B, k, st), "split kernel");
    PK_CUDA(pk::launch_to_interleaved(split.as<double>(), dst.p, B, 2 * k, true, st), "layout kernel");
    return 0;
}

// [k][B] FP32 high and low parts -> [B][k] double hi + lo (host or device).
static int download_pair(const void* hi, const void* lo, int B, int k, double scale, double* out, int memory,
                         DevBuf& stage, cudaStream_t st, std::string* err) {
    const long long total = (long long)B * k;
    if (total == 0 || !out) return 0;
    double* ddst = out;
    if (memory == kHost) {
        PK_CUDA(stage.ensure((size_t)total * sizeof(double)), "cudaMalloc");
        ddst = stage.as<double>();
    }
    PK_CUDA(pk::launch_from_interleaved_pair(static_cast<const float*>(hi), static_cast<const float*>(lo), ddst, B, k,
                                             scale, st),
            "layout kernel");
    if (memory == kHost) {
        PK_CUDA(cudaMemcpyAsync(out, ddst, (size_t)total * sizeof(double), cudaMemcpyDeviceToHost, st),
                "cudaMemcpyAsync");
        PK_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    }
    return 0;
}

// [k][B] (compute precision or double) -> [B][k] double (host or device).
static int download_interleaved(const void* src, int B, int k, bool f32, double scale, double* out, int memory,
                                DevBuf& stage, cudaStream_t st, std::string* err) {
    const long long total = (long long)B * k;
    if (total == 0 || !out) return 0;
    double* ddst = out;
    if (memory == kHost) {
        PK_CUDA(stage.ensure((size_t)total * sizeof(double)), "cudaMalloc");
        ddst = stage.as<double>();
    }
    PK_CUDA(pk::launch_from_interleaved(src, ddst, B, k, f32, st, scale), "layout kernel");
    if (memory == kHost) {
        PK_CUDA(cudaMemcpyAsync(out, ddst, (size_t)total * sizeof(double), cudaMemcpyDeviceToHost, st),
                "cudaMemcpyAsync");
        PK_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    }
    return 0;
}

int signals_create(const double* x, int n_exc, int len, int window, const double* im, int precision,
                   int memory, cudaStream_t st, std::shared_ptr<Signals>* out, std::string* err) {
    if (n_exc < 1 || len < 1 || !x) { *err = "excitation table must hold at least one sample of one signal"; return 1; }
    if (window < 0 || (window > 0 && !is_pow2((unsigned)window))) {
        *err = "interpolation window size must be a power of two (src/kernels.cu:115-117 masks with W-1)";
        return 1;
    }
    if (window > 0 && !im) { *err = "interpolation matrix missing"; return 1; }
    auto s = std::make_shared<Signals>();
    s->f32 = precision != kFP64;
    s->n_exc = n_exc;
    s->len = len;
    s->w = (unsigned)window;
    s->lw = 0;
    while (window > 0 && (1u << s->lw) < s->w) s->lw++;
    DevBuf stage;
    int rc = upload_conv(x, (long long)n_exc * len, s->f32, memory, s->x, stage, st, err);
    if (rc) return rc;
    if (window > 0) {
        rc = upload_conv(im, 2LL * window, s->f32, memory, s->im, stage, st, err);
        if (rc) return rc;
        // host copy of the weights (baked into specialised kernels)
        std::vector<double> w(2 * (size_t)window);
        if (memory == kHost) std::memcpy(w.data(), im, sizeof(double) * w.size());
        else PK_CUDA(cudaMemcpy(w.data(), im, sizeof(double) * w.size(), cudaMemcpyDeviceToHost), "cudaMemcpy");
        for (double& v : w) v = s->f32 ? (double)(float)v : v;
        s->im_host = w;
    }
    PK_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    *out = s;
    return 0;
}

int signals_update(Signals& s, const double* x, int n_exc, int len, int memory, cudaStream_t st, std::string* err) {
    if (n_exc < 1 || len < 1 || !x) { *err = "excitation table must hold at least one sample of one signal"; return 1; }
    int rc = upload_conv(x, (long long)n_exc * len, s.f32, memory, s.x, s.stage, st, err);
    if (rc) return rc;
    s.n_exc = n_exc;
    s.len = len;
    PK_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    return 0;
}

int Batch::reserve(int n_sys, int nsteps, std::string* err) {
    if (n_sys < 0 || nsteps < 0) { *err = "negative reservation"; return 1; }
    const Pattern& pat = plan->pat;
    const size_t n = (size_t)pat.n, P = (size_t)(pat.P() > 0 ? pat.P() : 1), rs = rsize();
    const size_t Bn = (size_t)(n_sys > 0 ? n_sys : 1), wide = std::max(P, n);
    const size_t C = nsteps > 0 ? (size_t)std::ceil(std::sqrt((double)nsteps)) : 1;
    const size_t nck = nsteps > 0 ? ((size_t)nsteps + C - 1) / C : 1;
    const size_t np = parts();   // kFP32Ext: high and low parts
    PK_CUDA(vals.ensure(Bn * P * np * rs), "cudaMalloc");
    PK_CUDA(x0.ensure(Bn * n * np * rs), "cudaMalloc");
    PK_CUDA(stage.ensure(Bn * wide * sizeof(double)), "cudaMalloc");
    if (ext()) PK_CUDA(split.ensure(Bn * wide * 2 * sizeof(double)), "cudaMalloc");
    PK_CUDA(exc.ensure(Bn * sizeof(int)), "cudaMalloc");
    PK_CUDA(state.ensure(Bn * n * np * rs), "cudaMalloc");
    PK_CUDA(out_max.ensure(Bn * n * rs), "cudaMalloc");
    PK_CUDA(out_sq.ensure(Bn * rs), "cudaMalloc");
    PK_CUDA(ckpt.ensure(Bn * 2 * n * nck * rs), "cudaMalloc");
    // the recomputed chunk, or the largest stored trajectory a request up to
    // this size may use (within adj_store_limit)
    const size_t chunk_bytes = Bn * n * (slot_vecs() * C + 1) * rs;
    PK_CUDA(adj_state.ensure(Bn * n * rs), "cudaMalloc");
    const size_t full_bytes = Bn * n * (slot_vecs() * (size_t)nsteps + 1) * rs;
    PK_CUDA(buf.ensure(std::max(chunk_bytes, nsteps > 0 ? std::min(full_bytes, adj_store_limit) : 0)), "cudaMalloc");
    PK_CUDA(pbar.ensure(Bn * P * sizeof(double)), "cudaMalloc");
    if (f32()) PK_CUDA(pkbuf.ensure(Bn * 2 * P * sizeof(float)), "cudaMalloc");
    PK_CUDA(dx0.ensure(Bn * n * rs), "cudaMalloc");
    PK_CUDA(gfin.ensure(Bn * n * rs), "cudaMalloc");
    PK_CUDA(gsq.ensure(Bn * rs), "cudaMalloc");
    PK_CUDA(lamc.ensure(Bn * n * rs), "cudaMalloc");
    PK_CUDA(adj_stage.ensure(Bn * wide * sizeof(double)), "cudaMalloc");
    inputs_set = false;   // grown buffers are fresh allocations
    return 0;
}

Batch::~Batch() {
    for (int i = 0; i < kReplayBufs; ++i) {
        if (replay_st[i]) cudaStreamDestroy(replay_st[i]);
        if (ev_replayed[i]) cudaEventDestroy(ev_replayed[i]);
        if (ev_free[i]) cudaEventDestroy(ev_free[i]);
    }
    if (ev_ckpt) cudaEventDestroy(ev_ckpt);
}

int Batch::resize(int n_sys, std::string* err) {
    if (n_sys < 0) { *err = "negative number of systems"; return 1; }
    B = n_sys;
    max_exc_ = -1;
    last_kind = last_adj_kind = kNone;
    inputs_set = false;
    return 0;
}

pk::GenPattern Plan::gen() const {
    pk::GenPattern g;
    g.data = gpat.as<int>();
    g.n = pat.n;
    g.n_sp = pat.n_sp;
    g.k_nnz = pat.k_nnz();
    g.g_nnz = pat.g_nnz();
    g.l_nnz = pat.l_nnz();
    g.p_nnz = pat.p_nnz();
    g.f_nnz = pat.f_nnz();
    g.P = pat.P();
    return g;
}

int plan_create(const Pattern& pat, int precision, bool generic_only, std::shared_ptr<Plan>* out,
                std::string* err) {
    std::string v = pat.validate();
    if (!v.empty()) { *err = v; return 1; }
    if (precision < kFP64 || precision > kFP32Ext) { *err = "unknown precision"; return 1; }
    if (precision == kFP32Ext && generic_only) {
        *err = "the extended-state precision runs on the pattern-specialised kernels only";
        return 1;
    }
    auto p = std::make_shared<Plan>();
    p->pat = pat;
    p->precision = precision;
    p->generic_only = generic_only;
    *out = p;
    return 0;
}

Literals literals_of(const Pattern& pat, int precision, const double* values, int n_sys) {
    const int P = pat.P();
    Literals lit;
    lit.is_lit.assign(P, 0);
    lit.value.assign(P, 0.0);
    lit.is_lit_lo.assign(P, 0);
    lit.value_lo.assign(P, 0.0);
    if (precision < 0 || !values || n_sys <= 0) return lit;
    const bool f = precision != kFP64;
    auto hi_of = [&](double v) { return f ? (double)(float)v : v; };
    auto lo_of = [](double v) { return (double)(float)(v - (double)(float)v); };   // kFP32Ext low part
    auto same_bits = [](double a, double b) { return std::memcmp(&a, &b, sizeof(double)) == 0; };
    for (int q = 0; q < P; ++q) {
        const double v0 = hi_of(values[q]);
        bool same = true;
        for (int b = 1; b < n_sys && same; ++b) same = same_bits(hi_of(values[(long long)b * P + q]), v0);
        lit.value[q] = v0;
        lit.is_lit[q] = same && std::isfinite(v0) ? 1 : 0;
        if (precision == kFP32Ext) {
            const double l0 = lo_of(values[q]);
            bool same_lo = true;
            for (int b = 1; b < n_sys && same_lo; ++b) same_lo = same_bits(lo_of(values[(long long)b * P + q]), l0);
            lit.value_lo[q] = l0;
            lit.is_lit_lo[q] = same_lo && std::isfinite(l0) ? 1 : 0;
        }
    }
    return lit;
}

int Plan::ensure_device(std::string* err) {
    if (gpat.p) return 0;
    std::vector<int> flat = pat.flat();
    PK_CUDA(gpat.ensure(flat.size() * sizeof(int)), "cudaMalloc");
    PK_CUDA(cudaMemcpy(gpat.p, flat.data(), flat.size() * sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy");
    return 0;
}

int batch_create(std::shared_ptr<Plan> plan, int B, std::unique_ptr<Batch>* out, std::string* err) {
    if (!plan) { *err = "null plan"; return 1; }
    if (B < 0) { *err = "negative number of systems"; return 1; }
    std::unique_ptr<Batch> b(new Batch());
    b->plan = plan;
    b->B = B;
    *out = std::move(b);
    return 0;
}

int Batch::set(const double* values, const double* x0h, const int* exc_index, int memory, cudaStream_t st,
               std::string* err) {
    const Pattern& pat = plan->pat;
    const int P = pat.P(), n = pat.n;
    const bool f = f32();
    if (B > 0 && ((P > 0 && !values) || !x0h || !exc_index)) { *err = "null input array"; return 1; }
    if (int rc0 = plan->ensure_device(err)) return rc0;
    int rc = ext() ? upload_split(values, B, P, memory, vals, split, stage, st, err)
                   : upload_interleaved(values, B, P, f, memory, vals, stage, st, err);
    if (rc) return rc;
    rc = ext() ? upload_split(x0h, B, n, memory, x0, split, stage, st, err)
               : upload_interleaved(x0h, B, n, f, memory, x0, stage, st, err);
    if (rc) return rc;
    PK_CUDA(exc.ensure((size_t)(B > 0 ? B : 1) * sizeof(int)), "cudaMalloc");
    std::vector<int> idx(B);
    if (B > 0) {
        if (memory == kHost) std::memcpy(idx.data(), exc_index, sizeof(int) * B);
        else PK_CUDA(cudaMemcpy(idx.data(), exc_index, sizeof(int) * B, cudaMemcpyDeviceToHost), "cudaMemcpy");
        PK_CUDA(cudaMemcpyAsync(exc.p, idx.data(), sizeof(int) * B, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
    }
    max_exc_ = -1;
    for (int i = 0; i < B; ++i) {
        if (idx[i] < 0) { *err = "negative excitation index"; return 1; }
        if (idx[i] > max_exc_) max_exc_ = idx[i];
    }
    // values shared by every instance become compile-time constants
    lit = literals_of(pat, memory == kHost && !plan->no_literals ? plan->precision : -1, values, B);
    PK_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    inputs_set = true;
    return 0;
}

static int check_comps(const std::vector<int>& c, int n, const char* what, unsigned long long* mask, std::string* err) {
    *mask = 0;
    int prev = -1;
    for (int v : c) {
        if (v < 0 || v >= n || v >= 64 || v <= prev) {
            *err = std::string(what) + " components must be ascending, unique, < n and < 64";
            return 1;
        }
        *mask |= 1ull << v;
        prev = v;
    }
    return 0;
}

template <typename R>
static void fill_fwd(pk::FwdArgs<R>& a, Batch& bt, const Signals& sig, double h, int step0, int nsteps,
                     const Reducers& red, unsigned long long mm, unsigned long long sm, int traj_every,
                     long long traj_slots) {
    std::memset(&a, 0, sizeof(a));
    a.vals = bt.vals.as<R>();
    a.state = bt.state.as<R>();
    a.exc_index = bt.exc.as<int>();
    a.scratch = bt.scratch.as<R>();
    a.out_max = bt.out_max.as<R>();
    a.out_sq = bt.out_sq.as<R>();
    a.traj = traj_every > 0 ? bt.traj.as<R>() : nullptr;
    a.traj_slots = traj_slots;
    a.traj_every = traj_every > 0 ? traj_every : 1;
    a.frc = sig.forcing<R>();
    a.gp = bt.plan->gen();
    a.h = (R)h;
    a.h2 = (R)(h / 2.0);
    a.h6 = (R)(h / 6.0);
    a.h6lo = (R)(h / 6.0 - (double)(R)(h / 6.0));
    a.B = bt.B;
    a.step0 = (unsigned)step0;
    a.nsteps = nsteps;
    a.max_start = red.max_start;
    a.sq_start = red.sq_start;
    a.max_mask = mm;
    a.sq_mask = sm;
}

// Threads per block of a thread-per-system forward: 128, halved down to 32
// while the batch would fill fewer blocks than the device has SMs, so that a
// small batch spreads its warps over more SMs (GB300: +8 % FP32, +13 % FP64 on
// 1024 one-DOF systems; +15 % FP64 on 4096 16-state chains).
static int tps_block(int B) {
    if (const char* e = std::getenv("PASIF_TPS_BLOCK")) {   // tuning override: 32, 64, 96 or 128
        const int v = std::atoi(e);
        if (v >= 32 && v <= 128 && v % 32 == 0) return v;
    }
    static const int sms = [] {
        int d = 0, s = 0;
        if (cudaGetDevice(&d) != cudaSuccess || cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, d) != cudaSuccess)
            return 0;
        return s;
    }();
    int block = 128;
    while (block > 32 && (B + block - 1) / block < sms) block /= 2;
    return block;
}

bool Batch::fwd_kernel(const Signals& sig, unsigned long long mm, unsigned long long sm, int traj_mode,
                       JitKernel* k, std::string* jerr) {
    const Pattern& pat = plan->pat;
    if (plan->generic_only || pat.n > kWsMaxN) {
        *jerr = "no specialised forward kernel for this plan";
        return false;
    }
    const bool f = f32();
    FwdKernelKey key;
    key.f32 = f;
    key.kahan = compensated();
    key.ext = ext();
    key.max_mask = mm;
    key.sq_mask = sm;
    key.traj = traj_mode;
    key.block = tps_block(B);
    key.window = (int)sig.w;
    key.wn.assign(sig.im_host.begin(), sig.im_host.begin() + sig.w);
    key.wc.assign(sig.im_host.begin() + sig.w, sig.im_host.end());
    key.slices = plan->slicing < 0 ? 0 : ws_slices(pat, f, plan->slicing > 0, B, ext());
    key.fast = plan->fast && traj_mode == 0 && !ext() && key.slices < 2;
    return get_fwd_kernel(pat, lit, key, k, jerr);
}

cudaError_t Batch::launch_fwd_jit(const JitKernel& k, const Signals& sig, double h, int step0, int nsteps,
                                  const Reducers& red, unsigned long long mm, unsigned long long sm, int traj_every,
                                  long long traj_slots, void* state_p, void* traj_p, cudaStream_t st,
                                  const void* comp_p, void* comp_out_p) {
    const dim3 grid((unsigned)((B + k.per_block - 1) / k.per_block));
    if (f32()) {
        pk::FwdArgs<float> a;
        fill_fwd(a, *this, sig, h, step0, nsteps, red, mm, sm, traj_every, traj_slots);
        a.state = static_cast<float*>(state_p);
        a.traj = static_cast<float*>(traj_p);
        a.comp = static_cast<const float*>(comp_p);
        a.comp_out = static_cast<float*>(comp_out_p);
        void* args[] = {&a};
        return cudaLaunchKernel((const void*)k.fn, grid, dim3(k.block), args, (size_t)k.smem, st);
    }
    pk::FwdArgs<double> a;
    fill_fwd(a, *this, sig, h, step0, nsteps, red, mm, sm, traj_every, traj_slots);
    a.state = static_cast<double*>(state_p);
    a.traj = static_cast<double*>(traj_p);
    a.comp = static_cast<const double*>(comp_p);
    a.comp_out = static_cast<double*>(comp_out_p);
    void* args[] = {&a};
    return cudaLaunchKernel((const void*)k.fn, grid, dim3(k.block), args, (size_t)k.smem, st);
}

int Batch::forward(const Signals& sig, double h, int step0, int nsteps, const Reducers& red, int traj_every,
                   long long traj_slots, cudaStream_t st, std::string* err) {
    const Pattern& pat = plan->pat;
    const int n = pat.n;
    const bool f = f32();
    if (sig.f32 != f) { *err = "signal table precision differs from the plan's"; return 1; }
    if (step0 < 0 || nsteps < 0) { *err = "negative step index or step count"; return 1; }
    if (B > 0 && !inputs_set) { *err = "batch inputs not set (set them after creating, resizing or reserving)"; return 5; }
    if (max_exc_ >= sig.n_exc) { *err = "excitation index beyond the signal table"; return 1; }
    if (!(h > 0.0) || !std::isfinite(h)) { *err = "time step must be positive and finite"; return 1; }
    unsigned long long mm = 0, sm = 0;
    if (check_comps(red.max_comp, n, "max reducer", &mm, err)) return 1;
    if (check_comps(red.sq_comp, n, "sum-of-squares reducer", &sm, err)) return 1;
    n_max = (int)red.max_comp.size();
    has_sq = !red.sq_comp.empty();
    last_h = h;
    const size_t rs = rsize();
    const size_t Bn = (size_t)(B > 0 ? B : 1);
    PK_CUDA(state.ensure(Bn * (size_t)n * parts() * rs), "cudaMalloc");   // kFP32Ext: high, then low parts
    PK_CUDA(out_max.ensure(Bn * (size_t)(n_max > 0 ? n_max : 1) * rs), "cudaMalloc");
    PK_CUDA(out_sq.ensure(Bn * rs), "cudaMalloc");
    if (traj_every > 0) PK_CUDA(traj.ensure(Bn * (size_t)n * (size_t)(traj_slots > 0 ? traj_slots : 1) * rs), "cudaMalloc");
    if (B == 0) { last_kind = kNone; return 0; }
    PK_CUDA(cudaMemcpyAsync(state.p, x0.p, (size_t)B * n * parts() * rs, cudaMemcpyDeviceToDevice, st),
            "cudaMemcpyAsync");
    const bool kahan = plan->precision == kFP32Kahan;
    JitKernel k;
    std::string jerr;
    if (fwd_kernel(sig, mm, sm, traj_every > 0 ? 1 : 0, &k, &jerr)) {
        // kFP32Ext: the low parts of the state follow the high parts in `state`, read and written in place
        char* lo = ext() ? state.as<char>() + (size_t)B * n * rs : nullptr;
        PK_CUDA(launch_fwd_jit(k, sig, h, step0, nsteps, red, mm, sm, traj_every, traj_slots, state.p,
                               traj_every > 0 ? traj.p : nullptr, st, lo, lo),
                "specialised forward kernel launch");
        last_kind = kSpecialised;
        last_jit = k;
        return 0;
    }
    if (!plan->generic_only) last_jit_error = jerr;
    if (ext()) {
        *err = "the extended-state precision needs the pattern-specialised kernel: " + jerr;
        return 3;
    }
    PK_CUDA(scratch.ensure(Bn * 6 * (size_t)n * rs), "cudaMalloc");
    cudaError_t e;
    if (f) {
        pk::FwdArgs<float> a;
        fill_fwd(a, *this, sig, h, step0, nsteps, red, mm, sm, traj_every, traj_slots);
        e = pk::launch_gen_fwd(a, kahan, st);
    } else {
        pk::FwdArgs<double> a;
        fill_fwd(a, *this, sig, h, step0, nsteps, red, mm, sm, traj_every, traj_slots);
        e = pk::launch_gen_fwd(a, kahan, st);
    }
    PK_CUDA(e, "generic forward kernel launch");
    last_kind = kGeneric;
    return 0;
}

int Batch::get(double* state_out, double* max_out, double* sq_out, double h, int memory, cudaStream_t st,
               std::string* err) {
    const int n = plan->pat.n;
    const bool f = f32();
    int rc = ext() ? download_pair(state.p, state.as<char>() + (size_t)B * n * rsize(), B, n, 1.0, state_out, memory,
                                   stage, st, err)
                   : download_interleaved(state.p, B, n, f, 1.0, state_out, memory, stage, st, err);
    if (rc) return rc;
    if (max_out && n_max > 0) {
        rc = download_interleaved(out_max.p, B, n_max, f, 1.0, max_out, memory, stage, st, err);
        if (rc) return rc;
    }
    if (sq_out && has_sq) {
        rc = download_interleaved(out_sq.p, B, 1, f, h, sq_out, memory, stage, st, err);
        if (rc) return rc;
    } else if (sq_out && B > 0) {   // no sum-of-squares reducer: defined as 0
        if (memory == kHost) std::memset(sq_out, 0, sizeof(double) * B);
        else PK_CUDA(cudaMemsetAsync(sq_out, 0, sizeof(double) * B, st), "cudaMemsetAsync");
    }
    PK_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    return 0;
}

int Batch::get_traj(double* out, long long slots, int memory, cudaStream_t st, std::string* err) {
    // [slots][n][B] -> [slots][B][n]
    const int n = plan->pat.n;
    const bool f = f32();
    const size_t rs = rsize();
    for (long long s = 0; s < slots; ++s) {
        const char* src = traj.as<char>() + (size_t)s * n * B * rs;
        int rc = download_interleaved(src, B, n, f, 1.0, out + (size_t)s * n * B, memory, stage, st, err);
        if (rc) return rc;
    }
    PK_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    return 0;
}

int Batch::adjoint(const Signals& sig, double h, int nsteps, const Reducers& red, const double* g_final,
                   const double* g_sq, double* d_values, double* d_x0, int memory, cudaStream_t st,
                   std::string* err) {
    const Pattern& pat = plan->pat;
    const int n = pat.n, P = pat.P();
    const bool f = f32();
    if (sig.f32 != f) { *err = "signal table precision differs from the plan's"; return 1; }
    if (nsteps < 0) { *err = "negative step count"; return 1; }
    if (B > 0 && !inputs_set) { *err = "batch inputs not set (set them after creating, resizing or reserving)"; return 5; }
    if (max_exc_ >= sig.n_exc) { *err = "excitation index beyond the signal table"; return 1; }
    if (!(h > 0.0) || !std::isfinite(h)) { *err = "time step must be positive and finite"; return 1; }
    unsigned long long sm = 0;
    if (check_comps(red.sq_comp, n, "sum-of-squares reducer", &sm, err)) return 1;
    if (B == 0) return 0;
    const int C = nsteps > 0 ? (int)std::ceil(std::sqrt((double)nsteps)) : 1;
    const int nck = nsteps > 0 ? (nsteps + C - 1) / C : 0;
    const size_t rs = rsize();
    const size_t Bn = (size_t)B;
    JitKernel jk;
    std::string jerr;
    const int slices = plan->slicing < 0 ? 0 : ws_slices_adjoint(pat, f, plan->slicing > 0, ext());
    const bool jit = !plan->generic_only &&
                     get_adj_kernel(pat, lit, f, compensated(), g_sq ? sm : 0ull, slices, &jk, &jerr, ext());
    if (!jit && !plan->generic_only) last_jit_error = jerr;
    if (!jit && ext()) {
        *err = "the extended-state precision needs the pattern-specialised adjoint kernel: " + jerr;
        return 3;
    }
    // kFP32Ext: the low parts of x0 (start of the forward passes)
    const char* x0lo = ext() ? x0.as<char>() + (size_t)B * n * rs : nullptr;
    // The trajectory the backward sweep reads, in one of three ways (same bits):
    //  stored   (within adj_store_limit): the batch's forward kernel writes
    //           every step's slot once;
    //  replayed (specialised forward kernel available): the forward kernel
    //           writes checkpoints every C steps, then, chunk by chunk in
    //           backward order, the chunk's slots from its checkpoint, each
    //           followed by the adjoint kernel's backward sweep over them;
    //  otherwise the adjoint kernel does the checkpoint pass and the chunk
    //           recomputes itself (in its own warp layout).
    JitKernel fk, ckk;
    std::string ferr;
    const bool stored = jit && adj_stores(B, nsteps) && fwd_kernel(sig, 0ull, 0ull, 2, &fk, &ferr);
    // replay only grids of 32 blocks or more: a small grid runs as one launch
    // (each of its many short replay launches would wait again for SMs that
    // other streams' work holds: 1-DOF adjoints in the served mix took 14 s
    // instead of 1.3 s)
    const long long adj_blocks = jit ? (B + jk.per_block - 1) / jk.per_block : 0;
    const bool replayed = !stored && jit && nsteps > 0 && adj_blocks >= 32 &&
                          fwd_kernel(sig, 0ull, 0ull, 2, &fk, &ferr) && fwd_kernel(sig, 0ull, 0ull, 3, &ckk, &ferr);
    const size_t vec = Bn * (size_t)n * rs;
    // Replayed: up to kReplayBufs chunk buffers, so that the forward replays
    // of the next chunks run on their own streams while the backward sweep
    // works through the current one (the replays are independent: each starts
    // from its checkpoint).  As many as the buffer already holds (a reserved
    // batch), or as fit in 256 MiB.
    const size_t chunk_sz = (slot_vecs() * (size_t)C + 1) * vec;
    int nbuf = 1;
    if (stored) {
        PK_CUDA(buf.ensure((slot_vecs() * (size_t)nsteps + 1) * vec), "cudaMalloc");
    } else {
        PK_CUDA(ckpt.ensure(Bn * 2 * n * (size_t)(nck > 0 ? nck : 1) * rs), "cudaMalloc");
        if (replayed) {
            const size_t cap = std::max(buf.bytes, std::min((size_t)kReplayBufs * chunk_sz, (size_t)256 << 20));
            nbuf = (int)std::max<size_t>(1, std::min<size_t>({(size_t)kReplayBufs, cap / chunk_sz, (size_t)nck}));
        }
        PK_CUDA(buf.ensure((size_t)nbuf * chunk_sz), "cudaMalloc");
    }
    if (nbuf > 1) {   // streams at the priority of st, events (made once per batch)
        int prio = 0;
        PK_CUDA(cudaStreamGetPriority(st, &prio), "cudaStreamGetPriority");
        for (int i = 0; i < nbuf; ++i) {
            if (replay_st[i] && replay_prio != prio) {
                PK_CUDA(cudaStreamDestroy(replay_st[i]), "cudaStreamDestroy");
                replay_st[i] = nullptr;
            }
            if (!replay_st[i])
                PK_CUDA(cudaStreamCreateWithPriority(&replay_st[i], cudaStreamNonBlocking, prio),
                        "cudaStreamCreateWithPriority");
            if (!ev_replayed[i]) PK_CUDA(cudaEventCreateWithFlags(&ev_replayed[i], cudaEventDisableTiming), "cudaEventCreate");
            if (!ev_free[i]) PK_CUDA(cudaEventCreateWithFlags(&ev_free[i], cudaEventDisableTiming), "cudaEventCreate");
        }
        replay_prio = prio;
        if (!ev_ckpt) PK_CUDA(cudaEventCreateWithFlags(&ev_ckpt, cudaEventDisableTiming), "cudaEventCreate");
    }
    if (replayed) PK_CUDA(adj_state.ensure(vec), "cudaMalloc");
    PK_CUDA(pbar.ensure(Bn * (size_t)(P > 0 ? P : 1) * sizeof(double)), "cudaMalloc");
    if (f) PK_CUDA(pkbuf.ensure(Bn * 2 * (size_t)(P > 0 ? P : 1) * sizeof(float)), "cudaMalloc");
    PK_CUDA(dx0.ensure(Bn * (size_t)n * rs), "cudaMalloc");
    if (g_final) {
        int rc = upload_interleaved(g_final, B, n, f, memory, gfin, adj_stage, st, err);
        if (rc) return rc;
    }
    if (g_sq) {
        int rc = upload_conv(g_sq, B, f, memory, gsq, adj_stage, st, err);
        if (rc) return rc;
    }
    if (stored) {   // the forward kernel's state runs in dx0 (replaced by the adjoint later)
        PK_CUDA(cudaMemcpyAsync(dx0.p, x0.p, vec, cudaMemcpyDeviceToDevice, st), "cudaMemcpyAsync");
        PK_CUDA(launch_fwd_jit(fk, sig, h, 0, nsteps, Reducers(), 0ull, 0ull, 1, nsteps, dx0.p, buf.p, st, x0lo),
                "trajectory forward kernel launch");
    }
    if (replayed) {   // checkpoints of state and compensation every C steps
        PK_CUDA(cudaMemcpyAsync(adj_state.p, x0.p, vec, cudaMemcpyDeviceToDevice, st), "cudaMemcpyAsync");
        PK_CUDA(launch_fwd_jit(ckk, sig, h, 0, nsteps, Reducers(), 0ull, 0ull, C, nck, adj_state.p, ckpt.p, st, x0lo),
                "checkpoint forward kernel launch");
        if (nbuf > 1) PK_CUDA(cudaEventRecord(ev_ckpt, st), "cudaEventRecord");
    }
    cudaError_t e;
#define PK_FILL_ADJ(R_)                                               \
    pk::AdjArgs<R_> a;                                                \
    std::memset(&a, 0, sizeof(a));                                    \
    a.vals = vals.as<R_>();                                           \
    a.x0 = x0.as<R_>();                                               \
    a.exc_index = exc.as<int>();                                      \
    a.ckpt = ckpt.as<R_>();                                           \
    a.buf = buf.as<R_>();                                             \
    a.scratch = scratch.as<R_>();                                     \
    a.pbar = pbar.as<double>();                                       \
    a.dx0 = dx0.as<R_>();                                             \
    a.g_final = g_final ? gfin.as<R_>() : nullptr;                    \
    a.g_sq = g_sq ? gsq.as<R_>() : nullptr;                           \
    a.frc = sig.forcing<R_>();                                        \
    a.gp = plan->gen();                                               \
    a.h = (R_)h;                                                      \
    a.h2 = (R_)(h / 2.0);                                             \
    a.h6 = (R_)(h / 6.0);                                             \
    a.B = B;                                                          \
    a.nsteps = nsteps;                                                \
    a.C = C;                                                          \
    a.nck = nck;                                                      \
    a.kahan = compensated() ? 1 : 0;                                  \
    a.ext = ext() ? 1 : 0;                                            \
    a.h6lo = (R_)(h / 6.0 - (double)(R_)(h / 6.0));                   \
    a.sq_start = red.sq_start;                                        \
    a.sq_mask = g_sq ? sm : 0ull;                                     \
    a.stored = stored || replayed ? 1 : 0;                             \
    a.pk = f ? pkbuf.as<R_>() : nullptr;
    const dim3 grid((unsigned)(jit ? (B + jk.per_block - 1) / jk.per_block : (B + 127) / 128));
    if (jit && compensated()) PK_CUDA(lamc.ensure(Bn * (size_t)n * rs), "cudaMalloc");
    // Specialised kernels over many blocks: forward segments and backward chunk
    // groups of about kAdjLaunchSteps·16/n steps each, so that a launch lasts
    // milliseconds and work on other streams (serving chunks, small adjoints) is
    // not held behind a whole adjoint that fills the SMs.  Small grids (a few
    // SMs) and short horizons run as one launch: split, each of their launches
    // would wait again for SMs held by others.
    auto launch_jit = [&](auto& a) -> cudaError_t {
        void* args[] = {&a};
        a.lamc = lamc.as<typename std::remove_pointer<decltype(a.dx0)>::type>();
        // Replayed: per chunk, backward order, its slots from its checkpoint then
        // its backward sweep; one chunk at a time keeps the slots in L2 between
        // the two (groups of chunks, 2016 steps for 16 states, ran 3 % slower).
        // With several chunk buffers, chunk k's replay runs on its buffer's stream
        // as soon as the checkpoints exist and the backward sweep two or more
        // chunks back has released that buffer; the sweep of chunk k waits for
        // its replay (events).  Same kernels on the same data: the same bits.
        if (replayed) {
            const size_t rsz = sizeof(*a.dx0);
            using RT = typename std::remove_pointer<decltype(a.buf)>::type;
            RT* const buf0 = a.buf;
            for (int k = nck - 1; k >= 0; --k) {
                const int t0 = k * C, t1 = std::min(nsteps, t0 + C);
                const int bi = (nck - 1 - k) % nbuf;
                char* const bp = static_cast<char*>(buf.p) + (size_t)bi * chunk_sz;
                const char* ck = static_cast<const char*>(ckpt.p) + (size_t)k * 2 * n * Bn * rsz;
                cudaStream_t rst = st;
                if (nbuf > 1) {
                    rst = replay_st[bi];
                    cudaError_t le = cudaStreamWaitEvent(rst, ev_ckpt, 0);
                    if (le == cudaSuccess && nck - 1 - k >= nbuf) le = cudaStreamWaitEvent(rst, ev_free[bi], 0);
                    if (le != cudaSuccess) return le;
                }
                // the forward runs on the checkpoint's state in place (no copy: with many
                // adjoints in flight, a copy per chunk queued behind the others' copies);
                // chunk k's checkpoint is not read again
                cudaError_t le = launch_fwd_jit(fk, sig, h, t0, t1 - t0, Reducers(), 0ull, 0ull, 1, t1 - t0,
                                                const_cast<char*>(ck), bp, rst, ck + (size_t)n * Bn * rsz);
                if (le != cudaSuccess) return le;
                if (nbuf > 1) {
                    le = cudaEventRecord(ev_replayed[bi], rst);
                    if (le == cudaSuccess) le = cudaStreamWaitEvent(st, ev_replayed[bi], 0);
                    if (le != cudaSuccess) return le;
                }
                a.phase = 2;
                a.k_hi = a.k_lo = k;
                a.slot_base = t0;
                a.buf = reinterpret_cast<RT*>(bp);
                le = cudaLaunchKernel((const void*)jk.fn, grid, dim3(jk.block), args, (size_t)jk.smem, st);
                if (le != cudaSuccess) return le;
                if (nbuf > 1) {
                    le = cudaEventRecord(ev_free[bi], st);
                    if (le != cudaSuccess) return le;
                }
            }
            a.buf = buf0;
            return cudaSuccess;
        }
        const int per = adj_group(n, C, nck);   // checkpoint intervals per launch
        if (nck <= 2 * per || grid.x < 32) {
            a.phase = 0;
            return cudaLaunchKernel((const void*)jk.fn, grid, dim3(jk.block), args, (size_t)jk.smem, st);
        }
        for (int t0 = 0; t0 < (stored ? 0 : nsteps); t0 += per * C) {   // stored: no forward segments
            a.phase = 1;
            a.t_begin = t0;
            a.t_end = std::min(nsteps, t0 + per * C);
            cudaError_t le = cudaLaunchKernel((const void*)jk.fn, grid, dim3(jk.block), args, (size_t)jk.smem, st);
            if (le != cudaSuccess) return le;
        }
        for (int khi = nck - 1; khi >= 0; khi -= per) {
            a.phase = 2;
            a.k_hi = khi;
            a.k_lo = std::max(0, khi - per + 1);
            cudaError_t le = cudaLaunchKernel((const void*)jk.fn, grid, dim3(jk.block), args, (size_t)jk.smem, st);
            if (le != cudaSuccess) return le;
        }
        return cudaSuccess;
    };
    if (!jit) PK_CUDA(scratch.ensure(Bn * 14 * (size_t)n * rs), "cudaMalloc");   // adj_run_generic's 14 vectors
    if (f) {
        PK_FILL_ADJ(float)
        e = jit ? launch_jit(a) : pk::launch_gen_adj(a, st);
    } else {
        PK_FILL_ADJ(double)
        e = jit ? launch_jit(a) : pk::launch_gen_adj(a, st);
    }
#undef PK_FILL_ADJ
    last_adj_kind = jit ? kSpecialised : kGeneric;
    PK_CUDA(e, "adjoint kernel launch");
    int rc = download_interleaved(pbar.p, B, P, false, 1.0, d_values, memory, adj_stage, st, err);
    if (rc) return rc;
    rc = ext() ? download_pair(dx0.p, lamc.p, B, n, 1.0, d_x0, memory, adj_stage, st, err)   // high + low parts
               : download_interleaved(dx0.p, B, n, f, 1.0, d_x0, memory, adj_stage, st, err);
    if (rc) return rc;
    PK_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    return 0;
}

int refgrad_run(const Plan& fwd, const Plan& bwd, int B, const double* fvals, const double* bvals,
                const double* x0h, const double* a0h, const int* exc_index, const Signals& sig, double h,
                int nsteps, int save, double* out, cudaStream_t st, std::string* err) {
    const int nf = fwd.pat.n, na = bwd.pat.n;
    const bool f = fwd.precision != kFP64;
    if (int rc0 = const_cast<Plan&>(fwd).ensure_device(err)) return rc0;
    if (int rc0 = const_cast<Plan&>(bwd).ensure_device(err)) return rc0;
    if (bwd.pat.n_sp != nf) { *err = "adjoint setpoint size differs from the forward state size"; return 1; }
    if (sig.f32 != f) { *err = "signal table precision differs from the plan's"; return 1; }
    if (B == 0) return 0;
    if (nsteps < 1) { *err = "gradient needs at least one step"; return 1; }
    const int S = (int)std::sqrt((double)nsteps);
    const int C = (int)std::ceil((double)nsteps / (double)S);
    const int lastC = C - (int)(((long long)S * C) % nsteps);
    const long long slots = (long long)S + C - 1;
    DevBuf dfv, dbv, dx0, da0, dexc, dtraj, dscr, dout, stage;
    int rc = upload_interleaved(fvals, B, fwd.pat.P(), f, kHost, dfv, stage, st, err);
    if (rc) return rc;
    rc = upload_interleaved(bvals, B, bwd.pat.P(), f, kHost, dbv, stage, st, err);
    if (rc) return rc;
    rc = upload_interleaved(x0h, B, nf, f, kHost, dx0, stage, st, err);
    if (rc) return rc;
    rc = upload_interleaved(a0h, B, na, f, kHost, da0, stage, st, err);
    if (rc) return rc;
    for (int i = 0; i < B; ++i)
        if (exc_index[i] < 0 || exc_index[i] >= sig.n_exc) { *err = "excitation index out of range"; return 1; }
    const size_t rs = f ? sizeof(float) : sizeof(double);
    PK_CUDA(dexc.ensure(sizeof(int) * B), "cudaMalloc");
    PK_CUDA(cudaMemcpyAsync(dexc.p, exc_index, sizeof(int) * B, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
    PK_CUDA(dtraj.ensure((size_t)slots * nf * B * rs), "cudaMalloc");
    PK_CUDA(cudaMemsetAsync(dtraj.p, 0, (size_t)slots * nf * B * rs, st), "cudaMemsetAsync");
    PK_CUDA(dscr.ensure((size_t)(5 * nf + 6 * na) * B * rs), "cudaMalloc");
    PK_CUDA(dout.ensure((size_t)na * B * rs), "cudaMalloc");
    cudaError_t e;
#define PK_FILL_RG(R_)                          \
    pk::RefGradArgs<R_> a;                      \
    std::memset(&a, 0, sizeof(a));              \
    a.fvals = dfv.as<R_>();                     \
    a.bvals = dbv.as<R_>();                     \
    a.x0 = dx0.as<R_>();                        \
    a.a0 = da0.as<R_>();                        \
    a.exc_index = dexc.as<int>();               \
    a.traj = dtraj.as<R_>();                    \
    a.scratch = dscr.as<R_>();                  \
    a.out = dout.as<R_>();                      \
    a.frc = sig.forcing<R_>();                  \
    a.fgp = fwd.gen();                          \
    a.bgp = bwd.gen();                          \
    a.h = (R_)h;                                \
    a.h2 = (R_)(h / 2.0);                       \
    a.h6 = (R_)(h / 6.0);                       \
    a.B = B;                                    \
    a.nsteps = nsteps;                          \
    a.S = S;                                    \
    a.C = C;                                    \
    a.lastC = lastC;                            \
    a.save = save;                              \
    a.slots = slots;
    if (f) {
        PK_FILL_RG(float)
        e = pk::launch_gen_refgrad(a, st);
    } else {
        PK_FILL_RG(double)
        e = pk::launch_gen_refgrad(a, st);
    }
#undef PK_FILL_RG
    PK_CUDA(e, "gradient kernel launch");
    return download_interleaved(dout.p, B, na, f, 1.0, out, kHost, stage, st, err);
}

}  // namespace pasif
