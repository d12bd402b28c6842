// pool.cpp -- serving pools (continuous batching of forward requests).
#include "pool.h"

#include <algorithm>
#include <cstring>
#include <iterator>

#include "generic_kernels.h"
#include "jit.h"

namespace pasif {

#define PL_CUDA(call, what)                                          \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) {                                     \
            *err = cuda_err(what, e_);                               \
            return e_ == cudaErrorMemoryAllocation ? 4 : 2;          \
        }                                                            \
    } while (0)

// 2W weights rounded to the compute precision, on the device.
static int upload_weights(const double* im, int window, bool f32, DevBuf& dst, std::string* err) {
    const size_t n = 2 * (size_t)window;
    if (f32) {
        std::vector<float> w(n);
        for (size_t i = 0; i < n; ++i) w[i] = (float)im[i];
        PL_CUDA(dst.ensure(n * sizeof(float)), "cudaMalloc");
        PL_CUDA(cudaMemcpy(dst.p, w.data(), n * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy");
    } else {
        PL_CUDA(dst.ensure(n * sizeof(double)), "cudaMalloc");
        PL_CUDA(cudaMemcpy(dst.p, im, n * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy");
    }
    return 0;
}

Pool::~Pool() {
    if (graph_) cudaGraphExecDestroy(graph_);
    if (remain_host_) cudaFreeHost(remain_host_);
    if (st_) cudaStreamDestroy(st_);
}

int Pool::create(const Pattern& pat, int precision, int window, const double* im, double h,
                 const std::vector<int>& max_comp, const std::vector<int>& sq_comp, int capacity,
                 long long arena_samples, int chunk, int slicing, std::unique_ptr<Pool>* out, std::string* err) {
    if (capacity < 1 || arena_samples < 1 || chunk < 1) { *err = "pool sizes must be positive"; return 1; }
    if (window < 0 || (window > 0 && ((window & (window - 1)) || !im))) {
        *err = "window must be 0 or a power of two with weights";
        return 1;
    }
    if (!(h > 0.0)) { *err = "time step must be positive"; return 1; }
    if (precision == kFP32Ext) { *err = "serving pools run FP64, FP32 or FP32 with compensated update"; return 1; }
    std::unique_ptr<Pool> p(new Pool());
    int rc = plan_create(pat, precision, false, &p->plan_, err);
    if (rc) return rc;
    rc = p->plan_->ensure_device(err);
    if (rc) return rc;
    const int n = pat.n;
    auto mask = [&](const std::vector<int>& c, unsigned long long* m) {
        *m = 0;
        int prev = -1;
        for (int v : c) {
            if (v < 0 || v >= n || v >= 64 || v <= prev) return false;
            *m |= 1ull << v;
            prev = v;
        }
        return true;
    };
    if (!mask(max_comp, &p->max_mask_) || !mask(sq_comp, &p->sq_mask_)) {
        *err = "reducer components must be ascending, unique, < n and < 64";
        return 1;
    }
    p->max_comp_ = max_comp;
    p->sq_comp_ = sq_comp;
    p->C_ = capacity;
    p->chunk_ = chunk;
    p->window_ = window;
    p->h_ = h;
    p->S_ = arena_samples;
    const bool f32 = precision != kFP64;
    const size_t rs = f32 ? sizeof(float) : sizeof(double);
    const size_t C = (size_t)capacity;
    const size_t P = (size_t)(pat.P() > 0 ? pat.P() : 1);
    PL_CUDA(p->vals_.ensure(P * C * rs), "cudaMalloc");
    PL_CUDA(p->state_.ensure((size_t)n * C * rs), "cudaMalloc");
    PL_CUDA(p->comp_.ensure((size_t)n * C * rs), "cudaMalloc");
    PL_CUDA(p->mx_.ensure((size_t)n * C * rs), "cudaMalloc");
    PL_CUDA(p->sq_.ensure(C * rs), "cudaMalloc");
    PL_CUDA(p->sqc_.ensure(C * rs), "cudaMalloc");
    PL_CUDA(p->step_.ensure(C * sizeof(unsigned)), "cudaMalloc");
    PL_CUDA(p->remain_.ensure(C * sizeof(int)), "cudaMalloc");
    PL_CUDA(p->ebase_.ensure(C * sizeof(long long)), "cudaMalloc");
    PL_CUDA(p->lim_.ensure(C * sizeof(long long)), "cudaMalloc");
    PL_CUDA(p->len_.ensure(C * sizeof(unsigned)), "cudaMalloc");
    PL_CUDA(p->mstart_.ensure(C * sizeof(int)), "cudaMalloc");
    PL_CUDA(p->sstart_.ensure(C * sizeof(int)), "cudaMalloc");
    PL_CUDA(p->arena_.ensure((size_t)arena_samples * rs), "cudaMalloc");
    // admission / harvest staging for a full pool and a table of up to 8M samples,
    // so that serving does not allocate (an allocation synchronises the device)
    PL_CUDA(p->scratch_.ensure(C * (sizeof(double) * (P + 3 * (size_t)n) + 64) +
                               sizeof(double) * (size_t)std::min<long long>(arena_samples, 1LL << 23)),
            "cudaMalloc");
    if (window > 0) {   // weights on the device for the steps outside whole intervals
        rc = upload_weights(im, window, f32, p->im_dev_, err);
        if (rc) return rc;
    }
    PL_CUDA(cudaMemset(p->remain_.p, 0, C * sizeof(int)), "cudaMemset");
    PL_CUDA(cudaMemset(p->vals_.p, 0, P * C * rs), "cudaMemset");
    PL_CUDA(cudaMemset(p->state_.p, 0, (size_t)n * C * rs), "cudaMemset");
    // every per-slot field defined from the start (a free slot's are read by
    // no kernel, but nothing is left uninitialised)
    PL_CUDA(cudaMemset(p->comp_.p, 0, (size_t)n * C * rs), "cudaMemset");
    PL_CUDA(cudaMemset(p->mx_.p, 0, (size_t)n * C * rs), "cudaMemset");
    PL_CUDA(cudaMemset(p->sq_.p, 0, C * rs), "cudaMemset");
    PL_CUDA(cudaMemset(p->sqc_.p, 0, C * rs), "cudaMemset");
    PL_CUDA(cudaMemset(p->step_.p, 0, C * sizeof(unsigned)), "cudaMemset");
    PL_CUDA(cudaMemset(p->ebase_.p, 0, C * sizeof(long long)), "cudaMemset");
    PL_CUDA(cudaMemset(p->lim_.p, 0, C * sizeof(long long)), "cudaMemset");
    PL_CUDA(cudaMemset(p->len_.p, 0, C * sizeof(unsigned)), "cudaMemset");
    PL_CUDA(cudaMemset(p->mstart_.p, 0, C * sizeof(int)), "cudaMemset");
    PL_CUDA(cudaMemset(p->sstart_.p, 0, C * sizeof(int)), "cudaMemset");
    // highest priority: a chunk's blocks are scheduled ahead of queued blocks of
    // lower-priority work (e.g. adjoint sweeps), which bounds forward latency
    int prio_least = 0, prio_greatest = 0;
    PL_CUDA(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest), "cudaDeviceGetStreamPriorityRange");
    PL_CUDA(cudaStreamCreateWithPriority(&p->st_, cudaStreamNonBlocking, prio_greatest), "cudaStreamCreate");
    PL_CUDA(cudaMallocHost((void**)&p->remain_host_, C * sizeof(int)), "cudaMallocHost");
    p->free_.resize(C);
    for (int i = 0; i < capacity; ++i) p->free_[i] = capacity - 1 - i;   // pop_back gives ascending slots
    p->holes_[0] = arena_samples;
    FwdKernelKey key;
    key.f32 = f32;
    key.kahan = precision == kFP32Kahan;
    key.max_mask = p->max_mask_;
    key.sq_mask = p->sq_mask_;
    key.window = window;
    key.slices = slicing < 0 ? 0 : ws_slices(pat, f32, slicing > 0);
    for (int i = 0; i < 2 * window; ++i) {
        const double w = f32 ? (double)(float)im[i] : im[i];
        p->im_.push_back(im[i]);
        (i < window ? key.wn : key.wc).push_back(w);
    }
    std::string jerr;
    if (!get_pool_kernel(pat, key, &p->k_, &jerr)) { *err = "pool kernel: " + jerr; return 3; }
    rc = p->build_graph(err);
    if (rc) return rc;
    *out = std::move(p);
    return 0;
}

int Pool::build_graph(std::string* err) {
    const bool f32 = plan_->precision != kFP64;
    const int window = window_;
    auto fill = [&](auto& a, auto rtag) {
        typedef decltype(rtag) R;
        std::memset(&a, 0, sizeof(a));
        a.vals = vals_.as<R>();
        a.state = state_.as<R>();
        a.comp = comp_.as<R>();
        a.mx = mx_.as<R>();
        a.sq = sq_.as<R>();
        a.sqc = sqc_.as<R>();
        a.step = step_.as<unsigned>();
        a.remain = remain_.as<int>();
        a.ebase = ebase_.as<long long>();
        a.lim = lim_.as<long long>();
        a.len = len_.as<unsigned>();
        a.max_start = mstart_.as<int>();
        a.sq_start = sstart_.as<int>();
        a.frc.x = arena_.as<R>();
        a.frc.im = window > 0 ? im_dev_.as<R>() : nullptr;
        a.frc.total = S_;
        a.frc.len = 0;
        a.frc.w = (unsigned)window;
        a.frc.lw = 0;
        while (window > 0 && (1u << a.frc.lw) < (unsigned)window) a.frc.lw++;
        a.h = (R)h_;
        a.h2 = (R)(h_ / 2.0);
        a.h6 = (R)(h_ / 6.0);
        a.C = C_;
        a.chunk = chunk_;
    };
    const dim3 grid((unsigned)((C_ + k_.per_block - 1) / k_.per_block));
    cudaGraph_t g = nullptr;
    PL_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    cudaError_t e;
    if (f32) {
        pk::PoolArgs<float> a;
        fill(a, 0.0f);
        void* args[] = {&a};
        e = cudaLaunchKernel((const void*)k_.fn, grid, dim3(k_.block), args, (size_t)k_.smem, st_);
    } else {
        pk::PoolArgs<double> a;
        fill(a, 0.0);
        void* args[] = {&a};
        e = cudaLaunchKernel((const void*)k_.fn, grid, dim3(k_.block), args, (size_t)k_.smem, st_);
    }
    cudaError_t e2 = cudaStreamEndCapture(st_, &g);
    PL_CUDA(e, "pool kernel capture");
    PL_CUDA(e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&graph_, g, 0);
    cudaGraphDestroy(g);
    PL_CUDA(e, "cudaGraphInstantiate");
    return 0;
}

long long Pool::arena_alloc(long long n) {
    for (auto it = holes_.begin(); it != holes_.end(); ++it) {
        if (it->second >= n) {
            const long long off = it->first, rest = it->second - n;
            holes_.erase(it);
            if (rest > 0) holes_[off + n] = rest;
            return off;
        }
    }
    return -1;
}

void Pool::arena_free(long long off, long long n) {
    auto it = holes_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != holes_.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        holes_.erase(nx);
    }
    if (it != holes_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            holes_.erase(it);
        }
    }
}

long long Pool::free_arena() const {
    long long best = 0;
    for (auto& h : holes_) best = std::max(best, h.second);
    return best;
}

int Pool::admit(int n_sys, const double* values, const double* x0, const int* exc_index, const double* signals,
                int n_exc, int len, int nsteps, int max_start, int sq_start, int* req_id, std::string* err) {
    const Pattern& pat = plan_->pat;
    const int n = pat.n, P = pat.P();
    if (failed_) { *err = "pool unusable after a failed admission (its device state is unknown)"; return 2; }
    if (n_sys < 1 || n_exc < 1 || len < 1 || nsteps < 0 || !values || !x0 || !exc_index || !signals) {
        *err = "bad request";
        return 1;
    }
    for (int i = 0; i < n_sys; ++i)
        if (exc_index[i] < 0 || exc_index[i] >= n_exc) { *err = "excitation index out of range"; return 1; }
    const long long table = (long long)n_exc * len;
    if (n_sys > C_ || table > S_) { *err = "request larger than the pool (slots or signal arena)"; return 1; }
    const bool f32 = plan_->precision != kFP64;
    // staging: values, x0, zeros, signals (double) | slots, step, remain, mstart, sstart (int) | ebase, lim (i64) | len (u32)
    auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
    const size_t o_vals = 0, o_x0 = al(o_vals + sizeof(double) * (size_t)n_sys * P);
    const size_t o_zero = al(o_x0 + sizeof(double) * (size_t)n_sys * n);
    const size_t o_sig = al(o_zero + sizeof(double) * (size_t)n_sys * n);
    const size_t o_slots = al(o_sig + sizeof(double) * (size_t)table);
    const size_t o_step = al(o_slots + sizeof(int) * n_sys), o_rem = al(o_step + sizeof(int) * n_sys);
    const size_t o_ms = al(o_rem + sizeof(int) * n_sys), o_ss = al(o_ms + sizeof(int) * n_sys);
    const size_t o_eb = al(o_ss + sizeof(int) * n_sys), o_lim = al(o_eb + sizeof(long long) * n_sys);
    const size_t o_len = al(o_lim + sizeof(long long) * n_sys), total = al(o_len + sizeof(unsigned) * n_sys);
    PL_CUDA(scratch_.ensure(total), "cudaMalloc");   // before any slot or arena space is taken
    if ((int)free_.size() < n_sys) { *err = "pool full"; return 5; }
    const long long off = arena_alloc(table);
    if (off < 0) { *err = "signal arena full"; return 5; }
    PoolRequest r;
    r.n_sys = n_sys;
    r.arena_off = off;
    r.arena_len = table;
    for (int i = 0; i < n_sys; ++i) {
        r.slots.push_back(free_.back());
        free_.pop_back();
    }
    // upload and scatter into the slots; `remain` last, so a slot becomes busy
    // only when everything else is in place
    auto stage = [&]() -> int {
        std::vector<unsigned char> host(total, 0);
        std::memcpy(&host[o_vals], values, sizeof(double) * (size_t)n_sys * P);
        std::memcpy(&host[o_x0], x0, sizeof(double) * (size_t)n_sys * n);
        std::memcpy(&host[o_sig], signals, sizeof(double) * (size_t)table);
        for (int i = 0; i < n_sys; ++i) {
            reinterpret_cast<int*>(&host[o_slots])[i] = r.slots[i];
            reinterpret_cast<unsigned*>(&host[o_step])[i] = 0u;
            reinterpret_cast<int*>(&host[o_rem])[i] = nsteps;
            reinterpret_cast<int*>(&host[o_ms])[i] = max_start;
            reinterpret_cast<int*>(&host[o_ss])[i] = sq_start;
            reinterpret_cast<long long*>(&host[o_eb])[i] = off + (long long)exc_index[i] * len;
            reinterpret_cast<long long*>(&host[o_lim])[i] = off + table;
            reinterpret_cast<unsigned*>(&host[o_len])[i] = (unsigned)len;
        }
        unsigned char* d = scratch_.as<unsigned char>();
        PL_CUDA(cudaMemcpyAsync(d, host.data(), total, cudaMemcpyHostToDevice, st_), "cudaMemcpyAsync");
        const int* dslots = reinterpret_cast<const int*>(d + o_slots);
        const double* dz = reinterpret_cast<const double*>(d + o_zero);
        const long long Cl = C_;
        PL_CUDA(pk::launch_scatter_cols(reinterpret_cast<const double*>(d + o_vals), vals_.p, dslots, n_sys, P, Cl, f32,
                                        st_),
                "scatter");
        PL_CUDA(pk::launch_scatter_cols(reinterpret_cast<const double*>(d + o_x0), state_.p, dslots, n_sys, n, Cl, f32,
                                        st_),
                "scatter");
        PL_CUDA(pk::launch_scatter_cols(dz, comp_.p, dslots, n_sys, n, Cl, f32, st_), "scatter");
        PL_CUDA(pk::launch_scatter_cols(dz, mx_.p, dslots, n_sys, n, Cl, f32, st_), "scatter");
        PL_CUDA(pk::launch_scatter_cols(dz, sq_.p, dslots, n_sys, 1, Cl, f32, st_), "scatter");
        PL_CUDA(pk::launch_scatter_cols(dz, sqc_.p, dslots, n_sys, 1, Cl, f32, st_), "scatter");
        const size_t rs = f32 ? sizeof(float) : sizeof(double);
        PL_CUDA(pk::launch_convert(reinterpret_cast<const double*>(d + o_sig),
                                   arena_.as<unsigned char>() + (size_t)off * rs, table, f32, st_),
                "convert");
        PL_CUDA(pk::launch_scatter_u32(reinterpret_cast<const unsigned*>(d + o_step), step_.as<unsigned>(), dslots, n_sys,
                                       st_),
                "scatter");
        PL_CUDA(pk::launch_scatter_i32(reinterpret_cast<const int*>(d + o_ms), mstart_.as<int>(), dslots, n_sys, st_),
                "scatter");
        PL_CUDA(pk::launch_scatter_i32(reinterpret_cast<const int*>(d + o_ss), sstart_.as<int>(), dslots, n_sys, st_),
                "scatter");
        PL_CUDA(pk::launch_scatter_i64(reinterpret_cast<const long long*>(d + o_eb), ebase_.as<long long>(), dslots,
                                       n_sys, st_),
                "scatter");
        PL_CUDA(pk::launch_scatter_i64(reinterpret_cast<const long long*>(d + o_lim), lim_.as<long long>(), dslots,
                                       n_sys, st_),
                "scatter");
        PL_CUDA(pk::launch_scatter_u32(reinterpret_cast<const unsigned*>(d + o_len), len_.as<unsigned>(), dslots, n_sys,
                                       st_),
                "scatter");
        PL_CUDA(pk::launch_scatter_i32(reinterpret_cast<const int*>(d + o_rem), remain_.as<int>(), dslots, n_sys, st_),
                "scatter");
        PL_CUDA(cudaStreamSynchronize(st_), "cudaStreamSynchronize");   // staging reused by the next admission
        return 0;
    };
    if (const int rc = stage()) {
        // part of the upload may have run (the `remain` scatter is queued
        // last, but a failed stream synchronisation leaves it unknown whether
        // it ran): the slots cannot be handed out again, nor the pool trusted
        failed_ = true;
        return rc;
    }
    *req_id = next_id_++;
    reqs_[*req_id] = r;
    return 0;
}

int Pool::launch(std::string* err) {
    if (failed_) { *err = "pool unusable after a failed admission (its device state is unknown)"; return 2; }
    if (reqs_.empty()) return 0;
    PL_CUDA(cudaGraphLaunch(graph_, st_), "cudaGraphLaunch");
    return 0;
}

int Pool::poll(std::vector<int>* finished, std::string* err) {
    finished->clear();
    if (reqs_.empty()) return 0;
    PL_CUDA(cudaMemcpyAsync(remain_host_, remain_.p, sizeof(int) * C_, cudaMemcpyDeviceToHost, st_), "cudaMemcpyAsync");
    PL_CUDA(cudaStreamSynchronize(st_), "cudaStreamSynchronize");
    for (auto& kv : reqs_) {
        bool done = true;
        for (int s : kv.second.slots)
            if (remain_host_[s] > 0) { done = false; break; }
        if (done) finished->push_back(kv.first);
    }
    return 0;
}

int Pool::harvest(int req_id, double* state, double* max, double* sq, std::string* err) {
    auto it = reqs_.find(req_id);
    if (it == reqs_.end()) { *err = "unknown request"; return 1; }
    const PoolRequest& r = it->second;
    // finished = every slot at 0 remaining steps, read after the last chunk
    // (a request harvested early would free slots a chunk may still advance)
    PL_CUDA(cudaMemcpyAsync(remain_host_, remain_.p, sizeof(int) * C_, cudaMemcpyDeviceToHost, st_), "cudaMemcpyAsync");
    PL_CUDA(cudaStreamSynchronize(st_), "cudaStreamSynchronize");
    for (int s : r.slots)
        if (remain_host_[s] > 0) { *err = "request not finished (poll until it is listed)"; return 5; }
    const int n = plan_->pat.n, m = r.n_sys;
    const bool f32 = plan_->precision != kFP64;
    const size_t so = 0, oo = (sizeof(double) * (size_t)m * n + 15) & ~(size_t)15;
    const size_t mo = oo + ((sizeof(int) * m + 15) & ~(size_t)15);
    const size_t qo = mo + ((sizeof(double) * (size_t)m * n + 15) & ~(size_t)15);
    const size_t total = qo + sizeof(double) * m;
    PL_CUDA(scratch_.ensure(total), "cudaMalloc");
    unsigned char* d = scratch_.as<unsigned char>();
    PL_CUDA(cudaMemcpyAsync(d + oo, r.slots.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st_), "cudaMemcpyAsync");
    const int* dslots = reinterpret_cast<const int*>(d + oo);
    PL_CUDA(pk::launch_gather_cols(state_.p, reinterpret_cast<double*>(d + so), dslots, m, n, C_, f32, 1.0, st_), "gather");
    PL_CUDA(pk::launch_gather_cols(mx_.p, reinterpret_cast<double*>(d + mo), dslots, m, n, C_, f32, 1.0, st_), "gather");
    PL_CUDA(pk::launch_gather_cols(sq_.p, reinterpret_cast<double*>(d + qo), dslots, m, 1, C_, f32, h_, st_), "gather");
    std::vector<double> hs((size_t)m * n), hm((size_t)m * n), hq(m);
    PL_CUDA(cudaMemcpyAsync(hs.data(), d + so, sizeof(double) * hs.size(), cudaMemcpyDeviceToHost, st_), "cudaMemcpyAsync");
    PL_CUDA(cudaMemcpyAsync(hm.data(), d + mo, sizeof(double) * hm.size(), cudaMemcpyDeviceToHost, st_), "cudaMemcpyAsync");
    PL_CUDA(cudaMemcpyAsync(hq.data(), d + qo, sizeof(double) * hq.size(), cudaMemcpyDeviceToHost, st_), "cudaMemcpyAsync");
    PL_CUDA(cudaStreamSynchronize(st_), "cudaStreamSynchronize");
    if (state) std::memcpy(state, hs.data(), sizeof(double) * hs.size());
    if (max)
        for (int i = 0; i < m; ++i)
            for (size_t c = 0; c < max_comp_.size(); ++c) max[(size_t)i * max_comp_.size() + c] = hm[(size_t)i * n + max_comp_[c]];
    if (sq) {
        if (sq_comp_.empty()) std::fill(sq, sq + m, 0.0);
        else std::memcpy(sq, hq.data(), sizeof(double) * m);
    }
    for (int s : r.slots) free_.push_back(s);
    arena_free(r.arena_off, r.arena_len);
    reqs_.erase(it);
    return 0;
}

}  // namespace pasif
