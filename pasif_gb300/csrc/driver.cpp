// driver.cpp -- __GpuDriver drop-in (src/__GpuDriver.cu, src/PASIfgpu.cpp).
//
// The reference integrates ONE concatenated system (all user systems
// block-diagonally, PASIf.py:475-543) replicated once per excitation signal
// (src/__GpuDriver.cu:896-938), with cuSPARSE SpMM + atomics per RK4 stage and
// one graph launch per step.  Here the concatenated system is split into its
// independent blocks (connected components of the coupling graph), blocks of
// identical pattern are grouped, and every (block, signal) pair becomes one
// instance of a batch that a single persistent kernel integrates for the
// whole horizon.  Per-destination term order is preserved by the split, so
// results are those of the canonical order the oracle fixes.
#include "driver.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <map>
#include <numeric>

namespace pasif {

namespace {

struct DSU {
    std::vector<int> p;
    explicit DSU(int n) : p(n) { std::iota(p.begin(), p.end(), 0); }
    int find(int x) {
        while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; }
        return x;
    }
    void unite(int a, int b) {
        a = find(a); b = find(b);
        if (a != b) { if (a < b) p[b] = a; else p[a] = b; }
    }
};

// Force pattern -> COO, dropping |v| <= eps (COOVector, src/helpers.cu:664-682).
void force_coo(const std::vector<double>& dense, std::vector<int>* idx, std::vector<double>* val) {
    for (size_t i = 0; i < dense.size(); ++i)
        if (std::fabs(dense[i]) > DBL_EPSILON) { idx->push_back((int)i); val->push_back(dense[i]); }
}

// Split forward system f (size nf) and, when b != nullptr, its adjoint b
// (size na, setpoint indices in the forward space) into blocks.
int decompose(const SystemIn& f, int nf, const SystemIn* b, int na, std::vector<Block>* out, std::string* err) {
    const int N = nf + (b ? na : 0);
    DSU d(N);
    for (int i = 0; i < nf; ++i)
        for (unsigned p = f.K.ptr[i]; p < f.K.ptr[i + 1]; ++p) d.unite(i, (int)f.K.col[p]);
    auto unite_coo = [&](const CooIn& c, int w, int off_src, int off_sp) {
        if (!c.set) return;
        for (size_t e = 0; e < c.val.size(); ++e) {
            const unsigned* ix = &c.idx[e * w];
            d.unite(off_src + (int)ix[0], off_src + (int)ix[1]);
            for (int k = 2; k < w; ++k) d.unite(off_src + (int)ix[0], off_sp + (int)ix[k]);
        }
    };
    unite_coo(f.G, 3, 0, 0);
    unite_coo(f.L, 4, 0, 0);
    unite_coo(f.Psi, 5, 0, 0);
    if (b) {
        for (int i = 0; i < na; ++i)
            for (unsigned p = b->K.ptr[i]; p < b->K.ptr[i + 1]; ++p) d.unite(nf + i, nf + (int)b->K.col[p]);
        unite_coo(b->G, 3, nf, 0);
        unite_coo(b->L, 4, nf, 0);
        unite_coo(b->Psi, 5, nf, 0);
    }
    std::map<int, int> root2blk;
    out->clear();
    std::vector<int> blk(N), loc(N);
    for (int x = 0; x < N; ++x) {
        int r = d.find(x);
        auto it = root2blk.find(r);
        int bi;
        if (it == root2blk.end()) { bi = (int)out->size(); root2blk[r] = bi; out->emplace_back(); }
        else bi = it->second;
        blk[x] = bi;
        Block& B = (*out)[bi];
        if (x < nf) { loc[x] = (int)B.nodes.size(); B.nodes.push_back(x); }
        else { loc[x] = (int)B.anodes.size(); B.anodes.push_back(x - nf); }
    }
    std::vector<int> fidx;
    std::vector<double> fval;
    force_coo(f.force, &fidx, &fval);
    std::vector<int> bfidx;
    std::vector<double> bfval;
    if (b) force_coo(b->force, &bfidx, &bfval);
    for (auto& B : *out) {
        B.pat = Pattern();
        B.pat.n = (int)B.nodes.size();
        B.pat.n_sp = B.pat.n;
        B.pat.k_ptr.push_back(0);
        if (b) {
            B.apat = Pattern();
            B.apat.n = (int)B.anodes.size();
            B.apat.n_sp = B.pat.n;
            B.apat.k_ptr.push_back(0);
        }
    }
    // K rows in CSR order (forward, then adjoint)
    for (int i = 0; i < nf; ++i) {
        Block& B = (*out)[blk[i]];
        for (unsigned p = f.K.ptr[i]; p < f.K.ptr[i + 1]; ++p) {
            B.pat.k_col.push_back(loc[f.K.col[p]]);
            B.vals.push_back(f.K.val[p]);
        }
        B.pat.k_ptr.push_back((int)B.pat.k_col.size());
    }
    if (b)
        for (int i = 0; i < na; ++i) {
            Block& B = (*out)[blk[nf + i]];
            for (unsigned p = b->K.ptr[i]; p < b->K.ptr[i + 1]; ++p) {
                B.apat.k_col.push_back(loc[nf + b->K.col[p]]);
                B.avals.push_back(b->K.val[p]);
            }
            B.apat.k_ptr.push_back((int)B.apat.k_col.size());
        }
    // tensors in COO order
    auto add_coo = [&](const CooIn& c, int w, bool adj) {
        if (!c.set) return;
        const int off = adj ? nf : 0;
        for (size_t e = 0; e < c.val.size(); ++e) {
            const unsigned* ix = &c.idx[e * w];
            Block& B = (*out)[blk[off + (int)ix[0]]];
            Pattern& P = adj ? B.apat : B.pat;
            std::vector<int>& dst = w == 3 ? P.g_idx : (w == 4 ? P.l_idx : P.p_idx);
            dst.push_back(loc[off + (int)ix[0]]);
            dst.push_back(loc[off + (int)ix[1]]);
            for (int k = 2; k < w; ++k) dst.push_back(loc[(int)ix[k]]);
            (adj ? B.avals : B.vals).push_back(c.val[e]);
        }
    };
    // values are appended per block in parameter order: K, Gamma, Lambda, Psi, F
    add_coo(f.G, 3, false);
    add_coo(f.L, 4, false);
    add_coo(f.Psi, 5, false);
    for (size_t e = 0; e < fidx.size(); ++e) {
        Block& B = (*out)[blk[fidx[e]]];
        B.pat.f_idx.push_back(loc[fidx[e]]);
        B.vals.push_back(fval[e]);
    }
    if (b) {
        add_coo(b->G, 3, true);
        add_coo(b->L, 4, true);
        add_coo(b->Psi, 5, true);
        for (size_t e = 0; e < bfidx.size(); ++e) {
            Block& B = (*out)[blk[nf + bfidx[e]]];
            B.apat.f_idx.push_back(loc[nf + bfidx[e]]);
            B.avals.push_back(bfval[e]);
        }
    }
    for (auto& B : *out) {
        std::string v = B.pat.validate();
        if (v.empty() && b) v = B.apat.validate();
        if (!v.empty()) { *err = "block pattern: " + v; return 1; }
    }
    return 0;
}

int check_system(const SystemIn& s, int n, int nsp, bool adjoint, std::string* err) {
    const char* who = adjoint ? "adjoint" : "forward";
    if (!s.ic_set) { *err = std::string(who) + " initial conditions not set"; return 5; }
    if (!s.K.set) { *err = std::string(who) + " K not set"; return 5; }
    if ((int)s.K.rows != n || (int)s.K.cols != n) {
        *err = std::string(who) + " K shape differs from the number of initial conditions";
        return 1;
    }
    if (s.K.ptr.size() != (size_t)n + 1 || s.K.ptr[0] != 0 || s.K.ptr[n] != s.K.val.size()) {
        *err = std::string(who) + " K: indptr must hold rows+1 entries from 0 to nnz";
        return 1;
    }
    for (int i = 0; i < n; ++i)
        if (s.K.ptr[i + 1] < s.K.ptr[i]) { *err = std::string(who) + " K: indptr decreasing"; return 1; }
    for (unsigned c : s.K.col)
        if ((int)c >= n) { *err = std::string(who) + " K: column index out of range"; return 1; }
    if (!s.force_set || (int)s.force.size() != n) {
        *err = std::string(who) + " force pattern must hold one value per state variable";
        return 1;
    }
    auto chk = [&](const CooIn& c, int w, const char* name) -> int {
        if (!c.set) return 0;
        if (!c.dims.empty() && (int)c.dims[0] != n && !c.val.empty()) {
            *err = std::string(who) + " " + name + ": first dimension differs from the state size";
            return 1;
        }
        for (size_t e = 0; e < c.val.size(); ++e) {
            const unsigned* ix = &c.idx[e * w];
            if ((int)ix[0] >= n || (int)ix[1] >= n) { *err = std::string(who) + " " + name + ": index out of range"; return 1; }
            for (int k = 2; k < w; ++k)
                if ((int)ix[k] >= nsp) { *err = std::string(who) + " " + name + ": setpoint index out of range"; return 1; }
        }
        return 0;
    };
    if (chk(s.G, 3, "Gamma") || chk(s.L, 4, "Lambda") || chk(s.Psi, 5, "Psi")) return 1;
    return 0;
}

}  // namespace

Driver::Driver(unsigned gpu, unsigned sample_rate, unsigned numsteps, bool dc, bool ds, bool dsol)
    : gpu_(gpu), sample_rate_(sample_rate), numsteps_(numsteps), dcompute_(dc), dsystem_(ds), dsolver_(dsol) {
    h_ = sample_rate_ ? 1.0 / (double)sample_rate_ : 0.0;
}

void Driver::info(const std::string& s) const { std::printf("[Info] pasif_gb300: %s\n", s.c_str()); }

int Driver::load_excitations(const double* const* sig, const long long* len, int n, unsigned sample_rate,
                             std::string* err) {
    sample_rate_ = sample_rate;
    h_ = sample_rate_ ? 1.0 / (double)sample_rate_ : 0.0;   // src/__GpuDriver.cu:632-636
    exc_.clear();
    exc_ok_ = false;
    signals_.reset();
    n_exc_ = 0;
    exc_len_ = 0;
    if (n < 1) { *err = "empty excitation set"; return 1; }
    for (int i = 0; i < n; ++i)
        if (len[i] != len[0]) { *err = "excitation vectors are not of the same size"; return 6; }
    if (len[0] < 1) { *err = "empty excitation signal"; return 1; }
    n_exc_ = n;
    exc_len_ = (int)len[0];
    exc_.resize((size_t)n * exc_len_);
    for (int i = 0; i < n; ++i)
        for (long long k = 0; k < exc_len_; ++k) exc_[(size_t)i * exc_len_ + k] = sig[i][k];
    exc_ok_ = true;
    // a change in the number of signals changes every batch
    groups_.clear();
    return 0;
}

long long sweep_chunk(long long n_instances, long long bytes_per_instance, long long budget) {
    if (n_instances <= 0) return 0;
    if (bytes_per_instance <= 0) return n_instances;
    const long long fit = budget / bytes_per_instance;
    return fit >= n_instances ? n_instances : fit;
}

int Driver::set_memory_budget(long long bytes, std::string* err) {
    if (bytes < 0) { *err = "negative memory budget"; return 1; }
    mem_budget_ = bytes;
    return 0;
}

// The budget of a solve: the set one, or 90 % of the free device memory plus
// `held` bytes the driver's own buffers for this solve already occupy.
long long Driver::budget_for(long long held) const {
    if (mem_budget_ > 0) return mem_budget_;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return 1LL << 62;   // unknown: no split
    }
    return (long long)((double)free_b * 0.9) + held;
}

int Driver::set_precision(int p, std::string* err) {
    if (p < kFP64 || p > kFP32Ext) { *err = "unknown precision"; return 1; }
    if (p != precision_) { precision_ = p; signals_.reset(); groups_.clear(); }
    return 0;
}

int Driver::set_k(bool fwd, unsigned rows, unsigned cols, const double* v, const unsigned* ind,
                  const unsigned* ptr, long long nnz, std::string* err) {
    SystemIn& s = fwd ? fwd_ : bwd_;
    if (nnz < 0 || (nnz > 0 && (!v || !ind)) || !ptr) { *err = "null CSR array"; return 1; }
    s.K.set = true;
    s.K.rows = rows;
    s.K.cols = cols;
    s.K.val.assign(v, v + nnz);
    s.K.col.assign(ind, ind + nnz);
    s.K.ptr.assign(ptr, ptr + rows + 1);
    (fwd ? sys_alloc_ : adj_alloc_) = false;
    groups_.clear();
    return 0;
}

int Driver::set_coo(bool fwd, int order, const unsigned* dims, const double* v, const unsigned* ind,
                    long long nnz, std::string* err) {
    SystemIn& s = fwd ? fwd_ : bwd_;
    if (nnz < 0 || (nnz > 0 && (!v || !ind)) || !dims) { *err = "null COO array"; return 1; }
    CooIn& c = order == 3 ? s.G : (order == 4 ? s.L : s.Psi);
    c.set = true;
    c.dims.assign(dims, dims + order);
    c.val.assign(v, v + nnz);
    c.idx.assign(ind, ind + nnz * order);
    (fwd ? sys_alloc_ : adj_alloc_) = false;
    groups_.clear();
    return 0;
}

int Driver::set_force(bool fwd, const double* v, long long n, std::string* err) {
    SystemIn& s = fwd ? fwd_ : bwd_;
    if (n < 0 || (n > 0 && !v)) { *err = "null force pattern"; return 1; }
    s.force_set = true;
    s.force.assign(v, v + n);
    (fwd ? sys_alloc_ : adj_alloc_) = false;
    groups_.clear();
    return 0;
}

int Driver::set_ic(bool fwd, const double* v, long long n, std::string* err) {
    SystemIn& s = fwd ? fwd_ : bwd_;
    if (n < 0 || (n > 0 && !v)) { *err = "null initial conditions"; return 1; }
    s.ic_set = true;
    s.ic.assign(v, v + n);
    (fwd ? nf_ : na_) = (int)n;
    (fwd ? sys_alloc_ : adj_alloc_) = false;
    groups_.clear();
    return 0;
}

int Driver::allocate_system(std::string* err) {
    int rc = check_system(fwd_, nf_, nf_, false, err);
    if (rc) return rc;
    sys_alloc_ = true;
    groups_.clear();
    if (dcompute_) info("forward system of " + std::to_string(nf_) + " states x " + std::to_string(n_exc_) + " excitations");
    return 0;
}

int Driver::allocate_adjoint(std::string* err) {
    if (!sys_alloc_) { *err = "the forward system must be allocated before the adjoint"; return 5; }
    int rc = check_system(bwd_, na_, nf_, true, err);
    if (rc) return rc;
    adj_alloc_ = true;
    bwd_state_.assign((size_t)(n_exc_ > 0 ? n_exc_ : 0) * na_, 0.0);
    for (int e = 0; e < n_exc_; ++e)
        for (int i = 0; i < na_; ++i) bwd_state_[(size_t)e * na_ + i] = bwd_.ic[i];
    return 0;
}

int Driver::set_interp(const double* m, long long size, unsigned window, std::string* err) {
    if (window == 0 || (window & (window - 1))) {
        *err = "interpolation window size must be a power of two";
        return 1;
    }
    if (size < 2LL * window || !m) {
        *err = "interpolation matrix needs at least two rows of window weights";
        return 1;
    }
    im_.assign(m, m + 2LL * window);
    window_ = window;
    signals_.reset();
    return 0;
}

int Driver::set_modulation(const double* m, long long n, std::string* err) {
    if (n < 0 || (n > 0 && !m)) { *err = "null modulation buffer"; return 1; }
    modulation_.assign(m, m + n);   // accepted and unused, as in the reference
    return 0;
}

int Driver::ensure_signals(std::string* err) {
    if (!exc_ok_) { *err = "no valid excitation set (signals must share one length)"; return 5; }
    if (!(h_ > 0.0) || !std::isfinite(h_)) { *err = "sample rate must be positive"; return 1; }
    if (signals_) return 0;
    if (cudaSetDevice((int)gpu_) != cudaSuccess) { *err = "cudaSetDevice failed"; return 2; }
    if (!stream_) {
        cudaError_t e = cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking);
        if (e != cudaSuccess) { *err = cuda_err("cudaStreamCreate", e); return 2; }
    }
    return signals_create(exc_.data(), n_exc_, exc_len_, (int)window_, window_ ? im_.data() : nullptr, precision_,
                          kHost, stream_, &signals_, err);
}

int Driver::build_forward_groups(std::string* err) {
    if (!groups_.empty()) return 0;
    int rc = decompose(fwd_, nf_, nullptr, 0, &blocks_, err);
    if (rc) return rc;
    std::map<std::string, int> key2g;
    for (int bi = 0; bi < (int)blocks_.size(); ++bi) {
        const std::string k = blocks_[bi].pat.key();
        auto it = key2g.find(k);
        if (it == key2g.end()) { key2g[k] = (int)groups_.size(); groups_.emplace_back(); groups_.back().blocks.push_back(bi); }
        else groups_[it->second].blocks.push_back(bi);
    }
    const int E = n_exc_;
    for (auto& g : groups_) {
        const Block& b0 = blocks_[g.blocks[0]];
        rc = plan_create(b0.pat, precision_, false, &g.plan, err);
        if (rc) return rc;
        const int nb = (int)g.blocks.size(), B = nb * E, P = b0.pat.P(), n = b0.pat.n;
        g.hvals.assign((size_t)B * P, 0.0);
        g.hx0.assign((size_t)B * n, 0.0);
        g.hexc.assign(B, 0);
        for (int e = 0; e < E; ++e)
            for (int c = 0; c < nb; ++c) {
                const Block& bl = blocks_[g.blocks[c]];
                const size_t b = (size_t)e * nb + c;
                for (int q = 0; q < P; ++q) g.hvals[b * P + q] = bl.vals[q];
                for (int i = 0; i < n; ++i) g.hx0[b * n + i] = fwd_.ic[bl.nodes[i]];
                g.hexc[b] = e;   // the instance's own signal, whatever batch it runs in
            }
        g.resident = 0;   // uploaded by the first solve, in one batch or in sequential ones
    }
    if (dcompute_)
        info(std::to_string(blocks_.size()) + " independent blocks in " + std::to_string(groups_.size()) +
             " pattern groups");
    return 0;
}

int Driver::run_forward(int traj_every, long long slots, std::vector<double>* final_out,
                        std::vector<double>* traj_out, std::string* err) {
    if (!sys_alloc_) { *err = "the system must be allocated before a solve"; return 5; }
    int rc = ensure_signals(err);
    if (rc) return rc;
    rc = build_forward_groups(err);
    if (rc) return rc;
    const int E = n_exc_;
    if (final_out) final_out->assign((size_t)nf_ * E, 0.0);
    if (traj_out) traj_out->assign((size_t)slots * nf_ * E, 0.0);
    Reducers none;
    if (dsolver_)
        info("RK4: " + std::to_string(numsteps_) + " steps, h=" + std::to_string(h_));
    last_chunks_ = 0;
    for (auto& g : groups_) {
        const int nb = (int)g.blocks.size(), B = nb * E, n = g.plan->pat.n, P = g.plan->pat.P();
        // device bytes per instance: values, x0 and state (high and low parts
        // in the extended-state mode), reducer output, trajectory slots,
        // upload staging and the generic kernel's work vectors
        const long long rs = precision_ == kFP64 ? 8 : 4, np = precision_ == kFP32Ext ? 2 : 1;
        const long long wide = std::max(P, n);
        const long long per = rs * ((long long)P * np + 2LL * n * np + 1 + (long long)n * std::max(0LL, slots) +
                                    6LL * n) + 8 * wide * (np == 2 ? 3 : 1) + 8;
        const long long chunk = sweep_chunk(B, per, budget_for(g.batch ? (long long)g.resident * per : 0));
        if (chunk <= 0) {
            *err = "one instance needs " + std::to_string(per) + " bytes of device memory, more than the budget";
            return 4;
        }
        const long long nchunk = (B + chunk - 1) / chunk;
        last_chunks_ += (int)nchunk;
        if (!g.batch || g.batch->B != (int)chunk || (nchunk > 1 && g.resident)) {
            g.batch.reset();
            rc = batch_create(g.plan, (int)chunk, &g.batch, err);
            if (rc) return rc;
            g.resident = 0;
        }
        for (long long c0 = 0; c0 < B; c0 += chunk) {
            const int m = (int)std::min<long long>(chunk, B - c0);
            if (nchunk > 1 || !g.resident) {   // one resident batch keeps its inputs between solves
                if (g.batch->B != m) {
                    rc = g.batch->resize(m, err);
                    if (rc) return rc;
                }
                rc = g.batch->set(g.hvals.data() + c0 * P, g.hx0.data() + c0 * n, g.hexc.data() + c0, kHost,
                                  stream_, err);
                if (rc) return rc;
                g.resident = nchunk == 1 ? m : 0;
            }
            rc = g.batch->forward(*signals_, h_, 0, (int)numsteps_, none, traj_every, slots, stream_, err);
            if (rc) return rc;
            last_kind_ = g.batch->last_kind;
            if (final_out) {
                std::vector<double> st((size_t)m * n);
                rc = g.batch->get(st.data(), nullptr, nullptr, h_, kHost, stream_, err);
                if (rc) return rc;
                for (int k = 0; k < m; ++k) {
                    const long long b = c0 + k;
                    const int e = (int)(b / nb), c = (int)(b % nb);
                    const Block& bl = blocks_[g.blocks[c]];
                    for (int i = 0; i < n; ++i) (*final_out)[(size_t)e * nf_ + bl.nodes[i]] = st[(size_t)k * n + i];
                }
            }
            if (traj_out && slots > 0) {
                std::vector<double> tr((size_t)slots * m * n);
                rc = g.batch->get_traj(tr.data(), slots, kHost, stream_, err);
                if (rc) return rc;
                for (long long s = 0; s < slots; ++s)
                    for (int k = 0; k < m; ++k) {
                        const long long b = c0 + k;
                        const int e = (int)(b / nb), c = (int)(b % nb);
                        const Block& bl = blocks_[g.blocks[c]];
                        for (int i = 0; i < n; ++i)
                            (*traj_out)[((size_t)s * E + e) * nf_ + bl.nodes[i]] = tr[((size_t)s * m + k) * n + i];
                    }
            }
        }
    }
    return 0;
}

int Driver::amplitudes(std::vector<double>* out, std::string* err) {
    return run_forward(0, 0, out, nullptr, err);
}

int Driver::trajectory(unsigned save, std::vector<double>* out, std::string* err) {
    if (save == 0) { *err = "saveSteps must be positive"; return 1; }
    const long long N = numsteps_;
    const long long slots = (N + save - 1) / save;
    std::vector<double> full;
    int rc = run_forward((int)save, slots, nullptr, &full, err);
    if (rc) return rc;
    const long long keep = ((long long)nf_ * n_exc_ * N) / (long long)save;   // src/__GpuDriver.cu:469
    out->assign(full.begin(), full.begin() + std::min<long long>(keep, (long long)full.size()));
    return 0;
}

int Driver::gradient(unsigned save, std::vector<double>* out, std::string* err) {
    if (!sys_alloc_ || !adj_alloc_) { *err = "the system and the jacobian must be set before a gradient"; return 5; }
    int rc = ensure_signals(err);
    if (rc) return rc;
    std::vector<Block> blocks;
    rc = decompose(fwd_, nf_, &bwd_, na_, &blocks, err);
    if (rc) return rc;
    std::map<std::string, std::vector<int>> groups;
    for (int bi = 0; bi < (int)blocks.size(); ++bi)
        groups[blocks[bi].pat.key() + "#" + blocks[bi].apat.key()].push_back(bi);
    const int E = n_exc_;
    std::vector<double> res((size_t)E * na_, 0.0);
    last_chunks_ = 0;
    for (auto& kv : groups) {
        const std::vector<int>& ids = kv.second;
        const Block& b0 = blocks[ids[0]];
        std::shared_ptr<Plan> fp, bp;
        rc = plan_create(b0.pat, precision_ == kFP64 ? kFP64 : kFP32, true, &fp, err);
        if (rc) return rc;
        rc = plan_create(b0.apat, precision_ == kFP64 ? kFP64 : kFP32, true, &bp, err);
        if (rc) return rc;
        const int nb = (int)ids.size(), B = nb * E;
        const int Pf = b0.pat.P(), Pb = b0.apat.P(), nf = b0.pat.n, na = b0.apat.n;
        std::vector<double> fv((size_t)B * Pf), bv((size_t)B * Pb), x0((size_t)B * nf), a0((size_t)B * na),
            o((size_t)B * na);
        std::vector<int> exc(B);
        for (int e = 0; e < E; ++e)
            for (int c = 0; c < nb; ++c) {
                const Block& bl = blocks[ids[c]];
                const size_t b = (size_t)e * nb + c;
                for (int q = 0; q < Pf; ++q) fv[b * Pf + q] = bl.vals[q];
                for (int q = 0; q < Pb; ++q) bv[b * Pb + q] = bl.avals[q];
                for (int i = 0; i < nf; ++i) x0[b * nf + i] = fwd_.ic[bl.nodes[i]];
                for (int i = 0; i < na; ++i) a0[b * na + i] = bwd_state_[(size_t)e * na_ + bl.anodes[i]];
                exc[b] = e;
            }
        if (dsystem_) {
            std::printf("[System] gradient group: %d blocks x %d signals, forward %s values", nb, E, b0.pat.key().c_str());
            for (double v : b0.vals) std::printf(" %.17g", v);
            std::printf("\n[System] adjoint %s values", b0.apat.key().c_str());
            for (double v : b0.avals) std::printf(" %.17g", v);
            std::printf("\n[System] a0");
            for (double v : a0) std::printf(" %.17g", v);
            std::printf("\n");
        }
        // device bytes per instance of _getGradient: the slot buffer, the
        // generic kernel's work vectors, values, states and output
        const long long rs = precision_ == kFP64 ? 8 : 4;
        const long long N = numsteps_, S = (long long)std::sqrt((double)N);
        const long long Cc = S > 0 ? (N + S - 1) / S : 1;
        const long long per = rs * ((S + Cc - 1) * nf + 5LL * nf + 6LL * na + Pf + Pb + nf + 2LL * na) + 8 * 4 + 4;
        const long long chunk = sweep_chunk(B, per, budget_for(0));
        if (chunk <= 0) {
            *err = "one instance needs " + std::to_string(per) + " bytes of device memory, more than the budget";
            return 4;
        }
        last_chunks_ += (int)((B + chunk - 1) / chunk);
        for (long long c0 = 0; c0 < B; c0 += chunk) {
            const int m = (int)std::min<long long>(chunk, B - c0);
            rc = refgrad_run(*fp, *bp, m, fv.data() + c0 * Pf, bv.data() + c0 * Pb, x0.data() + c0 * nf,
                             a0.data() + c0 * na, exc.data() + c0, *signals_, h_, (int)numsteps_, (int)save,
                             o.data() + c0 * na, stream_, err);
            if (rc) return rc;
        }
        for (int b = 0; b < B; ++b) {
            const int e = b / nb, c = b % nb;
            const Block& bl = blocks[ids[c]];
            for (int i = 0; i < na; ++i) res[(size_t)e * na_ + bl.anodes[i]] = o[(size_t)b * na + i];
        }
    }
    bwd_state_ = res;   // chained terminal condition (src/__GpuDriver.cu:743)
    *out = res;
    return 0;
}

}  // namespace pasif
