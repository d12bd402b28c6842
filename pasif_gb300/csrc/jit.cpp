// jit.cpp -- NVRTC code generation of pattern-specialised RK4 kernels.
//
// For one sparsity pattern the right-hand side becomes straight-line code:
// every state component, stage vector and per-instance value lives in a
// register, every index is a literal, and values shared by all instances of
// the batch are folded in as exact hexadecimal constants.  The RK4 loop,
// forcing and reducers come from rk4_core.cuh, compiled with the generated
// struct, so the specialised kernel performs the same operations, in the same
// order, as the generic kernel and the CPU oracle.
#include "jit.h"

#include <nvrtc.h>

#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <sstream>

#include "_embedded.h"

namespace pasif {

namespace {

std::string hexlit(double v) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%a", v);
    return std::string("R(") + buf + ")";
}

struct Emitter {
    const Pattern& pat;
    const Literals& lit;
    std::vector<int> slot;   // parameter -> loaded register slot (-1: literal)
    int nload = 0;

    Emitter(const Pattern& p, const Literals& l) : pat(p), lit(l) {
        const int P = pat.P();
        slot.assign(P, -1);
        for (int q = 0; q < P; ++q) {
            bool is_lit = q < (int)lit.is_lit.size() && lit.is_lit[q] && std::isfinite(lit.value[q]);
            if (!is_lit) slot[q] = nload++;
        }
    }

    std::string val(int q) const {
        if (slot[q] >= 0) return "p[" + std::to_string(slot[q]) + "]";
        return hexlit(lit.value[q]);
    }

    // rhs body.  Per destination, the terms [K row | Gamma | Lambda | Psi |
    // forcing] are dealt in turn to two partial sums (a, c), each fma-folded
    // from +0, and added when both are used: the canonical order of the
    // oracle and of GenSys::rhs.  `force` selects the FORCE=true body.
    void rhs(std::ostringstream& o, bool force) const {
        const int n = pat.n;
        const int go = pat.k_nnz(), lo = go + pat.g_nnz(), po = lo + pat.l_nnz(), fo = po + pat.p_nnz();
        // each term as (first factor expression, last factor expression)
        std::vector<std::vector<std::pair<std::string, std::string>>> terms(n);
        for (int i = 0; i < n; ++i)
            for (int q = pat.k_ptr[i]; q < pat.k_ptr[i + 1]; ++q)
                terms[i].push_back({val(q), "xs[" + std::to_string(pat.k_col[q]) + "]"});
        for (int e = 0; e < pat.g_nnz(); ++e) {
            const int* ix = &pat.g_idx[3 * e];
            terms[ix[0]].push_back({"m::mul(" + val(go + e) + ", xs[" + std::to_string(ix[1]) + "])",
                                    "xp[" + std::to_string(ix[2]) + "]"});
        }
        for (int e = 0; e < pat.l_nnz(); ++e) {
            const int* ix = &pat.l_idx[4 * e];
            terms[ix[0]].push_back({"m::mul(m::mul(" + val(lo + e) + ", xs[" + std::to_string(ix[1]) + "]), xp[" +
                                        std::to_string(ix[2]) + "])",
                                    "xp[" + std::to_string(ix[3]) + "]"});
        }
        for (int e = 0; e < pat.p_nnz(); ++e) {
            const int* ix = &pat.p_idx[5 * e];
            terms[ix[0]].push_back({"m::mul(m::mul(m::mul(" + val(po + e) + ", xs[" + std::to_string(ix[1]) +
                                        "]), xp[" + std::to_string(ix[2]) + "]), xp[" + std::to_string(ix[3]) + "])",
                                    "xp[" + std::to_string(ix[4]) + "]"});
        }
        if (force)
            for (int e = 0; e < pat.f_nnz(); ++e) terms[pat.f_idx[e]].push_back({val(fo + e), "u"});
        for (int i = 0; i < n; ++i) {
            if (terms[i].empty()) {
                o << "      f[" << i << "] = R(0);\n";
                continue;
            }
            for (size_t k = 0; k < terms[i].size(); ++k) {
                const char* acc = (k & 1) ? "c" : "a";
                if (k < 2)
                    o << "      " << acc << " = m::mul(" << terms[i][k].first << ", " << terms[i][k].second << ");\n";
                else
                    o << "      " << acc << " = m::fma(" << terms[i][k].first << ", " << terms[i][k].second << ", "
                      << acc << ");\n";
            }
            o << "      f[" << i << "] = " << (terms[i].size() >= 2 ? "m::add(a, c)" : "a") << ";\n";
        }
    }
};

const char* kHeaderNames[] = {"pk_args.h", "rk4_core.cuh"};

struct Cache {
    std::mutex mu;
    std::map<std::string, JitKernel> fwd;
    std::vector<cudaLibrary_t> libs;
};

Cache& cache() {
    static Cache* c = new Cache();   // intentionally leaked: libraries live until exit
    return *c;
}

// NVRTC: source -> sm_103a cubin (+ the compiler log when `log` is set).
bool to_cubin(const std::string& src, std::vector<char>* cubin, std::string* log, std::string* err) {
    nvrtcProgram prog;
    const char* headers[] = {pk_embedded::pk_args_h, pk_embedded::rk4_core_cuh};
    if (nvrtcCreateProgram(&prog, src.c_str(), "pasif_jit.cu", 2, headers, kHeaderNames) != NVRTC_SUCCESS) {
        *err = "nvrtcCreateProgram failed";
        return false;
    }
    const char* opts[] = {"-arch=sm_103a", "-std=c++17", "--fmad=false", "-lineinfo", "-DNDEBUG",
                          "--ptxas-options=-v"};
    nvrtcResult rc = nvrtcCompileProgram(prog, log ? 6 : 5, opts);
    size_t ls = 0;
    nvrtcGetProgramLogSize(prog, &ls);
    std::string text(ls, '\0');
    if (ls) nvrtcGetProgramLog(prog, &text[0]);
    while (!text.empty() && text.back() == '\0') text.pop_back();
    if (rc != NVRTC_SUCCESS) {
        *err = std::string("NVRTC compile failed: ") + nvrtcGetErrorString(rc) + "\n" + text;
        nvrtcDestroyProgram(&prog);
        return false;
    }
    if (log) *log = text;
    size_t cs = 0;
    nvrtcGetCUBINSize(prog, &cs);
    cubin->resize(cs);
    nvrtcGetCUBIN(prog, cubin->data());
    nvrtcDestroyProgram(&prog);
    return true;
}

bool compile(const std::string& src, const char* name, cudaKernel_t* fn, std::string* err) {
    std::vector<char> cubin;
    if (!to_cubin(src, &cubin, nullptr, err)) return false;
    cudaLibrary_t lib;
    cudaError_t ce = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (ce != cudaSuccess) {
        *err = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(ce);
        return false;
    }
    ce = cudaLibraryGetKernel(fn, lib, name);
    if (ce != cudaSuccess) {
        *err = std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(ce);
        return false;
    }
    cache().libs.push_back(lib);
    return true;
}

}  // namespace

std::string fwd_source(const Pattern& pat, const Literals& lit, const FwdKernelKey& key) {
    Emitter em(pat, lit);
    const int n = pat.n;
    std::ostringstream o;
    o << "// generated by pasif_gb300 jit.cpp: forward RK4, n=" << n << " P=" << pat.P() << "\n";
    o << "#include \"rk4_core.cuh\"\n";
    o << "namespace pk {\n";
    o << "typedef " << (key.f32 ? "float" : "double") << " R;\n";
    o << "struct JSys {\n";
    o << "  R p[" << (em.nload > 0 ? em.nload : 1) << "];\n";
    o << "  __device__ static constexpr int dim() { return " << n << "; }\n";
    o << "  __device__ __forceinline__ void load(const R* __restrict__ vals, long long B, int b) {\n";
    for (int q = 0; q < pat.P(); ++q)
        if (em.slot[q] >= 0) o << "    p[" << em.slot[q] << "] = vals[" << q << "LL * B + b];\n";
    o << "  }\n";
    o << "  template <bool FORCE, class V, class W, class F>\n";
    o << "  __device__ __forceinline__ void rhs(const V& xs, const W& xp, R u, F& f) const {\n";
    o << "    typedef M<R> m;\n    R a, c;\n";
    o << "    if (FORCE) {\n";
    em.rhs(o, true);
    o << "    } else {\n";
    em.rhs(o, false);
    o << "    }\n";
    o << "  }\n};\n";
    // forcing window and weights as compile-time constants
    const int W = key.window;
    o << "struct JW {\n  static constexpr int W = " << W << ";\n";
    for (int which = 0; which < 2; ++which) {
        o << "  __device__ static constexpr R " << (which ? "wc" : "wn") << "(int i) { return ";
        const std::vector<double>& wv = which ? key.wc : key.wn;
        for (int i = 0; i < W; ++i) o << "i == " << i << " ? " << hexlit(wv[i]) << " : ";
        o << "R(0); }\n";
    }
    o << "};\n}  // namespace pk\n";
    o << "extern \"C\" __global__ void __launch_bounds__(" << key.block << ") pk_fwd(pk::FwdArgs<pk::R> a) {\n";
    o << "  using namespace pk;\n";
    o << "  const int b = blockIdx.x * blockDim.x + threadIdx.x;\n";
    o << "  if (b >= a.B) return;\n";
    o << "  JSys sys;\n  sys.load(a.vals, (long long)a.B, b);\n";
    o << "  RegVec<R, " << n << "> Q, Cm, S, K, Mi, Mx;\n";
    o << "  fwd_run_iv<R, " << n << ", " << (key.kahan ? "true" : "false") << ", "
      << (key.max_mask ? "true" : "false") << ", " << (key.sq_mask ? "true" : "false") << ", "
      << (key.traj ? "true" : "false") << ", JW>(sys, a, b, "
      << key.max_mask << "ull, " << key.sq_mask << "ull, Q, Cm, S, K, Mi, Mx);\n";
    o << "}\n";
    return o.str();
}

bool fwd_compile_report(const Pattern& pat, const Literals& lit, const FwdKernelKey& key, std::string* report,
                        std::string* err) {
    std::vector<char> cubin;
    return to_cubin(fwd_source(pat, lit, key), &cubin, report, err);
}

namespace {

// JSys members shared by the forward and adjoint programs: values, load, rhs.
void emit_sys_head(std::ostringstream& o, const Pattern& pat, const Emitter& em, bool f32) {
    o << "#include \"rk4_core.cuh\"\n";
    o << "namespace pk {\n";
    o << "typedef " << (f32 ? "float" : "double") << " R;\n";
    o << "struct JSys {\n";
    o << "  R p[" << (em.nload > 0 ? em.nload : 1) << "];\n";
    o << "  __device__ static constexpr int dim() { return " << pat.n << "; }\n";
    o << "  __device__ __forceinline__ void load(const R* __restrict__ vals, long long B, int b) {\n";
    for (int q = 0; q < pat.P(); ++q)
        if (em.slot[q] >= 0) o << "    p[" << em.slot[q] << "] = vals[" << q << "LL * B + b];\n";
    o << "  }\n";
    o << "  template <bool FORCE, class V, class W, class F>\n";
    o << "  __device__ __forceinline__ void rhs(const V& xs, const W& xp, R u, F& f) const {\n";
    o << "    typedef M<R> m;\n    R a, c;\n";
    o << "    if (FORCE) {\n";
    em.rhs(o, true);
    o << "    } else {\n";
    em.rhs(o, false);
    o << "    }\n";
    o << "  }\n";
}

// VJP body in the operation order of GenSys::vjp (rk4_core.cuh).
void emit_vjp(std::ostringstream& o, const Pattern& pat, const Emitter& em) {
    const int n = pat.n;
    const int go = pat.k_nnz(), lo = go + pat.g_nnz(), po = lo + pat.l_nnz(), fo = po + pat.p_nnz();
    auto s = [](int v) { return std::to_string(v); };
    o << "  template <class V, class W, class O, class PB>\n";
    o << "  __device__ __forceinline__ void vjp(const V& y, const W& w, R u, O& out, PB& pb) const {\n";
    o << "    typedef M<R> m;\n";
    for (int i = 0; i < n; ++i) o << "    out[" << i << "] = R(0);\n";
    for (int i = 0; i < n; ++i)
        for (int q = pat.k_ptr[i]; q < pat.k_ptr[i + 1]; ++q) {
            const std::string j = s(pat.k_col[q]);
            o << "    out[" << j << "] = m::fma(" << em.val(q) << ", w[" << i << "], out[" << j << "]);\n";
            o << "    pacc_add(pb[" << q << "], w[" << i << "], y[" << j << "]);\n";
        }
    for (int e = 0; e < pat.g_nnz(); ++e) {
        const int* ix = &pat.g_idx[3 * e];
        const std::string i = s(ix[0]), j = s(ix[1]), k = s(ix[2]);
        o << "    { const R a_ = m::mul(" << em.val(go + e) << ", w[" << i << "]);\n";
        o << "      out[" << j << "] = m::fma(a_, y[" << k << "], out[" << j << "]);\n";
        o << "      out[" << k << "] = m::fma(a_, y[" << j << "], out[" << k << "]);\n";
        o << "      pacc_add(pb[" << go + e << "], m::mul(w[" << i << "], y[" << j << "]), y[" << k << "]); }\n";
    }
    for (int e = 0; e < pat.l_nnz(); ++e) {
        const int* ix = &pat.l_idx[4 * e];
        const std::string i = s(ix[0]), j = s(ix[1]), k = s(ix[2]), l = s(ix[3]);
        o << "    { const R a_ = m::mul(" << em.val(lo + e) << ", w[" << i << "]);\n";
        o << "      out[" << j << "] = m::fma(m::mul(a_, y[" << k << "]), y[" << l << "], out[" << j << "]);\n";
        o << "      out[" << k << "] = m::fma(m::mul(a_, y[" << j << "]), y[" << l << "], out[" << k << "]);\n";
        o << "      out[" << l << "] = m::fma(m::mul(a_, y[" << j << "]), y[" << k << "], out[" << l << "]);\n";
        o << "      pacc_add(pb[" << lo + e << "], m::mul(m::mul(w[" << i << "], y[" << j << "]), y[" << k
          << "]), y[" << l << "]); }\n";
    }
    for (int e = 0; e < pat.p_nnz(); ++e) {
        const int* ix = &pat.p_idx[5 * e];
        const std::string i = s(ix[0]), j = s(ix[1]), k = s(ix[2]), l = s(ix[3]), mm = s(ix[4]);
        o << "    { const R a_ = m::mul(" << em.val(po + e) << ", w[" << i << "]);\n";
        o << "      out[" << j << "] = m::fma(m::mul(m::mul(a_, y[" << k << "]), y[" << l << "]), y[" << mm << "], out["
          << j << "]);\n";
        o << "      out[" << k << "] = m::fma(m::mul(m::mul(a_, y[" << j << "]), y[" << l << "]), y[" << mm << "], out["
          << k << "]);\n";
        o << "      out[" << l << "] = m::fma(m::mul(m::mul(a_, y[" << j << "]), y[" << k << "]), y[" << mm << "], out["
          << l << "]);\n";
        o << "      out[" << mm << "] = m::fma(m::mul(m::mul(a_, y[" << j << "]), y[" << k << "]), y[" << l << "], out["
          << mm << "]);\n";
        o << "      pacc_add(pb[" << po + e << "], m::mul(m::mul(m::mul(w[" << i << "], y[" << j << "]), y[" << k
          << "]), y[" << l << "]), y[" << mm << "]); }\n";
    }
    for (int e = 0; e < pat.f_nnz(); ++e)
        o << "    pacc_add(pb[" << fo + e << "], w[" << pat.f_idx[e] << "], u);\n";
    o << "  }\n";
}

bool get_cached(const std::string& src, const char* name, int block, JitKernel* out, std::string* err) {
    Cache& c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    auto it = c.fwd.find(src);
    if (it != c.fwd.end()) {
        *out = it->second;
        return true;
    }
    JitKernel k;
    k.block = block;
    if (!compile(src, name, &k.fn, err)) return false;
    cudaFuncAttributes attr;
    if (cudaFuncGetAttributes(&attr, (const void*)k.fn) == cudaSuccess) {
        k.regs = attr.numRegs;
        k.local_bytes = (int)attr.localSizeBytes;
    }
    c.fwd[src] = k;
    *out = k;
    return true;
}

}  // namespace

bool compile_report(const std::string& src, std::string* report, std::string* err) {
    std::vector<char> cubin;
    return to_cubin(src, &cubin, report, err);
}

std::string adj_source(const Pattern& pat, const Literals& lit, bool f32, unsigned long long sq_mask) {
    Emitter em(pat, lit);
    std::ostringstream o;
    o << "// generated by pasif_gb300 jit.cpp: exact adjoint, n=" << pat.n << " P=" << pat.P() << "\n";
    emit_sys_head(o, pat, em, f32);
    emit_vjp(o, pat, em);
    o << "};\n}  // namespace pk\n";
    o << "extern \"C\" __global__ void __launch_bounds__(128) pk_adj(pk::AdjArgs<pk::R> a) {\n";
    o << "  using namespace pk;\n";
    o << "  const int b = blockIdx.x * blockDim.x + threadIdx.x;\n";
    o << "  if (b >= a.B) return;\n";
    o << "  JSys sys;\n  sys.load(a.vals, (long long)a.B, b);\n";
    const int P = pat.P() > 0 ? pat.P() : 1;
    if (f32) {
        o << "  RegVec<R, " << P << "> pacc;\n";
        o << "  adj_run_jit<R, " << pat.n << ", " << P << ", " << (sq_mask ? "true" : "false") << ", true>(sys, a, b, "
          << sq_mask << "ull, pacc);\n";
    } else {
        o << "  GVec<double> pacc{a.pbar + b, (long long)a.B};\n";
        o << "  adj_run_jit<R, " << pat.n << ", " << P << ", " << (sq_mask ? "true" : "false")
          << ", false>(sys, a, b, " << sq_mask << "ull, pacc);\n";
    }
    o << "}\n";
    return o.str();
}

std::string pool_source(const Pattern& pat, const FwdKernelKey& key) {
    Literals none;   // a pool's slots change owner: every value is loaded
    Emitter em(pat, none);
    std::ostringstream o;
    o << "// generated by pasif_gb300 jit.cpp: serving pool chunk, n=" << pat.n << " P=" << pat.P() << "\n";
    emit_sys_head(o, pat, em, key.f32);
    o << "};\n";
    const int W = key.window;
    o << "struct JW {\n  static constexpr int W = " << W << ";\n";
    for (int which = 0; which < 2; ++which) {
        o << "  __device__ static constexpr R " << (which ? "wc" : "wn") << "(int i) { return ";
        const std::vector<double>& wv = which ? key.wc : key.wn;
        for (int i = 0; i < W; ++i) o << "i == " << i << " ? " << hexlit(wv[i]) << " : ";
        o << "R(0); }\n";
    }
    o << "};\n}  // namespace pk\n";
    o << "extern \"C\" __global__ void __launch_bounds__(" << key.block << ") pk_pool(pk::PoolArgs<pk::R> p) {\n";
    o << "  using namespace pk;\n";
    o << "  const int b = blockIdx.x * blockDim.x + threadIdx.x;\n";
    o << "  if (b >= p.C) return;\n";
    o << "  if (p.remain[b] <= 0) return;\n";
    o << "  JSys sys;\n  sys.load(p.vals, (long long)p.C, b);\n";
    o << "  pool_run_iv<R, " << pat.n << ", " << (key.kahan ? "true" : "false") << ", "
      << (key.max_mask ? "true" : "false") << ", " << (key.sq_mask ? "true" : "false") << ", JW>(sys, p, b, "
      << key.max_mask << "ull, " << key.sq_mask << "ull);\n";
    o << "}\n";
    return o.str();
}

bool get_pool_kernel(const Pattern& pat, const FwdKernelKey& key, JitKernel* out, std::string* err) {
    if (pat.n <= 0 || pat.n > kJitMaxN) {
        *err = "state size outside the specialised range";
        return false;
    }
    return get_cached(pool_source(pat, key), "pk_pool", key.block, out, err);
}

bool get_adj_kernel(const Pattern& pat, const Literals& lit, bool f32, unsigned long long sq_mask, JitKernel* out,
                    std::string* err) {
    if (pat.n <= 0 || pat.n > kJitMaxN || pat.P() > 1024) {
        *err = "pattern outside the specialised range";
        return false;
    }
    return get_cached(adj_source(pat, lit, f32, sq_mask), "pk_adj", 128, out, err);
}

bool get_fwd_kernel(const Pattern& pat, const Literals& lit, const FwdKernelKey& key, JitKernel* out,
                    std::string* err) {
    if (pat.n <= 0 || pat.n > kJitMaxN) {
        *err = "state size outside the specialised range";
        return false;
    }
    const std::string src = fwd_source(pat, lit, key);
    Cache& c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    auto it = c.fwd.find(src);
    if (it != c.fwd.end()) {
        *out = it->second;
        return true;
    }
    JitKernel k;
    k.block = key.block;
    if (!compile(src, "pk_fwd", &k.fn, err)) return false;
    cudaFuncAttributes attr;
    if (cudaFuncGetAttributes(&attr, (const void*)k.fn) == cudaSuccess) {
        k.regs = attr.numRegs;
        k.local_bytes = (int)attr.localSizeBytes;
    }
    c.fwd[src] = k;
    *out = k;
    return true;
}

}  // namespace pasif
