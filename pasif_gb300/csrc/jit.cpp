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

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
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
    // extended-state mode: low parts of the values (loaded into q[], or
    // literals; a literal 0 drops the term from the low-part functions)
    bool ext = false;
    std::vector<int> slot_lo;
    int nload_lo = 0;

    Emitter(const Pattern& p, const Literals& l, bool ext_ = false) : pat(p), lit(l), ext(ext_) {
        const int P = pat.P();
        slot.assign(P, -1);
        slot_lo.assign(P, -1);
        for (int q = 0; q < P; ++q) {
            bool is_lit = q < (int)lit.is_lit.size() && lit.is_lit[q] && std::isfinite(lit.value[q]);
            if (!is_lit) slot[q] = nload++;
            if (ext && !lo_is_lit(l, q)) slot_lo[q] = nload_lo++;
        }
    }

    static bool lo_is_lit(const Literals& l, int q) {
        return q < (int)l.is_lit_lo.size() && l.is_lit_lo[q] && std::isfinite(l.value_lo[q]);
    }

    std::string val(int q) const {
        if (slot[q] >= 0) return "p[" + std::to_string(slot[q]) + "]";
        return hexlit(lit.value[q]);
    }

    // low part of value q ("" when it is the literal 0)
    std::string val_lo(int q) const {
        if (slot_lo[q] >= 0) return "q[" + std::to_string(slot_lo[q]) + "]";
        if (lit.value_lo[q] == 0.0) return "";
        return hexlit(lit.value_lo[q]);
    }

    // rhs body of the fast kernels (PASIF_PLAN_FAST): the products of state
    // components are formed once per evaluation and shared by every term that
    // uses them (operands sorted, built from the shared prefix), values 1 and
    // -1 fold into an add / subtract, each destination sums its terms in one
    // fma chain (two, added at the end, from four terms on), and the chains of
    // all destinations are emitted interleaved.  Not the canonical order: the
    // results differ from the oracle's in the last bits.
    void rhs_fast(std::ostringstream& o, bool force) const {
        const int n = pat.n;
        const int go = pat.k_nnz(), lo = go + pat.g_nnz(), po = lo + pat.l_nnz(), fo = po + pat.p_nnz();
        auto S = [](int v) { return std::to_string(v); };
        struct T { int q; std::vector<int> ops; bool force; };
        std::vector<std::vector<T>> terms(n);
        for (int i = 0; i < n; ++i)
            for (int q = pat.k_ptr[i]; q < pat.k_ptr[i + 1]; ++q) terms[i].push_back({q, {pat.k_col[q]}, false});
        for (int e = 0; e < pat.g_nnz(); ++e) {
            const int* ix = &pat.g_idx[3 * e];
            terms[ix[0]].push_back({go + e, {ix[1], ix[2]}, false});
        }
        for (int e = 0; e < pat.l_nnz(); ++e) {
            const int* ix = &pat.l_idx[4 * e];
            terms[ix[0]].push_back({lo + e, {ix[1], ix[2], ix[3]}, false});
        }
        for (int e = 0; e < pat.p_nnz(); ++e) {
            const int* ix = &pat.p_idx[5 * e];
            terms[ix[0]].push_back({po + e, {ix[1], ix[2], ix[3], ix[4]}, false});
        }
        if (force)
            for (int e = 0; e < pat.f_nnz(); ++e) terms[pat.f_idx[e]].push_back({fo + e, {}, true});
        std::map<std::vector<int>, std::string> mono;
        int nm = 0;
        std::function<std::string(const std::vector<int>&)> get = [&](const std::vector<int>& ops) -> std::string {
            if (ops.size() == 1) return "xs[" + S(ops[0]) + "]";
            auto it = mono.find(ops);
            if (it != mono.end()) return it->second;
            const std::string a = get(std::vector<int>(ops.begin(), ops.end() - 1));
            const std::string name = "mo" + S(nm++);
            o << "      const R " << name << " = m::mul(" << a << ", xs[" << S(ops.back()) << "]);\n";
            mono[ops] = name;
            return name;
        };
        // chains: (destination, chain index) -> the terms' (coefficient, monomial)
        struct Ch { int i, c; std::vector<std::pair<std::string, std::string>> t; };
        std::vector<Ch> chains;
        std::vector<int> nch(n, 0);
        for (int i = 0; i < n; ++i) {
            nch[i] = terms[i].size() >= 4 ? 2 : (terms[i].empty() ? 0 : 1);
            for (int c = 0; c < nch[i]; ++c) chains.push_back({i, c, {}});
        }
        for (int i = 0, base = 0; i < n; base += nch[i], ++i)
            for (size_t k = 0; k < terms[i].size(); ++k) {
                std::vector<int> ops = terms[i][k].ops;
                std::sort(ops.begin(), ops.end());
                const std::string m = terms[i][k].force ? "u" : get(ops);
                chains[base + (int)(k % (size_t)nch[i])].t.push_back({val(terms[i][k].q), m});
            }
        auto lit_is = [](const std::string& c, double v) { return c == hexlit(v); };
        size_t longest = 0;
        for (const Ch& c : chains) longest = std::max(longest, c.t.size());
        for (const Ch& c : chains) o << "      R c" << c.i << "_" << c.c << ";\n";
        for (size_t k = 0; k < longest; ++k)
            for (const Ch& c : chains) {
                if (k >= c.t.size()) continue;
                const std::string acc = "c" + S(c.i) + "_" + S(c.c);
                const std::string& co = c.t[k].first;
                const std::string& mo = c.t[k].second;
                if (k == 0) {
                    if (lit_is(co, 1.0)) o << "      " << acc << " = " << mo << ";\n";
                    else if (lit_is(co, -1.0)) o << "      " << acc << " = -" << mo << ";\n";
                    else o << "      " << acc << " = m::mul(" << co << ", " << mo << ");\n";
                } else {
                    if (lit_is(co, 1.0)) o << "      " << acc << " = m::add(" << acc << ", " << mo << ");\n";
                    else if (lit_is(co, -1.0)) o << "      " << acc << " = m::sub(" << acc << ", " << mo << ");\n";
                    else o << "      " << acc << " = m::fma(" << co << ", " << mo << ", " << acc << ");\n";
                }
            }
        for (int i = 0; i < n; ++i) {
            if (nch[i] == 0) o << "      f[" << i << "] = R(0);\n";
            else if (nch[i] == 1) o << "      f[" << i << "] = c" << i << "_0;\n";
            else o << "      f[" << i << "] = m::add(c" << i << "_0, c" << i << "_1);\n";
        }
    }

    // rhs_lo body: f = the right-hand side of the low parts of the values, one
    // fma chain per destination over the terms in canonical order (terms whose
    // low part is 0 contribute nothing and are left out).
    void rhs_lo(std::ostringstream& o) const {
        const int n = pat.n;
        const int go = pat.k_nnz(), lo = go + pat.g_nnz(), po = lo + pat.l_nnz(), fo = po + pat.p_nnz();
        std::vector<std::vector<std::pair<std::string, std::string>>> terms(n);
        auto S = [](int v) { return std::to_string(v); };
        for (int i = 0; i < n; ++i)
            for (int q = pat.k_ptr[i]; q < pat.k_ptr[i + 1]; ++q)
                if (!val_lo(q).empty()) terms[i].push_back({val_lo(q), "xs[" + S(pat.k_col[q]) + "]"});
        for (int e = 0; e < pat.g_nnz(); ++e) {
            const int* ix = &pat.g_idx[3 * e];
            if (val_lo(go + e).empty()) continue;
            terms[ix[0]].push_back({"m::mul(" + val_lo(go + e) + ", xs[" + S(ix[1]) + "])", "xp[" + S(ix[2]) + "]"});
        }
        for (int e = 0; e < pat.l_nnz(); ++e) {
            const int* ix = &pat.l_idx[4 * e];
            if (val_lo(lo + e).empty()) continue;
            terms[ix[0]].push_back({"m::mul(m::mul(" + val_lo(lo + e) + ", xs[" + S(ix[1]) + "]), xp[" + S(ix[2]) +
                                        "])",
                                    "xp[" + S(ix[3]) + "]"});
        }
        for (int e = 0; e < pat.p_nnz(); ++e) {
            const int* ix = &pat.p_idx[5 * e];
            if (val_lo(po + e).empty()) continue;
            terms[ix[0]].push_back({"m::mul(m::mul(m::mul(" + val_lo(po + e) + ", xs[" + S(ix[1]) + "]), xp[" +
                                        S(ix[2]) + "]), xp[" + S(ix[3]) + "])",
                                    "xp[" + S(ix[4]) + "]"});
        }
        for (int e = 0; e < pat.f_nnz(); ++e)
            if (!val_lo(fo + e).empty()) terms[pat.f_idx[e]].push_back({val_lo(fo + e), "u"});
        for (int i = 0; i < n; ++i) {
            if (terms[i].empty()) {
                o << "    f[" << i << "] = R(0);\n";
                continue;
            }
            for (size_t k = 0; k < terms[i].size(); ++k) {
                if (k == 0)
                    o << "    f[" << i << "] = m::mul(" << terms[i][k].first << ", " << terms[i][k].second << ");\n";
                else
                    o << "    f[" << i << "] = m::fma(" << terms[i][k].first << ", " << terms[i][k].second << ", f["
                      << i << "]);\n";
            }
        }
    }

    // rhs body of the packed-FP32 forward kernels (thread per system, FP32,
    // forward only: xs and xp are the same vector).  The operations and their
    // order per destination are those of rhs() below -- the oracle's bits --
    // but destinations 2m and 2m+1 are evaluated together: the k-th operation
    // of a partial sum of one and the k-th of the same partial sum of the
    // other become one f32x2 instruction (mul.rn / fma.rn / add.rn.f32x2, two
    // independent correctly rounded results), as do the multiplications
    // forming the terms' first factors, level by level.  What has no partner
    // (a longer partial sum, a deeper product) stays scalar.  A value that is
    // exactly 1 or -1 folds: 1*x = x, fma(1, x, s) = s + x, fma(-1, x, s) =
    // s - x, all exact, so the bits do not change.
    void rhs_pair(std::ostringstream& o, bool force) const {
        const int n = pat.n;
        const int go = pat.k_nnz(), lo = go + pat.g_nnz(), po = lo + pat.l_nnz(), fo = po + pat.p_nnz();
        auto S = [](int v) { return std::to_string(v); };
        struct T { std::string v; std::vector<int> ops; };   // value, state factors (none: the forcing term)
        std::vector<std::vector<T>> terms(n);
        for (int i = 0; i < n; ++i)
            for (int q = pat.k_ptr[i]; q < pat.k_ptr[i + 1]; ++q) terms[i].push_back({val(q), {pat.k_col[q]}});
        for (int e = 0; e < pat.g_nnz(); ++e) {
            const int* ix = &pat.g_idx[3 * e];
            terms[ix[0]].push_back({val(go + e), {ix[1], ix[2]}});
        }
        for (int e = 0; e < pat.l_nnz(); ++e) {
            const int* ix = &pat.l_idx[4 * e];
            terms[ix[0]].push_back({val(lo + e), {ix[1], ix[2], ix[3]}});
        }
        for (int e = 0; e < pat.p_nnz(); ++e) {
            const int* ix = &pat.p_idx[5 * e];
            terms[ix[0]].push_back({val(po + e), {ix[1], ix[2], ix[3], ix[4]}});
        }
        if (force)
            for (int e = 0; e < pat.f_nnz(); ++e) terms[pat.f_idx[e]].push_back({val(fo + e), {}});
        const std::string one = hexlit(1.0), mone = hexlit(-1.0);
        auto X = [&](int c) { return "xs[" + S(c) + "]"; };
        auto last_of = [&](const T& t) { return t.ops.empty() ? std::string("u") : X(t.ops.back()); };
        auto depth = [](const T& t) { return t.ops.empty() ? 0 : (int)t.ops.size() - 1; };
        // scalar first factor of t from level `from` on, given the factor so far
        auto scalar_first = [&](const T& t, int from, std::string f) {
            for (int l = from; l < depth(t); ++l) {
                if (f == one) f = X(t.ops[l]);
                else if (f == mone) f = "(-" + X(t.ops[l]) + ")";
                else f = "m::mul(" + f + ", " + X(t.ops[l]) + ")";
            }
            return f;
        };
        // scalar operation k of a partial sum held in `acc`
        auto scalar_op = [&](const std::string& acc, size_t k, const std::string& f, const std::string& l) {
            if (k == 0) {
                if (f == one) return acc + " = " + l + ";\n";
                if (f == mone) return acc + " = -" + l + ";\n";
                return acc + " = m::mul(" + f + ", " + l + ");\n";
            }
            if (f == one) return acc + " = m::add(" + acc + ", " + l + ");\n";
            if (f == mone) return acc + " = m::sub(" + acc + ", " + l + ");\n";
            return acc + " = m::fma(" + f + ", " + l + ", " + acc + ");\n";
        };
        auto P2 = [](const std::string& a, const std::string& b) { return "make_float2(" + a + ", " + b + ")"; };
        int nf = 0;
        for (int i = 0; i < n; i += 2) {
            const int j = i + 1;
            if (j >= n || terms[i].empty() || terms[j].empty()) {   // no partner: the scalar form
                for (int d = i; d < std::min(n, i + 2); ++d) {
                    if (terms[d].empty()) {
                        o << "      f[" << d << "] = R(0);\n";
                        continue;
                    }
                    o << "      {\n        R a" << (terms[d].size() >= 2 ? ", c" : "") << ";\n";
                    for (size_t k = 0; k < terms[d].size(); ++k) {
                        const T& t = terms[d][k];
                        o << "        " << scalar_op((k & 1) ? "c" : "a", k / 2, scalar_first(t, 0, t.v), last_of(t));
                    }
                    o << "        f[" << d << "] = " << (terms[d].size() >= 2 ? "m::add(a, c)" : "a") << ";\n      }\n";
                }
                continue;
            }
            const size_t ni = terms[i].size(), nj = terms[j].size();
            o << "      {\n        float2 pa" << (std::max(ni, nj) >= 2 ? ", pc" : "") << ";\n";
            for (size_t k = 0; k < std::max(ni, nj); ++k) {
                const std::string acc = (k & 1) ? "pc" : "pa";
                const size_t pos = k / 2;
                if (k < ni && k < nj) {
                    const T& ti = terms[i][k];
                    const T& tj = terms[j][k];
                    std::string fi = ti.v, fj = tj.v;
                    const int common = std::min(depth(ti), depth(tj));
                    for (int l = 0; l < common; ++l) {
                        if (fi == one && fj == one) {
                            fi = X(ti.ops[l]);
                            fj = X(tj.ops[l]);
                            continue;
                        }
                        const std::string nm = "ff" + S(nf++);
                        o << "        const float2 " << nm << " = M2::mul(" << P2(fi, fj) << ", "
                          << P2(X(ti.ops[l]), X(tj.ops[l])) << ");\n";
                        fi = nm + ".x";
                        fj = nm + ".y";
                    }
                    fi = scalar_first(ti, common, fi);
                    fj = scalar_first(tj, common, fj);
                    const std::string L = P2(last_of(ti), last_of(tj));
                    if (pos == 0) {
                        // ptxas may contract a packed multiply with a packed or scalar add that
                        // consumes it into one fma (rounding once instead of twice), whatever
                        // the rounding modifiers: a packed product is only used as the addend
                        // of the partial sum's next packed fma; otherwise two scalar products.
                        const bool next_fma2 = k + 2 < ni && k + 2 < nj &&
                                               !(depth(terms[i][k + 2]) == 0 && depth(terms[j][k + 2]) == 0 &&
                                                 terms[i][k + 2].v == terms[j][k + 2].v &&
                                                 (terms[i][k + 2].v == one || terms[i][k + 2].v == mone));
                        if (fi == one && fj == one) o << "        " << acc << " = " << L << ";\n";
                        else if (next_fma2) o << "        " << acc << " = M2::mul(" << P2(fi, fj) << ", " << L << ");\n";
                        else {
                            auto prod = [&](const std::string& f, const std::string& l) {
                                return f == one ? l : f == mone ? "(-" + l + ")" : "m::mul(" + f + ", " + l + ")";
                            };
                            o << "        " << acc << " = " << P2(prod(fi, last_of(ti)), prod(fj, last_of(tj))) << ";\n";
                        }
                    } else {
                        if (fi == one && fj == one) o << "        " << acc << " = M2::add(" << acc << ", " << L << ");\n";
                        else if (fi == mone && fj == mone) o << "        " << acc << " = M2::sub(" << acc << ", " << L << ");\n";
                        else o << "        " << acc << " = M2::fma(" << P2(fi, fj) << ", " << L << ", " << acc << ");\n";
                    }
                } else {   // only one destination has a k-th term
                    const T& t = k < ni ? terms[i][k] : terms[j][k];
                    const std::string lane = acc + (k < ni ? ".x" : ".y");
                    o << "        " << scalar_op(lane, pos, scalar_first(t, 0, t.v), last_of(t));
                }
            }
            if (ni >= 2 && nj >= 2) {
                o << "        const float2 r = M2::add(pa, pc);\n";
                o << "        f[" << i << "] = r.x;\n        f[" << j << "] = r.y;\n";
            } else {
                o << "        f[" << i << "] = " << (ni >= 2 ? "m::add(pa.x, pc.x)" : "pa.x") << ";\n";
                o << "        f[" << j << "] = " << (nj >= 2 ? "m::add(pa.y, pc.y)" : "pa.y") << ";\n";
            }
            o << "      }\n";
        }
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
    std::vector<const char*> opts = {"-arch=sm_103a", "-std=c++17", "--fmad=false", "-lineinfo", "-DNDEBUG"};
    // tuning override: one extra compiler option (e.g. a ptxas option)
    const char* extra = std::getenv("PASIF_NVRTC_OPT");
    if (extra && *extra) opts.push_back(extra);
    if (log) opts.push_back("--ptxas-options=-v");
    nvrtcResult rc = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
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

bool compile(const std::string& src, const char* name, cudaKernel_t* fn, cudaLibrary_t* lib, std::string* err) {
    std::vector<char> cubin;
    if (!to_cubin(src, &cubin, nullptr, err)) return false;
    cudaError_t ce = cudaLibraryLoadData(lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (ce != cudaSuccess) {
        *err = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(ce);
        return false;
    }
    ce = cudaLibraryGetKernel(fn, *lib, name);
    if (ce != cudaSuccess) {
        *err = std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(ce);
        cudaLibraryUnload(*lib);
        return false;
    }
    return true;
}


// ---- warp-sliced kernels ------------------------------------------------------

struct Term {
    int q;        // value index
    int kind;     // 0 K, 1 Gamma, 2 Lambda, 3 Psi, 4 forcing
    int ops[4];   // state operands in product order (kind + 1 of them; none for forcing)
};

// Terms of every destination in the canonical order: K row, Gamma, Lambda,
// Psi, forcing (the order Emitter::rhs and Pattern::flat use).
std::vector<std::vector<Term>> dest_terms(const Pattern& pat) {
    const int go = pat.k_nnz(), lo = go + pat.g_nnz(), po = lo + pat.l_nnz(), fo = po + pat.p_nnz();
    std::vector<std::vector<Term>> t(pat.n);
    for (int i = 0; i < pat.n; ++i)
        for (int q = pat.k_ptr[i]; q < pat.k_ptr[i + 1]; ++q) t[i].push_back({q, 0, {pat.k_col[q], 0, 0, 0}});
    for (int e = 0; e < pat.g_nnz(); ++e) {
        const int* ix = &pat.g_idx[3 * e];
        t[ix[0]].push_back({go + e, 1, {ix[1], ix[2], 0, 0}});
    }
    for (int e = 0; e < pat.l_nnz(); ++e) {
        const int* ix = &pat.l_idx[4 * e];
        t[ix[0]].push_back({lo + e, 2, {ix[1], ix[2], ix[3], 0}});
    }
    for (int e = 0; e < pat.p_nnz(); ++e) {
        const int* ix = &pat.p_idx[5 * e];
        t[ix[0]].push_back({po + e, 3, {ix[1], ix[2], ix[3], ix[4]}});
    }
    for (int e = 0; e < pat.f_nnz(); ++e) t[pat.f_idx[e]].push_back({fo + e, 4, {0, 0, 0, 0}});
    return t;
}

struct Slicing {
    int L = 0;
    std::vector<int> owner, local, pub;      // per component (pub: -1 = not published)
    std::vector<std::vector<int>> own;       // per slice: components in local order
    int NP = 0;
    int sq_owner = 0;
};

// Whether the first half of the states are displacements whose derivative is
// the matching velocity alone (x_i' = x_{n/2+i}, the first-order form of a
// mechanical system).
bool velocity_form(int n, const std::vector<std::vector<Term>>& dt) {
    if (n < 4 || (n & 1)) return false;
    for (int i = 0; i < n / 2; ++i)
        if (dt[i].size() != 1 || dt[i][0].kind != 0 || dt[i][0].ops[0] != n / 2 + i) return false;
    return true;
}

// Components ordered by reverse Cuthill-McKee on the interaction graph, cut
// into L contiguous runs of about equal work, so that strongly coupled
// components share a warp and few values cross warps.
// dof_pairs (patterns in velocity form): the pairs (x_i, x_{n/2+i}) in DOF
// order, cut into L runs of equal size, so that the interior slices of a
// banded or chained system are translates of one another.
Slicing make_slicing(const Pattern& pat, const std::vector<std::vector<Term>>& dt, int L, unsigned long long sq_mask,
                     bool adjoint, bool dof_pairs = false) {
    const int n = pat.n;
    std::vector<std::vector<int>> adj(n);
    std::vector<double> wt(n, 4.0);
    for (int i = 0; i < n; ++i)
        for (const Term& t : dt[i]) {
            wt[i] += 2.0 + (t.kind < 4 ? t.kind : 0);
            for (int k = 0; k < (t.kind < 4 ? t.kind + 1 : 0); ++k) {
                const int j = t.ops[k];
                if (j != i) { adj[i].push_back(j); adj[j].push_back(i); }
            }
        }
    for (auto& a : adj) {
        std::sort(a.begin(), a.end());
        a.erase(std::unique(a.begin(), a.end()), a.end());
    }
    std::vector<int> order, seen(n, 0);
    while ((int)order.size() < n) {
        int start = -1;
        for (int i = 0; i < n; ++i)
            if (!seen[i] && (start < 0 || adj[i].size() < adj[start].size())) start = i;
        seen[start] = 1;
        size_t head = order.size();
        order.push_back(start);
        while (head < order.size()) {
            const int v = order[head++];
            std::vector<int> nb;
            for (int u : adj[v])
                if (!seen[u]) { seen[u] = 1; nb.push_back(u); }
            std::stable_sort(nb.begin(), nb.end(), [&](int x, int y) { return adj[x].size() < adj[y].size(); });
            order.insert(order.end(), nb.begin(), nb.end());
        }
    }
    std::reverse(order.begin(), order.end());
    const bool by_dof = dof_pairs && velocity_form(n, dt);
    if (by_dof) {
        order.clear();
        for (int i = 0; i < n / 2; ++i) {
            order.push_back(i);
            order.push_back(n / 2 + i);
        }
    }
    double total = 0.0;
    for (double w : wt) total += w;
    Slicing s;
    s.owner.assign(n, 0);
    std::vector<std::vector<int>> runs(L);
    double cum = 0.0;
    for (size_t r = 0; r < order.size(); ++r) {
        const int v = order[r];
        int k = by_dof ? (int)(r / 2 * L / (order.size() / 2)) : (int)((cum + 0.5 * wt[v]) * L / total);
        k = std::max(0, std::min(L - 1, k));
        runs[k].push_back(v);
        cum += wt[v];
    }
    for (auto& r : runs)
        if (!r.empty()) s.own.push_back(r);
    s.L = (int)s.own.size();
    s.local.assign(n, 0);
    for (int w = 0; w < s.L; ++w)
        for (int k = 0; k < (int)s.own[w].size(); ++k) {
            s.owner[s.own[w][k]] = w;
            s.local[s.own[w][k]] = k;
        }
    // the lightest slice sums the squares (it reads the others' components)
    double best = 1e300;
    for (int w = 0; w < s.L; ++w) {
        double sw = 0.0;
        for (int v : s.own[w]) sw += wt[v];
        if (sw < best) { best = sw; s.sq_owner = w; }
    }
    std::vector<char> need(n, 0);
    for (int i = 0; i < n; ++i)
        for (const Term& t : dt[i]) {
            const int no = t.kind < 4 ? t.kind + 1 : 0;
            for (int k = 0; k < no; ++k)
                if (s.owner[t.ops[k]] != s.owner[i]) need[t.ops[k]] = 1;
            if (adjoint) {   // the VJP owner of an operand reads the term's weight and its other operands
                for (int k = 0; k < no; ++k) {
                    const int ok = s.owner[t.ops[k]];
                    if (ok != s.owner[i]) need[i] = 1;
                    for (int z = 0; z < no; ++z)
                        if (s.owner[t.ops[z]] != ok) need[t.ops[z]] = 1;
                }
            }
        }
    for (int i = 0; i < n && i < 64; ++i)
        if (((sq_mask >> i) & 1ull) && s.owner[i] != s.sq_owner) need[i] = 1;
    s.pub.assign(n, -1);
    for (int i = 0; i < n; ++i)
        if (need[i]) s.pub[i] = s.NP++;
    return s;
}

// Slices whose structs are translates of one another share one struct.
// Each slice's struct text comes with hooks \x01 <kind> <value> \x02 for
// its slice-dependent numbers (ws_source): component indices (N), published
// offsets (P), offsets of the compensated gradient totals (G), ranks of the
// max-tracked components (R), all of which must move by one constant per
// kind from slice to slice, and value indices (Q), which may move
// arbitrarily.  Slices with the same text apart from the hooks, and constant
// moves, form a group: one struct (the first member's), whose N/P/G/R
// numbers become runtime bases plus the first member's numbers and whose Q
// numbers are read from a per-warp table.  The warps of a group then run
// the same instructions: with one struct per warp the SM's instruction
// cache does not hold the code of all the warps of a block (GB300, 128-state
// chain adjoint, 8 warps: 13 "no instruction" stalls per issued
// instruction).  The operations are unchanged.
struct SliceGroup {
    int ref = 0;
    std::vector<int> members;
    std::vector<std::array<long long, 4>> shift;   // per member: N, P, G, R
    std::vector<std::vector<long long>> q;          // per member: the Q numbers in text order
};

std::vector<SliceGroup> share_slices(const std::vector<std::string>& src, std::ostringstream& o) {
    struct Code { std::string tmpl; std::vector<std::pair<char, long long>> hooks; };
    std::vector<Code> code(src.size());
    for (size_t w = 0; w < src.size(); ++w) {
        const std::string& t = src[w];
        for (size_t i = 0; i < t.size(); ++i) {
            if (t[i] != '\x01') { code[w].tmpl += t[i]; continue; }
            const size_t j = t.find('\x02', i);
            code[w].hooks.push_back({t[i + 1], std::stoll(t.substr(i + 2, j - i - 2))});
            code[w].tmpl += '\x01';
            code[w].tmpl += t[i + 1];
            i = j;
        }
    }
    auto kind_index = [](char k) { return k == 'N' ? 0 : k == 'P' ? 1 : k == 'G' ? 2 : k == 'R' ? 3 : -1; };
    bool share = true;
    if (const char* e = std::getenv("PASIF_WS_SHARE")) share = std::atoi(e) != 0;   // tuning override
    std::vector<SliceGroup> groups;
    for (int w = 0; w < (int)src.size(); ++w) {
        bool placed = false;
        for (SliceGroup& g : groups) {
            if (!share) break;
            const Code& r = code[g.ref];
            if (r.tmpl != code[w].tmpl) continue;
            std::array<long long, 4> sh{};
            std::array<bool, 4> set{};
            std::vector<long long> qv;
            bool ok = true;
            for (size_t h = 0; h < r.hooks.size() && ok; ++h) {
                const int k = kind_index(r.hooks[h].first);
                const long long d = code[w].hooks[h].second - r.hooks[h].second;
                if (k < 0) { qv.push_back(code[w].hooks[h].second); continue; }
                if (!set[k]) { set[k] = true; sh[k] = d; }
                else ok = sh[k] == d;
            }
            if (!ok) continue;
            g.members.push_back(w);
            g.shift.push_back(sh);
            g.q.push_back(qv);
            placed = true;
            break;
        }
        if (placed) continue;
        SliceGroup g;
        g.ref = w;
        g.members.push_back(w);
        g.shift.push_back({0, 0, 0, 0});
        std::vector<long long> qv;
        for (const auto& hk : code[w].hooks)
            if (kind_index(hk.first) < 0) qv.push_back(hk.second);
        g.q.push_back(qv);
        groups.push_back(g);
    }
    for (const SliceGroup& g : groups) {
        const Code& c = code[g.ref];
        const bool shared = g.members.size() > 1;
        const std::string name = "SL" + std::to_string(g.ref);
        size_t h = 0, qi = 0;
        std::string body;
        for (size_t i = 0; i < c.tmpl.size(); ++i) {
            const char ch = c.tmpl[i];
            if (ch == '\x03') { body += name; continue; }
            if (ch == '\x04') {
                if (shared) body += "  long long nb_ = 0; int pb_ = 0, gb_ = 0, rb_ = 0; const int* qt_ = nullptr;\n";
                continue;
            }
            if (ch != '\x01') { body += ch; continue; }
            const char kind = c.tmpl[++i];
            const long long v = c.hooks[h++].second;
            if (!shared) { body += std::to_string(v); continue; }
            switch (kind) {
                case 'N': body += "(nb_ + " + std::to_string(v) + ")"; break;
                case 'P': body += "(pb_ + " + std::to_string(v) + ")"; break;
                case 'G': body += "(gb_ + " + std::to_string(v) + ")"; break;
                case 'R': body += "(rb_ + " + std::to_string(v) + ")"; break;
                default: body += "qt_[" + std::to_string(qi++) + "]"; break;
            }
        }
        o << body;
        if (!shared) continue;
        // per-warp bases and value indices of the group's members (other rows unused)
        const int L = (int)src.size();
        const size_t nq = std::max<size_t>(g.q[0].size(), 1);
        o << "__device__ const long long " << name << "_NB[" << L << "] = {";
        for (int w = 0; w < L; ++w) {
            long long v = 0;
            for (size_t m = 0; m < g.members.size(); ++m)
                if (g.members[m] == w) v = g.shift[m][0];
            o << (w ? ", " : "") << v;
        }
        o << "};\n";
        o << "__device__ const int " << name << "_PGR[" << L << "][3] = {";
        for (int w = 0; w < L; ++w) {
            std::array<long long, 4> sh{};
            for (size_t m = 0; m < g.members.size(); ++m)
                if (g.members[m] == w) sh = g.shift[m];
            o << (w ? ", " : "") << "{" << sh[1] << ", " << sh[2] << ", " << sh[3] << "}";
        }
        o << "};\n";
        o << "__device__ const int " << name << "_QT[" << L << "][" << nq << "] = {";
        for (int w = 0; w < L; ++w) {
            const std::vector<long long>* qv = nullptr;
            for (size_t m = 0; m < g.members.size(); ++m)
                if (g.members[m] == w) qv = &g.q[m];
            o << (w ? ", " : "") << "{";
            for (size_t k = 0; k < nq; ++k) o << (k ? ", " : "") << (qv && k < qv->size() ? (*qv)[k] : 0);
            o << "}";
        }
        o << "};\n";
    }
    return groups;
}

std::string ws_source_impl(const Pattern& pat, const Literals& lit, const FwdKernelKey& key, int mode, int roll_force,
                           int* distinct, int dof_force = -1);

// Text that identifies a pattern's structure (memo keys).
std::string pattern_key(const Pattern& pat) {
    std::ostringstream k;
    k << pat.n << ':';
    for (const std::vector<int>* v : {&pat.k_ptr, &pat.k_col, &pat.g_idx, &pat.l_idx, &pat.p_idx, &pat.f_idx}) {
        for (int x : *v) k << x << ',';
        k << ';';
    }
    return k.str();
}

// Cut by displacement/velocity pairs (make_slicing's dof_pairs) where the
// default cut into L warps gives mostly distinct slices and this one gives at
// most L/2 distinct structs: a banded 32-DOF system (64 states) cut into 8
// warps has 8 distinct slices in the default order, 3 by pairs (the two ends
// and one shared interior struct).  Decided on the FP32 source with values
// loaded at run time, memoised per pattern.
bool ws_by_dof(const Pattern& pat, const std::vector<std::vector<Term>>& dt, int L, bool adjoint) {
    if (L < 4 || !velocity_form(pat.n, dt) || std::getenv("PASIF_WS_RCM")) return false;
    static std::mutex mu;
    static std::map<std::string, bool> memo;
    const std::string mk = pattern_key(pat) + (adjoint ? "a" : "f") + std::to_string(L);
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = memo.find(mk);
        if (it != memo.end()) return it->second;
    }
    FwdKernelKey key;
    key.f32 = true;
    key.kahan = true;
    key.slices = L;
    int d0 = 0, d1 = 0;
    ws_source_impl(pat, Literals(), key, adjoint ? 2 : 0, 0, &d0, 0);
    bool dof = false;
    if (2 * d0 > L) {
        ws_source_impl(pat, Literals(), key, adjoint ? 2 : 0, 0, &d1, 1);
        dof = 2 * d1 <= L;
    }
    std::lock_guard<std::mutex> g(mu);
    memo[mk] = dof;
    return dof;
}

// Source of the warp-sliced forward (mode 0: pk_fwd over FwdArgs), serving-
// pool (mode 1: pk_pool over PoolArgs) or exact-adjoint (mode 2: pk_adj over
// AdjArgs) kernel.
// roll_force: -1 = the rule below, 0 / 1 = unrolled / rolled stages.
// *distinct: number of distinct slice structs after share_slices.
std::string ws_source_impl(const Pattern& pat, const Literals& lit, const FwdKernelKey& key, int mode, int roll_force,
                           int* distinct, int dof_force) {
    const int n = pat.n;
    const bool adj = mode == 2;
    const auto dt = dest_terms(pat);
    const bool by_dof = dof_force >= 0 ? dof_force == 1 : ws_by_dof(pat, dt, key.slices, adj);
    const Slicing sl = make_slicing(pat, dt, key.slices, adj ? 0ull : key.sq_mask, adj, by_dof);
    auto S = [](long long v) { return std::to_string(v); };
    // every term in the global order of the VJP scatter (GenSys::vjp): K rows, Gamma, Lambda, Psi, forcing
    std::vector<std::pair<int, Term>> scatter;   // (destination, term)
    if (adj) {
        for (int kind = 0; kind <= 4; ++kind)
            for (int i = 0; i < n; ++i)
                for (const Term& t : dt[i])
                    if (t.kind == kind) scatter.push_back({i, t});
        std::stable_sort(scatter.begin(), scatter.end(), [](const std::pair<int, Term>& x, const std::pair<int, Term>& y) {
            return x.second.kind != y.second.kind ? x.second.kind < y.second.kind
                                                  : (x.second.kind == 0 ? x.first < y.first : x.second.q < y.second.q);
        });
    }
    // rolled stages when the slices are large (instruction cache), unrolled otherwise
    size_t terms = 0;
    for (const auto& t : dt) terms += t.size();
    // Forward, 4 warps: 16-state chain slices of ~22 terms 1.4x faster unrolled;
    // 32-, 64-state slices of 43-88 terms 1.2-2x faster rolled.  Adjoint (measured
    // gradient rates): 16-state chain 1.2x faster unrolled, 32- and 64-state chains
    // and the 64-state banded system 1.0-1.5x faster rolled, 128-state chain 1.35x
    // faster unrolled.
    bool roll = adj ? (n > 24 && n <= 96) : (double)terms / sl.L >= 30.0;
    if (roll_force >= 0) roll = roll_force != 0;
    if (const char* e = std::getenv("PASIF_WS_ROLL")) roll = std::atoi(e) != 0;   // tuning override
    std::ostringstream o;
    o << "// generated by pasif_gb300 jit.cpp: warp-sliced "
      << (mode == 0 ? "forward" : mode == 1 ? "serving pool" : "exact adjoint") << (key.ext ? " extended state" : "")
      << " RK4, n=" << n
      << " P=" << pat.P() << " slices=" << sl.L << " published=" << sl.NP << " rolled=" << (roll ? 1 : 0) << "\n";
    o << "#include \"rk4_core.cuh\"\nnamespace pk {\n";
    o << "typedef " << (key.f32 ? "float" : "double") << " R;\n";
    // Each slice's struct is first written with its slice-dependent indices as
    // hooks (share_slices): component indices (N), published offsets (P),
    // value indices (Q), offsets of the compensated gradient totals (G) and
    // ranks of the max-tracked components (R).
    std::vector<std::string> slice_src(sl.L);
    long long pk_off = 0;   // gradient totals: slice after slice, 64 floats per value
    auto H = [](char kind, long long v) { return std::string(1, '\x01') + kind + std::to_string(v) + '\x02'; };
    for (int w = 0; w < sl.L; ++w) {
        std::ostringstream slice_text;
        std::ostringstream& o = slice_text;
        const std::vector<int>& own = sl.own[w];
        const int MM = (int)own.size();
        auto mine = [&](int j) { return sl.owner[j] == w; };
        // values this slice reads: loaded slots (absent = literal)
        std::map<int, int> slot;
        auto need_val = [&](int q) {
            const bool is_lit = q < (int)lit.is_lit.size() && lit.is_lit[q] && std::isfinite(lit.value[q]);
            if (!is_lit && !slot.count(q)) {
                const int k = (int)slot.size();
                slot[q] = k;
            }
        };
        // extended-state mode: low parts of the same values (literal 0: the term drops out)
        std::map<int, int> slot_lo;
        auto need_lo = [&](int q) {
            if (!key.ext || Emitter::lo_is_lit(lit, q) || slot_lo.count(q)) return;
            const int k = (int)slot_lo.size();
            slot_lo[q] = k;
        };
        auto val_lo = [&](int q) -> std::string {
            if (slot_lo.count(q)) return "q[" + S(slot_lo[q]) + "]";
            if (lit.value_lo[q] == 0.0) return "";
            return hexlit(lit.value_lo[q]);
        };
        bool forced = false;
        std::vector<int> foreign, pown;   // pown: values of own destinations' terms (gradients kept here)
        for (int i : own)
            for (const Term& t : dt[i]) {
                need_val(t.q);
                need_lo(t.q);
                pown.push_back(t.q);
                if (t.kind == 4) forced = true;
                for (int k = 0; k < (t.kind < 4 ? t.kind + 1 : 0); ++k)
                    if (!mine(t.ops[k])) foreign.push_back(t.ops[k]);
            }
        std::vector<int> yforeign, wforeign;   // VJP: other operands and weights of terms that touch own components
        if (adj)
            for (const auto& it : scatter) {
                const Term& t = it.second;
                const int no = t.kind < 4 ? t.kind + 1 : 0;
                bool touches = mine(it.first);
                for (int k = 0; k < no; ++k) touches = touches || mine(t.ops[k]);
                if (!touches) continue;
                need_val(t.q);
                need_lo(t.q);
                if (!mine(it.first)) wforeign.push_back(it.first);
                for (int k = 0; k < no; ++k)
                    if (!mine(t.ops[k])) yforeign.push_back(t.ops[k]);
            }
        for (auto* v : {&foreign, &yforeign, &wforeign}) {
            std::sort(v->begin(), v->end());
            v->erase(std::unique(v->begin(), v->end()), v->end());
        }
        std::map<int, int> pslot;   // in the order the terms are visited
        for (int q : pown) pslot[q] = (int)pslot.size();
        std::vector<int> pq(pslot.size());
        for (auto& kv : pslot) pq[kv.second] = kv.first;
        // local names of the foreign operands: the same text for slices that are
        // translates of each other
        std::map<int, int> fx, fy, fw;
        for (int j : foreign) fx[j] = (int)fx.size();
        for (int j : yforeign) fy[j] = (int)fy.size();
        for (int i : wforeign) fw[i] = (int)fw.size();
        auto val = [&](int q) { return slot.count(q) ? "p[" + S(slot[q]) + "]" : hexlit(lit.value[q]); };
        auto x = [&](int j) { return mine(j) ? "X[" + S(sl.local[j]) + "]" : "x" + S(fx.at(j)); };
        o << "struct \x03 {\n\x04";
        o << "  static constexpr int MM = " << MM << ", NP = " << sl.NP << ", PO = " << std::max<size_t>(pown.size(), 1)
          << ";\n";
        o << "  static constexpr bool FORCED = " << (forced ? "true" : "false")
          << ", SQOWN = " << (w == sl.sq_owner ? "true" : "false") << ", ROLL = " << (roll ? "true" : "false")
          << ";\n";
        o << "  R p[" << std::max<size_t>(slot.size(), 1) << "];\n";
        if (key.ext) o << "  R q[" << std::max<size_t>(slot_lo.size(), 1) << "];   // low parts of the values\n";
        o << "  __device__ __forceinline__ void load(const R* __restrict__ vals, long long B, int b) {\n";
        {
            std::vector<int> qs(slot.size()), ql(slot_lo.size());
            for (auto& kv : slot) qs[kv.second] = kv.first;
            for (auto& kv : slot_lo) ql[kv.second] = kv.first;
            for (size_t k = 0; k < qs.size(); ++k)
                o << "    p[" << k << "] = vals[(long long)" << H('Q', qs[k]) << " * B + b];\n";
            for (size_t k = 0; k < ql.size(); ++k)
                o << "    q[" << k << "] = vals[(long long)" << H('Q', pat.P() + ql[k]) << " * B + b];\n";
        }
        o << "  }\n";
        o << "  template <class V> __device__ __forceinline__ void load_vec(V& X, const R* __restrict__ src, long long B,"
             " int b) const {\n";
        for (int k = 0; k < MM; ++k) o << "    X[" << k << "] = src[(long long)" << H('N', own[k]) << " * B + b];\n";
        o << "  }\n";
        o << "  __device__ __forceinline__ void prefetch_vec(const R* src, long long B, int b) const {\n";
        for (int k = 0; k < MM; ++k) o << "    pk_prefetch_l2(src + (long long)" << H('N', own[k]) << " * B + b);\n";
        o << "  }\n";
        o << "  template <class V> __device__ __forceinline__ void store_vec(const V& X, R* dst, long long B, int b)"
             " const {\n";
        for (int k = 0; k < MM; ++k) o << "    dst[(long long)" << H('N', own[k]) << " * B + b] = X[" << k << "];\n";
        o << "  }\n";
        o << "  template <class V> __device__ __forceinline__ void store_traj(const V& X, R* dst, long long B, int b)"
             " const { store_vec(X, dst, B, b); }\n";
        o << "  template <class V> __device__ __forceinline__ void publish(const V& X, R* buf) const {\n";
        for (int k = 0; k < MM; ++k)
            if (sl.pub[own[k]] >= 0) o << "    buf[" << H('P', sl.pub[own[k]] * 32) << "] = X[" << k << "];\n";
        o << "  }\n";
        o << "  template <class V> __device__ __forceinline__ void track_max(const V& X, V& Mx) const {\n";
        for (int k = 0; k < MM; ++k)
            if (own[k] < 64 && ((key.max_mask >> own[k]) & 1ull))
                o << "    Mx[" << k << "] = M<R>::max(Mx[" << k << "], M<R>::abs(X[" << k << "]));\n";
        o << "  }\n";
        o << "  template <class V> __device__ __forceinline__ void store_max(const V& Mx, R* out, long long B, int b)"
             " const {\n";
        {
            int rank = 0;
            for (int i = 0; i < n && i < 64; ++i)
                if ((key.max_mask >> i) & 1ull) {
                    if (sl.owner[i] == w) o << "    out[(long long)" << H('R', rank) << " * B + b] = Mx[" << sl.local[i] << "];\n";
                    ++rank;
                }
        }
        o << "  }\n";
        o << "  template <bool KAHAN, class V> __device__ __forceinline__ void add_sq(const V& X, const R* buf, R& sq,"
             " R& sqc) const {\n";
        if (w == sl.sq_owner) {
            o << "    typedef M<R> m;\n";
            for (int i = 0; i < n && i < 64; ++i)
                if ((key.sq_mask >> i) & 1ull) {
                    const std::string q = sl.owner[i] == w ? "X[" + S(sl.local[i]) + "]" : "buf[" + H('P', sl.pub[i] * 32) + "]";
                    o << "    { const R q = " << q << ";\n";
                    o << "      if (KAHAN) { const R y = m::sub(m::mul(q, q), sqc); const R t = m::add(sq, y);"
                         " sqc = m::sub(m::sub(t, sq), y); sq = t; } else { sq = m::fma(q, q, sq); } }\n";
                }
        }
        o << "  }\n";
        o << "  template <class V, class F> __device__ __forceinline__ void rhs(const V& X, const R* buf, R u, F& f)"
             " const {\n";
        o << "    typedef M<R> m;\n    R a, c;\n";
        for (int j : foreign) o << "    const R x" << fx.at(j) << " = buf[" << H('P', sl.pub[j] * 32) << "];\n";
        for (int k = 0; k < MM; ++k) {
            const int i = own[k];
            const std::vector<Term>& ts = dt[i];
            if (ts.empty()) {
                o << "    f[" << k << "] = R(0);\n";
                continue;
            }
            for (size_t e = 0; e < ts.size(); ++e) {
                const Term& t = ts[e];
                std::string first, last;
                if (t.kind == 4) {
                    first = val(t.q);
                    last = "u";
                } else {
                    first = val(t.q);
                    for (int z = 0; z < t.kind; ++z) first = "m::mul(" + first + ", " + x(t.ops[z]) + ")";
                    last = x(t.ops[t.kind]);
                }
                const char* acc = (e & 1) ? "c" : "a";
                if (e < 2) o << "    " << acc << " = m::mul(" << first << ", " << last << ");\n";
                else o << "    " << acc << " = m::fma(" << first << ", " << last << ", " << acc << ");\n";
            }
            o << "    f[" << k << "] = " << (ts.size() >= 2 ? "m::add(a, c)" : "a") << ";\n";
        }
        o << "  }\n";
        if (key.ext) {   // right-hand side of the low parts: one fma chain per destination
            o << "  template <class V, class F> __device__ __forceinline__ void rhs_lo(const V& X, const R* buf, R u,"
                 " F& f) const {\n";
            o << "    typedef M<R> m;\n";
            std::vector<int> used;
            for (int i : own)
                for (const Term& t : dt[i])
                    if (!val_lo(t.q).empty())
                        for (int k = 0; k < (t.kind < 4 ? t.kind + 1 : 0); ++k)
                            if (!mine(t.ops[k])) used.push_back(t.ops[k]);
            std::sort(used.begin(), used.end());
            used.erase(std::unique(used.begin(), used.end()), used.end());
            for (int j : used) o << "    const R x" << fx.at(j) << " = buf[" << H('P', sl.pub[j] * 32) << "];\n";
            for (int k = 0; k < MM; ++k) {
                int cnt = 0;
                for (const Term& t : dt[own[k]]) {
                    const std::string v = val_lo(t.q);
                    if (v.empty()) continue;
                    std::string first, last;
                    if (t.kind == 4) {
                        first = v;
                        last = "u";
                    } else {
                        first = v;
                        for (int z = 0; z < t.kind; ++z) first = "m::mul(" + first + ", " + x(t.ops[z]) + ")";
                        last = x(t.ops[t.kind]);
                    }
                    if (cnt == 0) o << "    f[" << k << "] = m::mul(" << first << ", " << last << ");\n";
                    else o << "    f[" << k << "] = m::fma(" << first << ", " << last << ", f[" << k << "]);\n";
                    ++cnt;
                }
                if (cnt == 0) o << "    f[" << k << "] = R(0);\n";
            }
            o << "    (void)u;\n  }\n";
        }
        if (adj) {
            auto W = [&](int i) { return mine(i) ? "W[" + S(sl.local[i]) + "]" : "w" + S(fw.at(i)); };
            auto Y = [&](int j) { return mine(j) ? "Y[" + S(sl.local[j]) + "]" : "y" + S(fy.at(j)); };
            auto out = [&](int j) { return "out[" + S(sl.local[j]) + "]"; };
            o << "  template <class V, class PA> __device__ __forceinline__ void vjp(const V& Y, const R* yb, const V& W,"
                 " const R* wb, R u, V& out, PA& pacc) const {\n";
            o << "    typedef M<R> m;\n";
            for (int j : yforeign) o << "    const R y" << fy.at(j) << " = yb[" << H('P', sl.pub[j] * 32) << "];\n";
            for (int i : wforeign) o << "    const R w" << fw.at(i) << " = wb[" << H('P', sl.pub[i] * 32) << "];\n";
            for (int k = 0; k < MM; ++k) o << "    out[" << k << "] = R(0);\n";
            for (const auto& it : scatter) {
                const int i = it.first;
                const Term& t = it.second;
                const int no = t.kind < 4 ? t.kind + 1 : 0;
                bool any = false;
                for (int k = 0; k < no; ++k) any = any || mine(t.ops[k]);
                const std::string ps = mine(i) ? "pacc[" + S(pslot[t.q]) + "]" : "";
                if (t.kind == 0) {
                    const int j = t.ops[0];
                    if (mine(j)) o << "    " << out(j) << " = m::fma(" << val(t.q) << ", " << W(i) << ", " << out(j) << ");\n";
                    if (mine(i)) o << "    pacc_add(" << ps << ", " << W(i) << ", " << Y(j) << ");\n";
                } else if (t.kind == 4) {
                    if (mine(i)) o << "    pacc_add(" << ps << ", " << W(i) << ", u);\n";
                } else {
                    if (any) {
                        o << "    { const R a_ = m::mul(" << val(t.q) << ", " << W(i) << ");\n";
                        for (int k = 0; k < no; ++k) {
                            const int j = t.ops[k];
                            if (!mine(j)) continue;
                            // product of the other operands in operand order; the last one is the fma factor
                            std::vector<int> oth;
                            for (int z = 0; z < no; ++z)
                                if (z != k) oth.push_back(t.ops[z]);
                            std::string f = "a_";
                            for (size_t z = 0; z + 1 < oth.size(); ++z) f = "m::mul(" + f + ", " + Y(oth[z]) + ")";
                            o << "      " << out(j) << " = m::fma(" << f << ", " << Y(oth.back()) << ", " << out(j)
                              << ");\n";
                        }
                        o << "    }\n";
                    }
                    if (mine(i)) {
                        std::string f = W(i);
                        for (int z = 0; z + 1 < no; ++z) f = "m::mul(" + f + ", " + Y(t.ops[z]) + ")";
                        o << "    pacc_add(" << ps << ", " << f << ", " << Y(t.ops[no - 1]) << ");\n";
                    }
                }
            }
            o << "  }\n";
            if (key.ext) {   // J_lo^T W in the scatter order of vjp, no parameter gradients
                o << "  template <class V> __device__ __forceinline__ void vjp_lo(const V& Y, const R* yb, const V& W,"
                     " const R* wb, R u, V& out) const {\n";
                o << "    typedef M<R> m;\n";
                for (int j : yforeign) o << "    const R y" << fy.at(j) << " = yb[" << H('P', sl.pub[j] * 32) << "];\n";
                for (int i : wforeign) o << "    const R w" << fw.at(i) << " = wb[" << H('P', sl.pub[i] * 32) << "];\n";
                for (int k = 0; k < MM; ++k) o << "    out[" << k << "] = R(0);\n";
                for (const auto& it : scatter) {
                    const int i = it.first;
                    const Term& t = it.second;
                    const int no = t.kind < 4 ? t.kind + 1 : 0;
                    const std::string v = val_lo(t.q);
                    if (v.empty() || t.kind == 4) continue;
                    if (t.kind == 0) {
                        const int j = t.ops[0];
                        if (mine(j)) o << "    " << out(j) << " = m::fma(" << v << ", " << W(i) << ", " << out(j) << ");\n";
                        continue;
                    }
                    bool any = false;
                    for (int k = 0; k < no; ++k) any = any || mine(t.ops[k]);
                    if (!any) continue;
                    o << "    { const R a_ = m::mul(" << v << ", " << W(i) << ");\n";
                    for (int k = 0; k < no; ++k) {
                        const int j = t.ops[k];
                        if (!mine(j)) continue;
                        std::vector<int> oth;
                        for (int z = 0; z < no; ++z)
                            if (z != k) oth.push_back(t.ops[z]);
                        std::string f = "a_";
                        for (size_t z = 0; z + 1 < oth.size(); ++z) f = "m::mul(" + f + ", " + Y(oth[z]) + ")";
                        o << "      " << out(j) << " = m::fma(" << f << ", " << Y(oth.back()) << ", " << out(j) << ");\n";
                    }
                    o << "    }\n";
                }
                o << "    (void)u;\n  }\n";
            }
            o << "  template <bool KAHAN, bool EXT, class V> __device__ __forceinline__ void add_sq_grad(V& LAM, V& CL,"
                 " const V& QN, R g) const {\n";
            for (int k = 0; k < MM; ++k)
                if (own[k] < 64 && ((key.sq_mask >> own[k]) & 1ull))
                    o << "    if (EXT) ext_add(LAM[" << k << "], CL[" << k << "], M<R>::mul(g, QN[" << k
                      << "])); else if (KAHAN) kahan_add(LAM[" << k << "], CL[" << k << "], M<R>::mul(g, QN[" << k
                      << "])); else LAM[" << k << "] = M<R>::fma(g, QN[" << k << "], LAM[" << k << "]);\n";
            o << "  }\n";
            o << "  template <class PV> __device__ __forceinline__ void store_pbar(const PV& PB, double* pbar, long long B,"
                 " int b) const {\n";
            for (size_t k = 0; k < pq.size(); ++k) o << "    pbar[(long long)" << H('Q', pq[k]) << " * B + b] = PB[" << k << "];\n";
            o << "  }\n";
            o << "  template <class PV> __device__ __forceinline__ void load_pbar(PV& PB, const double* pbar, long long B,"
                 " int b) const {\n";
            for (size_t k = 0; k < pq.size(); ++k) o << "    PB[" << k << "] = pbar[(long long)" << H('Q', pq[k]) << " * B + b];\n";
            o << "  }\n";
            o << "  __device__ __forceinline__ void zero_pbar(double* pbar, long long B, int b) const {\n";
            for (size_t k = 0; k < pq.size(); ++k) o << "    pbar[(long long)" << H('Q', pq[k]) << " * B + b] = 0.0;\n";
            o << "  }\n";
            // FP32 compensated per-chunk totals in shared memory, slice after
            // slice: the k-th value's sum at pk[64 (off + k)], its compensation
            // 32 floats further (pk holds the lane)
            auto PS = [&](size_t k) { return H('G', 64 * (pk_off + (long long)k)); };
            auto PC = [&](size_t k) { return H('G', 64 * (pk_off + (long long)k) + 32); };
            o << "  template <class PV> __device__ __forceinline__ void add_pk(const PV& ps, R* pk) const {\n";
            for (size_t k = 0; k < pq.size(); ++k)
                o << "    { R s_ = pk[" << PS(k) << "], c_ = pk[" << PC(k) << "]; kahan_add(s_, c_, ps[" << k
                  << "]); pk[" << PS(k) << "] = s_; pk[" << PC(k) << "] = c_; }\n";
            o << "  }\n";
            o << "  template <bool EXT> __device__ __forceinline__ void flush_pk(R* pk, double* pbar, long long B,"
                 " int b, double s) const {\n";
            for (size_t k = 0; k < pq.size(); ++k) {
                const std::string pb = "pbar[(long long)" + H('Q', pq[k]) + " * B + b]";
                o << "    { const double t_ = (double)pk[" << PS(k) << "] - (double)pk[" << PC(k) << "]; " << pb
                  << " = EXT ? M<double>::fma(s, t_, " << pb << ") : " << pb << " + t_; pk[" << PS(k)
                  << "] = R(0); pk[" << PC(k) << "] = R(0); }\n";
            }
            o << "  }\n";
            o << "  __device__ __forceinline__ void zero_pk(R* pk) const {\n";
            for (size_t k = 0; k < pq.size(); ++k) o << "    pk[" << PS(k) << "] = R(0); pk[" << PC(k) << "] = R(0);\n";
            o << "  }\n";
        }
        o << "};\n";
        slice_src[w] = slice_text.str();
        pk_off += (long long)pq.size();
    }
    const std::vector<SliceGroup> groups = share_slices(slice_src, o);
    if (distinct) *distinct = (int)groups.size();
    o << "}  // namespace pk\n";
    const std::string ext = key.ext ? "true" : "false";
    const std::string kahan = key.kahan ? "true" : "false", hmax = key.max_mask ? "true" : "false",
                      hsq = key.sq_mask ? "true" : "false", htraj = std::to_string(key.traj);
    const char* sig = mode == 0 ? "pk_fwd(pk::FwdArgs<pk::R> a)" : mode == 1 ? "pk_pool(pk::PoolArgs<pk::R> p)"
                                                                            : "pk_adj(pk::AdjArgs<pk::R> a)";
    o << "extern \"C\" __global__ void __launch_bounds__(" << 32 * sl.L << ") " << sig << " {\n";
    o << "  using namespace pk;\n";
    o << "  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;\n";
    o << "  const long long bb = (long long)blockIdx.x * 32 + lane;\n";
    o << "  const long long cnt = " << (mode == 1 ? "p.C" : "a.B") << ";\n";
    o << "  const bool valid = bb < cnt;\n";
    o << "  const int b = valid ? (int)bb : (int)cnt - 1;\n";
    o << "  R* sm = reinterpret_cast<R*>(pk_dyn_smem()) + lane;\n";
    std::ostringstream call;
    if (mode == 1)
        call << "ws_pool<R, " << kahan << ", " << hmax << ", " << hsq << ", " << n << ">(sl, p, sm, b, valid, w);";
    else if (mode == 0)
        call << "ws_fwd<R, " << kahan << ", " << hmax << ", " << hsq << ", " << htraj << ", " << n << ", " << ext
             << ">(sl, a, sm, b, valid);";
    else   // the Kahan mode of the forward passes is the plan's (AdjArgs::kahan)
        call << "ws_adj<R, " << kahan << ", " << hsq << ", " << (key.f32 ? "true" : "false") << ", " << n << ", " << ext
             << ">(sl, a, sm, b, valid);";
    o << "  switch (w) {\n";
    for (const SliceGroup& g : groups) {
        const std::string name = "SL" + std::to_string(g.ref);
        o << "   ";
        for (int m : g.members) o << " case " << m << ":";
        o << " { " << name << " sl; ";
        if (g.members.size() > 1)
            o << "sl.nb_ = " << name << "_NB[w]; sl.pb_ = " << name << "_PGR[w][0]; sl.gb_ = " << name
              << "_PGR[w][1]; sl.rb_ = " << name << "_PGR[w][2]; sl.qt_ = " << name << "_QT[w]; ";
        o << call.str() << " } break;\n";
    }
    o << "    default: break;\n  }\n}\n";
    // FP32 adjoint with a slice holding more than 16 values: their compensated
    // gradient totals in shared memory (ws_adj, PKREG false), 64 floats per value
    size_t max_po = 0;
    if (adj && key.f32) {
        const auto dt2 = dest_terms(pat);
        for (int w = 0; w < sl.L; ++w) {
            size_t po = 0;
            for (int i : sl.own[w]) po += dt2[i].size();
            max_po = std::max(max_po, po);
        }
    }
    const long long pk_floats = max_po > 16 ? 64LL * std::max<long long>(pat.P(), pk_off) : 0;
    o << "// ws-launch " << 32 * sl.L << " " << ((adj ? 6 : 2) * sl.NP * 32 + pk_floats) * (key.f32 ? 4 : 8)
      << "\n";
    return o.str();
}

// Warp-sliced kernel source.  Where most slices share one struct
// (share_slices) the stages are unrolled: with the warps of a block running
// the same code the instruction cache holds it (GB300, FP32-Kahan, 4096
// systems: 32-DOF chain adjoint, 16 warps, 1.0e9 adjoint system-steps/s
// unrolled vs 7.9e8 rolled; 16-DOF chain adjoint, 8 warps, 1.89e9 vs 1.46e9).
std::string ws_source(const Pattern& pat, const Literals& lit, const FwdKernelKey& key, int mode) {
    int distinct = 0;
    std::string src = ws_source_impl(pat, lit, key, mode, -1, &distinct);
    const bool rolled = src.find(" rolled=1") != std::string::npos;
    if (rolled && 2 * distinct <= key.slices && !std::getenv("PASIF_WS_ROLL"))
        src = ws_source_impl(pat, lit, key, mode, 0, &distinct);
    return src;
}

// Whether the slices of `pat` cut into L warps are translates of one
// another for the most part (at most L/2 distinct structs).
bool ws_shareable(const Pattern& pat, int L, bool adjoint) {
    FwdKernelKey key;
    key.f32 = true;
    key.kahan = true;
    key.slices = L;
    int distinct = 0;
    ws_source_impl(pat, Literals(), key, adjoint ? 2 : 0, 0, &distinct);
    return 2 * distinct <= L;
}

// Launch shape recorded by ws_source on its last line.
void ws_launch(const std::string& src, int* block, int* smem) {
    const size_t at = src.rfind("// ws-launch ");
    *block = 128;
    *smem = 0;
    if (at != std::string::npos) std::sscanf(src.c_str() + at, "// ws-launch %d %d", block, smem);
}

}  // namespace

// The thread's shared-memory ring of upcoming excitation samples (JW::ring):
// with one or two steps per sample interval (W <= 4) and a short step, a
// sample read one interval ahead leaves every step waiting for memory, so
// samples are copied asynchronously (cp.async) RING - 1 intervals before they
// are used.  Measured on GB300: 1024 one-DOF systems (86 FLOP per step, one
// sample per step from a 410 MB table) 3.5e9 -> 1.5e10 system-steps/s; 4096
// 16-state chains (644 FLOP per step), whose steps already cover the read,
// 9.2e9 -> 3.9e9, so longer steps keep the register read-ahead.
static void emit_sample_ring(std::ostringstream& o, int W, int block, const Pattern& pat) {
    const int spi = W == 0 ? 1 : W / 2;
    const long long flops = 4LL * (2 * pat.k_nnz() + 3 * pat.g_nnz() + 4 * pat.l_nnz() + 5 * pat.p_nnz() +
                                   2 * pat.f_nnz() + 3) + 13LL * pat.n;
    const int ring = spi <= 2 && flops <= 200 ? 16 : 0;
    o << "  static constexpr int RING = " << ring << ", RS = " << block << ";\n";
    if (ring)
        o << "  __device__ static R* ring() { __shared__ R r[" << ring * block << "]; return r + threadIdx.x; }\n";
    else
        o << "  __device__ static R* ring() { return nullptr; }\n";
}

namespace {
void emit_sys_head(std::ostringstream& o, const Pattern& pat, const Emitter& em, bool f32, bool fast = false,
                   bool pair = false);
}

// Packed-FP32 (f32x2) form of the thread-per-system forward (rk4_step's
// PAIR): 0 = scalar, 1 = packed stages with a scalar compensated update,
// 2 = packed update too; the bits are the same in every form.  Chosen from
// GB300 measurements of the forward (16384 systems; scalar -> packed):
// plain FP32 gains wherever a destination pair 2m, 2m+1 has work on both
// sides (2-DOF coupled +45 %, 4-DOF chain +17 %); with the compensated update
// only small dense systems gain (2-DOF coupled, n = 5, two coupled rows of 8
// terms: +13.5 %), spring chains lose (n = 4, 8, 16: -3 to -19 %: their rows
// pair with shifted columns, so most packed operands must be assembled), so
// compensated forwards are packed only for n <= 6 with a destination pair of
// at least 4 terms on each side.  The extended-state mode follows the
// compensated one (2-DOF coupled: packed stages +2 %, packed double-float
// update +5 % more).  PASIF_FP32X2 overrides the choice (tuning).
int fwd_paired(const Pattern& pat, const FwdKernelKey& key) {
    if (!key.f32 || key.fast || key.slices >= 2) return 0;
    std::vector<int> cnt(pat.n, 0);
    for (int i = 0; i < pat.n; ++i) cnt[i] = pat.k_ptr[i + 1] - pat.k_ptr[i];
    for (int e = 0; e < pat.g_nnz(); ++e) ++cnt[pat.g_idx[3 * e]];
    for (int e = 0; e < pat.l_nnz(); ++e) ++cnt[pat.l_idx[4 * e]];
    for (int e = 0; e < pat.p_nnz(); ++e) ++cnt[pat.p_idx[5 * e]];
    int both = 0, dense = 0;
    for (int i = 0; i + 1 < pat.n; i += 2) {
        both += cnt[i] > 0 && cnt[i + 1] > 0;
        dense += cnt[i] >= 4 && cnt[i + 1] >= 4;
    }
    if (both == 0) return 0;
    int mode = (!key.kahan && !key.ext) ? 2 : (pat.n <= 6 && dense > 0) ? 2 : 0;
    if (const char* e = std::getenv("PASIF_FP32X2")) mode = std::max(0, std::min(2, std::atoi(e)));
    return mode;
}

std::string fwd_source(const Pattern& pat, const Literals& lit, const FwdKernelKey& key) {
    if (key.slices >= 2) return ws_source(pat, lit, key, 0);
    Emitter em(pat, lit, key.ext);
    const int n = pat.n;
    const int pair = fwd_paired(pat, key);
    std::ostringstream o;
    o << "// generated by pasif_gb300 jit.cpp: forward RK4, n=" << n << " P=" << pat.P()
      << (key.ext ? " extended state" : "") << (key.fast ? " fast" : "") << (pair ? " packed FP32" : "") << "\n";
    emit_sys_head(o, pat, em, key.f32, key.fast, pair > 0);
    o << "};\n";
    // forcing window and weights as compile-time constants
    const int W = key.window;
    o << "struct JW {\n  static constexpr int W = " << W << ";\n";
    o << "  static constexpr bool FAST = " << (key.fast ? "true" : "false") << ";\n";
    o << "  static constexpr int PAIR = " << pair << ";\n";
    emit_sample_ring(o, W, key.block, pat);
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
      << key.traj << ", JW, " << (key.ext ? "true" : "false") << ">(sys, a, b, "
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
void emit_sys_head(std::ostringstream& o, const Pattern& pat, const Emitter& em, bool f32, bool fast, bool pair) {
    o << "#include \"rk4_core.cuh\"\n";
    o << "namespace pk {\n";
    o << "typedef " << (f32 ? "float" : "double") << " R;\n";
    o << "struct JSys {\n";
    o << "  R p[" << (em.nload > 0 ? em.nload : 1) << "];\n";
    if (em.ext) o << "  R q[" << (em.nload_lo > 0 ? em.nload_lo : 1) << "];   // low parts of the values\n";
    o << "  __device__ static constexpr int dim() { return " << pat.n << "; }\n";
    o << "  __device__ __forceinline__ void load(const R* __restrict__ vals, long long B, int b) {\n";
    for (int q = 0; q < pat.P(); ++q)
        if (em.slot[q] >= 0) o << "    p[" << em.slot[q] << "] = vals[" << q << "LL * B + b];\n";
    for (int q = 0; q < pat.P(); ++q)
        if (em.ext && em.slot_lo[q] >= 0)
            o << "    q[" << em.slot_lo[q] << "] = vals[" << (pat.P() + q) << "LL * B + b];\n";
    o << "  }\n";
    if (em.ext) {
        o << "  template <bool FORCE, class V, class W, class F>\n";
        o << "  __device__ __forceinline__ void rhs_lo(const V& xs, const W& xp, R u, F& f) const {\n";
        o << "    typedef M<R> m;\n";
        em.rhs_lo(o);
        o << "  }\n";
    }
    o << "  template <bool FORCE, class V, class W, class F>\n";
    o << "  __device__ __forceinline__ void rhs(const V& xs, const W& xp, R u, F& f) const {\n";
    if (pair) {   // packed-FP32 forward: xs and xp are the same vector
        o << "    typedef M<R> m;\n    (void)xp;\n";
        o << "    if (FORCE) {\n";
        em.rhs_pair(o, true);
        o << "    } else {\n";
        em.rhs_pair(o, false);
        o << "    }\n";
        o << "  }\n";
        return;
    }
    if (fast) {   // forward systems only: xs and xp are the same vector
        o << "    typedef M<R> m;\n    (void)xp;\n";
        o << "    if (FORCE) {\n";
        em.rhs_fast(o, true);
        o << "    } else {\n";
        em.rhs_fast(o, false);
        o << "    }\n";
        o << "  }\n";
        return;
    }
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

// vjp_lo: out = J_lo(y)^T w, the transposed Jacobian of the low parts of the
// values, in the scatter order of emit_vjp (no parameter gradients; terms
// whose low part is 0 are left out).
void emit_vjp_lo(std::ostringstream& o, const Pattern& pat, const Emitter& em) {
    const int n = pat.n;
    const int go = pat.k_nnz(), lo = go + pat.g_nnz(), po = lo + pat.l_nnz();
    auto s = [](int v) { return std::to_string(v); };
    o << "  template <class V, class W, class O>\n";
    o << "  __device__ __forceinline__ void vjp_lo(const V& y, const W& w, R u, O& out) const {\n";
    o << "    typedef M<R> m;\n";
    for (int i = 0; i < n; ++i) o << "    out[" << i << "] = R(0);\n";
    for (int i = 0; i < n; ++i)
        for (int q = pat.k_ptr[i]; q < pat.k_ptr[i + 1]; ++q) {
            if (em.val_lo(q).empty()) continue;
            const std::string j = s(pat.k_col[q]);
            o << "    out[" << j << "] = m::fma(" << em.val_lo(q) << ", w[" << i << "], out[" << j << "]);\n";
        }
    for (int e = 0; e < pat.g_nnz(); ++e) {
        if (em.val_lo(go + e).empty()) continue;
        const int* ix = &pat.g_idx[3 * e];
        const std::string i = s(ix[0]), j = s(ix[1]), k = s(ix[2]);
        o << "    { const R a_ = m::mul(" << em.val_lo(go + e) << ", w[" << i << "]);\n";
        o << "      out[" << j << "] = m::fma(a_, y[" << k << "], out[" << j << "]);\n";
        o << "      out[" << k << "] = m::fma(a_, y[" << j << "], out[" << k << "]); }\n";
    }
    for (int e = 0; e < pat.l_nnz(); ++e) {
        if (em.val_lo(lo + e).empty()) continue;
        const int* ix = &pat.l_idx[4 * e];
        const std::string i = s(ix[0]), j = s(ix[1]), k = s(ix[2]), l = s(ix[3]);
        o << "    { const R a_ = m::mul(" << em.val_lo(lo + e) << ", w[" << i << "]);\n";
        o << "      out[" << j << "] = m::fma(m::mul(a_, y[" << k << "]), y[" << l << "], out[" << j << "]);\n";
        o << "      out[" << k << "] = m::fma(m::mul(a_, y[" << j << "]), y[" << l << "], out[" << k << "]);\n";
        o << "      out[" << l << "] = m::fma(m::mul(a_, y[" << j << "]), y[" << k << "], out[" << l << "]); }\n";
    }
    for (int e = 0; e < pat.p_nnz(); ++e) {
        if (em.val_lo(po + e).empty()) continue;
        const int* ix = &pat.p_idx[5 * e];
        const std::string i = s(ix[0]), j = s(ix[1]), k = s(ix[2]), l = s(ix[3]), mm = s(ix[4]);
        o << "    { const R a_ = m::mul(" << em.val_lo(po + e) << ", w[" << i << "]);\n";
        o << "      out[" << j << "] = m::fma(m::mul(m::mul(a_, y[" << k << "]), y[" << l << "]), y[" << mm << "], out["
          << j << "]);\n";
        o << "      out[" << k << "] = m::fma(m::mul(m::mul(a_, y[" << j << "]), y[" << l << "]), y[" << mm << "], out["
          << k << "]);\n";
        o << "      out[" << l << "] = m::fma(m::mul(m::mul(a_, y[" << j << "]), y[" << k << "]), y[" << mm << "], out["
          << l << "]);\n";
        o << "      out[" << mm << "] = m::fma(m::mul(m::mul(a_, y[" << j << "]), y[" << k << "]), y[" << l << "], out["
          << mm << "]); }\n";
    }
    o << "    (void)u;\n  }\n";
}

// The cache lock is not held while NVRTC compiles (up to a second for a large
// pattern): the host threads of a server keep launching cached kernels while
// another thread compiles a new one.  Two threads compiling the same source
// both load it; the first to finish is the one kept.
bool get_cached(const std::string& src, const char* name, int block, JitKernel* out, std::string* err) {
    Cache& c = cache();
    {
        std::lock_guard<std::mutex> lk(c.mu);
        auto it = c.fwd.find(src);
        if (it != c.fwd.end()) {
            *out = it->second;
            return true;
        }
    }
    JitKernel k;
    k.block = block;
    k.per_block = block;
    if (src.find("// ws-launch ") != std::string::npos) {
        ws_launch(src, &k.block, &k.smem);
        k.per_block = 32;
    }
    cudaLibrary_t lib;
    if (!compile(src, name, &k.fn, &lib, err)) return false;
    if (k.smem > 48 * 1024) {
        cudaError_t ce = cudaFuncSetAttribute((const void*)k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, k.smem);
        if (ce != cudaSuccess) {
            *err = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(ce);
            cudaLibraryUnload(lib);
            return false;
        }
    }
    cudaFuncAttributes attr;
    if (cudaFuncGetAttributes(&attr, (const void*)k.fn) == cudaSuccess) {
        k.regs = attr.numRegs;
        k.local_bytes = (int)attr.localSizeBytes;
    }
    std::lock_guard<std::mutex> lk(c.mu);
    // loaded for the life of the process, the copy of a compile that another
    // thread finished first too (unloading a module may wait for the device,
    // which would stall the other threads' streams)
    c.libs.push_back(lib);
    auto it = c.fwd.find(src);
    if (it != c.fwd.end()) {
        *out = it->second;
        return true;
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

std::string adj_source(const Pattern& pat, const Literals& lit, bool f32, unsigned long long sq_mask, int slices,
                       bool kahan, bool ext) {
    if (slices >= 2) {
        FwdKernelKey key;
        key.f32 = f32;
        key.kahan = kahan;
        key.sq_mask = sq_mask;
        key.slices = slices;
        key.ext = ext;
        return ws_source(pat, lit, key, 2);
    }
    Emitter em(pat, lit, ext);
    std::ostringstream o;
    o << "// generated by pasif_gb300 jit.cpp: exact adjoint, n=" << pat.n << " P=" << pat.P()
      << (ext ? " extended state" : "") << "\n";
    emit_sys_head(o, pat, em, f32);
    emit_vjp(o, pat, em);
    if (ext) emit_vjp_lo(o, pat, em);
    o << "};\n}  // namespace pk\n";
    o << "extern \"C\" __global__ void __launch_bounds__(128) pk_adj(pk::AdjArgs<pk::R> a) {\n";
    o << "  using namespace pk;\n";
    o << "  const int b = blockIdx.x * blockDim.x + threadIdx.x;\n";
    o << "  if (b >= a.B) return;\n";
    o << "  JSys sys;\n  sys.load(a.vals, (long long)a.B, b);\n";
    const int P = pat.P() > 0 ? pat.P() : 1;
    if (f32) {
        o << "  RegVec<R, " << P << "> pacc;\n";
        o << "  adj_run_jit<R, " << pat.n << ", " << P << ", " << (sq_mask ? "true" : "false") << ", true, "
          << (ext ? "true" : "false") << ">(sys, a, b, " << sq_mask << "ull, pacc);\n";
    } else {
        o << "  GVec<double> pacc{a.pbar + b, (long long)a.B};\n";
        o << "  adj_run_jit<R, " << pat.n << ", " << P << ", " << (sq_mask ? "true" : "false")
          << ", false>(sys, a, b, " << sq_mask << "ull, pacc);\n";
    }
    o << "}\n";
    return o.str();
}

std::string pool_source(const Pattern& pat, const FwdKernelKey& key) {
    if (key.slices >= 2) return ws_source(pat, Literals(), key, 1);
    Literals none;   // a pool's slots change owner: every value is loaded
    Emitter em(pat, none);
    const int pair = fwd_paired(pat, key);   // packed FP32 where the forward kernel packs
    std::ostringstream o;
    o << "// generated by pasif_gb300 jit.cpp: serving pool chunk, n=" << pat.n << " P=" << pat.P()
      << (pair ? " packed FP32" : "") << "\n";
    emit_sys_head(o, pat, em, key.f32, false, pair > 0);
    o << "};\n";
    const int W = key.window;
    o << "struct JW {\n  static constexpr int W = " << W << ";\n";
    o << "  static constexpr bool FAST = false;\n";
    o << "  static constexpr int PAIR = " << pair << ";\n";
    emit_sample_ring(o, W, key.block, pat);
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
    if (pat.n <= 0 || pat.n > (key.slices >= 2 ? kWsMaxN : kJitMaxN)) {
        *err = "state size outside the specialised range";
        return false;
    }
    return get_cached(pool_source(pat, key), "pk_pool", key.block, out, err);
}

bool get_adj_kernel(const Pattern& pat, const Literals& lit, bool f32, bool kahan, unsigned long long sq_mask, int slices,
                    JitKernel* out, std::string* err, bool ext) {
    if (pat.n <= 0 || pat.n > (slices >= 2 ? kWsMaxN : kJitMaxN) || pat.P() > (slices >= 2 ? 8192 : 1024)) {
        *err = "pattern outside the specialised range";
        return false;
    }
    return get_cached(adj_source(pat, lit, f32, sq_mask, slices, kahan, ext), "pk_adj", 128, out, err);
}

bool get_fwd_kernel(const Pattern& pat, const Literals& lit, const FwdKernelKey& key, JitKernel* out,
                    std::string* err) {
    if (pat.n <= 0 || pat.n > (key.slices >= 2 ? kWsMaxN : kJitMaxN)) {
        *err = "state size outside the specialised range";
        return false;
    }
    return get_cached(fwd_source(pat, lit, key), "pk_fwd", key.block, out, err);
}

namespace {
// FP32 slices that share their code (ws_shareable) are cut finer: more warps
// per system, the same instructions for most of them.  GB300, FP32-Kahan,
// 4096 systems, default -> finer slices: forward 64-DOF chain (128 states) 4
// -> 16 warps 2.65e9 -> 3.68e9 system-steps/s, 32-DOF chain 4 -> 8 warps
// 4.0e9 -> 5.5e9; adjoint 64-DOF chain 8 -> 16 warps 3.6e8 -> 4.5e8 adjoint
// system-steps/s, 32-DOF chain 6 -> 16 warps 4.7e8 -> 1.0e9, 16-DOF chain 4
// -> 8 warps 1.45e9 -> 1.89e9.  So: 8 states per warp forward, 4 adjoint, at
// most 16 warps, where that cut shares (in the default order or by
// displacement/velocity pairs, ws_by_dof: 64-state banded system, 2048
// systems, forward 4 -> 8 warps 2.08e9 -> 2.77e9, adjoint 8 -> 16 warps
// 1.84e8 -> 2.73e8).  Patterns whose slices differ in both cuts keep the
// register-bound split.
// The extended-state and FP64 forwards gain from finer shared cuts too
// (4096 systems unless noted, system-steps/s, default -> 8 -> 16 warps):
// FP32-EXT 64-state chain 1.27e9 -> 4.69e9 -> 4.66e9, 64-state banded (2048
// systems) 8.4e8 -> 1.79e9 -> 1.97e9, 128-state chain 1.50e9 -> 2.40e9 ->
// 3.07e9, but 32-state chain 6.1e9 -> 5.9e9 -> 6.0e9; FP64 32-state chain
// 4.9e8 -> 5.2e8 -> 5.5e8, 64-state chain 2.73e8 -> 2.77e8 -> 2.81e8,
// 64-state banded 7.8e7 -> 7.9e7 -> 8.3e7, 128-state chain 1.35e8 ->
// 1.35e8 -> 1.41e8.  So: FP32-EXT 4 states per warp from 64 states, FP64 16
// warps from 32 states.
// L2: the finer cut to take where it shares (0: none).
int ws_more_if_shared(const Pattern& pat, int L, int L2, bool adjoint) {
    if (L2 <= 0 || std::getenv("PASIF_WS_SLICES") || std::getenv(adjoint ? "PASIF_WS_SLICES_ADJ" : "PASIF_WS_SLICES_FWD"))
        return L;
    L2 = std::min(L2, pat.n);
    if (L2 <= L) return L;
    // memoised per pattern: the check generates the kernel source
    static std::mutex mu;
    static std::map<std::string, bool> memo;
    const std::string key = pattern_key(pat) + (adjoint ? "a" : "f") + std::to_string(L2);
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = memo.find(key);
        if (it != memo.end()) return it->second ? L2 : L;
    }
    const bool ok = ws_shareable(pat, L2, adjoint);
    std::lock_guard<std::mutex> g(mu);
    memo[key] = ok;
    return ok ? L2 : L;
}
}  // namespace

int ws_slices(const Pattern& pat, bool f32, bool force, int B, bool ext) {
    const int n = pat.n;
    // Measured crossovers on GB300 (time sliced / thread per system, 4096 systems):
    // FP32 forward sliced from 28 states (16-state chain 1.34, 28 states 0.94).
    // FP64 forward: its long dependent chains want more warps than one per
    // system gives: 8-28 states 0.28-0.42; 4-5 states 0.47-0.59 for batches up
    // to 8192 systems, 0.99 at 16384; 2 states 1.01.
    if (n < 2 || n > kWsMaxN) return 0;
    if (!force) {
        const bool small_batch = B > 0 && B <= 8192;
        if (f32 ? n < 28 : (n < 3 || (n < 8 && !small_batch))) return 0;
    }
    const int L2 = force ? 0 : !f32 ? (n >= 32 ? 16 : 0) : ext ? (n >= 64 ? std::min(16, n / 4) : 0) : std::min(16, n / 8);
    return ws_more_if_shared(pat, ws_split(n, f32, force, false, ext), L2, false);
}

int ws_slices_adjoint(const Pattern& pat, bool f32, bool force, bool ext) {
    const int n = pat.n;
    // The adjoint keeps about twice the vectors of the forward.  Measured on
    // GB300 (time sliced / thread per system, 1024-4096 systems): FP32 5
    // states 0.75, 8 states 0.62, 4 states 0.93, 2 states 1.12; FP64 2 states
    // 0.68, 4-8 states 0.33-0.44.
    if (n < 2 || n > kWsMaxN || (!force && f32 && n < 5)) return 0;
    // FP64, shared slices: 2 states per warp up to 32 states (GB300, 4096
    // systems, default -> 8 -> 16 warps, adjoint system-steps/s: 16-state
    // chain 3.30e8 -> 3.63e8 -> 3.59e8, 32-state chain 1.79e8 -> 1.83e8 ->
    // 1.87e8; 64-state chain 9.1e7 -> 9.1e7 -> 9.0e7 keeps its cut).
    const int L2 = force ? 0 : f32 ? (ext ? 0 : std::min(16, n / 4)) : (n <= 32 ? std::min(16, n / 2) : 0);
    return ws_more_if_shared(pat, ws_split(n, f32, force, true, ext), L2, true);
}

int ws_split(int n, bool f32, bool force, bool adjoint, bool ext) {
    // Forward: four warps when the registers allow (up to 32 FP32 / 16 FP64
    // components per warp): each SM sub-partition then runs one slice's code.
    // Measured on GB300 (forward, FP32-Kahan): 128-state chain 4 warps 1.86e9
    // system-steps/s vs 8 warps 1.5e9, 16 warps 0.84e9; 64-state banded 1.68e9
    // vs 1.30e9.  The adjoint holds about twice the vectors: 11 FP32 / 6 FP64
    // components per warp, at least 4 and (FP32) at most 8 warps.  Gradient
    // rates: 16-state chain 4 warps 1.32e9 vs 2 warps 1.01e9; 128-state chain 8
    // warps 1.35e8 vs 16 warps 0.98e8.  FP32 adjoint of 4096 systems (M adjoint
    // system-steps/s): 64-state banded 6 warps 208, 8 warps 176, 12 warps 119;
    // 32-state chain 4 warps 770, 6 warps 740; 128-state chain 8 warps 134, 12
    // warps 89.  (512 systems, 16 blocks, prefer more warps by 5-10 %.)
    // the extended-state mode holds the low parts of the values and the
    // state besides: fewer components per warp (ptxas, 64-state banded system:
    // 4 warps spill 428 bytes forward, 3.9 KB adjoint)
    // FP32 adjoints were later cut at 8 components per warp: 64-state banded
    // system, FP32-Kahan, checkpointed (M adjoint system-steps/s, 6 -> 8
    // warps): 512 systems 41.6 -> 51.9, 2048 147 -> 177, 4096 250 -> 274;
    // 10 warps were slower again (37.8 / 118 / 180).
    const int cpw = force ? 2 : adjoint ? (f32 ? 8 : 6) : (f32 ? (ext ? 12 : 32) : 16);
    int L = std::max(4, (n + cpw - 1) / cpw);
    if (adjoint && f32 && !force) L = std::min(L, 8);
    if (const char* e = std::getenv("PASIF_WS_SLICES")) L = std::atoi(e);   // tuning override
    if (const char* e = std::getenv(adjoint ? "PASIF_WS_SLICES_ADJ" : "PASIF_WS_SLICES_FWD"))
        L = std::atoi(e);   // tuning override of one kind of kernel
    return std::max(2, std::min(16, std::min(L, n)));
}

}  // namespace pasif
