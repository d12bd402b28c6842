// rk4_core.cuh -- device-side building blocks of the batched RK4 engine.
//
// Compiled twice: by nvcc into the generic (pattern-interpreting) kernels of
// generic_kernels.cu, and by NVRTC together with a generated, pattern-
// specialised system struct (jit.cpp).  It therefore includes nothing but
// pk_args.h.
//
// Every floating-point operation on the solution path is an explicit
// round-to-nearest intrinsic (__fma_rn, __dmul_rn, ...): the compiler may not
// fuse or reorder them, and the operation order is the canonical one of the
// CPU oracle (per destination: CSR row of K, then Gamma, Lambda, Psi entries
// in COO order, then forcing, dealt in turn to two partial sums that start
// as the product of their first term, fold the rest with fma and are added).
// The reference's kernels sum the same terms with atomicAdd, in no fixed
// order (src/kernels.cu:22-64, src/__GpuDriver.cu:785-838).
#pragma once
#include "pk_args.h"

namespace pk {

template <typename R> struct M;

template <> struct M<double> {
    static __device__ __forceinline__ double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double abs(double a) { return fabs(a); }
    static __device__ __forceinline__ double max(double a, double b) { return fmax(a, b); }
};

template <> struct M<float> {
    static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float abs(float a) { return fabsf(a); }
    static __device__ __forceinline__ float max(float a, float b) { return fmaxf(a, b); }
};

// Packed FP32 (f32x2) arithmetic: two independent correctly rounded FP32
// operations in one instruction (sm_100 and later).  Each lane's result is
// the scalar __fmaf_rn / __fmul_rn / __fadd_rn / __fsub_rn of its operands,
// so code written with it keeps the bits of the scalar code.
#ifndef PK_HOST_EMU
// Inline PTX with explicit .rn modifiers.  Measured on GB300 (CUDA 13.0):
// ptxas still contracts a packed multiply (mul.rn.f32x2, or fma.rn.f32x2
// with a -0 addend) whose result feeds a packed subtract into one fma, which
// rounds once instead of twice; a scalar mul.rn.f32 is never contracted.  So
// a packed product is only ever used as a factor or as the addend of another
// packed fma; products that feed an add or subtract are scalar.
struct M2 {
    static __device__ __forceinline__ unsigned long long pack(float2 a) {
        unsigned long long r;
        asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
        return r;
    }
    static __device__ __forceinline__ float2 unpack(unsigned long long r) {
        float2 o;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(o.x), "=f"(o.y) : "l"(r));
        return o;
    }
    static __device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) {
        unsigned long long r;
        asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pack(a)), "l"(pack(b)), "l"(pack(c)));
        return unpack(r);
    }
    static __device__ __forceinline__ float2 mul(float2 a, float2 b) {
        unsigned long long r;
        asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack(a)), "l"(pack(b)));
        return unpack(r);
    }
    static __device__ __forceinline__ float2 add(float2 a, float2 b) {
        unsigned long long r;
        asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack(a)), "l"(pack(b)));
        return unpack(r);
    }
    static __device__ __forceinline__ float2 sub(float2 a, float2 b) {
        unsigned long long r;
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack(a)), "l"(pack(b)));
        return unpack(r);
    }
};
#else
struct M2 {
    static inline float2 fma(float2 a, float2 b, float2 c) { return make_float2(__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y)); }
    static inline float2 mul(float2 a, float2 b) { return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)); }
    static inline float2 add(float2 a, float2 b) { return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
    static inline float2 sub(float2 a, float2 b) { return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)); }
};
#endif

// L2 prefetch of the line holding p (an address inside an allocation): the
// backward sweep over a stored trajectory reads states written long before,
// from HBM; prefetched kPrefetchSteps steps ahead they are in L2 when needed.
constexpr int kPrefetchSteps = 8;

// Trajectory slot of the state after `step` when every `every`-th state from
// step0 is saved (-1: not saved); every == 1, the stored trajectory of the
// adjoint, needs no division.
__device__ __forceinline__ long long traj_slot(unsigned step, unsigned step0, int every) {
    if (every == 1) return (long long)step - (long long)step0;
    const unsigned e = (unsigned)every;
    if (step % e != 0u) return -1;
    return (long long)(step / e) - (long long)(step0 / e) - ((step0 % e) ? 1 : 0);
}

// Vectors per step in a slot of an adjoint trajectory ([n][B] each): FP64
// stores the state and the stage inputs Y2, Y3, Y4, so that the backward
// sweep evaluates no right-hand side (FP64 arithmetic is its cost: 1.07 s ->
// 0.88 s for 4096 16-state chains x 50000 steps on GB300); FP32 stores the
// state only and recomputes the stages (moving four times the data cost more
// than the arithmetic saved: 0.170 s -> 0.186 s on the same chains).
template <typename R> __device__ __forceinline__ constexpr int adj_slot_vecs() { return sizeof(R) == 8 ? 4 : 1; }
#ifndef PK_HOST_EMU
__device__ __forceinline__ void pk_prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
#else
static inline void pk_prefetch_l2(const void*) {}
#endif

// Register-resident vector (pattern-specialised kernels: every index is a
// compile-time constant after unrolling).
template <typename R, int N>
struct RegVec {
    R v[N];
    __device__ __forceinline__ R& operator[](int i) { return v[i]; }
    __device__ __forceinline__ const R& operator[](int i) const { return v[i]; }
};

// Strided vector in global memory, one element per system (coalesced when
// consecutive threads own consecutive systems).
template <typename R>
struct GVec {
    R* p;
    long long s;
    __device__ __forceinline__ R& operator[](int i) const { return p[(long long)i * s]; }
};

// Excitation seen by a stage at (step, off, half); src/kernels.cu:72-89 and
// src/kernels.cu:97-126.  Sample 0 and samples >= len give no force; the
// j+1 neighbour is read from the flat table (it crosses into the next signal
// at j = len-1, as in the reference) and reads 0 past its end.
template <typename R>
__device__ __forceinline__ R force_at(const Forcing<R>& f, long long ebase, unsigned step,
                                      unsigned off, unsigned half) {
    if (f.w == 0u) {
        const unsigned st = step + off;
        return (st < f.len && st > 0u) ? f.x[ebase + st] : R(0);
    }
    const unsigned s2 = ((step + off) << 1) + half;
    const unsigned idx = s2 & (f.w - 1u);
    const unsigned j = s2 >> f.lw;
    if (j < f.len && j > 0u) {
        const long long base = ebase + j;
        const R x0 = f.x[base];
        const R x1 = (base + 1 < f.total) ? f.x[base + 1] : R(0);
        const R wn = f.im[idx];
        const R wc = f.im[f.w + idx];
        return M<R>::fma(wc, x0, M<R>::mul(wn, x1));
    }
    return R(0);
}

// Parameter-gradient accumulation: into FP64 (fma of the FP32 or FP64
// factors promoted to double) or, for per-step partial sums, in the compute
// precision.
// s += inc with compensation c (the Kahan form of the state update).
template <typename R>
__device__ __forceinline__ void kahan_add(R& s, R& c, R inc) {
    const R y = M<R>::sub(inc, c);
    const R t = M<R>::add(s, y);
    c = M<R>::sub(M<R>::sub(t, s), y);
    s = t;
}

// Extended-state mode: the state is an unevaluated FP32 pair hi + lo (about
// 48 significant bits).  (hi, lo) += h6 sum + h cr with h/6 = h6 + h6lo: the
// rounding error of the product h6 sum (an fma), the low part of h/6 and the
// FP64-residual term h cr are collected in e; hi + p is split exactly
// (two-sum) and the low parts are renormalised into lo (fast two-sum).
template <typename R>
__device__ __forceinline__ void ext_update(R& hi, R& lo, R sum, R cr, R h, R h6, R h6lo) {
    typedef M<R> m;
    const R p = m::mul(h6, sum);
    R e = m::fma(h6, sum, -p);
    e = m::fma(h6lo, sum, e);
    e = m::fma(h, cr, e);
    const R t = m::add(hi, p);
    const R z = m::sub(t, hi);
    const R err = m::add(m::sub(hi, m::sub(t, z)), m::sub(p, z));
    const R l = m::add(lo, m::add(err, e));
    const R q = m::add(t, l);
    lo = m::sub(l, m::sub(q, t));
    hi = q;
}

// ext_update on components 2m, 2m+1 at once (packed FP32, the same
// operations lane by lane).  The product h6 sum is formed by two scalar
// multiplications: it feeds an add, and ptxas would contract a packed
// product into a packed add (M2).
__device__ __forceinline__ void ext_update2(float& hi0, float& hi1, float& lo0, float& lo1, float sum0, float sum1,
                                            float cr0, float cr1, float h, float h6, float h6lo) {
    typedef M2 p2;
    const float2 sum = make_float2(sum0, sum1);
    const float2 p = make_float2(__fmul_rn(h6, sum0), __fmul_rn(h6, sum1));
    float2 e = p2::fma(make_float2(h6, h6), sum, make_float2(-p.x, -p.y));
    e = p2::fma(make_float2(h6lo, h6lo), sum, e);
    e = p2::fma(make_float2(h, h), make_float2(cr0, cr1), e);
    const float2 hi = make_float2(hi0, hi1), lo = make_float2(lo0, lo1);
    const float2 t = p2::add(hi, p);
    const float2 z = p2::sub(t, hi);
    const float2 err = p2::add(p2::sub(hi, p2::sub(t, z)), p2::sub(p, z));
    const float2 l = p2::add(lo, p2::add(err, e));
    const float2 q = p2::add(t, l);
    const float2 nl = p2::sub(l, p2::sub(q, t));
    lo0 = nl.x;
    lo1 = nl.y;
    hi0 = q.x;
    hi1 = q.y;
}

// (hi, lo) += x (two-sum, renormalised).
template <typename R>
__device__ __forceinline__ void ext_add(R& hi, R& lo, R x) {
    typedef M<R> m;
    const R t = m::add(hi, x);
    const R z = m::sub(t, hi);
    const R err = m::add(m::sub(hi, m::sub(t, z)), m::sub(x, z));
    const R l = m::add(lo, err);
    const R q = m::add(t, l);
    lo = m::sub(l, m::sub(q, t));
    hi = q;
}

__device__ __forceinline__ void pacc_add(double& p, double x, double y) { p = __fma_rn(x, y, p); }
__device__ __forceinline__ void pacc_add(double& p, float x, float y) { p = __fma_rn((double)x, (double)y, p); }
__device__ __forceinline__ void pacc_add(float& p, float x, float y) { p = __fmaf_rn(x, y, p); }

// Pattern interpreted from GenPattern, values read from vals[p][B].
template <typename R>
struct GenSys {
    GenPattern g;
    const R* vals;
    long long B;
    int b;

    __device__ __forceinline__ int dim() const { return g.n; }
    __device__ __forceinline__ R val(int p) const { return vals[(long long)p * B + b]; }

    // f = K.xs + Gamma:(xs,xp) + Lambda:(xs,xp,xp) + Psi:(xs,xp,xp,xp) [+ F u]
    // Canonical accumulation: the terms of destination i (K row, Gamma,
    // Lambda, Psi, F; the per-destination lists built by Pattern::flat) are
    // dealt in turn to two partial sums, each starting as the product of its
    // first term and folding the others with one fma; f[i] is their sum when
    // i has two or more terms, the first with one, +0 with none.
    template <bool FORCE, class V, class W, class F>
    __device__ __noinline__ void rhs(const V& xs, const W& xp, R u, F& f) const {
        typedef M<R> m;
        const int* kp = g.data;
        const int* kc = kp + g.n + 1;
        const int* gi = kc + g.k_nnz;
        const int* li = gi + 3 * g.g_nnz;
        const int* pi = li + 4 * g.l_nnz;
        const int* fi = pi + 5 * g.p_nnz;
        const int* dp = fi + g.f_nnz;
        const int* tl = dp + g.n + 1;
        const int go = g.k_nnz, lo = go + g.g_nnz, po = lo + g.l_nnz, fo = po + g.p_nnz;
        for (int i = 0; i < g.n; ++i) {
            R a0 = R(0), a1 = R(0);
            int k = 0;
            for (int t = dp[i]; t < dp[i + 1]; ++t) {
                const int code = tl[t];
                const int kind = code >> 28, q = code & 0x0fffffff;
                R x, y;
                if (kind == 0) {
                    x = val(q);
                    y = xs[kc[q]];
                } else if (kind == 1) {
                    const int* ix = gi + 3 * (q - go);
                    x = m::mul(val(q), xs[ix[1]]);
                    y = xp[ix[2]];
                } else if (kind == 2) {
                    const int* ix = li + 4 * (q - lo);
                    x = m::mul(m::mul(val(q), xs[ix[1]]), xp[ix[2]]);
                    y = xp[ix[3]];
                } else if (kind == 3) {
                    const int* ix = pi + 5 * (q - po);
                    x = m::mul(m::mul(m::mul(val(q), xs[ix[1]]), xp[ix[2]]), xp[ix[3]]);
                    y = xp[ix[4]];
                } else {
                    if (!FORCE) break;   // forcing terms close every list
                    x = val(q);
                    y = u;
                    (void)fo;
                }
                if (k < 2) {
                    if (k) a1 = m::mul(x, y);
                    else a0 = m::mul(x, y);
                } else if (k & 1) {
                    a1 = m::fma(x, y, a1);
                } else {
                    a0 = m::fma(x, y, a0);
                }
                ++k;
            }
            f[i] = k >= 2 ? m::add(a0, a1) : a0;
        }
    }

    // out = J(y)^T w ; pb += (df/dp)^T w  (forward systems: xs == xp == y).
    template <class V, class W, class O, class PB>
    __device__ __noinline__ void vjp(const V& y, const W& w, R u, O& out, PB& pb) const {
        typedef M<R> m;
        const int* kp = g.data;
        const int* kc = kp + g.n + 1;
        const int* gi = kc + g.k_nnz;
        const int* li = gi + 3 * g.g_nnz;
        const int* pi = li + 4 * g.l_nnz;
        const int* fi = pi + 5 * g.p_nnz;
        for (int i = 0; i < g.n; ++i) out[i] = R(0);
        for (int i = 0; i < g.n; ++i) {
            const R wi = w[i];
            for (int p = kp[i]; p < kp[i + 1]; ++p) {
                const int j = kc[p];
                out[j] = m::fma(val(p), wi, out[j]);
                pacc_add(pb[p], wi, y[j]);
            }
        }
        int off = g.k_nnz;
        for (int e = 0; e < g.g_nnz; ++e) {
            const int* ix = gi + 3 * e;
            const R wi = w[ix[0]], yj = y[ix[1]], yk = y[ix[2]];
            const R a = m::mul(val(off + e), wi);
            out[ix[1]] = m::fma(a, yk, out[ix[1]]);
            out[ix[2]] = m::fma(a, yj, out[ix[2]]);
            pacc_add(pb[off + e], m::mul(wi, yj), yk);
        }
        off += g.g_nnz;
        for (int e = 0; e < g.l_nnz; ++e) {
            const int* ix = li + 4 * e;
            const R wi = w[ix[0]], yj = y[ix[1]], yk = y[ix[2]], yl = y[ix[3]];
            const R a = m::mul(val(off + e), wi);
            out[ix[1]] = m::fma(m::mul(a, yk), yl, out[ix[1]]);
            out[ix[2]] = m::fma(m::mul(a, yj), yl, out[ix[2]]);
            out[ix[3]] = m::fma(m::mul(a, yj), yk, out[ix[3]]);
            pacc_add(pb[off + e], m::mul(m::mul(wi, yj), yk), yl);
        }
        off += g.l_nnz;
        for (int e = 0; e < g.p_nnz; ++e) {
            const int* ix = pi + 5 * e;
            const R wi = w[ix[0]], yj = y[ix[1]], yk = y[ix[2]], yl = y[ix[3]], ym = y[ix[4]];
            const R a = m::mul(val(off + e), wi);
            out[ix[1]] = m::fma(m::mul(m::mul(a, yk), yl), ym, out[ix[1]]);
            out[ix[2]] = m::fma(m::mul(m::mul(a, yj), yl), ym, out[ix[2]]);
            out[ix[3]] = m::fma(m::mul(m::mul(a, yj), yk), ym, out[ix[3]]);
            out[ix[4]] = m::fma(m::mul(m::mul(a, yj), yk), yl, out[ix[4]]);
            pacc_add(pb[off + e], m::mul(m::mul(m::mul(wi, yj), yk), yl), ym);
        }
        off += g.p_nnz;
        for (int e = 0; e < g.f_nnz; ++e)
            pacc_add(pb[off + e], w[fi[e]], u);
    }
};

// One RK4 step (src/__GpuDriver.cu:693-713): k1 at u(step, half 0), k2 and k3
// at u(step, half 1), k4 at u(step+1, half 0); Q += h/6 (k1 + 2k2 + 2k3 + k4)
// with the sum formed as ((k1 + 2k2) + 2k3) + k4.  KAHAN: compensated update.
// N > 0: compile-time size (registers); N == 0: runtime size sys.dim().
// NSTG = 1: the step's state is also stored to stg[i sB]; NSTG = 4: and its
// stage inputs Y2, Y3, Y4 to stg[(j n + i) sB], j = 1..3: one slot of an
// adjoint trajectory (adj_slot_vecs).
// EXT (extended-state mode, N > 0 only): Q and Cm are the high and low parts
// of the state; the stages use the FP32 values (high parts) of the state and
// the parameters; the step adds, beside h/6 (k1 + 2k2 + 2k3 + k4), the term
// h f_lo(Q) of the low parts of the FP64 parameters (JSys::rhs_lo), evaluated
// once at the start of the step, with ext_update (h6lo: low part of h/6).
// FAST (fast kernels, PASIF_PLAN_FAST): the step's increment is summed as
// h/6 k1 - c + h/3 k2 + h/3 k3 + h/6 k4 directly (the compensation folded into
// its first fma, h/3 = 2 h6 exactly) instead of h/6 ((k1 + 2k2) + 2k3 + k4) - c:
// the same compensated update in fewer operations, not the oracle's bits.
// PAIR (packed-FP32 kernels, FP32 forward with a paired right-hand side):
// the same operations in the same order, components 2m and 2m+1 updated
// together by f32x2 instructions (M2): the bits of the scalar step.  PAIR 1
// leaves the compensated (Kahan) update scalar, PAIR 2 packs it too.
template <typename R, int N, bool KAHAN, int NSTG = 0, bool EXT = false, bool FAST = false, int PAIR = 0,
          class Sys, class V>
__device__ __forceinline__ void rk4_step(const Sys& sys, V& Q, V& Cm, V& S, V& K, V& Mi,
                                         R ua, R ub, R uc, R h, R h2, R h6, R* stg = nullptr, long long sB = 0,
                                         R h6lo = R(0)) {
    typedef M<R> m;
    static_assert(!EXT || N > 0, "extended-state steps need a compile-time state size");
    static_assert(!FAST || (!EXT && NSTG == 0), "fast steps are plain forward steps");
    static_assert(!PAIR || (sizeof(R) == 4 && N > 0 && !FAST && NSTG <= 1), "paired steps: FP32 forward");
    const int n = N ? N : sys.dim();
    if constexpr (PAIR) {
        typedef M2 p2;
        auto P = [](R x, R y) { return make_float2(x, y); };
        const float2 H2 = P(h2, h2), H = P(h, h), TWO = P(R(2), R(2)), H6 = P(h6, h6);
        if constexpr (NSTG >= 1) {
#pragma unroll
            for (int i = 0; i < N; ++i) stg[i * sB] = Q[i];
        }
        RegVec<R, EXT ? N : 1> Kc;
        if constexpr (EXT) sys.template rhs_lo<true>(Q, Q, ua, Kc);
        sys.template rhs<true>(Q, Q, ua, K);
#pragma unroll
        for (int i = 0; i + 1 < N; i += 2) {
            S[i] = K[i];
            S[i + 1] = K[i + 1];
            const float2 r = p2::fma(H2, P(K[i], K[i + 1]), P(Q[i], Q[i + 1]));
            Mi[i] = r.x;
            Mi[i + 1] = r.y;
        }
        if constexpr (N & 1) { S[N - 1] = K[N - 1]; Mi[N - 1] = m::fma(h2, K[N - 1], Q[N - 1]); }
#pragma unroll
        for (int stage = 0; stage < 2; ++stage) {
            sys.template rhs<true>(Mi, Mi, ub, K);
            const float2 HS = stage == 0 ? H2 : H;
#pragma unroll
            for (int i = 0; i + 1 < N; i += 2) {
                const float2 k = P(K[i], K[i + 1]);
                const float2 s = p2::fma(TWO, k, P(S[i], S[i + 1]));
                const float2 r = p2::fma(HS, k, P(Q[i], Q[i + 1]));
                S[i] = s.x;
                S[i + 1] = s.y;
                Mi[i] = r.x;
                Mi[i + 1] = r.y;
            }
            if constexpr (N & 1) {
                S[N - 1] = m::fma(R(2), K[N - 1], S[N - 1]);
                Mi[N - 1] = m::fma(stage == 0 ? h2 : h, K[N - 1], Q[N - 1]);
            }
        }
        sys.template rhs<true>(Mi, Mi, uc, K);
        if constexpr (EXT && PAIR == 1) {
#pragma unroll
            for (int i = 0; i < N; ++i) ext_update(Q[i], Cm[i], m::add(S[i], K[i]), Kc[i], h, h6, h6lo);
            return;
        }
        if constexpr (EXT) {
#pragma unroll
            for (int i = 0; i + 1 < N; i += 2) {
                const float2 sum = p2::add(P(S[i], S[i + 1]), P(K[i], K[i + 1]));
                ext_update2(Q[i], Q[i + 1], Cm[i], Cm[i + 1], sum.x, sum.y, Kc[i], Kc[i + 1], h, h6, h6lo);
            }
            if constexpr (N & 1) ext_update(Q[N - 1], Cm[N - 1], m::add(S[N - 1], K[N - 1]), Kc[N - 1], h, h6, h6lo);
            return;
        }
        if constexpr (KAHAN && PAIR == 1) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const R y = m::sub(m::mul(h6, m::add(S[i], K[i])), Cm[i]);
                const R t = m::add(Q[i], y);
                Cm[i] = m::sub(m::sub(t, Q[i]), y);
                Q[i] = t;
            }
            return;
        }
#pragma unroll
        for (int i = 0; i + 1 < N; i += 2) {
            const float2 sum = p2::add(P(S[i], S[i + 1]), P(K[i], K[i + 1]));
            const float2 q = P(Q[i], Q[i + 1]);
            float2 t;
            if constexpr (KAHAN) {
                const float2 c = P(Cm[i], Cm[i + 1]);
                // scalar products: ptxas would contract a packed multiply into the
                // packed subtract that consumes it (one rounding instead of two)
                const float2 y = p2::sub(P(m::mul(h6, sum.x), m::mul(h6, sum.y)), c);
                t = p2::add(q, y);
                const float2 cn = p2::sub(p2::sub(t, q), y);
                Cm[i] = cn.x;
                Cm[i + 1] = cn.y;
            } else {
                t = p2::fma(H6, sum, q);
            }
            Q[i] = t.x;
            Q[i + 1] = t.y;
        }
        if constexpr (N & 1) {
            const int i = N - 1;
            const R sum = m::add(S[i], K[i]);
            if constexpr (KAHAN) {
                const R y = m::sub(m::mul(h6, sum), Cm[i]);
                const R t = m::add(Q[i], y);
                Cm[i] = m::sub(m::sub(t, Q[i]), y);
                Q[i] = t;
            } else {
                Q[i] = m::fma(h6, sum, Q[i]);
            }
        }
        return;
    }
    if constexpr (FAST) {
        const R h3 = m::add(h6, h6);
        sys.template rhs<true>(Q, Q, ua, K);
#pragma unroll
        for (int i = 0; i < n; ++i) {
            S[i] = m::fma(h6, K[i], KAHAN ? -Cm[i] : R(0));
            Mi[i] = m::fma(h2, K[i], Q[i]);
        }
        sys.template rhs<true>(Mi, Mi, ub, K);
#pragma unroll
        for (int i = 0; i < n; ++i) { S[i] = m::fma(h3, K[i], S[i]); Mi[i] = m::fma(h2, K[i], Q[i]); }
        sys.template rhs<true>(Mi, Mi, ub, K);
#pragma unroll
        for (int i = 0; i < n; ++i) { S[i] = m::fma(h3, K[i], S[i]); Mi[i] = m::fma(h, K[i], Q[i]); }
        sys.template rhs<true>(Mi, Mi, uc, K);
#pragma unroll
        for (int i = 0; i < n; ++i) {
            const R y = m::fma(h6, K[i], S[i]);
            const R t = m::add(Q[i], y);
            if (KAHAN) Cm[i] = m::sub(m::sub(t, Q[i]), y);
            Q[i] = t;
        }
        return;
    }
    if constexpr (NSTG >= 1) {
#pragma unroll
        for (int i = 0; i < n; ++i) stg[i * sB] = Q[i];
    }
    RegVec<R, (EXT && N > 0) ? N : 1> Kc;
    if constexpr (EXT) sys.template rhs_lo<true>(Q, Q, ua, Kc);
    sys.template rhs<true>(Q, Q, ua, K);
#pragma unroll
    for (int i = 0; i < n; ++i) { S[i] = K[i]; Mi[i] = m::fma(h2, K[i], Q[i]); }
    if constexpr (NSTG == 4) {
#pragma unroll
        for (int i = 0; i < n; ++i) stg[(n + i) * sB] = Mi[i];
    }
    sys.template rhs<true>(Mi, Mi, ub, K);
#pragma unroll
    for (int i = 0; i < n; ++i) { S[i] = m::fma(R(2), K[i], S[i]); Mi[i] = m::fma(h2, K[i], Q[i]); }
    if constexpr (NSTG == 4) {
#pragma unroll
        for (int i = 0; i < n; ++i) stg[(2 * n + i) * sB] = Mi[i];
    }
    sys.template rhs<true>(Mi, Mi, ub, K);
#pragma unroll
    for (int i = 0; i < n; ++i) { S[i] = m::fma(R(2), K[i], S[i]); Mi[i] = m::fma(h, K[i], Q[i]); }
    if constexpr (NSTG == 4) {
#pragma unroll
        for (int i = 0; i < n; ++i) stg[(3 * n + i) * sB] = Mi[i];
    }
    sys.template rhs<true>(Mi, Mi, uc, K);
#pragma unroll
    for (int i = 0; i < n; ++i) {
        const R sum = m::add(S[i], K[i]);
        if constexpr (EXT) {
            ext_update(Q[i], Cm[i], sum, Kc[i], h, h6, h6lo);
        } else if (KAHAN) {
            const R inc = m::mul(h6, sum);
            const R y = m::sub(inc, Cm[i]);
            const R t = m::add(Q[i], y);
            Cm[i] = m::sub(m::sub(t, Q[i]), y);
            Q[i] = t;
        } else {
            Q[i] = m::fma(h6, sum, Q[i]);
        }
    }
}

// Forward integration of one instance with the max |q| and sum q^2 reducers.
template <typename R, int N, bool KAHAN, bool HMAX, bool HSQ, bool HTRAJ, class Sys, class V>
__device__ __forceinline__ void fwd_run(const Sys& sys, const FwdArgs<R>& a, int b,
                                        unsigned long long max_mask, unsigned long long sq_mask,
                                        V& Q, V& Cm, V& S, V& K, V& Mi, V& Mx) {
    typedef M<R> m;
    const int n = N ? N : sys.dim();
    const long long B = a.B;
    const long long ebase = (long long)a.exc_index[b] * (long long)a.frc.len;
#pragma unroll
    for (int i = 0; i < n; ++i) {
        Q[i] = a.state[i * B + b];
        if (KAHAN) Cm[i] = R(0);
        if (HMAX) Mx[i] = R(0);
    }
    R sq = R(0), sqc = R(0);
    R uc = force_at(a.frc, ebase, a.step0, 0u, 0u);
    for (int s = 0; s < a.nsteps; ++s) {
        const unsigned step = a.step0 + (unsigned)s;
        const R ua = uc;
        const R ub = force_at(a.frc, ebase, step, 0u, 1u);
        uc = force_at(a.frc, ebase, step, 1u, 0u);
        rk4_step<R, N, KAHAN>(sys, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6);
        if (HTRAJ) {
            const long long slot = traj_slot(step, a.step0, a.traj_every);
            if (slot >= 0 && slot < a.traj_slots) {
#pragma unroll
                for (int i = 0; i < n; ++i) a.traj[(slot * n + i) * B + b] = Q[i];
            }
        }
        if (HMAX && (long long)step >= (long long)a.max_start) {
#pragma unroll
            for (int i = 0; i < n; ++i)
                if (i < 64 && ((max_mask >> i) & 1ull)) Mx[i] = m::max(Mx[i], m::abs(Q[i]));
        }
        if (HSQ && (long long)step >= (long long)a.sq_start) {
#pragma unroll
            for (int i = 0; i < n; ++i)
                if (i < 64 && ((sq_mask >> i) & 1ull)) {
                    const R q = Q[i];
                    if (KAHAN) {
                        const R y = m::sub(m::mul(q, q), sqc);
                        const R t = m::add(sq, y);
                        sqc = m::sub(m::sub(t, sq), y);
                        sq = t;
                    } else {
                        sq = m::fma(q, q, sq);
                    }
                }
        }
    }
#pragma unroll
    for (int i = 0; i < n; ++i) a.state[i * B + b] = Q[i];
    if (HMAX) {
        int slot = 0;
#pragma unroll
        for (int i = 0; i < n; ++i)
            if (i < 64 && ((max_mask >> i) & 1ull)) { a.out_max[slot * B + b] = Mx[i]; ++slot; }
    }
    if (HSQ) a.out_sq[b] = sq;
}

// Flat read of the excitation table, 0 past its end.
template <typename R>
__device__ __forceinline__ R sample_at(const Forcing<R>& f, long long idx) {
    return idx < f.total ? f.x[idx] : R(0);
}

// Asynchronous copy of sample_at(f, idx) into shared memory (cp.async; past
// the table's end the source size is 0 and the slot is zero-filled), and its
// group commit / wait.
#ifndef PK_HOST_EMU
template <typename R>
__device__ __forceinline__ void sample_async(R* dst, const Forcing<R>& f, long long idx) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const bool ok = idx < f.total;
    const R* src = f.x + (ok ? idx : 0);
    const int n = ok ? (int)sizeof(R) : 0;
    if (sizeof(R) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory"); }
#else
template <typename R>
static inline void sample_async(R* dst, const Forcing<R>& f, long long idx) { *dst = sample_at(f, idx); }
static inline void async_commit() {}
template <int PENDING>
static inline void async_wait() {}
#endif

// Forward integration walking the excitation one sample interval at a time
// (pattern-specialised kernels).  WP::W is the interpolation window (0 =
// sample and hold) and WP::wn(i) / WP::wc(i) its next / current-sample
// weights, compile-time constants, so the W/2 steps of an interval need no
// index arithmetic; the three samples of the sliding window live in
// registers and the next one is loaded an interval ahead.  Every forcing
// value equals force_at's (same operations on the same operands); steps
// before the first and after the last whole interval use force_at.
//
// fwd_core_iv runs rc.nsteps steps from rc.step0 on state already in
// registers (Q, Kahan compensation Cm, reducers Mx / sq / sqc): the batch
// kernel calls it once per horizon, the serving pool once per chunk with the
// state carried in device memory between chunks, which gives the same bits
// as an uninterrupted run.
struct RunCtx {
    long long ebase;     // first sample of this instance's signal row
    unsigned step0;
    unsigned nsteps;
    int max_start;
    int sq_start;
};

// HTRAJ: 0 none; 1 the state after every traj_every-th step into a.traj
// ([slot][N][B]); 2 the adjoint trajectory: before every step its slot into
// a.traj ([step - step0][adj_slot_vecs][N][B], see rk4_step); 3 checkpoints
// for the adjoint: the state and compensation before every traj_every-th
// step into a.traj ([step / traj_every][2N][B]).
template <typename R, int N, bool KAHAN, bool HMAX, bool HSQ, int HTRAJ, class WP, bool EXT = false, class Sys,
          class V>
__device__ __forceinline__ void fwd_core_iv(const Sys& sys, const FwdArgs<R>& a, const Forcing<R>& frc, int b,
                                            const RunCtx& rc, unsigned long long max_mask,
                                            unsigned long long sq_mask, V& Q, V& Cm, V& S, V& K, V& Mi, V& Mx,
                                            R& sq, R& sqc) {
    typedef M<R> m;
    constexpr int W = WP::W;
    constexpr bool FASTK = WP::FAST && HTRAJ == 0 && !EXT;   // fast steps: plain forwards only
    // paired (f32x2) steps: FP32 forwards (extended state: packed stages only)
    constexpr int PAIRK = (WP::PAIR && !FASTK) ? WP::PAIR : 0;
    constexpr unsigned SPI = W == 0 ? 1u : (unsigned)(W / 2);
    constexpr int STG = HTRAJ == 2 ? adj_slot_vecs<R>() : 0;
    const long long B = a.B;
    const long long ebase = rc.ebase;
    const unsigned len = frc.len;
    auto slot = [&](unsigned step) -> R* {
        return STG ? a.traj + (long long)(step - a.step0) * STG * N * B + b : nullptr;
    };
    // HTRAJ == 3: checkpoints, the state and compensation before every
    // traj_every-th step
    auto pre = [&](unsigned step) {
        if constexpr (HTRAJ == 3) {
            if (step % (unsigned)a.traj_every == 0u) {
                R* ck = a.traj + (long long)(step / (unsigned)a.traj_every) * 2 * N * B + b;
#pragma unroll
                for (int i = 0; i < N; ++i) {
                    ck[i * B] = Q[i];
                    ck[(N + i) * B] = KAHAN ? Cm[i] : R(0);
                }
            }
        }
    };
    auto post = [&](unsigned step) {
        if (HTRAJ == 1) {
            const long long slot = traj_slot(step, a.step0, a.traj_every);
            if (slot >= 0 && slot < a.traj_slots) {
#pragma unroll
                for (int i = 0; i < N; ++i) a.traj[(slot * N + i) * B + b] = Q[i];
            }
        }
        if (HMAX && (long long)step >= (long long)rc.max_start) {
#pragma unroll
            for (int i = 0; i < N; ++i)
                if (i < 64 && ((max_mask >> i) & 1ull)) Mx[i] = m::max(Mx[i], m::abs(Q[i]));
        }
        if (HSQ && (long long)step >= (long long)rc.sq_start) {
#pragma unroll
            for (int i = 0; i < N; ++i)
                if (i < 64 && ((sq_mask >> i) & 1ull)) {
                    const R q = Q[i];
                    if (KAHAN) {
                        const R y = m::sub(m::mul(q, q), sqc);
                        const R t = m::add(sq, y);
                        sqc = m::sub(m::sub(t, sq), y);
                        sq = t;
                    } else {
                        sq = m::fma(q, q, sq);
                    }
                }
        }
    };
    unsigned s = rc.step0;
    const unsigned end = rc.step0 + rc.nsteps;
    while (s < end && (s % SPI) != 0u) {
        pre(s);
        rk4_step<R, N, KAHAN, STG, EXT, FASTK, PAIRK>(sys, Q, Cm, S, K, Mi, force_at(frc, ebase, s, 0u, 0u),
                                               force_at(frc, ebase, s, 0u, 1u), force_at(frc, ebase, s, 1u, 0u), a.h,
                                               a.h2, a.h6, slot(s), B, a.h6lo);
        post(s);
        ++s;
    }
    if (end - s >= SPI) {
        unsigned j = s / SPI;
        R x0 = sample_at(frc, ebase + j), x1 = sample_at(frc, ebase + j + 1), x2 = sample_at(frc, ebase + j + 2);
        // WP::RING > 0: sample j + 3 is copied into this thread's shared-memory
        // ring (slot (j + 3) % RING, stride RS) RING - 1 intervals before use
        constexpr int RING = WP::RING;
        R* const ring = WP::ring();
        if constexpr (RING > 0) {
#pragma unroll
            for (int q = 0; q < RING - 1; ++q) {
                sample_async(ring + ((j + 3u + (unsigned)q) % (unsigned)RING) * WP::RS, frc, ebase + j + 3 + q);
                async_commit();
            }
        }
        for (; end - s >= SPI; s += SPI, ++j) {
            R nxt;
            if constexpr (RING > 0) {
                async_wait<RING - 2>();   // the copy of sample j + 3 (the oldest of RING - 1) has landed
                nxt = ring[((j + 3u) % (unsigned)RING) * WP::RS];
                // refill the slot read in the previous interval
                sample_async(ring + ((j + 3u + RING - 1u) % (unsigned)RING) * WP::RS, frc, ebase + j + 3 + RING - 1);
                async_commit();
            } else {
                nxt = sample_at(frc, ebase + j + 3);
            }
            const bool g0 = j > 0u && j < len;
            const bool g1 = j + 1u > 0u && j + 1u < len;
            R uc;
            if (W == 0) uc = g0 ? x0 : R(0);
            else uc = g0 ? m::fma(WP::wc(0), x0, m::mul(WP::wn(0), x1)) : R(0);
#pragma unroll
            for (int r = 0; r < (int)SPI; ++r) {
                const R ua = uc;
                R ub, un;
                if (W == 0) {
                    ub = ua;
                    un = g1 ? x1 : R(0);
                } else {
                    ub = g0 ? m::fma(WP::wc(2 * r + 1), x0, m::mul(WP::wn(2 * r + 1), x1)) : R(0);
                    if (2 * r + 2 < W) un = g0 ? m::fma(WP::wc(2 * r + 2), x0, m::mul(WP::wn(2 * r + 2), x1)) : R(0);
                    else un = g1 ? m::fma(WP::wc(0), x1, m::mul(WP::wn(0), x2)) : R(0);
                }
                pre(s + (unsigned)r);
                rk4_step<R, N, KAHAN, STG, EXT, FASTK, PAIRK>(sys, Q, Cm, S, K, Mi, ua, ub, un, a.h, a.h2, a.h6,
                                                       slot(s + (unsigned)r), B, a.h6lo);
                post(s + (unsigned)r);
                uc = un;
            }
            x0 = x1;
            x1 = x2;
            x2 = nxt;
        }
        if constexpr (RING > 0) async_wait<0>();   // no copy outlives the loop
    }
    while (s < end) {
        pre(s);
        rk4_step<R, N, KAHAN, STG, EXT, FASTK, PAIRK>(sys, Q, Cm, S, K, Mi, force_at(frc, ebase, s, 0u, 0u),
                                               force_at(frc, ebase, s, 0u, 1u), force_at(frc, ebase, s, 1u, 0u), a.h,
                                               a.h2, a.h6, slot(s), B, a.h6lo);
        post(s);
        ++s;
    }
}

// One batch instance over the whole horizon (initial state in a.state, final
// state and reducers out).  HTRAJ as fwd_core_iv; 2 also stores the final
// state in slot nsteps (its state part).
template <typename R, int N, bool KAHAN, bool HMAX, bool HSQ, int HTRAJ, class WP, bool EXT = false, class Sys,
          class V>
__device__ __forceinline__ void fwd_run_iv(const Sys& sys, const FwdArgs<R>& a, int b,
                                           unsigned long long max_mask, unsigned long long sq_mask,
                                           V& Q, V& Cm, V& S, V& K, V& Mi, V& Mx) {
    const long long B = a.B;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        Q[i] = a.state[i * B + b];
        if (KAHAN) Cm[i] = a.comp ? a.comp[i * B + b] : R(0);
        if (HMAX) Mx[i] = R(0);
    }
    R sq = R(0), sqc = R(0);
    RunCtx rc;
    rc.ebase = (long long)a.exc_index[b] * (long long)a.frc.len;
    rc.step0 = a.step0;
    rc.nsteps = (unsigned)a.nsteps;
    rc.max_start = a.max_start;
    rc.sq_start = a.sq_start;
    fwd_core_iv<R, N, KAHAN, HMAX, HSQ, HTRAJ, WP, EXT>(sys, a, a.frc, b, rc, max_mask, sq_mask, Q, Cm, S, K, Mi, Mx,
                                                        sq, sqc);
#pragma unroll
    for (int i = 0; i < N; ++i) a.state[i * B + b] = Q[i];
    if (EXT && a.comp_out) {
#pragma unroll
        for (int i = 0; i < N; ++i) a.comp_out[i * B + b] = Cm[i];
    }
    if (HTRAJ == 2) {
#pragma unroll
        for (int i = 0; i < N; ++i) a.traj[((long long)a.nsteps * adj_slot_vecs<R>() * N + i) * B + b] = Q[i];
    }
    if (HMAX) {
        int slot = 0;
#pragma unroll
        for (int i = 0; i < N; ++i)
            if (i < 64 && ((max_mask >> i) & 1ull)) { a.out_max[slot * B + b] = Mx[i]; ++slot; }
    }
    if (HSQ) a.out_sq[b] = sq;
}

// Serving pool: slot b advances min(chunk, remaining) steps from its own step
// index, its state, Kahan compensation and reducers carried in device memory
// (PoolArgs, pk_args.h).  Free slots (remaining <= 0) return at once.
template <typename R, int N, bool KAHAN, bool HMAX, bool HSQ, class WP, class Sys>
__device__ __forceinline__ void pool_run_iv(const Sys& sys, const PoolArgs<R>& p, int b,
                                            unsigned long long max_mask, unsigned long long sq_mask) {
    const int rem = p.remain[b];
    if (rem <= 0) return;
    const long long C = p.C;
    RegVec<R, N> Q, Cm, S, K, Mi, Mx;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        Q[i] = p.state[i * C + b];
        if (KAHAN) Cm[i] = p.comp[i * C + b];
        if (HMAX) Mx[i] = p.mx[i * C + b];
    }
    R sq = HSQ ? p.sq[b] : R(0), sqc = HSQ ? p.sqc[b] : R(0);
    FwdArgs<R> a;   // the fields fwd_core_iv reads: B, h, h2, h6 (no trajectory)
    a.B = p.C;
    a.h = p.h;
    a.h2 = p.h2;
    a.h6 = p.h6;
    a.traj = nullptr;
    a.traj_every = 1;
    a.traj_slots = 0;
    a.step0 = 0;
    Forcing<R> frc = p.frc;
    frc.len = p.len[b];
    frc.total = p.lim[b];
    RunCtx rc;
    rc.ebase = p.ebase[b];
    rc.step0 = p.step[b];
    rc.nsteps = (unsigned)(rem < p.chunk ? rem : p.chunk);
    rc.max_start = p.max_start[b];
    rc.sq_start = p.sq_start[b];
    fwd_core_iv<R, N, KAHAN, HMAX, HSQ, 0, WP>(sys, a, frc, b, rc, max_mask, sq_mask, Q, Cm, S, K, Mi, Mx, sq, sqc);
#pragma unroll
    for (int i = 0; i < N; ++i) {
        p.state[i * C + b] = Q[i];
        if (KAHAN) p.comp[i * C + b] = Cm[i];
        if (HMAX) p.mx[i * C + b] = Mx[i];
    }
    if (HSQ) { p.sq[b] = sq; p.sqc[b] = sqc; }
    p.step[b] = rc.step0 + rc.nsteps;
    p.remain[b] = rem - (int)rc.nsteps;
}

// Exact discrete adjoint for pattern-specialised kernels: the same algorithm
// and operation order as adj_run_generic below, with every state-sized vector
// in registers (N compile-time) and the chunk states in the global buffer.
// PACC = RegVec<float, P> (FP32: parameter gradients summed per step in FP32,
// then added to the FP64 totals) or GVec<double> (FP64: straight into the
// FP64 totals, bit-identical to the generic kernel and the oracle).
template <typename R, int N, int P, bool HSQ, bool STEP_ACC, bool EXT = false, class Sys, class PACC>
__device__ __forceinline__ void adj_run_jit(const Sys& sys, const AdjArgs<R>& a, int b, unsigned long long sq_mask,
                                            PACC& pacc) {
    typedef M<R> m;
    const long long B = a.B;
    GVec<double> PB{a.pbar + b, B};
    const long long ebase = (long long)a.exc_index[b] * (long long)a.frc.len;
    constexpr int SV = adj_slot_vecs<R>();
    RegVec<R, N> Q, Cm, S, K, Mi;
    if (STEP_ACC) {
#pragma unroll
        for (int p = 0; p < P; ++p) pacc[p] = R(0);
    }
    if (a.phase != 2 && !a.stored) {   // forward pass with checkpoints
        const int t0 = a.phase == 1 ? a.t_begin : 0, t1 = a.phase == 1 ? a.t_end : a.nsteps;
        if (t0 == 0) {
            for (int p = 0; p < P; ++p) PB[p] = 0.0;
#pragma unroll
            for (int i = 0; i < N; ++i) { Q[i] = a.x0[i * B + b]; Cm[i] = EXT ? a.x0[(N + i) * B + b] : R(0); }
        } else {
            const R* ck = a.ckpt + (long long)(t0 / a.C) * 2 * N * B + b;
#pragma unroll
            for (int i = 0; i < N; ++i) { Q[i] = ck[i * B]; Cm[i] = ck[(N + i) * B]; }
        }
        for (int t = t0; t < t1; ++t) {
            if (t % a.C == 0) {
                R* ck = a.ckpt + (long long)(t / a.C) * 2 * N * B + b;
#pragma unroll
                for (int i = 0; i < N; ++i) { ck[i * B] = Q[i]; ck[(N + i) * B] = Cm[i]; }
            }
            const unsigned st = (unsigned)t;
            const R ua = force_at(a.frc, ebase, st, 0u, 0u);
            const R ub = force_at(a.frc, ebase, st, 0u, 1u);
            const R uc = force_at(a.frc, ebase, st, 1u, 0u);
            if constexpr (EXT) rk4_step<R, N, true, 0, true>(sys, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6, nullptr, 0, a.h6lo);
            else if (a.kahan) rk4_step<R, N, true>(sys, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6);
            else rk4_step<R, N, false>(sys, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6);
        }
        if (a.phase == 1) {   // the next segment starts from this checkpoint
            if (t1 < a.nsteps && t1 % a.C == 0) {
                R* ck = a.ckpt + (long long)(t1 / a.C) * 2 * N * B + b;
#pragma unroll
                for (int i = 0; i < N; ++i) { ck[i * B] = Q[i]; ck[(N + i) * B] = Cm[i]; }
            }
            return;
        }
    }
    RegVec<R, N> LAM, QN, CL;   // CL: compensation of LAM (Kahan mode)
    const int khi = a.phase == 2 ? a.k_hi : a.nck - 1, klo = a.phase == 2 ? a.k_lo : 0;
    // FP32 with few values: the FP64 totals in registers through the backward
    // launch (the same additions as into pbar, in the same order)
    constexpr bool PBREG = STEP_ACC && P <= 24;
    RegVec<double, PBREG ? P : 1> PR;
    // per-step sums added with compensation to FP32 totals, flushed into the
    // FP64 totals once per chunk of C steps (FP64 adds run at 1/64 of the FP32
    // rate on GB300: once per step they were a large part of the step)
    RegVec<R, PBREG ? P : 1> PK, PKC;
#pragma unroll
    for (int p = 0; p < (PBREG ? P : 1); ++p) { PR[p] = 0.0; PK[p] = R(0); PKC[p] = R(0); }
    if (khi == a.nck - 1) {
        if (a.stored && !PBREG)   // no forward pass in this kernel zeroed the totals
            for (int p = 0; p < P; ++p) PB[p] = 0.0;
#pragma unroll
        for (int i = 0; i < N; ++i) { LAM[i] = a.g_final ? a.g_final[i * B + b] : R(0); CL[i] = R(0); }
    } else {   // carried from the previous backward launch
#pragma unroll
        for (int i = 0; i < N; ++i) { LAM[i] = a.dx0[i * B + b]; CL[i] = a.kahan ? a.lamc[i * B + b] : R(0); }
        if constexpr (PBREG) {
#pragma unroll
            for (int p = 0; p < P; ++p) PR[p] = PB[p];
        }
    }
    const R gsq2h = a.g_sq ? m::mul(m::mul(a.g_sq[b], R(2)), a.h) : R(0);
    const double h6d = (double)a.h6 + (double)a.h6lo;   // h/6 (extended-state mode)
    for (int k = khi; k >= klo; --k) {
        const int start = k * a.C;
        const int end = (start + a.C < a.nsteps) ? start + a.C : a.nsteps;
        const int slot0 = a.stored ? a.slot_base : start;   // buf slot of step t: t - slot0
        if constexpr (STEP_ACC && !PBREG) {
            for (int p = 0; p < 2 * P; ++p) a.pk[(long long)p * B + b] = R(0);
        }
        if (!a.stored) {
            const R* ck = a.ckpt + (long long)k * 2 * N * B + b;
#pragma unroll
            for (int i = 0; i < N; ++i) { Q[i] = ck[i * B]; Cm[i] = ck[(N + i) * B]; }
            for (int t = start; t < end; ++t) {   // slot: state (and FP64: stage inputs) of step t
                R* bt = a.buf + (long long)(t - start) * SV * N * B + b;
                const unsigned st = (unsigned)t;
                const R ua = force_at(a.frc, ebase, st, 0u, 0u);
                const R ub = force_at(a.frc, ebase, st, 0u, 1u);
                const R uc = force_at(a.frc, ebase, st, 1u, 0u);
                if constexpr (EXT) rk4_step<R, N, true, SV, true>(sys, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6, bt, B, a.h6lo);
                else if (a.kahan) rk4_step<R, N, true, SV>(sys, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6, bt, B);
                else rk4_step<R, N, false, SV>(sys, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6, bt, B);
            }
        } else {
            const R* bt = a.buf + (long long)(end - slot0) * SV * N * B + b;
#pragma unroll
            for (int i = 0; i < N; ++i) Q[i] = bt[i * B];
        }
#pragma unroll
        for (int i = 0; i < N; ++i) QN[i] = Q[i];
        // the step's state and stage inputs, as the forward computed them; small
        // systems load the next step's slot one step ahead (latency hidden)
        R fa = force_at(a.frc, ebase, (unsigned)(end - 1), 0u, 0u);
        R fb = force_at(a.frc, ebase, (unsigned)(end - 1), 0u, 1u);
        R fc = force_at(a.frc, ebase, (unsigned)(end - 1), 1u, 0u);
        constexpr bool PIPE = SV * N <= 16;
        RegVec<R, PIPE ? SV * N : 1> nxt;
        if constexpr (PIPE) {
            const R* bt = a.buf + (long long)(end - 1 - slot0) * SV * N * B + b;
#pragma unroll
            for (int i = 0; i < SV * N; ++i) nxt[i] = bt[i * B];
        }
        for (int t = end - 1; t >= start; --t) {
            RegVec<R, N> QC, Y2, Y3, Y4, QB, KB, YB;
            if (a.stored && t - kPrefetchSteps >= slot0) {
                const R* pf = a.buf + (long long)(t - kPrefetchSteps - slot0) * SV * N * B + b;
#pragma unroll
                for (int i = 0; i < SV * N; ++i) pk_prefetch_l2(pf + i * B);
            }
            if constexpr (PIPE) {
#pragma unroll
                for (int i = 0; i < N; ++i) {
                    QC[i] = nxt[i];
                    if constexpr (SV == 4) {
                        Y2[i] = nxt[N + i];
                        Y3[i] = nxt[2 * N + i];
                        Y4[i] = nxt[3 * N + i];
                    }
                }
                if (t > start) {
                    const R* bt = a.buf + (long long)(t - 1 - slot0) * SV * N * B + b;
#pragma unroll
                    for (int i = 0; i < SV * N; ++i) nxt[i] = bt[i * B];
                }
            } else {
                const R* bt = a.buf + (long long)(t - slot0) * SV * N * B + b;
#pragma unroll
                for (int i = 0; i < N; ++i) {
                    QC[i] = bt[i * B];
                    if constexpr (SV == 4) {
                        Y2[i] = bt[(N + i) * B];
                        Y3[i] = bt[(2 * N + i) * B];
                        Y4[i] = bt[(3 * N + i) * B];
                    }
                }
            }
            if (HSQ && a.g_sq && t >= a.sq_start) {
#pragma unroll
                for (int i = 0; i < N; ++i)
                    if (i < 64 && ((sq_mask >> i) & 1ull)) {
                        if constexpr (EXT) ext_add(LAM[i], CL[i], m::mul(gsq2h, QN[i]));
                        else if (a.kahan) kahan_add(LAM[i], CL[i], m::mul(gsq2h, QN[i]));
                        else LAM[i] = m::fma(gsq2h, QN[i], LAM[i]);
                    }
            }
            // the forcing of step t, read one step ahead (uc of step t-1 is ua of step t)
            const R ua = fa, ub = fb, uc = fc;
            if (t > start) {
                fc = fa;
                fa = force_at(a.frc, ebase, (unsigned)(t - 1), 0u, 0u);
                fb = force_at(a.frc, ebase, (unsigned)(t - 1), 0u, 1u);
            }
            if constexpr (SV == 1) {   // the stage inputs, recomputed
                sys.template rhs<true>(QC, QC, ua, K);
#pragma unroll
                for (int i = 0; i < N; ++i) Y2[i] = m::fma(a.h2, K[i], QC[i]);
                sys.template rhs<true>(Y2, Y2, ub, K);
#pragma unroll
                for (int i = 0; i < N; ++i) Y3[i] = m::fma(a.h2, K[i], QC[i]);
                sys.template rhs<true>(Y3, Y3, ub, K);
#pragma unroll
                for (int i = 0; i < N; ++i) Y4[i] = m::fma(a.h, K[i], QC[i]);
            }
            // QB sums the step's increment of LAM: onto LAM itself (plain), or
            // from 0 and then added with compensation (Kahan mode)
#pragma unroll
            for (int i = 0; i < N; ++i) {
                KB[i] = EXT ? LAM[i] : m::mul(a.h6, LAM[i]);
                QB[i] = a.kahan ? R(0) : LAM[i];
            }
            // extended-state mode: the stage weights carry no h/6 (it multiplies the
            // step's sum in ext_update and the parameter sums below), and the
            // adjoint of the once-per-step term h f_lo(QC) adds h J_lo(QC)^T LAM
            RegVec<R, EXT ? N : 1> YC;
            if constexpr (EXT) sys.vjp_lo(QC, LAM, ua, YC);
            sys.vjp(Y4, KB, uc, YB, pacc);
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const R sb = EXT ? LAM[i] : m::mul(a.h6, LAM[i]);
                QB[i] = m::add(QB[i], YB[i]);
                KB[i] = m::fma(a.h, YB[i], m::mul(R(2), sb));
            }
            sys.vjp(Y3, KB, ub, YB, pacc);
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const R sb = EXT ? LAM[i] : m::mul(a.h6, LAM[i]);
                QB[i] = m::add(QB[i], YB[i]);
                KB[i] = m::fma(a.h2, YB[i], m::mul(R(2), sb));
            }
            sys.vjp(Y2, KB, ub, YB, pacc);
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const R sb = EXT ? LAM[i] : m::mul(a.h6, LAM[i]);
                QB[i] = m::add(QB[i], YB[i]);
                KB[i] = m::fma(a.h2, YB[i], sb);
            }
            sys.vjp(QC, KB, ua, YB, pacc);
#pragma unroll
            for (int i = 0; i < N; ++i) {
                if constexpr (EXT) ext_update(LAM[i], CL[i], m::add(QB[i], YB[i]), YC[i], a.h, a.h6, a.h6lo);
                else if (a.kahan) kahan_add(LAM[i], CL[i], m::add(QB[i], YB[i]));
                else LAM[i] = m::add(QB[i], YB[i]);
                QN[i] = QC[i];
            }
            if constexpr (PBREG) {   // compensated FP32 sums of this chunk (see PK)
#pragma unroll
                for (int p = 0; p < P; ++p) {
                    kahan_add(PK[p], PKC[p], pacc[p]);
                    pacc[p] = R(0);
                }
            } else if (STEP_ACC) {   // the same compensated sums, in a.pk
                for (int p = 0; p < P; ++p) {
                    R sm = a.pk[(long long)p * B + b], cm = a.pk[(long long)(P + p) * B + b];
                    kahan_add(sm, cm, pacc[p]);
                    a.pk[(long long)p * B + b] = sm;
                    a.pk[(long long)(P + p) * B + b] = cm;
                    pacc[p] = R(0);
                }
            }
        }
        if constexpr (STEP_ACC && !PBREG) {
            for (int p = 0; p < P; ++p) {
                const double sum = (double)a.pk[(long long)p * B + b] - (double)a.pk[(long long)(P + p) * B + b];
                PB[p] = EXT ? M<double>::fma(h6d, sum, PB[p]) : PB[p] + sum;
                a.pk[(long long)p * B + b] = R(0);
                a.pk[(long long)(P + p) * B + b] = R(0);
            }
        }
        if constexpr (PBREG) {   // the chunk's compensated FP32 sums into the FP64 totals
#pragma unroll
            for (int p = 0; p < P; ++p) {
                const double sum = (double)PK[p] - (double)PKC[p];
                PR[p] = EXT ? M<double>::fma(h6d, sum, PR[p]) : PR[p] + sum;
                PK[p] = R(0);
                PKC[p] = R(0);
            }
        }
    }
    if constexpr (PBREG) {
#pragma unroll
        for (int p = 0; p < P; ++p) PB[p] = PR[p];
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
        a.dx0[i * B + b] = LAM[i];
        if ((a.phase == 2 && a.kahan) || EXT) a.lamc[i * B + b] = CL[i];
    }
}

// Exact discrete adjoint of the RK4 map for one instance (generic storage):
// forward pass with checkpoints every C steps (state and Kahan compensation
// before step k*C), then per chunk in reverse: recompute the chunk's states
// into buf and sweep backward.  The reverse of one step, with lam = dL/dQ_{s+1}:
//   kb4 = h/6 lam, kb3 = kb2 = 2 h/6 lam, kb1 = h/6 lam
//   yb4 = J(Y4)^T kb4; kb3 += h  yb4
//   yb3 = J(Y3)^T kb3; kb2 += h/2 yb3
//   yb2 = J(Y2)^T kb2; kb1 += h/2 yb2
//   yb1 = J(Q)^T  kb1; lam_s = lam + yb4 + yb3 + yb2 + yb1
// with parameter gradients accumulated in FP64 at every VJP.
template <typename R, class Sys>
__device__ void adj_run_generic(const Sys& sys, const AdjArgs<R>& a, int b) {
    typedef M<R> m;
    const int n = sys.dim();
    const long long B = a.B;
    R* base = a.scratch + b;
    GVec<R> Q{base, B}, Cm{base + (long long)n * B, B}, S{base + 2LL * n * B, B},
        K{base + 3LL * n * B, B}, Mi{base + 4LL * n * B, B}, Y2{base + 5LL * n * B, B},
        Y3{base + 6LL * n * B, B}, Y4{base + 7LL * n * B, B}, LAM{base + 8LL * n * B, B},
        QB{base + 9LL * n * B, B}, KB{base + 10LL * n * B, B}, YB{base + 11LL * n * B, B},
        QN{base + 12LL * n * B, B}, CL{base + 13LL * n * B, B};   // CL: LAM compensation (Kahan mode)
    GVec<double> PB{a.pbar + b, B};
    const long long ebase = (long long)a.exc_index[b] * (long long)a.frc.len;
    const int P = sys.g.P;
    for (int p = 0; p < P; ++p) PB[p] = 0.0;
    for (int i = 0; i < n; ++i) { Q[i] = a.x0[i * B + b]; Cm[i] = R(0); }
    // forward pass with checkpoints
    for (int t = 0; t < a.nsteps; ++t) {
        if (t % a.C == 0) {
            R* ck = a.ckpt + (long long)(t / a.C) * 2 * n * B + b;
            for (int i = 0; i < n; ++i) { ck[i * B] = Q[i]; ck[(n + i) * B] = Cm[i]; }
        }
        const unsigned st = (unsigned)t;
        const R ua = force_at(a.frc, ebase, st, 0u, 0u);
        const R ub = force_at(a.frc, ebase, st, 0u, 1u);
        const R uc = force_at(a.frc, ebase, st, 1u, 0u);
        if (a.kahan) rk4_step<R, 0, true>(sys, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6);
        else rk4_step<R, 0, false>(sys, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6);
    }
    for (int i = 0; i < n; ++i) { LAM[i] = a.g_final ? a.g_final[i * B + b] : R(0); CL[i] = R(0); }
    const R gsq2h = a.g_sq ? m::mul(m::mul(a.g_sq[b], R(2)), a.h) : R(0);
    for (int k = a.nck - 1; k >= 0; --k) {
        const int start = k * a.C;
        const int end = (start + a.C < a.nsteps) ? start + a.C : a.nsteps;
        const R* ck = a.ckpt + (long long)k * 2 * n * B + b;
        for (int i = 0; i < n; ++i) { Q[i] = ck[i * B]; Cm[i] = ck[(n + i) * B]; }
        for (int t = start; t < end; ++t) {
            R* bt = a.buf + (long long)(t - start) * n * B + b;
            for (int i = 0; i < n; ++i) bt[i * B] = Q[i];
            const unsigned st = (unsigned)t;
            const R ua = force_at(a.frc, ebase, st, 0u, 0u);
            const R ub = force_at(a.frc, ebase, st, 0u, 1u);
            const R uc = force_at(a.frc, ebase, st, 1u, 0u);
            if (a.kahan) rk4_step<R, 0, true>(sys, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6);
            else rk4_step<R, 0, false>(sys, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6);
        }
        for (int i = 0; i < n; ++i) QN[i] = Q[i];
        for (int t = end - 1; t >= start; --t) {
            GVec<R> QC{a.buf + (long long)(t - start) * n * B + b, B};
            if (a.g_sq && t >= a.sq_start)
                for (int i = 0; i < n; ++i)
                    if (i < 64 && ((a.sq_mask >> i) & 1ull)) {
                        if (a.kahan) {
                            R l = LAM[i], c = CL[i];
                            kahan_add(l, c, m::mul(gsq2h, QN[i]));
                            LAM[i] = l;
                            CL[i] = c;
                        } else {
                            LAM[i] = m::fma(gsq2h, QN[i], LAM[i]);
                        }
                    }
            const unsigned st = (unsigned)t;
            const R ua = force_at(a.frc, ebase, st, 0u, 0u);
            const R ub = force_at(a.frc, ebase, st, 0u, 1u);
            const R uc = force_at(a.frc, ebase, st, 1u, 0u);
            sys.template rhs<true>(QC, QC, ua, K);
            for (int i = 0; i < n; ++i) Y2[i] = m::fma(a.h2, K[i], QC[i]);
            sys.template rhs<true>(Y2, Y2, ub, K);
            for (int i = 0; i < n; ++i) Y3[i] = m::fma(a.h2, K[i], QC[i]);
            sys.template rhs<true>(Y3, Y3, ub, K);
            for (int i = 0; i < n; ++i) Y4[i] = m::fma(a.h, K[i], QC[i]);
            // kb4 = sb; qb = lam (plain) or the increment from 0 (Kahan mode)
            for (int i = 0; i < n; ++i) { KB[i] = m::mul(a.h6, LAM[i]); QB[i] = a.kahan ? R(0) : LAM[i]; }
            sys.vjp(Y4, KB, uc, YB, PB);
            for (int i = 0; i < n; ++i) {
                const R sb = m::mul(a.h6, LAM[i]);
                QB[i] = m::add(QB[i], YB[i]);
                KB[i] = m::fma(a.h, YB[i], m::mul(R(2), sb));
            }
            sys.vjp(Y3, KB, ub, YB, PB);
            for (int i = 0; i < n; ++i) {
                const R sb = m::mul(a.h6, LAM[i]);
                QB[i] = m::add(QB[i], YB[i]);
                KB[i] = m::fma(a.h2, YB[i], m::mul(R(2), sb));
            }
            sys.vjp(Y2, KB, ub, YB, PB);
            for (int i = 0; i < n; ++i) {
                const R sb = m::mul(a.h6, LAM[i]);
                QB[i] = m::add(QB[i], YB[i]);
                KB[i] = m::fma(a.h2, YB[i], sb);
            }
            sys.vjp(QC, KB, ua, YB, PB);
            for (int i = 0; i < n; ++i) {
                if (a.kahan) {
                    R l = LAM[i], c = CL[i];
                    kahan_add(l, c, m::add(QB[i], YB[i]));
                    LAM[i] = l;
                    CL[i] = c;
                } else {
                    LAM[i] = m::add(QB[i], YB[i]);
                }
                QN[i] = QC[i];
            }
        }
    }
    for (int i = 0; i < n; ++i) a.dx0[i * B + b] = LAM[i];
}

// __GpuDriver::_getGradient for one instance; the literal buffer simulation
// of the oracle (checkpoint slots, chunk recompute, frozen scratch slot T).
template <typename R, class FSys, class BSys>
__device__ void refgrad_run_generic(const FSys& fs, const BSys& bs, const RefGradArgs<R>& a, int b) {
    typedef M<R> m;
    const int nf = fs.dim(), na = bs.dim();
    const long long B = a.B;
    R* base = a.scratch + b;
    GVec<R> Q{base, B}, Cm{base + (long long)nf * B, B}, S{base + 2LL * nf * B, B},
        K{base + 3LL * nf * B, B}, Mi{base + 4LL * nf * B, B};
    R* ab = base + 5LL * nf * B;
    GVec<R> A{ab, B}, M1{ab + (long long)na * B, B}, M2{ab + 2LL * na * B, B},
        M3{ab + 3LL * na * B, B}, M4{ab + 4LL * na * B, B}, MI{ab + 5LL * na * B, B};
    const long long ebase = (long long)a.exc_index[b] * (long long)a.frc.len;
    const long long slotstride = (long long)nf * B;
    R* tr = a.traj + b;
    const int N = a.nsteps, C = a.C;
    for (int i = 0; i < nf; ++i) Q[i] = a.x0[i * B + b];
    long long idx = 0;
    for (int t = 0; t < N; ++t) {
        const unsigned st = (unsigned)t;
        rk4_step<R, 0, false>(fs, Q, Cm, S, K, Mi, force_at(a.frc, ebase, st, 0u, 0u),
                              force_at(a.frc, ebase, st, 0u, 1u), force_at(a.frc, ebase, st, 1u, 0u),
                              a.h, a.h2, a.h6);
        if (t % C == 0) {
            for (int i = 0; i < nf; ++i) tr[idx * slotstride + (long long)i * B] = Q[i];
            ++idx;
        }
    }
    for (int i = 0; i < na; ++i) A[i] = a.a0[i * B + b];
    long long T = -1;
    for (long long sp = a.S - 1; sp >= 1; --sp) {
        const long long start = sp * C;
        long long end, sb;
        if (sp == a.S - 1) { end = N; sb = sp + (a.lastC - 1); }
        else { end = start + C; sb = sp + (C - 1); }
        for (int i = 0; i < nf; ++i) Q[i] = tr[sp * slotstride + (long long)i * B];
        idx = 0;
        for (long long t = start; t < end; ++t) {
            const unsigned st = (unsigned)t;
            rk4_step<R, 0, false>(fs, Q, Cm, S, K, Mi, force_at(a.frc, ebase, st, 0u, 0u),
                                  force_at(a.frc, ebase, st, 0u, 1u), force_at(a.frc, ebase, st, 1u, 0u),
                                  a.h, a.h2, a.h6);
            for (int i = 0; i < nf; ++i) tr[(idx + sp) * slotstride + (long long)i * B] = Q[i];
            ++idx;
        }
        if (T < 0) T = sb;
        long long spc = sb;
        GVec<R> TG{tr + T * slotstride, B};
        for (long long t = end - 1; t >= start; --t) {
            GVec<R> CUR{tr + spc * slotstride, B}, PRV{tr + (spc - 1) * slotstride, B};
            for (int i = 0; i < nf; ++i) TG[i] = CUR[i];
            bs.template rhs<false>(A, TG, R(0), M1);
            for (int i = 0; i < na; ++i) MI[i] = m::fma(a.h2, M1[i], A[i]);
            for (int i = 0; i < nf; ++i) TG[i] = m::mul(R(0.5), m::add(CUR[i], PRV[i]));
            bs.template rhs<false>(MI, TG, R(0), M2);
            for (int i = 0; i < na; ++i) MI[i] = m::fma(a.h2, M2[i], A[i]);
            bs.template rhs<false>(MI, TG, R(0), M3);
            for (int i = 0; i < na; ++i) MI[i] = m::fma(a.h, M3[i], A[i]);
            for (int i = 0; i < nf; ++i) TG[i] = PRV[i];
            bs.template rhs<false>(MI, TG, R(0), M4);
            for (int i = 0; i < na; ++i) {
                R sum = m::fma(R(2), M2[i], M1[i]);
                sum = m::fma(R(2), M3[i], sum);
                sum = m::add(sum, M4[i]);
                A[i] = m::fma(a.h6, sum, A[i]);
            }
            --spc;
        }
        if (sp == a.save) break;
    }
    for (int i = 0; i < na; ++i) a.out[i * B + b] = A[i];
}


// ---- warp-sliced systems ----------------------------------------------------
// For large state sizes the L warps of a block share 32 systems (lane = system):
// warp w owns a slice of the components (its state, compensation, stage vectors
// and the values of its destinations' terms in registers) and computes the
// right-hand side of its own destinations in the canonical order.  The
// components another slice reads are published to shared memory after every
// stage ([2 buffers][NP published][32 lanes]; a stage reads one buffer and
// writes the other, so one CTA barrier per stage suffices).  The warps run
// different (generated) code, so the barrier is the non-aligned
// barrier.sync, which may be reached from different instructions.  Every
// component sees the same operations in the same order as in rk4_step, so
// the results equal the thread-per-system kernels and the oracle bit for bit.
#ifndef PK_HOST_EMU
__device__ __forceinline__ unsigned char* pk_dyn_smem() {
    extern __shared__ __align__(16) unsigned char pk_smem_[];
    return pk_smem_;
}
__device__ __forceinline__ void pk_block_sync() { asm volatile("barrier.sync 0;" ::: "memory"); }
__device__ __forceinline__ unsigned pk_warp_max(unsigned v) { return __reduce_max_sync(0xffffffffu, v); }
#endif

// Steps rc.nsteps (<= T) of one system from rc.step0 with the block-uniform
// trip count T: steps past the system's own count leave its state and
// reducers untouched (serving pools mix slots at different steps in a block).
// `out` enables the stores of this lane (trajectory).
// One RK4 step of the slice (the operations of rk4_step): Q's foreign
// components are read from b0, the stage vectors pass through b1 and b0, and
// the new Q is published to b0.  act = false leaves Q and Cm unchanged.
//
// SL::ROLL: the four stages run as a rolled loop, so each slice's right-hand
// side appears once in the code.  The warps of a block execute different
// code; with large slices the unrolled stages of the warps sharing an SM
// sub-partition overflow its instruction cache (fetch stalls dominated), with
// small slices the unrolled form is faster (fewer instructions).
//
// NSTG: the slice's components of the state (1), and of the stage inputs Y2,
// Y3, Y4 (4), are also stored to stg + j part ([N][B] each) when `store`: one
// slot of an adjoint trajectory (as rk4_step).
// EXT: extended-state step (as rk4_step): the slice's part of h f_lo(Q) is
// evaluated with stage 1, from the same published Q.
template <typename R, bool KAHAN, int NSTG = 0, bool EXT = false, class SL, class V>
__device__ __forceinline__ void ws_step(const SL& sl, R* b0, R* b1, V& Q, V& Cm, V& S, V& K, V& Mi, R ua, R ub,
                                        R uc, R h, R h2, R h6, bool act, R* stg = nullptr, long long part = 0,
                                        long long sB = 0, int b = 0, bool store = false, R h6lo = R(0)) {
    typedef M<R> m;
    constexpr int MM = SL::MM;
    RegVec<R, EXT ? MM : 1> Kc;
#pragma unroll
    for (int i = 0; i < MM; ++i) Mi[i] = Q[i];   // stage 1 evaluates at Q
    if constexpr (NSTG >= 1) {
        if (store) sl.store_vec(Q, stg, sB, b);
    }
#pragma unroll(SL::ROLL ? 1 : 4)
    for (int st = 0; st < 4; ++st) {
        const R u = st == 0 ? ua : (st == 3 ? uc : ub);
        if constexpr (EXT) {
            if (st == 0) sl.rhs_lo(Mi, b0, u, Kc);
        }
        sl.rhs(Mi, (st & 1) ? b1 : b0, u, K);
        if (st == 3) {
#pragma unroll
            for (int i = 0; i < MM; ++i) {
                const R sum = m::add(S[i], K[i]);
                if constexpr (EXT) {
                    R hi = Q[i], lo = Cm[i];
                    ext_update(hi, lo, sum, Kc[i], h, h6, h6lo);
                    if (act) { Q[i] = hi; Cm[i] = lo; }
                } else if (KAHAN) {
                    const R inc = m::mul(h6, sum);
                    const R y = m::sub(inc, Cm[i]);
                    const R t = m::add(Q[i], y);
                    const R c = m::sub(m::sub(t, Q[i]), y);
                    if (act) { Cm[i] = c; Q[i] = t; }
                } else {
                    const R t = m::fma(h6, sum, Q[i]);
                    if (act) Q[i] = t;
                }
            }
            sl.publish(Q, b0);
        } else {
            const R c = st == 2 ? h : h2;
            if (st == 0) {
#pragma unroll
                for (int i = 0; i < MM; ++i) { S[i] = K[i]; Mi[i] = m::fma(c, K[i], Q[i]); }
            } else {
#pragma unroll
                for (int i = 0; i < MM; ++i) { S[i] = m::fma(R(2), K[i], S[i]); Mi[i] = m::fma(c, K[i], Q[i]); }
            }
            if constexpr (NSTG == 4) {
                if (store) sl.store_vec(Mi, stg + (long long)(st + 1) * part, sB, b);
            }
            sl.publish(Mi, (st & 1) ? b0 : b1);
        }
        pk_block_sync();
    }
}

// HTRAJ: as fwd_core_iv (1 states after every traj_every-th step, 2 the
// adjoint trajectory, 3 checkpoints).
template <typename R, bool KAHAN, bool HMAX, bool HSQ, int HTRAJ, int N, bool EXT = false, class SL, class V>
__device__ __forceinline__ void ws_core(const SL& sl, const FwdArgs<R>& a, const Forcing<R>& frc, R* sm, int b,
                                        bool out, const RunCtx& rc, unsigned T, V& Q, V& Cm, V& Mx, R& sq,
                                        R& sqc) {
    R* const b0 = sm;
    R* const b1 = sm + SL::NP * 32;
    const long long B = a.B;
    V S, K, Mi;
    sl.publish(Q, b0);
    pk_block_sync();
    // the forcing of step s is read during step s - 1 (its ua is the uc before)
    R na = R(0), nb = R(0), nc = R(0);
    if (SL::FORCED) {
        na = force_at(frc, rc.ebase, rc.step0, 0u, 0u);
        nb = force_at(frc, rc.ebase, rc.step0, 0u, 1u);
        nc = force_at(frc, rc.ebase, rc.step0, 1u, 0u);
    }
    for (unsigned s = 0; s < T; ++s) {
        const bool act = s < rc.nsteps;
        const unsigned step = rc.step0 + s;
        const R ua = na, ub = nb, uc = nc;
        if (SL::FORCED && s + 1 < T) {
            na = nc;
            nb = force_at(frc, rc.ebase, step + 1u, 0u, 1u);
            nc = force_at(frc, rc.ebase, step + 1u, 1u, 0u);
        }
        if constexpr (HTRAJ == 3) {   // checkpoint: state and compensation before the step
            if (out && act && step % (unsigned)a.traj_every == 0u) {
                R* ck = a.traj + (long long)(step / (unsigned)a.traj_every) * 2 * N * B;
                sl.store_vec(Q, ck, B, b);
                sl.store_vec(Cm, ck + (long long)N * B, B, b);
            }
        }
        if constexpr (HTRAJ == 2)
            ws_step<R, KAHAN, adj_slot_vecs<R>(), EXT>(sl, b0, b1, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6, act,
                                                       a.traj + (long long)(step - a.step0) * adj_slot_vecs<R>() * N * B,
                                                       (long long)N * B, B, b, out && act, a.h6lo);
        else
            ws_step<R, KAHAN, 0, EXT>(sl, b0, b1, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6, act, nullptr, 0, 0, 0,
                                      false, a.h6lo);
        if (act) {
            if (HTRAJ == 1 && out) {
                const long long slot = traj_slot(step, a.step0, a.traj_every);
                if (slot >= 0 && slot < a.traj_slots) sl.store_traj(Q, a.traj + slot * N * B, B, b);
            }
            if (HMAX && (long long)step >= (long long)rc.max_start) sl.track_max(Q, Mx);
            if (HSQ && SL::SQOWN && (long long)step >= (long long)rc.sq_start) sl.template add_sq<KAHAN>(Q, b0, sq, sqc);
        }
    }
}

// Batch forward (FwdArgs): lane b of every warp of the block; `valid` is false
// for the lanes past the batch, which run a copy of the last system and store
// nothing.
template <typename R, bool KAHAN, bool HMAX, bool HSQ, int HTRAJ, int N, bool EXT = false, class SL>
__device__ __forceinline__ void ws_fwd(SL& sl, const FwdArgs<R>& a, R* sm, int b, bool valid) {
    typedef RegVec<R, SL::MM> V;
    const long long B = a.B;
    sl.load(a.vals, B, b);
    V Q, Cm, Mx;
    sl.load_vec(Q, a.state, B, b);
#pragma unroll
    for (int i = 0; i < SL::MM; ++i) { Cm[i] = R(0); Mx[i] = R(0); }
    if (KAHAN && a.comp) sl.load_vec(Cm, a.comp, B, b);   // restart from a checkpoint
    R sq = R(0), sqc = R(0);
    RunCtx rc;
    rc.ebase = (long long)a.exc_index[b] * (long long)a.frc.len;
    rc.step0 = a.step0;
    rc.nsteps = (unsigned)a.nsteps;
    rc.max_start = a.max_start;
    rc.sq_start = a.sq_start;
    ws_core<R, KAHAN, HMAX, HSQ, HTRAJ, N, EXT>(sl, a, a.frc, sm, b, valid, rc, (unsigned)a.nsteps, Q, Cm, Mx, sq,
                                                sqc);
    if (!valid) return;
    sl.store_vec(Q, a.state, B, b);
    if (EXT && a.comp_out) sl.store_vec(Cm, a.comp_out, B, b);
    if (HTRAJ == 2) sl.store_vec(Q, a.traj + (long long)a.nsteps * adj_slot_vecs<R>() * N * B, B, b);
    if (HMAX) sl.store_max(Mx, a.out_max, B, b);
    if (HSQ && SL::SQOWN) a.out_sq[b] = sq;
}

// Serving-pool chunk (PoolArgs), as pool_run_iv: every busy slot of the
// block's 32 advances min(chunk, remaining) steps; warp 0 books the steps.
template <typename R, bool KAHAN, bool HMAX, bool HSQ, int N, class SL>
__device__ __forceinline__ void ws_pool(SL& sl, const PoolArgs<R>& p, R* sm, int b, bool valid, int warp) {
    typedef RegVec<R, SL::MM> V;
    const int rem = valid ? p.remain[b] : 0;
    const unsigned mine = rem > 0 ? (unsigned)(rem < p.chunk ? rem : p.chunk) : 0u;
    const unsigned T = pk_warp_max(mine);   // every warp of the block holds the same 32 slots
    if (T == 0u) return;
    const long long C = p.C;
    sl.load(p.vals, C, b);
    V Q, Cm, Mx;
    sl.load_vec(Q, p.state, C, b);
    if (KAHAN) sl.load_vec(Cm, p.comp, C, b);
    else {
#pragma unroll
        for (int i = 0; i < SL::MM; ++i) Cm[i] = R(0);
    }
    if (HMAX) sl.load_vec(Mx, p.mx, C, b);
    else {
#pragma unroll
        for (int i = 0; i < SL::MM; ++i) Mx[i] = R(0);
    }
    R sq = (HSQ && SL::SQOWN) ? p.sq[b] : R(0), sqc = (HSQ && SL::SQOWN) ? p.sqc[b] : R(0);
    FwdArgs<R> a;
    a.B = p.C;
    a.h = p.h;
    a.h2 = p.h2;
    a.h6 = p.h6;
    a.traj = nullptr;
    a.traj_every = 1;
    a.traj_slots = 0;
    a.step0 = 0;
    // A slot without steps in this chunk (free, finished, or a lane past the
    // pool) still runs the block's step loop for the exchanges and barriers,
    // but reads no forcing: its signal fields may be stale or never written.
    Forcing<R> frc = p.frc;
    frc.len = mine ? p.len[b] : 0u;
    frc.total = mine ? p.lim[b] : 0;
    RunCtx rc;
    rc.ebase = mine ? p.ebase[b] : 0;
    rc.step0 = mine ? p.step[b] : 0u;
    rc.nsteps = mine;
    rc.max_start = p.max_start[b];
    rc.sq_start = p.sq_start[b];
    ws_core<R, KAHAN, HMAX, HSQ, 0, N>(sl, a, frc, sm, b, false, rc, T, Q, Cm, Mx, sq, sqc);
    if (mine == 0u) return;
    sl.store_vec(Q, p.state, C, b);
    if (KAHAN) sl.store_vec(Cm, p.comp, C, b);
    if (HMAX) sl.store_vec(Mx, p.mx, C, b);
    if (HSQ && SL::SQOWN) { p.sq[b] = sq; p.sqc[b] = sqc; }
    if (warp == 0) {
        p.step[b] = rc.step0 + mine;
        p.remain[b] = rem - (int)mine;
    }
}

// Exact discrete adjoint, warp-sliced (the algorithm and operation order of
// adj_run_jit).  Shared memory: regions for QC, Y2, Y3, Y4 (the first two
// double as the forward passes' stage buffers) and two for the VJP weights
// KB, each [NP][32].  The VJP of a slice is its gather form: the owner of
// component j adds every contribution to out[j] in the global scatter order
// of GenSys::vjp; the owner of destination i accumulates the gradients of the
// values of i's terms (PO of them: FP64 totals, STEP_ACC: per-step FP32 sums
// first).
template <typename R, bool KAHAN, bool HSQ, bool STEP_ACC, int N, bool EXT = false, class SL>
__device__ __forceinline__ void ws_adj(SL& sl, const AdjArgs<R>& a, R* sm, int b, bool valid) {
    typedef M<R> m;
    typedef RegVec<R, SL::MM> V;
    constexpr int MM = SL::MM, NP = SL::NP, PO = SL::PO;
    const long long B = a.B;
    R* const rq = sm;
    R* const r2 = sm + NP * 32;
    R* const r3 = sm + 2 * NP * 32;
    R* const r4 = sm + 3 * NP * 32;
    R* const k0 = sm + 4 * NP * 32;
    R* const k1 = sm + 5 * NP * 32;
    // FP32 adjoints whose slices' gradient totals do not fit registers: the
    // compensated per-chunk totals in shared memory after the six regions,
    // two slots of 32 lanes per value (sum, compensation)
    R* const pkm = sm + 6 * NP * 32;
    constexpr int SV = adj_slot_vecs<R>();
    sl.load(a.vals, B, b);
    const long long ebase = (long long)a.exc_index[b] * (long long)a.frc.len;
    // FP64 totals in registers (FP64 path; FP32 with few values per slice), or
    // in pbar itself, the FP32 per-step sums (pst) added once per step (keeps
    // registers for the vectors).  Same additions in the same order either way.
    constexpr bool PBREG = !STEP_ACC || PO <= 16;
    RegVec<double, PBREG ? PO : 1> PB;
    RegVec<R, STEP_ACC ? PO : 1> pst;
    // FP32 with the totals in registers: the per-step sums go with
    // compensation into FP32 totals (PK, PKC), flushed into the FP64 totals
    // once per chunk (FP64 adds run at 1/64 of the FP32 rate on GB300)
    constexpr bool PKREG = STEP_ACC && PBREG;
    RegVec<R, PKREG ? PO : 1> PK, PKC;
#pragma unroll
    for (int p = 0; p < (PBREG ? PO : 1); ++p) PB[p] = 0.0;
#pragma unroll
    for (int p = 0; p < (PKREG ? PO : 1); ++p) { PK[p] = R(0); PKC[p] = R(0); }
#pragma unroll
    for (int p = 0; p < (STEP_ACC ? PO : 1); ++p) pst[p] = R(0);
    V Q, Cm, S, K, Mi;
    if (a.phase != 2 && !a.stored) {   // forward pass with checkpoints (phase 1: steps [t_begin, t_end))
        const int t0 = a.phase == 1 ? a.t_begin : 0, t1 = a.phase == 1 ? a.t_end : a.nsteps;
        if (t0 == 0) {
            if constexpr (STEP_ACC) {
                if (valid) sl.zero_pbar(a.pbar, B, b);
            }
            sl.load_vec(Q, a.x0, B, b);
            if constexpr (EXT) sl.load_vec(Cm, a.x0 + (long long)N * B, B, b);   // the low parts of x0
            else {
#pragma unroll
                for (int i = 0; i < MM; ++i) Cm[i] = R(0);
            }
        } else {
            const R* ck = a.ckpt + (long long)(t0 / a.C) * 2 * N * B;
            sl.load_vec(Q, ck, B, b);
            sl.load_vec(Cm, ck + (long long)N * B, B, b);
        }
        sl.publish(Q, rq);
        pk_block_sync();
        for (int t = t0; t < t1; ++t) {
            if (t % a.C == 0 && valid) {
                R* ck = a.ckpt + (long long)(t / a.C) * 2 * N * B;
                sl.store_vec(Q, ck, B, b);
                sl.store_vec(Cm, ck + (long long)N * B, B, b);
            }
            const unsigned st = (unsigned)t;
            const R ua = force_at(a.frc, ebase, st, 0u, 0u);
            const R ub = force_at(a.frc, ebase, st, 0u, 1u);
            const R uc = force_at(a.frc, ebase, st, 1u, 0u);
            ws_step<R, KAHAN, 0, EXT>(sl, rq, r2, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6, true, nullptr, 0, 0, 0,
                                      false, a.h6lo);
        }
        if (a.phase == 1) {   // the next segment starts from this checkpoint
            if (valid && t1 < a.nsteps && t1 % a.C == 0) {
                R* ck = a.ckpt + (long long)(t1 / a.C) * 2 * N * B;
                sl.store_vec(Q, ck, B, b);
                sl.store_vec(Cm, ck + (long long)N * B, B, b);
            }
            return;
        }
    }
    V LAM, QN, CL;   // CL: compensation of LAM (Kahan mode)
    const int khi = a.phase == 2 ? a.k_hi : a.nck - 1, klo = a.phase == 2 ? a.k_lo : 0;
    if (khi == a.nck - 1) {
        if constexpr (STEP_ACC) {   // no forward pass in this kernel zeroed the totals
            if (a.stored && valid) sl.zero_pbar(a.pbar, B, b);
        }
        if (a.g_final) sl.load_vec(LAM, a.g_final, B, b);
        else {
#pragma unroll
            for (int i = 0; i < MM; ++i) LAM[i] = R(0);
        }
#pragma unroll
        for (int i = 0; i < MM; ++i) CL[i] = R(0);
    } else {   // carried from the previous backward launch
        sl.load_vec(LAM, a.dx0, B, b);
        if (KAHAN) sl.load_vec(CL, a.lamc, B, b);
        else {
#pragma unroll
            for (int i = 0; i < MM; ++i) CL[i] = R(0);
        }
        if constexpr (PBREG) sl.load_pbar(PB, a.pbar, B, b);
    }
    const R gsq2h = a.g_sq ? m::mul(m::mul(a.g_sq[b], R(2)), a.h) : R(0);
    const double h6d = (double)a.h6 + (double)a.h6lo;   // h/6 (extended-state mode)
    for (int k = khi; k >= klo; --k) {
        const int start = k * a.C;
        const int end = (start + a.C < a.nsteps) ? start + a.C : a.nsteps;
        const int slot0 = a.stored ? a.slot_base : start;   // buf slot of step t: t - slot0
        if constexpr (STEP_ACC && !PKREG) sl.zero_pk(pkm);
        if (!a.stored) {
            const R* ck = a.ckpt + (long long)k * 2 * N * B;
            sl.load_vec(Q, ck, B, b);
            sl.load_vec(Cm, ck + (long long)N * B, B, b);
            sl.publish(Q, rq);
            pk_block_sync();
            for (int t = start; t < end; ++t) {   // slot: state (and FP64: stage inputs) of step t
                const unsigned st = (unsigned)t;
                const R ua = force_at(a.frc, ebase, st, 0u, 0u);
                const R ub = force_at(a.frc, ebase, st, 0u, 1u);
                const R uc = force_at(a.frc, ebase, st, 1u, 0u);
                ws_step<R, KAHAN, SV, EXT>(sl, rq, r2, Q, Cm, S, K, Mi, ua, ub, uc, a.h, a.h2, a.h6, true,
                                           a.buf + (long long)(t - start) * SV * N * B, (long long)N * B, B, b, valid,
                                           a.h6lo);
            }
        } else {
            sl.load_vec(Q, a.buf + (long long)(end - slot0) * SV * N * B, B, b);
        }
#pragma unroll
        for (int i = 0; i < MM; ++i) QN[i] = Q[i];
        // the step's slot as the forward computed it (own components: written by
        // this thread before the barriers above, or by an earlier kernel).  FP64
        // slots hold the stage inputs too, published to rq, r2, r3, r4 for the
        // other slices; small slices load the next step's slot one step ahead.
        constexpr bool PIPE = SV == 1 || MM <= 4;
        auto load_slot = [&](int t, V& q, V& y2, V& y3, V& y4) {
            const R* bt = a.buf + (long long)(t - slot0) * SV * N * B;
            sl.load_vec(q, bt, B, b);
            if constexpr (SV == 4) {
                sl.load_vec(y2, bt + (long long)N * B, B, b);
                sl.load_vec(y3, bt + 2LL * N * B, B, b);
                sl.load_vec(y4, bt + 3LL * N * B, B, b);
            }
        };
        V nQC, nY2, nY3, nY4;
        if constexpr (PIPE) load_slot(end - 1, nQC, nY2, nY3, nY4);
        R fa = force_at(a.frc, ebase, (unsigned)(end - 1), 0u, 0u);
        R fb = force_at(a.frc, ebase, (unsigned)(end - 1), 0u, 1u);
        R fc = force_at(a.frc, ebase, (unsigned)(end - 1), 1u, 0u);
        for (int t = end - 1; t >= start; --t) {
            V QC, Y2, Y3, Y4, QB, KB, YB;
            if (a.stored && t - kPrefetchSteps >= slot0) {
                const R* pf = a.buf + (long long)(t - kPrefetchSteps - slot0) * SV * N * B;
#pragma unroll
                for (int j = 0; j < SV; ++j) sl.prefetch_vec(pf + (long long)j * N * B, B, b);
            }
            if constexpr (PIPE) {
#pragma unroll
                for (int i = 0; i < MM; ++i) {
                    QC[i] = nQC[i];
                    if constexpr (SV == 4) { Y2[i] = nY2[i]; Y3[i] = nY3[i]; Y4[i] = nY4[i]; }
                }
                if (t > start) load_slot(t - 1, nQC, nY2, nY3, nY4);
            } else {
                load_slot(t, QC, Y2, Y3, Y4);
            }
            if (HSQ && a.g_sq && t >= a.sq_start) sl.template add_sq_grad<KAHAN, EXT>(LAM, CL, QN, gsq2h);
            // the forcing of step t, read one step ahead (uc of step t-1 is ua of step t)
            const R ua = fa, ub = fb, uc = fc;
            if (t > start) {
                fc = fa;
                fa = force_at(a.frc, ebase, (unsigned)(t - 1), 0u, 0u);
                fb = force_at(a.frc, ebase, (unsigned)(t - 1), 0u, 1u);
            }
#pragma unroll
            for (int i = 0; i < MM; ++i) {
                KB[i] = EXT ? LAM[i] : m::mul(a.h6, LAM[i]);   // extended-state mode: no h/6 (see adj_run_jit)
                QB[i] = KAHAN ? R(0) : LAM[i];   // the step's increment (Kahan) or LAM + it
            }
            V Yc;
            if constexpr (SV == 4) {
                sl.publish(QC, rq);
                sl.publish(Y2, r2);
                sl.publish(Y3, r3);
                sl.publish(Y4, r4);
                sl.publish(KB, k0);
                pk_block_sync();
#pragma unroll
                for (int i = 0; i < MM; ++i) Yc[i] = Y4[i];
            } else {
                // stages: Y2 = QC + h/2 f(QC), Y3 = QC + h/2 f(Y2), Y4 = QC + h f(Y3),
                // each published to its own region (rq, r2, r3, r4 follow each
                // other); rolled like ws_step so the right-hand side appears once
                sl.publish(QC, rq);
                sl.publish(KB, k0);
                pk_block_sync();
#pragma unroll
                for (int i = 0; i < MM; ++i) Yc[i] = QC[i];
#pragma unroll(SL::ROLL ? 1 : 3)
                for (int st = 0; st < 3; ++st) {
                    sl.rhs(Yc, rq + st * NP * 32, st == 0 ? ua : ub, K);
                    const R c = st == 2 ? a.h : a.h2;
#pragma unroll
                    for (int i = 0; i < MM; ++i) Yc[i] = m::fma(c, K[i], QC[i]);
                    if (st == 0) {
#pragma unroll
                        for (int i = 0; i < MM; ++i) Y2[i] = Yc[i];
                    } else if (st == 1) {
#pragma unroll
                        for (int i = 0; i < MM; ++i) Y3[i] = Yc[i];
                    } else {
#pragma unroll
                        for (int i = 0; i < MM; ++i) Y4[i] = Yc[i];
                    }
                    sl.publish(Yc, rq + (st + 1) * NP * 32);
                    pk_block_sync();
                }
            }
            // extended-state mode: h J_lo(QC)^T LAM, from QC (rq) and LAM (= KB, k0)
            V YC;
            if constexpr (EXT) sl.vjp_lo(QC, rq, KB, k0, ua, YC);
            // reverse sweep: VJPs at Y4, Y3, Y2, QC with weights from k0, k1, k0, k1
#pragma unroll(SL::ROLL ? 1 : 4)
            for (int st = 0; st < 4; ++st) {
                if (st == 1) {
#pragma unroll
                    for (int i = 0; i < MM; ++i) Yc[i] = Y3[i];
                } else if (st == 2) {
#pragma unroll
                    for (int i = 0; i < MM; ++i) Yc[i] = Y2[i];
                } else if (st == 3) {
#pragma unroll
                    for (int i = 0; i < MM; ++i) Yc[i] = QC[i];
                }   // st == 0: Yc holds Y4
                const R u = st == 0 ? uc : (st == 3 ? ua : ub);
                R* const yb = rq + (3 - st) * NP * 32;
                if constexpr (STEP_ACC) sl.vjp(Yc, yb, KB, (st & 1) ? k1 : k0, u, YB, pst);
                else sl.vjp(Yc, yb, KB, (st & 1) ? k1 : k0, u, YB, PB);
                if (st == 3) break;
                const R c = st == 0 ? a.h : a.h2;
#pragma unroll
                for (int i = 0; i < MM; ++i) {
                    const R sb = EXT ? LAM[i] : m::mul(a.h6, LAM[i]);
                    QB[i] = m::add(QB[i], YB[i]);
                    KB[i] = m::fma(c, YB[i], st < 2 ? m::mul(R(2), sb) : sb);
                }
                sl.publish(KB, (st & 1) ? k0 : k1);
                pk_block_sync();
            }
#pragma unroll
            for (int i = 0; i < MM; ++i) {
                if constexpr (EXT) ext_update(LAM[i], CL[i], m::add(QB[i], YB[i]), YC[i], a.h, a.h6, a.h6lo);
                else if (KAHAN) kahan_add(LAM[i], CL[i], m::add(QB[i], YB[i]));
                else LAM[i] = m::add(QB[i], YB[i]);
                QN[i] = QC[i];
            }
            if constexpr (STEP_ACC) {
                if constexpr (PBREG) {
#pragma unroll
                    for (int p = 0; p < PO; ++p) kahan_add(PK[p], PKC[p], pst[p]);
                } else {   // the same compensated sums, in shared memory
                    sl.add_pk(pst, pkm);
                }
#pragma unroll
                for (int p = 0; p < PO; ++p) pst[p] = R(0);
            }
            pk_block_sync();   // every slice is done with this step's regions
        }
        if constexpr (PKREG) {   // the chunk's compensated FP32 sums into the FP64 totals
#pragma unroll
            for (int p = 0; p < PO; ++p) {
                const double sum = (double)PK[p] - (double)PKC[p];
                PB[p] = EXT ? M<double>::fma(h6d, sum, PB[p]) : PB[p] + sum;
                PK[p] = R(0);
                PKC[p] = R(0);
            }
        } else if constexpr (STEP_ACC) {
            if (valid) sl.template flush_pk<EXT>(pkm, a.pbar, B, b, h6d);
        }
    }
    if (!valid) return;
    sl.store_vec(LAM, a.dx0, B, b);
    if ((KAHAN && a.phase == 2) || EXT) sl.store_vec(CL, a.lamc, B, b);
    if constexpr (PBREG) sl.store_pbar(PB, a.pbar, B, b);
}

}  // namespace pk
