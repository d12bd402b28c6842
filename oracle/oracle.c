/*
 * oracle.c -- CPU restatement of PASIf's RK4 hot path (TEST INFRASTRUCTURE:
 * loaded only by tests, the smoke check and bench.py's CPU-baseline leg).
 * Build: oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off); every fused
 * multiply-add is an explicit fma()/fmaf() so x86 and Arm builds agree bit
 * for bit.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#else
static int omp_get_max_threads(void) { return 1; }
#endif

#define R double
#define SFX(x) x##_d
#define FMA_ fma
#define FABS_ fabs
#define FMAX_ fmax
#include "oracle_core.inc"
#undef R
#undef SFX
#undef FMA_
#undef FABS_
#undef FMAX_

#define R float
#define SFX(x) x##_f
#define FMA_ fmaf
#define FABS_ fabsf
#define FMAX_ fmaxf
#include "oracle_core.inc"
#undef R
#undef SFX
#undef FMA_
#undef FABS_
#undef FMAX_

/* ---- drop-in level (double only, reel = double in the reference) -------- */

void orc_get_amplitudes_d(const orc_sys* s, const double* x0, const orc_exc* ex,
                          double h, int nsteps, double* out, int threads) {
    sysv_d v; excv_d xv;
    sysv_init_d(&v, s);
    excv_init_d(&xv, ex);
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int e = 0; e < ex->n_exc; ++e)
        integrate_v_d(&v, x0, e, &xv, h, 0, nsteps, 0, NULL, out + (long long)e * s->n, NULL, NULL);
    excv_free_d(&xv);
    sysv_free_d(&v);
}

/* src/__GpuDriver.cu:463-500 with forwardRungeKutta's save rule
 * (src/__GpuDriver.cu:668-687): the copy happens after the step. */
void orc_get_trajectory_d(const orc_sys* s, const double* x0, const orc_exc* ex,
                          double h, int nsteps, int save, double* out, long long out_len,
                          int threads) {
    sysv_d v; excv_d xv;
    const int n = s->n, E = ex->n_exc;
    sysv_init_d(&v, s);
    excv_init_d(&xv, ex);
    if (threads <= 0) threads = omp_get_max_threads();
    memset(out, 0, sizeof(double) * (size_t)out_len);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int e = 0; e < E; ++e) {
        double* Q = (double*)malloc(sizeof(double) * 6 * (size_t)n);
        double* w = Q + n;
        const double hr = h, h2 = h / 2.0, h6 = h / 6.0;
        memcpy(Q, x0, sizeof(double) * n);
        long long slot = 0;
        for (int t = 0; t < nsteps; ++t) {
            fwd_step_d(&v, Q, NULL, e, &xv, (unsigned)t, hr, h2, h6, w);
            if (t % save == 0) {
                long long base = slot * (long long)n * E + (long long)e * n;
                for (int i = 0; i < n; ++i)
                    if (base + i < out_len) out[base + i] = Q[i];
                ++slot;
            }
        }
        free(Q);
    }
    excv_free_d(&xv);
    sysv_free_d(&v);
}

/* __GpuDriver::_getGradient (src/__GpuDriver.cu:502-587) for one excitation
 * copy, including the quirks of the reference as it runs the first time:
 *  - S = floor(sqrt N), C = ceil(N/S), lastC = C - (S*C mod N)       :506-508
 *  - checkpoint slot i holds the state AFTER step i*C                :666-687
 *  - chunk sp restarts from slot sp at step index sp*C (one-step shift) :548-565
 *  - the recompute writes slot sp+i after step sp*C+i                :564-565
 *  - the backward graph is captured on the first chunk, so the scratch slot
 *    the setpoint kernels write (target_pos) stays at that chunk's start
 *    setpoint for every later chunk                                  :727-736,746-777
 *  - k1 sees traj[sp], k2/k3 the average of traj[sp] and traj[sp-1], k4
 *    traj[sp-1]; no forcing in the adjoint                            src/kernels.cu:163-196
 *  - chunk 0 is never integrated backward (loop stops at sp = 1)    :533
 *  - the adjoint state is chained from chunk to chunk                :743
 * The buffer gets one slot more than the reference's S+C-2 because the
 * reference writes one slot past its end when the last chunk is full. */
static void gradient_one_d(const sysv_d* fv, const double* x0, const sysv_d* bv, const double* a0,
                           int e, const excv_d* xv, double h, int N, int save, double* out) {
    const int nf = fv->s->n, na = bv->s->n;
    const int S = (int)sqrt((double)N);
    const int C = (int)ceil((double)N / (double)S);
    const int lastC = C - (int)(((long long)S * C) % N);
    const long long slots = (long long)S + C - 1;
    double* traj = (double*)calloc((size_t)(slots * nf), sizeof(double));
    double* Q = (double*)malloc(sizeof(double) * 6 * (size_t)nf);
    double* wf = Q + nf;
    double* A = (double*)malloc(sizeof(double) * 6 * (size_t)na);
    double *m1 = A + na, *m2 = A + 2 * na, *m3 = A + 3 * na, *m4 = A + 4 * na, *mi = A + 5 * na;
    const double h2 = h / 2.0, h6 = h / 6.0;
    long long T = -1;

    memcpy(Q, x0, sizeof(double) * nf);
    long long idx = 0;
    for (int t = 0; t < N; ++t) {
        fwd_step_d(fv, Q, NULL, e, xv, (unsigned)t, h, h2, h6, wf);
        if (t % C == 0) { memcpy(traj + idx * nf, Q, sizeof(double) * nf); ++idx; }
    }
    memcpy(A, a0, sizeof(double) * na);
    for (long long sp = S - 1; sp >= 1; --sp) {
        long long start = sp * C, end, sb;
        if (sp == S - 1) { end = N; sb = sp + (lastC - 1); }
        else { end = start + C; sb = sp + (C - 1); }
        memcpy(Q, traj + sp * nf, sizeof(double) * nf);
        idx = 0;
        for (long long t = start; t < end; ++t) {
            fwd_step_d(fv, Q, NULL, e, xv, (unsigned)t, h, h2, h6, wf);
            memcpy(traj + (idx + sp) * nf, Q, sizeof(double) * nf);
            ++idx;
        }
        if (T < 0) T = sb;
        long long spc = sb;
        double* tg = traj + T * nf;
        for (long long t = end - 1; t >= start; --t) {
            const double* cur = traj + spc * nf;
            const double* prv = traj + (spc - 1) * nf;
            memmove(tg, cur, sizeof(double) * nf);
            rhs_d(bv, A, tg, 0, 0.0, m1);
            for (int i = 0; i < na; ++i) mi[i] = fma(h2, m1[i], A[i]);
            for (int i = 0; i < nf; ++i) tg[i] = .5 * (cur[i] + prv[i]);
            rhs_d(bv, mi, tg, 0, 0.0, m2);
            for (int i = 0; i < na; ++i) mi[i] = fma(h2, m2[i], A[i]);
            rhs_d(bv, mi, tg, 0, 0.0, m3);
            for (int i = 0; i < na; ++i) mi[i] = fma(h, m3[i], A[i]);
            memmove(tg, prv, sizeof(double) * nf);
            rhs_d(bv, mi, tg, 0, 0.0, m4);
            for (int i = 0; i < na; ++i) {
                double sum = fma(2.0, m2[i], m1[i]);
                sum = fma(2.0, m3[i], sum);
                sum = sum + m4[i];
                A[i] = fma(h6, sum, A[i]);
            }
            --spc;
        }
        if (sp == save) break;
    }
    memcpy(out, A, sizeof(double) * na);
    free(traj); free(Q); free(A);
}

void orc_get_gradient_d(const orc_sys* fs, const double* x0, const orc_sys* bs,
                        const double* a0, const orc_exc* ex, double h, int nsteps,
                        int save, double* out, int threads) {
    sysv_d fv, bv; excv_d xv;
    sysv_init_d(&fv, fs);
    sysv_init_d(&bv, bs);
    excv_init_d(&xv, ex);
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int e = 0; e < ex->n_exc; ++e)
        gradient_one_d(&fv, x0, &bv, a0, e, &xv, h, nsteps, save, out + (long long)e * bs->n);
    excv_free_d(&xv);
    sysv_free_d(&bv);
    sysv_free_d(&fv);
}

/* ---- exact discrete adjoint of the RK4 map (plain update) --------------- */

/* out = J(y)^T w (out zeroed here) and pbar += (df/dp)^T w at state y with
 * forcing u.  Parameter order: K, Gamma, Lambda, Psi, F. */
static void vjp_d(const sysv_d* v, const double* y, const double* w, double u,
                  double* out, double* pbar) {
    const orc_sys* s = v->s;
    const int n = s->n;
    double* pk = pbar;
    double* pg = pk + s->k_nnz;
    double* pl = pg + s->g_nnz;
    double* pp = pl + s->l_nnz;
    double* pf = pp + s->p_nnz;
    for (int i = 0; i < n; ++i) out[i] = 0.0;
    for (int i = 0; i < n; ++i)
        for (int p = s->k_ptr[i]; p < s->k_ptr[i + 1]; ++p) {
            int j = s->k_col[p];
            out[j] = fma(v->kv[p], w[i], out[j]);
            pk[p] = fma(w[i], y[j], pk[p]);
        }
    for (int e = 0; e < s->g_nnz; ++e) {
        const int* ix = s->g_idx + 3 * e;
        double wi = w[ix[0]], yj = y[ix[1]], yk = y[ix[2]], a = v->gv[e] * wi;
        out[ix[1]] = fma(a, yk, out[ix[1]]);
        out[ix[2]] = fma(a, yj, out[ix[2]]);
        pg[e] = fma(wi * yj, yk, pg[e]);
    }
    for (int e = 0; e < s->l_nnz; ++e) {
        const int* ix = s->l_idx + 4 * e;
        double wi = w[ix[0]], yj = y[ix[1]], yk = y[ix[2]], yl = y[ix[3]], a = v->lv[e] * wi;
        out[ix[1]] = fma(a * yk, yl, out[ix[1]]);
        out[ix[2]] = fma(a * yj, yl, out[ix[2]]);
        out[ix[3]] = fma(a * yj, yk, out[ix[3]]);
        pl[e] = fma(wi * yj * yk, yl, pl[e]);
    }
    for (int e = 0; e < s->p_nnz; ++e) {
        const int* ix = s->p_idx + 5 * e;
        double wi = w[ix[0]], yj = y[ix[1]], yk = y[ix[2]], yl = y[ix[3]], ym = y[ix[4]];
        double a = v->pv[e] * wi;
        out[ix[1]] = fma(a * yk * yl, ym, out[ix[1]]);
        out[ix[2]] = fma(a * yj * yl, ym, out[ix[2]]);
        out[ix[3]] = fma(a * yj * yk, ym, out[ix[3]]);
        out[ix[4]] = fma(a * yj * yk, yl, out[ix[4]]);
        pp[e] = fma(wi * yj * yk * yl, ym, pp[e]);
    }
    for (int e = 0; e < s->f_nnz; ++e) pf[e] = fma(w[s->f_idx[e]], u, pf[e]);
}

static void adjoint_one_d(const sysv_d* v, const double* x0, int e, const excv_d* xv, double h,
                          int N, const orc_red* red, const double* gfin, double gsq,
                          double* pbar, double* dx0) {
    const int n = v->s->n;
    double* traj = (double*)malloc(sizeof(double) * (size_t)(N + 1) * n);
    double* w = (double*)malloc(sizeof(double) * 20 * (size_t)n);
    double *k1 = w + 5 * n, *k2 = w + 6 * n, *k3 = w + 7 * n, *k4 = w + 8 * n;
    double *y2 = w + 9 * n, *y3 = w + 10 * n, *y4 = w + 11 * n;
    double *lam = w + 12 * n, *kb1 = w + 13 * n, *kb2 = w + 14 * n, *kb3 = w + 15 * n;
    double *kb4 = w + 16 * n, *yb = w + 17 * n, *qb = w + 18 * n;
    const double h2 = h / 2.0, h6 = h / 6.0;
    memcpy(traj, x0, sizeof(double) * n);
    for (int s = 0; s < N; ++s) {
        memcpy(traj + (size_t)(s + 1) * n, traj + (size_t)s * n, sizeof(double) * n);
        fwd_step_d(v, traj + (size_t)(s + 1) * n, NULL, e, xv, (unsigned)s, h, h2, h6, w);
    }
    for (int i = 0; i < n; ++i) lam[i] = gfin ? gfin[i] : 0.0;
    for (int s = N - 1; s >= 0; --s) {
        const double* Qn = traj + (size_t)(s + 1) * n;
        const double* Q = traj + (size_t)s * n;
        if (red && red->n_sq > 0 && s >= red->sq_start)
            for (int c = 0; c < red->n_sq; ++c) {
                int ci = red->sq_comp[c];
                lam[ci] = fma(gsq * 2.0 * h, Qn[ci], lam[ci]);
            }
        double ua = force_d(xv, e, (unsigned)s, 0, 0);
        double ub = force_d(xv, e, (unsigned)s, 0, 1);
        double uc = force_d(xv, e, (unsigned)s, 1, 0);
        rhs_d(v, Q, Q, 1, ua, k1);
        for (int i = 0; i < n; ++i) y2[i] = fma(h2, k1[i], Q[i]);
        rhs_d(v, y2, y2, 1, ub, k2);
        for (int i = 0; i < n; ++i) y3[i] = fma(h2, k2[i], Q[i]);
        rhs_d(v, y3, y3, 1, ub, k3);
        for (int i = 0; i < n; ++i) y4[i] = fma(h, k3[i], Q[i]);
        for (int i = 0; i < n; ++i) {
            double sb = h6 * lam[i];
            kb1[i] = sb; kb2[i] = 2.0 * sb; kb3[i] = 2.0 * sb; kb4[i] = sb;
            qb[i] = lam[i];
        }
        vjp_d(v, y4, kb4, uc, yb, pbar);
        for (int i = 0; i < n; ++i) { qb[i] += yb[i]; kb3[i] = fma(h, yb[i], kb3[i]); }
        vjp_d(v, y3, kb3, ub, yb, pbar);
        for (int i = 0; i < n; ++i) { qb[i] += yb[i]; kb2[i] = fma(h2, yb[i], kb2[i]); }
        vjp_d(v, y2, kb2, ub, yb, pbar);
        for (int i = 0; i < n; ++i) { qb[i] += yb[i]; kb1[i] = fma(h2, yb[i], kb1[i]); }
        vjp_d(v, Q, kb1, ua, yb, pbar);
        for (int i = 0; i < n; ++i) lam[i] = qb[i] + yb[i];
    }
    memcpy(dx0, lam, sizeof(double) * n);
    free(traj); free(w);
}

void orc_batch_adjoint_d(const orc_sys* pattern, int n_sys, const double* values,
                         const double* x0, const int* exc_index, const orc_exc* ex,
                         double h, int nsteps, const orc_red* red,
                         const double* g_final, const double* g_sq,
                         double* dvalues, double* dx0, int threads) {
    const int P = pattern->k_nnz + pattern->g_nnz + pattern->l_nnz + pattern->p_nnz + pattern->f_nnz;
    const int n = pattern->n;
    excv_d xv;
    excv_init_d(&xv, ex);
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int b = 0; b < n_sys; ++b) {
        orc_sys inst; sysv_d v;
        instance_view_d(&inst, pattern, values + (long long)b * P);
        sysv_init_d(&v, &inst);
        double* pb = dvalues + (long long)b * P;
        for (int p = 0; p < P; ++p) pb[p] = 0.0;
        adjoint_one_d(&v, x0 + (long long)b * n, exc_index[b], &xv, h, nsteps, red,
                      g_final ? g_final + (long long)b * n : NULL, g_sq ? g_sq[b] : 0.0,
                      pb, dx0 + (long long)b * n);
        sysv_free_d(&v);
    }
    excv_free_d(&xv);
}
