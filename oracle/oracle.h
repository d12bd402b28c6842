/*
 * oracle.h -- CPU restatement of PASIf's RK4 hot path (TEST INFRASTRUCTURE).
 *
 * This library is the parity oracle of pasif_gb300.  Only the test suite, the
 * smoke check and the CPU-baseline leg of bench.py may load it; the product
 * path never calls it and never falls back to it.
 *
 * What it restates (file:line in the PASIf sources):
 *   - right-hand side  f = K.q + Gamma:(q x q) + Lambda:(q x q x q)
 *                        + Psi:(q x q x q x q) + F.u          src/kernels.cu:22-64
 *     with the Gamma/Lambda/Psi index roles (dest, source, setpoint...)  src/kernels.cu:52,56,61
 *     and the K product done by cusparseSpMM                    src/__GpuDriver.cu:785-838
 *   - forcing without interpolation (sample and hold, 0<idx<len)  src/kernels.cu:72-89
 *   - forcing with a W-window interpolation matrix             src/kernels.cu:97-126
 *   - the classical RK4 stage order and force times            src/__GpuDriver.cu:693-713
 *   - h, h/2, h/6 from h = 1/sampleRate                         src/__GpuDriver.cu:632-636
 *   - _getAmplitudes / _getTrajectory                          src/__GpuDriver.cu:416-500
 *   - _getGradient with its sqrt(N) checkpoint buffer, the
 *     frozen scratch slot and the setpoint copy kernels         src/__GpuDriver.cu:502-587,715-783
 *                                                              src/kernels.cu:163-196
 *
 * The reference sums the nonlinear terms with atomicAdd, so its FP order is
 * not fixed.  The oracle fixes one canonical order, which the CUDA kernels of
 * pasif_gb300 follow term for term:
 *   for every destination i, the terms in the order [CSR row of K | Gamma
 *   entries with dest i in COO order | Lambda | Psi | force entries] are dealt
 *   in turn to two partial sums (term k to sum k mod 2); a partial sum starts
 *   as the product of its first term, acc = term_without_last_factor *
 *   last_factor, and folds every further term with one fma; f[i] = sum0 +
 *   sum1 when i has two or more terms, sum0 with one, +0 with none.
 * Every function exists in double (suffix _d) and float (suffix _f); the float
 * versions round every input once to float and compute in float.
 */
#ifndef PASIF_ORACLE_H
#define PASIF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* One polynomial first-order system  dQ/dt = f(Q, Qp, u).  Q is the system's
 * own state ("source"), Qp the state the tensors' trailing indices read
 * ("setpoint"): Qp == Q for the forward problem, the forward trajectory for
 * the adjoint problem.  Values are always passed in double. */
typedef struct orc_sys {
    int n;                                   /* state size                      */
    int n_sp;                                /* setpoint state size (== n fwd)  */
    int k_nnz; const int* k_ptr; const int* k_col; const double* k_val;  /* CSR n x n */
    int g_nnz; const int* g_idx; const double* g_val;   /* (i, j, k)         */
    int l_nnz; const int* l_idx; const double* l_val;   /* (i, j, k, l)      */
    int p_nnz; const int* p_idx; const double* p_val;   /* (i, j, k, l, m)   */
    int f_nnz; const int* f_idx; const double* f_val;   /* force pattern     */
} orc_sys;

/* Excitation table and forcing mode shared by every instance of a run. */
typedef struct orc_exc {
    const double* x;      /* [n_exc * len] row-major, one row per signal      */
    int n_exc;
    int len;
    int w;                /* 0: sample and hold; else power-of-two window W    */
    const double* im;     /* >= 2*W interpolation weights (rows 0 and 1)       */
} orc_exc;

/* Reducers evaluated on the state after every step s >= start. */
typedef struct orc_red {
    int n_max; const int* max_comp; int max_start;      /* max |Q[c]|          */
    int n_sq;  const int* sq_comp;  int sq_start;       /* h * sum Q[c]^2      */
} orc_red;

/* Integrate one instance (one system driven by excitation row e) from x0 for
 * nsteps steps starting at step index step0.  mode: 0 plain, 1 Kahan update
 * (the Kahan mode only differs in the float build), 2 extended state (float
 * build: double-float state, FP32 residuals of the values applied once per
 * step, h/6 as h6 + h6lo; the output state is hi + lo).  Outputs (any may be NULL):
 * out_state[n], out_max[n_max], out_sq[1]. */
void orc_integrate_d(const orc_sys* s, const double* x0, int e, const orc_exc* ex,
                     double h, int step0, int nsteps, int mode, const orc_red* red,
                     double* out_state, double* out_max, double* out_sq);
void orc_integrate_f(const orc_sys* s, const double* x0, int e, const orc_exc* ex,
                     double h, int step0, int nsteps, int mode, const orc_red* red,
                     double* out_state, double* out_max, double* out_sq);

/* Batch of instances sharing one pattern: values[b][P] with
 * P = k_nnz+g_nnz+l_nnz+p_nnz+f_nnz in that order, x0[b][n], exc_index[b].
 * pattern->*_val pointers are ignored.  Runs with OpenMP over b. */
void orc_batch_forward_d(const orc_sys* pattern, int n_sys, const double* values,
                         const double* x0, const int* exc_index, const orc_exc* ex,
                         double h, int step0, int nsteps, int mode, const orc_red* red,
                         double* out_state, double* out_max, double* out_sq, int threads);
void orc_batch_forward_f(const orc_sys* pattern, int n_sys, const double* values,
                         const double* x0, const int* exc_index, const orc_exc* ex,
                         double h, int step0, int nsteps, int mode, const orc_red* red,
                         double* out_state, double* out_max, double* out_sq, int threads);

/* __GpuDriver::_getAmplitudes: the concatenated system replicated once per
 * excitation, integrated from step 0 for nsteps; out[e][n]. */
void orc_get_amplitudes_d(const orc_sys* s, const double* x0, const orc_exc* ex,
                          double h, int nsteps, double* out, int threads);

/* __GpuDriver::_getTrajectory(saveSteps): after step t with t % save == 0 the
 * extended state (all excitation copies) is stored; out holds
 * floor(n*n_exc*nsteps/save) values laid out [slot][e][n]. */
void orc_get_trajectory_d(const orc_sys* s, const double* x0, const orc_exc* ex,
                          double h, int nsteps, int save, double* out, long long out_len,
                          int threads);

/* __GpuDriver::_getGradient(save) for a fresh driver: the forward system fs
 * from x0, the adjoint system bs from a0 (terminal condition), both per
 * excitation copy; out[e][bs->n] is the final adjoint vector. */
void orc_get_gradient_d(const orc_sys* fs, const double* x0, const orc_sys* bs,
                        const double* a0, const orc_exc* ex, double h, int nsteps,
                        int save, double* out, int threads);

/* Exact discrete adjoint of the RK4 map (plain update) for a batch: loss
 * L_b = sum_c gf[b][c] * Q_N[c] + gsq[b] * h * sum_{s>=sq_start} sum_c Q_{s+1}[c]^2.
 * Outputs dvalues[b][P] and dx0[b][n].  Stores the whole trajectory. */
void orc_batch_adjoint_d(const orc_sys* pattern, int n_sys, const double* values,
                         const double* x0, const int* exc_index, const orc_exc* ex,
                         double h, int nsteps, const orc_red* red,
                         const double* g_final, const double* g_sq,
                         double* dvalues, double* dx0, int threads);

#ifdef __cplusplus
}
#endif
#endif
