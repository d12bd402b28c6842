// pk_args.h -- kernel argument blocks shared by the host engine, the nvcc-built
// generic kernels and the NVRTC-built pattern-specialised kernels.  Plain
// structs of pointers and scalars only: the same text is compiled by g++,
// nvcc and NVRTC, so the layouts agree by construction.
#pragma once

namespace pk {

// Excitation table in the compute precision plus the forcing mode.
// w == 0: sample and hold (src/kernels.cu:72-89); else window W = 2^lw
// interpolation with weights im[0..2W) (src/kernels.cu:97-126).
template <typename R>
struct Forcing {
    const R* x;          // [n_exc * len], one row per signal
    const R* im;         // 2*W weights: row 0 next-sample, row 1 current-sample
    long long total;     // n_exc * len
    unsigned len;
    unsigned w;
    unsigned lw;
    unsigned pad_;
};

// Generic (interpreted) pattern description: device array laid out as
// k_ptr[n+1] | k_col[k] | g_idx[3g] | l_idx[4l] | p_idx[5p] | f_idx[f].
struct GenPattern {
    const int* data;
    int n;
    int n_sp;
    int k_nnz, g_nnz, l_nnz, p_nnz, f_nnz;
    int P;
};

// Forward integration of a batch: one instance per thread.
template <typename R>
struct FwdArgs {
    const R* vals;              // [P][B] per-instance values (system-interleaved)
    R* state;                   // [n][B] initial state in, final state out
    const int* exc_index;       // [B]
    R* scratch;                 // generic kernels: [6n][B] work vectors
    R* out_max;                 // [n_max][B]
    R* out_sq;                  // [B] raw sum of squares (times h on the host)
    R* traj;                    // [slots][n][B] states after steps t with t % traj_every == 0
    long long traj_slots;
    int traj_every;
    int pad_;
    Forcing<R> frc;
    GenPattern gp;              // generic kernels only
    R h, h2, h6;
    int B;
    unsigned step0;
    int nsteps;
    int max_start;
    int sq_start;
    unsigned long long max_mask;   // components reduced by max |q|
    unsigned long long sq_mask;    // components reduced by sum q^2
    // Restart (pattern-specialised kernels): the initial Kahan compensation
    // [n][B], or null for zero.  With trajectory mode 3 (checkpoints) the
    // kernels store the state and compensation before every step t with
    // t % traj_every == 0 to traj + (t / traj_every) [2n][B].
    const R* comp;
    // Extended-state mode (FP32 stages, double-float state): comp holds the
    // initial low parts, comp_out receives the final ones ([n][B]), vals holds
    // [2P][B] (high parts, then the low parts of the FP64 values), and h6lo is
    // the low part of h/6 (h/6 = h6 + h6lo to about 48 bits).
    R* comp_out;
    R h6lo;
};

// Serving pool: C slots of one pattern, each slot an instance of some request
// at its own step index; one launch advances every busy slot by `chunk` steps.
template <typename R>
struct PoolArgs {
    const R* vals;              // [P][C]
    R* state;                   // [n][C]
    R* comp;                    // [n][C] Kahan compensation, carried between chunks
    R* mx;                      // [n][C] running max |q|
    R* sq;                      // [C] running sum q^2
    R* sqc;                     // [C] its compensation
    unsigned* step;             // [C] next step index
    int* remain;                // [C] steps left (<= 0: free slot)
    const long long* ebase;     // [C] first sample of the slot's signal row in the arena
    const long long* lim;       // [C] end of the slot's request table in the arena
    const unsigned* len;        // [C] signal length of the slot's request
    const int* max_start;       // [C]
    const int* sq_start;        // [C]
    Forcing<R> frc;             // x = the signal arena (len / total per slot)
    R h, h2, h6;
    int C;
    int chunk;
};

// Exact discrete adjoint of the RK4 map with sqrt(N) checkpoints.
template <typename R>
struct AdjArgs {
    const R* vals;              // [P][B]
    const R* x0;                // [n][B]
    const int* exc_index;       // [B]
    R* ckpt;                    // [nck][2n][B] state + compensation at steps k*C
    R* buf;                     // per step a slot: the state (FP64: and stage inputs Y2, Y3, Y4),
                                // [adj_slot_vecs][n][B]; slots [C] of the recomputed chunk, or
                                // (stored) [nsteps] + the final state (generic kernels: [C][n][B])
    R* scratch;                 // generic kernels: [16n][B]
    double* pbar;               // [P][B] parameter gradients (FP64 accumulation)
    R* dx0;                     // [n][B]
    const R* g_final;           // [n][B] or null
    const R* g_sq;              // [B] or null
    Forcing<R> frc;
    GenPattern gp;
    R h, h2, h6;
    int B;
    int nsteps;
    int C;
    int nck;
    int kahan;
    int sq_start;
    unsigned long long sq_mask;
    // Launch split (pattern-specialised kernels): phase 0 = the whole adjoint in
    // one launch; 1 = forward pass over steps [t_begin, t_end) (multiples of C
    // except t_end = nsteps), state carried in the checkpoints; 2 = backward
    // over chunks k_hi down to k_lo, the adjoint state carried in dx0 (and its
    // compensation in lamc).  Short launches let other streams' work in.
    int phase;
    int t_begin, t_end;
    int k_lo, k_hi;
    R* lamc;                    // [n][B] (Kahan mode; extended-state mode: low parts of the adjoint state)
    // Stored trajectory: buf already holds the slots of steps slot_base ..
    // (slot t - slot_base) and the state after the last of them (state part of
    // the next slot), written by a forward kernel launched first, so there is
    // no checkpoint pass and no chunk recompute in this kernel; chunks only
    // group the backward launches.  slot_base = 0: the whole trajectory.
    int stored;
    int slot_base;
    // Extended-state mode: vals [2P][B] (high, low parts), x0 [2n][B] (high,
    // low parts), h6lo the low part of h/6; parameter gradients are summed
    // per step without the h/6 factor and added as (h6 + h6lo) * sum in FP64.
    int ext;
    R h6lo;
    // FP32 adjoints: [2P][B] compensated FP32 totals of the chunk's gradient
    // sums (sum, compensation) for the values whose totals do not stay in
    // registers; flushed into pbar (FP64) at the end of every chunk
    R* pk;
};

// __GpuDriver::_getGradient semantics (see the oracle for the quirk list).
template <typename R>
struct RefGradArgs {
    const R* fvals;             // [Pf][B]
    const R* bvals;             // [Pb][B]
    const R* x0;                // [nf][B]
    const R* a0;                // [na][B]
    const int* exc_index;       // [B]
    R* traj;                    // [slots][nf][B]
    R* scratch;                 // generic kernels: [8(nf+na)][B]
    R* out;                     // [na][B]
    Forcing<R> frc;
    GenPattern fgp;
    GenPattern bgp;
    R h, h2, h6;
    int B;
    int nsteps;
    int S;
    int C;
    int lastC;
    int save;
    long long slots;
};

}  // namespace pk
