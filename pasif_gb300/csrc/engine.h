// engine.h -- batched RK4 engine: plans (pattern + precision), device signal
// tables and device-resident batches of instances.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "jit.h"
#include "pattern.h"
#include "pk_args.h"

namespace pasif {

// kFP32Ext: FP32 stages, state and adjoint state as double-float pairs (hi +
// lo), the FP64 values split into FP32 high parts (stages) and low parts (a
// once-per-step residual term), h/6 carried as h6 + h6lo: the precision mode
// for long horizons, where FP32 rounding of the values and of h/6 acts as a
// systematic perturbation of the system.  Pattern-specialised kernels only.
enum Precision { kFP64 = 0, kFP32 = 1, kFP32Kahan = 2, kFP32Ext = 3 };
enum Memory { kHost = 0, kDevice = 1 };
enum KernelKind { kNone = 0, kGeneric = 1, kSpecialised = 2 };

// Steps per launch of a split exact adjoint (forward segments, backward chunk groups).
constexpr int kAdjLaunchSteps = 2048;
// Default device memory an exact adjoint may hold for a stored forward trajectory.
constexpr size_t kAdjStoreDefault = (size_t)16 << 30;
// Checkpoint intervals (of C steps) per launch of a split exact adjoint:
// about kAdjLaunchSteps * 16 / n steps, at most the nck intervals there are.
inline int adj_group(int n, int C, int nck) {
    const int steps = kAdjLaunchSteps * 16 / (n > 16 ? n : 16);
    const int g = steps / (C > 0 ? C : 1) > 1 ? steps / (C > 0 ? C : 1) : 1;
    return g < nck ? g : (nck > 1 ? nck : 1);
}

// Growable device allocation.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf();
    cudaError_t ensure(size_t n);
    void release();
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

// Excitation table in the compute precision (src/__GpuDriver.cu:343-381 keeps
// it as reel on the device).
struct Signals {
    bool f32 = false;
    int n_exc = 0;
    int len = 0;
    unsigned w = 0, lw = 0;
    DevBuf x, im;
    DevBuf stage;                  // host-format staging of signals_update
    std::vector<double> im_host;   // the 2W weights rounded to the compute precision
    template <typename R> pk::Forcing<R> forcing() const {
        pk::Forcing<R> f;
        f.x = x.as<R>();
        f.im = w ? im.as<R>() : nullptr;
        f.total = (long long)n_exc * len;
        f.len = (unsigned)len;
        f.w = w;
        f.lw = lw;
        f.pad_ = 0;
        return f;
    }
};

// Build a signal table; x and im are host or device (memory) pointers.
int signals_create(const double* x, int n_exc, int len, int window, const double* im, int precision,
                   int memory, cudaStream_t st, std::shared_ptr<Signals>* out, std::string* err);
// New table of the same window / weights / precision in the existing device
// buffers (grown when needed): no allocation once they are large enough.
int signals_update(Signals& s, const double* x, int n_exc, int len, int memory, cudaStream_t st, std::string* err);

struct Plan {
    Pattern pat;
    int precision = kFP64;
    bool generic_only = false;
    bool no_literals = false;   // every value loaded: one kernel for all batches
    int slicing = 0;            // warp-sliced kernels: 0 by size, 1 always, -1 never
    bool fast = false;          // PASIF_PLAN_FAST: fast thread-per-system forward kernels (not the oracle's bits)
    DevBuf gpat;           // flat pattern for the generic kernels (uploaded on first use)
    pk::GenPattern gen() const;
    int ensure_device(std::string* err);
};

int plan_create(const Pattern& pat, int precision, bool generic_only, std::shared_ptr<Plan>* out,
                std::string* err);

// Values shared by every instance (host values[n_sys][P]) as compile-time
// constants of the specialised kernels, in the compute precision of
// `precision`; kFP32Ext also the low parts.  No values: no literals.
Literals literals_of(const Pattern& pat, int precision, const double* values, int n_sys);

struct Reducers {
    std::vector<int> max_comp;   // ascending, < 64
    int max_start = 0;
    std::vector<int> sq_comp;    // ascending, < 64
    int sq_start = 0;
};

// Instances of one plan, resident on the device in [k][B] layout.
struct Batch {
    std::shared_ptr<Plan> plan;
    int B = 0;
    DevBuf vals, x0, state, exc, out_max, out_sq, scratch, stage, traj;
    DevBuf ckpt, buf, pbar, dx0, gfin, gsq, adj_stage, lamc, adj_state;
    DevBuf split;                 // kFP32Ext: values / x0 split into high and low parts (device inputs)
    DevBuf pkbuf;                 // FP32 adjoints: [2P][B] compensated per-chunk gradient totals
    // Replayed adjoints: streams on which the chunks' forward replays run ahead
    // of the backward sweep (one per chunk buffer), and their events
    static constexpr int kReplayBufs = 4;
    cudaStream_t replay_st[kReplayBufs] = {};
    cudaEvent_t ev_ckpt = nullptr, ev_replayed[kReplayBufs] = {}, ev_free[kReplayBufs] = {};
    int replay_prio = 0;
    Batch() = default;
    Batch(const Batch&) = delete;
    Batch& operator=(const Batch&) = delete;
    ~Batch();
    Literals lit;
    int n_max = 0;
    bool has_sq = false;
    bool inputs_set = false;      // values / x0 / exc_index uploaded for the current B
    int max_exc_ = -1;
    double last_h = 0.0;          // time step of the last forward (scales sum q^2)
    int last_kind = kNone;
    int last_adj_kind = kNone;
    JitKernel last_jit;
    std::string last_jit_error;
    // Device memory the exact adjoint may hold for the whole forward
    // trajectory ([slot_vecs() nsteps + 1][n][B]: every step's state, FP64 also
    // its stage inputs); within it the trajectory is written once by the
    // forward kernel and read back, otherwise chunks of it are recomputed from
    // checkpoints every ceil(sqrt(nsteps)) steps.  Same results either way.
    size_t adj_store_limit = kAdjStoreDefault;
    size_t slot_vecs() const { return f32() ? 1 : 4; }   // adj_slot_vecs of rk4_core.cuh
    bool adj_stores(int n_sys, int nsteps) const {
        return nsteps > 0 && (slot_vecs() * (size_t)nsteps + 1) * (size_t)plan->pat.n * (size_t)n_sys * rsize() <=
                                 adj_store_limit;
    }

    bool f32() const { return plan->precision != kFP64; }
    bool ext() const { return plan->precision == kFP32Ext; }
    // compensated update (Kahan, or the double-float state of kFP32Ext)
    bool compensated() const { return plan->precision == kFP32Kahan || ext(); }
    // vectors per state-sized buffer (values, x0, state): high and low parts in kFP32Ext
    size_t parts() const { return ext() ? 2 : 1; }
    size_t rsize() const { return f32() ? sizeof(float) : sizeof(double); }
    // The specialised forward kernel for these reducers (false: none, *jerr why).
    // traj_mode: 0 none, 1 states every traj_every steps, 2 the adjoint trajectory.
    bool fwd_kernel(const Signals& sig, unsigned long long mm, unsigned long long sm, int traj_mode, JitKernel* k,
                    std::string* jerr);
    // Launch it over [step0, step0 + nsteps) on state_p ([n][B], updated in
    // place), trajectory slots (or checkpoints) into traj_p when traj_every >
    // 0, starting from the Kahan compensation comp_p ([n][B]; null: zero).
    cudaError_t launch_fwd_jit(const JitKernel& k, const Signals& sig, double h, int step0, int nsteps,
                               const Reducers& red, unsigned long long mm, unsigned long long sm, int traj_every,
                               long long traj_slots, void* state_p, void* traj_p, cudaStream_t st,
                               const void* comp_p = nullptr, void* comp_out_p = nullptr);

    // New instance count; the device buffers are kept and grown by the next
    // set / solve when needed (a batch reused for requests of any size).
    int resize(int n_sys, std::string* err);
    // Grow every device buffer to what a forward or an exact adjoint of n_sys
    // instances over nsteps steps uses, so that later calls up to that size
    // allocate nothing (no implicit device synchronisation).  A grown buffer
    // does not keep its contents: the inputs must be set again.
    int reserve(int n_sys, int nsteps, std::string* err);
    // values[B][P], x0[B][n] (double), exc_index[B]; host or device pointers.
    int set(const double* values, const double* x0h, const int* exc_index, int memory, cudaStream_t st,
            std::string* err);
    // Integrate nsteps from step0; trajectory (optional): every `traj_every`
    // steps into an internal [slots][n][B] buffer.
    int forward(const Signals& sig, double h, int step0, int nsteps, const Reducers& red, int traj_every,
                long long traj_slots, cudaStream_t st, std::string* err);
    // Results in [B][k] double order (host or device pointers; any may be null).
    int get(double* state_out, double* max_out, double* sq_out, double h, int memory, cudaStream_t st,
            std::string* err);
    int get_traj(double* out, long long slots, int memory, cudaStream_t st, std::string* err);
    // Exact discrete adjoint; g_final[B][n] and g_sq[B] may be null.
    int adjoint(const Signals& sig, double h, int nsteps, const Reducers& red, const double* g_final,
                const double* g_sq, double* d_values, double* d_x0, int memory, cudaStream_t st,
                std::string* err);
};

int batch_create(std::shared_ptr<Plan> plan, int B, std::unique_ptr<Batch>* out, std::string* err);

// __GpuDriver::_getGradient semantics for B instances of a (forward, adjoint)
// pattern pair.  All arrays host, [B][k] double.  out[B][na].
int refgrad_run(const Plan& fwd, const Plan& bwd, int B, const double* fvals, const double* bvals,
                const double* x0, const double* a0, const int* exc_index, const Signals& sig, double h,
                int nsteps, int save, double* out, cudaStream_t st, std::string* err);

std::string cuda_err(const char* what, cudaError_t e);

}  // namespace pasif
