// driver.h -- the __GpuDriver drop-in: the reference's concatenated
// block-diagonal system, replicated over excitation signals, re-expressed as
// batches of independent small systems for the engine.
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "engine.h"

namespace pasif {

struct CsrIn {
    bool set = false;
    unsigned rows = 0, cols = 0;
    std::vector<double> val;
    std::vector<unsigned> col, ptr;
};

struct CooIn {
    bool set = false;
    std::vector<unsigned> dims;
    std::vector<double> val;
    std::vector<unsigned> idx;   // dims.size() per entry
};

struct SystemIn {
    CsrIn K;
    CooIn G, L, Psi;
    bool force_set = false, ic_set = false;
    std::vector<double> force, ic;
};

// One independent block of the concatenated system (a connected component of
// its coupling graph): the global indices it owns and its local pattern.
struct Block {
    std::vector<int> nodes;     // forward state indices (ascending)
    std::vector<int> anodes;    // adjoint state indices (ascending; gradient only)
    Pattern pat, apat;
    std::vector<double> vals, avals;
};

// Blocks sharing one pattern, solved as one batch (instances = blocks x signals).
// The instances' inputs stay on the host too: a sweep larger than the device
// memory budget runs as sequential batches of `chunk` instances.
struct Group {
    std::vector<int> blocks;
    std::shared_ptr<Plan> plan, aplan;
    std::unique_ptr<Batch> batch;
    std::vector<double> hvals, hx0;   // [B][P], [B][n]; instance b = signal b / nb, block b % nb
    std::vector<int> hexc;            // [B]
    int resident = 0;                 // instances whose inputs the batch holds from instance 0 (0: none)
};

// Instances per sequential batch of a sweep of n_instances that need
// bytes_per_instance of device memory each, within `budget` bytes: all of
// them when they fit, else as many as fit; 0 when not even one does.  The
// reference splits its excitation copies the same way by free memory
// (numberOfSimulationToPerform, src/__GpuDriver.cu:420-449, 896-938).
long long sweep_chunk(long long n_instances, long long bytes_per_instance, long long budget);

class Driver {
public:
    Driver(unsigned gpu, unsigned sample_rate, unsigned numsteps, bool dc, bool ds, bool dsol);
    int load_excitations(const double* const* sig, const long long* len, int n, unsigned sample_rate,
                         std::string* err);
    int set_precision(int p, std::string* err);
    int set_k(bool fwd, unsigned rows, unsigned cols, const double* v, const unsigned* ind, const unsigned* ptr,
              long long nnz, std::string* err);
    int set_coo(bool fwd, int order, const unsigned* dims, const double* v, const unsigned* ind, long long nnz,
                std::string* err);
    int set_force(bool fwd, const double* v, long long n, std::string* err);
    int set_ic(bool fwd, const double* v, long long n, std::string* err);
    int allocate_system(std::string* err);
    int allocate_adjoint(std::string* err);
    int set_interp(const double* m, long long size, unsigned window, std::string* err);
    int set_modulation(const double* m, long long n, std::string* err);
    int amplitudes(std::vector<double>* out, std::string* err);
    int trajectory(unsigned save, std::vector<double>* out, std::string* err);
    int gradient(unsigned save, std::vector<double>* out, std::string* err);
    int last_kind() const { return last_kind_; }
    // Device memory a solve may use for its instances (0: automatic, 90 % of
    // what is free when the solve starts plus what the driver holds); a sweep
    // beyond it runs as sequential batches.  No reference counterpart as an
    // argument: the reference always takes the free memory.
    int set_memory_budget(long long bytes, std::string* err);
    // Sequential batches the last solve ran (1: the whole sweep at once).
    int last_chunks() const { return last_chunks_; }
    // Output sizes of the getters (no solve): nf * n_exc, na * n_exc and
    // floor(nf * n_exc * numsteps / save) (src/__GpuDriver.cu:420,469,580).
    long long amplitudes_size() const { return (long long)nf_ * n_exc_; }
    long long gradient_size() const { return (long long)na_ * n_exc_; }
    long long trajectory_size(unsigned save) const {
        return save ? ((long long)nf_ * n_exc_ * (long long)numsteps_) / (long long)save : 0;
    }

private:
    int ensure_signals(std::string* err);
    int build_forward_groups(std::string* err);
    int run_forward(int traj_every, long long slots, std::vector<double>* final_out,
                    std::vector<double>* traj_out, std::string* err);
    void info(const std::string& s) const;

    unsigned gpu_;
    unsigned sample_rate_, numsteps_;
    bool dcompute_, dsystem_, dsolver_;
    int precision_ = kFP64;
    double h_ = 0.0;
    std::vector<double> exc_;
    int n_exc_ = 0, exc_len_ = 0;
    bool exc_ok_ = false;
    std::vector<double> im_;
    unsigned window_ = 0;
    std::vector<double> modulation_;
    SystemIn fwd_, bwd_;
    int nf_ = 0, na_ = 0;
    bool sys_alloc_ = false, adj_alloc_ = false;
    std::vector<double> bwd_state_;   // [n_exc][na]: chained terminal condition
    std::vector<Block> blocks_;
    std::vector<Group> groups_;
    std::shared_ptr<Signals> signals_;
    int last_kind_ = kNone;
    long long mem_budget_ = 0;
    int last_chunks_ = 0;
    cudaStream_t stream_ = nullptr;
    long long budget_for(long long held) const;
};

}  // namespace pasif
