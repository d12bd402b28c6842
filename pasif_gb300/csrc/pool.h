// pool.h -- serving pools: continuous batching of forward requests.
//
// A pool owns C slots of one pattern class (pattern, precision, forcing
// window and weights, time step, reducers).  A request of n systems takes n
// free slots and a region of the pool's signal arena; every chunk launch (a
// CUDA graph replay of the specialised pk_pool kernel) advances each busy
// slot by up to `chunk` steps from its own step index, carrying state, Kahan
// compensation and reducers in device memory.  Finished requests are
// harvested between chunks and their slots re-used at once, so requests
// join and leave while others are running.  A slot computes exactly what a
// single-request batch computes (same operations in the same order), so a
// result does not depend on what else is in the pool.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "engine.h"

namespace pasif {

struct PoolRequest {
    std::vector<int> slots;
    long long arena_off = 0, arena_len = 0;
    int n_sys = 0;
};

class Pool {
public:
    ~Pool();
    static int create(const Pattern& pat, int precision, int window, const double* im, double h,
                      const std::vector<int>& max_comp, const std::vector<int>& sq_comp, int capacity,
                      long long arena_samples, int chunk, int slicing, std::unique_ptr<Pool>* out,
                      std::string* err);
    // PASIF_ERR_STATE (5) when slots or arena space are short: retry later.
    int admit(int n_sys, const double* values, const double* x0, const int* exc_index, const double* signals,
              int n_exc, int len, int nsteps, int max_start, int sq_start, int* req_id, std::string* err);
    int launch(std::string* err);                                        // one chunk, asynchronous
    int poll(std::vector<int>* finished, std::string* err);              // waits for the chunk
    int harvest(int req_id, double* state, double* max, double* sq, std::string* err);
    int free_slots() const { return (int)free_.size(); }
    long long free_arena() const;
    int active() const { return (int)reqs_.size(); }
    int n_max() const { return (int)max_comp_.size(); }
    cudaStream_t stream() const { return st_; }
    int precision() const { return plan_->precision; }

private:
    long long arena_alloc(long long n);
    void arena_free(long long off, long long n);
    int build_graph(std::string* err);

    std::shared_ptr<Plan> plan_;
    int C_ = 0, chunk_ = 0, window_ = 0;
    double h_ = 0.0;
    std::vector<double> im_;
    std::vector<int> max_comp_, sq_comp_;
    unsigned long long max_mask_ = 0, sq_mask_ = 0;
    long long S_ = 0;
    DevBuf vals_, state_, comp_, mx_, sq_, sqc_, step_, remain_, ebase_, lim_, len_, mstart_, sstart_, arena_;
    DevBuf scratch_;                       // staging for admissions / harvests
    DevBuf im_dev_;                        // forcing weights (compute precision)
    int* remain_host_ = nullptr;           // pinned
    std::vector<int> free_;
    std::map<long long, long long> holes_;  // arena free list: offset -> size
    std::map<int, PoolRequest> reqs_;
    int next_id_ = 1;
    // set when an admission failed after part of its upload was queued: the
    // device-side slot records may then be inconsistent (a slot may read as
    // busy with a stale request), so the pool refuses every further call
    bool failed_ = false;
    JitKernel k_;
    cudaStream_t st_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;
};

}  // namespace pasif
