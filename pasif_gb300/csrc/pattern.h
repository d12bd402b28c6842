// pattern.h -- host-side sparsity pattern of one polynomial system.
#pragma once
#include <string>
#include <vector>

namespace pasif {

// dQ/dt = K.xs + Gamma:(xs,xp) + Lambda:(xs,xp,xp) + Psi:(xs,xp,xp,xp) + F u.
// Index roles follow src/kernels.cu:52,56,61 (dest, source, setpoint...).
// Parameter order of one instance: K (CSR order), Gamma, Lambda, Psi, F.
struct Pattern {
    int n = 0;                     // state size
    int n_sp = 0;                  // setpoint (trailing-index) state size
    std::vector<int> k_ptr;        // n+1
    std::vector<int> k_col;        // k_nnz
    std::vector<int> g_idx;        // 3 * g_nnz
    std::vector<int> l_idx;        // 4 * l_nnz
    std::vector<int> p_idx;        // 5 * p_nnz
    std::vector<int> f_idx;        // f_nnz

    int k_nnz() const { return (int)k_col.size(); }
    int g_nnz() const { return (int)g_idx.size() / 3; }
    int l_nnz() const { return (int)l_idx.size() / 4; }
    int p_nnz() const { return (int)p_idx.size() / 5; }
    int f_nnz() const { return (int)f_idx.size(); }
    int P() const { return k_nnz() + g_nnz() + l_nnz() + p_nnz() + f_nnz(); }

    // Checks index ranges and CSR monotonicity; returns "" when valid.
    std::string validate() const;
    // GenPattern device layout: k_ptr | k_col | g | l | p | f.
    std::vector<int> flat() const;
    // Stable text key (used for grouping and kernel caching).
    std::string key() const;
};

}  // namespace pasif
