// pattern.cpp -- validation and serialisation of a system pattern.
#include "pattern.h"

#include <sstream>

namespace pasif {

std::string Pattern::validate() const {
    if (n < 0) return "negative state size";
    if (n_sp < 0) return "negative setpoint size";
    if ((int)k_ptr.size() != n + 1) return "K row pointer must hold n+1 entries";
    if (k_ptr[0] != 0) return "K row pointer must start at 0";
    for (int i = 0; i < n; ++i)
        if (k_ptr[i + 1] < k_ptr[i]) return "K row pointer must be non-decreasing";
    if (k_ptr[n] != (int)k_col.size()) return "K row pointer end differs from the number of columns";
    for (int c : k_col)
        if (c < 0 || c >= n) return "K column index out of range";
    if (g_idx.size() % 3 || l_idx.size() % 4 || p_idx.size() % 5) return "tensor index list length";
    auto chk = [&](const std::vector<int>& v, int w, const char* name) -> std::string {
        for (size_t e = 0; e < v.size(); e += w) {
            if (v[e] < 0 || v[e] >= n) return std::string(name) + " destination index out of range";
            if (v[e + 1] < 0 || v[e + 1] >= n) return std::string(name) + " source index out of range";
            for (int k = 2; k < w; ++k)
                if (v[e + k] < 0 || v[e + k] >= n_sp) return std::string(name) + " setpoint index out of range";
        }
        return "";
    };
    std::string r;
    if (!(r = chk(g_idx, 3, "Gamma")).empty()) return r;
    if (!(r = chk(l_idx, 4, "Lambda")).empty()) return r;
    if (!(r = chk(p_idx, 5, "Psi")).empty()) return r;
    for (int i : f_idx)
        if (i < 0 || i >= n) return "force index out of range";
    return "";
}

std::vector<int> Pattern::flat() const {
    std::vector<int> v;
    v.insert(v.end(), k_ptr.begin(), k_ptr.end());
    v.insert(v.end(), k_col.begin(), k_col.end());
    v.insert(v.end(), g_idx.begin(), g_idx.end());
    v.insert(v.end(), l_idx.begin(), l_idx.end());
    v.insert(v.end(), p_idx.begin(), p_idx.end());
    v.insert(v.end(), f_idx.begin(), f_idx.end());
    // per-destination term lists in canonical order: d_ptr[n+1] | term[P],
    // term = (kind << 28) | parameter index, kind 0 K, 1 Gamma, 2 Lambda,
    // 3 Psi, 4 F (forcing terms last in each list)
    std::vector<std::vector<int>> per(n);
    const int go = k_nnz(), lo = go + g_nnz(), po = lo + l_nnz(), fo = po + p_nnz();
    for (int i = 0; i < n; ++i)
        for (int q = k_ptr[i]; q < k_ptr[i + 1]; ++q) per[i].push_back(q);
    for (int e = 0; e < g_nnz(); ++e) per[g_idx[3 * e]].push_back((1 << 28) | (go + e));
    for (int e = 0; e < l_nnz(); ++e) per[l_idx[4 * e]].push_back((2 << 28) | (lo + e));
    for (int e = 0; e < p_nnz(); ++e) per[p_idx[5 * e]].push_back((3 << 28) | (po + e));
    for (int e = 0; e < f_nnz(); ++e) per[f_idx[e]].push_back((4 << 28) | (fo + e));
    int acc = 0;
    v.push_back(0);
    for (int i = 0; i < n; ++i) {
        acc += (int)per[i].size();
        v.push_back(acc);
    }
    for (int i = 0; i < n; ++i) v.insert(v.end(), per[i].begin(), per[i].end());
    return v;
}

std::string Pattern::key() const {
    std::ostringstream o;
    o << n << ':' << n_sp << "|K";
    for (int x : k_ptr) o << ',' << x;
    o << ';';
    for (int x : k_col) o << ',' << x;
    o << "|G";
    for (int x : g_idx) o << ',' << x;
    o << "|L";
    for (int x : l_idx) o << ',' << x;
    o << "|P";
    for (int x : p_idx) o << ',' << x;
    o << "|F";
    for (int x : f_idx) o << ',' << x;
    return o.str();
}

}  // namespace pasif
