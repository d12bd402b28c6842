// ref_driver.cu -- runs the REFERENCE's own __GpuDriver (compiled from the
// PASIf sources by oracle/ref/build_ref.sh) on a case file and prints the
// result vector.  Test infrastructure: used once, on a GPU machine, to produce the
// golden vectors under tests/golden/ that pin the CPU oracle to the
// reference's actual outputs.  Only the reference's public methods are called
// (src/__GpuDriver.cuh:18-83); nothing of the reference is copied here.
//
// Case file (whitespace separated):
//   E L  <E*L samples>  sample_rate numsteps
//   W nIM <nIM weights>                      (W = 0: no interpolation matrix)
//   K rows cols nnz <vals> <indices> <indptr>
//   G d0 d1 d2 nnz <vals> <3*nnz indices>
//   L d0..d3 nnz <vals> <4*nnz indices>
//   P d0..d4 nnz <vals> <5*nnz indices>
//   F n <vals>   IC n <vals>
//   has_bwd, then the same K G L P F IC blocks for the adjoint when 1
//   task: 0 amplitudes | 1 trajectory <save> | 2 gradient <save>
// An optional third argument names a file that receives the wall time of the
// getter call in seconds (oracle/ref/time_ref.py).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "__GpuDriver.cuh"

static FILE* g_in;

static double rd() {
    double v;
    if (std::fscanf(g_in, "%lf", &v) != 1) { std::fprintf(stderr, "bad case file\n"); std::_Exit(3); }
    return v;
}
static unsigned ru() { return (unsigned)rd(); }
template <typename T> static std::vector<T> rv(size_t n) {
    std::vector<T> v(n);
    for (auto& x : v) x = (T)rd();
    return v;
}

struct Sys {
    std::array<uint, 2> kn; std::vector<double> kv; std::vector<uint> ki, kp;
    std::array<uint, 3> gn; std::vector<double> gv; std::vector<uint> gi;
    std::array<uint, 4> ln; std::vector<double> lv; std::vector<uint> li;
    std::array<uint, 5> pn; std::vector<double> pv; std::vector<uint> pi;
    std::vector<double> f, ic;
};

static Sys read_sys() {
    Sys s;
    s.kn = {ru(), ru()};
    size_t nnz = ru();
    s.kv = rv<double>(nnz); s.ki = rv<uint>(nnz); s.kp = rv<uint>(s.kn[0] + 1);
    s.gn = {ru(), ru(), ru()}; nnz = ru(); s.gv = rv<double>(nnz); s.gi = rv<uint>(3 * nnz);
    s.ln = {ru(), ru(), ru(), ru()}; nnz = ru(); s.lv = rv<double>(nnz); s.li = rv<uint>(4 * nnz);
    s.pn = {ru(), ru(), ru(), ru(), ru()}; nnz = ru(); s.pv = rv<double>(nnz); s.pi = rv<uint>(5 * nnz);
    size_t n = ru(); s.f = rv<double>(n);
    n = ru(); s.ic = rv<double>(n);
    return s;
}

int main(int argc, char** argv) {
    if (argc < 3) { std::fprintf(stderr, "usage: ref_driver case.txt out.txt [seconds.txt]\n"); return 2; }
    g_in = std::fopen(argv[1], "r");
    if (!g_in) return 2;
    const size_t E = ru(), L = ru();
    std::vector<std::vector<double>> exc(E, std::vector<double>(L));
    for (auto& row : exc) for (auto& x : row) x = rd();
    const unsigned sr = ru(), N = ru();
    const unsigned W = ru();
    const size_t nim = ru();
    std::vector<double> im = rv<double>(nim);
    Sys f = read_sys();
    const int has_bwd = (int)ru();
    Sys b;
    if (has_bwd) b = read_sys();
    const int task = (int)ru();
    const unsigned save = task ? ru() : 0;
    std::fclose(g_in);

    __GpuDriver d(exc, sr, N, false, false, false, 0);
    d._setFwdK(f.kn, f.kv, f.ki, f.kp);
    d._setFwdGamma(f.gn, f.gv, f.gi);
    d._setFwdLambda(f.ln, f.lv, f.li);
    d._setFwdPsi(f.pn, f.pv, f.pi);
    d._setFwdForcePattern(f.f);
    d._setFwdInitialConditions(f.ic);
    d._allocateSystemOnDevice();
    if (W) d._setInterpolationMatrix(im, W);
    if (has_bwd) {
        d._setBwdK(b.kn, b.kv, b.ki, b.kp);
        d._setBwdGamma(b.gn, b.gv, b.gi);
        d._setBwdLambda(b.ln, b.lv, b.li);
        d._setBwdForcePattern(b.f);
        d._setBwdInitialConditions(b.ic);
        d._setBwdPsi(b.pn, b.pv, b.pi);
        d._allocateAdjointOnDevice();
    }
    std::vector<double> out;
    const auto t0 = std::chrono::steady_clock::now();
    if (task == 0) out = d._getAmplitudes();
    else if (task == 1) out = d._getTrajectory(save);
    else out = d._getGradient(save);
    cudaError_t e = cudaDeviceSynchronize();
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (argc > 3) {   // wall time of the getter call (the whole solve, host loop included)
        FILE* ft = std::fopen(argv[3], "w");
        std::fprintf(ft, "%.9f\n", secs);
        std::fclose(ft);
    }
    FILE* fo = std::fopen(argv[2], "w");
    std::fprintf(fo, "%d %zu\n", (int)e, out.size());
    for (double v : out) std::fprintf(fo, "%.17g\n", v);
    std::fclose(fo);
    // skip the reference's destructor: it destroys a graph instance that may
    // never have been created (src/__GpuDriver.cu, clearSystemStatesVector)
    std::fflush(stdout);
    std::_Exit(0);
}
