// Host build of the device code (test infrastructure): the generated
// pattern-specialised kernel (GEN_SOURCE) or the generic kernel is compiled by
// g++ with the CUDA intrinsics replaced by correctly rounded host arithmetic,
// and run one "thread" per instance over inputs read from files.  Lets the CPU
// test suite check the code generator and the device templates against the
// oracle without a GPU.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __noinline__
#define __restrict__
#define __launch_bounds__(x)
static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline double __dsub_rn(double a, double b) { return a - b; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
using std::fabs;
using std::fmax;
struct EmuDim { unsigned x, y, z; };
static EmuDim blockIdx, threadIdx, blockDim;

#include GEN_SOURCE

template <typename T>
static std::vector<T> readf(const char* dir, const char* name, size_t n) {
    std::vector<T> v(n > 0 ? n : 1);
    char path[1024];
    std::snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE* f = std::fopen(path, "rb");
    if (!f) { std::perror(path); std::exit(2); }
    if (n && std::fread(v.data(), sizeof(T), n, f) != n) { std::fprintf(stderr, "short read %s\n", path); std::exit(2); }
    std::fclose(f);
    return v;
}

// argv: dir B n P n_exc len window step0 nsteps h kahan
int main(int argc, char** argv) {
    if (argc < 12) return 1;
    const char* dir = argv[1];
    const int B = std::atoi(argv[2]), n = std::atoi(argv[3]), P = std::atoi(argv[4]);
    const int n_exc = std::atoi(argv[5]), len = std::atoi(argv[6]), W = std::atoi(argv[7]);
    const unsigned step0 = (unsigned)std::atoi(argv[8]);
    const int nsteps = std::atoi(argv[9]);
    const double h = std::atof(argv[10]);
    typedef pk::R R;
    auto vals = readf<R>(dir, "vals.bin", (size_t)P * B);
    auto state = readf<R>(dir, "x0.bin", (size_t)n * B);
    auto exc = readf<int>(dir, "exc.bin", (size_t)B);
    auto x = readf<R>(dir, "x.bin", (size_t)n_exc * len);
    auto im = readf<R>(dir, "im.bin", (size_t)2 * W);
    pk::Forcing<R> frc;
    std::memset(&frc, 0, sizeof frc);
    frc.x = x.data();
    frc.im = W ? im.data() : nullptr;
    frc.total = (long long)n_exc * len;
    frc.len = (unsigned)len;
    frc.w = (unsigned)W;
    while (W && (1u << frc.lw) < (unsigned)W) frc.lw++;
    blockDim.x = 128;
    char path[1024];
#ifndef EMU_ADJ
    pk::FwdArgs<R> a;
    std::memset(&a, 0, sizeof a);
    a.vals = vals.data();
    a.state = state.data();
    a.exc_index = exc.data();
    a.traj_every = 1;
    a.frc = frc;
    a.h = (R)h;
    a.h2 = (R)(h / 2.0);
    a.h6 = (R)(h / 6.0);
    a.B = B;
    a.step0 = step0;
    a.nsteps = nsteps;
    for (int b = 0; b < B; ++b) {
        blockIdx.x = (unsigned)(b / 128);
        threadIdx.x = (unsigned)(b % 128);
        pk_fwd(a);
    }
    std::snprintf(path, sizeof path, "%s/out.bin", dir);
    FILE* f = std::fopen(path, "wb");
    std::fwrite(state.data(), sizeof(R), state.size(), f);
    std::fclose(f);
#else
    // exact adjoint: argv[11] = kahan, argv[12] = sq_start; g_sq.bin, g_final.bin inputs
    const int kahan = std::atoi(argv[11]);
    const int sq_start = argc > 12 ? std::atoi(argv[12]) : 0;
    auto gsq = readf<R>(dir, "gsq.bin", (size_t)B);
    auto gfin = readf<R>(dir, "gfin.bin", (size_t)n * B);
    const int C = nsteps > 0 ? (int)std::ceil(std::sqrt((double)nsteps)) : 1;
    const int nck = nsteps > 0 ? (nsteps + C - 1) / C : 0;
    std::vector<R> ckpt((size_t)B * 2 * n * (nck > 0 ? nck : 1)), buf((size_t)B * n * C), dx0((size_t)B * n);
    std::vector<double> pbar((size_t)B * (P > 0 ? P : 1));
    pk::AdjArgs<R> a;
    std::memset(&a, 0, sizeof a);
    a.vals = vals.data();
    a.x0 = state.data();
    a.exc_index = exc.data();
    a.ckpt = ckpt.data();
    a.buf = buf.data();
    a.pbar = pbar.data();
    a.dx0 = dx0.data();
    a.g_final = gfin.data();
    a.g_sq = gsq.data();
    a.frc = frc;
    a.h = (R)h;
    a.h2 = (R)(h / 2.0);
    a.h6 = (R)(h / 6.0);
    a.B = B;
    a.nsteps = nsteps;
    a.C = C;
    a.nck = nck;
    a.kahan = kahan;
    a.sq_start = sq_start;
    for (int b = 0; b < B; ++b) {
        blockIdx.x = (unsigned)(b / 128);
        threadIdx.x = (unsigned)(b % 128);
        pk_adj(a);
    }
    std::snprintf(path, sizeof path, "%s/pbar.bin", dir);
    FILE* f = std::fopen(path, "wb");
    std::fwrite(pbar.data(), sizeof(double), pbar.size(), f);
    std::fclose(f);
    std::snprintf(path, sizeof path, "%s/dx0.bin", dir);
    f = std::fopen(path, "wb");
    std::fwrite(dx0.data(), sizeof(R), dx0.size(), f);
    std::fclose(f);
#endif
    return 0;
}
