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
#include <algorithm>
#include <barrier>
#include <thread>
#include <vector>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __noinline__
#define __restrict__
#define __launch_bounds__(x)
#define __shared__ static
static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline double __dsub_rn(double a, double b) { return a - b; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
struct float2 { float x, y; };
static inline float2 make_float2(float x, float y) { return float2{x, y}; }
using std::fabs;
using std::fmax;
struct EmuDim { unsigned x, y, z; };
static thread_local EmuDim blockIdx, threadIdx;
static EmuDim blockDim;

// Warp-sliced kernels: the L warps of a system run as L host threads sharing
// that system's shared-memory buffers, the CTA barrier is a std::barrier.
#define PK_HOST_EMU 1
static thread_local unsigned char* emu_smem = nullptr;
static thread_local std::barrier<>* emu_bar = nullptr;
static inline unsigned char* pk_dyn_smem() { return emu_smem; }
static inline void pk_block_sync() {
    if (emu_bar) emu_bar->arrive_and_wait();
}
static inline unsigned pk_warp_max(unsigned v) { return v; }   // one system per emulated block

static int emu_ws_slices() {
    const char* s = std::getenv("EMU_WS_L");
    return s ? std::atoi(s) : 0;
}

// Run `call` for system b: one thread per thread-per-system kernel, L barrier-
// synchronised threads for a warp-sliced one (EMU_WS_L, EMU_WS_SMEM bytes).
template <class F>
static void emu_launch(long long b, F&& call) {
    const int L = emu_ws_slices();
    if (L <= 0) {
        blockIdx.x = (unsigned)(b / 128);
        threadIdx.x = (unsigned)(b % 128);
        call();
        return;
    }
    const char* sz = std::getenv("EMU_WS_SMEM");
    std::vector<unsigned char> sm((sz ? std::atoll(sz) : 0) + 64, 0);
    std::barrier<> bar(L);
    std::vector<std::thread> th;
    for (int w = 0; w < L; ++w)
        th.emplace_back([&, w] {
            emu_smem = sm.data();
            emu_bar = &bar;
            blockIdx.x = (unsigned)(b / 32);
            threadIdx.x = (unsigned)(w * 32 + b % 32);
            call();
        });
    for (auto& t : th) t.join();
}

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

#ifdef EMU_POOL
// Serving pool: C slots, jobs admitted into given slots before given chunks,
// harvested after the chunk in which their slot ran out of steps.
// argv: dir C n P S W chunk h n_jobs n_chunks
// jobs.bin: int64 [J][8] = slot, admit_chunk, nsteps, ebase, lim, len, max_start, sq_start
// vals.bin [J][P], x0.bin [J][n], arena.bin [S], im.bin [2W] (compute precision)
// out: state.bin [J][n], mx.bin [J][n], sq.bin [J], done.bin int32 [J] (chunk of harvest)
int main(int argc, char** argv) {
    if (argc < 11) return 1;
    const char* dir = argv[1];
    const int C = std::atoi(argv[2]), n = std::atoi(argv[3]), P = std::atoi(argv[4]);
    const long long S = std::atoll(argv[5]);
    const int W = std::atoi(argv[6]), chunk = std::atoi(argv[7]);
    const double h = std::atof(argv[8]);
    const int J = std::atoi(argv[9]), T = std::atoi(argv[10]);
    typedef pk::R R;
    auto jobs = readf<long long>(dir, "jobs.bin", (size_t)J * 8);
    auto jv = readf<R>(dir, "vals.bin", (size_t)J * P);
    auto jx = readf<R>(dir, "x0.bin", (size_t)J * n);
    auto arena = readf<R>(dir, "arena.bin", (size_t)S);
    auto im = readf<R>(dir, "im.bin", (size_t)2 * W);
    std::vector<R> vals((size_t)(P > 0 ? P : 1) * C, R(0)), state((size_t)n * C, R(0)), comp((size_t)n * C, R(0)),
        mx((size_t)n * C, R(0)), sq(C, R(0)), sqc(C, R(0));
    std::vector<unsigned> step(C, 0u), len(C, 0u);
    std::vector<int> remain(C, 0), mstart(C, 0), sstart(C, 0), owner(C, -1), done(J, -1);
    std::vector<long long> ebase(C, 0), lim(C, 0);
    std::vector<R> os((size_t)J * n, R(0)), om((size_t)J * n, R(0)), oq(J, R(0));
    pk::PoolArgs<R> p;
    std::memset(&p, 0, sizeof p);
    p.vals = vals.data();
    p.state = state.data();
    p.comp = comp.data();
    p.mx = mx.data();
    p.sq = sq.data();
    p.sqc = sqc.data();
    p.step = step.data();
    p.remain = remain.data();
    p.ebase = ebase.data();
    p.lim = lim.data();
    p.len = len.data();
    p.max_start = mstart.data();
    p.sq_start = sstart.data();
    p.frc.x = arena.data();
    p.frc.im = W ? im.data() : nullptr;
    p.frc.total = S;
    p.frc.w = (unsigned)W;
    while (W && (1u << p.frc.lw) < (unsigned)W) p.frc.lw++;
    p.h = (R)h;
    p.h2 = (R)(h / 2.0);
    p.h6 = (R)(h / 6.0);
    p.C = C;
    p.chunk = chunk;
    blockDim.x = 128;
    auto harvest = [&](int c) {
        for (int b = 0; b < C; ++b) {
            const int j = owner[b];
            if (j < 0 || remain[b] > 0) continue;
            for (int i = 0; i < n; ++i) {
                os[(size_t)j * n + i] = state[(size_t)i * C + b];
                om[(size_t)j * n + i] = mx[(size_t)i * C + b];
            }
            oq[j] = sq[b];
            done[j] = c;
            owner[b] = -1;
        }
    };
    for (int c = 0; c <= T; ++c) {
        harvest(c);
        if (c == T) break;
        for (int j = 0; j < J; ++j) {
            const long long* q = &jobs[(size_t)j * 8];
            if (q[1] != c) continue;
            const int b = (int)q[0];
            if (b < 0 || b >= C || owner[b] >= 0) { std::fprintf(stderr, "slot %d busy\n", b); return 3; }
            owner[b] = j;
            for (int k = 0; k < P; ++k) vals[(size_t)k * C + b] = jv[(size_t)j * P + k];
            for (int i = 0; i < n; ++i) {
                state[(size_t)i * C + b] = jx[(size_t)j * n + i];
                comp[(size_t)i * C + b] = R(0);
                mx[(size_t)i * C + b] = R(0);
            }
            sq[b] = sqc[b] = R(0);
            step[b] = 0u;
            remain[b] = (int)q[2];
            ebase[b] = q[3];
            lim[b] = q[4];
            len[b] = (unsigned)q[5];
            mstart[b] = (int)q[6];
            sstart[b] = (int)q[7];
        }
        for (int b = 0; b < C; ++b) {
            emu_launch(b, [&] { pk_pool(p); });
        }
    }
    for (int j = 0; j < J; ++j)
        if (done[j] < 0) { std::fprintf(stderr, "job %d unfinished\n", j); return 4; }
    char path[1024];
    const struct { const char* name; const void* p; size_t bytes; } outs[] = {
        {"state.bin", os.data(), os.size() * sizeof(R)}, {"mx.bin", om.data(), om.size() * sizeof(R)},
        {"sq.bin", oq.data(), oq.size() * sizeof(R)}, {"done.bin", done.data(), done.size() * sizeof(int)}};
    for (const auto& o : outs) {
        std::snprintf(path, sizeof path, "%s/%s", dir, o.name);
        FILE* f = std::fopen(path, "wb");
        std::fwrite(o.p, 1, o.bytes, f);
        std::fclose(f);
    }
    return 0;
}
#else
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
    // EMU_EXT=1: extended-state mode, vals.bin [2P][B] and x0.bin [2n][B]
    // (high parts, then low parts); out.bin [2n][B]
    const char* ext_env = std::getenv("EMU_EXT");
    const int ext = ext_env ? std::atoi(ext_env) : 0;
    const size_t np = ext ? 2 : 1;
    auto vals = readf<R>(dir, "vals.bin", (size_t)P * B * np);
    auto state = readf<R>(dir, "x0.bin", (size_t)n * B * np);
    auto exc = readf<int>(dir, "exc.bin", (size_t)B);
    const R h6lo = (R)(h / 6.0 - (double)(R)(h / 6.0));
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
    if (ext) {
        a.comp = state.data() + (size_t)n * B;
        a.comp_out = state.data() + (size_t)n * B;
        a.h6lo = h6lo;
    }
    for (int b = 0; b < B; ++b) emu_launch(b, [&] { pk_fwd(a); });
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
    std::vector<R> ckpt((size_t)B * 2 * n * (nck > 0 ? nck : 1)), buf((size_t)B * 4 * n * C), dx0((size_t)B * n);
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
    a.kahan = kahan || ext;
    a.ext = ext;
    a.h6lo = ext ? h6lo : R(0);
    a.sq_start = sq_start;
    std::vector<R> lamc((size_t)B * n, R(0));
    a.lamc = lamc.data();
    std::vector<R> pk((size_t)B * 2 * (P > 0 ? P : 1), R(0));
    a.pk = pk.data();
    // EMU_ADJ_STORED=1: backward over a stored trajectory ([nsteps+1][4][n][B]
    // slots).  It is made by this kernel's own chunk recompute: the adjoint of
    // one step more, in one chunk, leaves slots 0..nsteps in its buffer.
    const char* stored = std::getenv("EMU_ADJ_STORED");
    std::vector<R> traj, ck1((size_t)B * 2 * n), dx1((size_t)B * n), lc1((size_t)B * n, R(0));
    std::vector<double> pb1(pbar.size());
    if (stored && std::atoi(stored) && nsteps > 0) {
        traj.assign((size_t)B * 4 * n * (nsteps + 1), R(0));
        pk::AdjArgs<R> f = a;
        f.ckpt = ck1.data();
        f.buf = traj.data();
        f.pbar = pb1.data();
        f.dx0 = dx1.data();
        f.lamc = lc1.data();
        f.C = nsteps + 1;
        f.nck = 1;
        f.nsteps = nsteps + 1;
        for (int b = 0; b < B; ++b) emu_launch(b, [&] { pk_adj(f); });
        a.buf = traj.data();
        a.stored = 1;
        std::fill(pbar.begin(), pbar.end(), -1.0);   // the stored backward must zero the totals itself
    }
    // EMU_ADJ_SPLIT=k: the launch split of Batch::adjoint with k checkpoint
    // intervals per launch (forward segments, then backward chunk groups)
    const char* split = std::getenv("EMU_ADJ_SPLIT");
    const int per = split ? std::atoi(split) : 0;
    if (per <= 0 || nck <= 2 * per) {
        for (int b = 0; b < B; ++b) emu_launch(b, [&] { pk_adj(a); });
    } else {
        for (int t0 = 0; t0 < (a.stored ? 0 : nsteps); t0 += per * C) {
            a.phase = 1;
            a.t_begin = t0;
            a.t_end = std::min(nsteps, t0 + per * C);
            for (int b = 0; b < B; ++b) emu_launch(b, [&] { pk_adj(a); });
        }
        for (int khi = nck - 1; khi >= 0; khi -= per) {
            a.phase = 2;
            a.k_hi = khi;
            a.k_lo = std::max(0, khi - per + 1);
            for (int b = 0; b < B; ++b) emu_launch(b, [&] { pk_adj(a); });
        }
    }
    std::snprintf(path, sizeof path, "%s/pbar.bin", dir);
    FILE* f = std::fopen(path, "wb");
    std::fwrite(pbar.data(), sizeof(double), pbar.size(), f);
    std::fclose(f);
    std::snprintf(path, sizeof path, "%s/dx0.bin", dir);
    f = std::fopen(path, "wb");
    std::fwrite(dx0.data(), sizeof(R), dx0.size(), f);
    std::fclose(f);
    std::snprintf(path, sizeof path, "%s/lamc.bin", dir);   // low parts of dx0 (extended-state mode)
    f = std::fopen(path, "wb");
    std::fwrite(lamc.data(), sizeof(R), lamc.size(), f);
    std::fclose(f);
#endif
    return 0;
}
#endif
