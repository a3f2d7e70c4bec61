// agb_batch.cu -- batched solves of independent boxes (periodic RVE
// homogenization): every problem of the batch advances through the same
// sequence of persistent tile kernels, one launch per multigrid step for the
// whole batch, each V-cycle replayed from one captured CUDA graph.
//
// Per problem the algorithm is the single-box solver's (MLMG V-cycles with
// 2+2 Fsmooth, BiCGStab bottom; FP32 cycles inside FP64 iterative refinement
// when params.precision == AGB_PREC_MIXED, and with params.krylov > 0 a
// flexible GCR of each problem over the FP32 V-cycle inside each
// refinement), with the bottom level of each problem where its own coarsening
// stops.  Problems that have converged are
// masked out of the remaining launches.  The stencil tile shape of every
// level is chosen by timing the candidate shapes on the batch's own data at
// the first solve (autotune), and kept for the following solves.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "agb.h"
#include "agb_internal.h"

using namespace agb;

namespace {

agb_status bfail(agb_status s, const char* msg)
{
    set_error(msg);
    return s;
}

#define BCK(call)                                                         \
    do {                                                                  \
        cudaError_t e_ = (call);                                          \
        if (e_ != cudaSuccess) return bfail(AGB_CUDA, cudaGetErrorString(e_)); \
    } while (0)
#define BTRY(...)                          \
    do {                                   \
        agb_status s_ = (__VA_ARGS__);     \
        if (s_ != AGB_OK) return s_;       \
    } while (0)

template <typename T> struct DevVec {
    T* d = nullptr;
    int n = 0;
};

struct BLevel {
    std::vector<BProb> probs;
    BProb* d_probs = nullptr;
    int shape = 0;
    std::vector<BTile> tS_smooth, t32_smooth, t32_full;
    BTile *d_tS_smooth = nullptr, *d_t32_smooth = nullptr, *d_t32_full = nullptr;
    // the same lists restricted to the problems still iterating (compact()),
    // padded to full length with end markers (prob = -1); the cycle graphs use these
    BTile *c_tS_smooth = nullptr, *c_t32_smooth = nullptr, *c_t32_full = nullptr;
    std::vector<int> bottoms;
    int* d_bottoms = nullptr;
    long long nvec = 0, ncoef = 0, nwork = 0;
    double *ddw64 = nullptr, *diag64 = nullptr, *dinv64 = nullptr;
    double *cor64 = nullptr, *res64 = nullptr, *rescor64 = nullptr, *tmp64 = nullptr;
    float *ddw32 = nullptr, *dinv32 = nullptr;
    float *cor32 = nullptr, *res32 = nullptr, *rescor32 = nullptr, *tmp32 = nullptr;
    float* hold32 = nullptr;   // F-cycle's kept interpolated correction (GCR path only)
    double* work = nullptr;
};

int levels_of(const int n[3], int maxc)
{
    int m[3] = {n[0], n[1], n[2]}, lev = 1;
    while (lev - 1 < maxc) {
        bool ok = true;
        for (int d = 0; d < 3; d++)
            if (m[d] % 2 != 0 || m[d] / 2 < 2) ok = false;
        if (!ok) break;
        for (int d = 0; d < 3; d++) m[d] /= 2;
        lev++;
    }
    return lev;
}

void make_tiles(const std::vector<BProb>& probs, const std::vector<int>& which, const int dims[3],
                std::vector<BTile>& out)
{
    out.clear();
    for (int p : which) {
        const LevelDesc& L = probs[p].L;
        const int nx = (L.nn[0] + dims[0] - 1) / dims[0], ny = (L.nn[1] + dims[1] - 1) / dims[1],
                  nz = (L.nn[2] + dims[2] - 1) / dims[2];
        for (int z = 0; z < nz; z++)
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++) out.push_back(BTile{p, (short)x, (short)y, (short)z, 0});
    }
}

}  // namespace

struct agb_batch_s {
    int np = 0, sym = 0, nc = 2;
    int per[3] = {1, 1, 1};
    BCTable bc;
    agb_solver_params p;
    double omega = 2.0 / 3.0;
    std::vector<int> n;          // 3 per problem
    std::vector<double> dx;      // 3 per problem
    std::vector<int> bottom;     // coarsest level per problem
    int Lmax = 1;
    std::vector<BLevel> lev;
    double *x64 = nullptr, *b64 = nullptr, *F0 = nullptr, *scale = nullptr, *sums = nullptr;
    float *rhs32 = nullptr, *sol32 = nullptr;
    int *d_active = nullptr, *d_iactive = nullptr;
    std::vector<int> active, iactive;
    double* d_norms = nullptr;
    double* h_norms = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaGraphExec_t g64 = nullptr, g32 = nullptr;
    long long g64_k = 0, g32_k = 0;
    // per-problem GCR over the FP32 cycle (params.krylov > 0): directions,
    // their images, per-problem scalars, one graph per number of stored directions
    std::vector<float*> kZ, kW;
    float* kr32 = nullptr;   // the GCR residual of each problem (the F-cycle overwrites res32 of level 0)
    double *kdots = nullptr, *kd2 = nullptr;
    std::vector<cudaGraphExec_t> gk;
    std::vector<long long> gk_k;
    long long compact_tiles = -1;   // level-0 tiles in the compacted lists (-1: not built)
    std::vector<int> compact_mask;
    int grid = 0;   // persistent grid: 4 CTAs per SM, set at creation
    bool model_set = false, prepared = false, tuned = false, f0_set = false;
    std::vector<void*> allocs;

    template <typename T> agb_status alloc(T** q, size_t count)
    {
        void* v = nullptr;
        if (cudaMalloc(&v, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess)
            return bfail(AGB_NOMEM, "cudaMalloc failed in the batch solver");
        cudaMemsetAsync(v, 0, std::max<size_t>(count, 1) * sizeof(T), st);
        allocs.push_back(v);
        *q = (T*)v;
        return AGB_OK;
    }
    template <typename T> agb_status upload_vec(const std::vector<T>& h, T** d)
    {
        BTRY(alloc(d, h.size()));
        if (!h.empty()) BCK(cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        return AGB_OK;
    }
};

namespace {

// ---------------------------------------------------------------------------
// batched cycle engine
// ---------------------------------------------------------------------------
template <typename T> struct BArr;
template <> struct BArr<double> {
    static double* cor(BLevel& l) { return l.cor64; }
    static double* res(BLevel& l) { return l.res64; }
    static double* rescor(BLevel& l) { return l.rescor64; }
    static double* tmp(BLevel& l) { return l.tmp64; }
    static const double* ddw(BLevel& l) { return l.ddw64; }
    static const double* dinv(BLevel& l) { return l.dinv64; }
};
template <> struct BArr<float> {
    static float* cor(BLevel& l) { return l.cor32; }
    static float* res(BLevel& l) { return l.res32; }
    static float* rescor(BLevel& l) { return l.rescor32; }
    static float* tmp(BLevel& l) { return l.tmp32; }
    static const float* ddw(BLevel& l) { return l.ddw32; }
    static const float* dinv(BLevel& l) { return l.dinv32; }
};

template <typename T> struct BEngine {
    agb_batch b;
    const int* act;
    typedef BArr<T> A;
    static constexpr int fp32 = sizeof(T) == 4;

    void smooth(int l, T* x, const T* rhs, int ns)
    {
        BLevel& v = b->lev[l];
        if (v.tS_smooth.empty()) return;
        for (int s = 0; s < ns; s++) {
            launch_batch_stencil<T>(b->st, b->sym, MODE_JACOBI, v.shape, b->grid, v.d_probs, v.c_tS_smooth,
                                    (int)v.tS_smooth.size(), act, b->bc, false, A::ddw(v), x, rhs, A::dinv(v), A::tmp(v),
                                    (T)b->omega, nullptr);
            launch_batch_stencil<T>(b->st, b->sym, MODE_JACOBI, v.shape, b->grid, v.d_probs, v.c_tS_smooth,
                                    (int)v.tS_smooth.size(), act, b->bc, false, A::ddw(v), A::tmp(v), rhs, A::dinv(v), x,
                                    (T)b->omega, nullptr);
        }
    }
    // x = 0, then the smoothing: the first sweep of a zero guess is
    // elementwise (BV_JACOBI0), the rest are stencil sweeps
    void smooth_from_zero(int l, T* x, const T* rhs, int ns)
    {
        BLevel& v = b->lev[l];
        if (ns <= 0 || v.tS_smooth.empty()) {
            launch_batch_vec(b->st, BV_ZERO, b->grid, v.d_probs, v.c_t32_smooth, (int)v.t32_smooth.size(), act, x,
                             nullptr, 0.0, nullptr, fp32);
            return;
        }
        launch_batch_vec(b->st, BV_JACOBI0, b->grid, v.d_probs, v.c_t32_smooth, (int)v.t32_smooth.size(), act,
                         A::tmp(v), rhs, b->omega, nullptr, fp32, A::dinv(v));
        launch_batch_stencil<T>(b->st, b->sym, MODE_JACOBI, v.shape, b->grid, v.d_probs, v.c_tS_smooth,
                                (int)v.tS_smooth.size(), act, b->bc, false, A::ddw(v), A::tmp(v), rhs, A::dinv(v), x,
                                (T)b->omega, nullptr);
        smooth(l, x, rhs, ns - 1);
    }
    // MLMG::mgVcycle(0, 0) for every problem, each with its own bottom level
    void vcycle() { vcycle_from(0, false); }
    // MLMG::mgVcycle(0, top) for the problems that have level top; with
    // skip_top_bottoms the problems whose bottom is level top are left alone
    // (the F-cycle solved them already)
    void vcycle_from(int top, bool skip_top_bottoms)
    {
        const int L = b->Lmax;
        for (int l = top; l < L; l++) {
            BLevel& v = b->lev[l];
            if (!v.t32_smooth.empty()) {
                smooth_from_zero(l, A::cor(v), A::res(v), b->p.pre_smooth);
                launch_batch_stencil<T>(b->st, b->sym, MODE_RESID, v.shape, b->grid, v.d_probs, v.c_tS_smooth,
                                        (int)v.tS_smooth.size(), act, b->bc, false, A::ddw(v), A::cor(v), A::res(v),
                                        nullptr, A::rescor(v), (T)0, nullptr);
                BLevel& c = b->lev[l + 1];
                launch_batch_transfer<T>(b->st, 1, false, b->grid, v.d_probs, c.d_probs, c.c_t32_full,
                                         (int)c.t32_full.size(), act, A::rescor(v), A::res(c));
            }
            if (!v.bottoms.empty() && !(skip_top_bottoms && l == top)) bottom(l);
        }
        for (int l = L - 2; l >= top; l--) {
            BLevel& v = b->lev[l];
            if (v.t32_smooth.empty()) continue;
            BLevel& c = b->lev[l + 1];
            launch_batch_transfer<T>(b->st, 0, false, b->grid, v.d_probs, c.d_probs, v.c_t32_smooth,
                                     (int)v.t32_smooth.size(), act, A::cor(c), A::cor(v));
            smooth(l, A::cor(v), A::res(v), b->p.post_smooth);
        }
    }
    void bottom(int l)
    {
        BLevel& v = b->lev[l];
        launch_batch_bottom(b->st, b->sym, fp32, v.d_probs, v.d_bottoms, (int)v.bottoms.size(), act, b->bc, false,
                            fp32 ? (const void*)BArr<float>::ddw(v) : (const void*)v.ddw64, v.diag64, A::cor(v),
                            A::res(v), v.work, b->p.bottom_max_iter, b->p.bottom_tol_rel, b->p.bottom_tol_abs,
                            b->p.bottom_smooth, b->p.final_smooth, b->omega);
    }
    // MLMG::mgFcycle for every problem (FP32; needs hold32 on every level):
    // the residual restricted to each problem's bottom and solved there, then
    // on the way up each level takes the prolonged correction, a V-cycle from
    // that level on the residual of it, and the sum.  The roles of res/rescor
    // and cor/hold are swapped around the V-cycle instead of copying, and
    // swapped back (the captured graph replays from the same roles).
    void fcycle()
    {
        const int L = b->Lmax;
        for (int l = 0; l + 1 < L; l++) {
            BLevel& v = b->lev[l];
            if (v.t32_smooth.empty()) continue;
            BLevel& c = b->lev[l + 1];
            launch_batch_transfer<T>(b->st, 1, false, b->grid, v.d_probs, c.d_probs, c.c_t32_full,
                                     (int)c.t32_full.size(), act, A::res(v), A::res(c));
        }
        for (int l = 0; l < L; l++)
            if (!b->lev[l].bottoms.empty()) bottom(l);
        for (int l = L - 2; l >= 0; l--) {
            BLevel& v = b->lev[l];
            if (v.t32_smooth.empty()) continue;
            BLevel& c = b->lev[l + 1];
            launch_batch_transfer<T>(b->st, 0, true, b->grid, v.d_probs, c.d_probs, v.c_t32_smooth,
                                     (int)v.t32_smooth.size(), act, A::cor(c), A::cor(v));
            launch_batch_stencil<T>(b->st, b->sym, MODE_RESID, v.shape, b->grid, v.d_probs, v.c_tS_smooth,
                                    (int)v.tS_smooth.size(), act, b->bc, false, A::ddw(v), A::cor(v), A::res(v),
                                    nullptr, A::rescor(v), (T)0, nullptr);
            std::swap(v.res32, v.rescor32);
            std::swap(v.cor32, v.hold32);
            vcycle_from(l, true);
            launch_batch_vec(b->st, BV_AXPY, b->grid, v.d_probs, v.c_t32_smooth, (int)v.t32_smooth.size(), act,
                             v.hold32, v.cor32, 1.0, nullptr, 1);
            std::swap(v.res32, v.rescor32);
            std::swap(v.cor32, v.hold32);
        }
    }
};

agb_status build_levels(agb_batch b)
{
    b->bottom.resize(b->np);
    b->Lmax = 1;
    for (int q = 0; q < b->np; q++) {
        const int nl = levels_of(&b->n[3 * q], b->p.max_coarsening_level < 0 ? 30 : b->p.max_coarsening_level);
        b->bottom[q] = nl - 1;
        b->Lmax = std::max(b->Lmax, nl);
    }
    b->lev.resize(b->Lmax);
    const int d32[3] = {32, 4, 2};
    for (int l = 0; l < b->Lmax; l++) {
        BLevel& v = b->lev[l];
        v.probs.resize(b->np);
        std::vector<int> full, smooth;
        for (int q = 0; q < b->np; q++) {
            BProb& P = v.probs[q];
            memset(&P, 0, sizeof(P));
            P.bottom = b->bottom[q];
            if (l > b->bottom[q]) continue;   // level absent: count 0
            int nc[3];
            double h[3];
            for (int d = 0; d < 3; d++) {
                nc[d] = b->n[3 * q + d] >> l;
                h[d] = b->dx[3 * q + d] * (double)(1 << l);
            }
            P.L = make_level(nc, b->per, h);
            P.vo = v.nvec;
            v.nvec += 3 * P.L.S;
            P.co = v.ncoef;
            v.ncoef += (long long)b->nc * P.L.S;
            for (int d = 0; d < 3; d++) {
                P.h1[d] = 0.5 / h[d];
                P.i1[d] = 1.0 / h[d];
                P.h2[d] = 1.0 / (h[d] * h[d]);
            }
            P.hm[0] = 0.25 / (h[0] * h[1]);
            P.hm[1] = 0.25 / (h[0] * h[2]);
            P.hm[2] = 0.25 / (h[1] * h[2]);
            full.push_back(q);
            if (l < b->bottom[q]) smooth.push_back(q);
            else {
                P.wo = v.nwork;
                v.nwork += 8 * 3 * P.L.S;
                v.bottoms.push_back(q);
            }
        }
        make_tiles(v.probs, full, d32, v.t32_full);
        make_tiles(v.probs, smooth, d32, v.t32_smooth);
        v.shape = 0;
        v.tS_smooth = v.t32_smooth;
        BTRY(b->upload_vec(v.probs, &v.d_probs));
        BTRY(b->upload_vec(v.t32_full, &v.d_t32_full));
        BTRY(b->upload_vec(v.t32_smooth, &v.d_t32_smooth));
        BTRY(b->upload_vec(v.tS_smooth, &v.d_tS_smooth));
        BTRY(b->upload_vec(v.bottoms, &v.d_bottoms));
        BTRY(b->alloc(&v.ddw64, v.ncoef));
        BTRY(b->alloc(&v.diag64, v.nvec));
        BTRY(b->alloc(&v.dinv64, v.nvec));
        BTRY(b->alloc(&v.cor64, v.nvec));
        BTRY(b->alloc(&v.res64, v.nvec));
        BTRY(b->alloc(&v.rescor64, v.nvec));
        BTRY(b->alloc(&v.tmp64, v.nvec));
        BTRY(b->alloc(&v.work, std::max<long long>(v.nwork, 1)));
        if (b->p.precision == AGB_PREC_MIXED) {
            BTRY(b->alloc(&v.ddw32, v.ncoef));
            BTRY(b->alloc(&v.dinv32, v.nvec));
            BTRY(b->alloc(&v.cor32, v.nvec));
            BTRY(b->alloc(&v.res32, v.nvec));
            BTRY(b->alloc(&v.rescor32, v.nvec));
            BTRY(b->alloc(&v.tmp32, v.nvec));
        }
    }
    const long long n0 = b->lev[0].nvec;
    BTRY(b->alloc(&b->x64, n0));
    BTRY(b->alloc(&b->b64, n0));
    if (b->p.precision == AGB_PREC_MIXED) {
        BTRY(b->alloc(&b->rhs32, n0));
        BTRY(b->alloc(&b->sol32, n0));
    }
    BTRY(b->alloc(&b->F0, 9 * (size_t)b->np));
    BTRY(b->alloc(&b->scale, b->np));
    BTRY(b->alloc(&b->sums, 9 * (size_t)b->np));
    BTRY(b->alloc(&b->d_active, b->np));
    BTRY(b->alloc(&b->d_iactive, b->np));
    BTRY(b->alloc(&b->d_norms, b->np));
    if (cudaMallocHost(&b->h_norms, sizeof(double) * b->np) != cudaSuccess)
        return bfail(AGB_NOMEM, "cudaMallocHost failed");
    b->active.assign(b->np, 1);
    b->iactive.assign(b->np, 1);
    return AGB_OK;
}

agb_status prepare(agb_batch b)
{
    if (!b->model_set) return bfail(AGB_STATE, "every problem's model must be set before solving");
    for (int l = 1; l < b->Lmax; l++) {
        BLevel& f = b->lev[l - 1];
        BLevel& c = b->lev[l];
        if (c.t32_full.empty()) continue;
        launch_batch_avg_ddw(b->st, b->grid, f.d_probs, c.d_probs, c.d_t32_full, (int)c.t32_full.size(), f.ddw64,
                             c.ddw64, b->nc);
    }
    for (int l = 0; l < b->Lmax; l++) {
        BLevel& v = b->lev[l];
        launch_batch_diag(b->st, b->sym, b->grid, v.d_probs, v.d_t32_full, (int)v.t32_full.size(), b->bc, v.ddw64,
                          v.diag64, v.dinv64, v.dinv32);
        if (v.ddw32) {
            LevelDesc flat;
            memset(&flat, 0, sizeof(flat));
            flat.S = v.ncoef;
            launch_convert<float, double>(b->st, flat, 1, v.ddw64, v.ddw32, 1.0);
        }
    }
    BCK(cudaGetLastError());
    b->prepared = true;
    return AGB_OK;
}

// time each stencil tile shape on the level's own data (FP32 Jacobi sweeps if
// mixed, else FP64) and keep the fastest
agb_status autotune(agb_batch b)
{
    const bool f32 = b->p.precision == AGB_PREC_MIXED;
    for (int l = 0; l < b->Lmax; l++) {
        BLevel& v = b->lev[l];
        std::vector<int> smooth;
        for (int q = 0; q < b->np; q++)
            if (l < b->bottom[q]) smooth.push_back(q);
        if (smooth.empty()) continue;
        float best = 1e30f;
        int best_s = 0;
        // AGB_BATCH_SHAPE=<shape> skips the timing and takes that shape where it serves
        const char* force = getenv("AGB_BATCH_SHAPE");
        int forced = force ? atoi(force) : -1;
        if (!batch_shape_ok(forced, b->sym, b->per)) forced = -1;
        for (int s = 0; s < batch_shape_count(); s++) {
            if (!batch_shape_ok(s, b->sym, b->per) || (forced >= 0 && s != forced)) continue;
            int dims[3];
            batch_shape_dims(s, dims);
            std::vector<BTile> tl;
            make_tiles(v.probs, smooth, dims, tl);
            BTile* d = nullptr;
            BCK(cudaMalloc(&d, tl.size() * sizeof(BTile)));
            BCK(cudaMemcpyAsync(d, tl.data(), tl.size() * sizeof(BTile), cudaMemcpyHostToDevice, b->st));
            const int reps = 3;
            for (int r = 0; r <= reps; r++) {
                if (r == 1) BCK(cudaEventRecord(b->e0, b->st));
                if (f32)
                    launch_batch_stencil<float>(b->st, b->sym, MODE_JACOBI, s, b->grid, v.d_probs, d, (int)tl.size(),
                                                nullptr, b->bc, false, v.ddw32, v.cor32, v.res32, v.dinv32, v.tmp32,
                                                (float)b->omega, nullptr);
                else
                    launch_batch_stencil<double>(b->st, b->sym, MODE_JACOBI, s, b->grid, v.d_probs, d, (int)tl.size(),
                                                 nullptr, b->bc, false, v.ddw64, v.cor64, v.res64, v.dinv64, v.tmp64,
                                                 b->omega, nullptr);
            }
            BCK(cudaEventRecord(b->e1, b->st));
            BCK(cudaEventSynchronize(b->e1));
            float ms = 0;
            cudaEventElapsedTime(&ms, b->e0, b->e1);
            cudaFree(d);
            if (ms < best) {
                best = ms;
                best_s = s;
            }
        }
        int dims[3];
        batch_shape_dims(best_s, dims);
        v.shape = best_s;
        make_tiles(v.probs, smooth, dims, v.tS_smooth);
        BTRY(b->upload_vec(v.tS_smooth, &v.d_tS_smooth));
    }
    for (auto& v : b->lev) {
        BTRY(b->alloc(&v.c_t32_full, v.t32_full.size()));
        BTRY(b->alloc(&v.c_t32_smooth, v.t32_smooth.size()));
        BTRY(b->alloc(&v.c_tS_smooth, v.tS_smooth.size()));
    }
    b->compact_tiles = -1;
    b->tuned = true;
    return AGB_OK;
}

// Rebuild the compacted tile lists for the problems with mask[q] != 0.  The
// lists stay supersets of the iterating problems' tiles (the kernels still
// check the mask), so they are rebuilt only when the level-0 tile count falls
// by more than 1/16: every skipped tile costs a kernel a dependent load pair.
agb_status compact(agb_batch b, const std::vector<int>& mask)
{
    BLevel& v0 = b->lev[0];
    long long keep = 0;
    for (const BTile& t : v0.t32_full) keep += mask[t.prob] != 0;
    bool subset = b->compact_tiles >= 0 && (int)b->compact_mask.size() == b->np;
    for (int q = 0; q < b->np && subset; q++) subset = !mask[q] || b->compact_mask[q];
    if (subset && keep * 16 > b->compact_tiles * 15) return AGB_OK;
    const BTile end{-1, 0, 0, 0, 0};
    std::vector<BTile> h;
    auto put = [&](const std::vector<BTile>& full, BTile* d) -> agb_status {
        h.clear();
        for (const BTile& t : full)
            if (mask[t.prob]) h.push_back(t);
        h.resize(full.size(), end);
        if (!h.empty()) BCK(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(BTile), cudaMemcpyHostToDevice, b->st));
        // h is reused: the copy must finish before the next list is written
        BCK(cudaStreamSynchronize(b->st));
        return AGB_OK;
    };
    for (auto& v : b->lev) {
        BTRY(put(v.t32_full, v.c_t32_full));
        BTRY(put(v.t32_smooth, v.c_t32_smooth));
        BTRY(put(v.tS_smooth, v.c_tS_smooth));
    }
    b->compact_tiles = keep;
    b->compact_mask = mask;
    return AGB_OK;
}

// Zero-mean projection per problem and component (with the per-problem max
// norm after it into d_norms when norms is set).  A fully periodic box is
// singular (rigid translations) and the operator is not conservative, so its
// left null vectors are constants only up to discretisation error: the solve
// projects the right-hand side and every fine residual (and, in the bottom
// solve, every Krylov residual and operator application), and so finds u with
// A u = b - c for a uniform body force c of the size of that error.
template <typename T> void project(agb_batch b, const int* act, T* y, bool norms, bool compacted = false)
{
    BLevel& v = b->lev[0];
    const BTile* tl = compacted ? v.c_t32_full : v.d_t32_full;
    cudaMemsetAsync(b->sums, 0, sizeof(double) * 3 * b->np, b->st);
    launch_batch_mean3<T>(b->st, b->grid, v.d_probs, tl, (int)v.t32_full.size(), act, y, b->sums, 0);
    launch_batch_mean3<T>(b->st, b->grid, v.d_probs, tl, (int)v.t32_full.size(), act, y, b->sums, 1,
                          norms ? (void*)b->d_norms : nullptr);
}

// compacted: use the lists of the problems still iterating (inside the cycle graphs)
// Stencil tiles of the finest level for all problems: the level's tuned list
// when it covers every problem (each has a coarser level), else the full list
// in the node-per-thread shape.
void fine_tiles(agb_batch b, bool compacted, int* shape, const BTile** tl, int* nt)
{
    BLevel& v = b->lev[0];
    bool tuned = b->tuned && !v.tS_smooth.empty();
    for (int q = 0; tuned && q < b->np; q++) tuned = b->bottom[q] > 0;
    *shape = tuned ? v.shape : 0;
    *tl = tuned ? (compacted ? v.c_tS_smooth : v.d_tS_smooth) : (compacted ? v.c_t32_full : v.d_t32_full);
    *nt = tuned ? (int)v.tS_smooth.size() : (int)v.t32_full.size();
}

template <typename T>
agb_status residual0(agb_batch b, const int* act, const T* x, const T* rhs, T* r, bool compacted = false)
{
    BLevel& v = b->lev[0];
    const bool sing = b->per[0] && b->per[1] && b->per[2];
    BCK(cudaMemsetAsync(b->d_norms, 0, sizeof(double) * b->np, b->st));
    int shape, nt;
    const BTile* tl;
    fine_tiles(b, compacted, &shape, &tl, &nt);
    launch_batch_stencil<T>(b->st, b->sym, MODE_RESID, shape, b->grid, v.d_probs, tl, nt, act, b->bc, false,
                            BArr<T>::ddw(v), x, rhs, nullptr, r, (T)0, sing ? nullptr : b->d_norms);
    if (sing) project<T>(b, act, r, true, compacted);
    BCK(cudaMemcpyAsync(b->h_norms, b->d_norms, sizeof(double) * b->np, cudaMemcpyDeviceToHost, b->st));
    return AGB_OK;
}

double norm_of(agb_batch b, int q, bool f32)
{
    if (!f32) return b->h_norms[q];
    float f;
    memcpy(&f, &b->h_norms[q], sizeof(float));
    return (double)f;
}

template <class Fn> agb_status bcapture(agb_batch b, cudaGraphExec_t* out, long long* kernels, Fn fn)
{
    cudaGraph_t g = nullptr;
    const long long k0 = launch_counter();
    BCK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    fn();
    const cudaError_t e = cudaStreamEndCapture(b->st, &g);
    if (e != cudaSuccess) return bfail(AGB_CUDA, cudaGetErrorString(e));
    *kernels = launch_counter() - k0;
    launch_counter() = k0;
    const cudaError_t e2 = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) return bfail(AGB_CUDA, cudaGetErrorString(e2));
    return AGB_OK;
}

// One GCR iteration of every problem still iterating (d_iactive), with k
// directions stored: z = V(r) (the batched FP32 V-cycle on res32(0), which it
// leaves unchanged), w = A z (projected on fully periodic problems), w and z
// orthogonalised against the stored directions, and the residual minimised
// over the new one; max |r| per problem into the norm slots (FP32 encoding).
void gcr_iter_body(agb_batch b, int k)
{
    BLevel& v0 = b->lev[0];
    const int* act = b->d_iactive;
    const int np = b->np;
    BEngine<float> E{b, act};
    launch_batch_vec(b->st, BV_COPY, b->grid, v0.d_probs, v0.c_t32_full, (int)v0.t32_full.size(), act, v0.res32,
                     b->kr32, 0.0, nullptr, 1);
    if (b->p.max_fmg_iter > 0) E.fcycle();
    else E.vcycle();
    float* z = b->kZ[k];
    float* w = b->kW[k];
    launch_batch_vec(b->st, BV_COPY, b->grid, v0.d_probs, v0.c_t32_full, (int)v0.t32_full.size(), act, z, v0.cor32,
                     0.0, nullptr, 1);
    int shape, nt;
    const BTile* tl;
    fine_tiles(b, true, &shape, &tl, &nt);
    launch_batch_stencil<float>(b->st, b->sym, MODE_APPLY, shape, b->grid, v0.d_probs, tl, nt, act, b->bc, false,
                                v0.ddw32, z, nullptr, nullptr, w, 0.0f, nullptr);
    if (b->per[0] && b->per[1] && b->per[2]) project<float>(b, act, w, false, true);
    cudaMemsetAsync(b->kdots, 0, sizeof(double) * (size_t)np * GCR_MAX, b->st);
    cudaMemsetAsync(b->kd2, 0, sizeof(double) * (size_t)np * 2, b->st);
    if (k > 0) {
        GcrVecs W, Z;
        for (int i = 0; i < k; i++) {
            W.v[i] = b->kW[i];
            Z.v[i] = b->kZ[i];
        }
        launch_batch_multidot(b->st, b->grid, v0.d_probs, v0.c_t32_full, (int)v0.t32_full.size(), act, k, w, W,
                              v0.dinv32, b->kdots, GCR_MAX);
        launch_batch_gcr_orth(b->st, b->grid, v0.d_probs, v0.c_t32_full, (int)v0.t32_full.size(), act, k, b->kdots,
                              GCR_MAX, W, Z, w, z);
    }
    GcrVecs P;
    P.v[0] = w;
    P.v[1] = b->kr32;
    launch_batch_multidot(b->st, b->grid, v0.d_probs, v0.c_t32_full, (int)v0.t32_full.size(), act, 2, w, P,
                          v0.dinv32, b->kd2, 2);
    cudaMemsetAsync(b->d_norms, 0, sizeof(double) * np, b->st);
    launch_batch_gcr_step(b->st, b->grid, v0.d_probs, v0.c_t32_full, (int)v0.t32_full.size(), act, b->kd2, w, z,
                          b->sol32, b->kr32, b->d_norms);
    cudaMemcpyAsync(b->h_norms, b->d_norms, sizeof(double) * np, cudaMemcpyDeviceToHost, b->st);
}

agb_status gcr_setup(agb_batch b, int m)
{
    BLevel& v0 = b->lev[0];
    if (b->p.max_fmg_iter > 0)
        for (auto& v : b->lev)
            if (!v.hold32 && v.nvec > 0) BTRY(b->alloc(&v.hold32, v.nvec));
    while ((int)b->kZ.size() < m) {
        float *z = nullptr, *w = nullptr;
        BTRY(b->alloc(&z, v0.nvec));
        BTRY(b->alloc(&w, v0.nvec));
        b->kZ.push_back(z);
        b->kW.push_back(w);
    }
    if (!b->kdots) {
        BTRY(b->alloc(&b->kdots, (size_t)b->np * GCR_MAX));
        BTRY(b->alloc(&b->kd2, (size_t)b->np * 2));
        BTRY(b->alloc(&b->kr32, v0.nvec));
    }
    b->gk.resize(m, nullptr);
    b->gk_k.resize(m, 0);
    for (int k = 0; k < m; k++)
        if (!b->gk[k]) BTRY(bcapture(b, &b->gk[k], &b->gk_k[k], [&] { gcr_iter_body(b, k); }));
    return AGB_OK;
}

}  // namespace

extern "C" {

agb_status agb_batch_create(int nprob, const int* n_cells, const double* dx, const int periodic[3], int sym,
                            const agb_solver_params* params, agb_batch* out)
{
    if (!out || !n_cells || !dx || nprob < 1) return bfail(AGB_BADARG, "bad argument");
    *out = nullptr;
    if (sym != AGB_ISO && sym != AGB_MAJORMINOR) return bfail(AGB_BADARG, "bad sym");
    for (int q = 0; q < nprob; q++)
        for (int d = 0; d < 3; d++)
            if (n_cells[3 * q + d] < 2 || n_cells[3 * q + d] > 32767 || !(dx[3 * q + d] > 0))
                return bfail(AGB_BADARG, "bad problem size");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return bfail(AGB_CUDA, "no usable CUDA device");
    }
    agb_batch b = new (std::nothrow) agb_batch_s();
    if (!b) return bfail(AGB_NOMEM, "host allocation failed");
    b->np = nprob;
    b->sym = sym;
    b->nc = sym == AGB_ISO ? 2 : 21;
    for (int d = 0; d < 3; d++) b->per[d] = periodic ? (periodic[d] ? 1 : 0) : 1;
    if (params) b->p = *params;
    else agb_default_params(&b->p);
    if (b->p.krylov < 0 || b->p.krylov > GCR_MAX) {
        delete b;
        return bfail(AGB_BADARG, "krylov must be in 0..16");
    }
    if (b->p.omega > 0) b->omega = b->p.omega;
    memset(&b->bc, 0, sizeof(b->bc));
    b->n.assign(n_cells, n_cells + 3 * nprob);
    b->dx.assign(dx, dx + 3 * nprob);
    cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    cudaEventCreate(&b->e0);
    cudaEventCreate(&b->e1);
    b->grid = sm_count() * 4;
    const agb_status s = build_levels(b);
    if (s != AGB_OK) {
        agb_batch_destroy(b);
        return s;
    }
    if (cudaStreamSynchronize(b->st) != cudaSuccess) {
        agb_batch_destroy(b);
        return bfail(AGB_CUDA, "stream sync failed");
    }
    *out = b;
    return AGB_OK;
}

agb_status agb_batch_destroy(agb_batch b)
{
    if (!b) return AGB_OK;
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->g64) cudaGraphExecDestroy(b->g64);
    if (b->g32) cudaGraphExecDestroy(b->g32);
    for (cudaGraphExec_t g : b->gk)
        if (g) cudaGraphExecDestroy(g);
    for (void* v : b->allocs) cudaFree(v);
    if (b->h_norms) cudaFreeHost(b->h_norms);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return AGB_OK;
}

agb_status agb_batch_set_bc(agb_batch b, const agb_bc* bc)
{
    if (!b || !bc) return bfail(AGB_BADARG, "null argument");
    for (int f = 0; f < AGB_NFACES; f++)
        for (int c = 0; c < 3; c++) {
            if (bc->type[f][c] < AGB_BC_DISP || bc->type[f][c] > AGB_BC_NONE) return bfail(AGB_BADARG, "bad BC type");
            b->bc.type[f][c] = (int8_t)bc->type[f][c];
            b->bc.val[f][c] = bc->val[f][c];
        }
    b->prepared = false;
    return AGB_OK;
}

agb_status agb_batch_set_model(agb_batch b, int prob, const double* ddw, int layout, int mem)
{
    if (!b || !ddw || prob < 0 || prob >= b->np) return bfail(AGB_BADARG, "bad argument");
    const BProb& P = b->lev[0].probs[prob];
    const LevelDesc& L = P.L;
    const size_t nfull = (size_t)(L.n[0] + 1) * (L.n[1] + 1) * (L.n[2] + 1) * b->nc;
    const double* src = ddw;
    double* stage = nullptr;
    if (mem == AGB_MEM_DEVICE) BCK(cudaStreamSynchronize(cudaStreamLegacy));   // the caller's writes of ddw
    if (mem == AGB_MEM_HOST) {
        BCK(cudaMalloc(&stage, nfull * sizeof(double)));
        BCK(cudaMemcpyAsync(stage, ddw, nfull * sizeof(double), cudaMemcpyHostToDevice, b->st));
        src = stage;
    }
    launch_import<double, double>(b->st, L, b->nc, src, b->lev[0].ddw64 + P.co, layout == AGB_LAYOUT_AOS, 0, L.nn[2],
                                  false);
    BCK(cudaGetLastError());
    BCK(cudaStreamSynchronize(b->st));
    if (stage) cudaFree(stage);
    b->model_set = true;
    b->prepared = false;
    return AGB_OK;
}

agb_status agb_batch_set_eigenstrain(agb_batch b, const double* F0)
{
    if (!b || !F0) return bfail(AGB_BADARG, "null argument");
    BCK(cudaMemcpyAsync(b->F0, F0, sizeof(double) * 9 * b->np, cudaMemcpyHostToDevice, b->st));
    BCK(cudaStreamSynchronize(b->st));
    b->f0_set = true;
    return AGB_OK;
}

agb_status agb_batch_solve(agb_batch b, double tol_rel, double tol_abs, agb_solve_report* reports,
                           agb_solve_report* total)
{
    if (!b) return bfail(AGB_BADARG, "null batch");
    if (!b->f0_set) return bfail(AGB_STATE, "agb_batch_set_eigenstrain must be called first");
    const bool mixed = b->p.precision == AGB_PREC_MIXED;
    if (!b->prepared) BTRY(prepare(b));
    if (!b->tuned) BTRY(autotune(b));
    BLevel& v0 = b->lev[0];
    const int np = b->np;
    const long long k_start = launch_counter();
    long long replayed = 0;
    BCK(cudaEventRecord(b->e0, b->st));
    // right-hand side of the Newton step at u = 0 and x = 0
    launch_batch_rhs(b->st, b->sym, b->grid, v0.d_probs, v0.d_t32_full, (int)v0.t32_full.size(), v0.ddw64, b->F0, b->b64);
    if (b->per[0] && b->per[1] && b->per[2]) project<double>(b, nullptr, b->b64, false);
    BCK(cudaMemsetAsync(b->x64, 0, sizeof(double) * v0.nvec, b->st));
    b->active.assign(np, 1);
    BCK(cudaMemcpyAsync(b->d_active, b->active.data(), sizeof(int) * np, cudaMemcpyHostToDevice, b->st));
    BTRY(residual0<double>(b, nullptr, b->x64, b->b64, v0.res64));
    BCK(cudaStreamSynchronize(b->st));
    std::vector<double> res0(np), target(np), norm(np), prev(np);
    std::vector<int> iters(np, 0), status(np, AGB_MAXITER), refine(np, 0);
    for (int q = 0; q < np; q++) {
        res0[q] = norm[q] = b->h_norms[q];
        target[q] = std::max(tol_abs, std::max(tol_rel, 1e-16) * res0[q]);
        if (std::isnan(norm[q])) { status[q] = AGB_NAN; b->active[q] = 0; }
        else if (norm[q] <= target[q]) { status[q] = AGB_OK; b->active[q] = 0; }
    }
    BCK(cudaMemcpyAsync(b->d_active, b->active.data(), sizeof(int) * np, cudaMemcpyHostToDevice, b->st));
    auto any = [](const std::vector<int>& a) { return std::any_of(a.begin(), a.end(), [](int x) { return x != 0; }); };

    if (!mixed) {
        if (!b->g64)
            BTRY(bcapture(b, &b->g64, &b->g64_k, [&] {
                BEngine<double> E{b, b->d_active};
                E.vcycle();
                launch_batch_vec(b->st, BV_AXPY, b->grid, v0.d_probs, v0.c_t32_full, (int)v0.t32_full.size(),
                                 b->d_active, b->x64, v0.cor64, 1.0, nullptr, 0);
                residual0<double>(b, b->d_active, b->x64, b->b64, v0.res64, true);
            }));
        for (int it = 0; it < b->p.max_iter && any(b->active); it++) {
            BTRY(compact(b, b->active));
            BCK(cudaGraphLaunch(b->g64, b->st));
            replayed += b->g64_k;
            BCK(cudaStreamSynchronize(b->st));
            for (int q = 0; q < np; q++) {
                if (!b->active[q]) continue;
                iters[q]++;
                norm[q] = b->h_norms[q];
                if (std::isnan(norm[q])) { status[q] = AGB_NAN; b->active[q] = 0; }
                else if (norm[q] <= target[q]) { status[q] = AGB_OK; b->active[q] = 0; }
            }
            BCK(cudaMemcpyAsync(b->d_active, b->active.data(), sizeof(int) * np, cudaMemcpyHostToDevice, b->st));
        }
    } else {
        if (!b->g32)
            BTRY(bcapture(b, &b->g32, &b->g32_k, [&] {
                BEngine<float> E{b, b->d_iactive};
                E.vcycle();
                launch_batch_vec(b->st, BV_AXPY, b->grid, v0.d_probs, v0.c_t32_full, (int)v0.t32_full.size(),
                                 b->d_iactive, b->sol32, v0.cor32, 1.0, nullptr, 1);
                residual0<float>(b, b->d_iactive, b->sol32, b->rhs32, v0.res32, true);
            }));
        const int m = std::min(std::max(b->p.krylov, 0), GCR_MAX);
        if (m > 0) BTRY(gcr_setup(b, m));
        std::vector<double> scale(np, 1.0), itol(np);
        for (int outer = 0; outer < b->p.max_refine && any(b->active); outer++) {
            for (int q = 0; q < np; q++) {
                scale[q] = b->active[q] ? norm[q] : 1.0;
                itol[q] = std::max(b->p.inner_tol_rel, 0.3 * target[q] / norm[q]);
                b->iactive[q] = b->active[q];
                prev[q] = 1.0;
            }
            BCK(cudaMemcpyAsync(b->scale, scale.data(), sizeof(double) * np, cudaMemcpyHostToDevice, b->st));
            BCK(cudaMemcpyAsync(b->d_iactive, b->iactive.data(), sizeof(int) * np, cudaMemcpyHostToDevice, b->st));
            launch_batch_vec(b->st, BV_SCALE_TO32, b->grid, v0.d_probs, v0.d_t32_full, (int)v0.t32_full.size(),
                             b->d_active, b->rhs32, v0.res64, 0.0, b->scale, 1);
            launch_batch_vec(b->st, BV_COPY, b->grid, v0.d_probs, v0.d_t32_full, (int)v0.t32_full.size(), b->d_active,
                             m > 0 ? b->kr32 : v0.res32, b->rhs32, 0.0, nullptr, 1);
            launch_batch_vec(b->st, BV_ZERO, b->grid, v0.d_probs, v0.d_t32_full, (int)v0.t32_full.size(), b->d_active,
                             b->sol32, nullptr, 0.0, nullptr, 1);
            std::vector<int> slow(np, 0);
            for (int it = 0; it < b->p.inner_max_iter && any(b->iactive); it++) {
                BTRY(compact(b, b->iactive));
                if (m > 0) {
                    const int k = it % m;   // restarted when all m directions are stored
                    BCK(cudaGraphLaunch(b->gk[k], b->st));
                    replayed += b->gk_k[k];
                } else {
                    BCK(cudaGraphLaunch(b->g32, b->st));
                    replayed += b->g32_k;
                }
                BCK(cudaStreamSynchronize(b->st));
                for (int q = 0; q < np; q++) {
                    if (!b->iactive[q]) continue;
                    iters[q]++;
                    const double r = norm_of(b, q, true);
                    if (std::isnan(r) || r <= itol[q]) b->iactive[q] = 0;
                    else {
                        slow[q] = r > 0.9 * prev[q] ? slow[q] + 1 : 0;
                        if (slow[q] >= 3) b->iactive[q] = 0;
                    }
                    prev[q] = r;
                }
                BCK(cudaMemcpyAsync(b->d_iactive, b->iactive.data(), sizeof(int) * np, cudaMemcpyHostToDevice, b->st));
            }
            launch_batch_vec(b->st, BV_ACC_FROM32, b->grid, v0.d_probs, v0.d_t32_full, (int)v0.t32_full.size(),
                             b->d_active, b->x64, b->sol32, 0.0, b->scale, 0);
            BTRY(residual0<double>(b, b->d_active, b->x64, b->b64, v0.res64));
            BCK(cudaStreamSynchronize(b->st));
            for (int q = 0; q < np; q++) {
                if (!b->active[q]) continue;
                refine[q]++;
                const double old = norm[q];
                norm[q] = b->h_norms[q];
                if (std::isnan(norm[q])) { status[q] = AGB_NAN; b->active[q] = 0; }
                else if (norm[q] <= target[q]) { status[q] = AGB_OK; b->active[q] = 0; }
                else if (norm[q] > 0.5 * old && refine[q] >= 2 && norm[q] > 0.9 * old) {
                    status[q] = AGB_STALL;
                    b->active[q] = 0;
                }
            }
            BCK(cudaMemcpyAsync(b->d_active, b->active.data(), sizeof(int) * np, cudaMemcpyHostToDevice, b->st));
        }
    }
    // displacement modulo rigid translations: zero mean per problem
    if (b->per[0] && b->per[1] && b->per[2]) project<double>(b, nullptr, b->x64, false);
    BCK(cudaEventRecord(b->e1, b->st));
    BCK(cudaStreamSynchronize(b->st));
    float ms = 0;
    cudaEventElapsedTime(&ms, b->e0, b->e1);
    agb_solve_report tot;
    memset(&tot, 0, sizeof(tot));
    tot.status = AGB_OK;
    for (int q = 0; q < np; q++) {
        if (reports) {
            agb_solve_report& r = reports[q];
            memset(&r, 0, sizeof(r));
            r.iterations = iters[q];
            r.status = status[q];
            r.res0 = res0[q];
            r.res_final = norm[q];
            r.rhs_norm = res0[q];
            r.nlevels = b->bottom[q] + 1;
            r.refinements = refine[q];
            r.solve_ms = ms;
        }
        tot.iterations = std::max(tot.iterations, iters[q]);
        tot.refinements = std::max(tot.refinements, refine[q]);
        if (status[q] != AGB_OK && tot.status == AGB_OK) tot.status = status[q];
        tot.res_final = std::max(tot.res_final, norm[q] / std::max(res0[q], 1e-300));
    }
    tot.nlevels = b->Lmax;
    tot.solve_ms = ms;
    tot.kernels = launch_counter() - k_start + replayed;
    if (total) *total = tot;
    return (agb_status)tot.status;
}

agb_status agb_batch_get_solution(agb_batch b, int prob, double* u, int mem)
{
    if (!b || !u || prob < 0 || prob >= b->np) return bfail(AGB_BADARG, "bad argument");
    const BProb& P = b->lev[0].probs[prob];
    const LevelDesc& L = P.L;
    const size_t nfull = (size_t)(L.n[0] + 1) * (L.n[1] + 1) * (L.n[2] + 1) * 3;
    double* dst = u;
    double* stage = nullptr;
    if (mem == AGB_MEM_DEVICE) BCK(cudaStreamSynchronize(cudaStreamLegacy));   // the caller's use of u
    if (mem == AGB_MEM_HOST) {
        BCK(cudaMalloc(&stage, nfull * sizeof(double)));
        dst = stage;
    }
    launch_export<double, double>(b->st, L, 3, b->x64 + P.vo, dst, false, 0, L.n[2] + 1, false);
    BCK(cudaGetLastError());
    if (stage) BCK(cudaMemcpyAsync(u, stage, nfull * sizeof(double), cudaMemcpyDeviceToHost, b->st));
    BCK(cudaStreamSynchronize(b->st));
    if (stage) cudaFree(stage);
    return AGB_OK;
}

agb_status agb_batch_mean_stress(agb_batch b, double* sigma)
{
    if (!b || !sigma) return bfail(AGB_BADARG, "null argument");
    BLevel& v0 = b->lev[0];
    BCK(cudaMemsetAsync(b->sums, 0, sizeof(double) * 9 * b->np, b->st));
    launch_batch_mean_stress(b->st, b->sym, b->grid, v0.d_probs, v0.d_t32_full, (int)v0.t32_full.size(), v0.ddw64,
                             b->F0, b->x64, b->sums);
    std::vector<double> h(9 * (size_t)b->np);
    BCK(cudaMemcpyAsync(h.data(), b->sums, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, b->st));
    BCK(cudaStreamSynchronize(b->st));
    for (int q = 0; q < b->np; q++) {
        const double cnt = (double)v0.probs[q].L.count();
        for (int a = 0; a < 9; a++) sigma[9 * q + a] = h[9 * q + a] / cnt;
    }
    return AGB_OK;
}

agb_status agb_batch_tuning(agb_batch b, int level, int dims[3])
{
    if (!b || !dims || level < 0 || level >= b->Lmax) return bfail(AGB_BADARG, "bad argument");
    batch_shape_dims(b->lev[level].shape, dims);
    return AGB_OK;
}

}  // extern "C"
