// kernels_batch.cu -- batched solves of many independent boxes (periodic RVEs
// of different sizes) with persistent tile kernels.
//
// A level arena holds every problem's fields of that level back to back
// (BProb gives the offsets).  A tile list names (problem, block) pairs; each
// kernel is launched with a grid sized to the GPU (a few CTAs per SM) and its
// CTAs stride over the tile list, so one launch covers all problems of the
// level whatever their sizes.  Problems already converged are skipped through
// the `active` flags, so the same captured graph serves every iteration.
//
// Per-node arithmetic is the single-box arithmetic of stencil.cuh
// (Operator/Elastic.cpp:141-292; transfers Operator.cpp:262-434).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <unordered_map>

#include "agb_internal.h"
#include "stencil.cuh"
#include "transfer.cuh"

namespace agb {

// The persistent launches ask for `grid` CTAs (a few per SM).  A CTA that is
// not resident from the start runs its share of the tiles after a resident
// one has finished all of its own, which adds a second wave; so each launch is
// trimmed to the CTAs of that kernel (256 threads) that fit on the device at
// once.  Queried once per kernel (the occupancy query is no stream operation,
// so it may also run while a graph is being captured).
static int fit_grid(const void* kernel, int grid, cudaStream_t)
{
    static std::mutex mu;
    static std::unordered_map<const void*, int> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(kernel);
    if (it != cache.end()) return std::min(grid, it->second);
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 256, 0) != cudaSuccess || per < 1 || sms < 1)
        return grid;
    cache[kernel] = sms * per;
    return std::min(grid, sms * per);
}

// Shapes 0-4: one node per thread (k_batch_stencil).  Shape 5: 32 x 8 columns
// marching through 16 planes (k_batch_march), for fully periodic isotropic
// batches only.
static const int kShapes[6][3] = {{32, 4, 2}, {32, 8, 1}, {16, 8, 2}, {8, 8, 4}, {64, 4, 1}, {32, 8, 16}};
constexpr int kMarchShape = 5;
int batch_shape_count() { return 6; }
void batch_shape_dims(int shape, int dims[3])
{
    for (int d = 0; d < 3; d++) dims[d] = kShapes[shape][d];
}
bool batch_shape_ok(int shape, int sym, const int per[3])
{
    if (shape < 0 || shape >= batch_shape_count()) return false;
    if (shape == kMarchShape) return sym == SYM_ISO && per[0] && per[1] && per[2];
    return true;
}

template <typename T> __device__ __forceinline__ Geo<T> geo_of(const BProb& p)
{
    Geo<T> g;
    for (int d = 0; d < 3; d++) {
        g.h1[d] = (T)p.h1[d];
        g.i1[d] = (T)p.i1[d];
        g.h2[d] = (T)p.h2[d];
        g.hm[d] = (T)p.hm[d];
    }
    g.cube = 0;   // the batched kernels keep the general row form
    return g;
}

template <typename T> struct BAcc {
    const T* __restrict__ x;
    const T* __restrict__ c;
    long long S;
    Nbr nb;
    __device__ __forceinline__ long long off(int di, int dj, int dk) const
    {
        return nb.base + nb.o[0][di + 1] + nb.o[1][dj + 1] + nb.o[2][dk + 1];
    }
    __device__ __forceinline__ T u(int p, int di, int dj, int dk) const { return __ldg(x + p * S + off(di, dj, dk)); }
    __device__ __forceinline__ T C(int m, int di, int dj, int dk) const { return __ldg(c + m * S + off(di, dj, dk)); }
};

template <typename T> struct SlotMax;
template <> struct SlotMax<double> {
    static __device__ void put(void* s, int p, double v)
    {
        atomicMax((unsigned long long*)s + p, (unsigned long long)__double_as_longlong(v));
    }
};
template <> struct SlotMax<float> {
    static __device__ void put(void* s, int p, float v) { atomicMax((unsigned int*)s + 2 * p, __float_as_uint(v)); }
};

// block max of v over threads sharing the tile (all of the CTA) -> slot[prob]
template <typename T> __device__ __forceinline__ void tile_max(T v, void* slots, int prob)
{
    __shared__ T red[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        const T w = __shfl_xor_sync(0xffffffffu, v, o);
        v = (w > v || w != w) ? w : v;
    }
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < (int)(blockDim.x >> 5) ? red[lane] : (T)0;
        for (int o = 16; o > 0; o >>= 1) {
            const T w = __shfl_xor_sync(0xffffffffu, v, o);
            v = (w > v || w != w) ? w : v;
        }
        if (lane == 0) SlotMax<T>::put(slots, prob, v);
    }
}

// node of the tile handled by this thread (1D CTA of 256 threads)
template <int BX, int BY, int BZ>
__device__ __forceinline__ bool tile_node(const BTile& t, const LevelDesc& L, int& i, int& j, int& k)
{
    const int tid = threadIdx.x;
    i = t.bx * BX + tid % BX;
    j = t.by * BY + (tid / BX) % BY;
    k = t.bz * BZ + tid / (BX * BY);
    return i < L.nn[0] && j < L.nn[1] && k < L.nn[2];
}

template <typename T, int SYM, int MODE, int BX, int BY, int BZ>
__global__ void __launch_bounds__(256) k_batch_stencil(const BProb* __restrict__ probs, const BTile* __restrict__ tiles,
                                                       int ntiles, const int* __restrict__ active, BCTable bc,
                                                       int uniform, const T* __restrict__ ddw,
                                                       const T* __restrict__ x, const T* __restrict__ b,
                                                       const T* __restrict__ dinv, T* __restrict__ out, T omega,
                                                       void* norm_slots)
{
    // residual norms: each thread keeps its max while the CTA's tiles stay in
    // one problem (tiles are ordered by problem) and the CTA flushes it to the
    // problem's slot when the problem changes
    T nrm = 0;
    int cur = -1;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        if (tl.prob < 0) break;   // compacted list: only end markers follow (uniform over the CTA)
        if (active && !active[tl.prob]) continue;   // uniform over the CTA
        if (MODE == MODE_RESID && norm_slots && tl.prob != cur) {
            if (cur >= 0) tile_max<T>(nrm, norm_slots, cur);
            nrm = 0;
            cur = tl.prob;
        }
        const BProb& P = probs[tl.prob];
        const LevelDesc& L = P.L;
        int i, j, k;
        const bool ok = tile_node<BX, BY, BZ>(tl, L, i, j, k);
        if (ok) {
            const Geo<T> g = geo_of<T>(P);
            const T* xp = x + P.vo;
            BAcc<T> acc{xp, ddw + P.co, L.S, make_nbr(L, i, j, k)};
            const int pos[3] = {i, j, k};
            int mn[3], mx[3];
            bool bnd = false;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                mn[d] = !L.per[d] && pos[d] == 0;
                mx[d] = !L.per[d] && pos[d] == L.n[d];
                bnd = bnd || mn[d] || mx[d];
            }
            T f[3];
            if (bnd) boundary_row<T, SYM>(acc, g, bc, mn, mx, f);
            else interior_row<T, SYM>(acc, g, uniform != 0, f);
            const long long q = P.vo + acc.nb.base;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const long long o = q + c * L.S;
                if (MODE == MODE_APPLY) out[o] = f[c];
                else if (MODE == MODE_RESID) {
                    const T r = b[o] - f[c];
                    out[o] = r;
                    const T a = fabs(r);
                    nrm = (a > nrm || a != a) ? a : nrm;
                } else {
                    out[o] = x[o] + omega * ((b[o] - f[c]) * dinv[o]);
                }
            }
        }
    }
    if (MODE == MODE_RESID && norm_slots && cur >= 0) tile_max<T>(nrm, norm_slots, cur);
}

// ---------------------------------------------------------------------------
// Marching tile kernel for fully periodic batches with isotropic moduli.
//
// A tile is a 32 x 8 block of columns of one problem and a chunk of up to 16
// planes.  The CTA walks its chunk plane by plane with the displacement in a
// shared-memory ring of three haloed planes (k-1, k, k+1) and the moduli in a
// ring of two (k, k+1); the moduli of the own column at k-1 stay in
// registers.  The halo wraps periodically (node -1 is node n-1, node n is
// node 0), so every stored node is an interior node of the stencil.  Each
// value is read from global memory once per tile instead of once per use,
// and the loads of plane k+2 are in flight (in registers) while plane k is
// computed.  The per-node arithmetic is interior_row's, as in k_batch_stencil.
// ---------------------------------------------------------------------------
constexpr int BM_X = 32, BM_Y = 8, BM_Z = 16;
constexpr int BMH_X = BM_X + 2, BMH_Y = BM_Y + 2;
constexpr int BM_HALO = BMH_X * BMH_Y;                  // 340 halo nodes per plane
constexpr int BM_PER_THREAD = (BM_HALO + 255) / 256;    // 2 per thread (256 threads)

template <typename T, int SYM> struct BMarchSmem {
    static constexpr int NC = NCoef<SYM>::value;
    T u[3][3][BM_HALO];    // [ring slot][component][halo node]
    T c[2][NC][BM_HALO];
};

template <typename T, int SYM> struct BMarchAcc {
    const BMarchSmem<T, SYM>* s;
    int h;               // halo-tile index of the node
    int um, u0, up;      // u ring slots of planes k-1, k, k+1
    int c0, cp;          // moduli ring slots of planes k, k+1
    T cm[NCoef<SYM>::value];
    __device__ __forceinline__ T u(int p, int di, int dj, int dk) const
    {
        const int r = dk < 0 ? um : (dk > 0 ? up : u0);
        return s->u[r][p][h + di + BMH_X * dj];
    }
    __device__ __forceinline__ T C(int m, int di, int dj, int dk) const
    {
        if (dk < 0) return cm[m];
        if (dk > 0) return s->c[cp][m][h];
        return s->c[c0][m][h + di + BMH_X * dj];
    }
};

__device__ __forceinline__ int pwrap(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

template <typename T, int SYM, int MODE>
__global__ void __launch_bounds__(256) k_batch_march(const BProb* __restrict__ probs, const BTile* __restrict__ tiles,
                                                     int ntiles, const int* __restrict__ active, int uniform,
                                                     const T* __restrict__ ddw, const T* __restrict__ x,
                                                     const T* __restrict__ b, const T* __restrict__ dinv,
                                                     T* __restrict__ out, T omega, void* norm_slots)
{
    __shared__ __align__(16) BMarchSmem<T, SYM> s;
    constexpr int NC = NCoef<SYM>::value;
    const int tid = threadIdx.x, tx = tid % BM_X, ty = tid / BM_X;
    T nrm = 0;
    int cur = -1;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        if (tl.prob < 0) break;   // compacted list: only end markers follow (uniform over the CTA)
        if (active && !active[tl.prob]) continue;
        if (MODE == MODE_RESID && norm_slots && tl.prob != cur) {
            if (cur >= 0) tile_max<T>(nrm, norm_slots, cur);
            nrm = 0;
            cur = tl.prob;
        }
        const BProb& P = probs[tl.prob];
        const LevelDesc& L = P.L;
        const Geo<T> g = geo_of<T>(P);
        const long long S = L.S, plane = (long long)L.P * L.nn[1];
        const T* xp = x + P.vo;
        const T* cq = ddw + P.co;
        const int i0 = tl.bx * BM_X, j0 = tl.by * BM_Y, k0 = tl.bz * BM_Z;
        const int k1 = min(k0 + BM_Z, L.n[2]);
        const int i = i0 + tx, j = j0 + ty;
        const bool mine = i < L.n[0] && j < L.n[1];
        // in-plane offsets of this thread's halo nodes, wrapped (fixed for the tile)
        long long hoff[BM_PER_THREAD];
#pragma unroll
        for (int q = 0; q < BM_PER_THREAD; q++) {
            const int e = min(tid + 256 * q, BM_HALO - 1);
            hoff[q] = (long long)pwrap(i0 - 1 + e % BMH_X, L.n[0]) +
                      (long long)L.P * pwrap(j0 - 1 + e / BMH_X, L.n[1]);
        }
        T ru[BM_PER_THREAD][3], rc[BM_PER_THREAD][NC];
        auto fetch = [&](int kk) {   // plane kk (wrapped) -> registers
            const long long pk = plane * pwrap(kk, L.n[2]);
#pragma unroll
            for (int q = 0; q < BM_PER_THREAD; q++) {
                if (tid + 256 * q < BM_HALO) {
#pragma unroll
                    for (int c = 0; c < 3; c++) ru[q][c] = __ldg(xp + c * S + hoff[q] + pk);
#pragma unroll
                    for (int m = 0; m < NC; m++) rc[q][m] = __ldg(cq + m * S + hoff[q] + pk);
                }
            }
        };
        auto stash = [&](int ur, int cr, bool with_c) {   // registers -> ring slots
#pragma unroll
            for (int q = 0; q < BM_PER_THREAD; q++) {
                const int e = tid + 256 * q;
                if (e < BM_HALO) {
#pragma unroll
                    for (int c = 0; c < 3; c++) s.u[ur][c][e] = ru[q][c];
                    if (with_c) {
#pragma unroll
                        for (int m = 0; m < NC; m++) s.c[cr][m][e] = rc[q][m];
                    }
                }
            }
        };
        BMarchAcc<T, SYM> acc;
        acc.s = &s;
        acc.h = (tx + 1) + BMH_X * (ty + 1);
        acc.um = 0; acc.u0 = 1; acc.up = 2;
        acc.c0 = 0; acc.cp = 1;
        {
            const long long p = (long long)min(i, L.n[0] - 1) + (long long)L.P * min(j, L.n[1] - 1) +
                                plane * pwrap(k0 - 1, L.n[2]);
#pragma unroll
            for (int m = 0; m < NC; m++) acc.cm[m] = __ldg(cq + m * S + p);
        }
        fetch(k0 - 1);
        stash(0, 0, false);
        fetch(k0);
        stash(1, 0, true);
        fetch(k0 + 1);
        for (int k = k0; k < k1; k++) {
            stash(acc.up, acc.cp, true);
            __syncthreads();
            if (k + 1 < k1) fetch(k + 2);
            if (mine) {
                T f[3];
                interior_row<T, SYM>(acc, g, uniform != 0, f);
                const long long q0 = P.vo + L.idx(i, j, k);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const long long o = q0 + c * S;
                    if (MODE == MODE_APPLY) out[o] = f[c];
                    else if (MODE == MODE_RESID) {
                        const T r = b[o] - f[c];
                        out[o] = r;
                        const T a = fabs(r);
                        nrm = (a > nrm || a != a) ? a : nrm;
                    } else {
                        out[o] = s.u[acc.u0][c][acc.h] + omega * ((b[o] - f[c]) * dinv[o]);
                    }
                }
            }
#pragma unroll
            for (int m = 0; m < NC; m++) acc.cm[m] = s.c[acc.c0][m][acc.h];
            __syncthreads();
            const int r = acc.um;
            acc.um = acc.u0;
            acc.u0 = acc.up;
            acc.up = r;
            acc.c0 ^= 1;
            acc.cp ^= 1;
        }
    }
    if (MODE == MODE_RESID && norm_slots && cur >= 0) tile_max<T>(nrm, norm_slots, cur);
}

// ---------------------------------------------------------------------------
// The FP32 marching tile kernel with asynchronous plane copies.  Same tiles,
// halo wrap and per-node arithmetic as k_batch_march, but every thread
// copies its halo values of a plane global -> shared with 4-byte cp.async
// (the wrapped halo rows are not contiguous), three planes ahead of the
// compute: u in a ring of 4 planes (k-1, k, k+1 and plane k+2 in flight),
// moduli in a ring of 3 (k, k+1, and k+2 in flight); one commit group per
// plane.  The copies of plane k+3 are issued as soon as plane k is done.
// ---------------------------------------------------------------------------
template <int SYM> struct BPipeSmem {
    static constexpr int NC = NCoef<SYM>::value;
    float u[4][3][BM_HALO];
    float c[3][NC][BM_HALO];
};

template <int SYM> struct BPipeAcc {
    const BPipeSmem<SYM>* s;
    int h;
    int um, u0, up, c0, cp;
    float cm[NCoef<SYM>::value];
    __device__ __forceinline__ float u(int p, int di, int dj, int dk) const
    {
        const int r = dk < 0 ? um : (dk > 0 ? up : u0);
        return s->u[r][p][h + di + BMH_X * dj];
    }
    __device__ __forceinline__ float C(int m, int di, int dj, int dk) const
    {
        if (dk < 0) return cm[m];
        if (dk > 0) return s->c[cp][m][h];
        return s->c[c0][m][h + di + BMH_X * dj];
    }
};

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int SYM, int MODE>
__global__ void __launch_bounds__(256, 3) k_batch_pipe(const BProb* __restrict__ probs, const BTile* __restrict__ tiles,
                                                    int ntiles, const int* __restrict__ active, int uniform,
                                                    const float* __restrict__ ddw, const float* __restrict__ x,
                                                    const float* __restrict__ b, const float* __restrict__ dinv,
                                                    float* __restrict__ out, float omega, void* norm_slots)
{
    __shared__ __align__(16) BPipeSmem<SYM> s;
    constexpr int NC = NCoef<SYM>::value;
    const int tid = threadIdx.x, tx = tid % BM_X, ty = tid / BM_X;
    float nrm = 0;
    int cur = -1;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        if (tl.prob < 0) break;   // compacted list: only end markers follow (uniform over the CTA)
        if (active && !active[tl.prob]) continue;
        if (MODE == MODE_RESID && norm_slots && tl.prob != cur) {
            if (cur >= 0) tile_max<float>(nrm, norm_slots, cur);
            nrm = 0;
            cur = tl.prob;
        }
        const BProb& P = probs[tl.prob];
        const LevelDesc& L = P.L;
        const Geo<float> g = geo_of<float>(P);
        const long long S = L.S, plane = (long long)L.P * L.nn[1];
        const float* xp = x + P.vo;
        const float* cq = ddw + P.co;
        const int i0 = tl.bx * BM_X, j0 = tl.by * BM_Y, k0 = tl.bz * BM_Z;
        const int k1 = min(k0 + BM_Z, L.n[2]);
        const int i = i0 + tx, j = j0 + ty;
        const bool mine = i < L.n[0] && j < L.n[1];
        long long hoff[BM_PER_THREAD];
#pragma unroll
        for (int q = 0; q < BM_PER_THREAD; q++) {
            const int e = min(tid + 256 * q, BM_HALO - 1);
            hoff[q] = (long long)pwrap(i0 - 1 + e % BMH_X, L.n[0]) +
                      (long long)L.P * pwrap(j0 - 1 + e / BMH_X, L.n[1]);
        }
        // copies of plane kk: u into ring slot (kk - k0 + 1) % 4, moduli (when
        // with_c) into (kk - k0) % 3; one commit group (empty past the chunk)
        auto issue = [&](int kk, bool with_c) {
            if (kk <= k1) {
                const long long pk = plane * pwrap(kk, L.n[2]);
                const int ur = (kk - k0 + 1) & 3, cr = (kk - k0 + 3) % 3;
#pragma unroll
                for (int q = 0; q < BM_PER_THREAD; q++) {
                    const int e = tid + 256 * q;
                    if (e < BM_HALO) {
#pragma unroll
                        for (int c = 0; c < 3; c++) cp_async4(&s.u[ur][c][e], xp + c * S + hoff[q] + pk);
                        if (with_c) {
#pragma unroll
                            for (int m = 0; m < NC; m++) cp_async4(&s.c[cr][m][e], cq + m * S + hoff[q] + pk);
                        }
                    }
                }
            }
            cp_commit();
        };
        BPipeAcc<SYM> acc;
        acc.s = &s;
        acc.h = (tx + 1) + BMH_X * (ty + 1);
        {
            const long long p = (long long)min(i, L.n[0] - 1) + (long long)L.P * min(j, L.n[1] - 1) +
                                plane * pwrap(k0 - 1, L.n[2]);
#pragma unroll
            for (int m = 0; m < NC; m++) acc.cm[m] = __ldg(cq + m * S + p);
        }
        issue(k0 - 1, false);
        issue(k0, true);
        issue(k0 + 1, true);
        issue(k0 + 2, true);
        // b and 1/D of the own node, one plane ahead in registers
        float bq[3] = {0, 0, 0}, dq[3] = {0, 0, 0};
        auto fetch_bd = [&](int kk, float* bb, float* dd) {
            if (!mine || kk >= k1) return;
            const long long q0 = P.vo + L.idx(i, j, kk);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                if (MODE != MODE_APPLY) bb[c] = __ldg(b + q0 + c * S);
                if (MODE == MODE_JACOBI) dd[c] = __ldg(dinv + q0 + c * S);
            }
        };
        fetch_bd(k0, bq, dq);
        for (int k = k0; k < k1; k++) {
            float bn[3] = {0, 0, 0}, dn[3] = {0, 0, 0};
            fetch_bd(k + 1, bn, dn);
            cp_wait1();   // every group but the newest (plane k+2) has landed
            __syncthreads();
            const int it = k - k0;
            acc.um = it & 3;
            acc.u0 = (it + 1) & 3;
            acc.up = (it + 2) & 3;
            acc.c0 = it % 3;
            acc.cp = (it + 1) % 3;
            if (mine) {
                float f[3];
                interior_row<float, SYM>(acc, g, uniform != 0, f);
                const long long q0 = P.vo + L.idx(i, j, k);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const long long o = q0 + c * S;
                    if (MODE == MODE_APPLY) out[o] = f[c];
                    else if (MODE == MODE_RESID) {
                        const float r = bq[c] - f[c];
                        out[o] = r;
                        const float a = fabsf(r);
                        nrm = (a > nrm || a != a) ? a : nrm;
                    } else {
                        out[o] = s.u[acc.u0][c][acc.h] + omega * ((bq[c] - f[c]) * dq[c]);
                    }
                }
            }
#pragma unroll
            for (int m = 0; m < NC; m++) acc.cm[m] = s.c[acc.c0][m][acc.h];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                bq[c] = bn[c];
                dq[c] = dn[c];
            }
            __syncthreads();
            issue(k + 3, true);   // into the slots of u(k-1) and moduli(k)
        }
        cp_wait0();
        __syncthreads();
    }
    if (MODE == MODE_RESID && norm_slots && cur >= 0) tile_max<float>(nrm, norm_slots, cur);
}

// Full weighting (restriction) or trilinear prolongation between the levels of
// every listed problem.  Tiles cover the destination level.
template <typename T>
__global__ void __launch_bounds__(256) k_batch_transfer(int restrict_not_interp, int assign,
                                                        const BProb* __restrict__ pf, const BProb* __restrict__ pc,
                                                        const BTile* __restrict__ tiles, int ntiles,
                                                        const int* __restrict__ active, const T* __restrict__ src,
                                                        T* __restrict__ dst)
{
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        if (tl.prob < 0) break;   // compacted list: only end markers follow (uniform over the CTA)
        if (active && !active[tl.prob]) continue;
        const LevelDesc& Lf = pf[tl.prob].L;
        const LevelDesc& Lc = pc[tl.prob].L;
        const LevelDesc& Ld = restrict_not_interp ? Lc : Lf;
        // tiles of batched transfers always use the 32x4x2 shape
        int i, j, k;
        if (!tile_node<32, 4, 2>(tl, Ld, i, j, k)) continue;
        if (restrict_not_interp) {
            const bool bI = !Lc.per[0] && (i == 0 || i == Lc.n[0]);
            const bool bJ = !Lc.per[1] && (j == 0 || j == Lc.n[1]);
            const bool bK = !Lc.per[2] && (k == 0 || k == Lc.n[2]);
            const long long q = pc[tl.prob].vo + Lc.idx(i, j, k);
            for (int c = 0; c < 3; c++) {
                const T* s = src + pf[tl.prob].vo + c * Lf.S;
                auto f = [&](int a, int b, int d) -> T {
                    return __ldg(s + Lf.idx(wrapn(2 * i + a, Lf.n[0], Lf.per[0]), wrapn(2 * j + b, Lf.n[1], Lf.per[1]),
                                            wrapn(2 * k + d, Lf.n[2], Lf.per[2])));
                };
                dst[q + c * Lc.S] = full_weight<T>(f, bI, bJ, bK);
            }
        } else {
            const int I = i >> 1, J = j >> 1, K = k >> 1;
            const int I1 = wrapn(I + 1, Lc.n[0], Lc.per[0]), J1 = wrapn(J + 1, Lc.n[1], Lc.per[1]),
                      K1 = wrapn(K + 1, Lc.n[2], Lc.per[2]);
            const bool ei = !(i & 1), ej = !(j & 1), ek = !(k & 1);
            const long long q = pf[tl.prob].vo + Lf.idx(i, j, k);
            for (int c = 0; c < 3; c++) {
                const T* cs = src + pc[tl.prob].vo + c * Lc.S;
                auto C = [&](int a, int b, int d) -> T { return __ldg(cs + Lc.idx(a ? I1 : I, b ? J1 : J, d ? K1 : K)); };
                const T v = interp_node<T>(C, ei, ej, ek);
                T* o = dst + q + c * Lf.S;
                *o = assign ? v : (*o + v);
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_batch_avg_ddw(const BProb* __restrict__ pf, const BProb* __restrict__ pc,
                                                       const BTile* __restrict__ tiles, int ntiles,
                                                       const double* __restrict__ fine, double* __restrict__ crse,
                                                       int ncoef)
{
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        const LevelDesc& Lf = pf[tl.prob].L;
        const LevelDesc& Lc = pc[tl.prob].L;
        int I, J, K;
        if (!tile_node<32, 4, 2>(tl, Lc, I, J, K)) continue;
        const bool bI = !Lc.per[0] && (I == 0 || I == Lc.n[0]);
        const bool bJ = !Lc.per[1] && (J == 0 || J == Lc.n[1]);
        const bool bK = !Lc.per[2] && (K == 0 || K == Lc.n[2]);
        const long long q = pc[tl.prob].co + Lc.idx(I, J, K);
        for (int m = 0; m < ncoef; m++) {
            const double* s = fine + pf[tl.prob].co + m * Lf.S;
            auto f = [&](int a, int b, int d) -> double {
                return s[Lf.idx(wrapn(2 * I + a, Lf.n[0], Lf.per[0]), wrapn(2 * J + b, Lf.n[1], Lf.per[1]),
                                wrapn(2 * K + d, Lf.n[2], Lf.per[2]))];
            };
            crse[q + m * Lc.S] = full_weight<double>(f, bI, bJ, bK);
        }
    }
}

template <int SYM>
__global__ void __launch_bounds__(256) k_batch_diag(const BProb* __restrict__ probs, const BTile* __restrict__ tiles,
                                                    int ntiles, BCTable bc, const double* __restrict__ ddw,
                                                    double* __restrict__ diag, double* __restrict__ dinv64,
                                                    float* __restrict__ dinv32)
{
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        const BProb& P = probs[tl.prob];
        const LevelDesc& L = P.L;
        int i, j, k;
        if (!tile_node<32, 4, 2>(tl, L, i, j, k)) continue;
        const int pos[3] = {i, j, k};
        int mn[3], mx[3];
        for (int d = 0; d < 3; d++) {
            mn[d] = !L.per[d] && pos[d] == 0;
            mx[d] = !L.per[d] && pos[d] == L.n[d];
        }
        const long long p = L.idx(i, j, k);
        double c[NCoef<SYM>::value];
        for (int m = 0; m < NCoef<SYM>::value; m++) c[m] = ddw[P.co + m * L.S + p];
        const DiagGeo<double> dg = make_diag_geo<double>(L);
        for (int q = 0; q < 3; q++) {
            const double d = diag_entry<double, SYM>(c, L, dg, bc, mn, mx, q);
            const long long o = P.vo + q * L.S + p;
            diag[o] = d;
            dinv64[o] = d != 0.0 ? 1.0 / d : 0.0;
            if (dinv32) dinv32[o] = d != 0.0 ? (float)(1.0 / d) : 0.0f;
        }
    }
}

// Per-node vector operations over the listed problems (3 components).
//   BV_ZERO        y = 0
//   BV_COPY        y = x
//   BV_AXPY        y += a x
//   BV_SCALE_TO32  y(float) = x(double) / scale[prob]
//   BV_ACC_FROM32  y(double) += x(float) * scale[prob]
//   BV_JACOBI0     y = a (x * x2): the first damped-Jacobi sweep from a zero
//                  guess (x the right-hand side, x2 = 1/D, a = omega), the
//                  sweep kernels' expression with A 0 = 0
__global__ void __launch_bounds__(256) k_batch_vec(int op, const BProb* __restrict__ probs,
                                                   const BTile* __restrict__ tiles, int ntiles,
                                                   const int* __restrict__ active, void* y, const void* x, double a,
                                                   const double* __restrict__ scale, int fp32, const void* x2)
{
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        if (tl.prob < 0) break;   // compacted list: only end markers follow (uniform over the CTA)
        if (active && !active[tl.prob]) continue;
        const BProb& P = probs[tl.prob];
        int i, j, k;
        if (!tile_node<32, 4, 2>(tl, P.L, i, j, k)) continue;
        const long long q0 = P.vo + P.L.idx(i, j, k);
        for (int c = 0; c < 3; c++) {
            const long long q = q0 + c * P.L.S;
            if (op == BV_SCALE_TO32) {
                ((float*)y)[q] = (float)(((const double*)x)[q] / scale[tl.prob]);
            } else if (op == BV_ACC_FROM32) {
                ((double*)y)[q] += (double)((const float*)x)[q] * scale[tl.prob];
            } else if (fp32) {
                float* yy = (float*)y;
                const float* xx = (const float*)x;
                if (op == BV_ZERO) yy[q] = 0.f;
                else if (op == BV_COPY) yy[q] = xx[q];
                else if (op == BV_JACOBI0) yy[q] = (float)a * (xx[q] * ((const float*)x2)[q]);
                else yy[q] += (float)a * xx[q];
            } else {
                double* yy = (double*)y;
                const double* xx = (const double*)x;
                if (op == BV_ZERO) yy[q] = 0.0;
                else if (op == BV_COPY) yy[q] = xx[q];
                else if (op == BV_JACOBI0) yy[q] = a * (xx[q] * ((const double*)x2)[q]);
                else yy[q] += a * xx[q];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// bottom solves: one CTA per problem (BiCGStab on the diagonally scaled
// system + smoothing, as the single-box k_bottom).  On a fully periodic box
// the Krylov residual and every operator application are projected to zero
// mean per component (the box is singular: rigid translations).
// ---------------------------------------------------------------------------
constexpr int BB_THREADS = 256;

template <typename R> __device__ __forceinline__ R bsum(R v, R* red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        R t = threadIdx.x < (BB_THREADS / 32) ? red[threadIdx.x] : (R)0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) red[32] = t;
    }
    __syncthreads();
    return red[32];
}

template <typename R> __device__ __forceinline__ R bmax(R v, R* red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        const R w = __shfl_xor_sync(0xffffffffu, v, o);
        v = (w > v || w != w) ? w : v;
    }
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        R t = threadIdx.x < (BB_THREADS / 32) ? red[threadIdx.x] : (R)0;
        for (int o = 16; o > 0; o >>= 1) {
            const R w = __shfl_xor_sync(0xffffffffu, t, o);
            t = (w > t || w != w) ? w : t;
        }
        if (threadIdx.x == 0) red[32] = t;
    }
    __syncthreads();
    return red[32];
}

template <typename R, int SYM>
__device__ void bapply(const BProb& P, const BCTable& bc, int uniform, const R* ddw, const R* x, R* y)
{
    const LevelDesc& L = P.L;
    const Geo<R> g = geo_of<R>(P);
    const long long cnt = L.count();
    for (long long e = threadIdx.x; e < cnt; e += blockDim.x) {
        const int i = (int)(e % L.nn[0]), j = (int)((e / L.nn[0]) % L.nn[1]),
                  k = (int)(e / ((long long)L.nn[0] * L.nn[1]));
        BAcc<R> acc{x, ddw, L.S, make_nbr(L, i, j, k)};
        const int pos[3] = {i, j, k};
        int mn[3], mx[3];
        bool bnd = false;
        for (int d = 0; d < 3; d++) {
            mn[d] = !L.per[d] && pos[d] == 0;
            mx[d] = !L.per[d] && pos[d] == L.n[d];
            bnd = bnd || mn[d] || mx[d];
        }
        R f[3];
        if (bnd) boundary_row<R, SYM>(acc, g, bc, mn, mx, f);
        else interior_row<R, SYM>(acc, g, uniform != 0, f);
        for (int c = 0; c < 3; c++) y[c * L.S + acc.nb.base] = f[c];
    }
}

template <typename R> __device__ void bmean3(const LevelDesc& L, const R* v, R* red, R m[3])
{
    const long long cnt = L.count();
    R s0 = 0, s1 = 0, s2 = 0;
    for (long long e = threadIdx.x; e < cnt; e += blockDim.x) {
        const long long q = L.idx((int)(e % L.nn[0]), (int)((e / L.nn[0]) % L.nn[1]),
                                  (int)(e / ((long long)L.nn[0] * L.nn[1])));
        s0 += v[q];
        s1 += v[L.S + q];
        s2 += v[2 * L.S + q];
    }
    m[0] = bsum(s0, red) / (R)cnt;
    m[1] = bsum(s1, red) / (R)cnt;
    m[2] = bsum(s2, red) / (R)cnt;
}

#define BFOR(q)                                                                                        \
    for (long long e_ = threadIdx.x; e_ < cnt; e_ += blockDim.x)                                       \
        for (int c_ = 0, i_ = (int)(e_ % L.nn[0]), j_ = (int)((e_ / L.nn[0]) % L.nn[1]),                \
                 k_ = (int)(e_ / ((long long)L.nn[0] * L.nn[1]));                                      \
             c_ < 3; c_++)                                                                             \
            for (long long q = c_ * L.S + L.idx(i_, j_, k_), once_ = 0; once_ < 1; once_++)

template <typename T, int SYM>
__global__ void __launch_bounds__(BB_THREADS) k_batch_bottom(const BProb* __restrict__ probs, const int* __restrict__ plist,
                                                            const int* __restrict__ active, BCTable bc, int uniform,
                                                            const T* __restrict__ ddw_all,
                                                            const double* __restrict__ diag_all, T* __restrict__ cor_all,
                                                            const T* __restrict__ res_all, double* __restrict__ work_all,
                                                            int maxiter, double eps_rel_d, double eps_abs_d, int nub,
                                                            int nuf, double omega_d)
{
    typedef T R;   // arithmetic in the cycle's precision
    const R eps_rel = (R)eps_rel_d, eps_abs = (R)eps_abs_d, omega = (R)omega_d;
    __shared__ R red[33];
    const int pid = plist[blockIdx.x];
    if (active && !active[pid]) return;
    const BProb& P = probs[pid];
    const LevelDesc& L = P.L;
    const long long n3 = 3 * L.S, cnt = L.count();
    const R* ddw = ddw_all + P.co;
    const double* diag = diag_all + P.vo;
    T* cor = cor_all + P.vo;
    const T* res = res_all + P.vo;
    R* w = reinterpret_cast<R*>(work_all + P.wo);
    R *r = w, *rh = w + n3, *p = w + 2 * n3, *v = w + 3 * n3, *s = w + 4 * n3, *t = w + 5 * n3, *sol = w + 6 * n3,
           *b = w + 7 * n3;
    BFOR(q)
    {
        b[q] = (R)res[q];
        sol[q] = 0.0;
    }
    __syncthreads();
    const bool sing = L.singular();
    R mb[3] = {0, 0, 0};
    if (sing) bmean3(L, b, red, mb);
    R lm = 0;
    BFOR(q)
    {
        r[q] = (b[q] - mb[c_]) / (R)diag[q];
        rh[q] = r[q];
        const R a = fabs(r[q]);
        lm = (a > lm || a != a) ? a : lm;
    }
    R rnorm = bmax(lm, red);
    const R rnorm0 = rnorm;
    int ret = 0;
    R rho_1 = 0, alpha = 0, om = 0;
    if (!(rnorm0 == 0 || rnorm0 < eps_abs)) {
        for (int iter = 1; iter <= maxiter; iter++) {
            R acc = 0;
            BFOR(q) acc += rh[q] * r[q];
            const R rho = bsum(acc, red);
            if (rho == 0) { ret = 1; break; }
            if (iter == 1) {
                BFOR(q) p[q] = r[q];
            } else {
                const R beta = (rho / rho_1) * (alpha / om);
                BFOR(q) p[q] = r[q] + beta * (p[q] - om * v[q]);
            }
            __syncthreads();
            bapply<R, SYM>(P, bc, uniform, ddw, p, v);
            __syncthreads();
            R mv[3] = {0, 0, 0};
            if (sing) bmean3(L, v, red, mv);
            acc = 0;
            BFOR(q)
            {
                v[q] = (v[q] - mv[c_]) / (R)diag[q];
                acc += rh[q] * v[q];
            }
            const R rhTv = bsum(acc, red);
            if (rhTv != 0) alpha = rho / rhTv;
            else { ret = 2; break; }
            lm = 0;
            BFOR(q)
            {
                sol[q] += alpha * p[q];
                s[q] = r[q] - alpha * v[q];
                const R a = fabs(s[q]);
                lm = (a > lm || a != a) ? a : lm;
            }
            rnorm = bmax(lm, red);
            if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
            bapply<R, SYM>(P, bc, uniform, ddw, s, t);
            __syncthreads();
            R mt[3] = {0, 0, 0};
            if (sing) bmean3(L, t, red, mt);
            R tt = 0, ts = 0;
            BFOR(q)
            {
                t[q] = (t[q] - mt[c_]) / (R)diag[q];
                tt += t[q] * t[q];
                ts += t[q] * s[q];
            }
            tt = bsum(tt, red);
            ts = bsum(ts, red);
            if (tt != 0) om = ts / tt;
            else { ret = 3; break; }
            lm = 0;
            BFOR(q)
            {
                sol[q] += om * s[q];
                r[q] = s[q] - om * t[q];
                const R a = fabs(r[q]);
                lm = (a > lm || a != a) ? a : lm;
            }
            rnorm = bmax(lm, red);
            if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
            if (om == 0) { ret = 4; break; }
            rho_1 = rho;
        }
        if (ret == 0 && rnorm > eps_rel * rnorm0 && rnorm > eps_abs) ret = 8;
        if (ret != 0) {
            BFOR(q) sol[q] = 0.0;
        }
    }
    __syncthreads();
    const int nsm = 2 * ((ret == 0) ? nub : nuf);
    for (int sw = 0; sw < nsm; sw++) {
        bapply<R, SYM>(P, bc, uniform, ddw, sol, t);
        __syncthreads();
        BFOR(q)
        {
            const R Rx = t[q] - sol[q] * (R)diag[q];
            s[q] = ((R)1 - omega) * sol[q] + omega * (b[q] - Rx) / (R)diag[q];
        }
        __syncthreads();
        BFOR(q) sol[q] = s[q];
        __syncthreads();
    }
    BFOR(q) cor[q] = (T)sol[q];
}

// rhs = -div(C : (0 - F0)) with a uniform eigenstrain F0 per problem: the
// Newton right-hand side at u = 0 of an affine model (Newton.H:199-231,
// Model/Solid/Affine/Isotropic.H:42-45) on a fully periodic box.
template <int SYM>
__global__ void __launch_bounds__(256) k_batch_rhs(const BProb* __restrict__ probs, const BTile* __restrict__ tiles,
                                                   int ntiles, const double* __restrict__ ddw,
                                                   const double* __restrict__ F0, double* __restrict__ rhs)
{
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        const BProb& P = probs[tl.prob];
        const LevelDesc& L = P.L;
        int i, j, k;
        if (!tile_node<32, 4, 2>(tl, L, i, j, k)) continue;
        const Nbr nb = make_nbr(L, i, j, k);
        double E[3][3];
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) E[a][c] = 0.0 - F0[tl.prob * 9 + a * 3 + c];
        double ret[3] = {0, 0, 0};
        for (int d = 0; d < 3; d++) {
            double cpv[NCoef<SYM>::value], cmv[NCoef<SYM>::value], Dp[3][3], Dm[3][3];
            for (int m = 0; m < NCoef<SYM>::value; m++) {
                cpv[m] = ddw[P.co + m * L.S + nb.base + nb.o[d][2]];
                cmv[m] = ddw[P.co + m * L.S + nb.base + nb.o[d][0]];
            }
            c_mul_mat<double, SYM>(cpv, E, Dp);
            c_mul_mat<double, SYM>(cmv, E, Dm);
            for (int r = 0; r < 3; r++) ret[r] += (Dp[r][d] - Dm[r][d]) / 2. / L.dx[d];
        }
        for (int r = 0; r < 3; r++) rhs[P.vo + r * L.S + nb.base] = 0.0 - ret[r];
    }
}

// Per-problem sums of sigma = C : (grad u - F0) over the stored nodes
// (central differences; fully periodic boxes), for the homogenized stress.
template <int SYM>
__global__ void __launch_bounds__(256) k_batch_mean_stress(const BProb* __restrict__ probs,
                                                           const BTile* __restrict__ tiles, int ntiles,
                                                           const double* __restrict__ ddw,
                                                           const double* __restrict__ F0,
                                                           const double* __restrict__ u, double* __restrict__ sums)
{
    __shared__ double red[9][8];
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        const BProb& P = probs[tl.prob];
        const LevelDesc& L = P.L;
        int i, j, k;
        double S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        if (tile_node<32, 4, 2>(tl, L, i, j, k)) {
            const Nbr nb = make_nbr(L, i, j, k);
            double G[3][3], c[NCoef<SYM>::value];
            for (int p = 0; p < 3; p++)
                for (int d = 0; d < 3; d++)
                    G[p][d] = (u[P.vo + p * L.S + nb.base + nb.o[d][2]] - u[P.vo + p * L.S + nb.base + nb.o[d][0]]) *
                                  0.5 / L.dx[d] -
                              F0[tl.prob * 9 + p * 3 + d];
            for (int m = 0; m < NCoef<SYM>::value; m++) c[m] = ddw[P.co + m * L.S + nb.base];
            c_mul_mat<double, SYM>(c, G, S);
        }
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int a = 0; a < 9; a++) {
            double v = S[a / 3][a % 3];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) red[a][warp] = v;
        }
        __syncthreads();
        if (threadIdx.x < 9) {
            double v = 0;
            for (int w = 0; w < 8; w++) v += red[threadIdx.x][w];
            atomicAdd(&sums[tl.prob * 9 + threadIdx.x], v);
        }
        __syncthreads();
    }
}

// per-problem component sums over the stored nodes (sums[prob*3 + c]); with
// `subtract`, y -= sums/count instead
template <typename T>
__global__ void __launch_bounds__(256) k_batch_mean3(const BProb* __restrict__ probs, const BTile* __restrict__ tiles,
                                                     int ntiles, const int* __restrict__ active, T* __restrict__ y,
                                                     double* __restrict__ sums, int subtract, void* norm_slots)
{
    // A CTA visits tiles t, t + gridDim.x, ...; tiles are ordered by problem, so
    // consecutive visits mostly stay in one problem.  Each thread accumulates
    // its sums (or its max |y|) while the problem stays the same, and the CTA
    // reduces and flushes them with one atomic per value when it changes.
    __shared__ double red[3][8];
    T s0 = 0, s1 = 0, s2 = 0;   // a thread's sums over its few nodes of one problem, in T
    T m = 0;
    T mean[3] = {0, 0, 0};      // subtract: the current problem's means (one division per problem change)
    int cur = -1;
    auto flush = [&]() {   // called by every thread of the CTA together
        if (cur < 0) return;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (subtract) {
            if (norm_slots) tile_max<T>(m, norm_slots, cur);
        } else {
            double v[3] = {(double)s0, (double)s1, (double)s2};
            for (int c = 0; c < 3; c++) {
                for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
                if (lane == 0) red[c][warp] = v[c];
            }
            __syncthreads();
            if (threadIdx.x < 3) {
                double t = 0;
                for (int w = 0; w < 8; w++) t += red[threadIdx.x][w];
                atomicAdd(&sums[cur * 3 + threadIdx.x], t);
            }
            __syncthreads();
        }
        s0 = s1 = s2 = 0;
        m = 0;
    };
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        if (tl.prob < 0) break;   // compacted list: only end markers follow (uniform over the CTA)
        if (active && !active[tl.prob]) continue;   // uniform over the CTA
        const BProb& P = probs[tl.prob];
        if (tl.prob != cur) {
            flush();
            cur = tl.prob;
            if (subtract) {
                const double cnt = (double)P.L.count();
                for (int c = 0; c < 3; c++) mean[c] = (T)(sums[cur * 3 + c] / cnt);
            }
        }
        int i, j, k;
        if (!tile_node<32, 4, 2>(tl, P.L, i, j, k)) continue;
        const long long q = P.vo + P.L.idx(i, j, k);
        if (subtract) {
            for (int c = 0; c < 3; c++) {
                const T v = y[q + c * P.L.S] - mean[c];
                y[q + c * P.L.S] = v;
                const T a = fabs(v);
                m = (a > m || a != a) ? a : m;
            }
        } else {
            s0 += y[q];
            s1 += y[q + P.L.S];
            s2 += y[q + 2 * P.L.S];
        }
    }
    flush();
}

template <typename T>
void launch_batch_mean3(cudaStream_t st, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                        const int* active, T* y, double* sums, int subtract, void* norm_slots)
{
    grid = fit_grid((const void*)k_batch_mean3<T>, grid, st);
    k_batch_mean3<T><<<grid, 256, 0, st>>>(probs, tiles, ntiles, active, y, sums, subtract, norm_slots);
    count_launch();
}
template void launch_batch_mean3<double>(cudaStream_t, int, const BProb*, const BTile*, int, const int*, double*,
                                         double*, int, void*);
template void launch_batch_mean3<float>(cudaStream_t, int, const BProb*, const BTile*, int, const int*, float*,
                                        double*, int, void*);

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
// The FP32 marching shape uses the asynchronous-copy kernel unless
// AGB_BATCH_PIPE=0 (then the register-prefetch kernel, as for FP64).
static bool batch_pipe_enabled()
{
    static const bool v = [] {
        const char* e = getenv("AGB_BATCH_PIPE");
        return !(e && e[0] == '0');
    }();
    return v;
}

template <typename T, int SYM, int MODE>
static void bst_shape(cudaStream_t st, int shape, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                      const int* active, const BCTable& bc, bool uniform, const T* ddw, const T* x, const T* b,
                      const T* dinv, T* out, T omega, void* norm)
{
#define L_(BX, BY, BZ)                                                                                      \
    grid = fit_grid((const void*)k_batch_stencil<T, SYM, MODE, BX, BY, BZ>, grid, st);                           \
    k_batch_stencil<T, SYM, MODE, BX, BY, BZ><<<grid, 256, 0, st>>>(probs, tiles, ntiles, active, bc, uniform ? 1 : 0, \
                                                                     ddw, x, b, dinv, out, omega, norm)
    // the marching shape is only chosen for isotropic fully periodic batches
    // (batch_shape_ok)
    if constexpr (SYM == SYM_ISO) {
        if (shape == kMarchShape) {
            if constexpr (sizeof(T) == 4) {
                if (batch_pipe_enabled()) {
                    grid = fit_grid((const void*)k_batch_pipe<SYM, MODE>, grid, st);
                    k_batch_pipe<SYM, MODE><<<grid, 256, 0, st>>>(probs, tiles, ntiles, active, uniform ? 1 : 0,
                                                                  (const float*)ddw, (const float*)x, (const float*)b,
                                                                  (const float*)dinv, (float*)out, (float)omega, norm);
                    count_launch();
                    return;
                }
            }
            grid = fit_grid((const void*)k_batch_march<T, SYM, MODE>, grid, st);
            k_batch_march<T, SYM, MODE><<<grid, 256, 0, st>>>(probs, tiles, ntiles, active, uniform ? 1 : 0, ddw, x, b,
                                                              dinv, out, omega, norm);
            count_launch();
            return;
        }
    }
    switch (shape) {
    case 0: L_(32, 4, 2); break;
    case 1: L_(32, 8, 1); break;
    case 2: L_(16, 8, 2); break;
    case 3: L_(8, 8, 4); break;
    default: L_(64, 4, 1); break;
    }
#undef L_
    count_launch();
}

template <typename T>
void launch_batch_stencil(cudaStream_t st, int sym, int mode, int shape, int grid, const BProb* probs,
                          const BTile* tiles, int ntiles, const int* active, const BCTable& bc, bool uniform,
                          const T* ddw, const T* x, const T* b, const T* dinv, T* out, T omega, void* norm_slots)
{
#define D_(S, M) bst_shape<T, S, M>(st, shape, grid, probs, tiles, ntiles, active, bc, uniform, ddw, x, b, dinv, out, omega, norm_slots)
    if (sym == SYM_ISO) {
        if (mode == MODE_APPLY) D_(SYM_ISO, MODE_APPLY);
        else if (mode == MODE_RESID) D_(SYM_ISO, MODE_RESID);
        else D_(SYM_ISO, MODE_JACOBI);
    } else {
        if (mode == MODE_APPLY) D_(SYM_MM, MODE_APPLY);
        else if (mode == MODE_RESID) D_(SYM_MM, MODE_RESID);
        else D_(SYM_MM, MODE_JACOBI);
    }
#undef D_
}

template <typename T>
void launch_batch_transfer(cudaStream_t st, int restrict_not_interp, bool assign, int grid, const BProb* pf,
                           const BProb* pc, const BTile* tiles, int ntiles, const int* active, const T* src, T* dst)
{
    grid = fit_grid((const void*)k_batch_transfer<T>, grid, st);
    k_batch_transfer<T><<<grid, 256, 0, st>>>(restrict_not_interp, assign ? 1 : 0, pf, pc, tiles, ntiles, active, src,
                                              dst);
    count_launch();
}

void launch_batch_avg_ddw(cudaStream_t st, int grid, const BProb* pf, const BProb* pc, const BTile* tiles, int ntiles,
                          const double* fine, double* crse, int ncoef)
{
    k_batch_avg_ddw<<<grid, 256, 0, st>>>(pf, pc, tiles, ntiles, fine, crse, ncoef);
    count_launch();
}

void launch_batch_diag(cudaStream_t st, int sym, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                       const BCTable& bc, const double* ddw, double* diag, double* dinv64, float* dinv32)
{
    if (sym == SYM_ISO) k_batch_diag<SYM_ISO><<<grid, 256, 0, st>>>(probs, tiles, ntiles, bc, ddw, diag, dinv64, dinv32);
    else k_batch_diag<SYM_MM><<<grid, 256, 0, st>>>(probs, tiles, ntiles, bc, ddw, diag, dinv64, dinv32);
    count_launch();
}

void launch_batch_vec(cudaStream_t st, int op, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                      const int* active, void* y, const void* x, double a, const double* scale, int fp32,
                      const void* x2)
{
    grid = fit_grid((const void*)k_batch_vec, grid, st);
    k_batch_vec<<<grid, 256, 0, st>>>(op, probs, tiles, ntiles, active, y, x, a, scale, fp32, x2);
    count_launch();
}

// ---------------------------------------------------------------------------
// Per-problem GCR over the batched FP32 cycle (the single-box inner_gcr32 on
// every problem at once).  Tiles are the 32 x 4 x 2 lists, ordered by
// problem; a CTA flushes its sums to the problem's slots when its tiles move
// to another problem.  Inner products are weighted by d^2 (d = 1/diag).
// ---------------------------------------------------------------------------

// out[p * stride + i] += sum over problem p's nodes of x v_i d^2, i < K
template <int K>
__global__ void __launch_bounds__(256) k_batch_multidot(const BProb* __restrict__ probs,
                                                        const BTile* __restrict__ tiles, int ntiles,
                                                        const int* __restrict__ active, const float* __restrict__ x,
                                                        GcrVecs V, const float* __restrict__ d,
                                                        double* __restrict__ out, int stride)
{
    __shared__ double red[K][8];
    float acc[K];
#pragma unroll
    for (int i = 0; i < K; i++) acc[i] = 0;
    int cur = -1;
    auto flush = [&]() {   // every thread of the CTA together
        if (cur < 0) return;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for (int i = 0; i < K; i++) {
            double a = (double)acc[i];
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            if (lane == 0) red[i][warp] = a;
            acc[i] = 0;
        }
        __syncthreads();
        if (threadIdx.x < K) {
            double t = 0;
            for (int w = 0; w < 8; w++) t += red[threadIdx.x][w];
            atomicAdd(out + (long long)cur * stride + threadIdx.x, t);
        }
        __syncthreads();
    };
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        if (tl.prob < 0) break;   // compacted list: only end markers follow (uniform over the CTA)
        if (active && !active[tl.prob]) continue;
        if (tl.prob != cur) {
            flush();
            cur = tl.prob;
        }
        const BProb& P = probs[tl.prob];
        int i, j, k;
        if (!tile_node<32, 4, 2>(tl, P.L, i, j, k)) continue;
        const long long q = P.vo + P.L.idx(i, j, k);
        for (int c = 0; c < 3; c++) {
            const long long e = q + c * P.L.S;
            const float dd = d[e];
            const float xw = x[e] * dd * dd;
#pragma unroll
            for (int m = 0; m < K; m++) acc[m] += xw * V.v[m][e];
        }
    }
    flush();
}

// w -= sum_i beta_i(p) W_i, z -= sum_i beta_i(p) Z_i on problem p's nodes, i < K
template <int K>
__global__ void __launch_bounds__(256) k_batch_gcr_orth(const BProb* __restrict__ probs,
                                                        const BTile* __restrict__ tiles, int ntiles,
                                                        const int* __restrict__ active,
                                                        const double* __restrict__ beta, int stride, GcrVecs W,
                                                        GcrVecs Z, float* __restrict__ w, float* __restrict__ z)
{
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        if (tl.prob < 0) break;
        if (active && !active[tl.prob]) continue;
        const BProb& P = probs[tl.prob];
        int i, j, k;
        if (!tile_node<32, 4, 2>(tl, P.L, i, j, k)) continue;
        float bb[K];
#pragma unroll
        for (int m = 0; m < K; m++) bb[m] = (float)beta[(long long)tl.prob * stride + m];
        const long long q = P.vo + P.L.idx(i, j, k);
        for (int c = 0; c < 3; c++) {
            const long long e = q + c * P.L.S;
            float tw = w[e], tz = z[e];
#pragma unroll
            for (int m = 0; m < K; m++) {
                tw -= bb[m] * W.v[m][e];
                tz -= bb[m] * Z.v[m][e];
            }
            w[e] = tw;
            z[e] = tz;
        }
    }
}

// with ww = dots[2p], rw = dots[2p+1]: (w, z) scaled to unit norm,
// c += (rw / ww) z, r -= (rw / ww) w, max |r| per problem -> norm_slots
__global__ void __launch_bounds__(256) k_batch_gcr_step(const BProb* __restrict__ probs,
                                                        const BTile* __restrict__ tiles, int ntiles,
                                                        const int* __restrict__ active,
                                                        const double* __restrict__ dots, float* __restrict__ w,
                                                        float* __restrict__ z, float* __restrict__ c,
                                                        float* __restrict__ r, void* norm_slots)
{
    float nrm = 0;
    int cur = -1;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        if (tl.prob < 0) break;
        if (active && !active[tl.prob]) continue;
        if (tl.prob != cur) {
            if (cur >= 0) tile_max<float>(nrm, norm_slots, cur);
            nrm = 0;
            cur = tl.prob;
        }
        const BProb& P = probs[tl.prob];
        int i, j, k;
        if (!tile_node<32, 4, 2>(tl, P.L, i, j, k)) continue;
        const double ww = dots[2 * tl.prob], rw = dots[2 * tl.prob + 1];
        const float inv = ww > 0 ? (float)(1.0 / sqrt(ww)) : 0.0f;
        const float a = ww > 0 ? (float)(rw / sqrt(ww)) : 0.0f;
        const long long q = P.vo + P.L.idx(i, j, k);
        for (int cc = 0; cc < 3; cc++) {
            const long long e = q + cc * P.L.S;
            const float wu = w[e] * inv, zu = z[e] * inv;
            w[e] = wu;
            z[e] = zu;
            c[e] += a * zu;
            const float rn = r[e] - a * wu;
            r[e] = rn;
            const float v = fabsf(rn);
            nrm = (v > nrm || v != v) ? v : nrm;
        }
    }
    if (cur >= 0) tile_max<float>(nrm, norm_slots, cur);
}

void launch_batch_multidot(cudaStream_t st, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                           const int* active, int k, const float* x, const GcrVecs& V, const float* d, double* out,
                           int stride)
{
    switch (k) {
#define K_(K)                                                                                                 \
    case K:                                                                                                   \
        k_batch_multidot<K><<<fit_grid((const void*)k_batch_multidot<K>, grid, st), 256, 0, st>>>(            \
            probs, tiles, ntiles, active, x, V, d, out, stride);                                              \
        break;
        K_(1) K_(2) K_(3) K_(4) K_(5) K_(6) K_(7) K_(8) K_(9) K_(10) K_(11) K_(12) K_(13) K_(14) K_(15) K_(16)
#undef K_
    default: return;
    }
    count_launch();
}

void launch_batch_gcr_orth(cudaStream_t st, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                           const int* active, int k, const double* beta, int stride, const GcrVecs& W,
                           const GcrVecs& Z, float* w, float* z)
{
    switch (k) {
#define K_(K)                                                                                                 \
    case K:                                                                                                   \
        k_batch_gcr_orth<K><<<fit_grid((const void*)k_batch_gcr_orth<K>, grid, st), 256, 0, st>>>(            \
            probs, tiles, ntiles, active, beta, stride, W, Z, w, z);                                          \
        break;
        K_(1) K_(2) K_(3) K_(4) K_(5) K_(6) K_(7) K_(8) K_(9) K_(10) K_(11) K_(12) K_(13) K_(14) K_(15) K_(16)
#undef K_
    default: return;
    }
    count_launch();
}

void launch_batch_gcr_step(cudaStream_t st, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                           const int* active, const double* dots, float* w, float* z, float* c, float* r,
                           void* norm_slots)
{
    grid = fit_grid((const void*)k_batch_gcr_step, grid, st);
    k_batch_gcr_step<<<grid, 256, 0, st>>>(probs, tiles, ntiles, active, dots, w, z, c, r, norm_slots);
    count_launch();
}

void launch_batch_bottom(cudaStream_t st, int sym, int fp32, const BProb* probs, const int* plist, int np,
                         const int* active, const BCTable& bc, bool uniform, const void* ddw, const double* diag,
                         void* cor, const void* res, double* work, int maxiter, double tol_rel, double tol_abs, int nub,
                         int nuf, double omega)
{
    if (np <= 0) return;
#define B_(T, S)                                                                                                     \
    k_batch_bottom<T, S><<<np, BB_THREADS, 0, st>>>(probs, plist, active, bc, uniform ? 1 : 0, (const T*)ddw, diag,  \
                                                    (T*)cor,                                                           \
                                                    (const T*)res, work, maxiter, tol_rel, tol_abs, nub, nuf, omega)
    if (fp32) {
        if (sym == SYM_ISO) B_(float, SYM_ISO);
        else B_(float, SYM_MM);
    } else {
        if (sym == SYM_ISO) B_(double, SYM_ISO);
        else B_(double, SYM_MM);
    }
#undef B_
    count_launch();
}

void launch_batch_rhs(cudaStream_t st, int sym, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                      const double* ddw, const double* F0, double* rhs)
{
    if (sym == SYM_ISO) k_batch_rhs<SYM_ISO><<<grid, 256, 0, st>>>(probs, tiles, ntiles, ddw, F0, rhs);
    else k_batch_rhs<SYM_MM><<<grid, 256, 0, st>>>(probs, tiles, ntiles, ddw, F0, rhs);
    count_launch();
}

void launch_batch_mean_stress(cudaStream_t st, int sym, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                              const double* ddw, const double* F0, const double* u, double* sums)
{
    if (sym == SYM_ISO) k_batch_mean_stress<SYM_ISO><<<grid, 256, 0, st>>>(probs, tiles, ntiles, ddw, F0, u, sums);
    else k_batch_mean_stress<SYM_MM><<<grid, 256, 0, st>>>(probs, tiles, ntiles, ddw, F0, u, sums);
    count_launch();
}

template void launch_batch_stencil<double>(cudaStream_t, int, int, int, int, const BProb*, const BTile*, int,
                                           const int*, const BCTable&, bool, const double*, const double*,
                                           const double*, const double*, double*, double, void*);
template void launch_batch_stencil<float>(cudaStream_t, int, int, int, int, const BProb*, const BTile*, int,
                                          const int*, const BCTable&, bool, const float*, const float*, const float*,
                                          const float*, float*, float, void*);
template void launch_batch_transfer<double>(cudaStream_t, int, bool, int, const BProb*, const BProb*, const BTile*,
                                            int, const int*, const double*, double*);
template void launch_batch_transfer<float>(cudaStream_t, int, bool, int, const BProb*, const BProb*, const BTile*, int,
                                           const int*, const float*, float*);

}  // namespace agb
