// kernels_tail.cu -- the coarsest levels of an FP32 cycle in one CTA.
//
// Below a few thousand nodes a level's kernels are latency-bound: every
// Jacobi sweep, residual and transfer of a 9^3- or 5^3-node level costs a
// launch of ~8 us for microseconds of work, and a 257^3 F-cycle visits those
// levels about a hundred and fifty times.  Here the tail of the hierarchy
// (levels t .. bottom, at most TAIL_MAX_LEVELS) runs inside one CTA: the
// moduli, 1/D and the cycle vectors of those levels are loaded into shared
// memory (compact node order i + nn0 (j + nn1 k), periodic images folded like
// the global kernels), the cycle's steps run there separated by barriers, and
// only the correction of level t goes back to global memory.
//
// The steps are those of the host cycle engine (MLMG::mgVcycle /
// mgFcycle restricted to levels t .. bottom): the same per-node rows
// (stencil.cuh), Jacobi update x + omega ((b - A x) / D), first sweep from a
// zero guess omega (b / D), nodal full-weighting restriction and trilinear
// prolongation (transfer.cuh), and the bottom solved by the dense inverse
// (cor = A^-1 res) or, where that inverse does not exist, by the dense
// BiCGStab of the bottom kernel on the level's global arrays.
#include <cuda_runtime.h>

#include <cstdlib>

#include "agb_internal.h"
#include "bottom.cuh"
#include "stencil.cuh"
#include "transfer.cuh"

namespace agb {

namespace {

constexpr int TAIL_THREADS = 512;

struct TailLevel {
    LevelDesc L;       // the level's global (padded) layout
    Geo<float> g;
    int cnt;           // stored nodes
    int c, d;          // shared-memory offsets (floats): moduli (nc x cnt), 1/D (3 x cnt)
    int cor, res, tmp, rsc, hold;   // vectors (3 x cnt each)
    const float* ddw;  // global moduli and 1/D of the level
    const float* dinv;
};

struct TailArgs {
    TailLevel lv[TAIL_MAX_LEVELS];
    int nlev;          // levels t .. t + nlev - 1 (the last is the bottom)
    int nc;            // modulus planes
    int uniform;
    float omega;
    int pre, post;     // Fsmooth calls (2 Jacobi sweeps each)
    BCTable bc;
    float* res_t;      // global residual of level t (input)
    float* cor_t;      // global correction of level t (output)
    // bottom: exact inverse, or the BiCGStab fallback on the level's global arrays
    const float* inv;
    const int* inv_ok;
    const double* A;   // dense bottom operator (FP64)
    const double* diag64;
    float* bres;       // global res / cor of the bottom level (fallback only)
    float* bcor;
    int maxiter, nub, nuf;
    double tol_rel, tol_abs, omega_d;
    int* ret_slot;
};

// Compact index of node (i, j, k) and its neighbour offsets (periodic images folded).
struct CNbr {
    int base;
    int o[3][3];
};

__device__ __forceinline__ CNbr cnbr(const LevelDesc& L, int i, int j, int k)
{
    CNbr nb;
    const int st[3] = {1, L.nn[0], L.nn[0] * L.nn[1]};
    const int pos[3] = {i, j, k};
    nb.base = i + st[1] * j + st[2] * k;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        nb.o[d][0] = -st[d];
        nb.o[d][1] = 0;
        nb.o[d][2] = st[d];
        if (L.per[d]) {
            if (pos[d] == 0) nb.o[d][0] = st[d] * (L.n[d] - 1);
            if (pos[d] == L.n[d] - 1) nb.o[d][2] = -st[d] * (L.n[d] - 1);
        }
    }
    return nb;
}

struct SmemAccT {
    const float* x;   // 3 x cnt
    const float* c;   // nc x cnt
    int cnt;
    CNbr nb;
    __device__ __forceinline__ int off(int di, int dj, int dk) const
    {
        return nb.base + nb.o[0][di + 1] + nb.o[1][dj + 1] + nb.o[2][dk + 1];
    }
    __device__ __forceinline__ float u(int p, int di, int dj, int dk) const { return x[p * cnt + off(di, dj, dk)]; }
    __device__ __forceinline__ float C(int m, int di, int dj, int dk) const { return c[m * cnt + off(di, dj, dk)]; }
};

__device__ __forceinline__ void node_of(const TailLevel& v, int e, int& i, int& j, int& k)
{
    i = e % v.L.nn[0];
    j = (e / v.L.nn[0]) % v.L.nn[1];
    k = e / (v.L.nn[0] * v.L.nn[1]);
}

// out = x + omega ((b - A x) / D) (MODE_JACOBI) or b - A x (MODE_RESID) on every node of the level.
template <int SYM, int MODE>
__device__ void tail_sweep(const TailArgs& a, const TailLevel& v, float* sm, int x, int b, int out)
{
    for (int e = threadIdx.x; e < v.cnt; e += blockDim.x) {
        int i, j, k;
        node_of(v, e, i, j, k);
        const int pos[3] = {i, j, k};
        int mn[3], mx[3];
        bool bnd = false;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            mn[d] = !v.L.per[d] && pos[d] == 0;
            mx[d] = !v.L.per[d] && pos[d] == v.L.n[d];
            bnd = bnd || mn[d] || mx[d];
        }
        SmemAccT acc{sm + x, sm + v.c, v.cnt, cnbr(v.L, i, j, k)};
        float f[3];
        if (bnd) boundary_row<float, SYM>(acc, v.g, a.bc, mn, mx, f);
        else interior_row<float, SYM>(acc, v.g, a.uniform != 0, f);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const int q = c * v.cnt + e;
            if (MODE == MODE_RESID) sm[out + q] = sm[b + q] - f[c];
            else sm[out + q] = sm[x + q] + a.omega * ((sm[b + q] - f[c]) * sm[v.d + q]);
        }
    }
    __syncthreads();
}

// Fsmooth x (ns calls of two sweeps), x = 0 first when `zero` (the first sweep
// of a zero guess is omega (b / D)).
template <int SYM>
__device__ void tail_smooth(const TailArgs& a, const TailLevel& v, float* sm, int x, int b, int ns, bool zero)
{
    if (zero) {
        if (ns <= 0) {
            for (int q = threadIdx.x; q < 3 * v.cnt; q += blockDim.x) sm[x + q] = 0.0f;
            __syncthreads();
            return;
        }
        for (int q = threadIdx.x; q < 3 * v.cnt; q += blockDim.x) sm[v.tmp + q] = a.omega * (sm[b + q] * sm[v.d + q]);
        __syncthreads();
        tail_sweep<SYM, MODE_JACOBI>(a, v, sm, v.tmp, b, x);
        ns -= 1;
    }
    for (int s = 0; s < ns; s++) {
        tail_sweep<SYM, MODE_JACOBI>(a, v, sm, x, b, v.tmp);
        tail_sweep<SYM, MODE_JACOBI>(a, v, sm, v.tmp, b, x);
    }
}

// crse(res of level vc) = R fine(vector `src` of level vf)
__device__ void tail_restrict(const TailLevel& vf, const TailLevel& vc, float* sm, int src, int dst)
{
    const LevelDesc &Lf = vf.L, &Lc = vc.L;
    for (int e = threadIdx.x; e < vc.cnt; e += blockDim.x) {
        int I, J, K;
        node_of(vc, e, I, J, K);
        const bool bI = !Lc.per[0] && (I == 0 || I == Lc.n[0]);
        const bool bJ = !Lc.per[1] && (J == 0 || J == Lc.n[1]);
        const bool bK = !Lc.per[2] && (K == 0 || K == Lc.n[2]);
        for (int c = 0; c < 3; c++) {
            const float* s = sm + src + c * vf.cnt;
            auto f = [&](int a, int b, int d) -> float {
                const int i = wrapn(2 * I + a, Lf.n[0], Lf.per[0]), j = wrapn(2 * J + b, Lf.n[1], Lf.per[1]),
                          k = wrapn(2 * K + d, Lf.n[2], Lf.per[2]);
                return s[i + Lf.nn[0] * (j + Lf.nn[1] * k)];
            };
            sm[dst + c * vc.cnt + e] = full_weight<float>(f, bI, bJ, bK);
        }
    }
    __syncthreads();
}

// fine(vector `dst` of level vf) (+)= P crse(vector `src` of level vc)
__device__ void tail_interp(const TailLevel& vf, const TailLevel& vc, float* sm, int src, int dst, bool assign)
{
    const LevelDesc &Lf = vf.L, &Lc = vc.L;
    for (int e = threadIdx.x; e < vf.cnt; e += blockDim.x) {
        int i, j, k;
        node_of(vf, e, i, j, k);
        const int I = i >> 1, J = j >> 1, K = k >> 1;
        const int I1 = wrapn(I + 1, Lc.n[0], Lc.per[0]), J1 = wrapn(J + 1, Lc.n[1], Lc.per[1]),
                  K1 = wrapn(K + 1, Lc.n[2], Lc.per[2]);
        for (int c = 0; c < 3; c++) {
            const float* s = sm + src + c * vc.cnt;
            auto C = [&](int a, int b, int d) -> float {
                return s[(a ? I1 : I) + Lc.nn[0] * ((b ? J1 : J) + Lc.nn[1] * (d ? K1 : K))];
            };
            const float t = interp_node<float>(C, !(i & 1), !(j & 1), !(k & 1));
            const int q = dst + c * vf.cnt + e;
            sm[q] = assign ? t : sm[q] + t;
        }
    }
    __syncthreads();
}

// cor = A^-1 res on the bottom level (two interleaved partial sums, as
// k_bottom_dense), or the dense BiCGStab on its global arrays.
__device__ void tail_bottom(const TailArgs& a, const TailLevel& v, float* sm, float* red_f, float* dense)
{
    const int nu = 3 * v.cnt;
    if (*a.inv_ok) {
        const float* xs = sm + v.res;   // compact order = the dense unknown order c * cnt + e
        for (int q = threadIdx.x; q < nu; q += blockDim.x) {
            float y0 = 0.0f, y1 = 0.0f;
            int j = 0;
            for (; j + 1 < nu; j += 2) {
                y0 = fmaf(a.inv[(long long)j * nu + q], xs[j], y0);
                y1 = fmaf(a.inv[(long long)(j + 1) * nu + q], xs[j + 1], y1);
            }
            if (j < nu) y0 = fmaf(a.inv[(long long)j * nu + q], xs[j], y0);
            sm[v.cor + q] = y0 + y1;
        }
        __syncthreads();
        return;
    }
    // fallback: res -> the level's global array, BiCGStab (one thread per unknown), cor back
    const LevelDesc& L = v.L;
    for (int q = threadIdx.x; q < nu; q += blockDim.x) {
        const int c = q / v.cnt, e = q - c * v.cnt;
        int i, j, k;
        node_of(v, e, i, j, k);
        a.bres[c * L.S + L.idx(i, j, k)] = sm[v.res + q];
    }
    __threadfence_block();
    __syncthreads();
    for (int q = threadIdx.x; q < nu * nu; q += blockDim.x) dense[q] = (float)a.A[q];
    __syncthreads();
    dense_bottom_block<float, float>(L, dense, dense + nu * nu, red_f, a.diag64, a.bcor, a.bres, a.maxiter, a.tol_rel,
                                     a.tol_abs, a.nub, a.nuf, a.omega_d, a.ret_slot);
    __threadfence_block();
    __syncthreads();
    for (int q = threadIdx.x; q < nu; q += blockDim.x) {
        const int c = q / v.cnt, e = q - c * v.cnt;
        int i, j, k;
        node_of(v, e, i, j, k);
        sm[v.cor + q] = __ldcg(a.bcor + c * L.S + L.idx(i, j, k));
    }
    __syncthreads();
}

// MLMG::mgVcycle from tail level l: right-hand side in the vector at offset
// lres of level l, correction into the vector at lcor, its residual into the
// scratch vector at lrsc (the deeper levels use their own res / cor / rsc)
template <int SYM>
__device__ void tail_vcycle(const TailArgs& a, float* sm, int l, int lres, int lcor, int lrsc, float* red_f,
                            float* dense)
{
    const int b = a.nlev - 1;
    for (int m = l; m < b; m++) {
        const TailLevel& v = a.lv[m];
        const int res = m == l ? lres : v.res, cor = m == l ? lcor : v.cor, rsc = m == l ? lrsc : v.rsc;
        tail_smooth<SYM>(a, v, sm, cor, res, a.pre, true);
        tail_sweep<SYM, MODE_RESID>(a, v, sm, cor, res, rsc);
        tail_restrict(v, a.lv[m + 1], sm, rsc, a.lv[m + 1].res);
    }
    tail_bottom(a, a.lv[b], sm, red_f, dense);
    for (int m = b - 1; m >= l; m--) {
        const TailLevel& v = a.lv[m];
        const int res = m == l ? lres : v.res, cor = m == l ? lcor : v.cor;
        tail_interp(v, a.lv[m + 1], sm, a.lv[m + 1].cor, cor, false);
        tail_smooth<SYM>(a, v, sm, cor, res, a.post, false);
    }
}

// fcycle = 0: MLMG::mgVcycle from level t.  fcycle = 1: the part of
// MLMG::mgFcycle below level t (the residual of t restricted down, the bottom
// solved, then on each level up to t: the prolonged correction, a V-cycle on
// its residual, and the sum).
template <int SYM>
__global__ void __launch_bounds__(TAIL_THREADS, 1) k_coarse_tail(TailArgs a, int fcycle)
{
    extern __shared__ __align__(16) float sm[];
    __shared__ float red_f[2 * 3 * 32];
    const int nc = a.nc;
    // load the moduli and 1/D of every tail level, and the residual of level t
    for (int m = 0; m < a.nlev; m++) {
        const TailLevel& v = a.lv[m];
        for (int q = threadIdx.x; q < v.cnt; q += blockDim.x) {
            int i, j, k;
            node_of(v, q, i, j, k);
            const long long p = v.L.idx(i, j, k);
            for (int c = 0; c < nc; c++) sm[v.c + c * v.cnt + q] = v.ddw[c * v.L.S + p];
            for (int c = 0; c < 3; c++) sm[v.d + c * v.cnt + q] = v.dinv[c * v.L.S + p];
            if (m == 0)
                for (int c = 0; c < 3; c++) sm[v.res + c * v.cnt + q] = __ldcg(a.res_t + c * v.L.S + p);
        }
    }
    __syncthreads();
    const TailLevel& vt = a.lv[0];
    // room for the dense fallback operator: after the last level's vectors
    float* dense = sm + a.lv[a.nlev - 1].hold + 3 * a.lv[a.nlev - 1].cnt;
    if (!fcycle) {
        tail_vcycle<SYM>(a, sm, 0, vt.res, vt.cor, vt.rsc, red_f, dense);
    } else {
        const int b = a.nlev - 1;
        for (int m = 0; m < b; m++) tail_restrict(a.lv[m], a.lv[m + 1], sm, a.lv[m].res, a.lv[m + 1].res);
        tail_bottom(a, a.lv[b], sm, red_f, dense);
        for (int m = b - 1; m >= 0; m--) {
            const TailLevel& v = a.lv[m];
            tail_interp(v, a.lv[m + 1], sm, a.lv[m + 1].cor, v.cor, true);
            tail_sweep<SYM, MODE_RESID>(a, v, sm, v.cor, v.res, v.rsc);
            // a V-cycle on that residual, its correction in `hold` (the
            // prolonged correction stays in `cor`; the level's own residual
            // is no longer needed and takes the V-cycle's), then cor += hold
            tail_vcycle<SYM>(a, sm, m, v.rsc, v.hold, v.res, red_f, dense);
            for (int q = threadIdx.x; q < 3 * v.cnt; q += blockDim.x) sm[v.cor + q] = sm[v.cor + q] + sm[v.hold + q];
            __syncthreads();
        }
    }
    // the correction of level t back to global memory
    for (int q = threadIdx.x; q < vt.cnt; q += blockDim.x) {
        int i, j, k;
        node_of(vt, q, i, j, k);
        const long long p = vt.L.idx(i, j, k);
        for (int c = 0; c < 3; c++) a.cor_t[c * vt.L.S + p] = sm[vt.cor + c * vt.cnt + q];
    }
}

}  // namespace

// Shared-memory floats the tail from level t needs (levels t .. bottom), or 0
// when it does not fit (more than TAIL_MAX_LEVELS levels, or above the limit).
size_t coarse_tail_floats(const LevelDesc* lv, int nlev, int t, int nc)
{
    const int nl = nlev - t;
    if (t < 1 || nl < 2 || nl > TAIL_MAX_LEVELS) return 0;
    size_t f = 0;
    for (int m = t; m < nlev; m++) f += (size_t)(nc + 3 + 5 * 3) * lv[m].count();
    const size_t nu = 3 * (size_t)lv[nlev - 1].count();
    if (nu > (size_t)DENSE_MAX) return 0;
    f += nu * nu + nu;   // dense fallback operator and its vector
    return f * sizeof(float) <= TAIL_SMEM_MAX ? f : 0;
}

bool launch_coarse_tail(cudaStream_t st, int sym, const TailSpec& s, int fcycle)
{
    TailArgs a;
    const int nl = s.nlev;
    if (nl < 2 || nl > TAIL_MAX_LEVELS) return false;
    a.nlev = nl;
    a.nc = sym == SYM_ISO ? 2 : 21;
    int off = 0;
    for (int m = 0; m < nl; m++) {
        TailLevel& v = a.lv[m];
        v.L = s.levels[m];
        v.g = make_geo<float>(v.L);
        v.cnt = (int)v.L.count();
        v.ddw = s.ddw[m];
        v.dinv = s.dinv[m];
        v.c = off; off += a.nc * v.cnt;
        v.d = off; off += 3 * v.cnt;
        v.cor = off; off += 3 * v.cnt;
        v.res = off; off += 3 * v.cnt;
        v.tmp = off; off += 3 * v.cnt;
        v.rsc = off; off += 3 * v.cnt;
        v.hold = off; off += 3 * v.cnt;
    }
    const int nu = 3 * a.lv[nl - 1].cnt;
    const size_t smem = ((size_t)off + (size_t)nu * nu + nu) * sizeof(float);
    if (smem > TAIL_SMEM_MAX) return false;
    a.uniform = s.uniform;
    a.omega = s.omega;
    a.pre = s.pre;
    a.post = s.post;
    a.bc = s.bc;
    a.res_t = s.res_t;
    a.cor_t = s.cor_t;
    a.inv = s.inv;
    a.inv_ok = s.inv_ok;
    a.A = s.A;
    a.diag64 = s.diag64;
    a.bres = s.bres;
    a.bcor = s.bcor;
    a.maxiter = s.maxiter;
    a.nub = s.nub;
    a.nuf = s.nuf;
    a.tol_rel = s.tol_rel;
    a.tol_abs = s.tol_abs;
    a.omega_d = s.omega;
    a.ret_slot = s.ret_slot;
    if (sym == SYM_ISO) k_coarse_tail<SYM_ISO><<<1, TAIL_THREADS, smem, st>>>(a, fcycle);
    else k_coarse_tail<SYM_MM><<<1, TAIL_THREADS, smem, st>>>(a, fcycle);
    count_launch();
    return true;
}

// The coarse tail serves the FP32 cycles when AGB_TAIL=1 (read when an
// operator is created).  Off by default: on GB300 the 257^3 mixed solve took
// 0.340 s with it against 0.337 s without (20949 against 33801 launches):
// captured in a graph, the small levels' launches cost about a microsecond
// each, and one CTA sweeping the 9^3-node level (half of its nodes boundary
// rows, so warps run both row forms) is no faster than the grid of launches.
bool use_coarse_tail()
{
    const char* s = getenv("AGB_TAIL");
    return s && s[0] == '1';
}

void init_tail_attributes()
{
    cudaFuncSetAttribute(k_coarse_tail<SYM_ISO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TAIL_SMEM_MAX);
    cudaFuncSetAttribute(k_coarse_tail<SYM_MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TAIL_SMEM_MAX);
}

}  // namespace agb
