// kernels_bottom.cu -- coarsest-level solve in one CTA, FP64.
//
// Restates AMReX MLMG's bottom step as Alamo configures it
// (Solver/Nonlocal/Linear.H:258 selects BiCGStab):
//   cor = 0; BiCGStab on the diagonally scaled system (MLCGSolver::solve_bicgstab
//   with Operator<Node>::normalize = divide by the diagonal, Operator.cpp:156-165);
//   a failed solve (anything but a clean convergence) zeroes the correction;
//   then `bottom_smooth` (after success) or `final_smooth` (after failure)
//   Fsmooth calls of 2 damped-Jacobi sweeps each.
// On a fully periodic box (singular: rigid translations) the Krylov residual
// and every operator application are projected to zero mean per component
// before the diagonal scaling, so that BiCGStab works on a consistent system;
// the smoothing uses the right-hand side as given.
// Every loop is bounded by maxiter / the smoothing counts; there is no
// spin-wait.  The return code lands in ret_slot: 0 converged, 1-4 breakdown,
// 8 not converged in maxiter.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>


#include "agb_internal.h"
#include "stencil.cuh"
#include "bottom.cuh"

namespace agb {

constexpr int BOT_THREADS = 512;

__device__ __forceinline__ double blk_sum(double v, double* red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (BOT_THREADS / 32) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) red[32] = t;
    }
    __syncthreads();
    return red[32];
}

__device__ __forceinline__ double blk_max(double v, double* red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        double w = __shfl_xor_sync(0xffffffffu, v, o);
        v = (w > v || w != w) ? w : v;
    }
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < (BOT_THREADS / 32) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            double w = __shfl_xor_sync(0xffffffffu, t, o);
            t = (w > t || w != w) ? w : t;
        }
        if (threadIdx.x == 0) red[32] = t;
    }
    __syncthreads();
    return red[32];
}

struct BotAcc {
    const double* x;
    const double* c;
    long long S;
    long long base;
    long long o[3][3];
    __device__ __forceinline__ long long off(int di, int dj, int dk) const
    {
        return base + o[0][di + 1] + o[1][dj + 1] + o[2][dk + 1];
    }
    __device__ __forceinline__ double u(int p, int di, int dj, int dk) const { return x[p * S + off(di, dj, dk)]; }
    __device__ __forceinline__ double C(int m, int di, int dj, int dk) const { return c[m * S + off(di, dj, dk)]; }
};

// y = A x over all nodes of the level (threads stride over nodes)
template <int SYM>
__device__ void cta_apply(const LevelDesc& L, const BCTable& bc, const Geo<double>& g, int uniform,
                          const double* ddw, const double* x, double* y)
{
    const long long cnt = L.count();
    const long long st[3] = {1, (long long)L.P, (long long)L.P * L.nn[1]};
    for (long long e = threadIdx.x; e < cnt; e += blockDim.x) {
        const int i = (int)(e % L.nn[0]);
        const int j = (int)((e / L.nn[0]) % L.nn[1]);
        const int k = (int)(e / ((long long)L.nn[0] * L.nn[1]));
        const int pos[3] = {i, j, k};
        BotAcc acc;
        acc.x = x;
        acc.c = ddw;
        acc.S = L.S;
        acc.base = L.idx(i, j, k);
        int mn[3], mx[3];
        bool bnd = false;
        for (int d = 0; d < 3; d++) {
            mn[d] = !L.per[d] && pos[d] == 0;
            mx[d] = !L.per[d] && pos[d] == L.n[d];
            bnd = bnd || mn[d] || mx[d];
            acc.o[d][0] = -st[d];
            acc.o[d][1] = 0;
            acc.o[d][2] = st[d];
            if (L.per[d]) {
                if (pos[d] == 0) acc.o[d][0] = st[d] * (L.n[d] - 1);
                if (pos[d] == L.n[d] - 1) acc.o[d][2] = -st[d] * (L.n[d] - 1);
            }
        }
        double f[3];
        if (bnd) boundary_row<double, SYM>(acc, g, bc, mn, mx, f);
        else interior_row<double, SYM>(acc, g, uniform != 0, f);
        for (int c = 0; c < 3; c++) y[c * L.S + acc.base] = f[c];
    }
}

// per-component means over the level's nodes (every stored node is unique on
// a fully periodic level)
__device__ void cta_mean3(const LevelDesc& L, const double* v, double* red, double m[3])
{
    const long long cnt = L.count();
    double s0 = 0, s1 = 0, s2 = 0;
    for (long long e = threadIdx.x; e < cnt; e += blockDim.x) {
        const long long q = L.idx((int)(e % L.nn[0]), (int)((e / L.nn[0]) % L.nn[1]),
                                  (int)(e / ((long long)L.nn[0] * L.nn[1])));
        s0 += v[q];
        s1 += v[L.S + q];
        s2 += v[2 * L.S + q];
    }
    m[0] = blk_sum(s0, red) / (double)cnt;
    m[1] = blk_sum(s1, red) / (double)cnt;
    m[2] = blk_sum(s2, red) / (double)cnt;
}

#define FOR_NODES(q)                                                                                     \
    for (long long e_ = threadIdx.x; e_ < cnt; e_ += blockDim.x)                                         \
        for (int c_ = 0, i_ = (int)(e_ % L.nn[0]), j_ = (int)((e_ / L.nn[0]) % L.nn[1]),                  \
                 k_ = (int)(e_ / ((long long)L.nn[0] * L.nn[1]));                                        \
             c_ < 3; c_++)                                                                               \
            for (long long q = c_ * L.S + L.idx(i_, j_, k_), once_ = 0; once_ < 1; once_++)

template <typename T, int SYM>
__global__ void __launch_bounds__(BOT_THREADS) k_bottom(LevelDesc L, BCTable bc, Geo<double> g, int uniform,
                                                        const double* __restrict__ ddw,
                                                        const double* __restrict__ diag, T* __restrict__ cor,
                                                        const T* __restrict__ res, double* __restrict__ work,
                                                        int maxiter, double eps_rel, double eps_abs, int nub,
                                                        int nuf, double omega, int* ret_slot)
{
    __shared__ double red[33];
    const long long n3 = 3 * L.S, cnt = L.count();
    double *r = work, *rh = work + n3, *p = work + 2 * n3, *v = work + 3 * n3, *s = work + 4 * n3,
           *t = work + 5 * n3, *sol = work + 6 * n3, *b = work + 7 * n3;
    FOR_NODES(q)
    {
        b[q] = (double)res[q];
        sol[q] = 0.0;
    }
    __syncthreads();
    const bool sing = L.singular();
    double mb[3] = {0, 0, 0};
    if (sing) cta_mean3(L, b, red, mb);
    // r = P(b - A*0)/D, P the zero-mean projection on a singular level (identity otherwise)
    double lm = 0;
    FOR_NODES(q)
    {
        r[q] = (b[q] - mb[c_]) / diag[q];
        rh[q] = r[q];
        const double a = fabs(r[q]);
        lm = (a > lm || a != a) ? a : lm;
    }
    double rnorm = blk_max(lm, red);
    const double rnorm0 = rnorm;
    int ret = 0;
    double rho_1 = 0, alpha = 0, om = 0;
    if (!(rnorm0 == 0 || rnorm0 < eps_abs)) {
        for (int iter = 1; iter <= maxiter; iter++) {
            double acc = 0;
            FOR_NODES(q) acc += rh[q] * r[q];
            const double rho = blk_sum(acc, red);
            if (rho == 0) { ret = 1; break; }
            if (iter == 1) {
                FOR_NODES(q) p[q] = r[q];
            } else {
                const double beta = (rho / rho_1) * (alpha / om);
                FOR_NODES(q) p[q] = r[q] + beta * (p[q] - om * v[q]);
            }
            __syncthreads();
            cta_apply<SYM>(L, bc, g, uniform, ddw, p, v);
            __syncthreads();
            double mv[3] = {0, 0, 0};
            if (sing) cta_mean3(L, v, red, mv);
            acc = 0;
            FOR_NODES(q)
            {
                v[q] = (v[q] - mv[c_]) / diag[q];
                acc += rh[q] * v[q];
            }
            const double rhTv = blk_sum(acc, red);
            if (rhTv != 0) alpha = rho / rhTv;
            else { ret = 2; break; }
            lm = 0;
            FOR_NODES(q)
            {
                sol[q] += alpha * p[q];
                s[q] = r[q] - alpha * v[q];
                const double a = fabs(s[q]);
                lm = (a > lm || a != a) ? a : lm;
            }
            rnorm = blk_max(lm, red);
            if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
            cta_apply<SYM>(L, bc, g, uniform, ddw, s, t);
            __syncthreads();
            double mt[3] = {0, 0, 0};
            if (sing) cta_mean3(L, t, red, mt);
            double tt = 0, ts = 0;
            FOR_NODES(q)
            {
                t[q] = (t[q] - mt[c_]) / diag[q];
                tt += t[q] * t[q];
                ts += t[q] * s[q];
            }
            tt = blk_sum(tt, red);
            ts = blk_sum(ts, red);
            if (tt != 0) om = ts / tt;
            else { ret = 3; break; }
            lm = 0;
            FOR_NODES(q)
            {
                sol[q] += om * s[q];
                r[q] = s[q] - om * t[q];
                const double a = fabs(r[q]);
                lm = (a > lm || a != a) ? a : lm;
            }
            rnorm = blk_max(lm, red);
            if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
            if (om == 0) { ret = 4; break; }
            rho_1 = rho;
        }
        if (ret == 0 && rnorm > eps_rel * rnorm0 && rnorm > eps_abs) ret = 8;
        if (!((ret == 0 || ret == 8) && rnorm < rnorm0)) {
            FOR_NODES(q) sol[q] = 0.0;
        }
        // MLMG::actualBottomSolve: anything but a clean solve discards the correction
        if (ret != 0) {
            FOR_NODES(q) sol[q] = 0.0;
        }
    }
    __syncthreads();
    // post-smoothing: Fsmooth = 2 Jacobi sweeps each
    const int nsm = 2 * ((ret == 0) ? nub : nuf);
    for (int sw = 0; sw < nsm; sw++) {
        cta_apply<SYM>(L, bc, g, uniform, ddw, sol, t);
        __syncthreads();
        FOR_NODES(q)
        {
            const double Rx = t[q] - sol[q] * diag[q];
            s[q] = (1. - omega) * sol[q] + omega * (b[q] - Rx) / diag[q];
        }
        __syncthreads();
        FOR_NODES(q) sol[q] = s[q];
        __syncthreads();
    }
    FOR_NODES(q) cor[q] = (T)sol[q];
    if (threadIdx.x == 0 && ret_slot) *ret_slot = ret;
}

// Neighbour offsets of node (i,j,k) in the padded layout, periodic wrap included.
struct UnitAcc {
    const double* c;
    long long S, base, unit;   // unit: padded node index of the unit vector's node
    int comp;                  // and its component
    long long o[3][3];
    __device__ __forceinline__ long long off(int di, int dj, int dk) const
    {
        return base + o[0][di + 1] + o[1][dj + 1] + o[2][dk + 1];
    }
    __device__ __forceinline__ double u(int p, int di, int dj, int dk) const
    {
        return (p == comp && off(di, dj, dk) == unit) ? 1.0 : 0.0;
    }
    __device__ __forceinline__ double C(int m, int di, int dj, int dk) const { return c[m * S + off(di, dj, dk)]; }
};

// A (column-major, entry (row r, column j) at j * nu + r) of the level:
// one thread per (row node, column unknown), rows of its three components.
template <int SYM>
__global__ void k_bottom_assemble(LevelDesc L, BCTable bc, Geo<double> g, int uniform,
                                  const double* __restrict__ ddw, double* __restrict__ A)
{
    const int cnt = (int)L.count(), nu = 3 * cnt;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt * nu) return;
    const int e = t % cnt, col = t / cnt;
    const int i = e % L.nn[0], j = (e / L.nn[0]) % L.nn[1], k = e / (L.nn[0] * L.nn[1]);
    const int ce = col % cnt;
    UnitAcc acc;
    acc.c = ddw;
    acc.S = L.S;
    acc.base = L.idx(i, j, k);
    acc.comp = col / cnt;
    acc.unit = L.idx(ce % L.nn[0], (ce / L.nn[0]) % L.nn[1], ce / (L.nn[0] * L.nn[1]));
    const long long st[3] = {1, (long long)L.P, (long long)L.P * L.nn[1]};
    const int pos[3] = {i, j, k};
    int mn[3], mx[3];
    bool bnd = false;
    for (int d = 0; d < 3; d++) {
        mn[d] = !L.per[d] && pos[d] == 0;
        mx[d] = !L.per[d] && pos[d] == L.n[d];
        bnd = bnd || mn[d] || mx[d];
        acc.o[d][0] = -st[d];
        acc.o[d][1] = 0;
        acc.o[d][2] = st[d];
        if (L.per[d]) {
            if (pos[d] == 0) acc.o[d][0] = st[d] * (L.n[d] - 1);
            if (pos[d] == L.n[d] - 1) acc.o[d][2] = -st[d] * (L.n[d] - 1);
        }
    }
    double f[3];
    if (bnd) boundary_row<double, SYM>(acc, g, bc, mn, mx, f);
    else interior_row<double, SYM>(acc, g, uniform != 0, f);
    for (int c = 0; c < 3; c++) A[(long long)col * nu + c * cnt + e] = f[c];
}

// The CTA copies the operator (FP64, column-major) into shared memory in R.
template <typename R> __device__ __forceinline__ void dense_load(R* A, const double* __restrict__ Ag, int nu)
{
    for (int q = threadIdx.x; q < nu * nu; q += blockDim.x) A[q] = (R)Ag[q];
}

// With `inv` set and *inv_ok (an exact inverse exists, k_bottom_invert), the
// bottom is the product cor = A^-1 res instead of the BiCGStab solve.
template <typename T, typename R>
__global__ void __launch_bounds__(DENSE_MAX) k_bottom_dense(LevelDesc L, const double* __restrict__ Ag,
                                                            const double* __restrict__ diag, T* __restrict__ cor,
                                                            const T* __restrict__ res, int maxiter, double eps_rel_d,
                                                            double eps_abs_d, int nub, int nuf, double omega_d,
                                                            int* ret_slot, const float* __restrict__ inv,
                                                            const int* __restrict__ inv_ok)
{
    pdl_entry();
    extern __shared__ __align__(16) unsigned char dsm_raw[];
    __shared__ R red[2 * 3 * 32];
    const int cnt = (int)L.count(), nu = 3 * cnt;
    if (inv && *inv_ok) {
        float* xs = reinterpret_cast<float*>(dsm_raw);
        const int q = threadIdx.x;
        const long long pq = q < nu ? dense_to_padded(L, q, cnt) : 0;
        if (q < nu) xs[q] = (float)__ldcg(res + pq);
        __syncthreads();
        if (q < nu) {
            float y0 = 0.0f, y1 = 0.0f;
            int j = 0;
            for (; j + 1 < nu; j += 2) {
                y0 = fmaf(inv[(long long)j * nu + q], xs[j], y0);
                y1 = fmaf(inv[(long long)(j + 1) * nu + q], xs[j + 1], y1);
            }
            if (j < nu) y0 = fmaf(inv[(long long)j * nu + q], xs[j], y0);
            cor[pq] = (T)(y0 + y1);
        }
        if (threadIdx.x == 0 && ret_slot) *ret_slot = 0;
        return;
    }
    R* A = reinterpret_cast<R*>(dsm_raw);
    dense_load<R>(A, Ag, nu);
    __syncthreads();
    dense_bottom_block<T, R>(L, A, A + nu * nu, red, diag, cor, res, maxiter, eps_rel_d, eps_abs_d, nub, nuf, omega_d,
                             ret_slot);
}

bool bottom_dense_fits(const LevelDesc& L) { return 3 * L.count() <= DENSE_MAX; }

// ---------------------------------------------------------------------------
// Exact coarsest solve for the FP32 cycles of the mixed solve.  Once per solve
// the dense operator (FP64, column-major) is inverted by Gauss-Jordan
// elimination with partial pivoting in one CTA, the matrix in shared memory
// (row-major), and stored in FP32 column-major (inv[j * nu + r] = A^-1(r, j))
// so that thread r of the product reads a coalesced column per j.  A fully
// periodic level (singular), or a pivot at or below 1e-13 of the largest
// |entry|, clears *ok and the cycles keep the BiCGStab bottom.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_bottom_invert(LevelDesc L, const double* __restrict__ Ag,
                                                       float* __restrict__ inv, int* __restrict__ ok)
{
    extern __shared__ __align__(16) unsigned char inv_raw[];
    double* M = reinterpret_cast<double*>(inv_raw);   // nu x nu, row-major
    __shared__ double fcol[DENSE_MAX];
    __shared__ int piv[DENSE_MAX];
    __shared__ double amax_s, pinv_s;
    __shared__ int bad_s;
    const int nu = 3 * (int)L.count();
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
    if (L.singular() || nu > DENSE_MAX) {
        if (tid == 0) *ok = 0;
        return;
    }
    double a = 0.0;
    for (int t = tid; t < nu * nu; t += nt) {
        const double v = Ag[t];
        M[(t % nu) * nu + t / nu] = v;
        a = fmax(a, fabs(v));
    }
    // block max of |A| (every warp's lane 0 folds into amax_s)
    for (int o = 16; o > 0; o >>= 1) a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
    if (tid == 0) {
        amax_s = 0.0;
        bad_s = 0;
    }
    __syncthreads();
    if (lane == 0) atomicMax(reinterpret_cast<unsigned long long*>(&amax_s), (unsigned long long)__double_as_longlong(a));
    __syncthreads();
    const double tol = 1e-13 * amax_s;
    for (int k = 0; k < nu; k++) {
        if (tid < 32) {
            // pivot: the largest |M(r, k)| for r >= k (ties to the lower row)
            double best = -1.0;
            int br = k;
            for (int r = k + lane; r < nu; r += 32) {
                const double v = fabs(M[r * nu + k]);
                if (v > best) {
                    best = v;
                    br = r;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int orow = __shfl_xor_sync(0xffffffffu, br, o);
                if (ob > best || (ob == best && orow < br)) {
                    best = ob;
                    br = orow;
                }
            }
            if (lane == 0) {
                piv[k] = br;
                if (!(best > tol)) bad_s = 1;
            }
        }
        __syncthreads();
        if (bad_s) break;   // uniform: every thread reads it after the barrier
        const int pr = piv[k];
        if (pr != k)
            for (int c = tid; c < nu; c += nt) {
                const double t = M[k * nu + c];
                M[k * nu + c] = M[pr * nu + c];
                M[pr * nu + c] = t;
            }
        __syncthreads();
        if (tid == 0) pinv_s = 1.0 / M[k * nu + k];
        __syncthreads();
        const double pinv = pinv_s;
        for (int c = tid; c < nu; c += nt) M[k * nu + c] = (c == k ? 1.0 : M[k * nu + c]) * pinv;
        for (int r = tid; r < nu; r += nt) fcol[r] = r == k ? 0.0 : M[r * nu + k];
        __syncthreads();
        for (int t = tid; t < nu * nu; t += nt) {
            const int r = t / nu, c = t - r * nu;
            if (r == k) continue;
            M[t] = (c == k ? 0.0 : M[t]) - fcol[r] * M[k * nu + c];
        }
        __syncthreads();
    }
    if (bad_s) {
        if (tid == 0) *ok = 0;
        return;
    }
    // undo the row interchanges: swap columns k <-> piv[k], last interchange first
    for (int k = nu - 1; k >= 0; k--) {
        const int pc = piv[k];
        if (pc != k)
            for (int r = tid; r < nu; r += nt) {
                const double t = M[r * nu + k];
                M[r * nu + k] = M[r * nu + pc];
                M[r * nu + pc] = t;
            }
        __syncthreads();
    }
    for (int t = tid; t < nu * nu; t += nt) {
        const int j = t / nu, r = t - j * nu;
        inv[t] = (float)M[r * nu + j];
    }
    if (tid == 0) *ok = 1;
}

// Exact coarsest solve unless AGB_BOTTOM_EXACT=0 (read when an operator is created).
bool use_exact_bottom()
{
    const char* s = getenv("AGB_BOTTOM_EXACT");
    return !(s && s[0] == '0');
}

void launch_bottom_invert(cudaStream_t st, const LevelDesc& L, const double* A, float* inv, int* ok)
{
    const size_t nu = 3 * (size_t)L.count();
    k_bottom_invert<<<1, 1024, nu * nu * sizeof(double), st>>>(L, A, inv, ok);
    count_launch();
}

// Small bottom levels use the dense path unless AGB_BOTTOM_DENSE=0.
bool use_dense_bottom()
{
    static bool v = [] {
        const char* s = getenv("AGB_BOTTOM_DENSE");
        return !(s && s[0] == '0');
    }();
    return v;
}

size_t bottom_dense_bytes(const LevelDesc& L)
{
    const size_t nu = 3 * (size_t)L.count();
    return nu * nu * sizeof(double);
}

void launch_bottom_assemble(cudaStream_t st, int sym, const LevelDesc& L, const BCTable& bc, bool uniform,
                            const double* ddw64, double* A)
{
    const Geo<double> g = make_geo<double>(L);
    const int cnt = (int)L.count(), work = cnt * 3 * cnt;
    const int blocks = (work + 255) / 256;
    if (sym == SYM_ISO) k_bottom_assemble<SYM_ISO><<<blocks, 256, 0, st>>>(L, bc, g, uniform ? 1 : 0, ddw64, A);
    else k_bottom_assemble<SYM_MM><<<blocks, 256, 0, st>>>(L, bc, g, uniform ? 1 : 0, ddw64, A);
    count_launch();
}

template <typename T>
void launch_bottom_dense(cudaStream_t st, const LevelDesc& L, const double* A, const double* diag64, T* cor,
                         const T* res, int maxiter, double tol_rel, double tol_abs, int* ret_slot, int nub, int nuf,
                         double omega, const float* inv, const int* inv_ok)
{
    const size_t nu = 3 * (size_t)L.count();
    const size_t smem = (nu * nu + nu) * sizeof(T);
    pdl_launch(k_bottom_dense<T, T>, dim3(1), dim3(DENSE_MAX), smem, st, L, A, diag64, cor, res, maxiter, tol_rel,
               tol_abs, nub, nuf, omega, ret_slot, inv, inv_ok);
    count_launch();
}

void init_bottom_attributes()
{
    const int smem = (DENSE_MAX * DENSE_MAX + DENSE_MAX) * (int)sizeof(double);
    cudaFuncSetAttribute(k_bottom_dense<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_bottom_dense<float, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_bottom_invert, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         DENSE_MAX * DENSE_MAX * (int)sizeof(double));
}

template void launch_bottom_dense<double>(cudaStream_t, const LevelDesc&, const double*, const double*, double*,
                                          const double*, int, double, double, int*, int, int, double, const float*,
                                          const int*);
template void launch_bottom_dense<float>(cudaStream_t, const LevelDesc&, const double*, const double*, float*,
                                         const float*, int, double, double, int*, int, int, double, const float*,
                                         const int*);

template <typename T>
void launch_bottom(cudaStream_t st, int sym, const LevelDesc& L, const BCTable& bc, bool uniform, const double* ddw64,
                   const double* diag64, T* cor, const T* res, double* work, int maxiter, double tol_rel,
                   double tol_abs, int* ret_slot, int nub, int nuf, double omega)
{
    const Geo<double> g = make_geo<double>(L);
    if (sym == SYM_ISO)
        k_bottom<T, SYM_ISO><<<1, BOT_THREADS, 0, st>>>(L, bc, g, uniform ? 1 : 0, ddw64, diag64, cor, res, work,
                                                        maxiter, tol_rel, tol_abs, nub, nuf, omega, ret_slot);
    else
        k_bottom<T, SYM_MM><<<1, BOT_THREADS, 0, st>>>(L, bc, g, uniform ? 1 : 0, ddw64, diag64, cor, res, work,
                                                       maxiter, tol_rel, tol_abs, nub, nuf, omega, ret_slot);
    count_launch();
}

template void launch_bottom<double>(cudaStream_t, int, const LevelDesc&, const BCTable&, bool, const double*,
                                    const double*, double*, const double*, double*, int, double, double, int*, int,
                                    int, double);
template void launch_bottom<float>(cudaStream_t, int, const LevelDesc&, const BCTable&, bool, const double*,
                                   const double*, float*, const float*, double*, int, double, double, int*, int, int,
                                   double);

}  // namespace agb

// ---------------------------------------------------------------------------
// Allocation-free coarsest-level solve (agb_bottom_solve_noalloc in agb.h)
//
// Some callers may not allocate device memory at the moment they need a
// bottom solve: a host framework that owns every device byte through its own
// arena and forbids cudaMalloc inside its solver hooks, or a time-stepping
// code that must not stall on cudaMalloc's implicit synchronisation in the
// middle of a step.  For them the BiCGStab
// work vectors live in a file-scope device array instead of a buffer of an
// operator handle.  The array is sized for boxes of at most
// AGB_NOALLOC_MAX_NODES nodes (a 16^3-cell box); every GPU that loads this
// library holds it (943 KB) until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

#include "agb.h"

namespace {

constexpr long long kScratchDoubles = 8LL * 3LL * AGB_NOALLOC_MAX_NODES;
static __device__ __align__(256) double g_bottom_scratch[kScratchDoubles];

constexpr int kMaxDevices = 256;
std::mutex g_scratch_mutex;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of g_bottom_scratch on the current device.  The name
// g_bottom_scratch is only a host-side stand-in: a kernel must be given the
// address that cudaGetSymbolAddress returns for the device it runs on.  The
// address is cached per device for the life of the process, which assumes
// one CUDA context per device: after cudaDeviceReset the cached address is
// stale, so a caller that resets a device must not call this entry point
// again in that process.
agb_status scratch_for_current_device(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        agb::set_error("no usable CUDA device for the allocation-free bottom solve");
        return AGB_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        agb::set_error("device index out of range");
        return AGB_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_bottom_scratch);
        if (e != cudaSuccess || !p) {
            agb::set_error("cudaGetSymbolAddress of the bottom-solve scratch failed");
            return AGB_CUDA;
        }
        g_scratch_addr[dev] = (double*)p;
    }
    *out = g_scratch_addr[dev];
    return AGB_OK;
}

}  // namespace

extern "C" agb_status agb_bottom_solve_noalloc(const int n_cells[3], const double dx[3], int sym, int uniform,
                                               const agb_bc* bc, const double* ddw, const double* diag,
                                               const double* res, double* cor, int* ret, int max_iter,
                                               double tol_rel, double tol_abs, int bottom_smooth, int final_smooth,
                                               double omega, void* stream)
{
    using namespace agb;
    if (!n_cells || !dx || !bc || !ddw || !diag || !res || !cor || !ret) {
        set_error("null argument");
        return AGB_BADARG;
    }
    if (sym != AGB_ISO && sym != AGB_MAJORMINOR) {
        set_error("sym must be AGB_ISO or AGB_MAJORMINOR");
        return AGB_BADARG;
    }
    long long nodes = 1;
    for (int d = 0; d < 3; d++) {
        if (n_cells[d] < 1 || !(dx[d] > 0)) {
            set_error("n_cells must be >= 1 and dx > 0");
            return AGB_BADARG;
        }
        nodes *= (long long)(n_cells[d] + 1);
    }
    if (nodes > AGB_NOALLOC_MAX_NODES) {
        set_error("box too large for the allocation-free bottom solve: more than AGB_NOALLOC_MAX_NODES nodes");
        return AGB_BADARG;
    }
    if (cor == res) {
        set_error("res and cor must be distinct, non-overlapping arrays");
        return AGB_BADARG;
    }
    if (max_iter < 0 || bottom_smooth < 0 || final_smooth < 0 || !(omega > 0 && omega < 2)) {
        set_error("bad iteration count, smoothing count or omega");
        return AGB_BADARG;
    }
    BCTable t;
    for (int f = 0; f < F_NFACES; f++)
        for (int c = 0; c < 3; c++) {
            if (bc->type[f][c] < AGB_BC_DISP || bc->type[f][c] > AGB_BC_NONE) {
                set_error("bad BC type");
                return AGB_BADARG;
            }
            // The box has no periodic direction: a periodic row would be an
            // empty row (zero diagonal) of the scaled system.
            if (bc->type[f][c] == AGB_BC_PERIODIC) {
                set_error("the allocation-free bottom solve takes no periodic BC type");
                return AGB_BADARG;
            }
            t.type[f][c] = (int8_t)bc->type[f][c];
            t.val[f][c] = bc->val[f][c];
        }
    // The caller's arrays are the unpadded reference layout: row pitch n0+1,
    // component stride = node count.
    LevelDesc L;
    for (int d = 0; d < 3; d++) {
        L.n[d] = n_cells[d];
        L.nn[d] = n_cells[d] + 1;
        L.per[d] = 0;
        L.dx[d] = dx[d];
    }
    L.P = L.nn[0];
    L.S = nodes;
    double* work = nullptr;
    const agb_status s = scratch_for_current_device(&work);
    if (s != AGB_OK) return s;
    // An error pending from earlier, unrelated work is not this call's: clear
    // it, so that the check after the launch sees only the launch's own
    // error (a broken context makes the launch itself fail).
    if (cudaPeekAtLastError() != cudaSuccess) cudaGetLastError();
    // Every scratch element the kernel reads is written earlier in the same
    // launch, so the contents left by a previous call need no clearing.
    launch_bottom<double>((cudaStream_t)stream, sym, L, t, uniform != 0, ddw, diag, cor, res, work, max_iter, tol_rel,
                          tol_abs, ret, bottom_smooth, final_smooth, omega);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(cudaGetErrorString(e));
        return AGB_CUDA;
    }
    return AGB_OK;
}
