// bottom.cuh -- the dense coarsest-level BiCGStab of one CTA (the dense
// bottom kernel's body), with its block reductions.
#pragma once
#include "agb_internal.h"
#include "stencil.cuh"

namespace agb {

// ---------------------------------------------------------------------------
// Dense coarsest level.  When the bottom level has at most DENSE_MAX unknowns
// (3 x nodes; 81 for the 3^3-node level of a 2^k-cell box) its operator is
// assembled once per solve as a dense matrix, column j = A e_j evaluated with
// the same per-node rows (stencil.cuh), and the bottom solve runs the same
// BiCGStab + smoothing as k_bottom with dense products, one thread per
// unknown, the operator read from shared memory instead of re-evaluating
// every stencil row.  Results equal k_bottom's up to the summation order of
// A x and of the dot products.
// ---------------------------------------------------------------------------
constexpr int DENSE_MAX = 128;   // unknowns (one thread each)

// Unknown q = c * cnt + e, e = i + nn0 * (j + nn1 * k) the node's place in the
// level's node enumeration.
__device__ __forceinline__ long long dense_to_padded(const LevelDesc& L, int q, int cnt)
{
    const int c = q / cnt, e = q - c * cnt;
    return c * L.S + L.idx(e % L.nn[0], (e / L.nn[0]) % L.nn[1], e / (L.nn[0] * L.nn[1]));
}

// The BiCGStab + smoothing of k_bottom on the dense operator, arithmetic in R.
// The FP64 solve runs it in FP64; the FP32 cycles of the mixed solve run it in
// FP32, like the rest of their cycle (GB300's FP64 rate per SM sub-partition
// is about 1/64 of its FP32 rate, so an FP64 bottom solve would cost more than
// the FP32 cycle around it).  The operator sits in shared memory
// (column-major, A[j * nu + q] = (A e_j)_q); thread q < nu owns unknown q and
// every thread of the CTA takes part in the barriers.  Each reduction costs
// one barrier: warps reduce by shuffles, write their partials to one of two
// alternating buffers, and after the barrier every thread combines the
// partials in warp order (so all threads hold the same value and take the
// same branches).  Reductions that need no value in between share a barrier:
// (max|r|, rh.r) at the end of an iteration, (t.t, t.s), and the publication
// of s with max|s|.  A x is summed as four interleaved partial sums.
enum { RED_SUM = 0, RED_MAX = 1 };

template <typename R> struct BlockRed {
    R* red;    // shared: 2 buffers x 3 values x 32 warps
    int buf;
    template <int N>
    __device__ __forceinline__ void run(R (&v)[N], const int (&op)[N])
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
#pragma unroll
        for (int k = 0; k < N; k++) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const R w = __shfl_xor_sync(0xffffffffu, v[k], o);
                if (op[k] == RED_SUM) v[k] += w;
                else v[k] = (w > v[k] || w != w) ? w : v[k];
            }
            if (lane == 0) red[(buf * 3 + k) * 32 + warp] = v[k];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < N; k++) {
            R t = red[(buf * 3 + k) * 32];
            for (int w = 1; w < nw; w++) {
                const R x = red[(buf * 3 + k) * 32 + w];
                if (op[k] == RED_SUM) t += x;
                else t = (x > t || x != x) ? x : t;
            }
            v[k] = t;
        }
        buf ^= 1;
    }
};

// Right-hand side read with L2-coherent loads (it may have been written
// earlier in the same kernel by other CTAs).  `red` holds 2 x 3 x 32 values.
template <typename T, typename R>
__device__ void dense_bottom_block(const LevelDesc& L, const R* __restrict__ A, R* __restrict__ xs, R* __restrict__ red,
                                   const double* __restrict__ diag, T* __restrict__ cor, const T* __restrict__ res,
                                   int maxiter, double eps_rel_d, double eps_abs_d, int nub, int nuf, double omega_d,
                                   int* ret_slot)
{
    const int cnt = (int)L.count(), nu = 3 * cnt;
    const int q = threadIdx.x;
    const bool ok = q < nu;
    const int comp = ok ? q / cnt : 0;
    const long long pq = ok ? dense_to_padded(L, q, cnt) : 0;
    const R b = ok ? (R)__ldcg(res + pq) : (R)0;
    const R d = ok ? (R)diag[pq] : (R)1;
    const R eps_rel = (R)eps_rel_d, eps_abs = (R)eps_abs_d, omega = (R)omega_d;
    const bool sing = L.singular();
    BlockRed<R> br{red, 0};
    // y = A x for the vector published in xs: four partial sums over j = 4t + s,
    // so the loads of the next columns overlap the multiply-adds
    auto product = [&]() -> R {
        R y0 = 0, y1 = 0, y2 = 0, y3 = 0;
        if (ok) {
            int j = 0;
#pragma unroll 2
            for (; j + 3 < nu; j += 4) {
                y0 += A[j * nu + q] * xs[j];
                y1 += A[(j + 1) * nu + q] * xs[j + 1];
                y2 += A[(j + 2) * nu + q] * xs[j + 2];
                y3 += A[(j + 3) * nu + q] * xs[j + 3];
            }
            for (; j < nu; j++) y0 += A[j * nu + q] * xs[j];
        }
        return (y0 + y1) + (y2 + y3);
    };
    auto publish = [&](R x) {
        if (ok) xs[q] = x;
    };
    // zero-mean projection per component (fully periodic level)
    auto project = [&](R v) -> R {
        R m[3] = {ok && comp == 0 ? v : (R)0, ok && comp == 1 ? v : (R)0, ok && comp == 2 ? v : (R)0};
        const int op[3] = {RED_SUM, RED_SUM, RED_SUM};
        br.run(m, op);
        const R mc = comp == 0 ? m[0] : (comp == 1 ? m[1] : m[2]);
        return ok ? v - mc / (R)cnt : (R)0;
    };
    R sol = 0, r = 0, rh = 0, p = 0, v = 0, sv = 0, t = 0;
    // r = P(b - A*0)/D, P the zero-mean projection on a singular level
    const R bp = sing ? project(b) : b;
    if (ok) {
        r = bp / d;
        rh = r;
    }
    R rnorm, rho;
    {
        R m[2] = {fabs(r), rh * r};
        const int op[2] = {RED_MAX, RED_SUM};
        br.run(m, op);
        rnorm = m[0];
        rho = m[1];
    }
    const R rnorm0 = rnorm;
    int ret = 0;
    R rho_1 = 0, alpha = 0, om = 0;
    if (!(rnorm0 == 0 || rnorm0 < eps_abs)) {
        for (int iter = 1; iter <= maxiter; iter++) {
            if (rho == 0) { ret = 1; break; }
            if (iter == 1) p = r;
            else {
                const R beta = (rho / rho_1) * (alpha / om);
                p = r + beta * (p - om * v);
            }
            // every thread finished reading xs (last product) before the last barrier
            publish(p);
            __syncthreads();
            v = product();
            if (sing) v = project(v);
            v = ok ? v / d : (R)0;
            {
                R m[1] = {rh * v};
                const int op[1] = {RED_SUM};
                br.run(m, op);
                if (m[0] != 0) alpha = rho / m[0];
                else { ret = 2; break; }
            }
            sol += alpha * p;
            sv = r - alpha * v;
            publish(sv);   // xs is free: every product(p) finished before the rh.v barrier
            {
                R m[1] = {fabs(sv)};
                const int op[1] = {RED_MAX};
                br.run(m, op);
                rnorm = m[0];
            }
            if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
            t = product();
            if (sing) t = project(t);
            t = ok ? t / d : (R)0;
            {
                R m[2] = {t * t, t * sv};
                const int op[2] = {RED_SUM, RED_SUM};
                br.run(m, op);
                if (m[0] != 0) om = m[1] / m[0];
                else { ret = 3; break; }
            }
            sol += om * sv;
            r = sv - om * t;
            rho_1 = rho;
            {
                R m[2] = {fabs(r), rh * r};
                const int op[2] = {RED_MAX, RED_SUM};
                br.run(m, op);
                rnorm = m[0];
                rho = m[1];
            }
            if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
            if (om == 0) { ret = 4; break; }
        }
        if (ret == 0 && rnorm > eps_rel * rnorm0 && rnorm > eps_abs) ret = 8;
        // MLMG::actualBottomSolve: anything but a clean solve discards the correction
        if (ret != 0 || !(rnorm < rnorm0)) sol = 0;
    }
    // post-smoothing: Fsmooth = 2 Jacobi sweeps each
    const int nsm = 2 * ((ret == 0) ? nub : nuf);
    for (int sw = 0; sw < nsm; sw++) {
        __syncthreads();   // the last product finished with xs
        publish(sol);
        __syncthreads();
        const R Ax = product();
        if (ok) {
            const R Rx = Ax - sol * d;
            sol = ((R)1 - omega) * sol + omega * (b - Rx) / d;
        }
    }
    if (ok) cor[pq] = (T)sol;
    if (threadIdx.x == 0 && ret_slot) *ret_slot = ret;
}

}  // namespace agb
