// kernels_stencil.cu -- Fapply / residual / damped-Jacobi / diagonal kernels.
//
//   MODE_APPLY   out = A x                          (Elastic::Fapply, Elastic.cpp:141-292)
//   MODE_RESID   out = b - A x, max|out| -> slot    (solutionResidual, Operator.cpp:636-657)
//   MODE_JACOBI  out = x + omega * (b - A x) / D    (one sweep of Operator<Node>::Fsmooth,
//                                                    Operator.cpp:107-147, with the reference's
//                                                    (1-w)x + w(b-(Ax-Dx))/D regrouped;
//                                                    `diag` carries 1/D)
//
// Two kernels share the per-node arithmetic of stencil.cuh:
//   k_stencil_node   one thread per node, every node of the level (small levels,
//                    boundary shells); global loads through the read-only path.
//   k_stencil_march  interior nodes of large levels: a (32 x 8) column tile
//                    marches in k; the three u planes and the modulus plane of
//                    the tile (+1 halo) are staged in shared memory, so each
//                    array element is read from HBM once per sweep.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>

#include "agb_internal.h"
#include "stencil.cuh"

namespace agb {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

template <typename T> struct MaxBits;
template <> struct MaxBits<double> {
    typedef unsigned long long U;
    static __device__ __forceinline__ U bits(double v) { return (U)__double_as_longlong(v); }
    static __device__ __forceinline__ void atomic(void* slot, double v)
    {
        atomicMax((unsigned long long*)slot, bits(v));
    }
};
template <> struct MaxBits<float> {
    typedef unsigned int U;
    static __device__ __forceinline__ U bits(float v) { return (U)__float_as_uint(v); }
    static __device__ __forceinline__ void atomic(void* slot, float v) { atomicMax((unsigned int*)slot, bits(v)); }
};

// max of |v| over the block (v >= 0 or NaN); one atomic per block.  NaN has the
// largest bit pattern of the non-negative encodings, so it propagates.
template <typename T>
__device__ __forceinline__ void block_max_to_slot(T v, void* slot)
{
    __shared__ T red[32];
    const int lane = (threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z)) & 31;
    const int warp = (threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z)) >> 5;
    const int nwarp = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T w = __shfl_xor_sync(0xffffffffu, v, o);
        v = (w > v || w != w) ? w : v;
    }
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < nwarp ? red[lane] : (T)0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            T w = __shfl_xor_sync(0xffffffffu, v, o);
            v = (w > v || w != w) ? w : v;
        }
        if (lane == 0) MaxBits<T>::atomic(slot, v);
    }
}

template <typename T> struct GlobalAcc {
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

template <typename T, int MODE>
__device__ __forceinline__ void epilogue(const T f[3], const T* __restrict__ x, const T* __restrict__ b,
                                         const T* __restrict__ dinv, T* __restrict__ out, long long S, long long p,
                                         T omega, T& nrm)
{
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const long long q = c * S + p;
        if (MODE == MODE_APPLY) {
            out[q] = f[c];
        } else if (MODE == MODE_RESID) {
            const T r = b[q] - f[c];
            out[q] = r;
            const T a = fabs(r);
            nrm = (a > nrm || a != a) ? a : nrm;
        } else {
            out[q] = x[q] + omega * ((b[q] - f[c]) * dinv[q]);
        }
    }
}

// ---------------------------------------------------------------------------
// one thread per node
// ---------------------------------------------------------------------------
template <typename T, int SYM, int MODE>
__global__ void __launch_bounds__(256) k_stencil_node(LevelDesc L, BCTable bc, Geo<T> g, int uniform,
                                                      const T* __restrict__ ddw, const T* __restrict__ x,
                                                      const T* __restrict__ b, const T* __restrict__ dinv,
                                                      T* __restrict__ out, T omega, void* norm_slot, int shell)
{
    pdl_entry();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    T nrm = 0;
    if (i < L.nn[0] && j < L.nn[1] && k < L.nn[2]) {
        const int pos[3] = {i, j, k};
        int mn[3], mx[3];
        bool bnd = false;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            mn[d] = !L.per[d] && pos[d] == 0;
            mx[d] = !L.per[d] && pos[d] == L.n[d];
            bnd = bnd || mn[d] || mx[d];
        }
        if (!shell || bnd) {
            GlobalAcc<T> acc{x, ddw, L.S, make_nbr(L, i, j, k)};
            T f[3];
            if (bnd) boundary_row<T, SYM>(acc, g, bc, mn, mx, f);
            else interior_row<T, SYM>(acc, g, uniform != 0, f);
            epilogue<T, MODE>(f, x, b, dinv, out, L.S, acc.nb.base, omega, nrm);
        }
    }
    if (MODE == MODE_RESID && norm_slot) block_max_to_slot<T>(nrm, norm_slot);
}

// ---------------------------------------------------------------------------
// boundary shell of a box with no periodic direction: one thread per boundary
// node, enumerated plane k=0, plane k=n2, then the rings of the planes between
// ---------------------------------------------------------------------------
// (with xf = 0 the x-face nodes between the y rows are left out: the TMA
// interior kernel computes them)
__host__ __device__ inline long long shell_count(const LevelDesc& L, int xf)
{
    const long long a = (long long)L.nn[0] * L.nn[1];
    return 2 * a + (long long)(L.nn[2] - 2) * (2LL * L.nn[0] + (xf ? 2LL * (L.nn[1] - 2) : 0LL));
}

__device__ __forceinline__ void shell_node(const LevelDesc& L, long long e, int xf, int& i, int& j, int& k)
{
    const long long a = (long long)L.nn[0] * L.nn[1];
    if (e < 2 * a) {
        k = e < a ? 0 : L.nn[2] - 1;
        const long long r = e < a ? e : e - a;
        j = (int)(r / L.nn[0]);
        i = (int)(r % L.nn[0]);
        return;
    }
    const long long e2 = e - 2 * a, pm = 2LL * L.nn[0] + (xf ? 2LL * (L.nn[1] - 2) : 0LL);
    k = 1 + (int)(e2 / pm);
    const int r = (int)(e2 % pm);
    if (r < 2 * L.nn[0]) {
        j = r < L.nn[0] ? 0 : L.nn[1] - 1;
        i = r < L.nn[0] ? r : r - L.nn[0];
    } else {
        const int r2 = r - 2 * L.nn[0];
        j = 1 + r2 / 2;
        i = (r2 & 1) ? L.nn[0] - 1 : 0;
    }
}

template <typename T, int SYM, int MODE>
__global__ void __launch_bounds__(256) k_stencil_shell(LevelDesc L, BCTable bc, Geo<T> g, const T* __restrict__ ddw,
                                                       const T* __restrict__ x, const T* __restrict__ b,
                                                       const T* __restrict__ dinv, T* __restrict__ out, T omega,
                                                       void* norm_slot, int xf)
{
    pdl_entry();
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    T nrm = 0;
    if (e < shell_count(L, xf)) {
        int i, j, k;
        shell_node(L, e, xf, i, j, k);
        const int pos[3] = {i, j, k};
        int mn[3], mx[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            mn[d] = pos[d] == 0;
            mx[d] = pos[d] == L.n[d];
        }
        GlobalAcc<T> acc{x, ddw, L.S, make_nbr(L, i, j, k)};
        T f[3];
        boundary_row<T, SYM>(acc, g, bc, mn, mx, f);
        epilogue<T, MODE>(f, x, b, dinv, out, L.S, acc.nb.base, omega, nrm);
    }
    if (MODE == MODE_RESID && norm_slot) block_max_to_slot<T>(nrm, norm_slot);
}

// ---------------------------------------------------------------------------
// k-marching interior kernel
// ---------------------------------------------------------------------------
constexpr int MT_X = 32, MT_Y = 8, MT_Z = 16;   // tile and k-chunk
constexpr int MH_X = MT_X + 2, MH_Y = MT_Y + 2; // with halo

template <typename T, int SYM> struct MarchSmem {
    static constexpr int NC = NCoef<SYM>::value;
    T u[3][3][MH_Y][MH_X];    // ring of 3 planes (k-1, k, k+1) x 3 components
    T c[2][NC][MH_Y][MH_X];   // modulus planes k and k+1 (ring of 2)
};

template <typename T, int SYM> struct SmemAcc {
    const MarchSmem<T, SYM>* s;
    int tx, ty;           // position in the halo tile (1..)
    int r0, r1, r2;       // u ring slots of planes k-1, k, k+1
    int cb, nb;           // modulus ring slots of planes k, k+1
    T cm[NCoef<SYM>::value];  // modulus at (i, j, k-1), kept in registers
    __device__ __forceinline__ T u(int p, int di, int dj, int dk) const
    {
        const int r = dk < 0 ? r0 : (dk > 0 ? r2 : r1);
        return s->u[r][p][ty + dj][tx + di];
    }
    __device__ __forceinline__ T C(int m, int di, int dj, int dk) const
    {
        if (dk < 0) return cm[m];
        if (dk > 0) return s->c[nb][m][ty][tx];
        return s->c[cb][m][ty + dj][tx + di];
    }
};

// Interior nodes only: i in [1, n0-1], j in [1, n1-1], k in [1, n2-1] of a
// level with no periodic direction.  Grid: (ceil((n0-1)/32), ceil((n1-1)/8),
// ceil((n2-1)/MT_Z)).
template <typename T, int SYM, int MODE>
__global__ void __launch_bounds__(MT_X* MT_Y) k_stencil_march(LevelDesc L, Geo<T> g, int uniform,
                                                                 const T* __restrict__ ddw, const T* __restrict__ x,
                                                                 const T* __restrict__ b,
                                                                 const T* __restrict__ dinv, T* __restrict__ out,
                                                                 T omega, void* norm_slot)
{
    pdl_entry();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    MarchSmem<T, SYM>& s = *reinterpret_cast<MarchSmem<T, SYM>*>(smem_raw);
    constexpr int NC = NCoef<SYM>::value;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + MT_X * ty;
    const int i0 = 1 + blockIdx.x * MT_X, j0 = 1 + blockIdx.y * MT_Y;
    const int k0 = 1 + blockIdx.z * MT_Z;
    const int k1 = min(k0 + MT_Z, L.n[2]);   // exclusive; interior k < n2
    const int i = i0 + tx, j = j0 + ty;
    const bool mine = (i < L.n[0]) && (j < L.n[1]);
    const long long S = L.S;
    const long long plane = (long long)L.P * L.nn[1];

    // halo tile loaders (nodes beyond the hi boundary read as 0 and are never used)
    auto load_u_plane = [&](int r, int kk) {
        for (int e = tid; e < MH_X * MH_Y; e += MT_X * MT_Y) {
            const int hx = e % MH_X, hy = e / MH_X;
            const int gi = i0 - 1 + hx, gj = j0 - 1 + hy;
            const bool ok = gi <= L.n[0] && gj <= L.n[1];
            const long long p = (long long)gi + (long long)L.P * gj + plane * kk;
#pragma unroll
            for (int c = 0; c < 3; c++) s.u[r][c][hy][hx] = ok ? __ldg(x + c * S + p) : (T)0;
        }
    };
    auto load_c_plane = [&](int r, int kk) {
        for (int e = tid; e < MH_X * MH_Y; e += MT_X * MT_Y) {
            const int hx = e % MH_X, hy = e / MH_X;
            const int gi = i0 - 1 + hx, gj = j0 - 1 + hy;
            const bool ok = gi <= L.n[0] && gj <= L.n[1];
            const long long p = (long long)gi + (long long)L.P * gj + plane * kk;
#pragma unroll
            for (int m = 0; m < NC; m++) s.c[r][m][hy][hx] = ok ? __ldg(ddw + m * S + p) : (T)0;
        }
    };

    SmemAcc<T, SYM> acc;
    acc.s = &s;
    acc.tx = tx + 1;
    acc.ty = ty + 1;
    acc.r0 = 0; acc.r1 = 1; acc.r2 = 2;
    acc.cb = 0; acc.nb = 1;
    {
        const long long p = (long long)min(i, L.n[0]) + (long long)L.P * min(j, L.n[1]) + plane * (k0 - 1);
#pragma unroll
        for (int m = 0; m < NC; m++) acc.cm[m] = __ldg(ddw + m * S + p);
    }
    load_u_plane(0, k0 - 1);
    load_u_plane(1, k0);
    load_c_plane(0, k0);
    T nrm = 0;
    for (int k = k0; k < k1; k++) {
        load_u_plane(acc.r2, k + 1);
        load_c_plane(acc.nb, k + 1);
        __syncthreads();
        if (mine) {
            T f[3];
            interior_row<T, SYM>(acc, g, uniform != 0, f);
            epilogue<T, MODE>(f, x, b, dinv, out, S, L.idx(i, j, k), omega, nrm);
        }
#pragma unroll
        for (int m = 0; m < NC; m++) acc.cm[m] = s.c[acc.cb][m][ty + 1][tx + 1];
        __syncthreads();
        const int t = acc.r0;
        acc.r0 = acc.r1;
        acc.r1 = acc.r2;
        acc.r2 = t;
        acc.cb ^= 1;
        acc.nb ^= 1;
    }
    if (MODE == MODE_RESID && norm_slot) block_max_to_slot<T>(nrm, norm_slot);
}

// ---------------------------------------------------------------------------
// cp.async-pipelined marching kernel (FP32 cycles on the finest levels)
//
// Same tile and per-node arithmetic as k_stencil_march, but the planes are
// copied global -> shared with 16-byte cp.async (L1 bypassed) two planes ahead
// of the compute: u in a ring of 4 planes, moduli in a ring of 3, so the loads
// of plane k+3 overlap the arithmetic of plane k.  Every halo row is 36
// elements wide and starts at i = 32t, 16-byte aligned (the level's row pitch
// leaves room for it).  Own-column values at k-1 (moduli) are kept in
// registers.
// ---------------------------------------------------------------------------
constexpr int PT_Z = 32;            // k-chunk of one CTA
constexpr int PW = 36;              // halo row width loaded (9 x 16 bytes)
constexpr int PU = 4, PC = 3;       // ring depths (u, moduli)

template <typename T, int SYM> struct PipeSmem {
    static constexpr int NC = NCoef<SYM>::value;
    T u[PU][3][MH_Y][PW];
    T c[PC][NC][MH_Y][PW];
};

template <typename T, int SYM> struct PipeAcc {
    const PipeSmem<T, SYM>* s;
    int tx, ty;            // halo-tile position of the node (1-based)
    int um, u0, up;        // u ring slots of planes k-1, k, k+1
    int c0, cp;            // moduli ring slots of planes k, k+1
    T cm[NCoef<SYM>::value];
    __device__ __forceinline__ T u(int p, int di, int dj, int dk) const
    {
        const int r = dk < 0 ? um : (dk > 0 ? up : u0);
        return s->u[r][p][ty + dj][tx + di];
    }
    __device__ __forceinline__ T C(int m, int di, int dj, int dk) const
    {
        if (dk < 0) return cm[m];
        if (dk > 0) return s->c[cp][m][ty][tx];
        return s->c[c0][m][ty + dj][tx + di];
    }
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    unsigned long long ga;
    asm volatile("cvta.to.global.u64 %0, %1;" : "=l"(ga) : "l"(gmem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(ga) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Queue the copy of plane kk of `ncomp` planes of src into dst[ncomp][MH_Y][PW].
template <typename T>
__device__ __forceinline__ void issue_plane(T* dst, const T* __restrict__ src, int ncomp, const LevelDesc& L, int i0,
                                            int j0, int kk, int tid)
{
    constexpr int VEC = 16 / sizeof(T);        // elements per 16-byte chunk
    constexpr int QPR = PW / VEC;              // chunks per halo row
    const int per_comp = MH_Y * QPR;
    const long long plane = (long long)L.P * L.nn[1] * kk;
    for (int e = tid; e < ncomp * per_comp; e += MT_X * MT_Y) {
        const int c = e / per_comp, rem = e - c * per_comp;
        const int row = rem / QPR, q = rem - row * QPR;
        const int gj = j0 - 1 + row;
        if (gj > L.n[1]) continue;   // rows past the hi boundary are never read
        const T* g = src + c * L.S + plane + (long long)L.P * gj + (i0 - 1) + q * VEC;
        cp_async16(dst + ((c * MH_Y + row) * PW + q * VEC), g);
    }
}

template <typename T, int SYM, int MODE>
__global__ void __launch_bounds__(MT_X* MT_Y) k_stencil_pipe(LevelDesc L, Geo<T> g, int uniform,
                                                                const T* __restrict__ ddw, const T* __restrict__ x,
                                                                const T* __restrict__ b, const T* __restrict__ dinv,
                                                                T* __restrict__ out, T omega, void* norm_slot)
{
    pdl_entry();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PipeSmem<T, SYM>& s = *reinterpret_cast<PipeSmem<T, SYM>*>(smem_raw);
    constexpr int NC = NCoef<SYM>::value;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + MT_X * ty;
    const int i0 = 1 + blockIdx.x * MT_X, j0 = 1 + blockIdx.y * MT_Y;
    const int k0 = 1 + blockIdx.z * PT_Z;
    const int k1 = min(k0 + PT_Z, L.n[2]);   // exclusive
    const int i = i0 + tx, j = j0 + ty;
    const bool mine = (i < L.n[0]) && (j < L.n[1]);
    const long long S = L.S;

    PipeAcc<T, SYM> acc;
    acc.s = &s;
    acc.tx = tx + 1;
    acc.ty = ty + 1;
    {
        const long long p = L.idx(min(i, L.n[0]), min(j, L.n[1]), k0 - 1);
#pragma unroll
        for (int m = 0; m < NC; m++) acc.cm[m] = __ldg(ddw + m * S + p);
    }
    // prologue: planes k0-1, k0, k0+1 of u and k0, k0+1 of the moduli, then k0+2
    issue_plane<T>(&s.u[0][0][0][0], x, 3, L, i0, j0, k0 - 1, tid);
    issue_plane<T>(&s.u[1][0][0][0], x, 3, L, i0, j0, k0, tid);
    issue_plane<T>(&s.u[2][0][0][0], x, 3, L, i0, j0, k0 + 1, tid);
    issue_plane<T>(&s.c[0][0][0][0], ddw, NC, L, i0, j0, k0, tid);
    issue_plane<T>(&s.c[1][0][0][0], ddw, NC, L, i0, j0, k0 + 1, tid);
    cp_async_commit();
    if (k0 + 2 <= k1) {
        issue_plane<T>(&s.u[3][0][0][0], x, 3, L, i0, j0, k0 + 2, tid);
        issue_plane<T>(&s.c[2][0][0][0], ddw, NC, L, i0, j0, k0 + 2, tid);
    }
    cp_async_commit();

    T nrm = 0;
    for (int k = k0; k < k1; k++) {
        const int it = k - k0;
        long long q = 0;
        T bq[3] = {0, 0, 0}, dq[3] = {0, 0, 0};
        if (mine) {
            q = L.idx(i, j, k);
            if (MODE != MODE_APPLY)
#pragma unroll
                for (int c = 0; c < 3; c++) bq[c] = __ldg(b + c * S + q);
            if (MODE == MODE_JACOBI)
#pragma unroll
                for (int c = 0; c < 3; c++) dq[c] = __ldg(dinv + c * S + q);
        }
        cp_async_wait1();
        __syncthreads();
        acc.um = it % PU;
        acc.u0 = (it + 1) % PU;
        acc.up = (it + 2) % PU;
        acc.c0 = it % PC;
        acc.cp = (it + 1) % PC;
        if (mine) {
            T f[3];
            interior_row<T, SYM>(acc, g, uniform != 0, f);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const long long o = c * S + q;
                if (MODE == MODE_APPLY) {
                    out[o] = f[c];
                } else if (MODE == MODE_RESID) {
                    const T r = bq[c] - f[c];
                    out[o] = r;
                    const T a = fabs(r);
                    nrm = (a > nrm || a != a) ? a : nrm;
                } else {
                    const T xc = s.u[acc.u0][c][ty + 1][tx + 1];
                    out[o] = xc + omega * ((bq[c] - f[c]) * dq[c]);
                }
            }
        }
#pragma unroll
        for (int m = 0; m < NC; m++) acc.cm[m] = s.c[acc.c0][m][ty + 1][tx + 1];
        __syncthreads();
        // refill the slots of u(k-1) and C(k) with plane k+3
        const int kk = k + 3;
        if (kk <= k1) {
            issue_plane<T>(&s.u[it % PU][0][0][0], x, 3, L, i0, j0, kk, tid);
            issue_plane<T>(&s.c[it % PC][0][0][0], ddw, NC, L, i0, j0, kk, tid);
        }
        cp_async_commit();
    }
    cp_async_wait0();
    if (MODE == MODE_RESID && norm_slot) block_max_to_slot<T>(nrm, norm_slot);
}

// ---------------------------------------------------------------------------
// diagonal
// ---------------------------------------------------------------------------
template <typename T, int SYM>
__global__ void k_diagonal(LevelDesc L, DiagGeo<T> dg, BCTable bc, const T* __restrict__ ddw, T* __restrict__ diag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= L.nn[0] || j >= L.nn[1] || k >= L.nn[2]) return;
    const int pos[3] = {i, j, k};
    int mn[3], mx[3];
    for (int d = 0; d < 3; d++) {
        mn[d] = !L.per[d] && pos[d] == 0;
        mx[d] = !L.per[d] && pos[d] == L.n[d];
    }
    const long long p = L.idx(i, j, k);
    T c[NCoef<SYM>::value];
    for (int m = 0; m < NCoef<SYM>::value; m++) c[m] = ddw[m * L.S + p];
    for (int q = 0; q < 3; q++) diag[q * L.S + p] = diag_entry<T, SYM>(c, L, dg, bc, mn, mx, q);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline dim3 node_grid(const LevelDesc& L, dim3 blk)
{
    return dim3((L.nn[0] + blk.x - 1) / blk.x, (L.nn[1] + blk.y - 1) / blk.y, (L.nn[2] + blk.z - 1) / blk.z);
}

// Smallest cell count per direction for which the interior goes to the
// marching kernel (AGB_MARCH_MIN_CELLS overrides; used for tile studies).
int march_min_cells()
{
    static int v = [] {
        const char* s = getenv("AGB_MARCH_MIN_CELLS");
        return s ? atoi(s) : 64;
    }();
    return v;
}

// FP32 interiors use the cp.async-pipelined kernel unless AGB_PIPE=0.
bool use_pipe_kernel()
{
    static bool v = [] {
        const char* s = getenv("AGB_PIPE");
        return !(s && s[0] == '0');
    }();
    return v;
}

template <typename T, int SYM, int MODE>
static void stencil_dispatch(cudaStream_t st, const LevelDesc& L, const BCTable& bc, bool uniform, const T* ddw,
                             const T* x, const T* b, const T* diag, T* out, T omega, void* norm_slot)
{
    const Geo<T> g = make_geo<T>(L);
    // The marching kernel pays one exposed load round trip per plane, so it
    // only wins once the box is large enough to fill every SM several times.
    const bool big = !L.per[0] && !L.per[1] && !L.per[2] && L.n[0] >= march_min_cells() &&
                     L.n[1] >= 16 && L.n[2] >= 16;
    if (big) {
        // interior by the marching kernel, boundary shell by the per-node
        // kernel (the TMA kernel also takes the x-face nodes)
        dim3 blk(MT_X, MT_Y, 1);
        bool tma = false;
        if (sizeof(T) == 4 && use_tma_kernel() && tma_supported(L) &&
            launch_stencil_tma(st, SYM, MODE, L, bc, uniform, reinterpret_cast<const float*>(ddw),
                               reinterpret_cast<const float*>(x), reinterpret_cast<const float*>(b),
                               reinterpret_cast<const float*>(diag), reinterpret_cast<float*>(out), (float)omega,
                               norm_slot)) {
            tma = true;   // launched by launch_stencil_tma
        } else if (sizeof(T) == 4 && use_pipe_kernel()) {
            const size_t smem = sizeof(PipeSmem<T, SYM>);
            dim3 grd((L.n[0] - 1 + MT_X - 1) / MT_X, (L.n[1] - 1 + MT_Y - 1) / MT_Y, (L.n[2] - 1 + PT_Z - 1) / PT_Z);
            pdl_launch(k_stencil_pipe<T, SYM, MODE>, grd, blk, smem, st, L, g, uniform ? 1 : 0, ddw, x, b, diag, out,
                       omega, norm_slot);
        } else {
            const size_t smem = sizeof(MarchSmem<T, SYM>);
            dim3 grd((L.n[0] - 1 + MT_X - 1) / MT_X, (L.n[1] - 1 + MT_Y - 1) / MT_Y, (L.n[2] - 1 + MT_Z - 1) / MT_Z);
            pdl_launch(k_stencil_march<T, SYM, MODE>, grd, blk, smem, st, L, g, uniform ? 1 : 0, ddw, x, b, diag, out,
                       omega, norm_slot);
        }
        count_launch();
        const int xf = tma ? 0 : 1;
        const long long ns = shell_count(L, xf);
        pdl_launch(k_stencil_shell<T, SYM, MODE>, dim3((unsigned)((ns + 255) / 256)), dim3(256), 0, st, L, bc, g, ddw,
                   x, b, diag, out, omega, norm_slot, xf);
        count_launch();
    } else {
        dim3 b2(32, 4, 2);
        // rows of at most 40 nodes (the 33^3 and 17^3 levels of a 2^k box
        // and below) in 8 x 8 x 4 blocks: fewer idle lanes than 32-wide rows
        // (solve 0.3247 against 0.3258 s at 257^3); AGB_NODE_NARROW overrides
        static const int narrow = [] {
            const char* e = getenv("AGB_NODE_NARROW");
            return e ? atoi(e) : 40;
        }();
        if (L.nn[0] <= narrow) b2 = dim3(8, 8, 4);
        pdl_launch(k_stencil_node<T, SYM, MODE>, node_grid(L, b2), b2, 0, st, L, bc, g, uniform ? 1 : 0, ddw, x, b,
                   diag, out, omega, norm_slot, 0);
        count_launch();
    }
}

template <typename T>
void launch_stencil(cudaStream_t st, int sym, int mode, const LevelDesc& L, const BCTable& bc, bool uniform,
                    const T* ddw, const T* x, const T* b, const T* diag, T* out, T omega, void* norm_slot)
{
#define DISP(S, M) stencil_dispatch<T, S, M>(st, L, bc, uniform, ddw, x, b, diag, out, omega, norm_slot)
    if (sym == SYM_ISO) {
        if (mode == MODE_APPLY) DISP(SYM_ISO, MODE_APPLY);
        else if (mode == MODE_RESID) DISP(SYM_ISO, MODE_RESID);
        else DISP(SYM_ISO, MODE_JACOBI);
    } else {
        if (mode == MODE_APPLY) DISP(SYM_MM, MODE_APPLY);
        else if (mode == MODE_RESID) DISP(SYM_MM, MODE_RESID);
        else DISP(SYM_MM, MODE_JACOBI);
    }
#undef DISP
}

template <typename T, int SYM>
static void set_attr()
{
    const int smem = (int)sizeof(MarchSmem<T, SYM>);
    cudaFuncSetAttribute(k_stencil_march<T, SYM, MODE_APPLY>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_stencil_march<T, SYM, MODE_RESID>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_stencil_march<T, SYM, MODE_JACOBI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (sizeof(T) == 4) {
        const int ps = (int)sizeof(PipeSmem<T, SYM>);
        cudaFuncSetAttribute(k_stencil_pipe<T, SYM, MODE_APPLY>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps);
        cudaFuncSetAttribute(k_stencil_pipe<T, SYM, MODE_RESID>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps);
        cudaFuncSetAttribute(k_stencil_pipe<T, SYM, MODE_JACOBI>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps);
    }
}

// Opt the marching kernels into their shared-memory size; called once per
// process before any launch (and so before any graph capture).
void init_kernel_attributes()
{
    set_attr<double, SYM_ISO>();
    set_attr<double, SYM_MM>();
    set_attr<float, SYM_ISO>();
    set_attr<float, SYM_MM>();
}

template <typename T>
void launch_diagonal(cudaStream_t st, int sym, const LevelDesc& L, const BCTable& bc, const T* ddw, T* diag)
{
    dim3 blk(32, 4, 2);
    const DiagGeo<T> dg = make_diag_geo<T>(L);
    if (sym == SYM_ISO) k_diagonal<T, SYM_ISO><<<node_grid(L, blk), blk, 0, st>>>(L, dg, bc, ddw, diag);
    else k_diagonal<T, SYM_MM><<<node_grid(L, blk), blk, 0, st>>>(L, dg, bc, ddw, diag);
    count_launch();
}

template void launch_stencil<double>(cudaStream_t, int, int, const LevelDesc&, const BCTable&, bool, const double*,
                                     const double*, const double*, const double*, double*, double, void*);
template void launch_stencil<float>(cudaStream_t, int, int, const LevelDesc&, const BCTable&, bool, const float*,
                                    const float*, const float*, const float*, float*, float, void*);
template void launch_diagonal<double>(cudaStream_t, int, const LevelDesc&, const BCTable&, const double*, double*);
template void launch_diagonal<float>(cudaStream_t, int, const LevelDesc&, const BCTable&, const float*, float*);

}  // namespace agb
