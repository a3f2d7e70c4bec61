// kernels_transfer.cu -- inter-level transfers and vector kernels.
//
//   restriction       Operator<Node>::restriction, Operator/Operator.cpp:262-363
//   interpolation     Operator<Node>::interpolation (additive), Operator.cpp:365-434;
//                     `assign` variant = MLMG interpAssign used by the F-cycle
//   average_ddw       Elastic::averageDownCoeffsSameAmrLevel, Operator/Elastic.cpp:748-910
//   import / export   reference nodal-box images (n+1 nodes per direction, SoA
//                     MultiFab components or AoS BaseFab<Matrix4>) <-> padded storage
#include <cuda_runtime.h>

#include <algorithm>

#include "agb_internal.h"
#include "transfer.cuh"

namespace agb {

static inline dim3 grid_for(const LevelDesc& L, dim3 blk)
{
    return dim3((L.nn[0] + blk.x - 1) / blk.x, (L.nn[1] + blk.y - 1) / blk.y, (L.nn[2] + blk.z - 1) / blk.z);
}

// Fine-level offsets of the nodes 2I-1, 2I, 2I+1 (periodic wrap) in the three
// directions of a coarse node, computed once per thread: each of the 27
// reads of a full weighting is then one add of three offsets.
struct FineOffsets {
    int ox[3];
    int oy[3];
    long long oz[3];
    __device__ __forceinline__ FineOffsets(const LevelDesc& Lf, int I, int J, int K)
    {
#pragma unroll
        for (int a = 0; a < 3; a++) {
            ox[a] = wrapn(2 * I + a - 1, Lf.n[0], Lf.per[0]);
            oy[a] = Lf.P * wrapn(2 * J + a - 1, Lf.n[1], Lf.per[1]);
            oz[a] = (long long)Lf.P * Lf.nn[1] * wrapn(2 * K + a - 1, Lf.n[2], Lf.per[2]);
        }
    }
    __device__ __forceinline__ long long at(int a, int b, int d) const { return ox[a + 1] + oy[b + 1] + oz[d + 1]; }
};

template <typename T>
__global__ void k_restrict(LevelDesc Lf, LevelDesc Lc, const T* __restrict__ fine, T* __restrict__ crse, int ncomp)
{
    pdl_entry();
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z * blockDim.z + threadIdx.z;
    if (I >= Lc.nn[0] || J >= Lc.nn[1] || K >= Lc.nn[2]) return;
    const bool bI = !Lc.per[0] && (I == 0 || I == Lc.n[0]);
    const bool bJ = !Lc.per[1] && (J == 0 || J == Lc.n[1]);
    const bool bK = !Lc.per[2] && (K == 0 || K == Lc.n[2]);
    const long long q = Lc.idx(I, J, K);
    const FineOffsets o(Lf, I, J, K);
    for (int c = 0; c < ncomp; c++) {
        const T* src = fine + c * Lf.S;
        auto f = [&](int a, int b, int d) -> T { return __ldg(src + o.at(a, b, d)); };
        crse[c * Lc.S + q] = full_weight<T>(f, bI, bJ, bK);
    }
}

template <typename T> struct Pair;
template <> struct Pair<float> { typedef float2 type; };
template <> struct Pair<double> { typedef double2 type; };

// Trilinear prolongation of the coarse correction.  A thread owns the fine
// pair i = 2I, 2I+1 of one row (the even node takes the coarse value at I,
// the odd one the mean with I+1), so a warp never splits on the parity of i;
// the parities of j and k are uniform over a warp (one row per warp).  The
// pair is read and written as one 8- or 16-byte vector (rows start on
// 32-byte boundaries and 2I is even).  Each fine value is the same
// expression, summed in the same order, as the per-node form
// (Operator.cpp:365-434).
template <typename T>
__global__ void k_interp(LevelDesc Lf, LevelDesc Lc, T* __restrict__ fine, const T* __restrict__ crse, int assign)
{
    pdl_entry();
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    const int i = 2 * I;
    if (i >= Lf.nn[0] || j >= Lf.nn[1] || k >= Lf.nn[2]) return;
    const bool two = i + 1 < Lf.nn[0];
    const int J = j >> 1, K = k >> 1;
    const int I1 = wrapn(I + 1, Lc.n[0], Lc.per[0]), J1 = wrapn(J + 1, Lc.n[1], Lc.per[1]),
              K1 = wrapn(K + 1, Lc.n[2], Lc.per[2]);
    const bool ej = !(j & 1), ek = !(k & 1);
    const long long q = Lf.idx(i, j, k);
    const long long r00 = Lc.idx(0, J, K), r10 = Lc.idx(0, J1, K), r01 = Lc.idx(0, J, K1), r11 = Lc.idx(0, J1, K1);
    for (int c = 0; c < 3; c++) {
        const T* cs = crse + c * Lc.S;
        // C(a, b, d): coarse value at (a ? I1 : I, b ? J1 : J, d ? K1 : K)
        auto C = [&](int a, int b, int d) -> T {
            const long long r = b ? (d ? r11 : r10) : (d ? r01 : r00);
            return __ldg(cs + r + (a ? I1 : I));
        };
        T te, to = (T)0;
        if (ej && ek) {
            te = C(0, 0, 0);
            if (two) to = (T)0.5 * (C(0, 0, 0) + C(1, 0, 0));
        } else if (ek) {
            te = (T)0.5 * (C(0, 0, 0) + C(0, 1, 0));
            if (two) to = (T)0.25 * (C(0, 0, 0) + C(1, 0, 0) + C(0, 1, 0) + C(1, 1, 0));
        } else if (ej) {
            te = (T)0.5 * (C(0, 0, 0) + C(0, 0, 1));
            if (two) to = (T)0.25 * (C(0, 0, 0) + C(0, 0, 1) + C(1, 0, 0) + C(1, 0, 1));
        } else {
            te = (T)0.25 * (C(0, 0, 0) + C(0, 1, 0) + C(0, 0, 1) + C(0, 1, 1));
            if (two)
                to = (T)0.125 * (C(0, 0, 0) + C(1, 0, 0) + C(0, 1, 0) + C(0, 0, 1) + C(0, 1, 1) + C(1, 0, 1) +
                                 C(1, 1, 0) + C(1, 1, 1));
        }
        T* o = fine + c * Lf.S + q;
        if (two) {
            typedef typename Pair<T>::type V;
            V v;
            if (assign) {
                v.x = te;
                v.y = to;
            } else {
                v = *reinterpret_cast<const V*>(o);
                v.x = v.x + te;
                v.y = v.y + to;
            }
            *reinterpret_cast<V*>(o) = v;
        } else {
            *o = assign ? te : (*o + te);
        }
    }
}

template <typename T>
__global__ void k_avg_ddw(LevelDesc Lf, LevelDesc Lc, const T* __restrict__ fine, T* __restrict__ crse, int ncoef)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z * blockDim.z + threadIdx.z;
    if (I >= Lc.nn[0] || J >= Lc.nn[1] || K >= Lc.nn[2]) return;
    const bool bI = !Lc.per[0] && (I == 0 || I == Lc.n[0]);
    const bool bJ = !Lc.per[1] && (J == 0 || J == Lc.n[1]);
    const bool bK = !Lc.per[2] && (K == 0 || K == Lc.n[2]);
    const long long q = Lc.idx(I, J, K);
    for (int m = 0; m < ncoef; m++) {
        const T* src = fine + m * Lf.S;
        auto f = [&](int a, int b, int d) -> T {
            return src[Lf.idx(wrapn(2 * I + a, Lf.n[0], Lf.per[0]), wrapn(2 * J + b, Lf.n[1], Lf.per[1]),
                              wrapn(2 * K + d, Lf.n[2], Lf.per[2]))];
        };
        crse[m * Lc.S + q] = full_weight<T>(f, bI, bJ, bK);
    }
}

template <typename TD, typename TS>
__global__ void k_convert(long long n, const TS* __restrict__ src, TD* __restrict__ dst, double scale)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        dst[e] = (TD)((double)src[e] * scale);
}

template <typename T>
__global__ void k_axpy(long long n, T* __restrict__ y, const T* __restrict__ x, T a)
{
    pdl_entry();
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        y[e] += a * x[e];
}

template <typename T> struct MaxSlot;
template <> struct MaxSlot<double> {
    static __device__ void put(void* s, double v) { atomicMax((unsigned long long*)s, (unsigned long long)__double_as_longlong(v)); }
};
template <> struct MaxSlot<float> {
    static __device__ void put(void* s, float v) { atomicMax((unsigned int*)s, __float_as_uint(v)); }
};

template <typename T>
__global__ void k_norm_inf(long long n, const T* __restrict__ x, void* slot)
{
    pdl_entry();
    T m = 0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const T a = fabs(x[e]);
        m = (a > m || a != a) ? a : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const T w = __shfl_xor_sync(0xffffffffu, m, o);
        m = (w > m || w != w) ? w : m;
    }
    if ((threadIdx.x & 31) == 0) MaxSlot<T>::put(slot, m);
}

// Reference nodal box (n+1 nodes per direction) -> padded storage, for the
// k-planes [k0, k0+kc).  With `chunk`, src holds only those planes (a staging
// slab); otherwise src is the whole box.
template <typename TD, typename TS>
__global__ void k_import(LevelDesc L, int ncomp, const TS* __restrict__ src, TD* __restrict__ dst, int aos, int k0,
                         int kc, int chunk)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = k0 + blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= L.nn[0] || j >= L.nn[1] || k >= L.nn[2] || k >= k0 + kc) return;
    const long long planeN = (long long)(L.n[0] + 1) * (L.n[1] + 1);
    const long long Nsrc = chunk ? planeN * kc : planeN * (L.n[2] + 1);
    const long long s = (long long)i + (long long)(L.n[0] + 1) * j + planeN * (chunk ? k - k0 : k);
    const long long q = L.idx(i, j, k);
    for (int c = 0; c < ncomp; c++) dst[c * L.S + q] = (TD)(aos ? src[s * ncomp + c] : src[c * Nsrc + s]);
}

// The same for interleaved (AoS) sources, through shared memory: a warp
// copies the contiguous 32 x ncomp source values of 32 consecutive nodes of a
// row into shared memory (coalesced), then writes each component's 32 values
// (coalesced).  Block (32, 8): one row segment per warp.
template <typename TD, typename TS>
__global__ void __launch_bounds__(256) k_import_aos(LevelDesc L, int ncomp, const TS* __restrict__ src,
                                                   TD* __restrict__ dst, int k0, int kc, int chunk)
{
    extern __shared__ __align__(16) unsigned char imp_raw[];
    TS* buf = reinterpret_cast<TS*>(imp_raw) + threadIdx.y * 32 * ncomp;
    const int lane = threadIdx.x;
    const long long r = (long long)blockIdx.y * blockDim.y + threadIdx.y;   // (j, k) row of the chunk
    const int j = (int)(r % L.nn[1]);
    const int k = k0 + (int)(r / L.nn[1]);
    const int i0 = blockIdx.x * 32;
    if (k >= k0 + kc || k >= L.nn[2]) return;   // uniform over the warp
    const int cnt = min(32, L.nn[0] - i0);
    const long long planeN = (long long)(L.n[0] + 1) * (L.n[1] + 1);
    const long long sb = ((long long)i0 + (long long)(L.n[0] + 1) * j + planeN * (chunk ? k - k0 : k)) * ncomp;
    for (int t = lane; t < cnt * ncomp; t += 32) buf[t] = src[sb + t];
    __syncwarp();
    if (lane < cnt) {
        const long long q = L.idx(i0 + lane, j, k);
        for (int c = 0; c < ncomp; c++) dst[c * L.S + q] = (TD)buf[lane * ncomp + c];
    }
}

// padded storage -> reference nodal box for planes [k0, k0+kc) (periodic images filled)
template <typename TD, typename TS>
__global__ void k_export(LevelDesc L, int ncomp, const TS* __restrict__ src, TD* __restrict__ dst, int aos, int k0,
                         int kc, int chunk)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = k0 + blockIdx.z * blockDim.z + threadIdx.z;
    if (i > L.n[0] || j > L.n[1] || k > L.n[2] || k >= k0 + kc) return;
    const long long planeN = (long long)(L.n[0] + 1) * (L.n[1] + 1);
    const long long Ndst = chunk ? planeN * kc : planeN * (L.n[2] + 1);
    const long long s = (long long)i + (long long)(L.n[0] + 1) * j + planeN * (chunk ? k - k0 : k);
    const int ii = (L.per[0] && i == L.n[0]) ? 0 : i;
    const int jj = (L.per[1] && j == L.n[1]) ? 0 : j;
    const int kk = (L.per[2] && k == L.n[2]) ? 0 : k;
    const long long q = L.idx(ii, jj, kk);
    for (int c = 0; c < ncomp; c++) {
        const TD v = (TD)src[c * L.S + q];
        if (aos) dst[s * ncomp + c] = v;
        else dst[c * Ndst + s] = v;
    }
}

// The first damped-Jacobi sweep from x = 0: A 0 = 0 in every row (interior,
// displacement, traction and Neumann rows alike), so x + omega (b - A x) / D
// is omega (b / D) node by node -- the sweep kernels' expression with x = 0,
// equal to theirs up to the sign of a zero.
template <typename T>
__global__ void k_jacobi_zero(long long n, T* __restrict__ out, const T* __restrict__ b, const T* __restrict__ dinv,
                              T omega)
{
    pdl_entry();
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        out[e] = omega * (b[e] * dinv[e]);
}

// y += a * x with x in FP32, y in FP64 (refinement accumulation)
__global__ void k_axpy_mixed(long long n, double* __restrict__ y, const float* __restrict__ x, double a)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        y[e] += a * (double)x[e];
}

// d <- 1/d in place (0 stays 0: padding)
__global__ void k_recip_inplace(long long n, float* __restrict__ d)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        d[e] = d[e] != 0.0f ? 1.0f / d[e] : 0.0f;
}

template <typename TD>
__global__ void k_recip(long long n, const double* __restrict__ d, TD* __restrict__ r)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        r[e] = d[e] != 0.0 ? (TD)(1.0 / d[e]) : (TD)0;
}

// per-component sums over the stored nodes (sums[0..2], accumulated) or, with
// `subtract`, x -= sums / count: the zero-mean normalization of a fully
// periodic box's displacement
template <typename T>
__global__ void k_mean3(LevelDesc L, T* __restrict__ x, double* __restrict__ sums, int subtract, void* norm_slot)
{
    pdl_entry();
    const long long cnt = L.count();
    double s[3] = {0, 0, 0};
    T m = 0;
    T mean[3] = {0, 0, 0};
    if (subtract)
        for (int c = 0; c < 3; c++) mean[c] = (T)(sums[c] / (double)cnt);
    const bool small = cnt <= 0x7fffffffLL;   // 32-bit index arithmetic
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        if (small) {
            const int ei = (int)e;
            i = ei % L.nn[0];
            j = (ei / L.nn[0]) % L.nn[1];
            k = ei / (L.nn[0] * L.nn[1]);
        } else {
            i = (int)(e % L.nn[0]);
            j = (int)((e / L.nn[0]) % L.nn[1]);
            k = (int)(e / ((long long)L.nn[0] * L.nn[1]));
        }
        const long long q = L.idx(i, j, k);
        for (int c = 0; c < 3; c++) {
            if (subtract) {
                const T v = x[c * L.S + q] - mean[c];
                x[c * L.S + q] = v;
                const T a = fabs(v);
                m = (a > m || a != a) ? a : m;
            } else s[c] += (double)x[c * L.S + q];
        }
    }
    if (subtract) {
        if (!norm_slot) return;
        for (int o = 16; o > 0; o >>= 1) {
            const T w = __shfl_xor_sync(0xffffffffu, m, o);
            m = (w > m || w != w) ? w : m;
        }
        if ((threadIdx.x & 31) == 0) MaxSlot<T>::put(norm_slot, m);
        return;
    }
    for (int c = 0; c < 3; c++) {
        double v = s[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&sums[c], v);
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline int blocks_1d(long long n)
{
    long long b = (n + 255) / 256;
    const long long cap = 16LL * sm_count();
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

template <typename T>
void launch_restriction(cudaStream_t st, const LevelDesc& Lf, const LevelDesc& Lc, const T* fine, T* crse, int ncomp)
{
    dim3 blk(32, 4, 2);
    pdl_launch(k_restrict<T>, grid_for(Lc, blk), blk, 0, st, Lf, Lc, fine, crse, ncomp); count_launch();
}

template <typename T>
void launch_interpolation(cudaStream_t st, const LevelDesc& Lf, const LevelDesc& Lc, T* fine, const T* crse,
                          bool assign)
{
    dim3 blk(32, 4, 2);
    // one thread per fine pair (2I, 2I+1) of a row
    const dim3 grd(((Lf.nn[0] + 1) / 2 + blk.x - 1) / blk.x, (Lf.nn[1] + blk.y - 1) / blk.y,
                   (Lf.nn[2] + blk.z - 1) / blk.z);
    pdl_launch(k_interp<T>, grd, blk, 0, st, Lf, Lc, fine, crse, assign ? 1 : 0); count_launch();
}

template <typename T>
void launch_average_ddw(cudaStream_t st, const LevelDesc& Lf, const LevelDesc& Lc, const T* fine, T* crse, int ncoef)
{
    dim3 blk(32, 4, 2);
    k_avg_ddw<T><<<grid_for(Lc, blk), blk, 0, st>>>(Lf, Lc, fine, crse, ncoef); count_launch();
}

template <typename TD, typename TS>
void launch_convert(cudaStream_t st, const LevelDesc& L, int ncomp, const TS* src, TD* dst, double scale)
{
    const long long n = (long long)ncomp * L.S;
    k_convert<TD, TS><<<blocks_1d(n), 256, 0, st>>>(n, src, dst, scale); count_launch();
}

template <typename T>
void launch_axpy(cudaStream_t st, const LevelDesc& L, int ncomp, T* y, const T* x, T a)
{
    const long long n = (long long)ncomp * L.S;
    pdl_launch(k_axpy<T>, dim3(blocks_1d(n)), dim3(256), 0, st, n, y, x, a); count_launch();
}

template <typename T>
void launch_jacobi_zero(cudaStream_t st, const LevelDesc& L, int ncomp, T* out, const T* b, const T* dinv, T omega)
{
    const long long n = (long long)ncomp * L.S;
    pdl_launch(k_jacobi_zero<T>, dim3(blocks_1d(n)), dim3(256), 0, st, n, out, b, dinv, omega); count_launch();
}

template <typename T>
void launch_zero(cudaStream_t st, const LevelDesc& L, int ncomp, T* y)
{
    cudaMemsetAsync(y, 0, sizeof(T) * (size_t)ncomp * (size_t)L.S, st);
}

template <typename T>
void launch_norm_inf(cudaStream_t st, const LevelDesc& L, int ncomp, const T* x, void* slot)
{
    const long long n = (long long)ncomp * L.S;
    pdl_launch(k_norm_inf<T>, dim3(blocks_1d(n)), dim3(256), 0, st, n, x, slot); count_launch();
}

template <typename TD, typename TS>
void launch_import(cudaStream_t st, const LevelDesc& L, int ncomp, const TS* src, TD* dst, bool aos, int k0, int kc,
                   bool chunk)
{
    if (aos && ncomp > 1 && ncomp <= 21) {
        const dim3 blk(32, 8);
        const long long rows = (long long)L.nn[1] * std::min(kc, L.nn[2] - k0);
        const dim3 grd((L.nn[0] + 31) / 32, (unsigned)((rows + 7) / 8));
        const size_t smem = 8 * 32 * (size_t)ncomp * sizeof(TS);
        k_import_aos<TD, TS><<<grd, blk, smem, st>>>(L, ncomp, src, dst, k0, kc, chunk ? 1 : 0);
        count_launch();
        return;
    }
    dim3 blk(32, 4, 2);
    dim3 grd((L.nn[0] + blk.x - 1) / blk.x, (L.nn[1] + blk.y - 1) / blk.y, (kc + blk.z - 1) / blk.z);
    k_import<TD, TS><<<grd, blk, 0, st>>>(L, ncomp, src, dst, aos ? 1 : 0, k0, kc, chunk ? 1 : 0); count_launch();
}

template <typename TD, typename TS>
void launch_export(cudaStream_t st, const LevelDesc& L, int ncomp, const TS* src, TD* dst, bool aos, int k0, int kc,
                   bool chunk)
{
    dim3 blk(32, 4, 2);
    dim3 grd((L.n[0] + 1 + blk.x - 1) / blk.x, (L.n[1] + 1 + blk.y - 1) / blk.y, (kc + blk.z - 1) / blk.z);
    k_export<TD, TS><<<grd, blk, 0, st>>>(L, ncomp, src, dst, aos ? 1 : 0, k0, kc, chunk ? 1 : 0); count_launch();
}

template <typename T>
void launch_remove_mean(cudaStream_t st, const LevelDesc& L, T* x, double* sums3, void* norm_slot)
{
    cudaMemsetAsync(sums3, 0, 3 * sizeof(double), st);
    const int g = blocks_1d(L.count());
    pdl_launch(k_mean3<T>, dim3(g), dim3(256), 0, st, L, x, sums3, 0, (void*)nullptr);
    count_launch();
    pdl_launch(k_mean3<T>, dim3(g), dim3(256), 0, st, L, x, sums3, 1, norm_slot);
    count_launch();
}

// sum x y (w == nullptr) or sum x y w^2
__global__ void k_dot(long long n, const double* __restrict__ x, const double* __restrict__ y,
                      const double* __restrict__ w, double* __restrict__ out)
{
    double s = 0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        s += w ? x[e] * y[e] * (w[e] * w[e]) : x[e] * y[e];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

void launch_dot(cudaStream_t st, long long n, const double* x, const double* y, double* out, const double* w)
{
    k_dot<<<blocks_1d(n), 256, 0, st>>>(n, x, y, w, out);
    count_launch();
}

// ---------------------------------------------------------------------------
// Vector kernels of the inner FP32 GCR (flexible, weighted inner product
// <a, b> = sum a b d^2 with d = 1/diag: the rows of the operator scaled to a
// unit diagonal, so that displacement, traction and interior rows weigh
// alike).  All scalars stay on the device; sums accumulate in FP64.
// ---------------------------------------------------------------------------

// out[i] += sum_e x[e] v_i[e] d[e]^2, i < k (out zeroed by the caller).  Each
// thread sums its elements in FP32 (a few dozen terms; FP64 arithmetic per
// element would bind on GB300's FP64 rate); threads, warps and blocks are
// combined in FP64.
template <int K>
__global__ void __launch_bounds__(256) k_multidot_w(long long n, const float* __restrict__ x, GcrVecs V,
                                                    const float* __restrict__ d, double* __restrict__ out)
{
    pdl_entry();
    float acc[K];
#pragma unroll
    for (int i = 0; i < K; i++) acc[i] = 0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float dd = d[e];
        const float xw = x[e] * dd * dd;
#pragma unroll
        for (int i = 0; i < K; i++) acc[i] += xw * V.v[i][e];
    }
    __shared__ double red[8][K];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int k = K;
#pragma unroll
    for (int i = 0; i < K; i++) {
        double a = (double)acc[i];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) red[warp][i] = a;
    }
    __syncthreads();
    if (threadIdx.x < k) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w][threadIdx.x];
        atomicAdd(out + threadIdx.x, t);
    }
}

// w -= sum_i beta_i W_i and z -= sum_i beta_i Z_i, i < K (classical Gram-Schmidt step)
template <int K>
__global__ void k_gcr_orth(long long n, const double* __restrict__ beta, GcrVecs W, GcrVecs Z,
                           float* __restrict__ w, float* __restrict__ z)
{
    pdl_entry();
    float b[K];
#pragma unroll
    for (int i = 0; i < K; i++) b[i] = (float)beta[i];
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        float tw = w[e], tz = z[e];
#pragma unroll
        for (int i = 0; i < K; i++) {
            tw -= b[i] * W.v[i][e];
            tz -= b[i] * Z.v[i][e];
        }
        w[e] = tw;
        z[e] = tz;
    }
}

// With ww = <w, w> and rw = <r, w> (dots[0], dots[1]): w, z scaled to unit
// norm, c += (rw / ww) z, r -= (rw / ww) w, and max |r| after it -> slot.
__global__ void k_gcr_step(long long n, const double* __restrict__ dots, float* __restrict__ w,
                           float* __restrict__ z, float* __restrict__ c, float* __restrict__ r, void* slot)
{
    pdl_entry();
    const double ww = dots[0], rw = dots[1];
    const float inv = ww > 0 ? (float)(1.0 / sqrt(ww)) : 0.0f;
    const float a = ww > 0 ? (float)(rw / sqrt(ww)) : 0.0f;   // coefficient of the unit direction
    float m = 0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float wu = w[e] * inv, zu = z[e] * inv;
        w[e] = wu;
        z[e] = zu;
        c[e] += a * zu;
        const float rn = r[e] - a * wu;
        r[e] = rn;
        const float t = fabsf(rn);
        m = (t > m || t != t) ? t : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float q = __shfl_xor_sync(0xffffffffu, m, o);
        m = (q > m || q != q) ? q : m;
    }
    if ((threadIdx.x & 31) == 0) MaxSlot<float>::put(slot, m);
}

void launch_multidot_w(cudaStream_t st, long long n, int k, const float* x, const GcrVecs& V, const float* d,
                       double* out)
{
    const int nb = blocks_1d(n);
    switch (k) {
#define K_(K) case K: pdl_launch(k_multidot_w<K>, dim3(nb), dim3(256), 0, st, n, x, V, d, out); break;
        K_(1) K_(2) K_(3) K_(4) K_(5) K_(6) K_(7) K_(8) K_(9) K_(10) K_(11) K_(12) K_(13) K_(14) K_(15) K_(16)
#undef K_
    default: return;
    }
    count_launch();
}

void launch_gcr_orth(cudaStream_t st, long long n, int k, const double* beta, const GcrVecs& W, const GcrVecs& Z,
                     float* w, float* z)
{
    const int nb = blocks_1d(n);
    switch (k) {
#define K_(K) case K: pdl_launch(k_gcr_orth<K>, dim3(nb), dim3(256), 0, st, n, beta, W, Z, w, z); break;
        K_(1) K_(2) K_(3) K_(4) K_(5) K_(6) K_(7) K_(8) K_(9) K_(10) K_(11) K_(12) K_(13) K_(14) K_(15) K_(16)
#undef K_
    default: return;
    }
    count_launch();
}

void launch_gcr_step(cudaStream_t st, long long n, const double* dots, float* w, float* z, float* c, float* r,
                     void* slot)
{
    pdl_launch(k_gcr_step, dim3(blocks_1d(n)), dim3(256), 0, st, n, dots, w, z, c, r, slot);
    count_launch();
}

void launch_recip_inplace(cudaStream_t st, const LevelDesc& L, int ncomp, float* d)
{
    const long long n = (long long)ncomp * L.S;
    k_recip_inplace<<<blocks_1d(n), 256, 0, st>>>(n, d);
    count_launch();
}

void launch_axpy_mixed(cudaStream_t st, const LevelDesc& L, int ncomp, double* y, const float* x, double a)
{
    const long long n = (long long)ncomp * L.S;
    k_axpy_mixed<<<blocks_1d(n), 256, 0, st>>>(n, y, x, a); count_launch();
}

template <typename TD>
void launch_recip(cudaStream_t st, const LevelDesc& L, int ncomp, const double* d, TD* r)
{
    const long long n = (long long)ncomp * L.S;
    k_recip<TD><<<blocks_1d(n), 256, 0, st>>>(n, d, r); count_launch();
}

#define INST(T)                                                                                              \
    template void launch_restriction<T>(cudaStream_t, const LevelDesc&, const LevelDesc&, const T*, T*, int); \
    template void launch_interpolation<T>(cudaStream_t, const LevelDesc&, const LevelDesc&, T*, const T*, bool); \
    template void launch_average_ddw<T>(cudaStream_t, const LevelDesc&, const LevelDesc&, const T*, T*, int); \
    template void launch_axpy<T>(cudaStream_t, const LevelDesc&, int, T*, const T*, T);                      \
    template void launch_zero<T>(cudaStream_t, const LevelDesc&, int, T*);                                   \
    template void launch_jacobi_zero<T>(cudaStream_t, const LevelDesc&, int, T*, const T*, const T*, T);     \
    template void launch_norm_inf<T>(cudaStream_t, const LevelDesc&, int, const T*, void*);                  \
    template void launch_recip<T>(cudaStream_t, const LevelDesc&, int, const double*, T*);                   \
    template void launch_remove_mean<T>(cudaStream_t, const LevelDesc&, T*, double*, void*);                 \
    template void launch_import<T, double>(cudaStream_t, const LevelDesc&, int, const double*, T*, bool, int, int, bool); \
    template void launch_import<T, float>(cudaStream_t, const LevelDesc&, int, const float*, T*, bool, int, int, bool);   \
    template void launch_export<T, double>(cudaStream_t, const LevelDesc&, int, const double*, T*, bool, int, int, bool); \
    template void launch_export<T, float>(cudaStream_t, const LevelDesc&, int, const float*, T*, bool, int, int, bool);
INST(double)
INST(float)
#undef INST
template void launch_convert<float, double>(cudaStream_t, const LevelDesc&, int, const double*, float*, double);
template void launch_convert<double, float>(cudaStream_t, const LevelDesc&, int, const float*, double*, double);
template void launch_convert<double, double>(cudaStream_t, const LevelDesc&, int, const double*, double*, double);

}  // namespace agb
