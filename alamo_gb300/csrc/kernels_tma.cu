// kernels_tma.cu -- FP32 interior stencil sweep with TMA plane copies.
//
// Same tile, k-march and per-node arithmetic (stencil.cuh) as the cp.async
// kernel k_stencil_pipe, but each plane of the 32 x 8 column tile (+1 halo,
// 36 x 10 elements) is brought into shared memory by two tensor copies
// (cp.async.bulk.tensor.4d: one box of the 3 displacement components, one
// box of the 2 or 21 modulus planes) issued by a producer warp and completed
// on an mbarrier, so the threads that compute spend no instructions on
// address arithmetic for the copies.  u planes live in a ring of 4 slots,
// moduli in a ring of 3; fill f brings plane k0-1+f (moduli from f = 1) and
// completes on the full barrier f % 4.  The slots fill f + 4 overwrites are
// released on the empty barrier f % 4 by each computing warp when it has
// finished plane k0+f, so warps never wait for one another plane by plane.
// Every wait on a barrier is bounded: after a wait runs out the thread stops
// waiting, the CTA's results are void, *err is set, and the producer waits
// (again bounded) for the copies it issued before the CTA exits.
//
// Tensor maps (one per array and level, cached by address) describe the
// padded level layout as a 4-D tensor (i, j, k, component) with strides
// (P, P nn1, S) elements; the box is (36, 10, 1, ncomp) and starts at
// i = 32 t, so every copy starts on a 16-byte boundary.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include "agb_internal.h"
#include "stencil.cuh"
#include "tma.cuh"

namespace agb {

namespace {

constexpr int TT_X = 32, TT_Y = 8, TT_Z = 16;      // tile and the default longest k-chunk
constexpr int TH_Y = TT_Y + 2, TW = 36;             // halo rows, halo row width (9 x 16 bytes)
constexpr int TU = 4, TC = 3;                       // ring depths

template <int NCOMP> struct SlotSize {
    // floats per slot, padded so every slot starts on a 128-byte boundary
    static constexpr int value = ((NCOMP * TH_Y * TW * 4 + 127) / 128) * 128 / 4;
};

template <int SYM> struct TmaLayout {
    static constexpr int NC = NCoef<SYM>::value;
    static constexpr int USLOT = SlotSize<3>::value;
    static constexpr int CSLOT = SlotSize<NC>::value;
    static constexpr int UBYTES = 3 * TH_Y * TW * 4;    // bytes one u box writes
    static constexpr int CBYTES = NC * TH_Y * TW * 4;   // bytes one modulus box writes
    static constexpr int C_OFF = TU * USLOT;             // floats
    static constexpr int BAR_OFF_BYTES = (C_OFF + TC * CSLOT) * 4;
    static constexpr int SMEM = BAR_OFF_BYTES + 2 * TU * 8 + 128;   // full + empty barriers, room to align the base
};

struct TmaAcc {
    const float* um;  // u slots of planes k-1, k, k+1
    const float* uk;
    const float* up;
    const float* c0;  // modulus slots of planes k, k+1
    const float* cp;
    int tx, ty;
    float cm[21];     // modulus at (i, j, k-1)
    __device__ __forceinline__ float u(int p, int di, int dj, int dk) const
    {
        const float* s = dk < 0 ? um : (dk > 0 ? up : uk);
        return s[(p * TH_Y + ty + dj) * TW + tx + di];
    }
    __device__ __forceinline__ float C(int m, int di, int dj, int dk) const
    {
        if (dk < 0) return cm[m];
        if (dk > 0) return cp[(m * TH_Y + ty) * TW + tx];
        return c0[(m * TH_Y + ty + dj) * TW + tx + di];
    }
};

// The CTA is 8 warps of interior nodes (one per tile row), a ninth, the face
// warp, and a tenth, the producer (its lane 0 issues the copies).  In the
// CTAs of the first and last column of tiles the face warp's lanes 0-7 and
// 8-15 take the x = 0 and x = n0 face nodes of the tile's rows, whose data
// (columns 0-1 and n0-1..n0 of the halo box) are in shared memory with the
// plane; every other node of the boundary shell is left to k_stencil_shell,
// whose remaining nodes (the z planes and the y rows) are contiguous in memory.
constexpr int TMA_WARPS = TT_Y + 2;   // 8 interior + face + producer
template <int SYM, int MODE>
__global__ void __launch_bounds__(TT_X* TMA_WARPS, 2)
    k_stencil_tma(LevelDesc L, Geo<float> g, int uniform, const __grid_constant__ CUtensorMap tmx,
                  const __grid_constant__ CUtensorMap tmc, const float* __restrict__ ddw, const float* __restrict__ b,
                  const float* __restrict__ dinv, float* __restrict__ out, float omega, void* norm_slot, int* err,
                  int kz, const BCTable bc)
{
    pdl_entry();
    typedef TmaLayout<SYM> Lay;
    constexpr int NC = Lay::NC;
    constexpr int CONSUMERS = TT_Y + 1;   // warps that compute (and release slots)
    extern __shared__ __align__(128) unsigned char tsm_raw[];
    float* tsm = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(tsm_raw) + 127) & ~(uintptr_t)127);
    const uint32_t full0 = smem_u32(reinterpret_cast<unsigned char*>(tsm) + Lay::BAR_OFF_BYTES);
    const uint32_t empty0 = full0 + 8 * TU;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + TT_X * ty;
    const int i0 = 1 + blockIdx.x * TT_X, j0 = 1 + blockIdx.y * TT_Y;
    const int k0 = 1 + blockIdx.z * kz;
    const int k1 = min(k0 + kz, L.n[2]);   // exclusive
    const int i = i0 + tx, j = j0 + ty;
    const bool producer = ty == TT_Y + 1;
    const bool face_warp = ty == TT_Y;
    const bool mine = ty < TT_Y && (i < L.n[0]) && (j < L.n[1]);
    // face warp: lane -> (side, row); the node (fi, fj, k) sits at column fcol of the halo box
    const int fside = tx >> 3, frow = tx & 7;
    const bool fmine = face_warp && tx < 16 && j0 + frow < L.n[1] &&
                       (fside == 0 ? blockIdx.x == 0 : blockIdx.x == gridDim.x - 1);
    const int fi = fside == 0 ? 0 : L.n[0];
    const int fcol = fi - (i0 - 1);
    const long long S = L.S;
    const int nfill = k1 - k0 + 2;            // fills 0 .. k1-k0+1 (planes k0-1 .. k1)

    if (tid == 0) {
        for (int s = 0; s < TU; s++) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, CONSUMERS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    float nrm = 0;
    if (producer) {
        // fill f: u plane k0-1+f -> u slot f%4; moduli plane k0-1+f -> c slot
        // (f-1)%3 (f >= 1); full barrier f%4.  Fill f >= 4 reuses the slots of
        // plane k0+f-5 (u) and k0+f-4 (moduli), free once every computing warp
        // has finished iteration f-4 (empty barrier f%4, its (f/4-1)-th phase).
        if (tx == 0) {
            bool ok = true;
            int issued = 0;
            for (int f = 0; f < nfill; f++) {
                if (f >= TU) {
                    ok = mbar_wait(empty0 + 8 * (f % TU), (uint32_t)(((f / TU) - 1) & 1));
                    if (!ok) break;
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                }
                const uint32_t bar = full0 + 8 * (f % TU);
                const bool withc = f >= 1;
                mbar_expect(bar, Lay::UBYTES + (withc ? Lay::CBYTES : 0));
                const int x0 = i0 - 1, y0 = j0 - 1, z = k0 - 1 + f;
                tma_load4(smem_u32(tsm + (f % TU) * Lay::USLOT), &tmx, x0, y0, z, 0, bar);
                if (withc) tma_load4(smem_u32(tsm + Lay::C_OFF + ((f - 1) % TC) * Lay::CSLOT), &tmc, x0, y0, z, 0, bar);
                issued = f + 1;
            }
            if (!ok) atomicExch(err, 1);
            // the CTA's shared memory must outlive the copies: wait (bounded)
            // for the last fills, which complete after all earlier ones
            for (int f = max(0, issued - TU); f < issued; f++)
                mbar_wait(full0 + 8 * (f % TU), (uint32_t)((f / TU) & 1));
        }
    } else {
        TmaAcc acc;
        acc.tx = tx + 1;
        acc.ty = ty + 1;
        if (mine) {
            const long long p = L.idx(i, j, k0 - 1);
#pragma unroll
            for (int m = 0; m < NC; m++) acc.cm[m] = __ldg(ddw + m * S + p);
        }
        int waited = 0;     // fills known complete
        // b and 1/D of the first two planes; later planes are fetched two planes ahead
        float bq[3] = {0, 0, 0}, dq[3] = {0, 0, 0};
        auto fetch = [&](int k, float* bb, float* dd) {
            if (!mine || k >= k1) return;
            const long long q = L.idx(i, j, k);
            if (MODE != MODE_APPLY)
#pragma unroll
                for (int c = 0; c < 3; c++) bb[c] = __ldg(b + c * S + q);
            if (MODE == MODE_JACOBI)
#pragma unroll
                for (int c = 0; c < 3; c++) dd[c] = __ldg(dinv + c * S + q);
        };
        float bn[3] = {0, 0, 0}, dn[3] = {0, 0, 0};
        fetch(k0, bq, dq);
        fetch(k0 + 1, bn, dn);
        for (int k = k0; k < k1; k++) {
            const int it = k - k0;
            const long long q = mine ? L.idx(i, j, k) : 0;
            float bnn[3] = {0, 0, 0}, dnn[3] = {0, 0, 0};
            fetch(k + 2, bnn, dnn);
            // planes k-1, k, k+1 = fills it, it+1, it+2
            bool good = true;
            for (int f = waited; f <= it + 2 && good; f++)
                good = mbar_wait(full0 + 8 * (f % TU), (uint32_t)((f / TU) & 1));
            good = __all_sync(0xffffffffu, good);   // the warp leaves the loop together
            if (!good) {
                // a wait ran out: the CTA's results are void; stop here (the
                // producer's waits on this warp's releases run out in turn)
                atomicExch(err, 1);
                break;
            }
            waited = it + 3;
            acc.um = tsm + (it % TU) * Lay::USLOT;
            acc.uk = tsm + ((it + 1) % TU) * Lay::USLOT;
            acc.up = tsm + ((it + 2) % TU) * Lay::USLOT;
            acc.c0 = tsm + Lay::C_OFF + (it % TC) * Lay::CSLOT;
            acc.cp = tsm + Lay::C_OFF + ((it + 1) % TC) * Lay::CSLOT;
            if (fmine) {
                // an x-face node: its boundary row from the same plane slots
                TmaAcc fa = acc;
                fa.tx = fcol;
                fa.ty = frow + 1;
                int mn[3] = {fside == 0, 0, 0}, mx[3] = {fside == 1, 0, 0};
                float f[3];
                boundary_row<float, SYM>(fa, g, bc, mn, mx, f);
                const long long qf = L.idx(fi, j0 + frow, k);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const long long o = c * S + qf;
                    if (MODE == MODE_APPLY) {
                        out[o] = f[c];
                    } else if (MODE == MODE_RESID) {
                        const float r = __ldg(b + o) - f[c];
                        out[o] = r;
                        const float a = fabsf(r);
                        nrm = (a > nrm || a != a) ? a : nrm;
                    } else {
                        out[o] = fa.u(c, 0, 0, 0) + omega * ((__ldg(b + o) - f[c]) * __ldg(dinv + o));
                    }
                }
            }
            if (mine) {
                float f[3];
                interior_row<float, SYM>(acc, g, uniform != 0, f);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const long long o = c * S + q;
                    if (MODE == MODE_APPLY) {
                        out[o] = f[c];
                    } else if (MODE == MODE_RESID) {
                        const float r = bq[c] - f[c];
                        out[o] = r;
                        const float a = fabsf(r);
                        nrm = (a > nrm || a != a) ? a : nrm;
                    } else {
                        const float xc = acc.uk[(c * TH_Y + ty + 1) * TW + tx + 1];
                        out[o] = xc + omega * ((bq[c] - f[c]) * dq[c]);
                    }
                }
                // the modulus of plane k becomes plane k-1's for the next plane
#pragma unroll
                for (int m = 0; m < NC; m++) acc.cm[m] = acc.c0[(m * TH_Y + ty + 1) * TW + tx + 1];
            }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                bq[c] = bn[c];
                dq[c] = dn[c];
                bn[c] = bnn[c];
                dn[c] = dnn[c];
            }
            // this warp is done with the u slot of plane k-1 and the moduli
            // slot of plane k: release them for fill it+4
            __syncwarp();
            if (tx == 0) mbar_arrive(empty0 + 8 * (it % TU));
        }
    }
    if (MODE == MODE_RESID && norm_slot) {
        // block max -> slot (same encoding as the other stencil kernels)
        __shared__ float red[32];
        for (int o = 16; o > 0; o >>= 1) {
            const float w = __shfl_xor_sync(0xffffffffu, nrm, o);
            nrm = (w > nrm || w != w) ? w : nrm;
        }
        if ((tid & 31) == 0) red[tid >> 5] = nrm;
        __syncthreads();
        if (tid < 32) {
            float v = tid < (TT_X * TMA_WARPS) / 32 ? red[tid] : 0.0f;
            for (int o = 16; o > 0; o >>= 1) {
                const float w = __shfl_xor_sync(0xffffffffu, v, o);
                v = (w > v || w != w) ? w : v;
            }
            if (tid == 0) atomicMax((unsigned int*)norm_slot, __float_as_uint(v));
        }
    }
}

// ---------------------------------------------------------------------------
// tensor maps
// ---------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return (PFN_cuTensorMapEncodeTiled_v12000)p;
    }();
    return fn;
}

typedef std::tuple<const void*, int, int, int, long long, int> MapKey;
std::mutex g_map_mutex;
std::map<MapKey, CUtensorMap> g_maps;

bool plane_map(const float* base, const LevelDesc& L, int ncomp, CUtensorMap* out)
{
    const MapKey key(base, L.P, L.nn[1], L.nn[2], L.S, ncomp);
    std::lock_guard<std::mutex> lock(g_map_mutex);
    auto it = g_maps.find(key);
    if (it != g_maps.end()) {
        *out = it->second;
        return true;
    }
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return false;
    CUtensorMap m;
    const cuuint64_t dims[4] = {(cuuint64_t)L.P, (cuuint64_t)L.nn[1], (cuuint64_t)L.nn[2], (cuuint64_t)ncomp};
    const cuuint64_t strides[3] = {(cuuint64_t)L.P * 4, (cuuint64_t)L.P * L.nn[1] * 4, (cuuint64_t)L.S * 4};
    const cuuint32_t box[4] = {(cuuint32_t)TW, (cuuint32_t)TH_Y, 1, (cuuint32_t)ncomp};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = enc(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (void*)base, dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    g_maps[key] = m;
    *out = m;
    return true;
}

__device__ int g_tma_error = 0;
int* g_tma_error_addr = nullptr;   // device address, looked up at initialisation

}  // namespace

// The TMA kernel serves FP32 interiors unless AGB_STENCIL=pipe or =march.
bool use_tma_kernel()
{
    static bool v = [] {
        const char* s = getenv("AGB_STENCIL");
        return !(s && (s[0] == 'p' || s[0] == 'm'));
    }();
    return v;
}

bool tma_supported(const LevelDesc& L)
{
    // 16-byte aligned strides; box width inside the padded row (make_level guarantees
    // P >= last tile start + 36 when x is not periodic)
    return !L.per[0] && (L.P % 4) == 0 && (L.S % 4) == 0 && encode_fn() != nullptr;
}

template <int SYM, int MODE>
static bool launch_tma_sm(cudaStream_t st, const LevelDesc& L, const BCTable& bc, bool uniform, const float* ddw,
                          const float* x, const float* b, const float* dinv, float* out, float omega, void* norm_slot)
{
    CUtensorMap mx, mc;
    if (!plane_map(x, L, 3, &mx) || !plane_map(ddw, L, NCoef<SYM>::value, &mc)) return false;
    int* err = g_tma_error_addr;
    if (!err) return false;
    const Geo<float> g = make_geo<float>(L);
    dim3 blk(TT_X, TMA_WARPS, 1);
    // k-chunk: the longest (least halo re-read) up to TT_Z planes
    // (AGB_TMA_KZ_MAX) that still gives at least three waves of 2 CTAs on
    // each SM, and no shorter than 4 planes (AGB_TMA_KZ_MIN)
    const int cxy = ((L.n[0] - 1 + TT_X - 1) / TT_X) * ((L.n[1] - 1 + TT_Y - 1) / TT_Y);
    static const int kz_max = [] {
        const char* e = getenv("AGB_TMA_KZ_MAX");
        const int v = e ? atoi(e) : TT_Z;
        return v >= 1 && v <= 256 ? v : TT_Z;
    }();
    static const int kz_min = [] {
        const char* e = getenv("AGB_TMA_KZ_MIN");
        const int v = e ? atoi(e) : 4;
        return v >= 1 && v <= kz_max ? v : 4;
    }();
    int kz = kz_max;
    while (kz > kz_min && (long long)cxy * ((L.n[2] - 1 + kz - 1) / kz) < 3LL * 2 * sm_count()) kz /= 2;
    dim3 grd((L.n[0] - 1 + TT_X - 1) / TT_X, (L.n[1] - 1 + TT_Y - 1) / TT_Y, (L.n[2] - 1 + kz - 1) / kz);
    pdl_launch(k_stencil_tma<SYM, MODE>, grd, blk, (size_t)TmaLayout<SYM>::SMEM, st, L, g, uniform ? 1 : 0, mx, mc, ddw,
               b, dinv, out, omega, norm_slot, err, kz, bc);
    return true;   // the caller counts the launch
}

bool launch_stencil_tma(cudaStream_t st, int sym, int mode, const LevelDesc& L, const BCTable& bc, bool uniform,
                        const float* ddw, const float* x, const float* b, const float* dinv, float* out, float omega,
                        void* norm_slot)
{
#define TM(S, M) return launch_tma_sm<S, M>(st, L, bc, uniform, ddw, x, b, dinv, out, omega, norm_slot)
    if (sym == SYM_ISO) {
        if (mode == MODE_APPLY) TM(SYM_ISO, MODE_APPLY);
        if (mode == MODE_RESID) TM(SYM_ISO, MODE_RESID);
        TM(SYM_ISO, MODE_JACOBI);
    }
    if (mode == MODE_APPLY) TM(SYM_MM, MODE_APPLY);
    if (mode == MODE_RESID) TM(SYM_MM, MODE_RESID);
    TM(SYM_MM, MODE_JACOBI);
#undef TM
}

// Reads and clears the error flag the TMA kernels set when a wait runs out.
int tma_error_take()
{
    int v = 0, z = 0;
    if (cudaMemcpyFromSymbol(&v, g_tma_error, sizeof(int)) != cudaSuccess) return 0;
    if (v) cudaMemcpyToSymbol(g_tma_error, &z, sizeof(int));
    return v;
}

void init_tma_attributes()
{
    if (cudaGetSymbolAddress((void**)&g_tma_error_addr, g_tma_error) != cudaSuccess) g_tma_error_addr = nullptr;
    cudaFuncSetAttribute(k_stencil_tma<SYM_ISO, MODE_APPLY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TmaLayout<SYM_ISO>::SMEM);
    cudaFuncSetAttribute(k_stencil_tma<SYM_ISO, MODE_RESID>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TmaLayout<SYM_ISO>::SMEM);
    cudaFuncSetAttribute(k_stencil_tma<SYM_ISO, MODE_JACOBI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TmaLayout<SYM_ISO>::SMEM);
    cudaFuncSetAttribute(k_stencil_tma<SYM_MM, MODE_APPLY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TmaLayout<SYM_MM>::SMEM);
    cudaFuncSetAttribute(k_stencil_tma<SYM_MM, MODE_RESID>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TmaLayout<SYM_MM>::SMEM);
    cudaFuncSetAttribute(k_stencil_tma<SYM_MM, MODE_JACOBI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TmaLayout<SYM_MM>::SMEM);
}

}  // namespace agb
