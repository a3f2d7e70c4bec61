// kernels_conv.cu -- 3x3x3 convolutions of the learned preconditioner.
//
// Implicit GEMM on the tensor cores (mma.sync m16n8k16, BF16 operands, FP32
// accumulation) over node fields of a fully periodic box, channels last:
// a field is [voxel][CP] with voxel = x + n0 (y + n1 z) and CP channels
// (a multiple of 16; unused channels hold zeros).  Padding is periodic, so
// every tap of every voxel is defined.
//
//   forward   out[v][co] = act(bias[co] + sum_tap sum_ci in[v + off(tap)][ci] W[tap][co][ci])
//   data grad = forward of dY with the flipped, transposed weights (conv3_flip)
//   weight grad dW[tap][co][ci] += sum_v dY[v][co] in[v + off(tap)][ci]
//
// Tile: 16 x 4 x 2 voxels per CTA (8 warps, one 16-voxel x-row each) with a
// one-voxel halo staged in shared memory; shared rows are padded by 8
// elements so the ldmatrix row addresses of a warp fall in distinct banks.
// Box edges must be multiples of 16 (x), 4 (y) and 2 (z).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "agb.h"
#include "agb_internal.h"

namespace agb {
namespace {

constexpr int CX = 16, CY = 4, CZ = 2;            // voxel tile
constexpr int HX = CX + 2, HY = CY + 2, HZ = CZ + 2;
constexpr int HVOX = HX * HY * HZ;                // 432 halo voxels
constexpr int CONV_THREADS = 256;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2(uint32_t addr, uint32_t& r0, uint32_t& r1)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0, %1}, [%2];" : "=r"(r0), "=r"(r1) : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t addr, uint32_t& r0, uint32_t& r1)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0, %1}, [%2];" : "=r"(r0), "=r"(r1) : "r"(addr));
}
__device__ __forceinline__ void mma_bf16(float d[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

struct Grid3 {
    int n[3];
    __device__ __forceinline__ long long vox(int x, int y, int z) const
    {
        x = x < 0 ? x + n[0] : (x >= n[0] ? x - n[0] : x);
        y = y < 0 ? y + n[1] : (y >= n[1] ? y - n[1] : y);
        z = z < 0 ? z + n[2] : (z >= n[2] ? z - n[2] : z);
        return (long long)x + (long long)n[0] * (y + (long long)n[1] * z);
    }
};

// Stage the halo tile of `src` ([voxel][cp] BF16) at tile origin (x0,y0,z0)
// into dst[HVOX][cp + 8] with periodic wrap; 16-byte chunks.
__device__ __forceinline__ void stage_halo(__nv_bfloat16* dst, const __nv_bfloat16* __restrict__ src, const Grid3& G,
                                           int cp, int x0, int y0, int z0)
{
    const int cpr = cp / 8;   // chunks per voxel
    const int cs = cp + 8;
    for (int e = threadIdx.x; e < HVOX * cpr; e += blockDim.x) {
        const int h = e / cpr, c = e - h * cpr;
        const int hx = h % HX, hy = (h / HX) % HY, hz = h / (HX * HY);
        const long long v = G.vox(x0 - 1 + hx, y0 - 1 + hy, z0 - 1 + hz);
        const uint4 val = *reinterpret_cast<const uint4*>(src + v * cp + c * 8);
        *reinterpret_cast<uint4*>(dst + h * cs + c * 8) = val;
    }
}

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
template <int NT, typename OutT, bool RELU>
__global__ void __launch_bounds__(CONV_THREADS) k_conv3_fwd(Grid3 G, int cinp, const __nv_bfloat16* __restrict__ in,
                                                            const __nv_bfloat16* __restrict__ w,
                                                            const float* __restrict__ bias, OutT* __restrict__ out)
{
    constexpr int COUTP = NT * 8;
    extern __shared__ __align__(16) unsigned char csm[];
    const int cs = cinp + 8;
    __nv_bfloat16* xs = reinterpret_cast<__nv_bfloat16*>(csm);
    __nv_bfloat16* ws = xs + HVOX * cs;
    const int tiles_x = G.n[0] / CX, tiles_y = G.n[1] / CY;
    const int t = blockIdx.x;
    const int x0 = (t % tiles_x) * CX, y0 = ((t / tiles_x) % tiles_y) * CY, z0 = (t / (tiles_x * tiles_y)) * CZ;
    stage_halo(xs, in, G, cinp, x0, y0, z0);
    {
        const int cpr = cinp / 8;
        for (int e = threadIdx.x; e < 27 * COUTP * cpr; e += blockDim.x) {
            const int row = e / cpr, c = e - row * cpr;   // row = tap * COUTP + co
            *reinterpret_cast<uint4*>(ws + row * cs + c * 8) =
                *reinterpret_cast<const uint4*>(w + (long long)row * cinp + c * 8);
        }
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wy = warp % CY, wz = warp / CY;
    float acc[NT][4];
#pragma unroll
    for (int nt = 0; nt < NT; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[nt][q] = 0.f;
    const uint32_t xs0 = smem_addr(xs), ws0 = smem_addr(ws);
    const int arow = lane & 15, akoff = (lane >> 4) * 8;   // ldmatrix.x4 row / k offset of this lane
    const int brow = lane & 7, bkoff = ((lane >> 3) & 1) * 8;
    for (int tap = 0; tap < 27; tap++) {
        const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
        const int hbase = ((wz + 1 + dz) * HY + (wy + 1 + dy)) * HX + (1 + dx);
        for (int kc = 0; kc < cinp; kc += 16) {
            uint32_t a0, a1, a2, a3;
            ldsm_x4(xs0 + (uint32_t)(((hbase + arow) * cs + kc + akoff) * 2), a0, a1, a2, a3);
#pragma unroll
            for (int nt = 0; nt < NT; nt++) {
                uint32_t b0, b1;
                ldsm_x2(ws0 + (uint32_t)(((tap * COUTP + nt * 8 + brow) * cs + kc + bkoff) * 2), b0, b1);
                mma_bf16(acc[nt], a0, a1, a2, a3, b0, b1);
            }
        }
    }
    const int g = lane >> 2, c2 = (lane & 3) * 2;
    const int y = y0 + wy, z = z0 + wz;
#pragma unroll
    for (int nt = 0; nt < NT; nt++) {
        const int co = nt * 8 + c2;
        const float bb0 = bias ? bias[co] : 0.f, bb1 = bias ? bias[co + 1] : 0.f;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const long long v = G.vox(x0 + g + 8 * h, y, z);
            float v0 = acc[nt][2 * h] + bb0, v1 = acc[nt][2 * h + 1] + bb1;
            if (RELU) {
                v0 = fmaxf(v0, 0.f);
                v1 = fmaxf(v1, 0.f);
            }
            if (sizeof(OutT) == 4) {
                float* o = reinterpret_cast<float*>(out);
                o[v * COUTP + co] = v0;
                o[v * COUTP + co + 1] = v1;
            } else {
                __nv_bfloat162 pr = __floats2bfloat162_rn(v0, v1);
                *reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<__nv_bfloat16*>(out) + v * COUTP + co) = pr;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// weight gradient.  blockIdx.y selects a group of TG taps; each warp owns a
// fixed set of (tap, co tile, ci tile) output tiles of the group and keeps
// their accumulators across all voxel tiles the CTA visits (grid-stride),
// then adds them to dw with one atomic per element.
// ---------------------------------------------------------------------------
constexpr int WG_MAX_OWN = 12;   // output tiles per warp

template <int MT>
__global__ void __launch_bounds__(CONV_THREADS) k_conv3_wgrad(Grid3 G, int cinp, int tg,
                                                              const __nv_bfloat16* __restrict__ in,
                                                              const __nv_bfloat16* __restrict__ dy,
                                                              float* __restrict__ dw)
{
    constexpr int COUTP = MT * 16;
    extern __shared__ __align__(16) unsigned char csm[];
    const int cs = cinp + 8, ds = COUTP + 8;
    __nv_bfloat16* xs = reinterpret_cast<__nv_bfloat16*>(csm);
    __nv_bfloat16* ys = xs + HVOX * cs;
    const int NTc = cinp / 8;
    const int tap0 = blockIdx.y * tg, ntap = min(tg, 27 - tap0);
    const int ntiles_out = ntap * MT * NTc;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float acc[WG_MAX_OWN][4];
#pragma unroll
    for (int o = 0; o < WG_MAX_OWN; o++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[o][q] = 0.f;
    const int tiles_x = G.n[0] / CX, tiles_y = G.n[1] / CY;
    const int ntile = tiles_x * tiles_y * (G.n[2] / CZ);
    const uint32_t xs0 = smem_addr(xs), ys0 = smem_addr(ys);
    for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
        const int x0 = (t % tiles_x) * CX, y0 = ((t / tiles_x) % tiles_y) * CY, z0 = (t / (tiles_x * tiles_y)) * CZ;
        __syncthreads();   // previous tile's reads are done
        stage_halo(xs, in, G, cinp, x0, y0, z0);
        {
            const int cpr = COUTP / 8;
            for (int e = threadIdx.x; e < CX * CY * CZ * cpr; e += blockDim.x) {
                const int r = e / cpr, c = e - r * cpr;   // r = tile voxel (x fastest)
                const int lx = r % CX, ly = (r / CX) % CY, lz = r / (CX * CY);
                const long long v = G.vox(x0 + lx, y0 + ly, z0 + lz);
                *reinterpret_cast<uint4*>(ys + r * ds + c * 8) =
                    *reinterpret_cast<const uint4*>(dy + v * COUTP + c * 8);
            }
        }
        __syncthreads();
        // K loop: the 8 rows of 16 voxels of the tile
        for (int row = 0; row < CY * CZ; row++) {
            const int ry = row % CY, rz = row / CY;
            uint32_t a[MT][4];
            {
                // A = dY^T (co x voxel): ldmatrix.trans of the [voxel][co] rows
                const int mi = lane >> 3, r8 = lane & 7;
                const int vrow = row * CX + (mi >> 1) * 8 + r8;
#pragma unroll
                for (int mt = 0; mt < MT; mt++)
                    ldsm_x4_t(ys0 + (uint32_t)((vrow * ds + mt * 16 + (mi & 1) * 8) * 2), a[mt][0], a[mt][1],
                              a[mt][2], a[mt][3]);
            }
#pragma unroll
            for (int o = 0; o < WG_MAX_OWN; o++) {
                const int id = warp + 8 * o;
                if (id >= ntiles_out) break;
                const int tl = id / (MT * NTc), rem = id - tl * (MT * NTc);
                const int mt = rem / NTc, nt = rem - mt * NTc;
                const int tap = tap0 + tl;
                const int dx = tap % 3 - 1, dyy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
                const int hbase = ((rz + 1 + dz) * HY + (ry + 1 + dyy)) * HX + (1 + dx);
                // B = shifted input (voxel x ci): ldmatrix.trans of the [voxel][ci] rows
                const int r16 = lane & 15;
                uint32_t b0, b1;
                ldsm_x2_t(xs0 + (uint32_t)(((hbase + r16) * cs + nt * 8) * 2), b0, b1);
                uint32_t a0 = a[0][0], a1 = a[0][1], a2 = a[0][2], a3 = a[0][3];
                if (MT > 1 && mt == 1) {
                    a0 = a[MT - 1][0];
                    a1 = a[MT - 1][1];
                    a2 = a[MT - 1][2];
                    a3 = a[MT - 1][3];
                }
                mma_bf16(acc[o], a0, a1, a2, a3, b0, b1);
            }
        }
    }
    const int g = lane >> 2, c2 = (lane & 3) * 2;
#pragma unroll
    for (int o = 0; o < WG_MAX_OWN; o++) {
        const int id = warp + 8 * o;
        if (id >= ntiles_out) break;
        const int tl = id / (MT * NTc), rem = id - tl * (MT * NTc);
        const int mt = rem / NTc, nt = rem - mt * NTc;
        const int tap = tap0 + tl;
        const int ci = nt * 8 + c2;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int co = mt * 16 + g + 8 * h;
            float* p = dw + ((long long)tap * COUTP + co) * cinp + ci;
            atomicAdd(p, acc[o][2 * h]);
            atomicAdd(p + 1, acc[o][2 * h + 1]);
        }
    }
}

// db[co] += sum_v dy[v][co]
__global__ void k_bias_grad(long long nvox, int coutp, const __nv_bfloat16* __restrict__ dy, float* __restrict__ db)
{
    __shared__ float red[32];
    const int co = blockIdx.y;
    float s = 0.f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox; v += (long long)gridDim.x * blockDim.x)
        s += __bfloat162float(dy[v * coutp + co]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(db + co, s);
    }
}

// wt[26 - tap][ci][co] = w[tap][co][ci]  (data gradient = forward with wt)
__global__ void k_conv3_flip(int cinp, int coutp, const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 27 * cinp * coutp) return;
    const int tap = e / (coutp * cinp), rem = e - tap * coutp * cinp;
    const int co = rem / cinp, ci = rem - co * cinp;
    wt[((26 - tap) * cinp + ci) * coutp + co] = w[e];
}

// dy *= (y > 0), both BF16 [count]
__global__ void k_relu_bwd(long long count, const __nv_bfloat16* __restrict__ y, __nv_bfloat16* __restrict__ dy)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count; e += (long long)gridDim.x * blockDim.x)
        if (!(__bfloat162float(y[e]) > 0.f)) dy[e] = __float2bfloat16(0.f);
}

// Adam on FP32 master weights; the BF16 copy used by the kernels is refreshed.
__global__ void k_adam(long long count, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count; e += (long long)gridDim.x * blockDim.x) {
        const float gg = g[e];
        const float mm = b1 * m[e] + (1.f - b1) * gg;
        const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
        m[e] = mm;
        v[e] = vv;
        const float ww = w[e] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
        w[e] = ww;
        if (wb) wb[e] = __float2bfloat16(ww);
    }
}

int conv_blocks(long long n)
{
    const long long b = (n + 255) / 256;
    const long long cap = 8LL * sm_count();
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

bool conv_box_ok(const int n[3]) { return n[0] % CX == 0 && n[1] % CY == 0 && n[2] % CZ == 0 && n[0] > 0; }

size_t fwd_smem(int cinp, int coutp) { return (size_t)(HVOX + 27 * coutp) * (cinp + 8) * 2; }
size_t wgrad_smem(int cinp, int coutp) { return (size_t)HVOX * (cinp + 8) * 2 + (size_t)CX * CY * CZ * (coutp + 8) * 2; }

template <int NT, typename OutT, bool RELU> void set_fwd_attr()
{
    cudaFuncSetAttribute(k_conv3_fwd<NT, OutT, RELU>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

}  // namespace

void init_conv_attributes()
{
    set_fwd_attr<1, float, false>();
    set_fwd_attr<1, float, true>();
    set_fwd_attr<1, __nv_bfloat16, false>();
    set_fwd_attr<1, __nv_bfloat16, true>();
    set_fwd_attr<2, float, false>();
    set_fwd_attr<2, float, true>();
    set_fwd_attr<2, __nv_bfloat16, false>();
    set_fwd_attr<2, __nv_bfloat16, true>();
    set_fwd_attr<4, float, false>();
    set_fwd_attr<4, float, true>();
    set_fwd_attr<4, __nv_bfloat16, false>();
    set_fwd_attr<4, __nv_bfloat16, true>();
    set_fwd_attr<6, float, false>();
    set_fwd_attr<6, float, true>();
    set_fwd_attr<6, __nv_bfloat16, false>();
    set_fwd_attr<6, __nv_bfloat16, true>();
    cudaFuncSetAttribute(k_conv3_wgrad<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_conv3_wgrad<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

}  // namespace agb

using namespace agb;

static bool g_conv_init = false;

static agb_status conv_check(const int n[3], int cinp, int coutp)
{
    if (!n) {
        set_error("null n");
        return AGB_BADARG;
    }
    if (!conv_box_ok(n)) {
        set_error("conv3: box edges must be multiples of 16 (x), 4 (y), 2 (z)");
        return AGB_BADARG;
    }
    if (cinp < 16 || cinp > 64 || cinp % 16) {
        set_error("conv3: input channels must be 16, 32, 48 or 64");
        return AGB_BADARG;
    }
    if (!g_conv_init) {
        init_conv_attributes();
        g_conv_init = true;
    }
    return AGB_OK;
}

extern "C" agb_status agb_conv3_forward(const int n[3], int cinp, int coutp, const void* in, const void* w,
                                        const float* bias, void* out, int out_f32, int relu, void* stream)
{
    agb_status s = conv_check(n, cinp, coutp);
    if (s != AGB_OK) return s;
    if (coutp != 8 && coutp != 16 && coutp != 32 && coutp != 48) {
        set_error("conv3: output channels must be 8, 16, 32 or 48");
        return AGB_BADARG;
    }
    if (!in || !w || !out) {
        set_error("null argument");
        return AGB_BADARG;
    }
    Grid3 G{{n[0], n[1], n[2]}};
    const int ntile = (n[0] / CX) * (n[1] / CY) * (n[2] / CZ);
    const size_t sm = fwd_smem(cinp, coutp);
    if (sm > 200 * 1024) {
        set_error("conv3: layer too wide for shared memory");
        return AGB_BADARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const __nv_bfloat16* x = (const __nv_bfloat16*)in;
    const __nv_bfloat16* ww = (const __nv_bfloat16*)w;
#define FWD(NT)                                                                                                     \
    do {                                                                                                            \
        if (out_f32) {                                                                                              \
            if (relu) k_conv3_fwd<NT, float, true><<<ntile, CONV_THREADS, sm, st>>>(G, cinp, x, ww, bias, (float*)out); \
            else k_conv3_fwd<NT, float, false><<<ntile, CONV_THREADS, sm, st>>>(G, cinp, x, ww, bias, (float*)out);    \
        } else {                                                                                                    \
            if (relu)                                                                                               \
                k_conv3_fwd<NT, __nv_bfloat16, true><<<ntile, CONV_THREADS, sm, st>>>(G, cinp, x, ww, bias,          \
                                                                                     (__nv_bfloat16*)out);          \
            else                                                                                                    \
                k_conv3_fwd<NT, __nv_bfloat16, false><<<ntile, CONV_THREADS, sm, st>>>(G, cinp, x, ww, bias,         \
                                                                                      (__nv_bfloat16*)out);         \
        }                                                                                                           \
    } while (0)
    switch (coutp) {
    case 8: FWD(1); break;
    case 16: FWD(2); break;
    case 32: FWD(4); break;
    default: FWD(6); break;
    }
#undef FWD
    count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(cudaGetErrorString(e));
        return AGB_CUDA;
    }
    return AGB_OK;
}

extern "C" agb_status agb_conv3_wgrad(const int n[3], int cinp, int coutp, const void* in, const void* dy, float* dw,
                                      float* db, void* stream)
{
    agb_status s = conv_check(n, cinp, coutp);
    if (s != AGB_OK) return s;
    if (coutp != 16 && coutp != 32) {
        set_error("conv3 wgrad: output channels must be 16 or 32 (pad 8 to 16)");
        return AGB_BADARG;
    }
    if (!in || !dy || !dw) {
        set_error("null argument");
        return AGB_BADARG;
    }
    Grid3 G{{n[0], n[1], n[2]}};
    const int MT = coutp / 16, NTc = cinp / 8;
    const int tg = std::min(27, std::max(1, 8 * WG_MAX_OWN / (MT * NTc)));
    const int ngroups = (27 + tg - 1) / tg;
    const int ntile = (n[0] / CX) * (n[1] / CY) * (n[2] / CZ);
    const int gx = std::max(1, std::min(ntile, sm_count() * 2 / ngroups + 1));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t sm = wgrad_smem(cinp, coutp);
    dim3 grid(gx, ngroups);
    if (MT == 1)
        k_conv3_wgrad<1><<<grid, CONV_THREADS, sm, st>>>(G, cinp, tg, (const __nv_bfloat16*)in,
                                                         (const __nv_bfloat16*)dy, dw);
    else
        k_conv3_wgrad<2><<<grid, CONV_THREADS, sm, st>>>(G, cinp, tg, (const __nv_bfloat16*)in,
                                                         (const __nv_bfloat16*)dy, dw);
    count_launch();
    if (db) {
        const long long nvox = (long long)n[0] * n[1] * n[2];
        k_bias_grad<<<dim3(sm_count(), coutp), 256, 0, st>>>(nvox, coutp, (const __nv_bfloat16*)dy, db);
        count_launch();
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(cudaGetErrorString(e));
        return AGB_CUDA;
    }
    return AGB_OK;
}

extern "C" agb_status agb_conv3_flip(int cinp, int coutp, const void* w, void* wt, void* stream)
{
    if (!w || !wt || cinp < 1 || coutp < 1) {
        set_error("bad argument");
        return AGB_BADARG;
    }
    const int total = 27 * cinp * coutp;
    k_conv3_flip<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(cinp, coutp, (const __nv_bfloat16*)w,
                                                                       (__nv_bfloat16*)wt);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA;
}

extern "C" agb_status agb_relu_backward(long long count, const void* y, void* dy, void* stream)
{
    if (!y || !dy || count < 0) {
        set_error("bad argument");
        return AGB_BADARG;
    }
    k_relu_bwd<<<conv_blocks(count), 256, 0, (cudaStream_t)stream>>>(count, (const __nv_bfloat16*)y,
                                                                     (__nv_bfloat16*)dy);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA;
}

extern "C" agb_status agb_adam_step(long long count, float* w, const float* g, float* m, float* v, void* w_bf16,
                                    float lr, float beta1, float beta2, float eps, int step, void* stream)
{
    if (!w || !g || !m || !v || count < 0 || step < 1) {
        set_error("bad argument");
        return AGB_BADARG;
    }
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    k_adam<<<conv_blocks(count), 256, 0, (cudaStream_t)stream>>>(count, w, g, m, v, (__nv_bfloat16*)w_bf16, lr, beta1,
                                                                 beta2, eps, c1, c2);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA;
}
