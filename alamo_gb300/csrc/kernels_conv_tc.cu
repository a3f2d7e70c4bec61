// kernels_conv_tc.cu -- 3x3x3 convolutions of the learned correction on the
// fifth-generation tensor cores (tcgen05.mma, accumulator in tensor memory),
// zero padding outside the box, any box size.
//
// Fields are channels-last BF16, voxel = x + nx (y + ny z), with a channel
// stride cs; a convolution reads the channel slice [c0, c0 + cin) of its input
// and writes [c0', c0' + cout) of its output, so concatenated skip inputs are
// slices of one buffer.
//
//   out[v][co] = act(bias[co] + sum_tap sum_ci in[v + off(tap)][ci] W[tap][co][ci]),
//   tap = (dx+1) + 3 (dy+1) + 9 (dz+1), in = 0 outside the box.
//
// Implicit GEMM: a CTA (4 warps) owns one line of 128 voxels (x0 .. x0+127 at
// one y, z), the GEMM's M = 128 rows; N = cout; K = 27 taps x cin, taken 16
// input channels (one stage) at a time.  For a stage, one thread issues
//   - two 4-D TMA copies of the halo lines (x0-1 .. x0+128, y-1 .. y+1, z-1 ..
//     z+1) for 8 channels each, written as [z][y][x][8 channels], out-of-box
//     voxels zero-filled by the copy;
//   - one bulk copy of the stage's weights, pre-packed as [tap][2][cout][8];
// and, once both land on an mbarrier, 27 tcgen05.mma (M = 128, N = cout,
// K = 16), one per tap, whose A operand is the halo block shifted by the tap:
// in the no-swizzle K-major operand layout each row (voxel) is 16 bytes, 8-row
// groups are 128 bytes apart and the second 8-channel half of K is one chunk
// further, so a shift by one voxel is a 16-byte move of the descriptor's start
// address.  tcgen05.commit signals a second mbarrier when the MMAs are done.
// The accumulator (128 lanes x cout FP32 columns of tensor memory) is read by
// the four warps with tcgen05.ld (warp w: lanes 32w .. 32w+31), bias and ReLU
// applied, and stored as BF16 or FP32 (16-byte stores, one voxel per thread).
//
// Every wait is bounded (about 1 s): a wait that runs out sets the error flag,
// the CTA issues no more work, waits (bounded) for what it issued, frees its
// tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <tuple>

#include "agb.h"
#include "agb_internal.h"
#include "tma.cuh"

namespace agb {
namespace {

constexpr int TC_M = 128;                  // voxels per CTA (GEMM rows)
constexpr int TC_HX = TC_M + 2;            // halo line length
constexpr int TC_CHUNK = 3 * 3 * TC_HX * 16;                   // bytes of one 8-channel halo block (18720)
constexpr int TC_CHUNK_PAD = (TC_CHUNK + 127) / 128 * 128;    // 18816: chunk distance in shared memory
constexpr int TC_THREADS = 128;

template <int COUT> struct TcLayout {
    static constexpr int A_BYTES = 2 * TC_CHUNK_PAD;          // two 8-channel halo blocks
    static constexpr int W_BYTES = 27 * 2 * COUT * 16;         // one stage of packed weights
    static constexpr int W_OFF = A_BYTES;
    static constexpr int BAR_OFF = W_OFF + W_BYTES;             // 8-byte aligned (W_BYTES multiple of 16)
    static constexpr int SMEM = BAR_OFF + 32 + 128;             // barriers, tmem slot, alignment room
    static constexpr int TMEM_COLS = COUT <= 32 ? 32 : (COUT <= 64 ? 64 : (COUT <= 128 ? 128 : 256));
};

// Shared-memory matrix descriptor of a no-swizzle K-major operand: start
// address, leading byte offset (between the two 8-element K halves), stride
// byte offset (between 8-row groups), descriptor version 1.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

struct TcArgs {
    int nx, ny, nz;
    int cin, in_c0;            // input channel slice (the tensor map covers all channels)
    int out_cs, out_c0;        // output channel stride and slice start
    int out_f32, relu;
    const __nv_bfloat16* wp;   // packed weights [stage][tap][2][cout][8]
    const float* bias;         // cout FP32, may be null
    void* out;
    int* err;
};

template <int COUT>
__global__ void __launch_bounds__(TC_THREADS) k_conv3_tc(const __grid_constant__ CUtensorMap tin, TcArgs a)
{
    typedef TcLayout<COUT> Lay;
    extern __shared__ __align__(128) unsigned char tc_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_raw) + 127) & ~(uintptr_t)127);
    const uint32_t sA = smem_u32(sm), sW = smem_u32(sm + Lay::W_OFF);
    const uint32_t bar_load = smem_u32(sm + Lay::BAR_OFF), bar_mma = bar_load + 8;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + Lay::BAR_OFF + 16);
    int* okflag = reinterpret_cast<int*>(sm + Lay::BAR_OFF + 20);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ntx = (a.nx + TC_M - 1) / TC_M;
    const int t = blockIdx.x;
    const int x0 = (t % ntx) * TC_M, y = (t / ntx) % a.ny, z = t / (ntx * a.ny);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"((uint32_t)Lay::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(bar_load, 1);
        mbar_init(bar_mma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *okflag = 1;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = *tmem_slot;

    if (tid == 0) {
        const int nstage = a.cin / 16;
        constexpr uint32_t idesc = umma_idesc_bf16(COUT);
        bool ok = true;
        int pend_load = -1, pend_mma = -1;   // parity of a phase issued and not seen complete
        for (int s = 0; s < nstage && ok; s++) {
            mbar_expect(bar_load, 2 * TC_CHUNK + Lay::W_BYTES);
            for (int c = 0; c < 2; c++)
                tma_load4(sA + c * TC_CHUNK_PAD, &tin, a.in_c0 + 16 * s + 8 * c, x0 - 1, y - 1, z - 1, bar_load);
            bulk_load(sW, a.wp + (size_t)s * 27 * 2 * COUT * 8, Lay::W_BYTES, bar_load);
            pend_load = s & 1;
            if (!mbar_wait(bar_load, (uint32_t)(s & 1))) {
                ok = false;
                break;
            }
            pend_load = -1;
#pragma unroll 1
            for (int tap = 0; tap < 27; tap++) {
                const int dx = tap % 3, dy = (tap / 3) % 3, dz = tap / 9;   // each offset + 1
                const uint32_t aaddr = sA + ((dz * 3 + dy) * TC_HX + dx) * 16;
                const uint32_t baddr = sW + tap * 2 * COUT * 16;
                umma_bf16(taddr, umma_desc(aaddr, TC_CHUNK_PAD, 128), umma_desc(baddr, COUT * 16, 128), idesc,
                          (s > 0 || tap > 0) ? 1u : 0u);
            }
            umma_commit(bar_mma);
            pend_mma = s & 1;
            if (!mbar_wait(bar_mma, (uint32_t)(s & 1))) {
                ok = false;
                break;
            }
            pend_mma = -1;
        }
        if (!ok) {
            // bounded drain of what is still in flight, then report
            if (pend_load >= 0) mbar_wait(bar_load, (uint32_t)pend_load);
            if (pend_mma >= 0) mbar_wait(bar_mma, (uint32_t)pend_mma);
            atomicExch(a.err, 1);
            *okflag = 0;
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (*okflag) {
        const int x = x0 + 32 * warp + lane;
        const bool mine = x < a.nx;
        const long long v = (long long)x + (long long)a.nx * (y + (long long)a.ny * z);
#pragma unroll
        for (int cb = 0; cb < COUT / 16; cb++) {
            float r[16];
            tmem_ld16(taddr + ((uint32_t)(32 * warp) << 16) + (uint32_t)(cb * 16), r);
#pragma unroll
            for (int i = 0; i < 16; i++) {
                float w = r[i] + (a.bias ? a.bias[cb * 16 + i] : 0.f);
                r[i] = (a.relu && w < 0.f) ? 0.f : w;
            }
            if (!mine) continue;
            const long long o = v * a.out_cs + a.out_c0 + cb * 16;
            if (a.out_f32) {
                float4* d = reinterpret_cast<float4*>(reinterpret_cast<float*>(a.out) + o);
#pragma unroll
                for (int q = 0; q < 4; q++) d[q] = make_float4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
            } else {
                uint4* d = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(a.out) + o);
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    uint32_t p[4];
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const __nv_bfloat162 h = __floats2bfloat162_rn(r[8 * q + 2 * e], r[8 * q + 2 * e + 1]);
                        p[e] = *reinterpret_cast<const uint32_t*>(&h);
                    }
                    d[q] = make_uint4(p[0], p[1], p[2], p[3]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr),
                     "r"((uint32_t)Lay::TMEM_COLS)
                     : "memory");
}

// wp[((s * 27 + tap) * 2 + h) * cout + co][e] = w[tap][co0 + co][16 s + 8 h + e], w of w_cout rows per tap
__global__ void k_conv3_tc_pack(int cin, int cout, const __nv_bfloat16* __restrict__ w, int w_cout, int co0,
                                __nv_bfloat16* __restrict__ wp)
{
    const long long total = 27LL * cout * cin;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(q % 8);
        long long r = q / 8;
        const int co = (int)(r % cout);
        r /= cout;
        const int h = (int)(r % 2);
        r /= 2;
        const int tap = (int)(r % 27);
        const int s = (int)(r / 27);
        wp[q] = w[((long long)tap * w_cout + co0 + co) * cin + 16 * s + 8 * h + e];
    }
}

PFN_cuTensorMapEncodeTiled_v12000 tc_encode_fn()
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

typedef std::tuple<const void*, int, int, int, int> TcKey;
std::mutex g_tc_mutex;
std::map<TcKey, CUtensorMap> g_tc_maps;

// Tensor map of a channels-last BF16 field (cs channels, nx x ny x nz
// voxels) with a box of 8 channels x TC_HX x 3 x 3 voxels.
bool tc_map(const void* base, int cs, const int n[3], CUtensorMap* out)
{
    const TcKey key(base, cs, n[0], n[1], n[2]);
    std::lock_guard<std::mutex> lock(g_tc_mutex);
    auto it = g_tc_maps.find(key);
    if (it != g_tc_maps.end()) {
        *out = it->second;
        return true;
    }
    PFN_cuTensorMapEncodeTiled_v12000 enc = tc_encode_fn();
    if (!enc) return false;
    CUtensorMap m;
    const cuuint64_t dims[4] = {(cuuint64_t)cs, (cuuint64_t)n[0], (cuuint64_t)n[1], (cuuint64_t)n[2]};
    const cuuint64_t strides[3] = {(cuuint64_t)cs * 2, (cuuint64_t)cs * 2 * n[0], (cuuint64_t)cs * 2 * n[0] * n[1]};
    const cuuint32_t box[4] = {8, (cuuint32_t)TC_HX, 3, 3};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    if (enc(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    if (g_tc_maps.size() > 4096) g_tc_maps.clear();
    g_tc_maps[key] = m;
    *out = m;
    return true;
}

__device__ int g_tc_error = 0;

template <int COUT> void tc_attr()
{
    cudaFuncSetAttribute(k_conv3_tc<COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcLayout<COUT>::SMEM);
}

}  // namespace

void init_conv_tc_attributes()
{
    tc_attr<16>();
    tc_attr<32>();
    tc_attr<48>();
    tc_attr<64>();
}

// Reads and clears the error flag the tensor-core convolution sets when a
// bounded wait runs out.
int conv_tc_error_take()
{
    int v = 0, z = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(int)) != cudaSuccess) return 0;
    if (v) cudaMemcpyToSymbol(g_tc_error, &z, sizeof(int));
    return v;
}

}  // namespace agb

using namespace agb;

extern "C" agb_status agb_conv3_tc_pack(int cin, int cout, const void* w, int w_cout, int w_co0, void* wp,
                                        void* stream)
{
    if (cin < 16 || cin % 16 || (cout != 16 && cout != 32 && cout != 48 && cout != 64) || !w || !wp ||
        w_co0 < 0 || w_co0 + cout > w_cout) {
        set_error("agb_conv3_tc_pack: cin must be a positive multiple of 16, cout 16, 32, 48 or 64, rows inside w");
        return AGB_BADARG;
    }
    const long long total = 27LL * cout * cin;
    const int blocks = (int)std::min<long long>((total + 255) / 256, 8LL * sm_count());
    k_conv3_tc_pack<<<blocks, 256, 0, (cudaStream_t)stream>>>(cin, cout, (const __nv_bfloat16*)w, w_cout, w_co0,
                                                               (__nv_bfloat16*)wp);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(cudaGetErrorString(e));
        return AGB_CUDA;
    }
    return AGB_OK;
}

extern "C" agb_status agb_conv3_tc(const int n[3], int cin, int cout, const void* in, int in_cs, int in_c0,
                                   const void* wp, const float* bias, void* out, int out_cs, int out_c0, int out_f32,
                                   int relu, void* stream)
{
    if (!n || !in || !wp || !out || n[0] < 1 || n[1] < 1 || n[2] < 1) {
        set_error("agb_conv3_tc: null argument or empty box");
        return AGB_BADARG;
    }
    if (cin < 16 || cin % 16 || (cout != 16 && cout != 32 && cout != 48 && cout != 64)) {
        set_error("agb_conv3_tc: cin must be a positive multiple of 16, cout 16, 32, 48 or 64");
        return AGB_BADARG;
    }
    if (in_cs % 8 || in_c0 % 8 || in_c0 < 0 || in_c0 + cin > in_cs || out_cs % 8 || out_c0 % 8 || out_c0 < 0 ||
        out_c0 + cout > out_cs || (out_f32 && (out_cs % 4 || out_c0 % 4)) ||
        (reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out) | reinterpret_cast<uintptr_t>(wp)) % 16) {
        set_error("agb_conv3_tc: channel strides and slice starts must be multiples of 8, pointers 16-byte aligned");
        return AGB_BADARG;
    }
    static int* err = [] {
        int* p = nullptr;
        if (cudaGetSymbolAddress((void**)&p, g_tc_error) != cudaSuccess) p = nullptr;
        return p;
    }();
    static bool attr = [] {
        init_conv_tc_attributes();
        return true;
    }();
    (void)attr;
    CUtensorMap m;
    if (!err || !tc_map(in, in_cs, n, &m)) {
        set_error("agb_conv3_tc: tensor map encoding failed");
        return AGB_CUDA;
    }
    TcArgs a;
    a.nx = n[0];
    a.ny = n[1];
    a.nz = n[2];
    a.cin = cin;
    a.in_c0 = in_c0;
    a.out_cs = out_cs;
    a.out_c0 = out_c0;
    a.out_f32 = out_f32;
    a.relu = relu;
    a.wp = (const __nv_bfloat16*)wp;
    a.bias = bias;
    a.out = out;
    a.err = err;
    const long long tiles = (long long)((n[0] + TC_M - 1) / TC_M) * n[1] * n[2];
    if (tiles > 0x7fffffffLL) {
        set_error("agb_conv3_tc: box too large");
        return AGB_BADARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    switch (cout) {
    case 16: k_conv3_tc<16><<<(unsigned)tiles, TC_THREADS, TcLayout<16>::SMEM, st>>>(m, a); break;
    case 32: k_conv3_tc<32><<<(unsigned)tiles, TC_THREADS, TcLayout<32>::SMEM, st>>>(m, a); break;
    case 48: k_conv3_tc<48><<<(unsigned)tiles, TC_THREADS, TcLayout<48>::SMEM, st>>>(m, a); break;
    default: k_conv3_tc<64><<<(unsigned)tiles, TC_THREADS, TcLayout<64>::SMEM, st>>>(m, a); break;
    }
    count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(cudaGetErrorString(e));
        return AGB_CUDA;
    }
    return AGB_OK;
}

extern "C" agb_status agb_conv3_tc_error(int* flag)
{
    if (!flag) {
        set_error("null argument");
        return AGB_BADARG;
    }
    *flag = conv_tc_error_take();
    return AGB_OK;
}
