// learned.cu -- the learned correction: a three-level convolutional
// encoder-decoder (U-Net) over the finest level of a box, used as an extra
// search direction in the mixed solve's inner flexible GCR.  No counterpart
// in the reference.
//
// Grids: the level's nodes g0 = n + 1 per direction (n divisible by 4, no
// periodic direction), g1 = n/2 + 1, g2 = n/4 + 1; down by full weighting
// (P^T / 8), up by trilinear prolongation P.  Activations are channels-last
// BF16, every convolution 3x3x3 with zero padding on the tensor cores
// (kernels_conv_tc.cu), FP32 accumulation.
//
//   layer  grid  cin -> cout  input                 output
//     0     g0   16 -> 16     features              a1
//     1     g0   16 -> 16     a1                    cat0[32:48] (skip 0)
//                             P^T/8 cat0[32:48]  -> p1 (g1, 16)
//     2     g1   16 -> 32     p1                    b1
//     3     g1   32 -> 32     b1                    cat1[64:96] (skip 1)
//                             P^T/8 cat1[64:96]  -> p2 (g2, 32)
//     4     g2   32 -> 64     p2                    c1
//     5     g2   64 -> 64     c1                    c2
//                             P c2               -> cat1[0:64]
//     6     g1   96 -> 32     cat1                  d1
//     7     g1   32 -> 32     d1                    e1
//                             P e1               -> cat0[0:32]
//     8     g0   48 -> 16     cat0                  f0
//     9     g0   16 -> 16     f0                    h0
//    10     g0   16 -> 16     h0                    out (FP32, linear)
//   ReLU after every layer but the last; 366,336 weights.
//
// Features per node (16 channels): r / s (3; s = RMS of r over the nodes),
// log(C_xxxx), log(C_yyyy), log(C_zzzz), log(C_yzyz), log(C_xzxz),
// log(C_xyxy) times 1/2 (lambda + 2 mu and mu for isotropic moduli), a
// boundary flag, zeros.  The correction is out[:, 0:3] times s h^2 (h^2 the
// mean of dx^2): the operator scales like C / h^2.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "agb.h"
#include "agb_internal.h"
#include "stencil.cuh"

namespace agb {
namespace {

constexpr int NL = AGB_UNET_LAYERS;
constexpr int NA = AGB_UNET_ACTS;
constexpr int FEAT = 16;
const int kCin[NL] = {16, 16, 16, 32, 32, 64, 96, 32, 48, 16, 16};
const int kCout[NL] = {16, 16, 32, 32, 64, 64, 32, 32, 16, 16, 16};
const int kLevel[NL] = {0, 0, 1, 1, 2, 2, 1, 1, 0, 0, 0};
// activation buffers: a0 features, a1, cat0, p1, b1, cat1, p2, c1, c2, d1, e1, f0, h0
enum { A_FEAT, A_A1, A_CAT0, A_P1, A_B1, A_CAT1, A_P2, A_C1, A_C2, A_D1, A_E1, A_F0, A_H0 };
const int kActLevel[NA] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 1, 1, 0, 0};
const int kActC[NA] = {16, 16, 48, 16, 32, 96, 32, 64, 64, 32, 32, 16, 16};

int lblocks(long long n)
{
    const long long b = (n + 255) / 256;
    const long long cap = 8LL * sm_count();
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

void level_grid(const int g0[3], int level, int g[3])
{
    for (int d = 0; d < 3; d++) g[d] = ((g0[d] - 1) >> level) + 1;
}

// sum of r^2 over the stored nodes of the level (FP32 field, FP64 sum)
__global__ void k_sumsq32(LevelDesc L, const float* __restrict__ r, double* __restrict__ acc)
{
    const long long cnt = L.count();
    double s = 0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
        const long long p = L.idx((int)(e % L.nn[0]), (int)((e / L.nn[0]) % L.nn[1]),
                                  (int)(e / ((long long)L.nn[0] * L.nn[1])));
        for (int c = 0; c < 3; c++) {
            const double v = r[c * L.S + p];
            s += v * v;
        }
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(acc, s);
}

template <int SYM>
__global__ void k_features(LevelDesc L, const float* __restrict__ r, const float* __restrict__ ddw,
                           const double* __restrict__ acc, __nv_bfloat16* __restrict__ feat)
{
    const long long cnt = L.count();
    const double ms = acc[0] / (3.0 * (double)cnt);
    const float inv = (float)(ms > 0 ? 1.0 / sqrt(ms) : 1.0);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % L.nn[0]), j = (int)((e / L.nn[0]) % L.nn[1]), k = (int)(e / ((long long)L.nn[0] * L.nn[1]));
        const long long p = L.idx(i, j, k);
        float f[FEAT];
#pragma unroll
        for (int c = 0; c < FEAT; c++) f[c] = 0.f;
#pragma unroll
        for (int c = 0; c < 3; c++) f[c] = r[c * L.S + p] * inv;
        float ax[3], sh[3];
        if (SYM == SYM_ISO) {
            const float lam = ddw[p], mu = ddw[L.S + p];
            ax[0] = ax[1] = ax[2] = lam + 2.f * mu;
            sh[0] = sh[1] = sh[2] = mu;
        } else {
            // Matrix4<3,MajorMinor> slots of C_xxxx, C_yyyy, C_zzzz, C_yzyz, C_xzxz, C_xyxy
            ax[0] = ddw[0 * L.S + p];
            ax[1] = ddw[15 * L.S + p];
            ax[2] = ddw[20 * L.S + p];
            sh[0] = ddw[18 * L.S + p];
            sh[1] = ddw[11 * L.S + p];
            sh[2] = ddw[6 * L.S + p];
        }
#pragma unroll
        for (int d = 0; d < 3; d++) {
            f[3 + d] = 0.5f * logf(fmaxf(ax[d], 1e-30f));
            f[6 + d] = 0.5f * logf(fmaxf(sh[d], 1e-30f));
        }
        const bool bnd = (!L.per[0] && (i == 0 || i == L.n[0])) || (!L.per[1] && (j == 0 || j == L.n[1])) ||
                         (!L.per[2] && (k == 0 || k == L.n[2]));
        f[9] = bnd ? 1.f : 0.f;
        __nv_bfloat16* o = feat + e * FEAT;
#pragma unroll
        for (int c = 0; c < FEAT; c += 2)
            *reinterpret_cast<__nv_bfloat162*>(o + c) = __floats2bfloat162_rn(f[c], f[c + 1]);
    }
}

// z (padded SoA) = out[v][0..2] * s * h2
__global__ void k_correction(LevelDesc L, const float* __restrict__ out, const double* __restrict__ acc, double h2,
                             float* __restrict__ z)
{
    const long long cnt = L.count();
    const double ms = acc[0] / (3.0 * (double)cnt);
    const float sc = (float)((ms > 0 ? sqrt(ms) : 1.0) * h2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
        const long long p = L.idx((int)(e % L.nn[0]), (int)((e / L.nn[0]) % L.nn[1]),
                                  (int)(e / ((long long)L.nn[0] * L.nn[1])));
#pragma unroll
        for (int c = 0; c < 3; c++) z[c * L.S + p] = out[e * FEAT + c] * sc;
    }
}

size_t act_elems(const int g0[3], int a)
{
    int g[3];
    level_grid(g0, kActLevel[a], g);
    return (size_t)g[0] * g[1] * g[2] * kActC[a];
}

}  // namespace
}  // namespace agb

using namespace agb;

struct agb_learned_s {
    void* wp[NL] = {nullptr};     // packed BF16 weights (agb_conv3_tc_pack layout)
    float* b[NL] = {nullptr};     // biases
    // solver workspace for one level size
    int g0[3] = {0, 0, 0};
    void* act[NA] = {nullptr};
    float* out = nullptr;
    double* acc = nullptr;
    ~agb_learned_s()
    {
        for (int l = 0; l < NL; l++) {
            cudaFree(wp[l]);
            cudaFree(b[l]);
        }
        release();
        cudaFree(acc);
    }
    void release()
    {
        for (int a = 0; a < NA; a++) {
            cudaFree(act[a]);
            act[a] = nullptr;
        }
        cudaFree(out);
        out = nullptr;
        g0[0] = g0[1] = g0[2] = 0;
    }
};

namespace agb {

// The network's forward pass on a g0 grid: feat = acts[A_FEAT] (given), the
// other activations into acts, the FP32 output into out.  Queued on st.
static agb_status unet_forward(agb_learned net, cudaStream_t st, const int g0[3], void* const* acts, float* out)
{
    int g[3][3];
    for (int l = 0; l < 3; l++) level_grid(g0, l, g[l]);
    auto conv = [&](int layer, int in, int in_c0, int outa, int out_c0, bool last) -> agb_status {
        const int lev = kLevel[layer];
        void* dst = last ? (void*)out : acts[outa];
        const int cs = last ? FEAT : kActC[outa];
        return agb_conv3_tc(g[lev], kCin[layer], kCout[layer], acts[in], kActC[in], in_c0, net->wp[layer], net->b[layer],
                            dst, cs, out_c0, last ? 1 : 0, last ? 0 : 1, (void*)st);
    };
#define CK_(x)                              \
    do {                                    \
        const agb_status s_ = (x);          \
        if (s_ != AGB_OK) return s_;        \
    } while (0)
    CK_(conv(0, A_FEAT, 0, A_A1, 0, false));
    CK_(conv(1, A_A1, 0, A_CAT0, 32, false));
    launch_prolong_t(st, g[0], g[1], 16, acts[A_CAT0], 48, 32, acts[A_P1], 16, 0, 0.f, 0.125f);
    CK_(conv(2, A_P1, 0, A_B1, 0, false));
    CK_(conv(3, A_B1, 0, A_CAT1, 64, false));
    launch_prolong_t(st, g[1], g[2], 32, acts[A_CAT1], 96, 64, acts[A_P2], 32, 0, 0.f, 0.125f);
    CK_(conv(4, A_P2, 0, A_C1, 0, false));
    CK_(conv(5, A_C1, 0, A_C2, 0, false));
    launch_prolong(st, g[1], g[2], 64, acts[A_C2], 64, 0, acts[A_CAT1], 96, 0, 0.f, 1.f);
    CK_(conv(6, A_CAT1, 0, A_D1, 0, false));
    CK_(conv(7, A_D1, 0, A_E1, 0, false));
    launch_prolong(st, g[0], g[1], 32, acts[A_E1], 32, 0, acts[A_CAT0], 48, 0, 0.f, 1.f);
    CK_(conv(8, A_CAT0, 0, A_F0, 0, false));
    CK_(conv(9, A_F0, 0, A_H0, 0, false));
    CK_(conv(10, A_H0, 0, -1, 0, true));
#undef CK_
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA;
}

bool learned_level_ok(const LevelDesc& L)
{
    return !L.per[0] && !L.per[1] && !L.per[2] && L.n[0] % 4 == 0 && L.n[1] % 4 == 0 && L.n[2] % 4 == 0 &&
           L.n[0] >= 4 && L.n[1] >= 4 && L.n[2] >= 4;
}

// Features of an FP32 residual r (padded SoA) with FP32 moduli ddw32
// (coefficient-major) into feat, the residual's sum of squares into acc[0].
static void features(agb_learned net, cudaStream_t st, int sym, const LevelDesc& L, const float* r,
                     const float* ddw32, void* feat, double* acc)
{
    (void)net;
    cudaMemsetAsync(acc, 0, sizeof(double), st);
    k_sumsq32<<<lblocks(L.count()), 256, 0, st>>>(L, r, acc);
    count_launch();
    if (sym == SYM_ISO)
        k_features<SYM_ISO><<<lblocks(L.count()), 256, 0, st>>>(L, r, ddw32, acc, (__nv_bfloat16*)feat);
    else
        k_features<SYM_MM><<<lblocks(L.count()), 256, 0, st>>>(L, r, ddw32, acc, (__nv_bfloat16*)feat);
    count_launch();
}

static agb_status ensure_workspace(agb_learned net, const int g0[3])
{
    if (net->g0[0] == g0[0] && net->g0[1] == g0[1] && net->g0[2] == g0[2]) return AGB_OK;
    net->release();
    for (int a = 0; a < NA; a++)
        if (cudaMalloc(&net->act[a], act_elems(g0, a) * sizeof(__nv_bfloat16)) != cudaSuccess) {
            net->release();
            return AGB_NOMEM;
        }
    const size_t V = (size_t)g0[0] * g0[1] * g0[2];
    if (cudaMalloc(&net->out, V * FEAT * sizeof(float)) != cudaSuccess) {
        net->release();
        return AGB_NOMEM;
    }
    for (int d = 0; d < 3; d++) net->g0[d] = g0[d];
    return AGB_OK;
}

// z = N(r): the learned direction for the FP32 residual r of level L (the
// finest level of a box for which learned_level_ok holds), all on `st`
// with no host synchronisation.
agb_status learned_direction(agb_learned net, cudaStream_t st, int sym, const LevelDesc& L, const float* r,
                             const float* ddw32, float* z)
{
    if (!learned_level_ok(L)) return AGB_BADARG;
    const int g0[3] = {L.nn[0], L.nn[1], L.nn[2]};
    const agb_status s = ensure_workspace(net, g0);
    if (s != AGB_OK) return s;
    features(net, st, sym, L, r, ddw32, net->act[A_FEAT], net->acc);
    const agb_status f = unet_forward(net, st, g0, net->act, net->out);
    if (f != AGB_OK) return f;
    const double h2 = (L.dx[0] * L.dx[0] + L.dx[1] * L.dx[1] + L.dx[2] * L.dx[2]) / 3.0;
    k_correction<<<lblocks(L.count()), 256, 0, st>>>(L, net->out, net->acc, h2, z);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA;
}

// Features of a residual held in the operator's FP32 work buffer (training
// path of agb_unet_features).
agb_status learned_features(cudaStream_t st, int sym, const LevelDesc& L, const float* r, const float* ddw32,
                            void* feat, double* acc)
{
    features(nullptr, st, sym, L, r, ddw32, feat, acc);
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA;
}

}  // namespace agb

extern "C" agb_status agb_unet_layers(int* cin, int* cout, int* level)
{
    if (!cin || !cout || !level) {
        set_error("null argument");
        return AGB_BADARG;
    }
    for (int l = 0; l < NL; l++) {
        cin[l] = kCin[l];
        cout[l] = kCout[l];
        level[l] = kLevel[l];
    }
    return AGB_OK;
}

extern "C" agb_status agb_unet_acts(int* level, int* channels)
{
    if (!level || !channels) {
        set_error("null argument");
        return AGB_BADARG;
    }
    for (int a = 0; a < NA; a++) {
        level[a] = kActLevel[a];
        channels[a] = kActC[a];
    }
    return AGB_OK;
}

extern "C" agb_status agb_unet_create(const float* weights, const float* biases, agb_learned* out)
{
    if (!out || !weights || !biases) {
        set_error("agb_unet_create: null argument");
        return AGB_BADARG;
    }
    *out = nullptr;
    agb_learned net = new (std::nothrow) agb_learned_s;
    if (!net) return AGB_NOMEM;
    const float* wq = weights;
    const float* bq = biases;
    agb_status st = AGB_OK;
    for (int l = 0; l < NL && st == AGB_OK; l++) {
        const size_t nw = (size_t)27 * kCout[l] * kCin[l];
        std::vector<__nv_bfloat16> hw(nw);
        for (size_t q = 0; q < nw; q++) hw[q] = __float2bfloat16(wq[q]);
        __nv_bfloat16* tmp = nullptr;
        if (cudaMalloc(&tmp, nw * sizeof(__nv_bfloat16)) != cudaSuccess ||
            cudaMalloc(&net->wp[l], nw * sizeof(__nv_bfloat16)) != cudaSuccess ||
            cudaMalloc(&net->b[l], kCout[l] * sizeof(float)) != cudaSuccess) {
            cudaFree(tmp);
            st = AGB_NOMEM;
            break;
        }
        if (cudaMemcpy(tmp, hw.data(), nw * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(net->b[l], bq, kCout[l] * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
            st = AGB_CUDA;
        if (st == AGB_OK) st = agb_conv3_tc_pack(kCin[l], kCout[l], tmp, kCout[l], 0, net->wp[l], nullptr);
        if (st == AGB_OK && cudaDeviceSynchronize() != cudaSuccess) st = AGB_CUDA;
        cudaFree(tmp);
        wq += nw;
        bq += kCout[l];
    }
    if (st == AGB_OK && cudaMalloc(&net->acc, sizeof(double)) != cudaSuccess) st = AGB_NOMEM;
    if (st != AGB_OK) {
        delete net;
        set_error("agb_unet_create: device allocation or upload failed");
        return st;
    }
    *out = net;
    return AGB_OK;
}

extern "C" agb_status agb_unet_set_weights(agb_learned net, const void* const* w_bf16, const float* const* biases,
                                           void* stream)
{
    if (!net || !w_bf16 || !biases) {
        set_error("agb_unet_set_weights: null argument");
        return AGB_BADARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    for (int l = 0; l < NL; l++) {
        const agb_status s = agb_conv3_tc_pack(kCin[l], kCout[l], w_bf16[l], kCout[l], 0, net->wp[l], stream);
        if (s != AGB_OK) return s;
        if (cudaMemcpyAsync(net->b[l], biases[l], kCout[l] * sizeof(float), cudaMemcpyDeviceToDevice, st) !=
            cudaSuccess) {
            set_error("agb_unet_set_weights: bias copy failed");
            return AGB_CUDA;
        }
    }
    return AGB_OK;
}

extern "C" agb_status agb_unet_forward(agb_learned net, const int g0[3], void* const* acts, float* out, void* stream)
{
    if (!net || !g0 || !acts || !out) {
        set_error("agb_unet_forward: null argument");
        return AGB_BADARG;
    }
    for (int d = 0; d < 3; d++)
        if (g0[d] < 5 || (g0[d] - 1) % 4) {
            set_error("agb_unet_forward: every grid edge must be 4 m + 1 nodes, m >= 1");
            return AGB_BADARG;
        }
    for (int a = 0; a < NA; a++)
        if (!acts[a]) {
            set_error("agb_unet_forward: null activation buffer");
            return AGB_BADARG;
        }
    return unet_forward(net, (cudaStream_t)stream, g0, acts, out);
}

extern "C" agb_status agb_learned_destroy(agb_learned net)
{
    delete net;
    return AGB_OK;
}
