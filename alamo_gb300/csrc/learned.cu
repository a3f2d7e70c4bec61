// learned.cu -- the learned correction network used inside the GCR solve.
//
// A stack of 3x3x3 convolutions (kernels_conv.cu) over the finest level of a
// fully periodic box, channels last, BF16 activations, FP32 accumulation.
// Features per node: the residual r / s (3 channels, s = RMS of r over the
// box), log(lambda) / 4, log(mu) / 4 (isotropic moduli; order one for
// stiffness contrasts up to ~100), zeros up to 16 channels.
// Output: the first 3 channels of the last layer, scaled back by s h^2 (the
// operator scales like C / h^2), as a displacement correction.  Hidden layers
// use ReLU; the last is linear.  No counterpart in the reference.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "agb.h"
#include "agb_internal.h"

namespace agb {
namespace {

constexpr int FEAT = 16;   // input and output channels of the network

__global__ void k_sumsq(LevelDesc L, const double* __restrict__ r, double* __restrict__ acc)
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

// feat[v][0..15] from r (padded SoA) and the isotropic moduli (coefficient-major)
__global__ void k_pack(LevelDesc L, const double* __restrict__ r, const double* __restrict__ ddw,
                       const double* __restrict__ acc, __nv_bfloat16* __restrict__ feat)
{
    const long long cnt = L.count();
    const double ms = acc[0] / (3.0 * (double)cnt);
    const double inv = ms > 0 ? 1.0 / sqrt(ms) : 1.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % L.nn[0]), j = (int)((e / L.nn[0]) % L.nn[1]), k = (int)(e / ((long long)L.nn[0] * L.nn[1]));
        const long long p = L.idx(i, j, k);
        float f[FEAT];
        for (int c = 0; c < FEAT; c++) f[c] = 0.f;
        for (int c = 0; c < 3; c++) f[c] = (float)(r[c * L.S + p] * inv);
        f[3] = (float)(0.25 * log(ddw[p]));
        f[4] = (float)(0.25 * log(ddw[L.S + p]));
        __nv_bfloat16* o = feat + e * FEAT;
        for (int c = 0; c < FEAT; c += 2) *reinterpret_cast<__nv_bfloat162*>(o + c) = __floats2bfloat162_rn(f[c], f[c + 1]);
    }
}

// e (padded SoA) = out[v][0..2] * s * h2
__global__ void k_unpack(LevelDesc L, const float* __restrict__ out, const double* __restrict__ acc, double h2,
                         double* __restrict__ e_out)
{
    const long long cnt = L.count();
    const double ms = acc[0] / (3.0 * (double)cnt);
    const double sc = (ms > 0 ? sqrt(ms) : 1.0) * h2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
        const long long p = L.idx((int)(e % L.nn[0]), (int)((e / L.nn[0]) % L.nn[1]),
                                  (int)(e / ((long long)L.nn[0] * L.nn[1])));
        for (int c = 0; c < 3; c++) e_out[c * L.S + p] = (double)out[e * FEAT + c] * sc;
    }
}

// The same features for a field in the reference layout (training data):
// r SoA over (n+1)^3 nodes with periodic duplicates, ddw AoS (lambda, mu).
__global__ void k_pack_ref(int n0, int n1, int n2, const double* __restrict__ r, const double* __restrict__ ddw,
                           double inv, __nv_bfloat16* __restrict__ feat)
{
    const long long cnt = (long long)n0 * n1 * n2;
    const long long N = (long long)(n0 + 1) * (n1 + 1) * (n2 + 1);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % n0), j = (int)((e / n0) % n1), k = (int)(e / ((long long)n0 * n1));
        const long long p = i + (long long)(n0 + 1) * (j + (long long)(n1 + 1) * k);
        float f[FEAT];
        for (int c = 0; c < FEAT; c++) f[c] = 0.f;
        for (int c = 0; c < 3; c++) f[c] = (float)(r[c * N + p] * inv);
        f[3] = (float)(0.25 * log(ddw[2 * p]));
        f[4] = (float)(0.25 * log(ddw[2 * p + 1]));
        __nv_bfloat16* o = feat + e * FEAT;
        for (int c = 0; c < FEAT; c += 2) *reinterpret_cast<__nv_bfloat162*>(o + c) = __floats2bfloat162_rn(f[c], f[c + 1]);
    }
}

int lblocks(long long n)
{
    const long long b = (n + 255) / 256;
    const long long cap = 8LL * sm_count();
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

}  // namespace
}  // namespace agb

using namespace agb;

struct agb_learned_s {
    int nl = 0;
    std::vector<int> cin, cout;
    std::vector<__nv_bfloat16*> w;
    std::vector<float*> b;
    long long cap = 0;            // voxels the scratch holds
    __nv_bfloat16* act[2] = {nullptr, nullptr};
    float* outf = nullptr;
    double* acc = nullptr;
    int maxc = FEAT;
    ~agb_learned_s()
    {
        for (auto p : w) cudaFree(p);
        for (auto p : b) cudaFree(p);
        cudaFree(act[0]);
        cudaFree(act[1]);
        cudaFree(outf);
        cudaFree(acc);
    }
};

namespace agb {

bool learned_box_ok(const LevelDesc& L)
{
    return L.singular() && L.n[0] % 16 == 0 && L.n[1] % 4 == 0 && L.n[2] % 2 == 0;
}

// e = N(r) on level L (fully periodic, stored nodes = voxels); all device, on `st`.
agb_status learned_apply(agb_learned net, cudaStream_t st, const LevelDesc& L, const double* r, const double* ddw64,
                         double* e)
{
    if (!learned_box_ok(L)) return AGB_BADARG;
    const long long nvox = L.count();
    if (nvox > net->cap) {
        cudaFree(net->act[0]);
        cudaFree(net->act[1]);
        cudaFree(net->outf);
        net->act[0] = net->act[1] = nullptr;
        net->outf = nullptr;
        if (cudaMalloc(&net->act[0], sizeof(__nv_bfloat16) * nvox * net->maxc) != cudaSuccess ||
            cudaMalloc(&net->act[1], sizeof(__nv_bfloat16) * nvox * net->maxc) != cudaSuccess ||
            cudaMalloc(&net->outf, sizeof(float) * nvox * FEAT) != cudaSuccess) {
            net->cap = 0;
            return AGB_NOMEM;
        }
        net->cap = nvox;
    }
    if (cudaMemsetAsync(net->acc, 0, sizeof(double), st) != cudaSuccess) return AGB_CUDA;
    k_sumsq<<<lblocks(nvox), 256, 0, st>>>(L, r, net->acc);
    count_launch();
    k_pack<<<lblocks(nvox), 256, 0, st>>>(L, r, ddw64, net->acc, net->act[0]);
    count_launch();
    const int n[3] = {L.n[0], L.n[1], L.n[2]};
    int cur = 0;
    for (int l = 0; l < net->nl; l++) {
        const bool last = l == net->nl - 1;
        void* out = last ? (void*)net->outf : (void*)net->act[1 - cur];
        const agb_status s = agb_conv3_forward(n, net->cin[l], net->cout[l], net->act[cur], net->w[l], net->b[l], out,
                                               last ? 1 : 0, last ? 0 : 1, (void*)st);
        if (s != AGB_OK) return s;
        cur = 1 - cur;
    }
    k_unpack<<<lblocks(nvox), 256, 0, st>>>(L, net->outf, net->acc, L.dx[0] * L.dx[0], e);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA;
}

}  // namespace agb

extern "C" agb_status agb_learned_create(int nlayers, const int* cin, const int* cout, const float* weights,
                                         const float* biases, agb_learned* out)
{
    if (!out || nlayers < 1 || nlayers > 16 || !cin || !cout || !weights || !biases) {
        set_error("agb_learned_create: bad argument");
        return AGB_BADARG;
    }
    *out = nullptr;
    for (int l = 0; l < nlayers; l++) {
        const bool ok_in = cin[l] == 16 || cin[l] == 32 || cin[l] == 48;
        const bool ok_out = cout[l] == 16 || cout[l] == 32 || cout[l] == 48;
        if (!ok_in || !ok_out || (l > 0 && cin[l] != cout[l - 1])) {
            set_error("agb_learned_create: channels must be 16, 32 or 48 and chain layer to layer");
            return AGB_BADARG;
        }
    }
    if (cin[0] != FEAT || cout[nlayers - 1] != FEAT) {
        set_error("agb_learned_create: the first layer takes 16 channels and the last gives 16");
        return AGB_BADARG;
    }
    agb_learned net = new agb_learned_s;
    net->nl = nlayers;
    const float* wp = weights;
    const float* bp = biases;
    for (int l = 0; l < nlayers; l++) {
        net->cin.push_back(cin[l]);
        net->cout.push_back(cout[l]);
        net->maxc = std::max(net->maxc, cout[l]);
        const size_t nw = (size_t)27 * cout[l] * cin[l];
        std::vector<__nv_bfloat16> hw(nw);
        for (size_t q = 0; q < nw; q++) hw[q] = __float2bfloat16(wp[q]);
        __nv_bfloat16* dw = nullptr;
        float* db = nullptr;
        if (cudaMalloc(&dw, nw * sizeof(__nv_bfloat16)) != cudaSuccess ||
            cudaMalloc(&db, cout[l] * sizeof(float)) != cudaSuccess) {
            cudaFree(dw);
            delete net;
            set_error("agb_learned_create: cudaMalloc failed");
            return AGB_NOMEM;
        }
        net->w.push_back(dw);
        net->b.push_back(db);
        if (cudaMemcpy(dw, hw.data(), nw * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(db, bp, cout[l] * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
            delete net;
            set_error("agb_learned_create: upload failed");
            return AGB_CUDA;
        }
        wp += nw;
        bp += cout[l];
    }
    if (cudaMalloc(&net->acc, sizeof(double)) != cudaSuccess) {
        delete net;
        set_error("agb_learned_create: cudaMalloc failed");
        return AGB_NOMEM;
    }
    *out = net;
    return AGB_OK;
}

extern "C" agb_status agb_learned_destroy(agb_learned net)
{
    delete net;
    return AGB_OK;
}

extern "C" agb_status agb_learned_features(const int n_cells[3], const double* r, const double* ddw, double scale,
                                           void* feat, void* stream)
{
    if (!n_cells || !r || !ddw || !feat || !(scale > 0)) {
        set_error("agb_learned_features: bad argument");
        return AGB_BADARG;
    }
    const long long cnt = (long long)n_cells[0] * n_cells[1] * n_cells[2];
    k_pack_ref<<<lblocks(cnt), 256, 0, (cudaStream_t)stream>>>(n_cells[0], n_cells[1], n_cells[2], r, ddw, 1.0 / scale,
                                                               (__nv_bfloat16*)feat);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? AGB_OK : AGB_CUDA;
}
