// kernels_conv.cu -- the learned correction's kernels besides the forward
// convolution (kernels_conv_tc.cu): weight and bias gradients, the weight
// flip of the data gradient, nodal grid transfers between the network's
// levels, masked gradient sums, and Adam.
//
// Fields are channels-last BF16 over nodal grids g = (gx, gy, gz), voxel =
// x + gx (y + gy z), with a channel stride cs and a channel slice [c0, c0 +
// C); the convolutions pad with zeros outside the grid.
//
//   wgrad     dW[tap][co][ci] += sum_v dy[v][co] in[v + off(tap)][ci]   (FP32)
//   bgrad     db[co] += sum_v dy[v][co]
//   flip      wt[26 - tap][ci][co] = w[tap][co][ci]: the data gradient of a
//             layer is the forward convolution of dy with wt
//   prolong   fine = beta fine + s P coarse, P trilinear between nodal grids
//             (fine node 2I = coarse node I; odd fine nodes average two)
//   prolong_t coarse = beta coarse + s P^T fine (P^T / 8 is full weighting)
//   axpby     y = (a + beta b) masked by m > 0 (ReLU backward), any of b, m absent
//   adam      Adam on FP32 master weights with a BF16 copy
// No counterpart in the reference.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "agb.h"
#include "agb_internal.h"

namespace agb {
namespace {

int conv_blocks(long long n)
{
    const long long b = (n + 255) / 256;
    const long long cap = 8LL * sm_count();
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

struct Grid {
    int g[3];
    __host__ __device__ long long count() const { return (long long)g[0] * g[1] * g[2]; }
};

// ---------------------------------------------------------------------------
// weight gradient: one CTA per (tap, 16-output block, 16-input block, voxel
// chunk); thread (co, ci) of a 16 x 16 block accumulates in FP32 over the
// chunk, staged 64 voxels at a time in shared memory; one atomic per output.
// ---------------------------------------------------------------------------
constexpr int WG_V = 64;          // voxels per staging step
constexpr int WG_CHUNK = 4096;    // voxels per CTA

__global__ void __launch_bounds__(256) k_wgrad0(Grid G, int cin, int cout, const __nv_bfloat16* __restrict__ x, int x_cs,
                                                int x_c0, const __nv_bfloat16* __restrict__ dy, int dy_cs, int dy_c0,
                                                float* __restrict__ dw)
{
    __shared__ float ds[WG_V][17], xs[WG_V][17];
    const int tap = blockIdx.y;
    const int nb_ci = cin / 16;
    const int co0 = (blockIdx.z / nb_ci) * 16, ci0 = (blockIdx.z % nb_ci) * 16;
    const int dx = tap % 3 - 1, dyy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
    const int tid = threadIdx.x, tco = tid >> 4, tci = tid & 15;
    const long long V = (long long)G.g[0] * G.g[1] * G.g[2];
    const long long v0 = (long long)blockIdx.x * WG_CHUNK;
    const long long v1 = min(V, v0 + WG_CHUNK);
    float acc = 0.f;
    for (long long vb = v0; vb < v1; vb += WG_V) {
        // stage dy[v][co0..+15] and x[v + off][ci0..+15] for 64 voxels (4 values per thread each)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = tid + 256 * q;   // 0 .. 1023
            const int vl = e >> 4, c = e & 15;
            const long long v = vb + vl;
            float d = 0.f, xv = 0.f;
            if (v < v1) {
                d = __bfloat162float(dy[v * dy_cs + dy_c0 + co0 + c]);
                const int ix = (int)(v % G.g[0]), iy = (int)((v / G.g[0]) % G.g[1]), iz = (int)(v / ((long long)G.g[0] * G.g[1]));
                const int jx = ix + dx, jy = iy + dyy, jz = iz + dz;
                if (jx >= 0 && jx < G.g[0] && jy >= 0 && jy < G.g[1] && jz >= 0 && jz < G.g[2]) {
                    const long long w = jx + (long long)G.g[0] * (jy + (long long)G.g[1] * jz);
                    xv = __bfloat162float(x[w * x_cs + x_c0 + ci0 + c]);
                }
            }
            ds[vl][c] = d;
            xs[vl][c] = xv;
        }
        __syncthreads();
#pragma unroll 8
        for (int v = 0; v < WG_V; v++) acc = fmaf(ds[v][tco], xs[v][tci], acc);
        __syncthreads();
    }
    atomicAdd(dw + ((long long)tap * cout + co0 + tco) * cin + ci0 + tci, acc);
}

// db[co] += sum_v dy[v][c0 + co]
__global__ void k_bgrad0(long long V, int cout, const __nv_bfloat16* __restrict__ dy, int dy_cs, int dy_c0,
                         float* __restrict__ db)
{
    __shared__ float red[32];
    const int co = blockIdx.y;
    float s = 0.f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        s += __bfloat162float(dy[v * dy_cs + dy_c0 + co]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(db + co, s);
    }
}

// wt[26 - tap][ci][co] = w[tap][co][ci]
__global__ void k_conv3_flip(int cin, int cout, const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 27 * cin * cout) return;
    const int tap = e / (cout * cin), rem = e - tap * cout * cin;
    const int co = rem / cin, ci = rem - co * cin;
    wt[((26 - tap) * cin + ci) * cout + co] = w[e];
}

// fine[v][fc0 + c] = beta fine + s sum over the coarse nodes of the trilinear weights
__global__ void k_prolong(Grid F, Grid Cg, int C, const __nv_bfloat16* __restrict__ crs, int c_cs, int c_c0,
                          __nv_bfloat16* __restrict__ fine, int f_cs, int f_c0, float beta, float s)
{
    const long long V = F.count();
    const long long total = V * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const long long v = e / C;
        const int ix = (int)(v % F.g[0]), iy = (int)((v / F.g[0]) % F.g[1]), iz = (int)(v / ((long long)F.g[0] * F.g[1]));
        const int xl = ix >> 1, yl = iy >> 1, zl = iz >> 1;
        const int xh = xl + (ix & 1), yh = yl + (iy & 1), zh = zl + (iz & 1);
        const int X[2] = {xl, xh}, Y[2] = {yl, yh}, Z[2] = {zl, zh};
        float acc = 0.f;
#pragma unroll
        for (int a = 0; a < 2; a++)
#pragma unroll
            for (int b = 0; b < 2; b++)
#pragma unroll
                for (int d = 0; d < 2; d++) {
                    const long long w = X[d] + (long long)Cg.g[0] * (Y[b] + (long long)Cg.g[1] * Z[a]);
                    acc += __bfloat162float(crs[w * c_cs + c_c0 + c]);
                }
        acc *= 0.125f;   // the eight corners, repeated where the fine node sits on a coarse line
        const long long o = v * f_cs + f_c0 + c;
        const float old = beta != 0.f ? __bfloat162float(fine[o]) : 0.f;
        fine[o] = __float2bfloat16(beta * old + s * acc);
    }
}

// coarse[V][cc0 + c] = beta coarse + s sum over the fine nodes 2I + d (d in
// {-1,0,1}^3, inside the grid) of prod_dim (d == 0 ? 1 : 1/2) fine
__global__ void k_prolong_t(Grid F, Grid Cg, int C, const __nv_bfloat16* __restrict__ fine, int f_cs, int f_c0,
                            __nv_bfloat16* __restrict__ crs, int c_cs, int c_c0, float beta, float s)
{
    const long long V = Cg.count();
    const long long total = V * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const long long v = e / C;
        const int I = (int)(v % Cg.g[0]), J = (int)((v / Cg.g[0]) % Cg.g[1]), K = (int)(v / ((long long)Cg.g[0] * Cg.g[1]));
        float acc = 0.f;
        for (int dz = -1; dz <= 1; dz++) {
            const int fz = 2 * K + dz;
            if (fz < 0 || fz >= F.g[2]) continue;
            for (int dy = -1; dy <= 1; dy++) {
                const int fy = 2 * J + dy;
                if (fy < 0 || fy >= F.g[1]) continue;
                for (int dx = -1; dx <= 1; dx++) {
                    const int fx = 2 * I + dx;
                    if (fx < 0 || fx >= F.g[0]) continue;
                    const float w = (dx ? 0.5f : 1.f) * (dy ? 0.5f : 1.f) * (dz ? 0.5f : 1.f);
                    const long long q = fx + (long long)F.g[0] * (fy + (long long)F.g[1] * fz);
                    acc += w * __bfloat162float(fine[q * f_cs + f_c0 + c]);
                }
            }
        }
        const long long o = v * c_cs + c_c0 + c;
        const float old = beta != 0.f ? __bfloat162float(crs[o]) : 0.f;
        crs[o] = __float2bfloat16(beta * old + s * acc);
    }
}

// y = (a + beta b) * (m > 0), b and m optional
__global__ void k_axpby_mask(long long V, int C, __nv_bfloat16* __restrict__ y, int y_cs, int y_c0,
                             const __nv_bfloat16* __restrict__ a, int a_cs, int a_c0, const __nv_bfloat16* __restrict__ b,
                             int b_cs, int b_c0, float beta, const __nv_bfloat16* __restrict__ m, int m_cs, int m_c0)
{
    const long long total = V * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const long long v = e / C;
        float r = __bfloat162float(a[v * a_cs + a_c0 + c]);
        if (b) r += beta * __bfloat162float(b[v * b_cs + b_c0 + c]);
        if (m && !(__bfloat162float(m[v * m_cs + m_c0 + c]) > 0.f)) r = 0.f;
        y[v * y_cs + y_c0 + c] = __float2bfloat16(r);
    }
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

bool slice_ok(int cs, int c0, int C) { return cs > 0 && c0 >= 0 && C > 0 && c0 + C <= cs; }

agb_status launched()
{
    count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(cudaGetErrorString(e));
        return AGB_CUDA;
    }
    return AGB_OK;
}

bool grid_ok(const int g[3]) { return g && g[0] > 0 && g[1] > 0 && g[2] > 0; }

}  // namespace

// Launchers shared with the network's forward pass (learned.cu).
void launch_prolong(cudaStream_t st, const int gf[3], const int gc[3], int C, const void* crs, int c_cs, int c_c0,
                    void* fine, int f_cs, int f_c0, float beta, float s)
{
    Grid F{{gf[0], gf[1], gf[2]}}, Cg{{gc[0], gc[1], gc[2]}};
    k_prolong<<<conv_blocks(F.count() * C), 256, 0, st>>>(F, Cg, C, (const __nv_bfloat16*)crs, c_cs, c_c0,
                                                           (__nv_bfloat16*)fine, f_cs, f_c0, beta, s);
    count_launch();
}

void launch_prolong_t(cudaStream_t st, const int gf[3], const int gc[3], int C, const void* fine, int f_cs, int f_c0,
                      void* crs, int c_cs, int c_c0, float beta, float s)
{
    Grid F{{gf[0], gf[1], gf[2]}}, Cg{{gc[0], gc[1], gc[2]}};
    k_prolong_t<<<conv_blocks(Cg.count() * C), 256, 0, st>>>(F, Cg, C, (const __nv_bfloat16*)fine, f_cs, f_c0,
                                                              (__nv_bfloat16*)crs, c_cs, c_c0, beta, s);
    count_launch();
}

}  // namespace agb

using namespace agb;

extern "C" agb_status agb_conv3_wgrad0(const int g[3], int cin, int cout, const void* x, int x_cs, int x_c0,
                                       const void* dy, int dy_cs, int dy_c0, float* dw, float* db, void* stream)
{
    if (!grid_ok(g) || !x || !dy || !dw || cin < 16 || cin % 16 || cout < 16 || cout % 16 ||
        !slice_ok(x_cs, x_c0, cin) || !slice_ok(dy_cs, dy_c0, cout)) {
        set_error("agb_conv3_wgrad0: bad argument (channels multiples of 16, slices inside their strides)");
        return AGB_BADARG;
    }
    Grid G{{g[0], g[1], g[2]}};
    const long long V = G.count();
    const long long chunks = (V + WG_CHUNK - 1) / WG_CHUNK;
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grid((unsigned)chunks, 27, (unsigned)((cout / 16) * (cin / 16)));
    k_wgrad0<<<grid, 256, 0, st>>>(G, cin, cout, (const __nv_bfloat16*)x, x_cs, x_c0, (const __nv_bfloat16*)dy, dy_cs,
                                   dy_c0, dw);
    agb_status s = launched();
    if (s != AGB_OK || !db) return s;
    k_bgrad0<<<dim3(sm_count(), cout), 256, 0, st>>>(V, cout, (const __nv_bfloat16*)dy, dy_cs, dy_c0, db);
    return launched();
}

extern "C" agb_status agb_conv3_flip(int cin, int cout, const void* w, void* wt, void* stream)
{
    if (!w || !wt || cin < 1 || cout < 1) {
        set_error("bad argument");
        return AGB_BADARG;
    }
    const int total = 27 * cin * cout;
    k_conv3_flip<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(cin, cout, (const __nv_bfloat16*)w,
                                                                       (__nv_bfloat16*)wt);
    return launched();
}

extern "C" agb_status agb_grid_prolong(const int gf[3], const int gc[3], int C, const void* crs, int c_cs, int c_c0,
                                       void* fine, int f_cs, int f_c0, float beta, float s, void* stream)
{
    if (!grid_ok(gf) || !grid_ok(gc) || !crs || !fine || !slice_ok(c_cs, c_c0, C) || !slice_ok(f_cs, f_c0, C)) {
        set_error("agb_grid_prolong: bad argument");
        return AGB_BADARG;
    }
    for (int d = 0; d < 3; d++)
        if (gf[d] != 2 * (gc[d] - 1) + 1) {
            set_error("agb_grid_prolong: fine nodes must be 2 (coarse nodes - 1) + 1 per direction");
            return AGB_BADARG;
        }
    launch_prolong((cudaStream_t)stream, gf, gc, C, crs, c_cs, c_c0, fine, f_cs, f_c0, beta, s);
    return launched();
}

extern "C" agb_status agb_grid_prolong_t(const int gf[3], const int gc[3], int C, const void* fine, int f_cs,
                                         int f_c0, void* crs, int c_cs, int c_c0, float beta, float s, void* stream)
{
    if (!grid_ok(gf) || !grid_ok(gc) || !crs || !fine || !slice_ok(c_cs, c_c0, C) || !slice_ok(f_cs, f_c0, C)) {
        set_error("agb_grid_prolong_t: bad argument");
        return AGB_BADARG;
    }
    for (int d = 0; d < 3; d++)
        if (gf[d] != 2 * (gc[d] - 1) + 1) {
            set_error("agb_grid_prolong_t: fine nodes must be 2 (coarse nodes - 1) + 1 per direction");
            return AGB_BADARG;
        }
    launch_prolong_t((cudaStream_t)stream, gf, gc, C, fine, f_cs, f_c0, crs, c_cs, c_c0, beta, s);
    return launched();
}

extern "C" agb_status agb_axpby_mask(long long nvox, int C, void* y, int y_cs, int y_c0, const void* a, int a_cs,
                                     int a_c0, const void* b, int b_cs, int b_c0, float beta, const void* m, int m_cs,
                                     int m_c0, void* stream)
{
    if (nvox < 0 || !y || !a || !slice_ok(y_cs, y_c0, C) || !slice_ok(a_cs, a_c0, C) ||
        (b && !slice_ok(b_cs, b_c0, C)) || (m && !slice_ok(m_cs, m_c0, C))) {
        set_error("agb_axpby_mask: bad argument");
        return AGB_BADARG;
    }
    k_axpby_mask<<<conv_blocks(nvox * C), 256, 0, (cudaStream_t)stream>>>(
        nvox, C, (__nv_bfloat16*)y, y_cs, y_c0, (const __nv_bfloat16*)a, a_cs, a_c0, (const __nv_bfloat16*)b, b_cs, b_c0,
        beta, (const __nv_bfloat16*)m, m_cs, m_c0);
    return launched();
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
    return launched();
}
