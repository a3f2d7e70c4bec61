// kernels_newton.cu -- the steps either side of the linear solve.
//
//   dw / stress   DW = C : (grad u - F0) per node with one-sided gradients on the
//                 boundary: Newton::prepareForSolve, Solver/Nonlocal/Newton.H:157-185;
//                 Model/Solid/Affine/Isotropic.H:42-45; stress output of
//                 Integrator/Base/Mechanics.H:210-236
//   newton_rhs    rhs = b - div DW (interior) | b - BC(u, grad u, DW) (boundary),
//                 Newton.H:199-231
//   bc_init       BC values into the RHS, BC/Operator/Elastic/Constant.H:100-194
//   traction_xhi  trac_hi[0] face integral, Integrator/Base/Mechanics.H:391-431
//   strain        eps = (grad u + grad u^T) / 2, Operator/Elastic.cpp:447-490
//   energy        W = sig : eps / 2 with sig = C : grad u, Operator/Elastic.cpp:552-597
#include <cuda_runtime.h>

#include "agb_internal.h"
#include "stencil.cuh"

namespace agb {

struct NAcc {
    const double* x;
    long long S;
    long long base;
    long long o[3][3];
    __device__ __forceinline__ double u(int p, int di, int dj, int dk) const
    {
        return x[p * S + base + o[0][di + 1] + o[1][dj + 1] + o[2][dk + 1]];
    }
};

__device__ __forceinline__ void node_setup(const LevelDesc& L, int i, int j, int k, NAcc& a, int mn[3], int mx[3])
{
    const long long st[3] = {1, (long long)L.P, (long long)L.P * L.nn[1]};
    const int pos[3] = {i, j, k};
    a.base = L.idx(i, j, k);
    a.S = L.S;
    for (int d = 0; d < 3; d++) {
        mn[d] = !L.per[d] && pos[d] == 0;
        mx[d] = !L.per[d] && pos[d] == L.n[d];
        a.o[d][0] = -st[d];
        a.o[d][1] = 0;
        a.o[d][2] = st[d];
        if (L.per[d]) {
            if (pos[d] == 0) a.o[d][0] = st[d] * (L.n[d] - 1);
            if (pos[d] == L.n[d] - 1) a.o[d][2] = -st[d] * (L.n[d] - 1);
        }
    }
}

__device__ __forceinline__ void gradient(const NAcc& a, const LevelDesc& L, const int mn[3], const int mx[3],
                                         double G[3][3])
{
    for (int p = 0; p < 3; p++) {
        const double u0 = a.u(p, 0, 0, 0);
        for (int d = 0; d < 3; d++) {
            const int ox = d == 0, oy = d == 1, oz = d == 2;
            if (mn[d]) G[p][d] = (a.u(p, ox, oy, oz) - u0) / L.dx[d];
            else if (mx[d]) G[p][d] = (u0 - a.u(p, -ox, -oy, -oz)) / L.dx[d];
            else G[p][d] = (a.u(p, ox, oy, oz) - a.u(p, -ox, -oy, -oz)) * 0.5 / L.dx[d];
        }
    }
}

template <int SYM>
__global__ void k_dw(LevelDesc L, const double* __restrict__ ddw, const double* __restrict__ F0,
                     const double* __restrict__ u, double* __restrict__ dw)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= L.nn[0] || j >= L.nn[1] || k >= L.nn[2]) return;
    NAcc a;
    a.x = u;
    int mn[3], mx[3];
    node_setup(L, i, j, k, a, mn, mx);
    double G[3][3], E[3][3], D[3][3], c[NCoef<SYM>::value];
    gradient(a, L, mn, mx, G);
    for (int r = 0; r < 3; r++)
        for (int s = 0; s < 3; s++) E[r][s] = G[r][s] - (F0 ? F0[(r * 3 + s) * L.S + a.base] : 0.0);
    for (int m = 0; m < NCoef<SYM>::value; m++) c[m] = ddw[m * L.S + a.base];
    c_mul_mat<double, SYM>(c, E, D);
    for (int r = 0; r < 3; r++)
        for (int s = 0; s < 3; s++) dw[(r * 3 + s) * L.S + a.base] = D[r][s];
}

// Elastic::Strain (non-Voigt, 9 per node, row-major) and Elastic::Energy per
// node, with the gradient stencils of Numeric::GetStencil (one-sided on the
// boundary).  Either output may be null.
template <int SYM>
__global__ void k_strain_energy(LevelDesc L, const double* __restrict__ ddw, const double* __restrict__ u,
                                double* __restrict__ eps, double* __restrict__ energy)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= L.nn[0] || j >= L.nn[1] || k >= L.nn[2]) return;
    NAcc a;
    a.x = u;
    int mn[3], mx[3];
    node_setup(L, i, j, k, a, mn, mx);
    double G[3][3], E[3][3];
    gradient(a, L, mn, mx, G);
    for (int r = 0; r < 3; r++)
        for (int s = 0; s < 3; s++) E[r][s] = 0.5 * (G[r][s] + G[s][r]);
    if (eps)
        for (int r = 0; r < 3; r++)
            for (int s = 0; s < 3; s++) eps[(r * 3 + s) * L.S + a.base] = E[r][s];
    if (energy) {
        double c[NCoef<SYM>::value], S[3][3];
        for (int m = 0; m < NCoef<SYM>::value; m++) c[m] = ddw[m * L.S + a.base];
        c_mul_mat<double, SYM>(c, G, S);
        double w = 0.0;
        for (int r = 0; r < 3; r++)
            for (int s = 0; s < 3; s++) w += 0.5 * S[r][s] * E[r][s];
        energy[a.base] = w;
    }
}

__global__ void k_newton_rhs(LevelDesc L, BCTable bc, const double* __restrict__ u, const double* __restrict__ b,
                             const double* __restrict__ dw, double* __restrict__ rhs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= L.nn[0] || j >= L.nn[1] || k >= L.nn[2]) return;
    NAcc a;
    a.x = u;
    int mn[3], mx[3];
    node_setup(L, i, j, k, a, mn, mx);
    const bool bnd = mn[0] | mx[0] | mn[1] | mx[1] | mn[2] | mx[2];
    double ret[3];
    if (bnd) {
        double G[3][3], S[3][3], uc[3], nrm[3];
        gradient(a, L, mn, mx, G);
        for (int r = 0; r < 3; r++) {
            uc[r] = u[r * L.S + a.base];
            for (int s = 0; s < 3; s++) S[r][s] = dw[(r * 3 + s) * L.S + a.base];
        }
        const int face = face_of(mn, mx, nrm);
        bc_set<double>(bc.type[face], uc, G, S, nrm, ret);
    } else {
        // Numeric::Divergence, Numeric/Stencil.H:588-657 (central)
        for (int r = 0; r < 3; r++) ret[r] = 0.0;
        for (int d = 0; d < 3; d++) {
            const long long pp = a.base + a.o[d][2], pm = a.base + a.o[d][0];
            for (int r = 0; r < 3; r++)
                ret[r] += (dw[(r * 3 + d) * L.S + pp] - dw[(r * 3 + d) * L.S + pm]) / 2. / L.dx[d];
        }
    }
    for (int r = 0; r < 3; r++) rhs[r * L.S + a.base] = b[r * L.S + a.base] - ret[r];
}

__global__ void k_bc_init(LevelDesc L, BCTable bc, double* __restrict__ rhs, int homogeneous)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= L.nn[0] || j >= L.nn[1] || k >= L.nn[2]) return;
    const int pos[3] = {i, j, k};
    int mn[3], mx[3];
    bool bnd = false;
    for (int d = 0; d < 3; d++) {
        mn[d] = !L.per[d] && pos[d] == 0;
        mx[d] = !L.per[d] && pos[d] == L.n[d];
        bnd = bnd || mn[d] || mx[d];
    }
    if (!bnd) return;
    double nrm[3];
    const int face = face_of(mn, mx, nrm);
    const long long q = L.idx(i, j, k);
    for (int d = 0; d < 3; d++)
        rhs[d * L.S + q] = (homogeneous && bc.type[face][d] == BCT_DISP) ? 0.0 : bc.val[face][d];
}

// one block; deterministic tree reduction over the xhi face quads
__global__ void k_traction_xhi(LevelDesc L, const double* __restrict__ s, double* __restrict__ out)
{
    __shared__ double red[3][256];
    const int i = L.n[0];
    const double da = L.dx[1] * L.dx[2];
    double acc[3] = {0, 0, 0};
    const long long nq = (long long)L.n[1] * L.n[2];
    for (long long e = threadIdx.x; e < nq; e += blockDim.x) {
        const int j = (int)(e % L.n[1]), k = (int)(e / L.n[1]);
        const int j1 = (L.per[1] && j + 1 == L.n[1]) ? 0 : j + 1;
        const int k1 = (L.per[2] && k + 1 == L.n[2]) ? 0 : k + 1;
        const long long a = L.idx(i, j, k), b = L.idx(i, j1, k), c = L.idx(i, j, k1), d = L.idx(i, j1, k1);
        for (int r = 0; r < 3; r++) {
            const long long o = (r * 3 + 0) * L.S;
            acc[r] += 0.25 * (s[o + a] + s[o + b] + s[o + c] + s[o + d]) * da;
        }
    }
    for (int r = 0; r < 3; r++) red[r][threadIdx.x] = acc[r];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int r = 0; r < 3; r++) red[r][threadIdx.x] += red[r][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int r = 0; r < 3; r++) out[r] = red[r][0];
}

static inline dim3 grid_of(const LevelDesc& L, dim3 blk)
{
    return dim3((L.nn[0] + blk.x - 1) / blk.x, (L.nn[1] + blk.y - 1) / blk.y, (L.nn[2] + blk.z - 1) / blk.z);
}

void launch_stress(cudaStream_t st, int sym, const LevelDesc& L, const double* ddw, const double* F0,
                   const double* u, double* sigma)
{
    dim3 blk(32, 4, 2);
    if (sym == SYM_ISO) k_dw<SYM_ISO><<<grid_of(L, blk), blk, 0, st>>>(L, ddw, F0, u, sigma);
    else k_dw<SYM_MM><<<grid_of(L, blk), blk, 0, st>>>(L, ddw, F0, u, sigma);
    count_launch();
}

void launch_strain_energy(cudaStream_t st, int sym, const LevelDesc& L, const double* ddw, const double* u,
                          double* eps, double* energy)
{
    dim3 blk(32, 4, 2);
    if (sym == SYM_ISO) k_strain_energy<SYM_ISO><<<grid_of(L, blk), blk, 0, st>>>(L, ddw, u, eps, energy);
    else k_strain_energy<SYM_MM><<<grid_of(L, blk), blk, 0, st>>>(L, ddw, u, eps, energy);
    count_launch();
}

void launch_newton_rhs(cudaStream_t st, int sym, const LevelDesc& L, const BCTable& bc, const double* ddw,
                       const double* F0, const double* u, const double* b, double* rhs, double* dw_work)
{
    launch_stress(st, sym, L, ddw, F0, u, dw_work);
    dim3 blk(32, 4, 2);
    k_newton_rhs<<<grid_of(L, blk), blk, 0, st>>>(L, bc, u, b, dw_work, rhs); count_launch();
}

void launch_bc_init(cudaStream_t st, const LevelDesc& L, const BCTable& bc, double* rhs, int homogeneous)
{
    dim3 blk(32, 4, 2);
    k_bc_init<<<grid_of(L, blk), blk, 0, st>>>(L, bc, rhs, homogeneous); count_launch();
}

void launch_traction_xhi(cudaStream_t st, const LevelDesc& L, const double* sigma, double* out3)
{
    k_traction_xhi<<<1, 256, 0, st>>>(L, sigma, out3); count_launch();
}

}  // namespace agb
