// kernels_micro.cu -- seeded synthetic microstructures generated on the GPU.
//
// The random draws (seed points, orientations, inclusion shapes) are made on
// the host from SplitMix64 streams (alamo_gb300/microstructure.py) and passed
// in as small parameter tables; these kernels evaluate the per-node fields
// that the host generators would build, so the fields of a 257^3 polycrystal
// or of 512 RVEs never cross the host link.  Counterparts in the reference:
//   Voronoi grains       IC/Voronoi.H (the reference draws its seeds with
//                        glibc rand(); here they come from SplitMix64)
//   ellipsoid inclusions IC/Ellipse.H (diffuse boundary as in the sphere case)
//   cubic moduli         Set/Matrix4_MajorMinor.H:518-556 (Cubic(), evaluated
//                        per grain on the host; the kernel gathers)
//   sphere + eigenstrain Integrator/Mechanics.H:249-253 (eta mixing of the
//                        two affine isotropic models)
// Node (i,j,k) of an n-cell box sits at (i/n0, j/n1, k/n2) of the unit cube,
// and the output is the AoS nodal field in the reference's layout (i fastest,
// n+1 nodes per direction).
#include <cuda_runtime.h>

#include <vector>

#include "agb.h"
#include "agb_internal.h"

namespace agb {
namespace {

struct Box {
    int n[3];
    __host__ __device__ long long count() const { return (long long)(n[0] + 1) * (n[1] + 1) * (n[2] + 1); }
};

__device__ __forceinline__ void node_of(const Box& b, long long e, int& i, int& j, int& k)
{
    i = (int)(e % (b.n[0] + 1));
    j = (int)((e / (b.n[0] + 1)) % (b.n[1] + 1));
    k = (int)(e / ((long long)(b.n[0] + 1) * (b.n[1] + 1)));
}

// Nearest seed (Euclidean, not periodic; the first one on ties), with the
// squared distance evaluated in the host generator's order without fused
// multiply-adds, so the grain ids equal the host's.
__global__ void k_gen_voronoi(Box b, int ng, const double* __restrict__ seeds, const double* __restrict__ table,
                              double* __restrict__ ddw, int* __restrict__ ids)
{
    const long long cnt = b.count();
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_of(b, e, i, j, k);
        const double x = (double)i / b.n[0], y = (double)j / b.n[1], z = (double)k / b.n[2];
        int best = 0;
        double bd = 0;
        for (int g = 0; g < ng; g++) {
            const double dx = __dsub_rn(x, seeds[3 * g]), dy = __dsub_rn(y, seeds[3 * g + 1]),
                         dz = __dsub_rn(z, seeds[3 * g + 2]);
            const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            if (g == 0 || d2 < bd) {
                bd = d2;
                best = g;
            }
        }
        if (ids) ids[e] = best;
        for (int m = 0; m < 21; m++) ddw[e * 21 + m] = table[best * 21 + m];
    }
}

// Isotropic (lambda = mu = contrast) field of diffuse ellipsoidal inclusions
// in a unit matrix.  Per inclusion (16 doubles): centre[3], semi-axes[3],
// rotation R[9] (row-major; the inclusion frame is y = d R), log(contrast).
// The nearest periodic image of each inclusion is used.
__global__ void k_gen_ellipsoids(Box b, int ninc, const double* __restrict__ inc, double width_cells,
                                 double* __restrict__ ddw)
{
    const long long cnt = b.count();
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_of(b, e, i, j, k);
        const double p[3] = {(double)i / b.n[0], (double)j / b.n[1], (double)k / b.n[2]};
        double logc = 0.0;
        for (int q = 0; q < ninc; q++) {
            const double* P = inc + 16 * q;
            double d[3];
            for (int a = 0; a < 3; a++) {
                d[a] = p[a] - P[a];
                d[a] -= rint(d[a]);
            }
            double r2 = 0.0;
            for (int c = 0; c < 3; c++) {
                const double y = d[0] * P[6 + c] + d[1] * P[9 + c] + d[2] * P[12 + c];
                const double t = y / P[3 + c];
                r2 += t * t;
            }
            const double s = (sqrt(r2) - 1.0) * ((P[3] + P[4] + P[5]) / 3.0);
            const double wq = width_cells * fmax(1.0, P[15] / log(10.0));   // wider above contrast 10
            const double phi = 0.5 * (1.0 - tanh(s * b.n[0] / wq));
            const double v = phi * P[15];
            logc = v > logc ? v : logc;
        }
        const double c = exp(logc);
        ddw[2 * e] = c;
        ddw[2 * e + 1] = c;
    }
}

// Centred sphere: eta = (1 - tanh((r - R)/(2 dx)))/2, moduli and the
// isotropic eigenstrain eig * eta * I mixed by eta.
__global__ void k_gen_sphere(Box b, double R, double lm, double mm, double li, double mi, double eig,
                             double* __restrict__ ddw, double* __restrict__ F0)
{
    const long long cnt = b.count();
    const double dx = 1.0 / b.n[0];
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_of(b, e, i, j, k);
        const double x = (double)i / b.n[0] - 0.5, y = (double)j / b.n[1] - 0.5, z = (double)k / b.n[2] - 0.5;
        const double r = sqrt(x * x + y * y + z * z);
        const double eta = 0.5 * (1.0 - tanh((r - R) / (2.0 * dx)));
        ddw[2 * e] = eta * li + (1.0 - eta) * lm;
        ddw[2 * e + 1] = eta * mi + (1.0 - eta) * mm;
        if (F0)
            for (int m = 0; m < 9; m++) F0[9 * e + m] = (m == 0 || m == 4 || m == 8) ? eta * eig : 0.0;
    }
}

int gen_blocks(long long n)
{
    const long long b = (n + 255) / 256;
    const long long cap = 8LL * sm_count();
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

// Device scratch for host-side outputs and the parameter tables.
struct Dev {
    std::vector<void*> p;
    ~Dev()
    {
        for (void* q : p) cudaFree(q);
    }
    template <typename T> T* get(size_t count)
    {
        void* q = nullptr;
        if (cudaMalloc(&q, count * sizeof(T)) != cudaSuccess) return nullptr;
        p.push_back(q);
        return (T*)q;
    }
};

agb_status check_box(const int n[3], Box& b)
{
    if (!n) {
        set_error("null n_cells");
        return AGB_BADARG;
    }
    for (int d = 0; d < 3; d++) {
        if (n[d] < 1) {
            set_error("n_cells must be >= 1");
            return AGB_BADARG;
        }
        b.n[d] = n[d];
    }
    return AGB_OK;
}

#define GEN_CK(x)                                                   \
    do {                                                            \
        cudaError_t e_ = (x);                                       \
        if (e_ != cudaSuccess) {                                    \
            set_error(cudaGetErrorString(e_));                      \
            return AGB_CUDA;                                        \
        }                                                           \
    } while (0)

}  // namespace
}  // namespace agb

using namespace agb;

extern "C" agb_status agb_gen_voronoi_cubic(const int n_cells[3], int ngrains, const double* seeds,
                                            const double* table, double* ddw, int* ids, int mem, void* stream)
{
    Box b;
    agb_status s = check_box(n_cells, b);
    if (s != AGB_OK) return s;
    if (ngrains < 1 || !seeds || !table || !ddw) {
        set_error("need ngrains >= 1, seeds, table and ddw");
        return AGB_BADARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const long long cnt = b.count();
    Dev dev;
    double* d_seeds = dev.get<double>(3 * (size_t)ngrains);
    double* d_table = dev.get<double>(21 * (size_t)ngrains);
    double* out = mem == AGB_MEM_DEVICE ? ddw : dev.get<double>(21 * (size_t)cnt);
    int* oid = ids ? (mem == AGB_MEM_DEVICE ? ids : dev.get<int>((size_t)cnt)) : nullptr;
    if (!d_seeds || !d_table || !out || (ids && !oid)) {
        set_error("cudaMalloc failed in agb_gen_voronoi_cubic");
        return AGB_NOMEM;
    }
    GEN_CK(cudaMemcpyAsync(d_seeds, seeds, sizeof(double) * 3 * ngrains, cudaMemcpyHostToDevice, st));
    GEN_CK(cudaMemcpyAsync(d_table, table, sizeof(double) * 21 * ngrains, cudaMemcpyHostToDevice, st));
    k_gen_voronoi<<<gen_blocks(cnt), 256, 0, st>>>(b, ngrains, d_seeds, d_table, out, oid);
    count_launch();
    GEN_CK(cudaGetLastError());
    if (mem != AGB_MEM_DEVICE) {
        GEN_CK(cudaMemcpyAsync(ddw, out, sizeof(double) * 21 * cnt, cudaMemcpyDeviceToHost, st));
        if (ids) GEN_CK(cudaMemcpyAsync(ids, oid, sizeof(int) * cnt, cudaMemcpyDeviceToHost, st));
    }
    // the parameter tables (and host-side staging) are freed on return
    GEN_CK(cudaStreamSynchronize(st));
    return AGB_OK;
}

extern "C" agb_status agb_gen_ellipsoids(const int n_cells[3], int ninc, const double* inclusions, double width_cells,
                                         double* ddw, int mem, void* stream)
{
    Box b;
    agb_status s = check_box(n_cells, b);
    if (s != AGB_OK) return s;
    if (ninc < 0 || (ninc > 0 && !inclusions) || !ddw || !(width_cells > 0)) {
        set_error("need ninc >= 0, the inclusion table, ddw and width_cells > 0");
        return AGB_BADARG;
    }
    for (int q = 0; q < ninc; q++)
        for (int a = 3; a < 6; a++)
            if (!(inclusions[16 * q + a] > 0)) {
                set_error("inclusion semi-axes must be positive");
                return AGB_BADARG;
            }
    cudaStream_t st = (cudaStream_t)stream;
    const long long cnt = b.count();
    Dev dev;
    double* d_inc = dev.get<double>(16 * (size_t)(ninc > 0 ? ninc : 1));
    double* out = mem == AGB_MEM_DEVICE ? ddw : dev.get<double>(2 * (size_t)cnt);
    if (!d_inc || !out) {
        set_error("cudaMalloc failed in agb_gen_ellipsoids");
        return AGB_NOMEM;
    }
    if (ninc > 0) GEN_CK(cudaMemcpyAsync(d_inc, inclusions, sizeof(double) * 16 * ninc, cudaMemcpyHostToDevice, st));
    k_gen_ellipsoids<<<gen_blocks(cnt), 256, 0, st>>>(b, ninc, d_inc, width_cells, out);
    count_launch();
    GEN_CK(cudaGetLastError());
    if (mem != AGB_MEM_DEVICE) GEN_CK(cudaMemcpyAsync(ddw, out, sizeof(double) * 2 * cnt, cudaMemcpyDeviceToHost, st));
    GEN_CK(cudaStreamSynchronize(st));
    return AGB_OK;
}

extern "C" agb_status agb_gen_sphere(const int n_cells[3], double radius, double lam_m, double mu_m, double lam_i,
                                     double mu_i, double eig, double* ddw, double* F0, int mem, void* stream)
{
    Box b;
    agb_status s = check_box(n_cells, b);
    if (s != AGB_OK) return s;
    if (!ddw) {
        set_error("null ddw");
        return AGB_BADARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const long long cnt = b.count();
    Dev dev;
    double* out = mem == AGB_MEM_DEVICE ? ddw : dev.get<double>(2 * (size_t)cnt);
    double* f0 = F0 ? (mem == AGB_MEM_DEVICE ? F0 : dev.get<double>(9 * (size_t)cnt)) : nullptr;
    if (!out || (F0 && !f0)) {
        set_error("cudaMalloc failed in agb_gen_sphere");
        return AGB_NOMEM;
    }
    k_gen_sphere<<<gen_blocks(cnt), 256, 0, st>>>(b, radius, lam_m, mu_m, lam_i, mu_i, eig, out, f0);
    count_launch();
    GEN_CK(cudaGetLastError());
    if (mem != AGB_MEM_DEVICE) {
        GEN_CK(cudaMemcpyAsync(ddw, out, sizeof(double) * 2 * cnt, cudaMemcpyDeviceToHost, st));
        if (F0) GEN_CK(cudaMemcpyAsync(F0, f0, sizeof(double) * 9 * cnt, cudaMemcpyDeviceToHost, st));
    }
    GEN_CK(cudaStreamSynchronize(st));
    return AGB_OK;
}
