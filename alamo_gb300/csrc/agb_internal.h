// agb_internal.h -- types shared by the host driver and the sm_103a kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

// Truncated unit normals of BC/Operator/Elastic/Elastic.H:79-80 (kept as the
// reference writes them: the edge/corner traction rows depend on these digits).
#define AGB_SQRT3INV 0.57735026919
#define AGB_SQRT2INV 0.70710678118

namespace agb {

// BC::Operator::Elastic::Elastic::Face (3D) and ::Type, Elastic.H:26,35-43
enum Face {
    F_XLO, F_YLO, F_ZLO, F_XHI, F_YHI, F_ZHI,
    F_YLO_ZLO, F_YLO_ZHI, F_YHI_ZLO, F_YHI_ZHI,
    F_ZLO_XLO, F_ZLO_XHI, F_ZHI_XLO, F_ZHI_XHI,
    F_XLO_YLO, F_XLO_YHI, F_XHI_YLO, F_XHI_YHI,
    F_XLO_YLO_ZLO, F_XLO_YLO_ZHI, F_XLO_YHI_ZLO, F_XLO_YHI_ZHI,
    F_XHI_YLO_ZLO, F_XHI_YLO_ZHI, F_XHI_YHI_ZLO, F_XHI_YHI_ZHI,
    F_NFACES
};
enum BCType { BCT_DISP = 0, BCT_TRAC = 1, BCT_PERIODIC = 2, BCT_NEUMANN = 3, BCT_NONE = 4 };

struct BCTable {
    int8_t type[F_NFACES][3];
    double val[F_NFACES][3];
};

// One multigrid level of one box.  Nodes are stored i-fastest with a padded
// row pitch P (multiple of 8 elements, so every row starts on a 32-byte sector
// for float and a 64-byte line pair for double).  Periodic directions store n
// nodes (node n is the image of node 0); the others store n+1.
struct LevelDesc {
    int n[3];        // cells
    int nn[3];       // stored nodes per direction
    int per[3];      // periodic flags
    int P;           // row pitch (elements)
    long long S;     // component stride (elements), multiple of 64
    double dx[3];

    __host__ __device__ long long idx(int i, int j, int k) const
    {
        return (long long)i + (long long)P * ((long long)j + (long long)nn[1] * k);
    }
    __host__ __device__ long long count() const { return (long long)nn[0] * nn[1] * nn[2]; }
};

inline LevelDesc make_level(const int n[3], const int per[3], const double dx[3])
{
    LevelDesc L;
    for (int d = 0; d < 3; d++) {
        L.n[d] = n[d];
        L.per[d] = per[d] ? 1 : 0;
        L.nn[d] = per[d] ? n[d] : n[d] + 1;
        L.dx[d] = dx[d];
    }
    L.P = (L.nn[0] + 7) / 8 * 8;
    long long s = (long long)L.P * L.nn[1] * L.nn[2];
    L.S = (s + 63) / 64 * 64;
    return L;
}

// Number of kernels this library has launched (or recorded into a graph) in
// this process; the benchmark reports kernels per solve from it.
long long& launch_counter();
inline void count_launch() { ++launch_counter(); }

enum StencilMode { MODE_APPLY = 0, MODE_RESID = 1, MODE_JACOBI = 2 };

// Launchers (kernels_*.cu).  All work is queued on `st`; none synchronizes.
template <typename T>
void launch_stencil(cudaStream_t st, int sym, int mode, const LevelDesc& L, const BCTable& bc, bool uniform,
                    const T* ddw, const T* x, const T* b, const T* diag, T* out, T omega, void* norm_slot);
template <typename T>
void launch_diagonal(cudaStream_t st, int sym, const LevelDesc& L, const BCTable& bc, const T* ddw, T* diag);
template <typename T>
void launch_restriction(cudaStream_t st, const LevelDesc& Lf, const LevelDesc& Lc, const T* fine, T* crse,
                        int ncomp);
template <typename T>
void launch_interpolation(cudaStream_t st, const LevelDesc& Lf, const LevelDesc& Lc, T* fine, const T* crse,
                          bool assign);
template <typename T>
void launch_average_ddw(cudaStream_t st, const LevelDesc& Lf, const LevelDesc& Lc, const T* fine, T* crse,
                        int ncoef);
template <typename TD, typename TS>
void launch_convert(cudaStream_t st, const LevelDesc& L, int ncomp, const TS* src, TD* dst, double scale);
template <typename T>
void launch_axpy(cudaStream_t st, const LevelDesc& L, int ncomp, T* y, const T* x, T a);
template <typename T>
void launch_zero(cudaStream_t st, const LevelDesc& L, int ncomp, T* y);
template <typename T>
void launch_norm_inf(cudaStream_t st, const LevelDesc& L, int ncomp, const T* x, void* norm_slot);

// full nodal box (reference MultiFab image, n+1 nodes per direction, unpadded)
// <-> internal padded storage.  `aos` selects the per-node interleaved modulus
// layout of a BaseFab<Matrix4>.
// Only planes k in [k0, k0+kc) are moved; with `chunk` the box side holds just those planes.
template <typename TD, typename TS>
void launch_import(cudaStream_t st, const LevelDesc& L, int ncomp, const TS* src, TD* dst, bool aos, int k0, int kc,
                   bool chunk);
template <typename TD, typename TS>
void launch_export(cudaStream_t st, const LevelDesc& L, int ncomp, const TS* src, TD* dst, bool aos, int k0, int kc,
                   bool chunk);
void launch_axpy_mixed(cudaStream_t st, const LevelDesc& L, int ncomp, double* y, const float* x, double a);
template <typename TD>
void launch_recip(cudaStream_t st, const LevelDesc& L, int ncomp, const double* d, TD* r);
void init_kernel_attributes();

template <typename T>
void launch_bottom(cudaStream_t st, int sym, const LevelDesc& L, const BCTable& bc, bool uniform,
                   const double* ddw64, const double* diag64, T* cor, const T* res, double* work, int maxiter,
                   double tol_rel, double tol_abs, int* ret_slot, int nub, int nuf, double omega);

void launch_newton_rhs(cudaStream_t st, int sym, const LevelDesc& L, const BCTable& bc, const double* ddw,
                       const double* F0, const double* u, const double* b, double* rhs, double* dw_work);
void launch_stress(cudaStream_t st, int sym, const LevelDesc& L, const double* ddw, const double* F0,
                   const double* u, double* sigma);
void launch_traction_xhi(cudaStream_t st, const LevelDesc& L, const double* sigma, double* out3);
void launch_bc_init(cudaStream_t st, const LevelDesc& L, const BCTable& bc, double* rhs, int homogeneous);

}  // namespace agb
