// agb_internal.h -- types shared by the host driver and the sm_103a kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "agb.h"

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

    // fully periodic: the operator is singular (rigid translations)
    __host__ __device__ bool singular() const { return per[0] && per[1] && per[2]; }

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
    // Row pitch: a multiple of 8 elements, and (for levels the marching
    // kernels may serve: no periodic x) wide enough that their 36-element halo
    // rows (starting at i = 32t) stay inside a row.
    const int last_tile = n[0] >= 2 ? 32 * ((n[0] - 2) / 32) : 0;
    const int need = (L.per[0] || L.nn[0] > last_tile + 36) ? L.nn[0] : last_tile + 36;
    L.P = (need + 7) / 8 * 8;
    long long s = (long long)L.P * L.nn[1] * L.nn[2];
    L.S = (s + 63) / 64 * 64;
    return L;
}

// Number of kernels this library has launched (or recorded into a graph) in
// this process; the benchmark reports kernels per solve from it.
long long& launch_counter();
inline void count_launch() { ++launch_counter(); }
// Streaming multiprocessors of the current device (queried once per device;
// 1 if the query fails, which only shrinks grid-stride grids).
int sm_count();
// Sets the thread-local message agb_last_error() returns.
void set_error(const char* msg);

enum StencilMode { MODE_APPLY = 0, MODE_RESID = 1, MODE_JACOBI = 2 };

// Programmatic dependent launch.  The multigrid cycle is a chain of short
// kernels on one stream; launched by pdl_launch, a kernel may be scheduled
// while the kernel before it drains, so its launch and prologue overlap that
// kernel's tail.  Every kernel launched so starts with pdl_entry():
// griddepcontrol.wait returns once the preceding grid has completed and its
// writes are visible (so nothing the kernel reads or writes is touched
// before), then launch_dependents lets the next kernel of the chain be
// scheduled.  Launched without the attribute both are no-ops.  Off unless
// AGB_PDL=1: on GB300 the 257^3 mixed solve measured 0.368 s with the
// attribute and 0.337 s without it.
__device__ __forceinline__ void pdl_entry()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
bool pdl_enabled();

template <typename... KArgs, typename... Args>
inline void pdl_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args)
{
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

// ---------------------------------------------------------------------------
// Batched solves: many independent boxes of different sizes per level.
// Each problem's fields of one level live back to back in a level arena;
// work is described by tiles (problem, block coordinates) that persistent
// kernels stride over.
// ---------------------------------------------------------------------------
struct BProb {
    LevelDesc L;
    long long vo;     // element offset of this problem's 3-component vectors in the level arena
    long long co;     // element offset of its moduli (ncoef planes)
    long long wo;     // element offset of its bottom-solve work (8 x 3 planes, FP64)
    int bottom;       // coarsest level of this problem
    int pad;
    double h1[3], i1[3], h2[3], hm[3];   // reciprocal grid factors (FP64)
};

struct BTile {
    int prob;
    short bx, by, bz;   // block coordinates inside the problem's level grid
    short pad;
};

enum BatchVecOp { BV_ZERO = 0, BV_COPY = 1, BV_AXPY = 2, BV_SCALE_TO32 = 3, BV_ACC_FROM32 = 4, BV_JACOBI0 = 5 };

template <typename T>
void launch_batch_stencil(cudaStream_t st, int sym, int mode, int shape, int grid, const BProb* probs,
                          const BTile* tiles, int ntiles, const int* active, const BCTable& bc, bool uniform,
                          const T* ddw, const T* x, const T* b, const T* dinv, T* out, T omega, void* norm_slots);
template <typename T>
void launch_batch_transfer(cudaStream_t st, int restrict_not_interp, bool assign, int grid, const BProb* pf,
                           const BProb* pc, const BTile* tiles, int ntiles, const int* active, const T* src, T* dst);
void launch_batch_avg_ddw(cudaStream_t st, int grid, const BProb* pf, const BProb* pc, const BTile* tiles, int ntiles,
                          const double* fine, double* crse, int ncoef);
void launch_batch_diag(cudaStream_t st, int sym, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                       const BCTable& bc, const double* ddw, double* diag, double* dinv64, float* dinv32);
void launch_batch_vec(cudaStream_t st, int op, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                      const int* active, void* y, const void* x, double a, const double* scale, int fp32,
                      const void* x2 = nullptr);
void launch_batch_bottom(cudaStream_t st, int sym, int fp32, const BProb* probs, const int* plist, int np,
                         const int* active, const BCTable& bc, bool uniform, const void* ddw, const double* diag,
                         void* cor, const void* res, double* work, int maxiter, double tol_rel, double tol_abs, int nub,
                         int nuf, double omega);
void launch_batch_rhs(cudaStream_t st, int sym, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                      const double* ddw, const double* F0, double* rhs);
void launch_batch_mean_stress(cudaStream_t st, int sym, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                              const double* ddw, const double* F0, const double* u, double* sums);
// per-problem component sums of y over the stored nodes into sums (3 per
// problem, zeroed by the caller), or (subtract) y -= sums / count, with the
// per-problem max |y| after it into norm_slots when given
template <typename T>
void launch_batch_mean3(cudaStream_t st, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                        const int* active, T* y, double* sums, int subtract, void* norm_slots = nullptr);
int batch_shape_count();
void batch_shape_dims(int shape, int dims[3]);
// Per-problem GCR over the batched FP32 cycle (kernels_batch.cu; GcrVecs
// and GCR_MAX as for the single-box inner GCR).  Tiles: the 32 x 4 x 2 lists.
struct GcrVecs;
void launch_batch_multidot(cudaStream_t st, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                           const int* active, int k, const float* x, const GcrVecs& V, const float* d, double* out,
                           int stride);
void launch_batch_gcr_orth(cudaStream_t st, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                           const int* active, int k, const double* beta, int stride, const GcrVecs& W,
                           const GcrVecs& Z, float* w, float* z);
void launch_batch_gcr_step(cudaStream_t st, int grid, const BProb* probs, const BTile* tiles, int ntiles,
                           const int* active, const double* dots, float* w, float* z, float* c, float* r,
                           void* norm_slots);
// whether stencil tile shape `shape` serves batches of this symmetry and periodicity
bool batch_shape_ok(int shape, int sym, const int per[3]);

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
// out = omega (b / D): the first damped-Jacobi sweep from a zero guess
template <typename T>
void launch_jacobi_zero(cudaStream_t st, const LevelDesc& L, int ncomp, T* out, const T* b, const T* dinv, T omega);
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
// d <- 1/d (FP32, in place; zeros stay zero)
void launch_recip_inplace(cudaStream_t st, const LevelDesc& L, int ncomp, float* d);
// Inner FP32 GCR (kernels_transfer.cu): up to GCR_MAX stored directions.
constexpr int GCR_MAX = 16;
struct GcrVecs {
    const float* v[GCR_MAX];
};
// out[i] += sum x v_i d^2 (i < k)
void launch_multidot_w(cudaStream_t st, long long n, int k, const float* x, const GcrVecs& V, const float* d,
                       double* out);
// w -= sum beta_i W_i, z -= sum beta_i Z_i (i < k)
void launch_gcr_orth(cudaStream_t st, long long n, int k, const double* beta, const GcrVecs& W, const GcrVecs& Z,
                     float* w, float* z);
// normalise (w, z) by sqrt(dots[0]), c += (dots[1] / dots[0]) z, r -= ... w, max |r| -> slot
void launch_gcr_step(cudaStream_t st, long long n, const double* dots, float* w, float* z, float* c, float* r,
                     void* slot);
// *out += sum x[e] y[e] over n elements (padding entries are zero in every vector)
// sum x y, or sum x y w^2 when w is given
void launch_dot(cudaStream_t st, long long n, const double* x, const double* y, double* out,
                const double* w = nullptr);
// learned correction network (learned.cu)
// learned correction (learned.cu): the U-Net direction z = N(r) of an FP32
// residual on the finest level of a box (no periodic direction, edges
// divisible by 4), queued on st without host synchronisation
bool learned_level_ok(const LevelDesc& L);
agb_status learned_direction(agb_learned net, cudaStream_t st, int sym, const LevelDesc& L, const float* r,
                             const float* ddw32, float* z);
agb_status learned_features(cudaStream_t st, int sym, const LevelDesc& L, const float* r, const float* ddw32,
                            void* feat, double* acc);
// nodal grid transfers of channels-last BF16 fields (kernels_conv.cu)
void launch_prolong(cudaStream_t st, const int gf[3], const int gc[3], int C, const void* crs, int c_cs, int c_c0,
                    void* fine, int f_cs, int f_c0, float beta, float s);
void launch_prolong_t(cudaStream_t st, const int gf[3], const int gc[3], int C, const void* fine, int f_cs, int f_c0,
                      void* crs, int c_cs, int c_c0, float beta, float s);
// x -= per-component mean over the stored nodes (sums3: 3 doubles of scratch);
// with norm_slot, also max |x| after the subtraction (atomic max into a zeroed slot)
template <typename T>
void launch_remove_mean(cudaStream_t st, const LevelDesc& L, T* x, double* sums3, void* norm_slot = nullptr);
template <typename TD>
void launch_recip(cudaStream_t st, const LevelDesc& L, int ncomp, const double* d, TD* r);
void init_kernel_attributes();
// FP32 interior sweep with TMA plane copies, and the x-face boundary rows of
// the interior's y and z range (kernels_tma.cu); false = not launched
bool use_tma_kernel();
bool tma_supported(const LevelDesc& L);
bool launch_stencil_tma(cudaStream_t st, int sym, int mode, const LevelDesc& L, const BCTable& bc, bool uniform,
                        const float* ddw, const float* x, const float* b, const float* dinv, float* out, float omega,
                        void* norm_slot);
int tma_error_take();   // 1 if a TMA kernel's bounded wait ran out since the last call
void init_tma_attributes();

// Dense coarsest level (at most 128 unknowns): A assembled once per solve,
// BiCGStab + smoothing of launch_bottom on it in one CTA; or, with inv and
// *inv_ok set (launch_bottom_invert), the exact product cor = A^-1 res.
bool bottom_dense_fits(const LevelDesc& L);
bool use_dense_bottom();
bool use_exact_bottom();
size_t bottom_dense_bytes(const LevelDesc& L);
void launch_bottom_assemble(cudaStream_t st, int sym, const LevelDesc& L, const BCTable& bc, bool uniform,
                            const double* ddw64, double* A);
void launch_bottom_invert(cudaStream_t st, const LevelDesc& L, const double* A, float* inv, int* ok);
template <typename T>
void launch_bottom_dense(cudaStream_t st, const LevelDesc& L, const double* A, const double* diag64, T* cor,
                         const T* res, int maxiter, double tol_rel, double tol_abs, int* ret_slot, int nub, int nuf,
                         double omega, const float* inv = nullptr, const int* inv_ok = nullptr);
void init_bottom_attributes();
template <typename T>
void launch_bottom(cudaStream_t st, int sym, const LevelDesc& L, const BCTable& bc, bool uniform,
                   const double* ddw64, const double* diag64, T* cor, const T* res, double* work, int maxiter,
                   double tol_rel, double tol_abs, int* ret_slot, int nub, int nuf, double omega);

void launch_newton_rhs(cudaStream_t st, int sym, const LevelDesc& L, const BCTable& bc, const double* ddw,
                       const double* F0, const double* u, const double* b, double* rhs, double* dw_work);
void launch_stress(cudaStream_t st, int sym, const LevelDesc& L, const double* ddw, const double* F0,
                   const double* u, double* sigma);
void launch_strain_energy(cudaStream_t st, int sym, const LevelDesc& L, const double* ddw, const double* u,
                          double* eps, double* energy);
void launch_traction_xhi(cudaStream_t st, const LevelDesc& L, const double* sigma, double* out3);
void launch_bc_init(cudaStream_t st, const LevelDesc& L, const BCTable& bc, double* rhs, int homogeneous);

}  // namespace agb
