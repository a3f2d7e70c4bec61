/*
 * agb.h -- C ABI of alamo_gb300: a GB300 (sm_103a) implementation of Alamo's
 * nodal linear-elastic multigrid solve, drop-in for the
 * Operator::Elastic<SYM> / Solver::Nonlocal::Linear path.
 *
 * Conventions
 *   - Every function returns agb_status; no C++ exception crosses the ABI.
 *     agb_last_error() gives a thread-local message for the last failure.
 *   - Field arguments are the memory image of the reference's single-box
 *     nodal MultiFab of the level: (n0+1)(n1+1)(n2+1) nodes, i fastest, the
 *     three components one after the other (SoA), FP64 unless the name ends in
 *     _f32.  In periodic directions node n duplicates node 0 (inputs must keep
 *     them equal; outputs do).
 *   - Modulus fields (Set::Matrix4<3,SYM> per node) are AGB_LAYOUT_AOS, the
 *     memory image of a BaseFab<Matrix4>: 2 doubles (lambda, mu) for
 *     AGB_ISO, the 21 doubles of Matrix4<3,MajorMinor>::data for
 *     AGB_MAJORMINOR; or AGB_LAYOUT_SOA (coefficient-major).
 *   - `mem` says whether pointers are host (AGB_MEM_HOST) or device
 *     (AGB_MEM_DEVICE) memory.  Host pointers may be pageable or pinned.
 *     Device fields are read after the work queued on the legacy default
 *     stream when the call is made has completed; work the caller queued on
 *     other streams must be complete before the call.
 *   - One handle is not re-entrant; distinct handles may be used from
 *     distinct host threads.  Each operator owns one CUDA stream; calls
 *     return after their work has completed.
 *   - The library owns every device buffer it uses.  There is no CPU
 *     fallback: without a usable GPU every call returns AGB_CUDA.
 *
 * The reference interface each entry point replaces is cited beside it
 * (paths relative to the alamo source tree).
 */
#ifndef AGB_H
#define AGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    AGB_OK = 0,
    AGB_MAXITER = 1,   /* max_iter reached before tol (MLMG "failed to converge") */
    AGB_STALL = 2,     /* residual stopped decreasing */
    AGB_NAN = 3,       /* NaN in a residual (Elastic.cpp:262-286 aborts on this) */
    AGB_BADARG = 4,
    AGB_CUDA = 5,      /* CUDA error or no usable device */
    AGB_NOMEM = 6,
    AGB_STATE = 7      /* call out of order (e.g. solve before set_model) */
} agb_status;

enum { AGB_ISO = 0, AGB_MAJORMINOR = 1 };                  /* Set::Sym::Isotropic, Set::Sym::MajorMinor */
enum { AGB_MEM_HOST = 0, AGB_MEM_DEVICE = 1 };
enum { AGB_LAYOUT_AOS = 0, AGB_LAYOUT_SOA = 1 };
enum { AGB_PREC_F64 = 0, AGB_PREC_MIXED = 1 };

/* BC::Operator::Elastic::Elastic::Type, BC/Operator/Elastic/Elastic.H:26 */
enum { AGB_BC_DISP = 0, AGB_BC_TRAC = 1, AGB_BC_PERIODIC = 2, AGB_BC_NEUMANN = 3, AGB_BC_NONE = 4 };

/* BC::Operator::Elastic::Elastic::Face (3D), BC/Operator/Elastic/Elastic.H:35-43 */
#define AGB_NFACES 26
enum {
    AGB_XLO, AGB_YLO, AGB_ZLO, AGB_XHI, AGB_YHI, AGB_ZHI,
    AGB_YLO_ZLO, AGB_YLO_ZHI, AGB_YHI_ZLO, AGB_YHI_ZHI,
    AGB_ZLO_XLO, AGB_ZLO_XHI, AGB_ZHI_XLO, AGB_ZHI_XHI,
    AGB_XLO_YLO, AGB_XLO_YHI, AGB_XHI_YLO, AGB_XHI_YHI,
    AGB_XLO_YLO_ZLO, AGB_XLO_YLO_ZHI, AGB_XLO_YHI_ZLO, AGB_XLO_YHI_ZHI,
    AGB_XHI_YLO_ZLO, AGB_XHI_YLO_ZHI, AGB_XHI_YHI_ZLO, AGB_XHI_YHI_ZHI
};

/* BC::Operator::Elastic::Constant state: m_bc_type / m_bc_val at the
 * current time (Constant.H:435-436). */
typedef struct {
    int type[AGB_NFACES][3];
    double val[AGB_NFACES][3];
} agb_bc;

/* Solver::Nonlocal::Linear parameters (Linear.H:231-250, 296-382) plus the
 * mixed-precision controls. */
typedef struct {
    int max_iter;             /* MLMG max iterations (default 200) */
    int fixed_iter;           /* <0 off */
    int pre_smooth;           /* Fsmooth calls before restriction (each = 2 Jacobi sweeps), default 2 */
    int post_smooth;          /* default 2 */
    int final_smooth;         /* after a failed bottom solve, default 8 */
    int bottom_smooth;        /* after a converged bottom solve, default 0 */
    int max_fmg_iter;         /* iterations run as F-cycles; Linear.H:261 sets 1e8; 0 = V-cycles */
    int bottom_max_iter;      /* default 200 */
    double bottom_tol_rel;    /* default 1e-4 */
    double bottom_tol_abs;    /* <0 off */
    double omega;             /* Jacobi damping; < 0 (default) keeps the operator's, 2/3 (Operator.H:123) */
    int max_coarsening_level; /* default 30 */
    int verbose;
    int precision;            /* AGB_PREC_F64 (plain) or AGB_PREC_MIXED (FP32 cycles in FP64 refinement) */
    double inner_tol_rel;     /* mixed: residual reduction asked of each FP32 inner solve (default 1e-4) */
    int inner_max_iter;       /* mixed: FP32 cycles per refinement step (default 60) */
    int max_refine;           /* mixed: refinement steps (default 20) */
    int use_graph;            /* replay each cycle from a captured CUDA graph (default 1) */
    int krylov;               /* mixed: 0 (default) = the FP32 cycles alone, as MLMG iterates; k in 1..16 =
                                 flexible GCR over the FP32 cycle with up to k stored directions (an
                                 extension: no reference counterpart) */
} agb_solver_params;

typedef struct {
    int iterations;           /* MLMG cycles (plain) or FP32 cycles in total (mixed) */
    int status;               /* agb_status of the solve */
    double res0;              /* ||b - A x0||_inf (FP64) */
    double res_final;         /* ||b - A x||_inf (FP64) at return */
    double rhs_norm;          /* ||b||_inf */
    int nlevels;
    int refinements;          /* mixed: FP64 residual evaluations after the first */
    double solve_ms;          /* device time of the solve (CUDA events on the operator stream) */
    long long kernels;        /* kernels this library launched for the solve (graph replays included) */
} agb_solve_report;

typedef struct agb_op_s* agb_op;
typedef struct agb_solver_s* agb_solver;

void agb_default_params(agb_solver_params* p);
const char* agb_last_error(void);
const char* agb_version(void);

/* Operator::Elastic<SYM>::Elastic(geom, grids, dmap, info) + define,
 * Operator/Elastic.cpp:10-55; LPInfo max_coarsening_level sets the depth. */
agb_status agb_op_create(const int n_cells[3], const double dx[3], const int periodic[3], int sym,
                         int max_coarsening_level, agb_op* out);
agb_status agb_op_destroy(agb_op op);
/* Elastic::SetBC, Operator/Elastic.H:61-65 */
agb_status agb_op_set_bc(agb_op op, const agb_bc* bc);
/* Elastic::SetModel(amrlev, MultiTab), Operator/Elastic.cpp:89-116 (copies) */
agb_status agb_op_set_model(agb_op op, const double* ddw, int layout, int mem);
/* Elastic::SetUniform, Elastic.H:105 */
agb_status agb_op_set_uniform(agb_op op, int uniform);
/* Operator<Node>::SetOmega, Operator.H:57 */
agb_status agb_op_set_omega(agb_op op, double omega);
agb_status agb_op_num_levels(agb_op op, int* nlevels);
agb_status agb_op_level_cells(agb_op op, int level, int n_cells[3]);
/* Operator<Node>::prepareForSolve: averageDownCoeffs + Diagonal(true), Operator.cpp:253-260 */
agb_status agb_op_prepare(agb_op op);
/* modulus of a level after averaging (Elastic.cpp:748-910), for inspection */
agb_status agb_op_get_model(agb_op op, int level, double* ddw, int layout, int mem);
/* Elastic::Fapply(amrlev=0, mglev, f, u), Operator/Elastic.cpp:141-292 */
agb_status agb_op_fapply(agb_op op, int level, double* f, const double* u, int mem);
agb_status agb_op_fapply_f32(agb_op op, int level, float* f, const float* u, int mem);
/* Elastic::Diagonal(amrlev=0, mglev, diag), Operator/Elastic.cpp:298-379 */
agb_status agb_op_diagonal(agb_op op, int level, double* diag, int mem);
/* Operator<Node>::Fsmooth(amrlev=0, mglev, x, b): 2 damped-Jacobi sweeps, Operator.cpp:88-154 */
agb_status agb_op_fsmooth(agb_op op, int level, double* x, const double* b, int mem);
agb_status agb_op_fsmooth_f32(agb_op op, int level, float* x, const float* b, int mem);
/* Operator<Node>::solutionResidual: r = b - A x, Operator.cpp:636-645 */
agb_status agb_op_residual(agb_op op, int level, double* r, const double* x, const double* b, int mem);
/* Operator<Node>::restriction(amrlev, cmglev, crse, fine), Operator.cpp:262-363 */
agb_status agb_op_restriction(agb_op op, int crse_level, double* crse, const double* fine, int mem);
/* Operator<Node>::interpolation(amrlev, fmglev, fine, crse): fine += P crse, Operator.cpp:365-434 */
agb_status agb_op_interpolation(agb_op op, int fine_level, double* fine, const double* crse, int mem);

/* Solver::Nonlocal::Linear::Define(op), Linear.H:36-43 */
agb_status agb_solver_create(agb_op op, const agb_solver_params* params, agb_solver* out);
agb_status agb_solver_destroy(agb_solver s);
/* Linear::solve(sol, rhs, tol_rel, tol_abs): MLMG solve, sol updated in place,
 * Linear.H:131-147.  Like MLMG::solve it re-runs prepareForSolve (coefficient
 * averaging and diagonals) on every call.  Convergence: ||b - A x||_inf <=
 * max(tol_abs, tol_rel * max(||b||_inf, ||b - A x0||_inf)). */
agb_status agb_solve(agb_solver s, double* sol, const double* rhs, double tol_rel, double tol_abs, int mem,
                     agb_solve_report* report);
/* Linear::apply(out, in), Linear.H:169-174 */
agb_status agb_apply(agb_solver s, double* out, const double* in, int mem);

/* Newton-step helpers (one Newton iteration = the linear-model solve):
 *   BC::Operator::Elastic::Constant::Init, Constant.H:100-194
 *   Newton::prepareForSolve RHS, Solver/Nonlocal/Newton.H:144-275
 *   Newton::solve, Newton.H:279-358 (u += dsol)
 *   stress = DW(grad u), Integrator/Base/Mechanics.H:210-236 (9 per node, row-major, AoS)
 *   trac_hi[0] integral, Integrator/Base/Mechanics.H:391-431
 * F0 (eigenstrain, 9 doubles per node, AoS row-major, Model/Solid/Affine) may be NULL. */
agb_status agb_bc_init(agb_op op, double* rhs, int homogeneous, int mem);
agb_status agb_newton_rhs(agb_op op, const double* F0, const double* u, const double* b, double* rhs, int mem);
agb_status agb_newton_solve(agb_solver s, const double* F0, double* u, const double* b, double tol_rel,
                            double tol_abs, int mem, agb_solve_report* report);
agb_status agb_stress(agb_op op, const double* F0, const double* u, double* sigma9, int mem);
agb_status agb_traction_xhi(agb_op op, const double* F0, const double* u, double trac[3], int mem);
/* Elastic::Strain(amrlev, eps, u, voigt = false), Operator/Elastic.cpp:428-490:
 * eps9 = (grad u + grad u^T)/2, 9 per node, row-major, AoS (may be NULL);
 * Elastic::Energy(amrlev, energy, u), Elastic.cpp:552-597: energy = sig : eps
 * / 2 per node with sig = C : grad u (may be NULL; the reference adds this to
 * the values already in its output field, this call writes it).  Gradients
 * one-sided on the boundary as Numeric::GetStencil gives them. */
agb_status agb_strain_energy(agb_op op, const double* u, double* eps9, double* energy, int mem);

/* Batched RVE homogenization: `nprob` independent boxes (sizes n_cells[3*q..],
 * cell sizes dx[3*q..]; periodic in the directions of `periodic`, NULL = all)
 * solved together -- one persistent launch per multigrid step for the whole
 * batch, each V-cycle replayed from a captured CUDA graph, tile shapes picked
 * by timing on the batch at the first solve.  Each problem's right-hand side is
 * the Newton step at u = 0 of an affine model with a uniform eigenstrain F0
 * (9 doubles per problem; F0 = -macroscopic strain), the setting of
 * Model/Solid/Affine with Newton.H:199-231.  Per problem the algorithm is the
 * single-box solver's, V-cycles; params.precision selects plain FP64 or FP32
 * cycles in FP64 refinement.  For fully periodic boxes the solution is returned
 * modulo rigid translation (zero mean). */
typedef struct agb_batch_s* agb_batch;
agb_status agb_batch_create(int nprob, const int* n_cells, const double* dx, const int periodic[3], int sym,
                            const agb_solver_params* params, agb_batch* out);
agb_status agb_batch_destroy(agb_batch b);
agb_status agb_batch_set_bc(agb_batch b, const agb_bc* bc);
agb_status agb_batch_set_model(agb_batch b, int prob, const double* ddw, int layout, int mem);
agb_status agb_batch_set_eigenstrain(agb_batch b, const double* F0);
/* reports: one per problem (may be NULL); total: iterations = max over problems,
 * res_final = max relative residual, solve_ms, kernels. */
agb_status agb_batch_solve(agb_batch b, double tol_rel, double tol_abs, agb_solve_report* reports,
                           agb_solve_report* total);
agb_status agb_batch_get_solution(agb_batch b, int prob, double* u, int mem);
/* volume-averaged stress C : (grad u - F0) per problem (9 doubles, host) */
agb_status agb_batch_mean_stress(agb_batch b, double* sigma);
/* the stencil tile shape the autotuner chose for a level */
agb_status agb_batch_tuning(agb_batch b, int level, int dims[3]);

/* Timing hook used by the benchmark: runs `reps` launches of one internal
 * stencil sweep (mode 0 apply, 1 residual, 2 Jacobi) at `level` in FP64
 * (precision AGB_PREC_F64) or FP32 (AGB_PREC_MIXED) on the operator's resident
 * buffers, and returns the mean device time of one launch in ms (CUDA events
 * on the operator stream). */
agb_status agb_op_time_sweep(agb_op op, int level, int precision, int mode, int reps, double* ms_per_launch);

/* Measured FP64 fused-multiply-add throughput of the current device: one
 * launch of 4 CTAs per SM, 256 threads, 8 independent FMA chains of
 * 16 * iters steps per thread, timed with CUDA events on a private stream
 * after one warm-up launch.  Writes TFLOP/s (an FMA counts 2) and, when ms is
 * not NULL, the launch's time.  The FP64 stencils are bound by this pipe. */
agb_status agb_fp64_fma_peak(int iters, double* tflops, float* ms);

/* Pinned host memory (for callers that want asynchronous copies). */
agb_status agb_host_alloc(size_t bytes, void** p);
agb_status agb_host_free(void* p);

/* Nodal plotfile in the AMReX plotfile format, as Integrator::WritePlotFile
 * writes its nodal fields (Integrator/Integrator.cpp:795-1055) for one level
 * and one box: <plot_file>/<step, 5 digits>node/{Header, Level_0/Cell_H,
 * Level_0/Cell_D_00000, Checkpoint}, and the header's name appended to
 * <plot_file>/nodeoutput.visit (restarted at step 0).  Each field is SoA over
 * the (n+1)^3 nodes with 1, 3 or 9 components, named like Set::Field
 * (name; name_x.._z; name_xx, name_xy, .. name_zz row-major); `mem` says
 * where the fields are.  The box spans prob_lo..prob_hi. */
agb_status agb_write_node_plotfile(const char* plot_file, int step, double time, const int n_cells[3],
                                   const double prob_lo[3], const double prob_hi[3], int nfields,
                                   const char* const* names, const int* ncomp, const double* const* fields,
                                   int mem);

/* Synthetic microstructures evaluated on the GPU (the per-node fields of the
 * seeded generators; the random draws are made by the caller).  Output is the
 * AoS nodal field of an n-cell box of the unit cube (node (i,j,k) at
 * (i/n0, j/n1, k/n2), i fastest, n+1 nodes per direction), host or device
 * memory per `mem`; the call returns once the field is written.
 * Reference counterparts: IC/Voronoi.H (its seeds come from glibc rand()),
 * IC/Ellipse.H, Set/Matrix4_MajorMinor.H:518-556 (Cubic), and the eta mixing
 * of Integrator/Mechanics.H:249-253. */
/* Voronoi polycrystal: nearest of `ngrains` seeds (3 doubles each; Euclidean,
 * not periodic, first seed on ties), 21 MajorMinor doubles per grain from
 * `table`; ids (optional) receives the grain of every node. */
agb_status agb_gen_voronoi_cubic(const int n_cells[3], int ngrains, const double* seeds, const double* table,
                                 double* ddw, int* ids, int mem, void* stream);
/* Isotropic unit matrix with `ninc` diffuse ellipsoidal inclusions, 16 doubles
 * each: centre[3], semi-axes[3], rotation R[9] (row-major, inclusion frame
 * y = d R, d the nearest periodic image of node - centre), log(contrast).
 * lambda = mu = exp(max over inclusions of phi * log(contrast)), phi =
 * (1 - tanh(s n0 / w))/2, s = (|y / axes| - 1) * mean(axes), w = width_cells *
 * max(1, log10(contrast)). */
agb_status agb_gen_ellipsoids(const int n_cells[3], int ninc, const double* inclusions, double width_cells,
                              double* ddw, int mem, void* stream);
/* Centred sphere of radius `radius`: eta = (1 - tanh((r - radius)/(2 dx)))/2,
 * lambda/mu mixed by eta; F0 (optional, 9 per node) = eig * eta * I. */
agb_status agb_gen_sphere(const int n_cells[3], double radius, double lam_m, double mu_m, double lam_i, double mu_i,
                          double eig, double* ddw, double* F0, int mem, void* stream);

/* 3x3x3 convolution on the fifth-generation tensor cores (tcgen05.mma with
 * the accumulator in tensor memory, halo lines brought by TMA), zero padding
 * outside the box, any box size; no reference counterpart.  Fields are
 * channels-last BF16 with channel stride in_cs / out_cs (multiples of 8):
 * the call reads channels [in_c0, in_c0 + cin) and writes [out_c0, out_c0 +
 * cout) (slice starts multiples of 8), so a concatenation of skip inputs is
 * one buffer.  cin a multiple of 16, cout 16, 32, 48 or 64.  wp holds the
 * weights packed by agb_conv3_tc_pack from [27][cout][cin] BF16 (27 cin cout
 * elements: rows w_co0 .. w_co0 + cout of a [27][w_cout][cin] array, so a wide
 * layer runs as several convolutions); bias (FP32, cout) may be NULL; out FP32 when out_f32; ReLU when
 * relu.  Device pointers, 16-byte aligned; queued on `stream`.
 * agb_conv3_tc_error reports (and clears) a bounded wait of the kernel that
 * ran out since the last call. */
agb_status agb_conv3_tc_pack(int cin, int cout, const void* w, int w_cout, int w_co0, void* wp, void* stream);
agb_status agb_conv3_tc(const int n[3], int cin, int cout, const void* in, int in_cs, int in_c0, const void* wp,
                        const float* bias, void* out, int out_cs, int out_c0, int out_f32, int relu, void* stream);
agb_status agb_conv3_tc_error(int* flag);

/* Learned correction (no reference counterpart): a three-level
 * convolutional encoder-decoder (U-Net, channels 16/32/64, 3x3x3
 * convolutions on the tensor cores with zero padding, skip connections,
 * full-weighting down and trilinear up between nodal grids of g, (g-1)/2+1
 * and (g-1)/4+1 nodes) that maps the features of a residual -- r / s (s its
 * RMS), half logs of the axial and shear moduli, a boundary flag -- to a
 * displacement correction (output channels 0-2 times s h^2).  Set on a
 * mixed-precision solver with krylov > 0, every inner GCR iteration adds,
 * after the multigrid direction, the network's direction on the residual the
 * cycle left; it is kept if it removes at least min_gain of the weighted
 * residual norm squared, and after max_fail rejections in a row -- or a
 * refinement step whose FP64 residual stalls -- the solve goes on with the
 * multigrid directions alone.  Boxes: no periodic direction, edges divisible
 * by 4.
 *   agb_unet_layers / agb_unet_acts: the topology (per layer cin, cout, grid
 *     level; per forward activation its grid level and channels).
 *   agb_unet_create: weights [27][cout][cin] FP32 per layer, concatenated,
 *     and biases (cout per layer).
 *   agb_unet_set_weights: replace the weights from device BF16 arrays and
 *     FP32 biases, one pointer per layer (training).
 *   agb_unet_forward: the forward pass on a grid of g0 nodes (edges 4 m + 1),
 *     acts[0] the features, acts[1..] the other activations (caller-owned
 *     device buffers, kept for the backward pass), out FP32 [voxel][16].
 *   agb_unet_features: the features of a residual (reference layout, host
 *     or device per mem) of an operator's finest level, and its RMS.
 *   agb_solver_set_learned / agb_solver_learned_stats: attach a network
 *     (NULL detaches) and read the last solve's counts of learned directions
 *     tried and kept, and whether the network was still in use at its end. */
#define AGB_UNET_LAYERS 11
#define AGB_UNET_ACTS 13
typedef struct agb_learned_s* agb_learned;
agb_status agb_unet_layers(int* cin, int* cout, int* level);
agb_status agb_unet_acts(int* level, int* channels);
agb_status agb_unet_create(const float* weights, const float* biases, agb_learned* out);
agb_status agb_unet_set_weights(agb_learned net, const void* const* w_bf16, const float* const* biases, void* stream);
agb_status agb_unet_forward(agb_learned net, const int g0[3], void* const* acts, float* out, void* stream);
agb_status agb_unet_features(agb_op op, const double* r, int mem, void* feat, double* rms);
agb_status agb_learned_destroy(agb_learned net);
agb_status agb_solver_set_learned(agb_solver s, agb_learned net, double min_gain, int max_fail);
agb_status agb_solver_learned_stats(agb_solver s, int* tried, int* kept, int* active);

/* Training kernels of the learned correction, channels-last BF16 fields over
 * nodal grids g (voxel = x + g0 (y + g1 z)), channel slices [c0, c0 + C) of
 * buffers with channel stride cs; device pointers, queued on `stream`.
 *   wgrad0: dw[tap][co][ci] += sum_v dy[v][co] x[v + off(tap)][ci], zero
 *     padding (FP32, accumulated); db[co] += sum_v dy[v][co] (db may be NULL).
 *   flip: wt[26 - tap][ci][co] = w[tap][co][ci]; the data gradient of a layer
 *     is the forward convolution of dy with wt.
 *   grid_prolong: fine = beta fine + s P coarse (trilinear, fine = 2 (coarse
 *     - 1) + 1 nodes); grid_prolong_t: coarse = beta coarse + s P^T fine.
 *   axpby_mask: y = (a + beta b) where m > 0, else 0 (b, m may be NULL).
 *   adam_step: Adam on FP32 weights w with gradient g and moments m, v; the
 *     BF16 copy w_bf16 (may be NULL) is refreshed. */
agb_status agb_conv3_wgrad0(const int g[3], int cin, int cout, const void* x, int x_cs, int x_c0, const void* dy,
                            int dy_cs, int dy_c0, float* dw, float* db, void* stream);
agb_status agb_conv3_flip(int cin, int cout, const void* w, void* wt, void* stream);
agb_status agb_grid_prolong(const int gf[3], const int gc[3], int C, const void* crs, int c_cs, int c_c0, void* fine,
                            int f_cs, int f_c0, float beta, float s, void* stream);
agb_status agb_grid_prolong_t(const int gf[3], const int gc[3], int C, const void* fine, int f_cs, int f_c0, void* crs,
                              int c_cs, int c_c0, float beta, float s, void* stream);
agb_status agb_axpby_mask(long long nvox, int C, void* y, int y_cs, int y_c0, const void* a, int a_cs, int a_c0,
                          const void* b, int b_cs, int b_c0, float beta, const void* m, int m_cs, int m_c0,
                          void* stream);
agb_status agb_adam_step(long long count, float* w, const float* g, float* m, float* v, void* w_bf16, float lr,
                         float beta1, float beta2, float eps, int step, void* stream);

/* Allocation-free coarsest-level solve.  No counterpart in the reference: it
 * exists for callers that may not allocate device memory when they need a
 * bottom solve -- a host framework that owns all device memory through its
 * own arena and forbids cudaMalloc inside solver hooks, or a time-stepping
 * code that must not stall on cudaMalloc's implicit synchronisation in the
 * middle of a step.  It computes what the solve's bottom step computes
 * (BiCGStab on the diagonally scaled system, then smoothing) for one box with
 * no periodic direction, without calling cudaMalloc, cudaFree or any
 * allocating routine: its work vectors live in a device array of the library
 * sized for AGB_NOALLOC_MAX_NODES nodes (a 16^3-cell box), which every GPU that
 * loads the library keeps (943 KB) until the process exits.
 *   - All array arguments are DEVICE pointers in the unpadded reference
 *     layout: ddw coefficient-major (AGB_LAYOUT_SOA), diag / res / cor with the
 *     three components one after the other; *ret receives the BiCGStab code
 *     (0 converged, 1-4 breakdown, 8 not converged).  res and cor must not
 *     overlap (cor is written while res is read).
 *   - Larger boxes, and any periodic BC type, are rejected with AGB_BADARG.
 *   - The work is queued on `stream` (a cudaStream_t; NULL = default stream)
 *     and the call returns without waiting: results are valid once that
 *     stream has been synchronized.
 *   - The first call on a device looks up the array's device address (once
 *     per device, with that device current); make that first call before any
 *     stream capture.  The address is kept for the life of the process: a
 *     caller that resets a device (cudaDeviceReset) must not call this entry
 *     point again in that process.
 *   - Every call shares the one array: calls whose work overlaps on the GPU
 *     (several streams, several host threads) race and corrupt each other.
 *     Each call writes every scratch element before reading it, so nothing
 *     left by an earlier call leaks into a result. */
#define AGB_NOALLOC_MAX_NODES 4913
agb_status agb_bottom_solve_noalloc(const int n_cells[3], const double dx[3], int sym, int uniform,
                                    const agb_bc* bc, const double* ddw, const double* diag, const double* res,
                                    double* cor, int* ret, int max_iter, double tol_rel, double tol_abs,
                                    int bottom_smooth, int final_smooth, double omega, void* stream);

#ifdef __cplusplus
}
#endif
#endif
