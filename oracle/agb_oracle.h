/*
 * agb_oracle.h -- CPU restatement of Alamo's nodal linear-elastic multigrid path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * it.  The product library (alamo_gb300/libalamo_gb300.so) never links or calls
 * it, and nothing here runs on a GPU.
 *
 * Every routine is plain FP64 C, compiled with -ffp-contract=off so that the
 * operation order below (which follows the reference source line by line) is
 * the rounding order on every host.  Each function cites the reference
 * file:line it restates (paths relative to the alamo source tree).
 *
 * Parity status: the operator, smoother, transfer and averaging routines are
 * restated from the reference source; the full-solve path is pinned by the
 * reference's analytic UniaxialTension answer and the tests/Solid
 * linear-cubic.dat / affine-cubic.dat traction-vs-time KATs.  The MLMG cycle
 * schedule and BiCGStab bottom solver live in AMReX 26.06, which is not in the
 * reference tree; they are restated from AMReX's published algorithm, so
 * iteration counts (not solutions) are parity-unpinned.
 *
 * Data layout (identical to the product C ABI):
 *   node (i,j,k) of a level with n[d] cells has flat index
 *       i + (n0+1)*(j + (n1+1)*k),   N = (n0+1)(n1+1)(n2+1)
 *   vector fields are SoA: component c of node p at [c*N + p]
 *   (the component order of an AMReX nodal MultiFab);
 *   modulus fields are AoS: 2 doubles (lambda, mu) or 21 doubles
 *   (Matrix4<3,MajorMinor>::data) per node, the memory image of a
 *   BaseFab<Set::Matrix4<3,SYM>>.
 *   In periodic directions node n duplicates node 0; inputs must keep the
 *   duplicates equal and outputs keep them equal.
 */
#ifndef AGB_ORACLE_H
#define AGB_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_ISO = 0, ORC_MAJORMINOR = 1 };
/* BC::Operator::Elastic::Elastic::Type, BC/Operator/Elastic/Elastic.H:26 */
enum { ORC_DISP = 0, ORC_TRAC = 1, ORC_PERIODIC = 2, ORC_NEUMANN = 3, ORC_NONE = 4 };
/* BC::Operator::Elastic::Elastic::Face (3D), BC/Operator/Elastic/Elastic.H:35-43 */
enum {
    ORC_XLO, ORC_YLO, ORC_ZLO, ORC_XHI, ORC_YHI, ORC_ZHI,
    ORC_YLO_ZLO, ORC_YLO_ZHI, ORC_YHI_ZLO, ORC_YHI_ZHI,
    ORC_ZLO_XLO, ORC_ZLO_XHI, ORC_ZHI_XLO, ORC_ZHI_XHI,
    ORC_XLO_YLO, ORC_XLO_YHI, ORC_XHI_YLO, ORC_XHI_YHI,
    ORC_XLO_YLO_ZLO, ORC_XLO_YLO_ZHI, ORC_XLO_YHI_ZLO, ORC_XLO_YHI_ZHI,
    ORC_XHI_YLO_ZLO, ORC_XHI_YLO_ZHI, ORC_XHI_YHI_ZLO, ORC_XHI_YHI_ZHI,
    ORC_NFACES
};

typedef struct {
    int n[3];                 /* cells per direction (nodes = n+1) */
    double dx[3];             /* cell size */
    int periodic[3];
    int sym;                  /* ORC_ISO or ORC_MAJORMINOR */
    int uniform;              /* Elastic::m_uniform: drop the grad(C) term */
    int bc_type[ORC_NFACES][3];
    double bc_val[ORC_NFACES][3];
} orc_grid;

typedef struct {
    int max_iter;             /* MLMG max_iters (AMReX default 200) */
    int fixed_iter;           /* <0: off */
    int pre_smooth;           /* Fsmooth calls before restriction (each = 2 Jacobi sweeps) */
    int post_smooth;
    int final_smooth;         /* smoothing after a failed bottom solve (AMReX nuf = 8) */
    int bottom_smooth;        /* smoothing after a converged bottom solve (AMReX nub = 0) */
    int max_fmg_iter;         /* iterations done as F-cycles before switching to V-cycles */
    int bottom_max_iter;      /* BiCGStab iteration cap (AMReX default 200) */
    double bottom_tol_rel;    /* AMReX default 1e-4 */
    double bottom_tol_abs;    /* <0: off */
    double omega;             /* Jacobi damping, Operator.H:123 default 2/3 */
    int max_coarsening_level; /* LPInfo max_coarsening_level */
    int verbose;
} orc_solver_params;

typedef struct {
    int iterations;
    int status;               /* 0 converged, 1 max_iter reached, 2 NaN */
    double res0;              /* ||b - A x0||_inf */
    double res_final;
    int nlevels;
    double t_setup;           /* wall seconds: coefficient averaging, diagonals, first residual */
    double t_iter;            /* wall seconds spent in the iterations */
} orc_report;

int    orc_ncoef(int sym);
int    orc_num_threads(void);
long   orc_nnodes(const orc_grid* g);
void   orc_default_params(orc_solver_params* p);
void   orc_coarsen(const orc_grid* fine, orc_grid* crse);
int    orc_num_levels(const orc_grid* g, int max_coarsening_level);

void   orc_cubic(double C11, double C12, double C44, const double R[9], double out21[21]);
void   orc_quat_to_rot(const double q[4], double R[9]);

void   orc_fapply(const orc_grid* g, const double* ddw, const double* u, double* f);
void   orc_diagonal(const orc_grid* g, const double* ddw, double* diag);
void   orc_fsmooth(const orc_grid* g, const double* ddw, const double* diag,
                   double* x, const double* b, double omega);
void   orc_residual(const orc_grid* g, const double* ddw, const double* x,
                    const double* b, double* r);
void   orc_restriction(const orc_grid* fine_g, const double* fine, double* crse);
void   orc_interpolation(const orc_grid* fine_g, double* fine, const double* crse);
void   orc_average_ddw(const orc_grid* fine_g, const double* fine_ddw, double* crse_ddw);
double orc_norm_inf(const orc_grid* g, const double* v);

void   orc_bc_init(const orc_grid* g, double* rhs, int homogeneous);
void   orc_newton_rhs(const orc_grid* g, const double* ddw, const double* F0,
                      const double* u, const double* b, double* rhs);
void   orc_stress(const orc_grid* g, const double* ddw, const double* F0,
                  const double* u, double* sigma9);
void   orc_traction_xhi(const orc_grid* g, const double* ddw, const double* F0,
                        const double* u, double trac[3]);

int    orc_solve(const orc_grid* g, const double* ddw, const orc_solver_params* p,
                 double* x, const double* b, double tol_rel, double tol_abs,
                 orc_report* rep);
/* orc_solve in pieces: begin (prepareForSolve + first residual), iterate
 * (up to max_steps more MLMG iterations; returns the status so far: 0
 * converged, 1 still running / max_iter reached, 2 NaN), end (frees the
 * state, fills rep).  x must be the same array across the calls. */
typedef struct orc_session orc_session;
orc_session* orc_solve_begin(const orc_grid* g, const double* ddw, const orc_solver_params* p, const double* x,
                             const double* b, double tol_rel, double tol_abs);
int    orc_solve_iterate(orc_session* s, double* x, int max_steps);
int    orc_solve_end(orc_session* s, double* x, orc_report* rep);
void   orc_strain_energy(const orc_grid* g, const double* ddw, const double* u, double* eps9, double* energy);
int    orc_bottom_solve(const orc_grid* g, const double* ddw, const double* diag, const double* res,
                        double* cor, const orc_solver_params* p);
int    orc_newton_solve(const orc_grid* g, const double* ddw, const double* F0,
                        const orc_solver_params* p, double* u, const double* b,
                        double tol_rel, double tol_abs, orc_report* rep);

#ifdef __cplusplus
}
#endif
#endif
