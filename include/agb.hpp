// agb.hpp -- header-only C++ shim over the C ABI of agb.h that keeps the call
// shape of Alamo's Operator::Elastic<SYM> and Solver::Nonlocal::Linear /
// Newton for single-box, single-level callers (Integrator::Base::Mechanics
// TimeStepBegin, Newton::solve).  Fields are plain arrays in the memory layout
// of the reference's nodal MultiFab of one box (component-major, i fastest);
// a caller holding a MultiFab with one FAB passes fab.dataPtr() after
// trimming ghost nodes.  Errors throw agb::Error (the reference aborts through
// Util::Abort); the C ABI itself never throws.
#ifndef AGB_HPP
#define AGB_HPP

#include <array>
#include <stdexcept>
#include <string>
#include <vector>

#include "agb.h"

namespace agb {

struct Error : std::runtime_error {
    agb_status status;
    Error(agb_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(agb_status s)
{
    if (s != AGB_OK) throw Error(s, std::string("alamo_gb300: ") + agb_last_error());
}

namespace BC {
// BC::Operator::Elastic::Constant (BC/Operator/Elastic/Constant.H:31-194)
class Constant {
public:
    enum Type { Displacement = AGB_BC_DISP, Traction = AGB_BC_TRAC, Periodic = AGB_BC_PERIODIC,
                Neumann = AGB_BC_NEUMANN, None = AGB_BC_NONE };
    Constant()
    {
        for (int f = 0; f < AGB_NFACES; f++)
            for (int d = 0; d < 3; d++) {
                m.type[f][d] = AGB_BC_DISP;
                m.val[f][d] = 0.0;
            }
    }
    // Constant::Set(face, direction, type, value), Constant.H:53-61
    void Set(int face, int direction, Type type, double value)
    {
        m.type[face][direction] = type;
        m.val[face][direction] = value;
    }
    const agb_bc& c() const { return m; }

protected:
    agb_bc m;
};
}  // namespace BC

namespace Operator {
// Operator::Elastic<SYM> on one box (Operator/Elastic.H:21-190)
template <int SYM> class Elastic {
public:
    Elastic(std::array<int, 3> n_cells, std::array<double, 3> dx, std::array<int, 3> periodic = {0, 0, 0},
            int max_coarsening_level = 30)
    {
        check(agb_op_create(n_cells.data(), dx.data(), periodic.data(), SYM, max_coarsening_level, &op_));
    }
    ~Elastic() { agb_op_destroy(op_); }
    Elastic(const Elastic&) = delete;
    Elastic& operator=(const Elastic&) = delete;

    void SetBC(const BC::Constant* bc) { check(agb_op_set_bc(op_, &bc->c())); }
    // SetModel(amrlev, MultiTab): one Matrix4 per node, AoS as in BaseFab<Matrix4>
    void SetModel(const double* ddw, int mem = AGB_MEM_HOST) { check(agb_op_set_model(op_, ddw, AGB_LAYOUT_AOS, mem)); }
    void SetUniform(bool u) { check(agb_op_set_uniform(op_, u ? 1 : 0)); }
    void SetOmega(double w) { check(agb_op_set_omega(op_, w)); }
    void prepareForSolve() { check(agb_op_prepare(op_)); }
    int NMGLevels() const
    {
        int n = 0;
        check(agb_op_num_levels(op_, &n));
        return n;
    }
    // MLNodeLinOp virtuals with amrlev = 0
    void Fapply(int amrlev, int mglev, double* f, const double* u, int mem = AGB_MEM_HOST) const
    {
        (void)amrlev;
        check(agb_op_fapply(op_, mglev, f, u, mem));
    }
    void Fsmooth(int amrlev, int mglev, double* x, const double* b, int mem = AGB_MEM_HOST) const
    {
        (void)amrlev;
        check(agb_op_fsmooth(op_, mglev, x, b, mem));
    }
    void Diagonal(int amrlev, int mglev, double* diag, int mem = AGB_MEM_HOST)
    {
        (void)amrlev;
        check(agb_op_diagonal(op_, mglev, diag, mem));
    }
    void restriction(int amrlev, int cmglev, double* crse, const double* fine, int mem = AGB_MEM_HOST) const
    {
        (void)amrlev;
        check(agb_op_restriction(op_, cmglev, crse, fine, mem));
    }
    void interpolation(int amrlev, int fmglev, double* fine, const double* crse, int mem = AGB_MEM_HOST) const
    {
        (void)amrlev;
        check(agb_op_interpolation(op_, fmglev, fine, crse, mem));
    }
    agb_op handle() const { return op_; }

private:
    agb_op op_ = nullptr;
};
}  // namespace Operator

namespace Solver {
namespace Nonlocal {
// Solver::Nonlocal::Linear (Solver/Nonlocal/Linear.H:18-392)
class Linear {
public:
    Linear() { agb_default_params(&p_); }
    template <class OP> explicit Linear(OP& op) : Linear() { Define(op); }
    ~Linear() { Clear(); }
    template <class OP> void Define(OP& op)
    {
        if (s_) throw Error(AGB_STATE, "Solver cannot be re-defined");
        op_ = op.handle();
        check(agb_solver_create(op_, &p_, &s_));
    }
    void Clear()
    {
        if (s_) agb_solver_destroy(s_);
        s_ = nullptr;
    }
    // Linear::solve(sol, rhs, tol_rel, tol_abs): returns the final ||b - A x||_inf
    double solve(double* sol, const double* rhs, double tol_rel, double tol_abs, int mem = AGB_MEM_HOST)
    {
        check(agb_solve(s_, sol, rhs, tol_rel, tol_abs, mem, &last_));
        return last_.res_final;
    }
    void apply(double* out, const double* in, int mem = AGB_MEM_HOST) { check(agb_apply(s_, out, in, mem)); }
    void setMaxIter(int v) { p_.max_iter = v; }
    void setBottomMaxIter(int v) { p_.bottom_max_iter = v; }
    void setMaxFmgIter(int v) { p_.max_fmg_iter = v; }
    void setFixedIter(int v) { p_.fixed_iter = v; }
    void setVerbose(int v) { p_.verbose = v; }
    void setPreSmooth(int v) { p_.pre_smooth = v; }
    void setPostSmooth(int v) { p_.post_smooth = v; }
    void setMixedPrecision(bool on) { p_.precision = on ? AGB_PREC_MIXED : AGB_PREC_F64; }
    // mixed precision: flexible GCR over the FP32 cycle with k stored
    // directions (0: the cycles alone, as MLMG iterates; no reference setter)
    void setKrylov(int k) { p_.krylov = k; }
    const agb_solve_report& report() const { return last_; }

protected:
    agb_solver_params p_;
    agb_solver s_ = nullptr;
    agb_op op_ = nullptr;
    agb_solve_report last_{};
};

// Solver::Nonlocal::Newton for linear models: one Newton iteration
class Newton : public Linear {
public:
    using Linear::Linear;
    double solve(double* u, const double* b, const double* F0, double tol_rel, double tol_abs,
                 int mem = AGB_MEM_HOST)
    {
        check(agb_newton_solve(s_, F0, u, b, tol_rel, tol_abs, mem, &last_));
        return last_.res_final;
    }
};
}  // namespace Nonlocal
}  // namespace Solver

}  // namespace agb

#endif
