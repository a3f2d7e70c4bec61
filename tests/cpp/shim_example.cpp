// A caller written against the reference's call shape (Operator::Elastic,
// Solver::Nonlocal::Newton) through include/agb.hpp: tests/Solid's
// linear-cubic tension case at t = 0.5 (u_x = 0.005 on +x), 4^3 cells.
// Prints the xhi traction; exit code 0 on success.
#include <cstdio>
#include <vector>

#include "agb.hpp"

int main()
{
    using agb::BC::Constant;
    const int n = 4;
    const size_t N = (n + 1) * (n + 1) * (n + 1);
    agb::Operator::Elastic<AGB_MAJORMINOR> op({n, n, n}, {1.0 / n, 1.0 / n, 1.0 / n});

    // TensionTest uniaxial_stress, DISP mode (TensionTest.H:115-214)
    Constant bc;
    for (int f = 0; f < AGB_NFACES; f++)
        for (int d = 0; d < 3; d++) bc.Set(f, d, Constant::Traction, 0.0);
    const int xlo[] = {AGB_XLO, AGB_XLO_YLO, AGB_XLO_YHI, AGB_ZLO_XLO, AGB_ZHI_XLO, AGB_XLO_YLO_ZLO, AGB_XLO_YLO_ZHI,
                       AGB_XLO_YHI_ZLO, AGB_XLO_YHI_ZHI};
    const int xhi[] = {AGB_XHI, AGB_XHI_YLO, AGB_XHI_YHI, AGB_ZLO_XHI, AGB_ZHI_XHI, AGB_XHI_YLO_ZLO, AGB_XHI_YLO_ZHI,
                       AGB_XHI_YHI_ZLO, AGB_XHI_YHI_ZHI};
    const int ylo[] = {AGB_YLO, AGB_XLO_YLO, AGB_XHI_YLO, AGB_YLO_ZLO, AGB_YLO_ZHI, AGB_XLO_YLO_ZLO, AGB_XLO_YLO_ZHI,
                       AGB_XHI_YLO_ZLO, AGB_XHI_YLO_ZHI};
    const int zlo[] = {AGB_ZLO, AGB_YLO_ZLO, AGB_YHI_ZLO, AGB_ZLO_XLO, AGB_ZLO_XHI, AGB_XLO_YLO_ZLO, AGB_XLO_YHI_ZLO,
                       AGB_XHI_YLO_ZLO, AGB_XHI_YHI_ZLO};
    for (int f : xlo) bc.Set(f, 0, Constant::Displacement, 0.0);
    for (int f : xhi) bc.Set(f, 0, Constant::Displacement, 0.005);
    for (int f : ylo) bc.Set(f, 1, Constant::Displacement, 0.0);
    for (int f : zlo) bc.Set(f, 2, Constant::Displacement, 0.0);
    op.SetBC(&bc);

    // Matrix4<3,MajorMinor>::Cubic(168.3, 1.221, 0.757) with R = I
    double C[21] = {0};
    C[0] = C[15] = C[20] = 168.3;
    C[3] = C[5] = C[17] = 1.221;
    C[6] = C[11] = C[18] = 0.757;
    std::vector<double> ddw(21 * N);
    for (size_t p = 0; p < N; p++)
        for (int m = 0; m < 21; m++) ddw[21 * p + m] = C[m];
    op.SetModel(ddw.data());

    std::vector<double> b(3 * N, 0.0), u(3 * N, 0.0);
    agb::check(agb_bc_init(op.handle(), b.data(), 0, AGB_MEM_HOST));
    agb::Solver::Nonlocal::Newton solver(op);
    double res = solver.solve(u.data(), b.data(), nullptr, 1e-10, 0.0);
    double trac[3];
    agb::check(agb_traction_xhi(op.handle(), nullptr, u.data(), trac, AGB_MEM_HOST));
    std::printf("iterations %d residual %.3e trac_xhi_x %.6f\n", solver.report().iterations, res, trac[0]);
    // tests/Solid/reference/linear-cubic.dat at t = 0.5: 0.841466 (tolerance 1e-4)
    const double ref = 0.841466;
    return (trac[0] - ref) / ref < 1e-4 && (ref - trac[0]) / ref < 1e-4 ? 0 : 1;
}
