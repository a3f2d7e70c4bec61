// plotfile.cu -- nodal plotfile output in the AMReX plotfile format (host code).
//
// Restates what Alamo's Integrator::WritePlotFile (Integrator.cpp:795-1055)
// produces for its nodal fields on one level and one box: the directory
// <plot_file>/<step, 5 digits>node holding
//   Header                  the plotfile header ("HyperCLaw-V1.1": component
//                           names, geometry, level and grid extents)
//   Level_0/Cell_H          the FabArray header of the level (VisMF header
//                           version 1, written "NFiles"; one nodal box;
//                           per-component minima and maxima in scientific
//                           notation with 16 digits after the point)
//   Level_0/Cell_D_00000    one FAB: a text header line, then the components
//                           one after the other as little-endian IEEE doubles,
//                           i fastest over the (n+1)^3 nodes
//   Checkpoint              the level's cell-centred BoxArray
// and a line naming the header appended to <plot_file>/nodeoutput.visit.
// Component names follow Set::Field: a 3-component field `disp` is written as
// disp_x, disp_y, disp_z (Set.H:172-186), a 9-component field as
// stress_xx, stress_xy, ... stress_zz in row-major order (Set.H:209-234).
#include <cuda_runtime.h>

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "agb.h"
#include "agb_internal.h"

namespace {

using agb::set_error;

bool make_dir(const std::string& p)
{
    if (mkdir(p.c_str(), 0755) == 0) return true;
    return errno == EEXIST;
}

std::string box_str(int h0, int h1, int h2, int t)
{
    char b[160];
    snprintf(b, sizeof(b), "((0,0,0) (%d,%d,%d) (%d,%d,%d))", h0, h1, h2, t, t, t);
    return b;
}

const char* vec_suffix[3] = {"_x", "_y", "_z"};
const char* mat_suffix[9] = {"_xx", "_xy", "_xz", "_yx", "_yy", "_yz", "_zx", "_zy", "_zz"};

}  // namespace

extern "C" agb_status agb_write_node_plotfile(const char* plot_file, int step, double time, const int n_cells[3],
                                              const double prob_lo[3], const double prob_hi[3], int nfields,
                                              const char* const* names, const int* ncomp,
                                              const double* const* fields, int mem)
{
    if (!plot_file || !n_cells || !prob_lo || !prob_hi || nfields < 1 || !names || !ncomp || !fields) {
        set_error("agb_write_node_plotfile: null argument");
        return AGB_BADARG;
    }
    for (int d = 0; d < 3; d++)
        if (n_cells[d] < 1 || !(prob_hi[d] > prob_lo[d])) {
            set_error("agb_write_node_plotfile: bad box");
            return AGB_BADARG;
        }
    if (step < 0 || step > 99999) {
        set_error("agb_write_node_plotfile: step must be in 0..99999");
        return AGB_BADARG;
    }
    std::vector<std::string> comp_names;
    for (int f = 0; f < nfields; f++) {
        if (!names[f] || !fields[f] || !(ncomp[f] == 1 || ncomp[f] == 3 || ncomp[f] == 9)) {
            set_error("agb_write_node_plotfile: every field needs a name, data and 1, 3 or 9 components");
            return AGB_BADARG;
        }
        for (int c = 0; c < ncomp[f]; c++)
            comp_names.push_back(std::string(names[f]) +
                                 (ncomp[f] == 3 ? vec_suffix[c] : (ncomp[f] == 9 ? mat_suffix[c] : "")));
    }
    const int nc = (int)comp_names.size();
    const long long N = (long long)(n_cells[0] + 1) * (n_cells[1] + 1) * (n_cells[2] + 1);

    // gather every component on the host, in file order
    std::vector<double> data((size_t)nc * N);
    size_t off = 0;
    for (int f = 0; f < nfields; f++) {
        const size_t bytes = sizeof(double) * (size_t)ncomp[f] * N;
        if (mem == AGB_MEM_DEVICE) {
            if (cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess ||
                cudaMemcpy(data.data() + off, fields[f], bytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
                set_error("agb_write_node_plotfile: device copy failed");
                return AGB_CUDA;
            }
        } else {
            memcpy(data.data() + off, fields[f], bytes);
        }
        off += (size_t)ncomp[f] * N;
    }
    std::vector<double> mn(nc), mx(nc);
    for (int c = 0; c < nc; c++) {
        const double* p = data.data() + (size_t)c * N;
        double a = p[0], b = p[0];
        for (long long q = 1; q < N; q++) {
            a = p[q] < a ? p[q] : a;
            b = p[q] > b ? p[q] : b;
        }
        mn[c] = a;
        mx[c] = b;
    }

    char stepname[16];
    snprintf(stepname, sizeof(stepname), "%05d", step);
    const std::string root = plot_file;
    const std::string dir = root + "/" + stepname + "node";
    if (!make_dir(root) || !make_dir(dir) || !make_dir(dir + "/Level_0")) {
        set_error(("agb_write_node_plotfile: cannot create " + dir).c_str());
        return AGB_BADARG;
    }
    double dx[3];
    for (int d = 0; d < 3; d++) dx[d] = (prob_hi[d] - prob_lo[d]) / n_cells[d];
    const std::string cellbox = box_str(n_cells[0] - 1, n_cells[1] - 1, n_cells[2] - 1, 0);
    const std::string nodebox = box_str(n_cells[0], n_cells[1], n_cells[2], 1);

    // Header
    {
        FILE* h = fopen((dir + "/Header").c_str(), "w");
        if (!h) {
            set_error("agb_write_node_plotfile: cannot write Header");
            return AGB_BADARG;
        }
        fprintf(h, "HyperCLaw-V1.1\n%d\n", nc);
        for (const auto& s : comp_names) fprintf(h, "%s\n", s.c_str());
        fprintf(h, "3\n%.17g\n0\n", time);
        fprintf(h, "%.17g %.17g %.17g \n", prob_lo[0], prob_lo[1], prob_lo[2]);
        fprintf(h, "%.17g %.17g %.17g \n", prob_hi[0], prob_hi[1], prob_hi[2]);
        fprintf(h, "\n%s \n%d \n", cellbox.c_str(), step);
        fprintf(h, "%.17g %.17g %.17g \n", dx[0], dx[1], dx[2]);
        fprintf(h, "0\n0\n");
        fprintf(h, "0 1 %.17g\n%d\n", time, step);
        for (int d = 0; d < 3; d++) fprintf(h, "%.17g %.17g\n", prob_lo[d], prob_hi[d]);
        fprintf(h, "Level_0/Cell\n");
        fclose(h);
    }
    // FabArray header
    {
        FILE* h = fopen((dir + "/Level_0/Cell_H").c_str(), "w");
        if (!h) {
            set_error("agb_write_node_plotfile: cannot write Cell_H");
            return AGB_BADARG;
        }
        fprintf(h, "1\n1\n%d\n0\n(1 0\n%s\n)\n1\nFabOnDisk: Cell_D_00000 0\n\n", nc, nodebox.c_str());
        fprintf(h, "1,%d\n", nc);
        for (int c = 0; c < nc; c++) fprintf(h, "%.16e,", mn[c]);
        fprintf(h, "\n\n1,%d\n", nc);
        for (int c = 0; c < nc; c++) fprintf(h, "%.16e,", mx[c]);
        fprintf(h, "\n\n");
        fclose(h);
    }
    // FAB
    {
        FILE* d = fopen((dir + "/Level_0/Cell_D_00000").c_str(), "wb");
        if (!d) {
            set_error("agb_write_node_plotfile: cannot write Cell_D_00000");
            return AGB_BADARG;
        }
        fprintf(d, "FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))%s %d\n", nodebox.c_str(), nc);
        // doubles as stored in memory: little-endian on every host this library builds for
        const size_t w = fwrite(data.data(), sizeof(double), data.size(), d);
        fclose(d);
        if (w != data.size()) {
            set_error("agb_write_node_plotfile: short write");
            return AGB_BADARG;
        }
    }
    // the level's cell-centred BoxArray
    {
        FILE* c = fopen((dir + "/Checkpoint").c_str(), "w");
        if (c) {
            fprintf(c, "(1 0\n%s\n)", cellbox.c_str());
            fclose(c);
        }
    }
    {
        FILE* v = fopen((root + "/nodeoutput.visit").c_str(), step == 0 ? "w" : "a");
        if (v) {
            fprintf(v, "%snode/Header\n", stepname);
            fclose(v);
        }
    }
    return AGB_OK;
}
