/*
 * agb_oracle.c -- CPU restatement of Alamo's nodal linear-elastic multigrid
 * path.  TEST INFRASTRUCTURE ONLY (see agb_oracle.h): the checker for the
 * CUDA library, never part of the product.
 *
 * Build: see oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off).
 */
#include "agb_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* BC/Operator/Elastic/Elastic.H:79-80 -- the reference's truncated normals */
#define SQRT3INV 0.57735026919
#define SQRT2INV 0.70710678118

enum { ST_LO = 0, ST_HI = 1, ST_CENTRAL = 2 }; /* Numeric::StencilType, Stencil.H:21 */

int orc_ncoef(int sym) { return sym == ORC_ISO ? 2 : 21; }

int orc_num_threads(void) { return omp_get_max_threads(); }

long orc_nnodes(const orc_grid* g)
{
    return (long)(g->n[0] + 1) * (g->n[1] + 1) * (g->n[2] + 1);
}

static inline long IDX(const orc_grid* g, int i, int j, int k)
{
    return i + (long)(g->n[0] + 1) * (j + (long)(g->n[1] + 1) * k);
}

/* periodic image of a node index (node n duplicates node 0) */
static inline int WRAP(int i, int n, int per)
{
    if (per) {
        if (i < 0) return i + n;
        if (i > n) return i - n;
    }
    return i;
}

typedef struct {
    const orc_grid* g;
    long N;
} ctx_t;

static inline double UV(const orc_grid* g, long N, const double* u, int i, int j, int k, int p)
{
    i = WRAP(i, g->n[0], g->periodic[0]);
    j = WRAP(j, g->n[1], g->periodic[1]);
    k = WRAP(k, g->n[2], g->periodic[2]);
    return u[p * N + IDX(g, i, j, k)];
}

static inline const double* CV(const orc_grid* g, const double* ddw, int i, int j, int k)
{
    i = WRAP(i, g->n[0], g->periodic[0]);
    j = WRAP(j, g->n[1], g->periodic[1]);
    k = WRAP(k, g->n[2], g->periodic[2]);
    return ddw + IDX(g, i, j, k) * orc_ncoef(g->sym);
}

/* ------------------------------------------------------------------------ */
/* Set::Matrix4 contractions                                                 */
/* ------------------------------------------------------------------------ */

/* Matrix4<3,Isotropic> * Matrix, Set/Matrix4_Isotropic.H:137-157 (storage: lambda, mu) */
static void iso_mul_mat(const double* C, double b[3][3], double r[3][3])
{
    const double lambda = C[0], mu = C[1];
    r[0][0] = (lambda + 2. * mu) * b[0][0] + lambda * b[1][1] + lambda * b[2][2];
    r[1][1] = lambda * b[0][0] + (lambda + 2. * mu) * b[1][1] + lambda * b[2][2];
    r[2][2] = lambda * b[0][0] + lambda * b[1][1] + (lambda + 2. * mu) * b[2][2];
    r[1][2] = mu * (b[1][2] + b[2][1]); r[2][1] = r[1][2];
    r[2][0] = mu * (b[2][0] + b[0][2]); r[0][2] = r[2][0];
    r[0][1] = mu * (b[0][1] + b[1][0]); r[1][0] = r[0][1];
}

/* Matrix4<3,Isotropic> * Matrix3, Set/Matrix4_Isotropic.H:163-173; b[i][j][k] = b(i,j,k) */
static void iso_mul_m3(const double* C, double b[3][3][3], double r[3])
{
    const double lambda = C[0], mu = C[1];
    for (int i = 0; i < 3; i++) {
        r[i] = 0.0;
        for (int j = 0; j < 3; j++)
            r[i] += mu * (b[i][j][j] + b[j][i][j]) + lambda * b[j][j][i];
    }
}

/* Matrix4<3,MajorMinor> * Matrix, Set/Matrix4_MajorMinor.H:675-691 */
static void mm_mul_mat(const double* a, double b[3][3], double r[3][3])
{
    r[0][0] = a[0] * b[0][0] + a[1] * (b[0][1] + b[1][0]) + a[2] * (b[0][2] + b[2][0]) + a[3] * b[1][1] + a[4] * (b[1][2] + b[2][1]) + a[5] * b[2][2];
    r[1][1] = a[3] * b[0][0] + a[8] * (b[0][1] + b[1][0]) + a[12] * (b[0][2] + b[2][0]) + a[15] * b[1][1] + a[16] * (b[1][2] + b[2][1]) + a[17] * b[2][2];
    r[2][2] = a[5] * b[0][0] + a[10] * (b[0][1] + b[1][0]) + a[14] * (b[0][2] + b[2][0]) + a[17] * b[1][1] + a[19] * (b[1][2] + b[2][1]) + a[20] * b[2][2];
    r[1][2] = a[4] * b[0][0] + a[9] * (b[0][1] + b[1][0]) + a[13] * (b[0][2] + b[2][0]) + a[16] * b[1][1] + a[18] * (b[1][2] + b[2][1]) + a[19] * b[2][2];
    r[2][0] = a[2] * b[0][0] + a[7] * (b[0][1] + b[1][0]) + a[11] * (b[0][2] + b[2][0]) + a[12] * b[1][1] + a[13] * (b[1][2] + b[2][1]) + a[14] * b[2][2];
    r[0][1] = a[1] * b[0][0] + a[6] * (b[0][1] + b[1][0]) + a[7] * (b[0][2] + b[2][0]) + a[8] * b[1][1] + a[9] * (b[1][2] + b[2][1]) + a[10] * b[2][2];
    r[2][1] = r[1][2];
    r[0][2] = r[2][0];
    r[1][0] = r[0][1];
}

/* Matrix4<3,MajorMinor> * Matrix3, Set/Matrix4_MajorMinor.H:709-767 */
static void mm_mul_m3(const double* a, double b[3][3][3], double r[3])
{
#define B(i, j, k) b[i][j][k]
    r[0] = a[0] * B(0,0,0) +
           a[1] * (B(0,1,0) + B(1,0,0) + B(0,0,1)) +
           a[2] * (B(0,2,0) + B(2,0,0) + B(0,0,2)) +
           a[3] * B(1,1,0) +
           a[4] * (B(1,2,0) + B(2,1,0)) +
           a[5] * B(2,2,0) +
           a[6] * (B(0,1,1) + B(1,0,1)) +
           a[7] * (B(0,2,1) + B(2,0,1) + B(0,1,2) + B(1,0,2)) +
           a[8] * B(1,1,1) +
           a[9] * (B(1,2,1) + B(2,1,1)) +
           a[10] * B(2,2,1) +
           a[11] * (B(0,2,2) + B(2,0,2)) +
           a[12] * B(1,1,2) +
           a[13] * (B(1,2,2) + B(2,1,2)) +
           a[14] * B(2,2,2);
    r[1] = a[1] * B(0,0,0) +
           a[4] * B(0,0,2) +
           a[3] * B(0,0,1) +
           a[6] * (B(0,1,0) + B(1,0,0)) +
           a[7] * (B(0,2,0) + B(2,0,0)) +
           a[8] * (B(1,1,0) + B(0,1,1) + B(1,0,1)) +
           a[9] * (B(1,2,0) + B(2,1,0) + B(0,1,2) + B(1,0,2)) +
           a[10] * B(2,2,0) +
           a[12] * (B(0,2,1) + B(2,0,1)) +
           a[13] * (B(0,2,2) + B(2,0,2)) +
           a[15] * B(1,1,1) +
           a[16] * (B(1,2,1) + B(2,1,1) + B(1,1,2)) +
           a[17] * B(2,2,1) +
           a[18] * (B(1,2,2) + B(2,1,2)) +
           a[19] * B(2,2,2);
    r[2] = a[2] * B(0,0,0) +
           a[4] * B(0,0,1) +
           a[5] * B(0,0,2) +
           a[7] * (B(0,1,0) + B(1,0,0)) +
           a[9] * (B(0,1,1) + B(1,0,1)) +
           a[10] * (B(0,1,2) + B(1,0,2)) +
           a[11] * (B(0,2,0) + B(2,0,0)) +
           a[12] * B(1,1,0) +
           a[13] * (B(1,2,0) + B(2,1,0) + B(0,2,1) + B(2,0,1)) +
           a[14] * (B(2,2,0) + B(0,2,2) + B(2,0,2)) +
           a[16] * B(1,1,1) +
           a[17] * B(1,1,2) +
           a[18] * (B(1,2,1) + B(2,1,1)) +
           a[19] * (B(2,2,1) + B(1,2,2) + B(2,1,2)) +
           a[20] * B(2,2,2);
#undef B
}

static void c_mul_mat(int sym, const double* C, double b[3][3], double r[3][3])
{
    if (sym == ORC_ISO) iso_mul_mat(C, b, r);
    else mm_mul_mat(C, b, r);
}

static void c_mul_m3(int sym, const double* C, double b[3][3][3], double r[3])
{
    if (sym == ORC_ISO) iso_mul_m3(C, b, r);
    else mm_mul_m3(C, b, r);
}

/* MajorMinor uid -> storage slot, Set/Matrix4_MajorMinor.H:327-375 */
static int mm_slot(int i, int j, int k, int l)
{
    int uid = i + 3 * j + 9 * k + 27 * l;
    switch (uid) {
    case 0: return 0;
    case 27: case 9: case 3: case 1: return 1;
    case 54: case 18: case 6: case 2: return 2;
    case 36: case 4: return 3;
    case 63: case 45: case 7: case 5: return 4;
    case 72: case 8: return 5;
    case 30: case 12: case 28: case 10: return 6;
    case 57: case 21: case 33: case 15: case 55: case 19: case 29: case 11: return 7;
    case 39: case 37: case 31: case 13: return 8;
    case 66: case 48: case 64: case 46: case 34: case 16: case 32: case 14: return 9;
    case 75: case 73: case 35: case 17: return 10;
    case 60: case 24: case 56: case 20: return 11;
    case 42: case 58: case 22: case 38: return 12;
    case 69: case 51: case 61: case 25: case 65: case 47: case 59: case 23: return 13;
    case 78: case 74: case 62: case 26: return 14;
    case 40: return 15;
    case 67: case 49: case 43: case 41: return 16;
    case 76: case 44: return 17;
    case 70: case 52: case 68: case 50: return 18;
    case 79: case 77: case 71: case 53: return 19;
    case 80: return 20;
    }
    return -1;
}

/*
 * Matrix4<3,MajorMinor>::Cubic(C11,C12,C44,R), Set/Matrix4_MajorMinor.H:518-547.
 * The reference builds a cubic tensor that is NOT minor-symmetric (C_ijji = 0
 * for i != j), rotates it, and writes every (p,q,s,t) into the 21-slot store in
 * loop order; each slot therefore keeps the value of the LAST (p,q,s,t) that
 * maps to it.  Restated here with the same loop and the same aliasing.
 */
void orc_cubic(double C11, double C12, double C44, const double R[9], double out[21])
{
    double Ct[3][3][3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) {
                    if (i == j && j == k && k == l) Ct[i][j][k][l] = C11;
                    else if (i == k && j == l) Ct[i][j][k][l] = C44;
                    else if (i == j && k == l) Ct[i][j][k][l] = C12;
                    else Ct[i][j][k][l] = 0.0;
                }
#define RR(a, b) R[(a) * 3 + (b)]
    for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++)
            for (int s = 0; s < 3; s++)
                for (int t = 0; t < 3; t++) {
                    int slot = mm_slot(p, q, s, t);
                    out[slot] = 0.0;
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++)
                            for (int k = 0; k < 3; k++)
                                for (int l = 0; l < 3; l++)
                                    out[slot] += RR(p, i) * RR(s, k) * Ct[i][j][k][l] * RR(q, j) * RR(t, l);
                }
#undef RR
}

/*
 * Rotation matrix of a quaternion (w,x,y,z), normalised first, as
 * Matrix4_MajorMinor.H:557-562 does with Eigen's q.normalized().toRotationMatrix().
 * Row-major R[3*r+c].
 */
void orc_quat_to_rot(const double q_in[4], double R[9])
{
    double n = sqrt(q_in[0] * q_in[0] + q_in[1] * q_in[1] + q_in[2] * q_in[2] + q_in[3] * q_in[3]);
    double w = q_in[0] / n, x = q_in[1] / n, y = q_in[2] / n, z = q_in[3] / n;
    double tx = 2 * x, ty = 2 * y, tz = 2 * z;
    double twx = tx * w, twy = ty * w, twz = tz * w;
    double txx = tx * x, txy = ty * x, txz = tz * x;
    double tyy = ty * y, tyz = tz * y, tzz = tz * z;
    R[0] = 1 - (tyy + tzz); R[1] = txy - twz;       R[2] = txz + twy;
    R[3] = txy + twz;       R[4] = 1 - (txx + tzz); R[5] = tyz - twx;
    R[6] = txz - twy;       R[7] = tyz + twx;       R[8] = 1 - (txx + tyy);
}

/* ------------------------------------------------------------------------ */
/* Boundary classification and boundary rows                                */
/* ------------------------------------------------------------------------ */

typedef struct {
    int mn[3], mx[3];   /* node on the lo / hi face of a non-periodic direction */
} bflags;

static inline bflags node_flags(const orc_grid* g, int i, int j, int k)
{
    bflags f;
    int ii[3] = {i, j, k};
    for (int d = 0; d < 3; d++) {
        f.mn[d] = !g->periodic[d] && ii[d] == 0;
        f.mx[d] = !g->periodic[d] && ii[d] == g->n[d];
    }
    return f;
}

static inline int is_boundary(const bflags* f)
{
    return f->mn[0] || f->mx[0] || f->mn[1] || f->mx[1] || f->mn[2] || f->mx[2];
}

/*
 * Region of a boundary node and its outward normal, in the precedence order
 * of Constant::operator(), BC/Operator/Elastic/Constant.H:373-400 (corners,
 * then YZ, ZX, XY edges, then faces).
 */
static int face_of(const bflags* f, double nrm[3])
{
    const int xl = f->mn[0], xh = f->mx[0], yl = f->mn[1], yh = f->mx[1], zl = f->mn[2], zh = f->mx[2];
    const double s3 = SQRT3INV, s2 = SQRT2INV;
#define RET(face, a, b, c) do { nrm[0] = (a); nrm[1] = (b); nrm[2] = (c); return (face); } while (0)
    if (xl && yl && zl) RET(ORC_XLO_YLO_ZLO, -s3, -s3, -s3);
    if (xl && yl && zh) RET(ORC_XLO_YLO_ZHI, -s3, -s3, +s3);
    if (xl && yh && zl) RET(ORC_XLO_YHI_ZLO, -s3, +s3, -s3);
    if (xl && yh && zh) RET(ORC_XLO_YHI_ZHI, -s3, +s3, +s3);
    if (xh && yl && zl) RET(ORC_XHI_YLO_ZLO, +s3, -s3, -s3);
    if (xh && yl && zh) RET(ORC_XHI_YLO_ZHI, +s3, -s3, +s3);
    if (xh && yh && zl) RET(ORC_XHI_YHI_ZLO, +s3, +s3, -s3);
    if (xh && yh && zh) RET(ORC_XHI_YHI_ZHI, +s3, +s3, +s3);
    if (yl && zl) RET(ORC_YLO_ZLO, 0, -s2, -s2);
    if (yl && zh) RET(ORC_YLO_ZHI, 0, -s2, +s2);
    if (yh && zl) RET(ORC_YHI_ZLO, 0, +s2, -s2);
    if (yh && zh) RET(ORC_YHI_ZHI, 0, +s2, +s2);
    if (zl && xl) RET(ORC_ZLO_XLO, -s2, 0, -s2);
    if (zl && xh) RET(ORC_ZLO_XHI, +s2, 0, -s2);
    if (zh && xl) RET(ORC_ZHI_XLO, -s2, 0, +s2);
    if (zh && xh) RET(ORC_ZHI_XHI, +s2, 0, +s2);
    if (xl && yl) RET(ORC_XLO_YLO, -s2, -s2, 0);
    if (xl && yh) RET(ORC_XLO_YHI, -s2, +s2, 0);
    if (xh && yl) RET(ORC_XHI_YLO, +s2, -s2, 0);
    if (xh && yh) RET(ORC_XHI_YHI, +s2, +s2, 0);
    if (xl) RET(ORC_XLO, -1, 0, 0);
    if (xh) RET(ORC_XHI, +1, 0, 0);
    if (yl) RET(ORC_YLO, 0, -1, 0);
    if (yh) RET(ORC_YHI, 0, +1, 0);
    if (zl) RET(ORC_ZLO, 0, 0, -1);
    if (zh) RET(ORC_ZHI, 0, 0, +1);
#undef RET
    nrm[0] = nrm[1] = nrm[2] = 0;
    return -1;
}

/* Constant::set, BC/Operator/Elastic/Constant.H:408-425 */
static void bc_set(const int type[3], const double u[3], double gradu[3][3],
                   double sig[3][3], const double n[3], double f[3])
{
    for (int i = 0; i < 3; i++) {
        f[i] = 0.0;
        if (type[i] == ORC_DISP) f[i] = u[i];
        else if (type[i] == ORC_TRAC) f[i] = sig[i][0] * n[0] + sig[i][1] * n[1] + sig[i][2] * n[2];
        else if (type[i] == ORC_NEUMANN) f[i] = gradu[i][0] * n[0] + gradu[i][1] * n[1] + gradu[i][2] * n[2];
    }
}

/* ------------------------------------------------------------------------ */
/* Stencils, Numeric/Stencil.H                                               */
/* ------------------------------------------------------------------------ */

static inline void stencil_types(const bflags* f, int st[3])
{
    /* GetStencil, Stencil.H:41-60: lo face -> Hi (forward), hi face -> Lo (backward) */
    for (int d = 0; d < 3; d++) st[d] = f->mn[d] ? ST_HI : (f->mx[d] ? ST_LO : ST_CENTRAL);
}

/* Stencil<T,1,0,0>::D etc., Stencil.H:70-191 */
static double d1(const orc_grid* g, long N, const double* u, int i, int j, int k, int p, int d, int st)
{
    int o[3] = {0, 0, 0};
    o[d] = 1;
    double h = g->dx[d];
    if (st == ST_LO) return (UV(g, N, u, i, j, k, p) - UV(g, N, u, i - o[0], j - o[1], k - o[2], p)) / h;
    if (st == ST_HI) return (UV(g, N, u, i + o[0], j + o[1], k + o[2], p) - UV(g, N, u, i, j, k, p)) / h;
    return (UV(g, N, u, i + o[0], j + o[1], k + o[2], p) - UV(g, N, u, i - o[0], j - o[1], k - o[2], p)) * 0.5 / h;
}

static void gradient(const orc_grid* g, long N, const double* u, int i, int j, int k,
                     const int st[3], double gradu[3][3])
{
    for (int p = 0; p < 3; p++)
        for (int d = 0; d < 3; d++) gradu[p][d] = d1(g, N, u, i, j, k, p, d, st[d]);
}

/* central 2nd and mixed derivatives, Stencil.H:197-301 (default Central stencil) */
static void hessian(const orc_grid* g, long N, const double* u, int i, int j, int k, double gg[3][3][3])
{
    const double* dx = g->dx;
    for (int p = 0; p < 3; p++) {
#define U(a, b, c) UV(g, N, u, i + (a), j + (b), k + (c), p)
        gg[p][0][0] = (U(1, 0, 0) - 2.0 * U(0, 0, 0) + U(-1, 0, 0)) / dx[0] / dx[0];
        gg[p][1][1] = (U(0, 1, 0) - 2.0 * U(0, 0, 0) + U(0, -1, 0)) / dx[1] / dx[1];
        gg[p][2][2] = (U(0, 0, 1) - 2.0 * U(0, 0, 0) + U(0, 0, -1)) / dx[2] / dx[2];
        gg[p][0][1] = 0.5 * 0.5 * (U(1, 1, 0) + U(-1, -1, 0) - U(1, -1, 0) - U(-1, 1, 0)) / (dx[0] * dx[1]);
        gg[p][1][0] = gg[p][0][1];
        gg[p][0][2] = 0.5 * 0.5 * (U(1, 0, 1) + U(-1, 0, -1) - U(1, 0, -1) - U(-1, 0, 1)) / (dx[0] * dx[2]);
        gg[p][1][2] = 0.5 * 0.5 * (U(0, 1, 1) + U(0, -1, -1) - U(0, 1, -1) - U(0, -1, 1)) / (dx[1] * dx[2]);
        gg[p][2][0] = gg[p][0][2];
        gg[p][2][1] = gg[p][1][2];
#undef U
    }
}

/* ------------------------------------------------------------------------ */
/* Elastic::Fapply, Operator/Elastic.cpp:141-292                             */
/* ------------------------------------------------------------------------ */

static void node_fapply(const orc_grid* g, long N, const double* ddw, const double* u,
                        int i, int j, int k, double f[3])
{
    const int nc = orc_ncoef(g->sym);
    bflags fl = node_flags(g, i, j, k);
    int st[3];
    stencil_types(&fl, st);
    double uc[3], gradu[3][3], sig[3][3];
    for (int p = 0; p < 3; p++) uc[p] = UV(g, N, u, i, j, k, p);
    gradient(g, N, u, i, j, k, st, gradu);
    const double* C = CV(g, ddw, i, j, k);
    c_mul_mat(g->sym, C, gradu, sig);                              /* Elastic.cpp:195 */
    if (is_boundary(&fl)) {                                        /* Elastic.cpp:200-203 */
        double nrm[3];
        int face = face_of(&fl, nrm);
        bc_set(g->bc_type[face], uc, gradu, sig, nrm, f);
        return;
    }
    double gg[3][3][3];
    hessian(g, N, u, i, j, k, gg);                                 /* Elastic.cpp:211-232 */
    c_mul_m3(g->sym, C, gg, f);                                    /* Elastic.cpp:243 */
    if (!g->uniform) {                                             /* Elastic.cpp:245-254 */
        double M[3][3][3], cg[21];
        for (int d = 0; d < 3; d++) {
            int o[3] = {0, 0, 0};
            o[d] = 1;
            const double* Cp = CV(g, ddw, i + o[0], j + o[1], k + o[2]);
            const double* Cm = CV(g, ddw, i - o[0], j - o[1], k - o[2]);
            for (int m = 0; m < nc; m++) cg[m] = (Cp[m] - Cm[m]) * 0.5 / g->dx[d];
            c_mul_mat(g->sym, cg, gradu, M[d]);
        }
        for (int r = 0; r < 3; r++) f[r] += (M[0][r][0] + M[1][r][1] + M[2][r][2]);
    }
}

void orc_fapply(const orc_grid* g, const double* ddw, const double* u, double* f)
{
    const long N = orc_nnodes(g);
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= g->n[2]; k++)
        for (int j = 0; j <= g->n[1]; j++)
            for (int i = 0; i <= g->n[0]; i++) {
                double r[3];
                node_fapply(g, N, ddw, u, i, j, k, r);
                long p = IDX(g, i, j, k);
                f[p] = r[0]; f[N + p] = r[1]; f[2 * N + p] = r[2];
            }
}

/* ------------------------------------------------------------------------ */
/* Elastic::Diagonal, Operator/Elastic.cpp:298-379                           */
/* ------------------------------------------------------------------------ */

void orc_diagonal(const orc_grid* g, const double* ddw, double* diag)
{
    const long N = orc_nnodes(g);
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= g->n[2]; k++)
        for (int j = 0; j <= g->n[1]; j++)
            for (int i = 0; i <= g->n[0]; i++) {
                bflags fl = node_flags(g, i, j, k);
                const double* C = CV(g, ddw, i, j, k);
                long idx = IDX(g, i, j, k);
                int bnd = is_boundary(&fl);
                for (int p = 0; p < 3; p++) {
                    double dval = 0.0;
                    if (bnd) {
                        /* Gradient_Diagonal<Matrix>, Stencil.H:906-930 */
                        double gu[3][3], sig[3][3], uu[3] = {0, 0, 0}, nrm[3], f[3];
                        for (int q = 0; q < 3; q++)
                            for (int d = 0; d < 3; d++) {
                                double e = (p == q ? 1.0 : 0.0);
                                gu[q][d] = ((!fl.mx[d] ? 0.0 : e) - (!fl.mn[d] ? 0.0 : e)) /
                                           ((fl.mn[d] || fl.mx[d] ? 1.0 : 2.0) * g->dx[d]);
                            }
                        c_mul_mat(g->sym, C, gu, sig);
                        uu[p] = 1.0;
                        int face = face_of(&fl, nrm);
                        bc_set(g->bc_type[face], uu, gu, sig, nrm, f);
                        dval = f[p];
                    } else {
                        /* Gradient_Diagonal<Matrix3>, Stencil.H:932-962 */
                        double gg[3][3][3], f[3];
                        for (int q = 0; q < 3; q++)
                            for (int a = 0; a < 3; a++)
                                for (int b = 0; b < 3; b++) gg[q][a][b] = 0.0;
                        gg[p][0][0] = -2.0 / g->dx[0] / g->dx[0];
                        gg[p][1][1] = -2.0 / g->dx[1] / g->dx[1];
                        gg[p][2][2] = -2.0 / g->dx[2] / g->dx[2];
                        c_mul_m3(g->sym, C, gg, f);
                        dval += f[p];
                    }
                    diag[p * N + idx] = dval;
                }
            }
}

/* ------------------------------------------------------------------------ */
/* Operator<Node>::Fsmooth (2 damped-Jacobi sweeps), Operator/Operator.cpp:88-154 */
/* ------------------------------------------------------------------------ */

void orc_fsmooth(const orc_grid* g, const double* ddw, const double* diag,
                 double* x, const double* b, double omega)
{
    const long N = orc_nnodes(g);
    double* Ax = (double*)malloc(sizeof(double) * 3 * N);
    for (int ctr = 0; ctr < 2; ctr++) {
        orc_fapply(g, ddw, x, Ax);
#pragma omp parallel for schedule(static)
        for (long q = 0; q < 3 * N; q++) {
            double Dx = x[q] * diag[q];
            double Rx = Ax[q] - Dx;
            x[q] = (1. - omega) * x[q] + omega * (b[q] - Rx) / diag[q];
        }
    }
    free(Ax);
}

/* Operator<Node>::solutionResidual / correctionResidual, Operator.cpp:636-657 */
void orc_residual(const orc_grid* g, const double* ddw, const double* x,
                  const double* b, double* r)
{
    const long N = orc_nnodes(g);
    orc_fapply(g, ddw, x, r);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < 3 * N; q++) r[q] = b[q] + (-1.0) * r[q];
}

double orc_norm_inf(const orc_grid* g, const double* v)
{
    const long N = orc_nnodes(g);
    double m = 0.0;
    for (long q = 0; q < 3 * N; q++) {
        double a = fabs(v[q]);
        if (a > m || a != a) m = a;
    }
    return m;
}

/* ------------------------------------------------------------------------ */
/* Full weighting shared by restriction and coefficient averaging            */
/* ------------------------------------------------------------------------ */

void orc_coarsen(const orc_grid* fine, orc_grid* crse)
{
    *crse = *fine;
    for (int d = 0; d < 3; d++) {
        crse->n[d] = fine->n[d] / 2;
        crse->dx[d] = fine->dx[d] * 2.0;
    }
}

/*
 * One coarse value of the nodal full weighting with lower-dimensional
 * stencils on the coarse domain boundary:
 *   Operator<Node>::restriction, Operator/Operator.cpp:294-352 and
 *   Elastic::averageDownCoeffsSameAmrLevel, Operator/Elastic.cpp:786-829.
 * F(a,b,c) fetches the fine value at (i+a, j+b, k+c).
 */
#define FW_BODY(F, OUT)                                                                         \
    do {                                                                                        \
        int bI = (I == lo[0] || I == hi[0]), bJ = (J == lo[1] || J == hi[1]),                   \
            bK = (K == lo[2] || K == hi[2]);                                                    \
        if (bI && bJ && bK) OUT = F(0, 0, 0);                                                   \
        else if (bJ && bK) OUT = 0.25 * F(-1, 0, 0) + 0.5 * F(0, 0, 0) + 0.25 * F(1, 0, 0);     \
        else if (bK && bI) OUT = 0.25 * F(0, -1, 0) + 0.5 * F(0, 0, 0) + 0.25 * F(0, 1, 0);     \
        else if (bI && bJ) OUT = 0.25 * F(0, 0, -1) + 0.5 * F(0, 0, 0) + 0.25 * F(0, 0, 1);     \
        else if (bI)                                                                            \
            OUT = (+F(0, -1, -1) + 2.0 * F(0, 0, -1) + F(0, 1, -1) + 2.0 * F(0, -1, 0) +         \
                   4.0 * F(0, 0, 0) + 2.0 * F(0, 1, 0) + F(0, -1, 1) + 2.0 * F(0, 0, 1) +       \
                   F(0, 1, 1)) / 16.0;                                                          \
        else if (bJ)                                                                            \
            OUT = (+F(-1, 0, -1) + 2.0 * F(-1, 0, 0) + F(-1, 0, 1) + 2.0 * F(0, 0, -1) +         \
                   4.0 * F(0, 0, 0) + 2.0 * F(0, 0, 1) + F(1, 0, -1) + 2.0 * F(1, 0, 0) +       \
                   F(1, 0, 1)) / 16.0;                                                          \
        else if (bK)                                                                            \
            OUT = (+F(-1, -1, 0) + 2.0 * F(0, -1, 0) + F(1, -1, 0) + 2.0 * F(-1, 0, 0) +         \
                   4.0 * F(0, 0, 0) + 2.0 * F(1, 0, 0) + F(-1, 1, 0) + 2.0 * F(0, 1, 0) +       \
                   F(1, 1, 0)) / 16.0;                                                          \
        else                                                                                    \
            OUT = (F(-1, -1, -1) + F(-1, -1, 1) + F(-1, 1, -1) + F(-1, 1, 1) + F(1, -1, -1) +    \
                   F(1, -1, 1) + F(1, 1, -1) + F(1, 1, 1)) / 64.0 +                             \
                  (F(0, -1, -1) + F(0, -1, 1) + F(0, 1, -1) + F(0, 1, 1) + F(-1, 0, -1) +        \
                   F(1, 0, -1) + F(-1, 0, 1) + F(1, 0, 1) + F(-1, -1, 0) + F(-1, 1, 0) +        \
                   F(1, -1, 0) + F(1, 1, 0)) / 32.0 +                                           \
                  (F(-1, 0, 0) + F(0, -1, 0) + F(0, 0, -1) + F(1, 0, 0) + F(0, 1, 0) +          \
                   F(0, 0, 1)) / 16.0 +                                                         \
                  F(0, 0, 0) / 8.0;                                                             \
    } while (0)

void orc_restriction(const orc_grid* gf, const double* fine, double* crse)
{
    orc_grid gc;
    orc_coarsen(gf, &gc);
    const long Nf = orc_nnodes(gf), Nc = orc_nnodes(&gc);
    /* bx = grownnodaltilebox(-1,1) & growPeriodicDomain(1): periodic lo/hi move into the ghosts */
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = gc.periodic[d] ? -1 : 0;
        hi[d] = gc.periodic[d] ? gc.n[d] + 1 : gc.n[d];
    }
#pragma omp parallel for schedule(static)
    for (int K = 0; K <= gc.n[2]; K++)
        for (int J = 0; J <= gc.n[1]; J++)
            for (int I = 0; I <= gc.n[0]; I++) {
                const int i = 2 * I, j = 2 * J, k = 2 * K;
                for (int n = 0; n < 3; n++) {
#define FF(a, b, c) UV(gf, Nf, fine, i + (a), j + (b), k + (c), n)
                    double v;
                    FW_BODY(FF, v);
                    crse[n * Nc + IDX(&gc, I, J, K)] = v;
#undef FF
                }
            }
}

void orc_average_ddw(const orc_grid* gf, const double* fine_ddw, double* crse_ddw)
{
    orc_grid gc;
    orc_coarsen(gf, &gc);
    const int nc = orc_ncoef(gf->sym);
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = gc.periodic[d] ? -2 : 0;
        hi[d] = gc.periodic[d] ? gc.n[d] + 2 : gc.n[d];
    }
#pragma omp parallel for schedule(static)
    for (int K = 0; K <= gc.n[2]; K++)
        for (int J = 0; J <= gc.n[1]; J++)
            for (int I = 0; I <= gc.n[0]; I++) {
                const int i = 2 * I, j = 2 * J, k = 2 * K;
                double* out = crse_ddw + IDX(&gc, I, J, K) * nc;
                for (int m = 0; m < nc; m++) {
#define FF(a, b, c) (CV(gf, fine_ddw, i + (a), j + (b), k + (c))[m])
                    double v;
                    FW_BODY(FF, v);
                    out[m] = v;
#undef FF
                }
            }
}

/* Operator<Node>::interpolation (additive), Operator/Operator.cpp:365-434 */
void orc_interpolation(const orc_grid* gf, double* fine, const double* crse)
{
    orc_grid gc;
    orc_coarsen(gf, &gc);
    const long Nf = orc_nnodes(gf), Nc = orc_nnodes(&gc);
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= gf->n[2]; k++)
        for (int j = 0; j <= gf->n[1]; j++)
            for (int i = 0; i <= gf->n[0]; i++) {
                const int I = i / 2, J = j / 2, K = k / 2;
                for (int n = 0; n < 3; n++) {
#define C(a, b, c) crse[n * Nc + IDX(&gc, I + (a), J + (b), K + (c))]
                    double t;
                    if (i % 2 == 0 && j % 2 == 0 && k % 2 == 0) t = C(0, 0, 0);
                    else if (j % 2 == 0 && k % 2 == 0) t = 0.5 * (C(0, 0, 0) + C(1, 0, 0));
                    else if (k % 2 == 0 && i % 2 == 0) t = 0.5 * (C(0, 0, 0) + C(0, 1, 0));
                    else if (i % 2 == 0 && j % 2 == 0) t = 0.5 * (C(0, 0, 0) + C(0, 0, 1));
                    else if (i % 2 == 0) t = 0.25 * (C(0, 0, 0) + C(0, 1, 0) + C(0, 0, 1) + C(0, 1, 1));
                    else if (j % 2 == 0) t = 0.25 * (C(0, 0, 0) + C(0, 0, 1) + C(1, 0, 0) + C(1, 0, 1));
                    else if (k % 2 == 0) t = 0.25 * (C(0, 0, 0) + C(1, 0, 0) + C(0, 1, 0) + C(1, 1, 0));
                    else
                        t = 0.125 * (C(0, 0, 0) + C(1, 0, 0) + C(0, 1, 0) + C(0, 0, 1) + C(0, 1, 1) +
                                     C(1, 0, 1) + C(1, 1, 0) + C(1, 1, 1));
#undef C
                    long p = n * Nf + IDX(gf, i, j, k);
                    fine[p] = fine[p] + t;
                }
            }
}

/* ------------------------------------------------------------------------ */
/* BC values into the RHS, Constant::Init, Constant.H:100-194                */
/* ------------------------------------------------------------------------ */

void orc_bc_init(const orc_grid* g, double* rhs, int homogeneous)
{
    const long N = orc_nnodes(g);
    for (int k = 0; k <= g->n[2]; k++)
        for (int j = 0; j <= g->n[1]; j++)
            for (int i = 0; i <= g->n[0]; i++) {
                bflags fl = node_flags(g, i, j, k);
                if (!is_boundary(&fl)) continue;
                double nrm[3];
                int face = face_of(&fl, nrm);
                for (int d = 0; d < 3; d++) {
                    if (homogeneous && g->bc_type[face][d] == ORC_DISP) rhs[d * N + IDX(g, i, j, k)] = 0.0;
                    else rhs[d * N + IDX(g, i, j, k)] = g->bc_val[face][d];
                }
            }
}

/* ------------------------------------------------------------------------ */
/* Newton::prepareForSolve RHS, Solver/Nonlocal/Newton.H:157-231             */
/* DW = C:(grad u - F0) (Model/Solid/Affine/Isotropic.H:42-45); F0 may be NULL */
/* ------------------------------------------------------------------------ */

static void node_dw(const orc_grid* g, long N, const double* ddw, const double* F0,
                    const double* u, int i, int j, int k, double gradu[3][3], double dw[3][3])
{
    bflags fl = node_flags(g, i, j, k);
    int st[3];
    stencil_types(&fl, st);
    gradient(g, N, u, i, j, k, st, gradu);
    double e[3][3];
    long idx = IDX(g, WRAP(i, g->n[0], g->periodic[0]), WRAP(j, g->n[1], g->periodic[1]),
                   WRAP(k, g->n[2], g->periodic[2]));
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) e[a][b] = gradu[a][b] - (F0 ? F0[idx * 9 + a * 3 + b] : 0.0);
    c_mul_mat(g->sym, CV(g, ddw, i, j, k), e, dw);
}

void orc_newton_rhs(const orc_grid* g, const double* ddw, const double* F0,
                    const double* u, const double* b, double* rhs)
{
    const long N = orc_nnodes(g);
    double* dw = (double*)malloc(sizeof(double) * 9 * N);
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= g->n[2]; k++)
        for (int j = 0; j <= g->n[1]; j++)
            for (int i = 0; i <= g->n[0]; i++) {
                double gu[3][3], d[3][3];
                node_dw(g, N, ddw, F0, u, i, j, k, gu, d);
                long p = IDX(g, i, j, k);
                for (int a = 0; a < 3; a++)
                    for (int c = 0; c < 3; c++) dw[p * 9 + a * 3 + c] = d[a][c];
            }
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= g->n[2]; k++)
        for (int j = 0; j <= g->n[1]; j++)
            for (int i = 0; i <= g->n[0]; i++) {
                bflags fl = node_flags(g, i, j, k);
                long p = IDX(g, i, j, k);
                double ret[3];
                if (is_boundary(&fl)) {
                    int st[3];
                    stencil_types(&fl, st);
                    double gu[3][3], sg[3][3], uc[3], nrm[3];
                    gradient(g, N, u, i, j, k, st, gu);
                    for (int a = 0; a < 3; a++) {
                        uc[a] = u[a * N + p];
                        for (int c = 0; c < 3; c++) sg[a][c] = dw[p * 9 + a * 3 + c];
                    }
                    int face = face_of(&fl, nrm);
                    bc_set(g->bc_type[face], uc, gu, sg, nrm, ret);
                } else {
                    /* Numeric::Divergence, Stencil.H:588-657 (central in the interior) */
                    for (int a = 0; a < 3; a++) ret[a] = 0.0;
                    for (int d = 0; d < 3; d++) {
                        int o[3] = {0, 0, 0};
                        o[d] = 1;
                        long pp = IDX(g, WRAP(i + o[0], g->n[0], g->periodic[0]), WRAP(j + o[1], g->n[1], g->periodic[1]),
                                      WRAP(k + o[2], g->n[2], g->periodic[2]));
                        long pm = IDX(g, WRAP(i - o[0], g->n[0], g->periodic[0]), WRAP(j - o[1], g->n[1], g->periodic[1]),
                                      WRAP(k - o[2], g->n[2], g->periodic[2]));
                        for (int a = 0; a < 3; a++)
                            ret[a] += (dw[pp * 9 + a * 3 + d] - dw[pm * 9 + a * 3 + d]) / 2. / g->dx[d];
                    }
                }
                for (int a = 0; a < 3; a++) rhs[a * N + p] = b[a * N + p] - ret[a];
            }
    free(dw);
}

/* stress = DW(grad u) per node, Integrator/Base/Mechanics.H:210-236; sigma9 AoS row-major */
void orc_stress(const orc_grid* g, const double* ddw, const double* F0, const double* u, double* sigma9)
{
    const long N = orc_nnodes(g);
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= g->n[2]; k++)
        for (int j = 0; j <= g->n[1]; j++)
            for (int i = 0; i <= g->n[0]; i++) {
                double gu[3][3], d[3][3];
                node_dw(g, N, ddw, F0, u, i, j, k, gu, d);
                long p = IDX(g, i, j, k);
                for (int a = 0; a < 3; a++)
                    for (int c = 0; c < 3; c++) sigma9[p * 9 + a * 3 + c] = d[a][c];
            }
}

/* Elastic::Strain (voigt = false) and Elastic::Energy, Operator/Elastic.cpp:428-490,
 * 552-597: eps = (grad u + grad u^T)/2 (9 per node, row-major) and W = sig : eps / 2
 * with sig = C : grad u; either output may be NULL */
void orc_strain_energy(const orc_grid* g, const double* ddw, const double* u, double* eps9, double* energy)
{
    const long N = orc_nnodes(g);
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= g->n[2]; k++)
        for (int j = 0; j <= g->n[1]; j++)
            for (int i = 0; i <= g->n[0]; i++) {
                double gu[3][3], sig[3][3], e[3][3];
                node_dw(g, N, ddw, NULL, u, i, j, k, gu, sig);
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) e[a][b] = 0.5 * (gu[a][b] + gu[b][a]);
                const long p = IDX(g, i, j, k);
                if (eps9)
                    for (int a = 0; a < 3; a++)
                        for (int b = 0; b < 3; b++) eps9[p * 9 + a * 3 + b] = e[a][b];
                if (energy) {
                    double w = 0.0;
                    for (int a = 0; a < 3; a++)
                        for (int b = 0; b < 3; b++) w += 0.5 * sig[a][b] * e[a][b];
                    energy[p] = w;
                }
            }
}

/* trac_hi[0] integral over the xhi face, Integrator/Base/Mechanics.H:391-431 */
void orc_traction_xhi(const orc_grid* g, const double* ddw, const double* F0, const double* u, double trac[3])
{
    const long N = orc_nnodes(g);
    double* s = (double*)malloc(sizeof(double) * 9 * N);
    orc_stress(g, ddw, F0, u, s);
    const double da = g->dx[1] * g->dx[2];
    trac[0] = trac[1] = trac[2] = 0.0;
    const int i = g->n[0];
    for (int k = 0; k < g->n[2]; k++)
        for (int j = 0; j < g->n[1]; j++) {
            long a = IDX(g, i, j, k), b = IDX(g, i, j + 1, k), c = IDX(g, i, j, k + 1), d = IDX(g, i, j + 1, k + 1);
            for (int r = 0; r < 3; r++) {
                double m = 0.25 * (s[a * 9 + r * 3] + s[b * 9 + r * 3] + s[c * 9 + r * 3] + s[d * 9 + r * 3]);
                trac[r] += m * da;
            }
        }
    free(s);
}

/* ------------------------------------------------------------------------ */
/* MLMG-equivalent driver (AMReX 26.06 MLMG restated from its algorithm)     */
/* ------------------------------------------------------------------------ */

void orc_default_params(orc_solver_params* p)
{
    p->max_iter = 200;
    p->fixed_iter = -1;
    p->pre_smooth = 2;
    p->post_smooth = 2;
    p->final_smooth = 8;
    p->bottom_smooth = 0;
    p->max_fmg_iter = 100000000;   /* Solver/Nonlocal/Linear.H:261 */
    p->bottom_max_iter = 200;
    p->bottom_tol_rel = 1e-4;
    p->bottom_tol_abs = -1.0;
    p->omega = 2. / 3.;
    p->max_coarsening_level = 30;
    p->verbose = 0;
}

int orc_num_levels(const orc_grid* g, int max_coarsening_level)
{
    int n[3] = {g->n[0], g->n[1], g->n[2]}, lev = 1;
    while (lev - 1 < max_coarsening_level) {
        int ok = 1;
        for (int d = 0; d < 3; d++)
            if (n[d] % 2 != 0 || n[d] / 2 < 2) ok = 0;
        if (!ok) break;
        for (int d = 0; d < 3; d++) n[d] /= 2;
        lev++;
    }
    return lev;
}

typedef struct {
    int L;
    orc_grid g[32];
    long N[32];
    double* ddw[32];
    double* diag[32];
    double* cor[32];
    double* res[32];
    double* rescor[32];
    double* hold[32];
    const orc_solver_params* p;
} mg_t;

static void mg_smooth(mg_t* m, int l, double* x, const double* b, int nsmooth)
{
    for (int s = 0; s < nsmooth; s++) orc_fsmooth(&m->g[l], m->ddw[l], m->diag[l], x, b, m->p->omega);
}

static double dotxy(const orc_grid* g, const double* x, const double* y)
{
    /* owner-masked dot product: periodic duplicate nodes counted once */
    const long N = orc_nnodes(g);
    double s = 0.0;
    for (int c = 0; c < 3; c++)
        for (int k = 0; k <= g->n[2]; k++) {
            if (g->periodic[2] && k == g->n[2]) continue;
            for (int j = 0; j <= g->n[1]; j++) {
                if (g->periodic[1] && j == g->n[1]) continue;
                for (int i = 0; i <= g->n[0]; i++) {
                    if (g->periodic[0] && i == g->n[0]) continue;
                    long q = c * N + IDX(g, i, j, k);
                    s += x[q] * y[q];
                }
            }
        }
    return s;
}

static int fully_periodic(const orc_grid* g) { return g->periodic[0] && g->periodic[1] && g->periodic[2]; }

/* Subtract the per-component mean over the unique nodes (periodic images
 * counted once).
 *
 * A fully periodic box has the rigid translations as null space.  The
 * reference has no fully periodic elastic solve (its operator is never
 * singular, Operator.H:96-97); this project's periodic RVE solves follow the
 * idea of MLMG's makeSolvable instead: the right-hand side and every
 * fine-level residual are projected to zero mean, and so are the residual and
 * every operator application of the bottom Krylov solve.  Because the
 * operator is not conservative its left null vectors are constants only up to
 * discretisation error, so the solve finds u with  A u = b - c  for a uniform
 * body force c (per component) of the size of that error, rather than
 * A u = b.  The returned displacement has zero mean. */
static void remove_mean(const orc_grid* g, double* v)
{
    const long N = orc_nnodes(g);
    const long cnt = (long)g->n[0] * g->n[1] * g->n[2];
    for (int c = 0; c < 3; c++) {
        double s = 0.0;
        for (int k = 0; k < g->n[2]; k++)
            for (int j = 0; j < g->n[1]; j++)
                for (int i = 0; i < g->n[0]; i++) s += v[c * N + IDX(g, i, j, k)];
        const double mean = s / (double)cnt;
        for (long q = 0; q < N; q++) v[c * N + q] -= mean;
    }
}

/*
 * BiCGStab on the diagonally scaled system (MLCGSolver::solve_bicgstab with
 * Operator<Node>::normalize = divide by the diagonal, Operator.cpp:156-165).
 * Returns 0 converged, 1..4 breakdown, 8 not converged.  On a fully periodic
 * box the residual and each operator application are projected to zero mean
 * before the scaling (see remove_mean).
 */
static int bottom_bicgstab(mg_t* m, int l, double* sol, const double* rhs)
{
    const orc_grid* g = &m->g[l];
    const int sing = fully_periodic(g);
    const long n3 = 3 * m->N[l];
    const double* D = m->diag[l];
    const double eps_rel = m->p->bottom_tol_rel, eps_abs = m->p->bottom_tol_abs;
    double* buf = (double*)calloc(8 * n3, sizeof(double));
    double *r = buf, *rh = buf + n3, *p = buf + 2 * n3, *v = buf + 3 * n3, *s = buf + 4 * n3,
           *t = buf + 5 * n3, *sorig = buf + 6 * n3;
    orc_residual(g, m->ddw[l], sol, rhs, r);
    if (sing) remove_mean(g, r);
    for (long q = 0; q < n3; q++) r[q] /= D[q];
    for (long q = 0; q < n3; q++) { sorig[q] = sol[q]; sol[q] = 0.0; rh[q] = r[q]; }
    double rnorm = orc_norm_inf(g, r);
    const double rnorm0 = rnorm;
    int ret = 0;
    double rho_1 = 0, alpha = 0, omega = 0;
    if (rnorm0 == 0 || rnorm0 < eps_abs) {
        for (long q = 0; q < n3; q++) sol[q] = sorig[q];
        free(buf);
        return 0;
    }
    int last_iter = 0;
    for (int iter = 1; iter <= m->p->bottom_max_iter; iter++) {
        last_iter = iter;
        const double rho = dotxy(g, rh, r);
        if (rho == 0) { ret = 1; break; }
        if (iter == 1) {
            for (long q = 0; q < n3; q++) p[q] = r[q];
        } else {
            const double beta = (rho / rho_1) * (alpha / omega);
            for (long q = 0; q < n3; q++) p[q] = r[q] + beta * (p[q] - omega * v[q]);
        }
        orc_fapply(g, m->ddw[l], p, v);
        if (sing) remove_mean(g, v);
        for (long q = 0; q < n3; q++) v[q] /= D[q];
        double rhTv = dotxy(g, rh, v);
        if (rhTv != 0) alpha = rho / rhTv;
        else { ret = 2; break; }
        for (long q = 0; q < n3; q++) { sol[q] += alpha * p[q]; s[q] = r[q] - alpha * v[q]; }
        rnorm = orc_norm_inf(g, s);
        if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
        orc_fapply(g, m->ddw[l], s, t);
        if (sing) remove_mean(g, t);
        for (long q = 0; q < n3; q++) t[q] /= D[q];
        double tt = dotxy(g, t, t), ts = dotxy(g, t, s);
        if (tt != 0) omega = ts / tt;
        else { ret = 3; break; }
        for (long q = 0; q < n3; q++) { sol[q] += omega * s[q]; r[q] = s[q] - omega * t[q]; }
        rnorm = orc_norm_inf(g, r);
        if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
        if (omega == 0) { ret = 4; break; }
        rho_1 = rho;
    }
    if (ret == 0 && rnorm > eps_rel * rnorm0 && rnorm > eps_abs) ret = 8;
    if (m->p->verbose > 1)
        fprintf(stderr, "oracle bottom: ret %d after %d iterations, |r| %.3e of %.3e\n", ret, last_iter, rnorm, rnorm0);
    if ((ret == 0 || ret == 8) && rnorm < rnorm0) {
        for (long q = 0; q < n3; q++) sol[q] += sorig[q];
    } else {
        for (long q = 0; q < n3; q++) sol[q] = sorig[q];
    }
    free(buf);
    return ret;
}

/* MLMG::actualBottomSolve: cor = 0, BiCGStab, zero on failure, then smooth;
 * returns the BiCGStab code */
static int mg_bottom(mg_t* m)
{
    const int l = m->L - 1;
    const long n3 = 3 * m->N[l];
    for (long q = 0; q < n3; q++) m->cor[l][q] = 0.0;
    int ret = bottom_bicgstab(m, l, m->cor[l], m->res[l]);
    if (ret != 0 && ret != 9)
        for (long q = 0; q < n3; q++) m->cor[l][q] = 0.0;
    int nsm = (ret == 0) ? m->p->bottom_smooth : m->p->final_smooth;
    mg_smooth(m, l, m->cor[l], m->res[l], nsm);
    return ret;
}

/* The bottom step of one level on its own: cor <- BiCGStab(res) + smoothing,
 * as mg_bottom does on the coarsest level of a solve.  diag is the level's
 * Diagonal; returns the BiCGStab code (0 converged, 1-4 breakdown, 8 not
 * converged). */
int orc_bottom_solve(const orc_grid* g, const double* ddw, const double* diag, const double* res, double* cor,
                     const orc_solver_params* p)
{
    mg_t m;
    memset(&m, 0, sizeof(m));
    m.p = p;
    m.L = 1;
    m.g[0] = *g;
    m.N[0] = orc_nnodes(g);
    m.ddw[0] = (double*)ddw;
    m.diag[0] = (double*)diag;
    m.res[0] = (double*)res;
    m.cor[0] = cor;
    return mg_bottom(&m);
}

/* MLMG::mgVcycle(amrlev=0, mglev_top) */
static void mg_vcycle(mg_t* m, int top)
{
    const int bot = m->L - 1;
    for (int l = top; l < bot; l++) {
        const long n3 = 3 * m->N[l];
        for (long q = 0; q < n3; q++) m->cor[l][q] = 0.0;
        mg_smooth(m, l, m->cor[l], m->res[l], m->p->pre_smooth);
        orc_residual(&m->g[l], m->ddw[l], m->cor[l], m->res[l], m->rescor[l]);
        orc_restriction(&m->g[l], m->rescor[l], m->res[l + 1]);
    }
    mg_bottom(m);
    for (int l = bot - 1; l >= top; l--) {
        orc_interpolation(&m->g[l], m->cor[l], m->cor[l + 1]);
        mg_smooth(m, l, m->cor[l], m->res[l], m->p->post_smooth);
    }
}

/* MLMG::mgFcycle */
static void mg_fcycle(mg_t* m)
{
    const int bot = m->L - 1;
    for (int l = 1; l <= bot; l++) orc_restriction(&m->g[l - 1], m->res[l - 1], m->res[l]);
    mg_bottom(m);
    for (int l = bot - 1; l >= 0; l--) {
        const long n3 = 3 * m->N[l];
        for (long q = 0; q < n3; q++) m->cor[l][q] = 0.0;
        orc_interpolation(&m->g[l], m->cor[l], m->cor[l + 1]);
        orc_residual(&m->g[l], m->ddw[l], m->cor[l], m->res[l], m->rescor[l]);
        for (long q = 0; q < n3; q++) { m->res[l][q] = m->rescor[l][q]; m->hold[l][q] = m->cor[l][q]; }
        mg_vcycle(m, l);
        for (long q = 0; q < n3; q++) m->cor[l][q] += m->hold[l][q];
    }
}

/* A solve in progress: the hierarchy after prepareForSolve, the right-hand
 * side and the stopping target.  orc_solve = begin + iterate (to the end) +
 * end; the split form lets a caller run the iterations of one solve in
 * several timed pieces. */
struct orc_session {
    mg_t m;
    orc_grid g;
    const double* b;
    double* bproj;
    int sing;
    double max_norm, target, norm;
    orc_report rep;
};

orc_session* orc_solve_begin(const orc_grid* g, const double* ddw, const orc_solver_params* p, const double* x,
                             const double* b, double tol_rel, double tol_abs)
{
    orc_session* s = (orc_session*)calloc(1, sizeof(orc_session));
    mg_t* m = &s->m;
    m->p = p;
    s->g = *g;
    const double t0 = omp_get_wtime();
    m->L = orc_num_levels(g, p->max_coarsening_level);
    const int nc = orc_ncoef(g->sym);
    m->g[0] = *g;
    for (int l = 1; l < m->L; l++) orc_coarsen(&m->g[l - 1], &m->g[l]);
    for (int l = 0; l < m->L; l++) {
        m->N[l] = orc_nnodes(&m->g[l]);
        long n3 = 3 * m->N[l];
        m->ddw[l] = (l == 0) ? (double*)ddw : (double*)malloc(sizeof(double) * nc * m->N[l]);
        m->diag[l] = (double*)malloc(sizeof(double) * n3);
        m->cor[l] = (double*)calloc(n3, sizeof(double));
        m->res[l] = (double*)calloc(n3, sizeof(double));
        m->rescor[l] = (double*)calloc(n3, sizeof(double));
        m->hold[l] = (double*)calloc(n3, sizeof(double));
    }
    /* Operator<Node>::prepareForSolve, Operator.cpp:253-260 */
    for (int l = 1; l < m->L; l++) orc_average_ddw(&m->g[l - 1], m->ddw[l - 1], m->ddw[l]);
    for (int l = 0; l < m->L; l++) orc_diagonal(&m->g[l], m->ddw[l], m->diag[l]);

    /* fully periodic box: solve with the zero-mean part of b (see remove_mean) */
    s->sing = fully_periodic(g);
    if (s->sing) {
        s->bproj = (double*)malloc(sizeof(double) * 3 * m->N[0]);
        memcpy(s->bproj, b, sizeof(double) * 3 * m->N[0]);
        remove_mean(g, s->bproj);
        b = s->bproj;
    }
    s->b = b;
    orc_residual(&m->g[0], m->ddw[0], x, b, m->res[0]);
    if (s->sing) remove_mean(g, m->res[0]);
    const double resnorm0 = orc_norm_inf(g, m->res[0]);
    const double rhsnorm0 = orc_norm_inf(g, b);
    s->max_norm = (rhsnorm0 >= resnorm0) ? rhsnorm0 : resnorm0;
    double rel = tol_rel > 1e-16 ? tol_rel : 1e-16;
    s->target = tol_abs > rel * s->max_norm ? tol_abs : rel * s->max_norm;
    s->rep.res0 = resnorm0;
    s->rep.iterations = 0;
    s->rep.nlevels = m->L;
    s->rep.status = (resnorm0 <= s->target) ? 0 : 1;
    s->rep.res_final = resnorm0;
    s->norm = resnorm0;
    s->rep.t_setup = omp_get_wtime() - t0;
    return s;
}

int orc_solve_iterate(orc_session* s, double* x, int max_steps)
{
    mg_t* m = &s->m;
    const orc_solver_params* p = m->p;
    const double t1 = omp_get_wtime();
    const long n3 = 3 * m->N[0];
    for (int step = 0; step < max_steps && s->rep.status == 1 && s->rep.iterations < p->max_iter; step++) {
        const int iter = s->rep.iterations;
        if (iter < p->max_fmg_iter) mg_fcycle(m);
        else mg_vcycle(m, 0);
        for (long q = 0; q < n3; q++) x[q] += m->cor[0][q];
        orc_residual(&m->g[0], m->ddw[0], x, s->b, m->res[0]);
        if (s->sing) remove_mean(&s->g, m->res[0]);
        s->norm = orc_norm_inf(&s->g, m->res[0]);
        s->rep.iterations = iter + 1;
        if (p->verbose)
            fprintf(stderr, "oracle MLMG iter %d resid %.6e rel %.6e\n", iter + 1, s->norm, s->norm / s->max_norm);
        if (s->norm != s->norm) { s->rep.status = 2; break; }
        if (s->norm <= s->target) { s->rep.status = 0; break; }
        if (p->fixed_iter > 0 && iter + 1 >= p->fixed_iter) { s->rep.status = 0; break; }
    }
    s->rep.res_final = s->norm;
    s->rep.t_iter += omp_get_wtime() - t1;
    return s->rep.status;
}

int orc_solve_end(orc_session* s, double* x, orc_report* rep)
{
    mg_t* m = &s->m;
    if (s->sing) remove_mean(&s->g, x);   /* solution modulo rigid translation */
    if (rep) *rep = s->rep;
    const int st = s->rep.status;
    for (int l = 0; l < m->L; l++) {
        if (l > 0) free(m->ddw[l]);
        free(m->diag[l]); free(m->cor[l]); free(m->res[l]); free(m->rescor[l]); free(m->hold[l]);
    }
    free(s->bproj);
    free(s);
    return st;
}

int orc_solve(const orc_grid* g, const double* ddw, const orc_solver_params* p,
              double* x, const double* b, double tol_rel, double tol_abs, orc_report* rep)
{
    orc_session* s = orc_solve_begin(g, ddw, p, x, b, tol_rel, tol_abs);
    orc_solve_iterate(s, x, p->max_iter);
    return orc_solve_end(s, x, rep);
}

/* Newton::solve with one Newton iteration (linear models), Newton.H:279-358 */
int orc_newton_solve(const orc_grid* g, const double* ddw, const double* F0,
                     const orc_solver_params* p, double* u, const double* b,
                     double tol_rel, double tol_abs, orc_report* rep)
{
    const long N = orc_nnodes(g);
    double* rhs = (double*)malloc(sizeof(double) * 3 * N);
    double* dsol = (double*)calloc(3 * N, sizeof(double));
    orc_newton_rhs(g, ddw, F0, u, b, rhs);
    int st = orc_solve(g, ddw, p, dsol, rhs, tol_rel, tol_abs, rep);
    for (long q = 0; q < 3 * N; q++) u[q] += dsol[q];
    free(rhs);
    free(dsol);
    return st;
}
