// stencil.cuh -- per-node arithmetic of Alamo's nodal elastic operator, shared
// by every sm_103a kernel of this library (templated on the arithmetic type T =
// double or float and on the modulus symmetry).
//
// Reference semantics (paths relative to the alamo source tree):
//   interior row  f = C : grad grad u + sum_j (d_j C : grad u).col(j)
//                 Operator/Elastic.cpp:205-254
//   boundary row  f = BC(u, grad u, C : grad u), Operator/Elastic.cpp:195-203 and
//                 BC/Operator/Elastic/Constant.H:344-425
//   stencils      Numeric/Stencil.H:41-301
//   contractions  Set/Matrix4_Isotropic.H:137-173, Set/Matrix4_MajorMinor.H:675-767
//
// The expressions keep the reference's term grouping; scale factors such as
// 0.5/dx are applied as precomputed reciprocals and the compiler may fuse
// multiply-adds, so FP64 results agree with the reference to rounding
// (~1e-15 relative), not bit for bit.
#pragma once
#include <cstdint>

#include "agb_internal.h"

namespace agb {

enum { SYM_ISO = 0, SYM_MM = 1 };

template <int SYM> struct NCoef;
template <> struct NCoef<SYM_ISO> { static constexpr int value = 2; };
template <> struct NCoef<SYM_MM> { static constexpr int value = 21; };

// Reciprocal grid factors for one level in the arithmetic type.
template <typename T> struct Geo {
    T h1[3];   // 0.5/dx : central first derivative
    T i1[3];   // 1/dx   : one-sided first derivative
    T h2[3];   // 1/dx^2 : second derivative
    T hm[3];   // 0.25/(dx_a dx_b) for (x,y), (x,z), (y,z)
    int cube;  // dx equal in all directions
};

template <typename T> __host__ __device__ inline Geo<T> make_geo(const LevelDesc& L)
{
    Geo<T> g;
    for (int d = 0; d < 3; d++) {
        g.h1[d] = (T)(0.5 / L.dx[d]);
        g.i1[d] = (T)(1.0 / L.dx[d]);
        g.h2[d] = (T)(1.0 / (L.dx[d] * L.dx[d]));
    }
    g.hm[0] = (T)(0.25 / (L.dx[0] * L.dx[1]));
    g.hm[1] = (T)(0.25 / (L.dx[0] * L.dx[2]));
    g.hm[2] = (T)(0.25 / (L.dx[1] * L.dx[2]));
    g.cube = L.dx[0] == L.dx[1] && L.dx[1] == L.dx[2];
    return g;
}

// ---------------------------------------------------------------------------
// Contractions.  b is a 3x3 matrix (row-major), H a Matrix3 H[i][j][k] = b(i,j,k).
// ---------------------------------------------------------------------------

// Matrix4<3,Isotropic> * Matrix (coefficients: lambda, mu)
template <typename T>
__device__ __forceinline__ void iso_mul_mat(const T* c, const T b[3][3], T r[3][3])
{
    const T lambda = c[0], mu = c[1];
    r[0][0] = (lambda + (T)2 * mu) * b[0][0] + lambda * b[1][1] + lambda * b[2][2];
    r[1][1] = lambda * b[0][0] + (lambda + (T)2 * mu) * b[1][1] + lambda * b[2][2];
    r[2][2] = lambda * b[0][0] + lambda * b[1][1] + (lambda + (T)2 * mu) * b[2][2];
    r[1][2] = mu * (b[1][2] + b[2][1]); r[2][1] = r[1][2];
    r[2][0] = mu * (b[2][0] + b[0][2]); r[0][2] = r[2][0];
    r[0][1] = mu * (b[0][1] + b[1][0]); r[1][0] = r[0][1];
}

// Matrix4<3,MajorMinor> * Matrix
template <typename T>
__device__ __forceinline__ void mm_mul_mat(const T* a, const T b[3][3], T r[3][3])
{
    const T s01 = b[0][1] + b[1][0], s02 = b[0][2] + b[2][0], s12 = b[1][2] + b[2][1];
    r[0][0] = a[0] * b[0][0] + a[1] * s01 + a[2] * s02 + a[3] * b[1][1] + a[4] * s12 + a[5] * b[2][2];
    r[1][1] = a[3] * b[0][0] + a[8] * s01 + a[12] * s02 + a[15] * b[1][1] + a[16] * s12 + a[17] * b[2][2];
    r[2][2] = a[5] * b[0][0] + a[10] * s01 + a[14] * s02 + a[17] * b[1][1] + a[19] * s12 + a[20] * b[2][2];
    r[1][2] = a[4] * b[0][0] + a[9] * s01 + a[13] * s02 + a[16] * b[1][1] + a[18] * s12 + a[19] * b[2][2];
    r[2][0] = a[2] * b[0][0] + a[7] * s01 + a[11] * s02 + a[12] * b[1][1] + a[13] * s12 + a[14] * b[2][2];
    r[0][1] = a[1] * b[0][0] + a[6] * s01 + a[7] * s02 + a[8] * b[1][1] + a[9] * s12 + a[10] * b[2][2];
    r[2][1] = r[1][2];
    r[0][2] = r[2][0];
    r[1][0] = r[0][1];
}

template <typename T, int SYM>
__device__ __forceinline__ void c_mul_mat(const T* c, const T b[3][3], T r[3][3])
{
    if (SYM == SYM_ISO) iso_mul_mat(c, b, r);
    else mm_mul_mat(c, b, r);
}

// Matrix4<3,Isotropic> * Matrix3
template <typename T>
__device__ __forceinline__ void iso_mul_m3(const T* c, const T H[3][3][3], T r[3])
{
    const T lambda = c[0], mu = c[1];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        T s = 0;
#pragma unroll
        for (int j = 0; j < 3; j++) s += mu * (H[i][j][j] + H[j][i][j]) + lambda * H[j][j][i];
        r[i] = s;
    }
}

// Matrix4<3,MajorMinor> * Matrix3 (term grouping of Matrix4_MajorMinor.H:715-764)
template <typename T>
__device__ __forceinline__ void mm_mul_m3(const T* a, const T H[3][3][3], T r[3])
{
#define B(i, j, k) H[i][j][k]
    r[0] = a[0] * B(0,0,0) + a[1] * (B(0,1,0) + B(1,0,0) + B(0,0,1)) + a[2] * (B(0,2,0) + B(2,0,0) + B(0,0,2)) +
           a[3] * B(1,1,0) + a[4] * (B(1,2,0) + B(2,1,0)) + a[5] * B(2,2,0) + a[6] * (B(0,1,1) + B(1,0,1)) +
           a[7] * (B(0,2,1) + B(2,0,1) + B(0,1,2) + B(1,0,2)) + a[8] * B(1,1,1) + a[9] * (B(1,2,1) + B(2,1,1)) +
           a[10] * B(2,2,1) + a[11] * (B(0,2,2) + B(2,0,2)) + a[12] * B(1,1,2) + a[13] * (B(1,2,2) + B(2,1,2)) +
           a[14] * B(2,2,2);
    r[1] = a[1] * B(0,0,0) + a[4] * B(0,0,2) + a[3] * B(0,0,1) + a[6] * (B(0,1,0) + B(1,0,0)) +
           a[7] * (B(0,2,0) + B(2,0,0)) + a[8] * (B(1,1,0) + B(0,1,1) + B(1,0,1)) +
           a[9] * (B(1,2,0) + B(2,1,0) + B(0,1,2) + B(1,0,2)) + a[10] * B(2,2,0) + a[12] * (B(0,2,1) + B(2,0,1)) +
           a[13] * (B(0,2,2) + B(2,0,2)) + a[15] * B(1,1,1) + a[16] * (B(1,2,1) + B(2,1,1) + B(1,1,2)) +
           a[17] * B(2,2,1) + a[18] * (B(1,2,2) + B(2,1,2)) + a[19] * B(2,2,2);
    r[2] = a[2] * B(0,0,0) + a[4] * B(0,0,1) + a[5] * B(0,0,2) + a[7] * (B(0,1,0) + B(1,0,0)) +
           a[9] * (B(0,1,1) + B(1,0,1)) + a[10] * (B(0,1,2) + B(1,0,2)) + a[11] * (B(0,2,0) + B(2,0,0)) +
           a[12] * B(1,1,0) + a[13] * (B(1,2,0) + B(2,1,0) + B(0,2,1) + B(2,0,1)) +
           a[14] * (B(2,2,0) + B(0,2,2) + B(2,0,2)) + a[16] * B(1,1,1) + a[17] * B(1,1,2) +
           a[18] * (B(1,2,1) + B(2,1,1)) + a[19] * (B(2,2,1) + B(1,2,2) + B(2,1,2)) + a[20] * B(2,2,2);
#undef B
}

template <typename T, int SYM>
__device__ __forceinline__ void c_mul_m3(const T* c, const T H[3][3][3], T r[3])
{
    if (SYM == SYM_ISO) iso_mul_m3(c, H, r);
    else mm_mul_m3(c, H, r);
}

// Column d of (dC : G) where dC = C(+e_d) - C(-e_d), returned unscaled.
// Only the Matrix4 slots that feed column d are differenced (15 of 21).
template <typename T, int SYM, int D, class A>
__device__ __forceinline__ void dC_col(const A& acc, const T G[3][3], T out[3])
{
    constexpr int dx = D == 0, dy = D == 1, dz = D == 2;
    if (SYM == SYM_ISO) {
        const T dl = acc.C(0, dx, dy, dz) - acc.C(0, -dx, -dy, -dz);
        const T dm = acc.C(1, dx, dy, dz) - acc.C(1, -dx, -dy, -dz);
        T r[3][3];
        const T c[2] = {dl, dm};
        iso_mul_mat(c, G, r);
        out[0] = r[0][D]; out[1] = r[1][D]; out[2] = r[2][D];
    } else {
        const T s01 = G[0][1] + G[1][0], s02 = G[0][2] + G[2][0], s12 = G[1][2] + G[2][1];
#define DC(m) (acc.C(m, dx, dy, dz) - acc.C(m, -dx, -dy, -dz))
        // rows of mm_mul_mat: r00 {0..5}, r11 {3,8,12,15,16,17}, r22 {5,10,14,17,19,20},
        // r12 {4,9,13,16,18,19}, r20 {2,7,11,12,13,14}, r01 {1,6,7,8,9,10}
        if (D == 0) {
            out[0] = DC(0) * G[0][0] + DC(1) * s01 + DC(2) * s02 + DC(3) * G[1][1] + DC(4) * s12 + DC(5) * G[2][2];
            out[1] = DC(1) * G[0][0] + DC(6) * s01 + DC(7) * s02 + DC(8) * G[1][1] + DC(9) * s12 + DC(10) * G[2][2];
            out[2] = DC(2) * G[0][0] + DC(7) * s01 + DC(11) * s02 + DC(12) * G[1][1] + DC(13) * s12 + DC(14) * G[2][2];
        } else if (D == 1) {
            out[0] = DC(1) * G[0][0] + DC(6) * s01 + DC(7) * s02 + DC(8) * G[1][1] + DC(9) * s12 + DC(10) * G[2][2];
            out[1] = DC(3) * G[0][0] + DC(8) * s01 + DC(12) * s02 + DC(15) * G[1][1] + DC(16) * s12 + DC(17) * G[2][2];
            out[2] = DC(4) * G[0][0] + DC(9) * s01 + DC(13) * s02 + DC(16) * G[1][1] + DC(18) * s12 + DC(19) * G[2][2];
        } else {
            out[0] = DC(2) * G[0][0] + DC(7) * s01 + DC(11) * s02 + DC(12) * G[1][1] + DC(13) * s12 + DC(14) * G[2][2];
            out[1] = DC(4) * G[0][0] + DC(9) * s01 + DC(13) * s02 + DC(16) * G[1][1] + DC(18) * s12 + DC(19) * G[2][2];
            out[2] = DC(5) * G[0][0] + DC(10) * s01 + DC(14) * s02 + DC(17) * G[1][1] + DC(19) * s12 + DC(20) * G[2][2];
        }
#undef DC
    }
}

// Neighbour offsets of a node, periodic images folded in.
struct Nbr {
    long long base;
    long long o[3][3];   // o[d][delta+1]
};

__device__ __forceinline__ Nbr make_nbr(const LevelDesc& L, int i, int j, int k)
{
    Nbr nb;
    nb.base = L.idx(i, j, k);
    const long long st[3] = {1, (long long)L.P, (long long)L.P * L.nn[1]};
    const int pos[3] = {i, j, k};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        nb.o[d][0] = -st[d];
        nb.o[d][1] = 0;
        nb.o[d][2] = st[d];
        if (L.per[d]) {
            if (pos[d] == 0) nb.o[d][0] = st[d] * (L.n[d] - 1);
            if (pos[d] == L.n[d] - 1) nb.o[d][2] = -st[d] * (L.n[d] - 1);
        }
    }
    return nb;
}

// ---------------------------------------------------------------------------
// Interior row.  A provides u(c,di,dj,dk) and C(m,di,dj,dk) relative to the node.
// ---------------------------------------------------------------------------
// The same row on cubic cells (FP64): with h2 = 1/dx^2, hm = h2/4 and
// h1^2 = h2/4 the second differences enter unscaled, the mixed ones times
// 1/4, the first differences unscaled, and the row is scaled by h2 once:
// f = h2 (C : H' + (1/4) sum_d (dC_d : G')_{:,d}).  Fifteen FP64 operations
// fewer per node than the general form (the sweep is bound by the FP64
// pipe); the value differs from it by rounding only.
template <typename T, int SYM, class A>
__device__ __forceinline__ void interior_row_cube(const A& acc, const Geo<T>& g, bool uniform, T f[3])
{
    T H[3][3][3];
#pragma unroll
    for (int p = 0; p < 3; p++) {
        const T u0 = acc.u(p, 0, 0, 0);
        H[p][0][0] = acc.u(p, 1, 0, 0) - (T)2 * u0 + acc.u(p, -1, 0, 0);
        H[p][1][1] = acc.u(p, 0, 1, 0) - (T)2 * u0 + acc.u(p, 0, -1, 0);
        H[p][2][2] = acc.u(p, 0, 0, 1) - (T)2 * u0 + acc.u(p, 0, 0, -1);
        H[p][0][1] = (acc.u(p, 1, 1, 0) + acc.u(p, -1, -1, 0) - acc.u(p, 1, -1, 0) - acc.u(p, -1, 1, 0)) * (T)0.25;
        H[p][0][2] = (acc.u(p, 1, 0, 1) + acc.u(p, -1, 0, -1) - acc.u(p, 1, 0, -1) - acc.u(p, -1, 0, 1)) * (T)0.25;
        H[p][1][2] = (acc.u(p, 0, 1, 1) + acc.u(p, 0, -1, -1) - acc.u(p, 0, 1, -1) - acc.u(p, 0, -1, 1)) * (T)0.25;
        H[p][1][0] = H[p][0][1];
        H[p][2][0] = H[p][0][2];
        H[p][2][1] = H[p][1][2];
    }
    T c[NCoef<SYM>::value];
#pragma unroll
    for (int m = 0; m < NCoef<SYM>::value; m++) c[m] = acc.C(m, 0, 0, 0);
    c_mul_m3<T, SYM>(c, H, f);
    if (!uniform) {
        T G[3][3];
#pragma unroll
        for (int p = 0; p < 3; p++) {
            G[p][0] = acc.u(p, 1, 0, 0) - acc.u(p, -1, 0, 0);
            G[p][1] = acc.u(p, 0, 1, 0) - acc.u(p, 0, -1, 0);
            G[p][2] = acc.u(p, 0, 0, 1) - acc.u(p, 0, 0, -1);
        }
        T c0[3], c1[3], c2[3];
        dC_col<T, SYM, 0>(acc, G, c0);
        dC_col<T, SYM, 1>(acc, G, c1);
        dC_col<T, SYM, 2>(acc, G, c2);
#pragma unroll
        for (int r = 0; r < 3; r++) f[r] += (T)0.25 * (c0[r] + c1[r] + c2[r]);
    }
#pragma unroll
    for (int r = 0; r < 3; r++) f[r] *= g.h2[0];
}

template <typename T, int SYM, class A>
__device__ __forceinline__ void interior_row(const A& acc, const Geo<T>& g, bool uniform, T f[3])
{
    if constexpr (sizeof(T) == 8) {
        if (g.cube) {
            interior_row_cube<T, SYM>(acc, g, uniform, f);
            return;
        }
    }
    T H[3][3][3];
#pragma unroll
    for (int p = 0; p < 3; p++) {
        const T u0 = acc.u(p, 0, 0, 0);
        H[p][0][0] = (acc.u(p, 1, 0, 0) - (T)2 * u0 + acc.u(p, -1, 0, 0)) * g.h2[0];
        H[p][1][1] = (acc.u(p, 0, 1, 0) - (T)2 * u0 + acc.u(p, 0, -1, 0)) * g.h2[1];
        H[p][2][2] = (acc.u(p, 0, 0, 1) - (T)2 * u0 + acc.u(p, 0, 0, -1)) * g.h2[2];
        H[p][0][1] = (acc.u(p, 1, 1, 0) + acc.u(p, -1, -1, 0) - acc.u(p, 1, -1, 0) - acc.u(p, -1, 1, 0)) * g.hm[0];
        H[p][0][2] = (acc.u(p, 1, 0, 1) + acc.u(p, -1, 0, -1) - acc.u(p, 1, 0, -1) - acc.u(p, -1, 0, 1)) * g.hm[1];
        H[p][1][2] = (acc.u(p, 0, 1, 1) + acc.u(p, 0, -1, -1) - acc.u(p, 0, 1, -1) - acc.u(p, 0, -1, 1)) * g.hm[2];
        H[p][1][0] = H[p][0][1];
        H[p][2][0] = H[p][0][2];
        H[p][2][1] = H[p][1][2];
    }
    T c[NCoef<SYM>::value];
#pragma unroll
    for (int m = 0; m < NCoef<SYM>::value; m++) c[m] = acc.C(m, 0, 0, 0);
    c_mul_m3<T, SYM>(c, H, f);
    if (!uniform) {
        T G[3][3];
#pragma unroll
        for (int p = 0; p < 3; p++) {
            G[p][0] = (acc.u(p, 1, 0, 0) - acc.u(p, -1, 0, 0)) * g.h1[0];
            G[p][1] = (acc.u(p, 0, 1, 0) - acc.u(p, 0, -1, 0)) * g.h1[1];
            G[p][2] = (acc.u(p, 0, 0, 1) - acc.u(p, 0, 0, -1)) * g.h1[2];
        }
        T c0[3], c1[3], c2[3];
        dC_col<T, SYM, 0>(acc, G, c0);
        dC_col<T, SYM, 1>(acc, G, c1);
        dC_col<T, SYM, 2>(acc, G, c2);
#pragma unroll
        for (int r = 0; r < 3; r++) f[r] += c0[r] * g.h1[0] + c1[r] * g.h1[1] + c2[r] * g.h1[2];
    }
}

// ---------------------------------------------------------------------------
// Boundary rows
// ---------------------------------------------------------------------------

// Region index and outward normal in the precedence order of
// Constant::operator(), BC/Operator/Elastic/Constant.H:373-400.  mn/mx flag the
// node on the lo/hi face of a non-periodic direction.
__host__ __device__ inline int face_of(const int mn[3], const int mx[3], double nrm[3])
{
    const double s3 = AGB_SQRT3INV, s2 = AGB_SQRT2INV;
    const int xl = mn[0], xh = mx[0], yl = mn[1], yh = mx[1], zl = mn[2], zh = mx[2];
#define RET(face, a, b, c) { nrm[0] = (a); nrm[1] = (b); nrm[2] = (c); return (face); }
    if (xl && yl && zl) RET(F_XLO_YLO_ZLO, -s3, -s3, -s3);
    if (xl && yl && zh) RET(F_XLO_YLO_ZHI, -s3, -s3, +s3);
    if (xl && yh && zl) RET(F_XLO_YHI_ZLO, -s3, +s3, -s3);
    if (xl && yh && zh) RET(F_XLO_YHI_ZHI, -s3, +s3, +s3);
    if (xh && yl && zl) RET(F_XHI_YLO_ZLO, +s3, -s3, -s3);
    if (xh && yl && zh) RET(F_XHI_YLO_ZHI, +s3, -s3, +s3);
    if (xh && yh && zl) RET(F_XHI_YHI_ZLO, +s3, +s3, -s3);
    if (xh && yh && zh) RET(F_XHI_YHI_ZHI, +s3, +s3, +s3);
    if (yl && zl) RET(F_YLO_ZLO, 0, -s2, -s2);
    if (yl && zh) RET(F_YLO_ZHI, 0, -s2, +s2);
    if (yh && zl) RET(F_YHI_ZLO, 0, +s2, -s2);
    if (yh && zh) RET(F_YHI_ZHI, 0, +s2, +s2);
    if (zl && xl) RET(F_ZLO_XLO, -s2, 0, -s2);
    if (zl && xh) RET(F_ZLO_XHI, +s2, 0, -s2);
    if (zh && xl) RET(F_ZHI_XLO, -s2, 0, +s2);
    if (zh && xh) RET(F_ZHI_XHI, +s2, 0, +s2);
    if (xl && yl) RET(F_XLO_YLO, -s2, -s2, 0);
    if (xl && yh) RET(F_XLO_YHI, -s2, +s2, 0);
    if (xh && yl) RET(F_XHI_YLO, +s2, -s2, 0);
    if (xh && yh) RET(F_XHI_YHI, +s2, +s2, 0);
    if (xl) RET(F_XLO, -1, 0, 0);
    if (xh) RET(F_XHI, +1, 0, 0);
    if (yl) RET(F_YLO, 0, -1, 0);
    if (yh) RET(F_YHI, 0, +1, 0);
    if (zl) RET(F_ZLO, 0, 0, -1);
    if (zh) RET(F_ZHI, 0, 0, +1);
#undef RET
    nrm[0] = nrm[1] = nrm[2] = 0;
    return -1;
}

// Constant::set, Constant.H:408-425
template <typename T>
__device__ __forceinline__ void bc_set(const int8_t* type, const T u[3], const T G[3][3], const T S[3][3],
                                       const double nd[3], T f[3])
{
    const T n[3] = {(T)nd[0], (T)nd[1], (T)nd[2]};
#pragma unroll
    for (int i = 0; i < 3; i++) {
        T v = 0;
        if (type[i] == BCT_DISP) v = u[i];
        else if (type[i] == BCT_TRAC) v = S[i][0] * n[0] + S[i][1] * n[1] + S[i][2] * n[2];
        else if (type[i] == BCT_NEUMANN) v = G[i][0] * n[0] + G[i][1] * n[1] + G[i][2] * n[2];
        f[i] = v;
    }
}

// Boundary row of Fapply at a node with lo/hi flags mn/mx (at least one set).
template <typename T, int SYM, class A>
__device__ __forceinline__ void boundary_row(const A& acc, const Geo<T>& g, const BCTable& bc, const int mn[3],
                                             const int mx[3], T f[3])
{
    T G[3][3], S[3][3], u[3];
#pragma unroll
    for (int p = 0; p < 3; p++) {
        u[p] = acc.u(p, 0, 0, 0);
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const int ox = d == 0, oy = d == 1, oz = d == 2;
            if (mn[d]) G[p][d] = (acc.u(p, ox, oy, oz) - u[p]) * g.i1[d];          // StencilType::Hi
            else if (mx[d]) G[p][d] = (u[p] - acc.u(p, -ox, -oy, -oz)) * g.i1[d];  // StencilType::Lo
            else G[p][d] = (acc.u(p, ox, oy, oz) - acc.u(p, -ox, -oy, -oz)) * g.h1[d];
        }
    }
    T c[NCoef<SYM>::value];
#pragma unroll
    for (int m = 0; m < NCoef<SYM>::value; m++) c[m] = acc.C(m, 0, 0, 0);
    c_mul_mat<T, SYM>(c, G, S);
    double nrm[3];
    const int face = face_of(mn, mx, nrm);
    bc_set<T>(bc.type[face], u, G, S, nrm, f);
}

// -2 / dx_d^2 in the arithmetic type, as the interior diagonal uses it
// (evaluated once per launch or thread, not per entry: FP64 division is slow).
template <typename T> struct DiagGeo {
    T h2m[3];
};
template <typename T> __host__ __device__ inline DiagGeo<T> make_diag_geo(const LevelDesc& L)
{
    DiagGeo<T> dg;
    for (int d = 0; d < 3; d++) dg.h2m[d] = (T)(-2.0 / L.dx[d] / L.dx[d]);
    return dg;
}

// Diagonal of one component p at a node, Operator/Elastic.cpp:321-365.
template <typename T, int SYM>
__device__ __forceinline__ T diag_entry(const T* c, const LevelDesc& L, const DiagGeo<T>& dg, const BCTable& bc,
                                        const int mn[3], const int mx[3], int p)
{
    const bool bnd = mn[0] | mx[0] | mn[1] | mx[1] | mn[2] | mx[2];
    if (bnd) {
        // Gradient_Diagonal<Matrix>, Numeric/Stencil.H:906-930
        T G[3][3], S[3][3], u[3] = {0, 0, 0}, f[3];
        for (int q = 0; q < 3; q++)
            for (int d = 0; d < 3; d++) {
                const double e = (p == q) ? 1.0 : 0.0;
                G[q][d] = (T)(((!mx[d] ? 0.0 : e) - (!mn[d] ? 0.0 : e)) / ((mn[d] || mx[d] ? 1.0 : 2.0) * L.dx[d]));
            }
        c_mul_mat<T, SYM>(c, G, S);
        u[p] = 1;
        double nrm[3];
        const int face = face_of(mn, mx, nrm);
        bc_set<T>(bc.type[face], u, G, S, nrm, f);
        return f[p];
    }
    // Gradient_Diagonal<Matrix3>, Numeric/Stencil.H:932-962
    T H[3][3][3];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++)
            for (int d = 0; d < 3; d++) H[a][b][d] = 0;
    for (int d = 0; d < 3; d++) H[p][d][d] = dg.h2m[d];
    T f[3];
    c_mul_m3<T, SYM>(c, H, f);
    return f[p];
}

}  // namespace agb
