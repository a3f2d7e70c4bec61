// transfer.cuh -- per-node arithmetic of the inter-level transfers, shared
// by the single-box and batched kernels.
//
//   restriction     Operator<Node>::restriction, Operator/Operator.cpp:262-363
//   prolongation    Operator<Node>::interpolation, Operator.cpp:365-434
#pragma once
#include "agb_internal.h"

namespace agb {

// index i of a direction of n cells, folded into [0, n) when periodic
__device__ __forceinline__ int wrapn(int i, int n, int per)
{
    if (per) {
        if (i < 0) return i + n;
        if (i >= n) return i - n;
    }
    return i;
}

// Nodal full weighting with lower-dimensional stencils on the coarse domain
// boundary; the same weights serve the residual restriction and the modulus
// averaging.  F(a,b,c) returns the fine value at (2I+a, 2J+b, 2K+c).
template <typename T, class F>
__device__ __forceinline__ T full_weight(const F& f, bool bI, bool bJ, bool bK)
{
    if (bI && bJ && bK) return f(0, 0, 0);
    if (bJ && bK) return (T)0.25 * f(-1, 0, 0) + (T)0.5 * f(0, 0, 0) + (T)0.25 * f(1, 0, 0);
    if (bK && bI) return (T)0.25 * f(0, -1, 0) + (T)0.5 * f(0, 0, 0) + (T)0.25 * f(0, 1, 0);
    if (bI && bJ) return (T)0.25 * f(0, 0, -1) + (T)0.5 * f(0, 0, 0) + (T)0.25 * f(0, 0, 1);
    if (bI)
        return (f(0, -1, -1) + (T)2 * f(0, 0, -1) + f(0, 1, -1) + (T)2 * f(0, -1, 0) + (T)4 * f(0, 0, 0) +
                (T)2 * f(0, 1, 0) + f(0, -1, 1) + (T)2 * f(0, 0, 1) + f(0, 1, 1)) * (T)(1.0 / 16.0);
    if (bJ)
        return (f(-1, 0, -1) + (T)2 * f(-1, 0, 0) + f(-1, 0, 1) + (T)2 * f(0, 0, -1) + (T)4 * f(0, 0, 0) +
                (T)2 * f(0, 0, 1) + f(1, 0, -1) + (T)2 * f(1, 0, 0) + f(1, 0, 1)) * (T)(1.0 / 16.0);
    if (bK)
        return (f(-1, -1, 0) + (T)2 * f(0, -1, 0) + f(1, -1, 0) + (T)2 * f(-1, 0, 0) + (T)4 * f(0, 0, 0) +
                (T)2 * f(1, 0, 0) + f(-1, 1, 0) + (T)2 * f(0, 1, 0) + f(1, 1, 0)) * (T)(1.0 / 16.0);
    return (f(-1, -1, -1) + f(-1, -1, 1) + f(-1, 1, -1) + f(-1, 1, 1) + f(1, -1, -1) + f(1, -1, 1) + f(1, 1, -1) +
            f(1, 1, 1)) * (T)(1.0 / 64.0) +
           (f(0, -1, -1) + f(0, -1, 1) + f(0, 1, -1) + f(0, 1, 1) + f(-1, 0, -1) + f(1, 0, -1) + f(-1, 0, 1) +
            f(1, 0, 1) + f(-1, -1, 0) + f(-1, 1, 0) + f(1, -1, 0) + f(1, 1, 0)) * (T)(1.0 / 32.0) +
           (f(-1, 0, 0) + f(0, -1, 0) + f(0, 0, -1) + f(1, 0, 0) + f(0, 1, 0) + f(0, 0, 1)) * (T)(1.0 / 16.0) +
           f(0, 0, 0) * (T)(1.0 / 8.0);
}

// Trilinear prolongation at the fine node (2I + !ei, 2J + !ej, 2K + !ek):
// C(a, b, d) returns the coarse value at (I + a, J + b, K + d) (periodic
// images folded in by the caller).
template <typename T, class F>
__device__ __forceinline__ T interp_node(const F& C, bool ei, bool ej, bool ek)
{
    if (ei && ej && ek) return C(0, 0, 0);
    if (ej && ek) return (T)0.5 * (C(0, 0, 0) + C(1, 0, 0));
    if (ek && ei) return (T)0.5 * (C(0, 0, 0) + C(0, 1, 0));
    if (ei && ej) return (T)0.5 * (C(0, 0, 0) + C(0, 0, 1));
    if (ei) return (T)0.25 * (C(0, 0, 0) + C(0, 1, 0) + C(0, 0, 1) + C(0, 1, 1));
    if (ej) return (T)0.25 * (C(0, 0, 0) + C(0, 0, 1) + C(1, 0, 0) + C(1, 0, 1));
    if (ek) return (T)0.25 * (C(0, 0, 0) + C(1, 0, 0) + C(0, 1, 0) + C(1, 1, 0));
    return (T)0.125 * (C(0, 0, 0) + C(1, 0, 0) + C(0, 1, 0) + C(0, 0, 1) + C(0, 1, 1) + C(1, 0, 1) + C(1, 1, 0) +
                       C(1, 1, 1));
}

}  // namespace agb
