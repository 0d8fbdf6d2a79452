// Element-level formulas shared by the assembly and the adjoint kernels:
// local edge geometry of a brick, its curl-curl and mass entries, and the
// 1-D table interpolation of the normal field.
#pragma once
#include "mtgpu_internal.cuh"

namespace mtgpu {

// local edge -> direction (0 x, 1 y, 2 z), the grouping of T_Portrait.h:37-51
__device__ __forceinline__ int ldir(int l) { return l >> 2; }

// side (0/1) of local edge l along axis a (a != its direction), from the
// edge midpoints of T_Brick.h:201-214
__device__ __forceinline__ int lpos(int l, int a)
{
    // bit 0 / bit 1 of the position inside the direction group:
    // x-edges (y, z) = (l&1, l>>1 &1); y-edges (x, z) = (l>>1 &1, l&1);
    // z-edges (x, y) = (l&1, l>>1 &1)
    const int d = l >> 2, k = l & 3;
    if (d == 0) return a == 1 ? (k & 1) : ((k >> 1) & 1);
    if (d == 1) return a == 0 ? ((k >> 1) & 1) : (k & 1);
    return a == 0 ? (k & 1) : ((k >> 1) & 1);
}

// entries (i, j) of the local curl-curl b and mass c matrices of a brick
// (closed forms of T_Brick.cpp:123-455 in tensor-product form; see
// oracle/mtcalc_oracle.c orc_brick_bc for the derivation)
__device__ __forceinline__ void brick_entry(int i, int j, const double h[3], double &b, double &c)
{
    const int da = ldir(i), db = ldir(j);
    if (da == db) {
        const int t1 = (da + 1) % 3, t2 = (da + 2) % 3;
        const bool s1 = lpos(i, t1) == lpos(j, t1);
        const bool s2 = lpos(i, t2) == lpos(j, t2);
        const double M1 = s1 ? 2.0 / 3.0 : 1.0 / 3.0, M2 = s2 ? 2.0 / 3.0 : 1.0 / 3.0;
        const double K1 = s1 ? 1.0 : -1.0, K2 = s2 ? 1.0 : -1.0;
        const double m1 = 2.0 * h[t1] / (h[da] * h[t2]);
        const double m2 = 2.0 * h[t2] / (h[da] * h[t1]);
        b = m1 * K2 * M1 + m2 * K1 * M2;
        c = (h[t1] * h[t2] / h[da]) * M1 * M2;
    } else {
        const int q = 3 - da - db;
        const double sa = lpos(i, db) ? 1.0 : -1.0;
        const double sb = lpos(j, da) ? 1.0 : -1.0;
        const double Mq = lpos(i, q) == lpos(j, q) ? 2.0 / 3.0 : 1.0 / 3.0;
        b = -(2.0 * h[q] / (h[da] * h[db])) * sa * sb * Mq;
        c = 0.0;
    }
}

__device__ __forceinline__ void cell_h(const double *xyz, const int *nver, int stride, int cell,
                                       double h[3])
{
    const int n0 = nver[(long long)cell * stride], n7 = nver[(long long)cell * stride + 7];
    h[0] = xyz[3 * n7 + 0] - xyz[3 * n0 + 0];
    h[1] = xyz[3 * n7 + 1] - xyz[3 * n0 + 1];
    h[2] = xyz[3 * n7 + 2] - xyz[3 * n0 + 2];
}

// linear interpolation of a 1-D table (For_Solvers.cpp:236-270); the table
// is sorted ascending, the interval is found by bisection
__device__ __forceinline__ double spline(double x, int n, const double *z, const double *v)
{
    if (x < z[0]) return v[0];
    if (x > z[n - 1]) return v[n - 1];
    int lo = 0, hi = n - 2;
    while (lo < hi) {   // smallest t with x <= z[t+1]
        const int mid = (lo + hi) >> 1;
        if (x <= z[mid + 1]) hi = mid; else lo = mid + 1;
    }
    const double xi = (x - z[lo]) / (z[lo + 1] - z[lo]);
    return (1.0 - xi) * v[lo] + xi * v[lo + 1];
}

}  // namespace mtgpu
