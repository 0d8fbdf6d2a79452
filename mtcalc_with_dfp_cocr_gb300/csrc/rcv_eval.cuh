// Device helpers shared by the two receiver output paths (receivers.cu:
// direct evaluation at the receiver; smoothing.cu: subdomain smoothing):
// the edge-element field in one brick, Harm1D's 1-D normal field at the
// receiver depth, and the total E and H of a receiver.
#pragma once
#include <cmath>

namespace mtgpu {
namespace rcv {

constexpr double kPi = 3.1415926535897932384626433832795;   // OutputNu/stdafx.h:32
constexpr double kMu0 = 1.25663706143591729e-6;              // OutputNu/stdafx.h:31
constexpr double kMu0_1d = 4.0 * 3.1415926535897932 * 1e-7;  // Harm1D/divgrad_1d.cpp:288

// Harm1D's table interpolation (divgrad_1d.cpp:50-88): the first interval
// [z_i, z_i+1] holding x, constant beyond the ends
__device__ inline double table_value(double x, int n, const double *z, const double *v)
{
    if (x < z[0]) return v[0];
    if (x > z[n - 1]) return v[n - 1];
    int lo = 0, hi = n - 2;
    while (lo < hi) {   // smallest t with x <= z[t+1]
        const int mid = (lo + hi) >> 1;
        if (x <= z[mid + 1]) hi = mid; else lo = mid + 1;
    }
    const double t = (x - z[lo]) / (z[lo + 1] - z[lo]);
    return (1.0 - t) * v[lo] + t * v[lo + 1];
}

// Harm1D's table derivative (divgrad_1d.cpp:90-138): end slopes outside
// [z_1, z_n-2]; inside, node slopes (weighted means of the adjacent interval
// slopes) interpolated over the interval ending at the first z_i >= x
__device__ inline double table_slope(double x, int n, const double *z, const double *v)
{
    if (x < z[1]) return (v[1] - v[0]) / (z[1] - z[0]);
    if (x > z[n - 2]) return (v[n - 1] - v[n - 2]) / (z[n - 1] - z[n - 2]);
    int lo = 1, hi = n - 1;
    while (lo < hi) {   // smallest i >= 1 with x <= z[i]
        const int mid = (lo + hi) >> 1;
        if (x <= z[mid]) hi = mid; else lo = mid + 1;
    }
    const int i = lo;
    if (i < 2 || i + 1 >= n) return (v[i] - v[i - 1]) / (z[i] - z[i - 1]);
    const double w0 = (z[i - 1] - z[i - 2]) / (z[i] - z[i - 2]);
    const double d0 = (v[i - 1] - v[i - 2]) / (z[i - 1] - z[i - 2]) * (1.0 - w0) +
                      (v[i] - v[i - 1]) / (z[i] - z[i - 1]) * w0;
    const double w1 = (z[i] - z[i - 1]) / (z[i + 1] - z[i - 1]);
    const double d1 = (v[i] - v[i - 1]) / (z[i] - z[i - 1]) * (1.0 - w1) +
                      (v[i + 1] - v[i]) / (z[i + 1] - z[i]) * w1;
    const double t = (x - z[i - 1]) / (z[i] - z[i - 1]);
    return (1.0 - t) * d0 + t * d1;
}

__device__ __forceinline__ double lin0(double t) { return 0.5 * (1.0 - t); }
__device__ __forceinline__ double lin1(double t) { return 0.5 * (1.0 + t); }

// A and curl A at local point (xi, eta, zeta) of a brick with sizes
// (hx, hy, hz) from its 12 edge values v (complex): edge i of direction d
// carries (2/h_d) l_a l_b in the two other local coordinates
// (T_Brick.cpp:980-1137), the curl uses l0' = -1/2, l1' = 1/2
// (T_Brick.cpp:1484-1618, 1842-1918).
__device__ inline void brick_eval(const double2 (&v)[12], double xi, double et, double ze,
                                  double hx, double hy, double hz, double2 (&A)[3],
                                  double2 (&C)[3])
{
    const double cx[4] = {lin0(et) * lin0(ze), lin1(et) * lin0(ze), lin0(et) * lin1(ze),
                          lin1(et) * lin1(ze)};
    const double cy[4] = {lin0(ze) * lin0(xi), lin1(ze) * lin0(xi), lin0(ze) * lin1(xi),
                          lin1(ze) * lin1(xi)};
    const double cz[4] = {lin0(xi) * lin0(et), lin1(xi) * lin0(et), lin0(xi) * lin1(et),
                          lin1(xi) * lin1(et)};
    const double sx = 2.0 / hx, sy = 2.0 / hy, sz = 2.0 / hz;
    const double rx = 2.0 / (hy * hz), ry = 2.0 / (hx * hz), rz = 2.0 / (hx * hy);
#define MTGPU_PART(f)                                                                      \
    {                                                                                      \
        A[0].f = sx * (v[0].f * cx[0] + v[1].f * cx[1] + v[2].f * cx[2] + v[3].f * cx[3]); \
        A[1].f = sy * (v[4].f * cy[0] + v[5].f * cy[1] + v[6].f * cy[2] + v[7].f * cy[3]); \
        A[2].f = sz * (v[8].f * cz[0] + v[9].f * cz[1] + v[10].f * cz[2] + v[11].f * cz[3]); \
        C[0].f = rx * (lin0(xi) * (v[4].f - v[5].f - v[8].f + v[10].f) +                  \
                       lin1(xi) * (v[6].f - v[7].f - v[9].f + v[11].f));                  \
        C[1].f = ry * (lin0(et) * (v[2].f - v[0].f + v[8].f - v[9].f) +                   \
                       lin1(et) * (v[3].f - v[1].f + v[10].f - v[11].f));                 \
        C[2].f = rz * (lin0(ze) * (v[0].f - v[1].f - v[4].f + v[6].f) +                   \
                       lin1(ze) * (v[2].f - v[3].f - v[5].f + v[7].f));                   \
    }
    MTGPU_PART(x)
    MTGPU_PART(y)
#undef MTGPU_PART
}

// Total fields of receiver r in system k from A and curl A there:
// E = -i omega A plus the 1-D field on x and y; H = curl A / mu0 plus the
// 1-D field on x and y (give_out_vec_mt.cpp:135-195, 232-266; Harm1D
// divgrad_1d.cpp:290-330); and the scalars rho, |Z| of
// give_out_vec_mt.cpp:247-264.  z: the receiver depth.
__device__ inline void total_fields(const double2 (&A)[3], const double2 (&C)[3], double w,
                                    int alfa, double z, int n1d, const double *z1d,
                                    const double *us, const double *uc, double2 *e_out,
                                    double2 *h_out, double2 *scal)
{
    double2 E[3], H[3];
    for (int d = 0; d < 3; d++) {
        E[d] = make_double2(w * A[d].y, -w * A[d].x);
        H[d] = make_double2(C[d].x / kMu0, C[d].y / kMu0);
    }
    {
        const double a = alfa ? 1.0 : 0.0;
        double ds = kMu0_1d, dc = 0.0;
        if (z < 0.0) {
            ds = table_slope(z, n1d, z1d, us);
            dc = table_slope(z, n1d, z1d, uc);
        }
        const double zz = z > 0.0 ? 0.0 : z;
        const double fs = table_value(zz, n1d, z1d, us), fc = table_value(zz, n1d, z1d, uc);
        E[0].x += w * a * fc;
        E[0].y += -w * a * fs;
        E[1].x += w * (1.0 - a) * fc;
        E[1].y += w * (a - 1.0) * fs;
        H[0].x += (a - 1.0) * ds / kMu0;
        H[0].y += (a - 1.0) * dc / kMu0;
        H[1].x += a * ds / kMu0;
        H[1].y += a * dc / kMu0;
    }
    for (int d = 0; d < 3; d++) {
        e_out[d] = E[d];
        h_out[d] = H[d];
    }
    const double ere = sqrt(E[0].x * E[0].x + E[1].x * E[1].x + E[2].x * E[2].x);
    const double eim = sqrt(E[0].y * E[0].y + E[1].y * E[1].y + E[2].y * E[2].y);
    const double hre = sqrt(H[0].x * H[0].x + H[1].x * H[1].x + H[2].x * H[2].x);
    const double him = sqrt(H[0].y * H[0].y + H[1].y * H[1].y + H[2].y * H[2].y);
    const double q = sqrt(ere * ere + eim * eim) / sqrt(hre * hre + him * him);
    *scal = make_double2(q * q / (w * kMu0), q);
}

}  // namespace rcv
}  // namespace mtgpu
