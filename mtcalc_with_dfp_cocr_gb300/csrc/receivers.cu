// Receivers: E and H at receiver points from device solutions, and the MT
// responses (impedance tensor, tipper, apparent resistivities) per receiver
// and frequency.  Replaces the direct-evaluation output of the reference
// (Code/OutputNu/give_out_vec_mt.cpp:101-266 with
// OutputVect3d::OutputFieldAtReceivers, OutputArbitrary.cpp:202-293) and the
// impedance program Code/calcimpedance/calcimpedance.for:125-301.
//
// Work is tiny next to the solve (receivers x systems threads), so every
// kernel runs in FP64 with one thread per (receiver, system) or (receiver,
// frequency); the only sizeable step is the one-off receiver location, a
// scan of all bricks against the receiver list staged in shared memory.
#include "receivers.cuh"

#include <climits>
#include <cmath>

namespace mtgpu {
namespace {

constexpr double kPi = 3.1415926535897932384626433832795;   // OutputNu/stdafx.h:32
constexpr double kMu0 = 1.25663706143591729e-6;              // OutputNu/stdafx.h:31
constexpr double kMu0_1d = 4.0 * 3.1415926535897932 * 1e-7;  // Harm1D/divgrad_1d.cpp:288
constexpr int kLocChunk = 256;                               // receivers per shared-memory pass

__global__ void k_rcv_init(int nrec, int *elem)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nrec) elem[r] = INT_MAX;
}

// elem[r] = the lowest brick index whose closed box [vertex 0, vertex 7]
// holds receiver r (OutputArbitrary.cpp:385-500 keeps the first one found
// in index order).  One thread per brick; receivers pass through shared
// memory in chunks.
__global__ void __launch_bounds__(kThreads)
k_rcv_locate(int kpar, const int *__restrict__ nver, int nver_stride,
             const double *__restrict__ xyz, int nrec, const double *__restrict__ rec, int *elem)
{
    __shared__ double sx[kLocChunk], sy[kLocChunk], sz[kLocChunk];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double lo[3] = {0, 0, 0}, hi[3] = {-1, -1, -1};   // empty box for idle threads
    if (e < kpar) {
        const int v0 = nver[(long long)e * nver_stride], v7 = nver[(long long)e * nver_stride + 7];
        for (int d = 0; d < 3; d++) {
            lo[d] = xyz[3 * v0 + d];
            hi[d] = xyz[3 * v7 + d];
        }
    }
    for (int base = 0; base < nrec; base += kLocChunk) {
        const int n = min(kLocChunk, nrec - base);
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            sx[j] = rec[3 * (base + j)];
            sy[j] = rec[3 * (base + j) + 1];
            sz[j] = rec[3 * (base + j) + 2];
        }
        __syncthreads();
        for (int j = 0; j < n; j++) {
            if (sx[j] >= lo[0] && sx[j] <= hi[0] && sy[j] >= lo[1] && sy[j] <= hi[1] &&
                sz[j] >= lo[2] && sz[j] <= hi[2])
                atomicMin(&elem[base + j], e);
        }
    }
}

// per receiver: its brick's 12 edges, local coordinates and sizes
__global__ void k_rcv_prepare(int nrec, int *elem, const int *__restrict__ nver, int nver_stride,
                              const int *__restrict__ ed, int ed_stride,
                              const double *__restrict__ xyz, const double *__restrict__ rec,
                              int *edge, double4 *loc, double4 *hsz)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    int e = elem[r];
    if (e == INT_MAX) {
        elem[r] = -1;
        for (int i = 0; i < 12; i++) edge[12 * r + i] = 0;
        loc[r] = make_double4(0, 0, 0, rec[3 * r + 2]);
        hsz[r] = make_double4(1, 1, 1, 0);
        return;
    }
    const int v0 = nver[(long long)e * nver_stride], v7 = nver[(long long)e * nver_stride + 7];
    double l[3], h[3];
    for (int d = 0; d < 3; d++) {
        const double a = xyz[3 * v0 + d], b = xyz[3 * v7 + d];
        h[d] = b - a;
        // T_Brick.cpp:2010-2023 (Xi, Eta, Zeta)
        l[d] = (2.0 * rec[3 * r + d] - a - b) / h[d];
    }
    for (int i = 0; i < 12; i++) edge[12 * r + i] = ed[(long long)e * ed_stride + i];
    loc[r] = make_double4(l[0], l[1], l[2], rec[3 * r + 2]);
    hsz[r] = make_double4(h[0], h[1], h[2], 0.0);
}

// Harm1D's table interpolation (divgrad_1d.cpp:50-88): the first interval
// [z_i, z_i+1] holding x, constant beyond the ends
__device__ double table_value(double x, int n, const double *z, const double *v)
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
__device__ double table_slope(double x, int n, const double *z, const double *v)
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

// One thread per (receiver, system).  A from the 12 edge DOFs of the
// receiver's brick (edge i of direction d carries (2/h_d) l_a l_b in the two
// other local coordinates, T_Brick.cpp:980-1137), curl A from l0' = -1/2,
// l1' = 1/2 (T_Brick.cpp:1484-1618, 1842-1918).  E = -i omega A plus the 1-D
// field on x and y; H = curl A / mu0 plus the 1-D field on x and y
// (give_out_vec_mt.cpp:135-195, 232-266; Harm1D divgrad_1d.cpp:290-330).
__global__ void k_rcv_fields(int nrec, int S, long long x_stride, const double2 *__restrict__ x,
                             const double *__restrict__ omega, const int *__restrict__ alfa,
                             int n1d, const double *__restrict__ z1d,
                             const double *__restrict__ usin, const double *__restrict__ ucos,
                             const int *__restrict__ elem, const int *__restrict__ edge,
                             const double4 *__restrict__ loc, const double4 *__restrict__ hsz,
                             double2 *e_out, double2 *h_out, double2 *scal)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (r >= nrec || k >= S) return;
    const double w = omega[k];
    double2 A[3] = {}, C[3] = {};
    if (elem[r] >= 0) {
        const double4 L = loc[r], Hs = hsz[r];
        const double xi = L.x, et = L.y, ze = L.z, hx = Hs.x, hy = Hs.y, hz = Hs.z;
        const double2 *xs = x + (long long)k * x_stride;
        double2 v[12];
#pragma unroll
        for (int i = 0; i < 12; i++) v[i] = xs[edge[12 * r + i]];
        const double cx[4] = {lin0(et) * lin0(ze), lin1(et) * lin0(ze), lin0(et) * lin1(ze),
                              lin1(et) * lin1(ze)};
        const double cy[4] = {lin0(ze) * lin0(xi), lin1(ze) * lin0(xi), lin0(ze) * lin1(xi),
                              lin1(ze) * lin1(xi)};
        const double cz[4] = {lin0(xi) * lin0(et), lin1(xi) * lin0(et), lin0(xi) * lin1(et),
                              lin1(xi) * lin1(et)};
        const double sx = 2.0 / hx, sy = 2.0 / hy, sz = 2.0 / hz;
        const double rx = 2.0 / (hy * hz), ry = 2.0 / (hx * hz), rz = 2.0 / (hx * hy);
#define MTGPU_PART(f)                                                                         \
        {                                                                                     \
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
    double2 E[3], H[3];
    for (int d = 0; d < 3; d++) {
        E[d] = make_double2(w * A[d].y, -w * A[d].x);
        H[d] = make_double2(C[d].x / kMu0, C[d].y / kMu0);
    }
    // 1-D normal field at the receiver depth
    {
        const double z = loc[r].w;
        const double a = alfa[k] ? 1.0 : 0.0;
        const double *us = usin + (long long)k * n1d, *uc = ucos + (long long)k * n1d;
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
    const long long o = ((long long)k * nrec + r) * 3;
    for (int d = 0; d < 3; d++) {
        e_out[o + d] = E[d];
        h_out[o + d] = H[d];
    }
    // give_out_vec_mt.cpp:247-264: moduli of the real and imaginary parts
    const double ere = sqrt(E[0].x * E[0].x + E[1].x * E[1].x + E[2].x * E[2].x);
    const double eim = sqrt(E[0].y * E[0].y + E[1].y * E[1].y + E[2].y * E[2].y);
    const double hre = sqrt(H[0].x * H[0].x + H[1].x * H[1].x + H[2].x * H[2].x);
    const double him = sqrt(H[0].y * H[0].y + H[1].y * H[1].y + H[2].y * H[2].y);
    const double q = sqrt(ere * ere + eim * eim) / sqrt(hre * hre + him * him);
    scal[(long long)k * nrec + r] = make_double2(q * q / (w * kMu0), q);
}

// calcimpedance.for:163-171: quadrant rule, then the near-axis overrides in
// order (a later match wins); 0 where nothing matches
__device__ double mt_phase(double re, double im, bool overrides)
{
    double f = 0.0;
    if (re > 0.0 && im > 0.0) f = atan(im / re);
    if (re < 0.0 && im > 0.0) f = atan(im / re) + kPi;
    if (re < 0.0 && im < 0.0) f = atan(im / re) - kPi;
    if (re > 0.0 && im < 0.0) f = atan(im / re);
    if (overrides) {
        if (re > 0.0 && fabs(im) < 1e-15) f = 0.0;
        if (fabs(re) < 1e-15 && im > 0.0) f = kPi / 2.0;
        if (re < 0.0 && fabs(im) < 1e-15) f = kPi;
        if (fabs(re) < 1e-15 && im < 0.0) f = -kPi / 2.0;
    }
    return f;
}

__device__ __forceinline__ double det3(double a, double b, double c, double d, double e,
                                       double f, double g, double h, double i)
{
    return a * e * i + d * h * c + b * f * g - c * e * g - b * d * i - a * f * h;
}

// One thread per (receiver, frequency).  With the X- and Y-polarisation
// fields, E = Z H for both gives the real 4x4 system B u = f of
// calcimpedance.for:125-156 per right-hand side (Ex, Ey, Hz); B is inverted
// by cofactors over a first-row determinant (makeQ, :346-416), in FP64.
__global__ void k_mt_response(int nrec, int nf, const double *__restrict__ omega,
                              const int *__restrict__ sys_x, const int *__restrict__ sys_y,
                              const double2 *__restrict__ E, const double2 *__restrict__ H,
                              double *out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (r >= nrec || f >= nf) return;
    const double2 *e0 = E + ((long long)sys_x[f] * nrec + r) * 3;
    const double2 *h0 = H + ((long long)sys_x[f] * nrec + r) * 3;
    const double2 *e1 = E + ((long long)sys_y[f] * nrec + r) * 3;
    const double2 *h1 = H + ((long long)sys_y[f] * nrec + r) * 3;
    double B[16];
    const double2 *hh[2] = {h0, h1};
    for (int p = 0; p < 2; p++) {
        const double2 hx = hh[p][0], hy = hh[p][1];
        double *r0 = B + 8 * p, *r1 = B + 8 * p + 4;
        r0[0] = hx.x; r0[1] = -hx.y; r0[2] = hy.x; r0[3] = -hy.y;
        r1[0] = hx.y; r1[1] = hx.x;  r1[2] = hy.y; r1[3] = hy.x;
    }
    double cof[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double m[9];
            int k = 0;
            for (int rr = 0; rr < 4; rr++) {
                if (rr == i) continue;
                for (int c = 0; c < 4; c++)
                    if (c != j) m[k++] = B[4 * rr + c];
            }
            cof[4 * i + j] = (((i + j) & 1) ? -1.0 : 1.0) *
                             det3(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8]);
        }
    double det = 0.0;
    for (int j = 0; j < 4; j++) det += B[j] * cof[j];
    double u[12];   // Zxx, Zxy | Zyx, Zyy | Wzx, Wzy as (re, im)
    for (int c = 0; c < 3; c++) {
        const double2 a = c < 2 ? e0[c] : h0[2], b = c < 2 ? e1[c] : h1[2];
        const double fv[4] = {a.x, a.y, b.x, b.y};
        for (int i = 0; i < 4; i++) {
            double s = 0.0;
            for (int j = 0; j < 4; j++) s += cof[4 * j + i] / det * fv[j];
            u[4 * c + i] = s;
        }
    }
    const double mu0 = 4.0 * kPi * 1e-7;   // calcimpedance.for:41
    const double deg = 180.0 / kPi, w = omega[f];
    double *o = out + ((long long)f * nrec + r) * MTGPU_MT_RECORD;
    for (int i = 0; i < 12; i++) o[i] = u[i];
    for (int k = 0; k < 4; k++) {
        const double re = u[2 * k], im = u[2 * k + 1];
        const double m = sqrt(re * re + im * im), ph = mt_phase(re, im, true);
        o[MTGPU_MT_ZABS + k] = m;
        o[MTGPU_MT_ZPHASE + k] = -ph * deg;
        o[MTGPU_MT_RHO + k] = m * m / (mu0 * w);
        o[MTGPU_MT_RHOPHASE + k] = -2.0 * ph * deg;
    }
    // calcimpedance.for:259-276: det Z = Zxx Zyy - Zyx Zxy
    const double dre = (u[0] * u[6] - u[1] * u[7]) - (u[4] * u[2] - u[5] * u[3]);
    const double dim = (u[0] * u[7] + u[1] * u[6]) - (u[4] * u[3] + u[5] * u[2]);
    const double zmod = sqrt(sqrt(dre * dre + dim * dim));
    o[MTGPU_MT_RHOEFF] = zmod * zmod / (mu0 * w);
    o[MTGPU_MT_RHOEFF + 1] = -2.0 * (mt_phase(dre, dim, false) / 2.0) * deg;
    for (int k = 0; k < 2; k++) {
        const double re = u[8 + 2 * k], im = u[9 + 2 * k];
        o[MTGPU_MT_WABS + k] = sqrt(re * re + im * im);
        o[MTGPU_MT_WABS + 2 + k] = -mt_phase(re, im, true) * deg;
    }
}

}  // namespace
}  // namespace mtgpu

using namespace mtgpu;

extern "C" {

void mtgpu_receivers_destroy(mtgpu_receivers *r)
{
    if (!r) return;
    if (r->st) cudaStreamSynchronize(r->st);
    dev_free(r->d_elem);
    dev_free(r->d_edge);
    dev_free(r->d_loc);
    dev_free(r->d_h);
    dev_free(r->d_omega);
    dev_free(r->d_tab);
    dev_free(r->d_int);
    dev_free(r->d_contrib);
    dev_free(r->d_misfit);
    dev_free(r->d_touch_ptr);
    dev_free(r->d_touch_edge);
    dev_free(r->d_touch_slot);
    if (r->st) cudaStreamDestroy(r->st);
    delete r;
}

int mtgpu_receivers_create(const mtgpu_assembly *a, int nrec, const double *xyz_rec,
                           mtgpu_receivers **out)
{
    MTGPU_CHECK_ARG(a && xyz_rec && out, "null argument");
    MTGPU_CHECK_ARG(nrec > 0, "nrec must be positive");
    *out = nullptr;
    auto *r = new mtgpu_receivers_s();
    r->nrec = nrec;
    r->nb = a->P.nb;
    int rc = MTGPU_OK;
    double *d_rec = nullptr;
    do {
        cudaError_t e = cudaStreamCreateWithFlags(&r->st, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            set_last_error(e, "cudaStreamCreateWithFlags", __FILE__, __LINE__);
            rc = MTGPU_ERR_CUDA;
            break;
        }
        if ((rc = dev_alloc(&r->d_elem, nrec)) || (rc = dev_alloc(&r->d_edge, (size_t)12 * nrec)) ||
            (rc = dev_alloc(&r->d_loc, nrec)) || (rc = dev_alloc(&r->d_h, nrec)) ||
            (rc = dev_alloc(&d_rec, (size_t)3 * nrec)))
            break;
        // the assembly's uploads run on its own stream
        e = cudaStreamSynchronize(a->st);
        if (e != cudaSuccess) {
            set_last_error(e, "cudaStreamSynchronize", __FILE__, __LINE__);
            rc = MTGPU_ERR_CUDA;
            break;
        }
        e = cudaMemcpyAsync(d_rec, xyz_rec, sizeof(double) * 3 * nrec, cudaMemcpyHostToDevice,
                            r->st);
        if (e != cudaSuccess) {
            set_last_error(e, "cudaMemcpyAsync", __FILE__, __LINE__);
            rc = MTGPU_ERR_CUDA;
            break;
        }
        const ParamMatrix &P = a->P;
        k_rcv_init<<<ceil_div(nrec, kThreads), kThreads, 0, r->st>>>(nrec, r->d_elem);
        k_rcv_locate<<<ceil_div(P.kpar, kThreads), kThreads, 0, r->st>>>(
            P.kpar, P.d_nver, P.nver_stride, P.d_xyz, nrec, d_rec, r->d_elem);
        k_rcv_prepare<<<ceil_div(nrec, kThreads), kThreads, 0, r->st>>>(
            nrec, r->d_elem, P.d_nver, P.nver_stride, P.d_ed, P.ed_stride, P.d_xyz, d_rec,
            r->d_edge, r->d_loc, r->d_h);
        note_launches(3);
        r->elem.resize(nrec);
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(r->elem.data(), r->d_elem, sizeof(int) * nrec,
                                cudaMemcpyDeviceToHost, r->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(r->st);
        if (e != cudaSuccess) {
            set_last_error(e, "receiver location", __FILE__, __LINE__);
            rc = MTGPU_ERR_CUDA;
            break;
        }
        for (int i = 0; i < nrec; i++) r->n_unlocated += r->elem[i] < 0;
    } while (0);
    dev_free(d_rec);
    if (rc) {
        mtgpu_receivers_destroy(r);
        return rc;
    }
    *out = r;
    return MTGPU_OK;
}

int mtgpu_receivers_info(const mtgpu_receivers *r, int *nrec, int *n_unlocated, int *elem)
{
    MTGPU_CHECK_ARG(r != nullptr, "null receivers");
    if (nrec) *nrec = r->nrec;
    if (n_unlocated) *n_unlocated = r->n_unlocated;
    if (elem)
        for (int i = 0; i < r->nrec; i++) elem[i] = r->elem[i];
    return MTGPU_OK;
}

int mtgpu_receivers_fields(mtgpu_receivers *r, int S, const double *nu, const int *alfa, int n1d,
                           const double *z1d, const double *usin, const double *ucos,
                           const double *d_x, double *d_e, double *d_h, double *d_rho_imp)
{
    MTGPU_CHECK_ARG(r && nu && alfa && z1d && usin && ucos && d_x && d_e && d_h,
                    "null argument");
    MTGPU_CHECK_ARG(S > 0 && S <= 65535, "S must be in [1, 65535]");
    MTGPU_CHECK_ARG(n1d >= 3, "the 1-D table needs at least 3 points");
    for (int i = 1; i < n1d; i++)
        MTGPU_CHECK_ARG(z1d[i] > z1d[i - 1], "z1d must be strictly ascending");
    MTGPU_CHECK_ARG(((uintptr_t)d_x % 16) == 0 && ((uintptr_t)d_e % 16) == 0 &&
                        ((uintptr_t)d_h % 16) == 0 && ((uintptr_t)d_rho_imp % 16) == 0,
                    "device arrays must be 16-byte aligned");
    int rc;
    if ((rc = ensure(&r->d_omega, &r->cap_omega, (size_t)S)) ||
        (rc = ensure(&r->d_int, &r->cap_int, (size_t)S)) ||
        (rc = ensure(&r->d_tab, &r->cap_tab, (size_t)n1d * (2 * S + 1))))
        return rc;
    std::vector<double> om(S);
    for (int k = 0; k < S; k++) om[k] = nu[k] * 2.0 * kPi;   // give_out_vec_mt.cpp:107
    double *d_z1d = r->d_tab, *d_us = r->d_tab + n1d, *d_uc = d_us + (size_t)S * n1d;
    MTGPU_TRY(cudaMemcpyAsync(r->d_omega, om.data(), sizeof(double) * S, cudaMemcpyHostToDevice,
                              r->st));
    MTGPU_TRY(cudaMemcpyAsync(r->d_int, alfa, sizeof(int) * S, cudaMemcpyHostToDevice, r->st));
    MTGPU_TRY(cudaMemcpyAsync(d_z1d, z1d, sizeof(double) * n1d, cudaMemcpyHostToDevice, r->st));
    MTGPU_TRY(cudaMemcpyAsync(d_us, usin, sizeof(double) * S * n1d, cudaMemcpyHostToDevice,
                              r->st));
    MTGPU_TRY(cudaMemcpyAsync(d_uc, ucos, sizeof(double) * S * n1d, cudaMemcpyHostToDevice,
                              r->st));
    dim3 grid(ceil_div(r->nrec, 128), S);
    k_rcv_fields<<<grid, 128, 0, r->st>>>(r->nrec, S, r->nb, (const double2 *)d_x, r->d_omega,
                                          r->d_int, n1d, d_z1d, d_us, d_uc, r->d_elem,
                                          r->d_edge, r->d_loc, r->d_h, (double2 *)d_e,
                                          (double2 *)d_h, (double2 *)d_rho_imp);
    note_launches(1);
    MTGPU_TRY(cudaGetLastError());
    MTGPU_TRY(cudaStreamSynchronize(r->st));
    return MTGPU_OK;
}

int mtgpu_mt_response(mtgpu_receivers *r, int nf, const double *nu, const int *sys_x,
                      const int *sys_y, int S, const double *d_e, const double *d_h,
                      double *d_out)
{
    MTGPU_CHECK_ARG(r && nu && sys_x && sys_y && d_e && d_h && d_out, "null argument");
    MTGPU_CHECK_ARG(nf > 0 && nf <= 65535, "nf must be in [1, 65535]");
    for (int f = 0; f < nf; f++)
        MTGPU_CHECK_ARG(sys_x[f] >= 0 && sys_x[f] < S && sys_y[f] >= 0 && sys_y[f] < S,
                        "system index out of range");
    int rc;
    if ((rc = ensure(&r->d_omega, &r->cap_omega, (size_t)nf)) ||
        (rc = ensure(&r->d_int, &r->cap_int, (size_t)2 * nf)))
        return rc;
    std::vector<double> om(nf);
    for (int f = 0; f < nf; f++) om[f] = 2.0 * kPi * nu[f];   // calcimpedance.for:50
    MTGPU_TRY(cudaMemcpyAsync(r->d_omega, om.data(), sizeof(double) * nf,
                              cudaMemcpyHostToDevice, r->st));
    MTGPU_TRY(cudaMemcpyAsync(r->d_int, sys_x, sizeof(int) * nf, cudaMemcpyHostToDevice, r->st));
    MTGPU_TRY(cudaMemcpyAsync(r->d_int + nf, sys_y, sizeof(int) * nf, cudaMemcpyHostToDevice,
                              r->st));
    dim3 grid(ceil_div(r->nrec, 128), nf);
    k_mt_response<<<grid, 128, 0, r->st>>>(r->nrec, nf, r->d_omega, r->d_int, r->d_int + nf,
                                           (const double2 *)d_e, (const double2 *)d_h, d_out);
    note_launches(1);
    MTGPU_TRY(cudaGetLastError());
    MTGPU_TRY(cudaStreamSynchronize(r->st));
    return MTGPU_OK;
}

}  // extern "C"
