// Adjoint gradient of the impedance misfit
//
//     J(sigma) = sum_{f, r} sum_{i, j in {x, y}} |Z_ij(f, r) - Zobs_ij(f, r)|^2
//
// with respect to the log-conductivity of every cell.  The reference has no
// gradient; this is new capability on top of the solve stage.
//
// Forward: for every system k (frequency omega_k, polarisation) the
// anomalous potential u_k solves A_k u_k = b_k with A_k = K + i omega_k M(sigma)
// and b_k = i omega_k (M(sigma0) - M(sigma)) a0_k (a0_k: the 1-D potential as
// edge values), Dirichlet rows being identity rows.  So
//     dR_k/dsigma_c = i omega_k P C_c (u_k + a0_k)
// (C_c the mass matrix of cell c, P the non-Dirichlet rows).  The receiver
// fields are linear in u_k; with g_k = dJ/du_k (dJ = 2 Re sum_k g_k^T du_k)
// the adjoint solve A_k lambda_k = g_k (A_k is complex symmetric, so the
// forward solver serves) gives
//     dJ/dln sigma_c = sigma_c sum_k -2 Re(lambda_k^T i omega_k P C_c (u_k + a0_k)).
//
// Kernels: k_adj_source (per receiver and frequency: Z, the misfit, and the
// derivatives of J with respect to E and H mapped onto the 12 edges of the
// receiver's brick), k_adj_gather (per touched edge, in a fixed order: no
// atomics, reproducible), k_adj_grad (per cell, fused over all systems).
#include "fem.cuh"
#include "receivers.cuh"

#include <algorithm>
#include <cmath>

namespace mtgpu {
namespace {

constexpr double kPi = 3.1415926535897932384626433832795;
constexpr double kMu0 = 1.25663706143591729e-6;

__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double lin0(double t) { return 0.5 * (1.0 - t); }
__device__ __forceinline__ double lin1(double t) { return 0.5 * (1.0 + t); }

// Weights of A_x, A_y (wa) and curl_x, curl_y (wc) at local point (xi, eta,
// zeta) of a brick as linear forms in its 12 edge values (the same basis and
// curl as the field evaluation: lowest-order edge functions (2/h_d) l_a l_b,
// l0' = -1/2, l1' = 1/2).
__device__ __forceinline__ void field_weights(double xi, double et, double ze, double hx,
                                              double hy, double hz, double wa[2][12],
                                              double wc[2][12])
{
    for (int i = 0; i < 12; i++) wa[0][i] = wa[1][i] = wc[0][i] = wc[1][i] = 0.0;
    const double sx = 2.0 / hx, sy = 2.0 / hy;
    wa[0][0] = sx * lin0(et) * lin0(ze);
    wa[0][1] = sx * lin1(et) * lin0(ze);
    wa[0][2] = sx * lin0(et) * lin1(ze);
    wa[0][3] = sx * lin1(et) * lin1(ze);
    wa[1][4] = sy * lin0(ze) * lin0(xi);
    wa[1][5] = sy * lin1(ze) * lin0(xi);
    wa[1][6] = sy * lin0(ze) * lin1(xi);
    wa[1][7] = sy * lin1(ze) * lin1(xi);
    // curl_x = dAz/dy - dAy/dz
    const double rx = 2.0 / (hy * hz), a0 = rx * lin0(xi), a1 = rx * lin1(xi);
    wc[0][4] = a0;  wc[0][5] = -a0; wc[0][6] = a1;  wc[0][7] = -a1;
    wc[0][8] = -a0; wc[0][9] = -a1; wc[0][10] = a0; wc[0][11] = a1;
    // curl_y = dAx/dz - dAz/dx
    const double ry = 2.0 / (hx * hz), b0 = ry * lin0(et), b1 = ry * lin1(et);
    wc[1][0] = -b0; wc[1][1] = -b1; wc[1][2] = b0;  wc[1][3] = b1;
    wc[1][8] = b0;  wc[1][9] = -b0; wc[1][10] = b1; wc[1][11] = -b1;
}

// One thread per (receiver, frequency f) with systems sx = sys_x[f] and
// sy = sys_y[f].  With the 2x2 field matrices (columns = polarisation)
// EE = [E_x; E_y], HH = [H_x; H_y]: Z = EE HH^-1, the misfit term
// |Z - Zobs|^2, and with W = conj(Z - Zobs):
//   dJ = 2 Re sum (G_E . dEE + G_H . dHH),  G_E = W HH^-T,  G_H = -Z^T G_E;
// E = -i omega A(u) + ..., H = curl(u) / mu0 + ... map G_E, G_H onto the
// 12 edges of the receiver's brick: contrib[sys][r][12].
__global__ void k_adj_source(int nrec, int nf, const double *__restrict__ omega,
                             const int *__restrict__ sys_x, const int *__restrict__ sys_y,
                             const double2 *__restrict__ E, const double2 *__restrict__ H,
                             const double2 *__restrict__ zobs, const int *__restrict__ elem,
                             const double4 *__restrict__ loc, const double4 *__restrict__ hsz,
                             double2 *contrib, double *misfit)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (r >= nrec || f >= nf) return;
    const int sys[2] = {sys_x[f], sys_y[f]};
    double2 EE[2][2], HH[2][2];   // [component x/y][polarisation]
    for (int p = 0; p < 2; p++)
        for (int d = 0; d < 2; d++) {
            EE[d][p] = E[((long long)sys[p] * nrec + r) * 3 + d];
            HH[d][p] = H[((long long)sys[p] * nrec + r) * 3 + d];
        }
    const double2 det = csub(cmul(HH[0][0], HH[1][1]), cmul(HH[0][1], HH[1][0]));
    double2 Hi[2][2];
    Hi[0][0] = cdiv(HH[1][1], det);
    Hi[0][1] = cdiv(make_double2(-HH[0][1].x, -HH[0][1].y), det);
    Hi[1][0] = cdiv(make_double2(-HH[1][0].x, -HH[1][0].y), det);
    Hi[1][1] = cdiv(HH[0][0], det);
    double2 Z[2][2], W[2][2];
    double J = 0.0;
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            Z[i][j] = cadd(cmul(EE[i][0], Hi[0][j]), cmul(EE[i][1], Hi[1][j]));
            const double2 o = zobs[((long long)f * nrec + r) * 4 + 2 * i + j];
            const double2 d = csub(Z[i][j], o);
            J += d.x * d.x + d.y * d.y;
            W[i][j] = cconj(d);
        }
    misfit[(long long)f * nrec + r] = J;
    // G_E[i][p] = sum_j W[i][j] Hi[p][j];  G_H[q][p] = -sum_i Z[i][q] G_E[i][p]
    double2 GE[2][2], GH[2][2];
    for (int i = 0; i < 2; i++)
        for (int p = 0; p < 2; p++) GE[i][p] = cadd(cmul(W[i][0], Hi[p][0]), cmul(W[i][1], Hi[p][1]));
    for (int q = 0; q < 2; q++)
        for (int p = 0; p < 2; p++) {
            const double2 t = cadd(cmul(Z[0][q], GE[0][p]), cmul(Z[1][q], GE[1][p]));
            GH[q][p] = make_double2(-t.x, -t.y);
        }
    const double w = omega[f];
    double wa[2][12], wc[2][12];
    const bool located = elem[r] >= 0;
    if (located) {
        const double4 L = loc[r], Hs = hsz[r];
        field_weights(L.x, L.y, L.z, Hs.x, Hs.y, Hs.z, wa, wc);
    }
    for (int p = 0; p < 2; p++) {
        // dE_d = -i w wa_d . du, dH_d = wc_d . du / mu0
        const double2 ge0 = cmul(GE[0][p], make_double2(0.0, -w));
        const double2 ge1 = cmul(GE[1][p], make_double2(0.0, -w));
        const double2 gh0 = cscale(GH[0][p], 1.0 / kMu0), gh1 = cscale(GH[1][p], 1.0 / kMu0);
        double2 *c = contrib + ((long long)sys[p] * nrec + r) * 12;
        for (int i = 0; i < 12; i++) {
            double2 v = make_double2(0.0, 0.0);
            if (located)
                v = cadd(cadd(cscale(ge0, wa[0][i]), cscale(ge1, wa[1][i])),
                         cadd(cscale(gh0, wc[0][i]), cscale(gh1, wc[1][i])));
            c[i] = v;
        }
    }
}

// src[k][edge] = sum of the contributions of system k landing on edge, in
// ascending (receiver, local edge) order; one thread per (touched edge, system)
__global__ void k_adj_gather(int n_touch, int S, int nrec, long long nb,
                             const int *__restrict__ ptr, const int *__restrict__ edge,
                             const int *__restrict__ slot, const double2 *__restrict__ contrib,
                             double2 *src)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (t >= n_touch || k >= S) return;
    double2 s = make_double2(0.0, 0.0);
    const double2 *c = contrib + (long long)k * nrec * 12;
    for (int q = ptr[t]; q < ptr[t + 1]; q++) s = cadd(s, c[slot[q]]);
    src[(long long)k * nb + edge[t]] = s;
}

// One thread per cell: for every system k,
//   t_k = sum_{i not Dirichlet} lambda_k[e_i] sum_{j} C_ij (u_k + a0_k)[e_j]
// (C the cell's mass matrix, nonzero on same-direction pairs only) and
//   grad[c] = sigma_c sum_k 2 omega_k Im t_k   ( = -2 Re(i omega_k t_k) ).
// a0_k on an edge: (h_d / 2) times the 1-D potential at the edge midpoint
// times (alfa, 1 - alfa, 0), as in the right-hand side assembly.
__global__ void k_adj_grad(int kpar, int S, long long nb, const double2 *__restrict__ u,
                           const double2 *__restrict__ lam, const double *__restrict__ omega,
                           const int *__restrict__ alfa, int n1d, const double *__restrict__ z1d,
                           const double *__restrict__ usin, const double *__restrict__ ucos,
                           const int *__restrict__ nver, int nver_stride,
                           const int *__restrict__ ed, int ed_stride,
                           const int *__restrict__ edges, const double *__restrict__ xyz,
                           const int *__restrict__ nvkat, const double *__restrict__ sig,
                           const unsigned char *__restrict__ bedge, double *grad)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kpar) return;
    double h[3];
    cell_h(xyz, nver, nver_stride, c, h);
    int e[12];
    double zm[12];
    bool inner[12];
    for (int l = 0; l < 12; l++) {
        e[l] = ed[(long long)c * ed_stride + l];
        zm[l] = 0.5 * (xyz[3 * edges[2 * e[l]] + 2] + xyz[3 * edges[2 * e[l] + 1] + 2]);
        inner[l] = bedge[e[l]] == 0;
    }
    // mass entries of the three 4x4 same-direction blocks
    double C[3][4][4];
    for (int d = 0; d < 3; d++)
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                double b, cc;
                brick_entry(4 * d + i, 4 * d + j, h, b, cc);
                C[d][i][j] = cc;
            }
    double acc = 0.0;
    for (int k = 0; k < S; k++) {
        const double2 *uk = u + (long long)k * nb, *lk = lam + (long long)k * nb;
        const double *us = usin + (long long)k * n1d, *uc = ucos + (long long)k * n1d;
        const double wx = alfa[k] ? 1.0 : 0.0;
        double2 ut[12];
        for (int l = 0; l < 12; l++) {
            ut[l] = uk[e[l]];
            const int d = l >> 2;
            if (d < 2) {
                const double wd = 0.5 * h[d] * (d == 0 ? wx : 1.0 - wx);
                ut[l].x += wd * spline(zm[l], n1d, z1d, us);
                ut[l].y += wd * spline(zm[l], n1d, z1d, uc);
            }
        }
        double2 t = make_double2(0.0, 0.0);
        for (int d = 0; d < 3; d++)
            for (int i = 0; i < 4; i++) {
                if (!inner[4 * d + i]) continue;
                double2 ci = make_double2(0.0, 0.0);
                for (int j = 0; j < 4; j++) ci = cadd(ci, cscale(ut[4 * d + j], C[d][i][j]));
                t = cadd(t, cmul(lk[e[4 * d + i]], ci));
            }
        acc += 2.0 * omega[k] * t.y;
    }
    grad[c] = acc * sig[nvkat[c]];
}

}  // namespace
}  // namespace mtgpu

using namespace mtgpu;

namespace {

// edges touched by the receivers' bricks, each with its (receiver, slot)
// list in ascending order
int build_touch(mtgpu_receivers *r)
{
    if (r->d_touch_ptr) return MTGPU_OK;
    std::vector<int> edge(12 * (size_t)r->nrec);
    MTGPU_TRY(cudaMemcpyAsync(edge.data(), r->d_edge, sizeof(int) * edge.size(),
                              cudaMemcpyDeviceToHost, r->st));
    MTGPU_TRY(cudaStreamSynchronize(r->st));
    std::vector<std::pair<int, int>> es;   // (edge, receiver * 12 + slot)
    for (int q = 0; q < r->nrec; q++)
        if (r->elem[q] >= 0)
            for (int i = 0; i < 12; i++) es.push_back({edge[12 * q + i], 12 * q + i});
    std::sort(es.begin(), es.end());
    std::vector<int> ptr{0}, ue, slot;
    for (size_t i = 0; i < es.size(); i++) {
        if (i == 0 || es[i].first != es[i - 1].first) {
            if (i) ptr.push_back((int)i);
            ue.push_back(es[i].first);
        }
        slot.push_back(es[i].second);
    }
    if (!es.empty()) ptr.push_back((int)es.size());
    r->n_touch = (int)ue.size();
    int rc;
    if ((rc = dev_alloc(&r->d_touch_ptr, ptr.size())) ||
        (rc = dev_alloc(&r->d_touch_edge, std::max<size_t>(ue.size(), 1))) ||
        (rc = dev_alloc(&r->d_touch_slot, std::max<size_t>(slot.size(), 1))))
        return rc;
    MTGPU_TRY(cudaMemcpyAsync(r->d_touch_ptr, ptr.data(), sizeof(int) * ptr.size(),
                              cudaMemcpyHostToDevice, r->st));
    if (!ue.empty()) {
        MTGPU_TRY(cudaMemcpyAsync(r->d_touch_edge, ue.data(), sizeof(int) * ue.size(),
                                  cudaMemcpyHostToDevice, r->st));
        MTGPU_TRY(cudaMemcpyAsync(r->d_touch_slot, slot.data(), sizeof(int) * slot.size(),
                                  cudaMemcpyHostToDevice, r->st));
    }
    MTGPU_TRY(cudaStreamSynchronize(r->st));
    return MTGPU_OK;
}

}  // namespace

extern "C" {

int mtgpu_adjoint_source(mtgpu_receivers *r, int nf, const double *nu, const int *sys_x,
                         const int *sys_y, int S, const double *d_e, const double *d_h,
                         const double *d_zobs, double *d_src, double *misfit)
{
    MTGPU_CHECK_ARG(r && nu && sys_x && sys_y && d_e && d_h && d_zobs && d_src,
                    "null argument");
    MTGPU_CHECK_ARG(r->output == MTGPU_OUTPUT_DIRECT,
                    "the adjoint source differentiates the direct receiver output only");
    MTGPU_CHECK_ARG(nf > 0 && nf <= 65535 && S > 0 && S <= 65535, "bad nf or S");
    std::vector<int> used(S, 0);
    for (int f = 0; f < nf; f++) {
        MTGPU_CHECK_ARG(sys_x[f] >= 0 && sys_x[f] < S && sys_y[f] >= 0 && sys_y[f] < S,
                        "system index out of range");
        MTGPU_CHECK_ARG(sys_x[f] != sys_y[f], "the two polarisations must be different systems");
        MTGPU_CHECK_ARG(!used[sys_x[f]] && !used[sys_y[f]],
                        "a system may belong to one frequency only");
        used[sys_x[f]] = used[sys_y[f]] = 1;
    }
    int rc = build_touch(r);
    if (rc) return rc;
    if ((rc = ensure(&r->d_omega, &r->cap_omega, (size_t)nf)) ||
        (rc = ensure(&r->d_int, &r->cap_int, (size_t)2 * nf)) ||
        (rc = ensure(&r->d_contrib, &r->cap_contrib, (size_t)S * r->nrec * 12)) ||
        (rc = ensure(&r->d_misfit, &r->cap_misfit, (size_t)nf * r->nrec)))
        return rc;
    std::vector<double> om(nf);
    for (int f = 0; f < nf; f++) om[f] = 2.0 * kPi * nu[f];
    MTGPU_TRY(cudaMemcpyAsync(r->d_omega, om.data(), sizeof(double) * nf,
                              cudaMemcpyHostToDevice, r->st));
    MTGPU_TRY(cudaMemcpyAsync(r->d_int, sys_x, sizeof(int) * nf, cudaMemcpyHostToDevice, r->st));
    MTGPU_TRY(cudaMemcpyAsync(r->d_int + nf, sys_y, sizeof(int) * nf, cudaMemcpyHostToDevice,
                              r->st));
    MTGPU_TRY(cudaMemsetAsync(r->d_contrib, 0, sizeof(double2) * S * r->nrec * 12, r->st));
    MTGPU_TRY(cudaMemsetAsync(d_src, 0, sizeof(double2) * S * (size_t)r->nb, r->st));
    dim3 g1(ceil_div(r->nrec, 128), nf);
    k_adj_source<<<g1, 128, 0, r->st>>>(r->nrec, nf, r->d_omega, r->d_int, r->d_int + nf,
                                        (const double2 *)d_e, (const double2 *)d_h,
                                        (const double2 *)d_zobs, r->d_elem, r->d_loc, r->d_h,
                                        r->d_contrib, r->d_misfit);
    int launches = 1;
    if (r->n_touch) {
        dim3 g2(ceil_div(r->n_touch, 128), S);
        k_adj_gather<<<g2, 128, 0, r->st>>>(r->n_touch, S, r->nrec, r->nb, r->d_touch_ptr,
                                            r->d_touch_edge, r->d_touch_slot, r->d_contrib,
                                            (double2 *)d_src);
        launches++;
    }
    note_launches(launches);
    MTGPU_TRY(cudaGetLastError());
    if (misfit) {
        std::vector<double> m((size_t)nf * r->nrec);
        MTGPU_TRY(cudaMemcpyAsync(m.data(), r->d_misfit, sizeof(double) * m.size(),
                                  cudaMemcpyDeviceToHost, r->st));
        MTGPU_TRY(cudaStreamSynchronize(r->st));
        double s = 0.0;
        for (double v : m) s += v;
        *misfit = s;
    }
    MTGPU_TRY(cudaStreamSynchronize(r->st));
    return MTGPU_OK;
}

int mtgpu_adjoint_gradient(mtgpu_assembly *a, int S, const double *nu, const int *alfa, int n1d,
                           const double *z1d, const double *usin, const double *ucos,
                           const double *d_u, const double *d_lambda, double *d_grad)
{
    MTGPU_CHECK_ARG(a && nu && alfa && z1d && usin && ucos && d_u && d_lambda && d_grad,
                    "null argument");
    MTGPU_CHECK_ARG(S > 0, "S must be positive");
    MTGPU_CHECK_ARG(n1d >= 2, "the 1-D table needs at least 2 points");
    const ParamMatrix &P = a->P;
    std::vector<double> om(S);
    for (int k = 0; k < S; k++) om[k] = 2.0 * kPi * nu[k];
    double *d_om = nullptr, *d_tab = nullptr;
    int *d_alfa = nullptr;
    int rc;
    if ((rc = dev_alloc(&d_om, S)) || (rc = dev_alloc(&d_alfa, S)) ||
        (rc = dev_alloc(&d_tab, (size_t)n1d * (2 * S + 1)))) {
        dev_free(d_om);
        dev_free(d_alfa);
        return rc;
    }
    double *d_z = d_tab, *d_us = d_tab + n1d, *d_uc = d_us + (size_t)S * n1d;
    cudaError_t e = cudaMemcpyAsync(d_om, om.data(), sizeof(double) * S, cudaMemcpyHostToDevice,
                                    a->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_alfa, alfa, sizeof(int) * S, cudaMemcpyHostToDevice, a->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_z, z1d, sizeof(double) * n1d, cudaMemcpyHostToDevice, a->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_us, usin, sizeof(double) * S * n1d, cudaMemcpyHostToDevice, a->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_uc, ucos, sizeof(double) * S * n1d, cudaMemcpyHostToDevice, a->st);
    if (e == cudaSuccess) {
        k_adj_grad<<<ceil_div(P.kpar, 128), 128, 0, a->st>>>(
            P.kpar, S, P.nb, (const double2 *)d_u, (const double2 *)d_lambda, d_om, d_alfa, n1d,
            d_z, d_us, d_uc, P.d_nver, P.nver_stride, P.d_ed, P.ed_stride, P.d_edges, P.d_xyz,
            P.d_nvkat, P.d_sig, P.d_bedge, d_grad);
        note_launches(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->st);
    dev_free(d_om);
    dev_free(d_alfa);
    dev_free(d_tab);
    if (e != cudaSuccess) {
        set_last_error(e, "mtgpu_adjoint_gradient", __FILE__, __LINE__);
        return MTGPU_ERR_CUDA;
    }
    return MTGPU_OK;
}

}  // extern "C"
