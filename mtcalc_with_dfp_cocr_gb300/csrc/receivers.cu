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
#include "rcv_eval.cuh"
#include "receivers.cuh"

#include <climits>
#include <cmath>

namespace mtgpu {
namespace {

using rcv::kPi;
constexpr int kLocChunk = 256;                               // receivers per shared-memory pass

__global__ void k_rcv_init(int nrec, int *elem)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nrec) elem[r] = INT_MAX;
}

// elem[r] = the lowest brick index whose closed box [vertex 0, vertex 7],
// grown by `grow` on every side, holds receiver r.  The direct output keeps
// the first brick found in index order with no growth
// (OutputArbitrary.cpp:385-500); the smoothing output grows the boxes by
// 1e-6 and, for A, skips the bricks of material 0, the air
// (OutputResultant3d.cpp:293-450): nvkat != NULL selects that.  One thread
// per brick; receivers pass through shared memory in chunks.
__global__ void __launch_bounds__(kThreads)
k_rcv_locate(int kpar, const int *__restrict__ nver, int nver_stride,
             const double *__restrict__ xyz, int nrec, const double *__restrict__ rec, double grow,
             const int *__restrict__ nvkat, int *elem)
{
    __shared__ double sx[kLocChunk], sy[kLocChunk], sz[kLocChunk];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double lo[3] = {0, 0, 0}, hi[3] = {-1, -1, -1};   // empty box for idle threads
    if (e < kpar && !(nvkat && nvkat[e] == 0)) {
        const int v0 = nver[(long long)e * nver_stride], v7 = nver[(long long)e * nver_stride + 7];
        for (int d = 0; d < 3; d++) {
            lo[d] = xyz[3 * v0 + d] - grow;
            hi[d] = xyz[3 * v7 + d] + grow;
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

// One thread per (receiver, system): A and curl A at the receiver from the
// 12 edge values of its brick, then the total fields.
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
    double2 A[3] = {}, C[3] = {};
    if (elem[r] >= 0) {
        const double4 L = loc[r], Hs = hsz[r];
        const double2 *xs = x + (long long)k * x_stride;
        double2 v[12];
#pragma unroll
        for (int i = 0; i < 12; i++) v[i] = xs[edge[12 * r + i]];
        rcv::brick_eval(v, L.x, L.y, L.z, Hs.x, Hs.y, Hs.z, A, C);
    }
    const long long o = (long long)k * nrec + r;
    rcv::total_fields(A, C, omega[k], alfa[k], loc[r].w, n1d, z1d, usin + (long long)k * n1d,
                      ucos + (long long)k * n1d, e_out + 3 * o, h_out + 3 * o, scal + o);
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

int locate_receivers(const ParamMatrix &P, int nrec, const double *d_rec, double grow,
                     bool skip_air, int *d_elem, cudaStream_t st)
{
    k_rcv_init<<<ceil_div(nrec, kThreads), kThreads, 0, st>>>(nrec, d_elem);
    k_rcv_locate<<<ceil_div(P.kpar, kThreads), kThreads, 0, st>>>(
        P.kpar, P.d_nver, P.nver_stride, P.d_xyz, nrec, d_rec, grow,
        skip_air ? P.d_nvkat : nullptr, d_elem);
    note_launches(2);
    MTGPU_TRY(cudaGetLastError());
    return MTGPU_OK;
}

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
    if (r->sm) {
        r->sm->release();
        delete r->sm;
    }
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
    r->rec.assign(xyz_rec, xyz_rec + (size_t)3 * nrec);
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
            P.kpar, P.d_nver, P.nver_stride, P.d_xyz, nrec, d_rec, 0.0, nullptr, r->d_elem);
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

int mtgpu_receivers_set_output(mtgpu_receivers *r, const mtgpu_assembly *a, int mode, int levels)
{
    MTGPU_CHECK_ARG(r != nullptr, "null receivers");
    MTGPU_CHECK_ARG(mode == MTGPU_OUTPUT_DIRECT || mode == MTGPU_OUTPUT_SMOOTH, "unknown mode");
    if (mode == MTGPU_OUTPUT_DIRECT) {
        r->output = mode;
        return MTGPU_OK;
    }
    MTGPU_CHECK_ARG(a != nullptr, "the smoothing output needs the assembly");
    MTGPU_CHECK_ARG(a->P.nb == r->nb, "the assembly is not the receivers' mesh");
    MTGPU_CHECK_ARG(levels >= 0 && levels <= 64, "levels must be in [0, 64]");
    MTGPU_CHECK_ARG(a->nver_stride >= 8 && !a->xyz.empty(), "the assembly has no host mesh");
    if (r->sm) {
        r->sm->release();
        delete r->sm;
        r->sm = nullptr;
    }
    r->output = MTGPU_OUTPUT_DIRECT;
    auto *sm = new Smoothing();
    sm->levels = levels;
    int rc = smoothing_build(*sm, *a, r->nrec, r->rec.data(), r->st);
    if (rc) {
        sm->release();
        delete sm;
        return rc;
    }
    r->sm = sm;
    r->asm_ = a;
    r->output = mode;
    return MTGPU_OK;
}

int mtgpu_receivers_smoothing_info(const mtgpu_receivers *r, int max_sub, int *nsub, int *material,
                                   int *cells, int *nodes, int *iterations)
{
    MTGPU_CHECK_ARG(r != nullptr, "null receivers");
    MTGPU_CHECK_ARG(r->output == MTGPU_OUTPUT_SMOOTH && r->sm, "the output is not smoothed");
    const Smoothing &sm = *r->sm;
    if (nsub) *nsub = sm.nsub;
    for (int s = 0; s < sm.nsub && s < max_sub; s++) {
        if (material) material[s] = sm.sub_material[s];
        if (cells) cells[s] = sm.sub_cells[s];
        if (nodes) nodes[s] = sm.sub_nodes[s];
    }
    if (iterations) *iterations = sm.iterations;
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
    if (r->output == MTGPU_OUTPUT_SMOOTH) {
        int rc2 = smoothing_fields(*r->sm, r->asm_->P, r->nrec, S, r->nb, (const double2 *)d_x,
                                   r->d_omega, r->d_int, n1d, d_z1d, d_us, d_uc, r->d_loc,
                                   (double2 *)d_e, (double2 *)d_h, (double2 *)d_rho_imp, r->st);
        if (rc2) return rc2;
    } else {
        dim3 grid(ceil_div(r->nrec, 128), S);
        k_rcv_fields<<<grid, 128, 0, r->st>>>(r->nrec, S, r->nb, (const double2 *)d_x,
                                              r->d_omega, r->d_int, n1d, d_z1d, d_us, d_uc,
                                              r->d_elem, r->d_edge, r->d_loc, r->d_h,
                                              (double2 *)d_e, (double2 *)d_h,
                                              (double2 *)d_rho_imp);
        note_launches(1);
        MTGPU_TRY(cudaGetLastError());
    }
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
