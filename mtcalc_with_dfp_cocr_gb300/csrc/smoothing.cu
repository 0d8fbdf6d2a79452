// Receiver output by subdomain L2-projection smoothing: the reference's
// default E/H output path (Code/OutputNu: Give_out_vec_mt::Give_out_on_hex
// with OutputResultant3d, give_out_vec_mt.cpp:200-237, OutputResultant3d.cpp:
// 76-199, 293-450; Subdomain::Init / AsmGlobalMatrix / AsmGlobalVector,
// Subdomain.cpp:132-661).  Per receiver output type:
//
//   * the receivers are located in the first brick (index order) whose box
//     grown by 1e-6 holds them; for A the air (material 0) is skipped;
//   * curl A is smoothed over one subdomain of all materials, A over one
//     subdomain per material holding a receiver; a subdomain is its
//     receivers' bricks grown `levels` times by every brick of its material
//     sharing a node with it;
//   * in each subdomain the brick-centre values (A or curl A of the edge
//     solution) are projected onto the nodal trilinear functions:
//     M u = f with M the nodal mass matrix and f_i = sum over the bricks at
//     node i of (the brick matrix's row sum) x (the centre value);
//   * the receiver value is the trilinear interpolant of u in its brick.
//
// The reference factorises M with PARDISO and solves one value type at a
// time.  Here every (subdomain, value type, system) is one column of a
// batched Jacobi-preconditioned conjugate-gradient solve in FP64 to a
// relative residual of 1e-14 (the diagonally scaled trilinear mass matrix
// has a condition number below ~30, so 40-60 iterations), on all value
// types of all systems at once.  The subdomains, the mass matrix and the
// interpolation weights are built once per receiver set on the host; the
// per-call work (centre values, right-hand sides, CG, interpolation) runs on
// the device.
//
// Vector layout: [column][padded node], column = value * S + system with
// values (x re, x im, y re, y im, z re, z im); every subdomain's node range
// is padded to a multiple of the 256-thread block so that a block's rows
// belong to one subdomain and its dot-product partials to one (subdomain,
// column) problem.  Conforming (tensor) meshes only: no terminal nodes.
#include "rcv_eval.cuh"
#include "receivers.cuh"

#include <algorithm>
#include <climits>
#include <cmath>

namespace mtgpu {
namespace {

constexpr int kBlk = 256;            // nodes per block (padding unit)
constexpr double kTol2 = 1e-28;      // (relative residual 1e-14)^2
constexpr int kMaxIter = 2000;       // guard; the CG needs well under 100
constexpr int kCheckEvery = 8;

// brick-centre values: one thread per (brick of a subdomain, system)
__global__ void k_sm_centre(int ncell, int S, const int *__restrict__ cell,
                            const int *__restrict__ cell_sub, const int *__restrict__ nver,
                            int nver_stride, const int *__restrict__ ed, int ed_stride,
                            const double *__restrict__ xyz, long long x_stride,
                            const double2 *__restrict__ x, double *val)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (i >= ncell || k >= S) return;
    const long long g = cell[i];
    const int v0 = nver[g * nver_stride], v7 = nver[g * nver_stride + 7];
    const double hx = xyz[3 * v7] - xyz[3 * v0], hy = xyz[3 * v7 + 1] - xyz[3 * v0 + 1],
                 hz = xyz[3 * v7 + 2] - xyz[3 * v0 + 2];
    const double2 *xs = x + (long long)k * x_stride;
    double2 v[12];
#pragma unroll
    for (int j = 0; j < 12; j++) v[j] = xs[ed[g * ed_stride + j]];
    double2 A[3], C[3];
    rcv::brick_eval(v, 0.0, 0.0, 0.0, hx, hy, hz, A, C);
    const double2 *f = cell_sub[i] == 0 ? C : A;
    for (int d = 0; d < 3; d++) {
        val[((long long)(2 * d) * S + k) * ncell + i] = f[d].x;
        val[((long long)(2 * d + 1) * S + k) * ncell + i] = f[d].y;
    }
}

template <int N>
__device__ __forceinline__ void block_sum(double (&v)[N], double *out_addr[N])
{
    __shared__ double part[N][kBlk / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int n = 0; n < N; n++) {
        double s = v[n];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) part[n][w] = s;
    }
    __syncthreads();
    if (threadIdx.x < N) {
        double s = 0.0;
        for (int j = 0; j < kBlk / 32; j++) s += part[threadIdx.x][j];
        atomicAdd(out_addr[threadIdx.x], s);
    }
}

// problem scalars, [quantity][problem]
enum { kRz = 0, kPq, kRz2, kRr, kFf, kBeta, kNq };

// f = sum over the node's bricks of g_c val_c; x = 0, r = f, z = f / diag,
// p = z; (r, z) and (f, f) per problem
__global__ void __launch_bounds__(kBlk)
k_sm_init(int npad, int ncell, int nsub, const int *__restrict__ blk_sub,
          const int *__restrict__ nc_ptr, const int *__restrict__ nc,
          const double *__restrict__ cell_g, const double *__restrict__ val,
          const double *__restrict__ diag, double *x, double *r, double *z, double *p,
          double *scal, int nprob)
{
    const int n = blockIdx.x * kBlk + threadIdx.x;
    const int col = blockIdx.y;
    const long long o = (long long)col * npad + n;
    double f = 0.0;
    for (int j = nc_ptr[n]; j < nc_ptr[n + 1]; j++) {
        const int c = nc[j];
        f += cell_g[c] * val[(long long)col * ncell + c];
    }
    const double zz = f / diag[n];
    x[o] = 0.0;
    r[o] = f;
    z[o] = zz;
    p[o] = zz;
    const int pr = col * nsub + blk_sub[blockIdx.x];
    double v[2] = {f * zz, f * f};
    double *dst[2] = {scal + kRz * nprob + pr, scal + kFf * nprob + pr};
    block_sum<2>(v, dst);
}

// a problem whose right-hand side is zero is done at the start
__global__ void k_sm_start(int nprob, const double *scal, int *done)
{
    const int pr = blockIdx.x * blockDim.x + threadIdx.x;
    if (pr < nprob) done[pr] = !(scal[kFf * nprob + pr] > 0.0);
}

// q = M p, (p, q)
__global__ void __launch_bounds__(kBlk)
k_sm_spmv(int npad, int nsub, const int *__restrict__ blk_sub, const int *__restrict__ mptr,
          const int *__restrict__ mcol, const double *__restrict__ mval,
          const double *__restrict__ p, double *q, double *scal, const int *__restrict__ done,
          int nprob)
{
    const int col = blockIdx.y;
    const int pr = col * nsub + blk_sub[blockIdx.x];
    if (done[pr]) return;   // uniform over the block
    const int n = blockIdx.x * kBlk + threadIdx.x;
    const double *pc = p + (long long)col * npad;
    double s = 0.0;
    for (int j = mptr[n]; j < mptr[n + 1]; j++) s += mval[j] * pc[mcol[j]];
    q[(long long)col * npad + n] = s;
    double v[1] = {pc[n] * s};
    double *dst[1] = {scal + kPq * nprob + pr};
    block_sum<1>(v, dst);
}

// x += alpha p, r -= alpha q, z = r / diag; (r, z), (r, r)
__global__ void __launch_bounds__(kBlk)
k_sm_update(int npad, int nsub, const int *__restrict__ blk_sub, const double *__restrict__ diag,
            double *x, double *r, double *z, const double *__restrict__ p,
            const double *__restrict__ q, double *scal, const int *__restrict__ done, int nprob)
{
    const int col = blockIdx.y;
    const int pr = col * nsub + blk_sub[blockIdx.x];
    if (done[pr]) return;
    const int n = blockIdx.x * kBlk + threadIdx.x;
    const long long o = (long long)col * npad + n;
    const double pq = scal[kPq * nprob + pr];
    const double al = pq > 0.0 ? scal[kRz * nprob + pr] / pq : 0.0;
    x[o] += al * p[o];
    const double rr = r[o] - al * q[o];
    const double zz = rr / diag[n];
    r[o] = rr;
    z[o] = zz;
    double v[2] = {rr * zz, rr * rr};
    double *dst[2] = {scal + kRz2 * nprob + pr, scal + kRr * nprob + pr};
    block_sum<2>(v, dst);
}

// per problem: beta, the stop test, reset of the partial sums; counts the
// problems still running
__global__ void k_sm_scalars(int nprob, double *scal, int *done, int *active)
{
    const int pr = blockIdx.x * blockDim.x + threadIdx.x;
    if (pr >= nprob || done[pr]) return;
    const double rz = scal[kRz * nprob + pr], rz2 = scal[kRz2 * nprob + pr];
    const bool stop = scal[kRr * nprob + pr] <= kTol2 * scal[kFf * nprob + pr] ||
                      !(scal[kPq * nprob + pr] > 0.0) || !(rz > 0.0);
    scal[kBeta * nprob + pr] = rz > 0.0 ? rz2 / rz : 0.0;
    scal[kRz * nprob + pr] = rz2;
    scal[kPq * nprob + pr] = 0.0;
    scal[kRz2 * nprob + pr] = 0.0;
    scal[kRr * nprob + pr] = 0.0;
    if (stop)
        done[pr] = 1;
    else
        atomicAdd(active, 1);
}

// p = z + beta p
__global__ void __launch_bounds__(kBlk)
k_sm_direction(int npad, int nsub, const int *__restrict__ blk_sub, const double *__restrict__ z,
               double *p, const double *__restrict__ scal, const int *__restrict__ done, int nprob)
{
    const int col = blockIdx.y;
    const int pr = col * nsub + blk_sub[blockIdx.x];
    if (done[pr]) return;
    const long long o = (long long)col * npad + blockIdx.x * kBlk + threadIdx.x;
    p[o] = z[o] + scal[kBeta * nprob + pr] * p[o];
}

// receiver values (trilinear interpolation of the nodal solutions) and the
// total fields: one thread per (receiver, system)
__global__ void k_sm_receivers(int nrec, int S, int npad, const int *__restrict__ rn,
                               const double *__restrict__ rw, const double *__restrict__ u,
                               const double *__restrict__ omega, const int *__restrict__ alfa,
                               int n1d, const double *__restrict__ z1d,
                               const double *__restrict__ usin, const double *__restrict__ ucos,
                               const double4 *__restrict__ loc, double2 *e_out, double2 *h_out,
                               double2 *scal)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (r >= nrec || k >= S) return;
    double2 F[2][3] = {};   // curl A, A
    for (int t = 0; t < 2; t++) {
        const int *nn = rn + (r * 2 + t) * 8;
        const double *ww = rw + (r * 2 + t) * 8;
        if (nn[0] < 0) continue;
        for (int v = 0; v < 6; v++) {
            const double *uc = u + ((long long)v * S + k) * npad;
            double s = 0.0;
            for (int l = 0; l < 8; l++) s += ww[l] * uc[nn[l]];
            if (v & 1)
                F[t][v >> 1].y = s;
            else
                F[t][v >> 1].x = s;
        }
    }
    const long long o = (long long)k * nrec + r;
    rcv::total_fields(F[1], F[0], omega[k], alfa[k], loc[r].w, n1d, z1d,
                      usin + (long long)k * n1d, ucos + (long long)k * n1d, e_out + 3 * o,
                      h_out + 3 * o, scal + o);
}

// ------------------------------------------------------------- host set-up
struct SubBuild {
    std::vector<int> cells, nodes;   // ascending global indices
};

// Subdomain.cpp:132-246: seed bricks, then `levels` rounds of every allowed
// brick sharing a node with the current node set
SubBuild grow_subdomain(const ::mtgpu_assembly_s &a, const std::vector<int> &seed, int material,
                        int levels)
{
    const int kpar = a.P.kpar, kuz = a.P.kuzlov, ns = a.nver_stride;
    std::vector<unsigned char> in_cell(kpar, 0), in_node(kuz, 0);
    auto allowed = [&](int c) { return material < 0 || a.nvkat[c] == material; };
    for (int c : seed) {
        if (c < 0 || !allowed(c) || in_cell[c]) continue;
        in_cell[c] = 1;
        for (int j = 0; j < 8; j++) in_node[a.nver[(size_t)c * ns + j]] = 1;
    }
    std::vector<int> fresh;
    for (int lv = 0; lv < levels; lv++) {
        fresh.clear();
        for (int c = 0; c < kpar; c++) {
            if (in_cell[c] || !allowed(c)) continue;
            for (int j = 0; j < 8; j++)
                if (in_node[a.nver[(size_t)c * ns + j]]) {
                    fresh.push_back(c);
                    break;
                }
        }
        for (int c : fresh) {
            in_cell[c] = 1;
            for (int j = 0; j < 8; j++) in_node[a.nver[(size_t)c * ns + j]] = 1;
        }
    }
    SubBuild s;
    for (int c = 0; c < kpar; c++)
        if (in_cell[c]) s.cells.push_back(c);
    for (int n = 0; n < kuz; n++)
        if (in_node[n]) s.nodes.push_back(n);
    return s;
}

// T_Brick::Phi_node at a point of a brick (T_Brick.cpp:866-887, 2010-2023)
void trilinear_weights(const double *lo, const double *hi, const double *p, double *w)
{
    double l0[3], l1[3];
    for (int d = 0; d < 3; d++) {
        const double t = (2.0 * p[d] - lo[d] - hi[d]) / (hi[d] - lo[d]);
        l0[d] = 0.5 * (1.0 - t);
        l1[d] = 0.5 * (1.0 + t);
    }
    for (int j = 0; j < 8; j++)
        w[j] = ((j & 1) ? l1[0] : l0[0]) * ((j & 2) ? l1[1] : l0[1]) * ((j & 4) ? l1[2] : l0[2]);
}

}  // namespace

void Smoothing::release()
{
    dev_free(d_cell);
    dev_free(d_cell_sub);
    dev_free(d_cell_g);
    dev_free(d_nc_ptr);
    dev_free(d_nc);
    dev_free(d_mptr);
    dev_free(d_mcol);
    dev_free(d_mval);
    dev_free(d_mdiag);
    dev_free(d_blk_sub);
    dev_free(d_rn);
    dev_free(d_rw);
    dev_free(d_val);
    dev_free(d_x);
    dev_free(d_r);
    dev_free(d_z);
    dev_free(d_p);
    dev_free(d_q);
    dev_free(d_scal);
    dev_free(d_done);
    dev_free(d_active);
    S_cap = 0;
}

template <class T>
static int upload(T **d, const std::vector<T> &h, cudaStream_t st)
{
    int rc = dev_alloc(d, h.size());
    if (rc) return rc;
    if (!h.empty())
        MTGPU_TRY(cudaMemcpyAsync(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, st));
    return MTGPU_OK;
}

int smoothing_build(Smoothing &sm, const ::mtgpu_assembly_s &a, int nrec, const double *xyz_rec,
                    cudaStream_t st)
{
    const ParamMatrix &P = a.P;
    const int ns = a.nver_stride;
    // receiver bricks: curl A (all materials) and A (air skipped), boxes + 1e-6
    std::vector<int> eb(nrec), ea(nrec);
    {
        int *d_e = nullptr;
        double *d_rec = nullptr;
        int rc;
        if ((rc = dev_alloc(&d_e, (size_t)2 * nrec)) || (rc = dev_alloc(&d_rec, (size_t)3 * nrec))) {
            dev_free(d_e);
            return rc;
        }
        cudaError_t e = cudaMemcpyAsync(d_rec, xyz_rec, sizeof(double) * 3 * nrec,
                                        cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
            rc = locate_receivers(P, nrec, d_rec, 1e-6, false, d_e, st);
            if (!rc) rc = locate_receivers(P, nrec, d_rec, 1e-6, true, d_e + nrec, st);
            if (!rc) {
                e = cudaMemcpyAsync(eb.data(), d_e, sizeof(int) * nrec, cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(ea.data(), d_e + nrec, sizeof(int) * nrec,
                                        cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            }
        }
        dev_free(d_e);
        dev_free(d_rec);
        if (rc) return rc;
        if (e != cudaSuccess) {
            set_last_error(e, "smoothing receiver location", __FILE__, __LINE__);
            return MTGPU_ERR_CUDA;
        }
        for (int r = 0; r < nrec; r++) {
            if (eb[r] == INT_MAX) eb[r] = -1;
            if (ea[r] == INT_MAX) ea[r] = -1;
        }
    }
    // subdomains: curl A over all materials, A per material with a receiver
    std::vector<int> mats;
    for (int r = 0; r < nrec; r++)
        if (ea[r] >= 0) mats.push_back(a.nvkat[ea[r]]);
    std::sort(mats.begin(), mats.end());
    mats.erase(std::unique(mats.begin(), mats.end()), mats.end());
    std::vector<SubBuild> subs;
    std::vector<int> sub_mat;
    subs.push_back(grow_subdomain(a, eb, -1, sm.levels));
    sub_mat.push_back(-1);
    for (int m : mats) {
        subs.push_back(grow_subdomain(a, ea, m, sm.levels));
        sub_mat.push_back(m);
    }
    sm.nsub = (int)subs.size();
    sm.sub_cells.clear();
    sm.sub_nodes.clear();
    sm.sub_material = sub_mat;
    // padded node numbering, bricks, mass matrix, node -> bricks
    std::vector<int> node_off(sm.nsub + 1, 0), cell_off(sm.nsub + 1, 0);
    for (int s = 0; s < sm.nsub; s++) {
        const int nn = (int)subs[s].nodes.size();
        node_off[s + 1] = node_off[s] + (nn + kBlk - 1) / kBlk * kBlk;
        cell_off[s + 1] = cell_off[s] + (int)subs[s].cells.size();
        sm.sub_cells.push_back((int)subs[s].cells.size());
        sm.sub_nodes.push_back(nn);
    }
    sm.npad = node_off[sm.nsub];
    sm.ncell = cell_off[sm.nsub];
    sm.nblk = sm.npad / kBlk;
    std::vector<int> cell(sm.ncell), cell_sub(sm.ncell), blk_sub(sm.nblk);
    std::vector<double> cell_g(sm.ncell), mdiag(sm.npad, 1.0);
    std::vector<int> mptr(sm.npad + 1, 0), mcol, nc_ptr(sm.npad + 1, 0), nc;
    std::vector<double> mval;
    std::vector<int> loc(P.kuzlov, -1);
    for (int s = 0; s < sm.nsub; s++) {
        const SubBuild &B = subs[s];
        const int n0 = node_off[s], nn = (int)B.nodes.size();
        for (int b = node_off[s] / kBlk; b < node_off[s + 1] / kBlk; b++) blk_sub[b] = s;
        for (int i = 0; i < nn; i++) loc[B.nodes[i]] = i;
        // rows of up to 27 (column, value) slots
        std::vector<int> rc(27 * (size_t)nn, -1), cnt(nn, 0);
        std::vector<double> rv(27 * (size_t)nn, 0.0);
        std::vector<std::vector<int>> adj(nn);
        for (size_t ci = 0; ci < B.cells.size(); ci++) {
            const int c = B.cells[ci], gi = cell_off[s] + (int)ci;
            cell[gi] = c;
            cell_sub[gi] = s;
            const int *nv = &a.nver[(size_t)c * ns];
            const double *x0 = &a.xyz[3 * (size_t)nv[0]], *x7 = &a.xyz[3 * (size_t)nv[7]];
            // Hex_Local_Matrix.cpp:120-198
            const double t2 = (x7[0] - x0[0]) * (x7[1] - x0[1]) * (x7[2] - x0[2]);
            const double t[4] = {t2 / 27.0, t2 / 54.0, t2 / 108.0, t2 / 216.0};
            double g = 0.0;   // row sum (Subdomain.cpp:504-505), corner 0
            for (int k = 0; k < 8; k++) g += t[__builtin_popcount(k)];
            cell_g[gi] = g;
            int li[8];
            for (int j = 0; j < 8; j++) li[j] = loc[nv[j]];
            for (int j = 0; j < 8; j++) {
                adj[li[j]].push_back(gi);
                for (int k = 0; k < 8; k++) {
                    const double bv = t[__builtin_popcount(j ^ k)];
                    const size_t base = 27 * (size_t)li[j];
                    int q = 0;
                    while (q < cnt[li[j]] && rc[base + q] != li[k]) q++;
                    if (q == cnt[li[j]]) {
                        if (q == 27) {
                            set_last_message("smoothing: a node with more than 27 neighbours "
                                             "(the mesh is not a conforming hexahedral mesh)");
                            return MTGPU_ERR_ARG;
                        }
                        rc[base + q] = li[k];
                        rv[base + q] = 0.0;
                        cnt[li[j]]++;
                    }
                    rv[base + q] += bv;
                }
            }
        }
        for (int i = 0; i < nn; i++) {
            const size_t base = 27 * (size_t)i;
            std::vector<std::pair<int, double>> row(cnt[i]);
            for (int q = 0; q < cnt[i]; q++) row[q] = {rc[base + q], rv[base + q]};
            std::sort(row.begin(), row.end());
            for (auto &e : row) {
                mcol.push_back(n0 + e.first);
                mval.push_back(e.second);
                if (e.first == i) mdiag[n0 + i] = e.second;
            }
            mptr[n0 + i + 1] = (int)mcol.size();
            for (int c : adj[i]) nc.push_back(c);
            nc_ptr[n0 + i + 1] = (int)nc.size();
        }
        for (int i = nn; i < node_off[s + 1] - n0; i++) {   // padding rows
            mptr[n0 + i + 1] = (int)mcol.size();
            nc_ptr[n0 + i + 1] = (int)nc.size();
        }
        for (int i = 0; i < nn; i++) loc[B.nodes[i]] = -1;
    }
    // receivers: padded nodes and trilinear weights of their brick, per type
    std::vector<int> rn((size_t)nrec * 16, -1);
    std::vector<double> rw((size_t)nrec * 16, 0.0);
    for (int r = 0; r < nrec; r++) {
        for (int t = 0; t < 2; t++) {
            const int c = t == 0 ? eb[r] : ea[r];
            if (c < 0) continue;
            int s = 0;
            if (t == 1) s = 1 + (int)(std::lower_bound(mats.begin(), mats.end(), a.nvkat[c]) -
                                      mats.begin());
            const SubBuild &B = subs[s];
            const int *nv = &a.nver[(size_t)c * ns];
            for (int j = 0; j < 8; j++) {
                auto it = std::lower_bound(B.nodes.begin(), B.nodes.end(), nv[j]);
                rn[(size_t)(r * 2 + t) * 8 + j] = node_off[s] + (int)(it - B.nodes.begin());
            }
            trilinear_weights(&a.xyz[3 * (size_t)nv[0]], &a.xyz[3 * (size_t)nv[7]],
                              xyz_rec + 3 * (size_t)r, &rw[(size_t)(r * 2 + t) * 8]);
        }
    }
    int rc;
    if ((rc = upload(&sm.d_cell, cell, st)) || (rc = upload(&sm.d_cell_sub, cell_sub, st)) ||
        (rc = upload(&sm.d_cell_g, cell_g, st)) || (rc = upload(&sm.d_nc_ptr, nc_ptr, st)) ||
        (rc = upload(&sm.d_nc, nc, st)) || (rc = upload(&sm.d_mptr, mptr, st)) ||
        (rc = upload(&sm.d_mcol, mcol, st)) || (rc = upload(&sm.d_mval, mval, st)) ||
        (rc = upload(&sm.d_mdiag, mdiag, st)) || (rc = upload(&sm.d_blk_sub, blk_sub, st)) ||
        (rc = upload(&sm.d_rn, rn, st)) || (rc = upload(&sm.d_rw, rw, st)) ||
        (rc = dev_alloc(&sm.d_active, 1)))
        return rc;
    MTGPU_TRY(cudaStreamSynchronize(st));   // the host vectors go out of scope
    return MTGPU_OK;
}

int smoothing_fields(Smoothing &sm, const ParamMatrix &P, int nrec, int S, long long x_stride,
                     const double2 *d_x, const double *d_omega, const int *d_alfa, int n1d,
                     const double *d_z1d, const double *d_us, const double *d_uc,
                     const double4 *d_loc, double2 *d_e, double2 *d_h, double2 *d_scal,
                     cudaStream_t st)
{
    // grow-only work arrays
    const int ncol = 6 * S, nprob = ncol * sm.nsub;
    if (S > sm.S_cap) {
        for (double **p : {&sm.d_val, &sm.d_x, &sm.d_r, &sm.d_z, &sm.d_p, &sm.d_q, &sm.d_scal})
            dev_free(*p);
        dev_free(sm.d_done);
        sm.S_cap = 0;
        const size_t nv = (size_t)ncol * sm.npad;
        int rc;
        if ((rc = dev_alloc(&sm.d_val, (size_t)ncol * std::max(sm.ncell, 1))) ||
            (rc = dev_alloc(&sm.d_x, nv)) || (rc = dev_alloc(&sm.d_r, nv)) ||
            (rc = dev_alloc(&sm.d_z, nv)) || (rc = dev_alloc(&sm.d_p, nv)) ||
            (rc = dev_alloc(&sm.d_q, nv)) || (rc = dev_alloc(&sm.d_scal, (size_t)kNq * nprob)) ||
            (rc = dev_alloc(&sm.d_done, (size_t)nprob)))
            return rc;
        sm.S_cap = S;
    }
    MTGPU_TRY(cudaMemsetAsync(sm.d_scal, 0, sizeof(double) * kNq * nprob, st));
    unsigned long long launches = 0;
    sm.iterations = 0;
    if (sm.npad > 0) {
        k_sm_centre<<<dim3(ceil_div(sm.ncell, kThreads), S), kThreads, 0, st>>>(
            sm.ncell, S, sm.d_cell, sm.d_cell_sub, P.d_nver, P.nver_stride, P.d_ed, P.ed_stride,
            P.d_xyz, x_stride, d_x, sm.d_val);
        const dim3 grid(sm.nblk, ncol);
        k_sm_init<<<grid, kBlk, 0, st>>>(sm.npad, sm.ncell, sm.nsub, sm.d_blk_sub, sm.d_nc_ptr,
                                         sm.d_nc, sm.d_cell_g, sm.d_val, sm.d_mdiag, sm.d_x,
                                         sm.d_r, sm.d_z, sm.d_p, sm.d_scal, nprob);
        const int gp = ceil_div(nprob, kThreads);
        k_sm_start<<<gp, kThreads, 0, st>>>(nprob, sm.d_scal, sm.d_done);
        launches += 3;
        MTGPU_TRY(cudaGetLastError());
        int active = 1;
        while (active > 0 && sm.iterations < kMaxIter) {
            for (int it = 0; it < kCheckEvery; it++) {
                // the count of running problems comes from the last scalars pass
                if (it == kCheckEvery - 1)
                    MTGPU_TRY(cudaMemsetAsync(sm.d_active, 0, sizeof(int), st));
                k_sm_spmv<<<grid, kBlk, 0, st>>>(sm.npad, sm.nsub, sm.d_blk_sub, sm.d_mptr,
                                                 sm.d_mcol, sm.d_mval, sm.d_p, sm.d_q, sm.d_scal,
                                                 sm.d_done, nprob);
                k_sm_update<<<grid, kBlk, 0, st>>>(sm.npad, sm.nsub, sm.d_blk_sub, sm.d_mdiag,
                                                   sm.d_x, sm.d_r, sm.d_z, sm.d_p, sm.d_q,
                                                   sm.d_scal, sm.d_done, nprob);
                k_sm_scalars<<<gp, kThreads, 0, st>>>(nprob, sm.d_scal, sm.d_done, sm.d_active);
                k_sm_direction<<<grid, kBlk, 0, st>>>(sm.npad, sm.nsub, sm.d_blk_sub, sm.d_z,
                                                      sm.d_p, sm.d_scal, sm.d_done, nprob);
                launches += 4;
            }
            sm.iterations += kCheckEvery;
            MTGPU_TRY(cudaGetLastError());
            MTGPU_TRY(cudaMemcpyAsync(&active, sm.d_active, sizeof(int), cudaMemcpyDeviceToHost,
                                      st));
            MTGPU_TRY(cudaStreamSynchronize(st));
        }
        if (active > 0) {
            set_last_message("receiver smoothing: the projection solve did not converge");
            note_launches(launches);
            return MTGPU_MAXITER;
        }
    }
    k_sm_receivers<<<dim3(ceil_div(nrec, 128), S), 128, 0, st>>>(
        nrec, S, sm.npad, sm.d_rn, sm.d_rw, sm.d_x, d_omega, d_alfa, n1d, d_z1d, d_us, d_uc,
        d_loc, d_e, d_h, d_scal);
    note_launches(launches + 1);
    MTGPU_TRY(cudaGetLastError());
    return MTGPU_OK;
}

}  // namespace mtgpu
