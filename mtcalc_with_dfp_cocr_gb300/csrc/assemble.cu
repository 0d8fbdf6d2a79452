// Device assembly of the edge-element system of the MT forward problem.
//
// The reference builds it on the host element by element
// (Code/BuildMatrix/t_global_slae.cpp:80-134, T_Brick.cpp:123-455 and
// 1361-1395) and writes it to files.  Here every row of the matrix is built
// by one GPU thread, which visits the (at most four) cells that share its
// edge in increasing cell order — the order in which the reference adds the
// element contributions — so no atomics are needed and every entry is summed
// in the reference's order.
//
// The result is kept in parametric form A(omega) = K + i omega M over one
// SELL-32 pattern:
//   K = sum_cells B / mu          (curl-curl, every edge pair of a cell)
//   M = sum_cells sigma C         (mass, parallel edge pairs only)
// with the homogeneous Dirichlet rows and columns of
// Code/BuildMatrix/bound_cond_vec_harm.cpp:260-307 already applied
// (identity on boundary rows).  The right-hand side of each system is
// assembled from the 1-D normal field table of its frequency
// (T_Brick.cpp:1361-1395, 1463-1495).
#include "assemble.cuh"
#include "fem.cuh"

#include <climits>

namespace mtgpu {

void ParamMatrix::release()
{
    dev_free(d_wc); dev_free(d_wr); dev_free(d_pc); dev_free(d_pr);
    dev_free(d_nc); dev_free(d_nr);
    dev_free(d_col_c); dev_free(d_col_r);
    dev_free(d_kc); dev_free(d_mc); dev_free(d_kr);
    dev_free(d_ec_ptr); dev_free(d_ec_cell);
    dev_free(d_xyz); dev_free(d_nver); dev_free(d_ed); dev_free(d_edges); dev_free(d_nvkat);
    dev_free(d_mu); dev_free(d_sig); dev_free(d_sig0);
    dev_free(d_bedge);
    dev_free(d_bnode);
    nb = nslices = 0;
}

namespace {

// ---------------------------------------------- edge -> cell adjacency
__global__ void k_ec_count(int kpar, const int *ed, int stride, int *cnt)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kpar) return;
    for (int l = 0; l < 12; l++) atomicAdd(&cnt[ed[(long long)c * stride + l] + 1], 1);
}

__global__ void k_ec_fill(int kpar, const int *ed, int stride, const int *ptr, int *fill,
                          int *cell_loc)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kpar) return;
    for (int l = 0; l < 12; l++) {
        const int e = ed[(long long)c * stride + l];
        const int k = atomicAdd(&fill[e], 1);
        cell_loc[ptr[e] + k] = c * 16 + l;   // cell and local index packed
    }
}

// cells of an edge in increasing order (insertion sort; lists are short)
__global__ void k_ec_sort(int nb, const int *ptr, int *cell_loc)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nb) return;
    const int b = ptr[e], n = ptr[e + 1] - b;
    for (int a = 1; a < n; a++) {
        const int v = cell_loc[b + a];
        int q = a - 1;
        while (q >= 0 && cell_loc[b + q] > v) {
            cell_loc[b + q + 1] = cell_loc[b + q];
            q--;
        }
        cell_loc[b + q + 1] = v;
    }
}

constexpr int kMaxRow = 64;   // distinct columns of one row (33 on a tensor mesh)

// the sorted distinct columns of row e with their parallel flag
__device__ int row_columns(int e, const int *ec_ptr, const int *ec_cell, const int *ed,
                           int stride, int *cols, unsigned char *par)
{
    int n = 0;
    for (int t = ec_ptr[e]; t < ec_ptr[e + 1]; t++) {
        const int cl = ec_cell[t];
        const int cell = cl >> 4, li = cl & 15;
        for (int lj = 0; lj < 12; lj++) {
            const int j = ed[(long long)cell * stride + lj];
            int q = 0;
            while (q < n && cols[q] != j) q++;
            if (q == n && n < kMaxRow) {
                cols[n] = j;
                par[n] = ldir(li) == ldir(lj);
                n++;
            }
        }
    }
    for (int a = 1; a < n; a++) {
        const int v = cols[a];
        const unsigned char p = par[a];
        int q = a - 1;
        while (q >= 0 && cols[q] > v) {
            cols[q + 1] = cols[q];
            par[q + 1] = par[q];
            q--;
        }
        cols[q + 1] = v;
        par[q + 1] = p;
    }
    return n;
}

__global__ void k_row_counts(int nb, const int *ec_ptr, const int *ec_cell, const int *ed,
                             int stride, int *nc, int *nr, int *overflow)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nb) return;
    int cols[kMaxRow];
    unsigned char par[kMaxRow];
    const int n = row_columns(e, ec_ptr, ec_cell, ed, stride, cols, par);
    int c = 0;
    for (int q = 0; q < n; q++) c += par[q];
    nc[e] = c;
    nr[e] = n - c;
    // a row with more distinct columns than kMaxRow cannot be represented
    int raw = 0;
    for (int t = ec_ptr[e]; t < ec_ptr[e + 1]; t++) raw += 12;
    if (n == kMaxRow && raw > kMaxRow) atomicExch(overflow, 1);
}

__global__ void k_widths2(int nb, int nslices, const int *nc, const int *nr, int *wc, int *wr,
                          unsigned long long *tot)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslices) return;
    int a = 0, b = 0;
    unsigned long long sa = 0, sb = 0;
    for (int l = 0; l < kSlice; l++) {
        const int i = s * kSlice + l;
        if (i < nb) {
            a = max(a, nc[i]);
            b = max(b, nr[i]);
            sa += nc[i];
            sb += nr[i];
        }
    }
    wc[s] = a;
    wr[s] = b;
    atomicAdd(&tot[0], sa);
    atomicAdd(&tot[1], sb);
}

__device__ __forceinline__ long long slot(const long long *p, int row, int k)
{
    return p[row / kSlice] + (long long)k * kSlice + (row % kSlice);
}

// Pattern and values of every row.  Contributions of the row's cells are
// added in increasing cell order; Dirichlet rows become identity rows and
// Dirichlet columns are zeroed.
__global__ void k_row_fill(int nb, int nslices, const int *ec_ptr, const int *ec_cell,
                           const int *ed, int ed_stride, const int *nver, int nver_stride,
                           const double *xyz, const int *nvkat, const double *mu,
                           const double *sig, const unsigned char *bedge, const int *wc,
                           const int *wr, const long long *pc, const long long *pr,
                           int *col_c, double *kc, double *mc, int *col_r, double *kr)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nslices * kSlice) return;
    const int s = e / kSlice;
    if (e >= nb) {
        // padding rows of the last slice
        const int last = nb - 1;
        for (int k = 0; k < wc[s]; k++) {
            const long long t = pc[s] + (long long)k * kSlice + (e % kSlice);
            col_c[t] = last; kc[t] = 0.0; mc[t] = 0.0;
        }
        for (int k = 0; k < wr[s]; k++) {
            const long long t = pr[s] + (long long)k * kSlice + (e % kSlice);
            col_r[t] = last; kr[t] = 0.0;
        }
        return;
    }
    int cols[kMaxRow];
    unsigned char par[kMaxRow];
    double K[kMaxRow], M[kMaxRow];
    const int n = row_columns(e, ec_ptr, ec_cell, ed, ed_stride, cols, par);
    for (int q = 0; q < n; q++) K[q] = M[q] = 0.0;
    for (int t = ec_ptr[e]; t < ec_ptr[e + 1]; t++) {
        const int cl = ec_cell[t];
        const int cell = cl >> 4, li = cl & 15;
        double h[3];
        cell_h(xyz, nver, nver_stride, cell, h);
        const int mat = nvkat[cell];
        const double muc = mu[mat], sc = sig[mat];
        for (int lj = 0; lj < 12; lj++) {
            const int j = ed[(long long)cell * ed_stride + lj];
            // binary search of column j
            int lo = 0, hi = n - 1, q = -1;
            while (lo <= hi) {
                const int mid = (lo + hi) >> 1;
                if (cols[mid] == j) { q = mid; break; }
                if (cols[mid] < j) lo = mid + 1; else hi = mid - 1;
            }
            if (q < 0) continue;
            double b, c;
            brick_entry(li, lj, h, b, c);
            K[q] = __dadd_rn(K[q], __ddiv_rn(b, muc));
            M[q] = __dadd_rn(M[q], __dmul_rn(c, sc));
        }
    }
    const bool brow = bedge[e] != 0;
    int qc = 0, qr = 0;
    for (int q = 0; q < n; q++) {
        const int j = cols[q];
        double kv = K[q], mv = M[q];
        if (brow || bedge[j]) {
            kv = (j == e) ? 1.0 : 0.0;
            mv = 0.0;
        }
        if (par[q]) {
            const long long t = slot(pc, e, qc++);
            col_c[t] = j; kc[t] = kv; mc[t] = mv;
        } else {
            const long long t = slot(pr, e, qr++);
            col_r[t] = j; kr[t] = kv;
        }
    }
    for (; qc < wc[s]; qc++) {
        const long long t = slot(pc, e, qc);
        col_c[t] = e; kc[t] = 0.0; mc[t] = 0.0;
    }
    for (; qr < wr[s]; qr++) {
        const long long t = slot(pr, e, qr);
        col_r[t] = e; kr[t] = 0.0;
    }
}

__global__ void k_bedge(int nb, const int *edges, const unsigned char *bnode, unsigned char *bedge)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nb) return;
    bedge[e] = bnode[edges[2 * e]] && bnode[edges[2 * e + 1]];
}

__global__ void k_bnode(int nbnd, const int *bnd, unsigned char *bnode)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nbnd) bnode[bnd[i]] = 1;
}

// A0 as edge values of every system: the 1-D field of the system's
// frequency at the edge midpoint times (alfa, 1 - alfa, 0), dotted with
// J t = (h_d / 2) e_d (T_Brick.cpp:1463-1495).  h_d is the edge's length
// (the cell size along d).  a0[k][e] = (sin, cos) parts.
__global__ void k_a0(int nb, int S, const int *alfa, int n1d, const double *z1d,
                     const double *usin, const double *ucos, const int *edges, const double *xyz,
                     double2 *a0)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (e >= nb || k >= S) return;
    const int n1 = edges[2 * e], n2 = edges[2 * e + 1];
    const double dx = xyz[3 * n2] - xyz[3 * n1], dy = xyz[3 * n2 + 1] - xyz[3 * n1 + 1];
    const int d = dx != 0.0 ? 0 : (dy != 0.0 ? 1 : 2);
    double as = 0.0, ac = 0.0;
    if (d != 2) {
        const double h = d == 0 ? dx : dy;
        const double wx = alfa[k] ? 1.0 : 0.0;
        const double wd = d == 0 ? wx : 1.0 - wx;
        const double zm = 0.5 * (xyz[3 * n1 + 2] + xyz[3 * n2 + 2]);
        const double *us = usin + (long long)k * n1d, *uc = ucos + (long long)k * n1d;
        as = __dmul_rn(0.5 * h, __dmul_rn(spline(zm, n1d, z1d, us), wd));
        ac = __dmul_rn(0.5 * h, __dmul_rn(spline(zm, n1d, z1d, uc), wd));
    }
    a0[(long long)k * nb + e] = make_double2(as, ac);
}

// Right-hand sides of S systems: b = i omega (sigma0 - sigma) C A0 summed
// over the row's cells (T_Brick.cpp:1361-1395), zero on Dirichlet rows.
__global__ void k_rhs(int nb, int S, const double *omega, const double2 *a0,
                      const int *ec_ptr, const int *ec_cell, const int *ed, int ed_stride,
                      const int *nver, int nver_stride, const double *xyz,
                      const int *nvkat, const double *sig, const double *sig0,
                      const unsigned char *bedge, double2 *rhs, long long rhs_stride,
                      int interleaved)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (e >= nb || k >= S) return;
    double pre = 0.0, pim = 0.0;
    if (!bedge[e]) {
        const double w = omega[k];
        const double2 *ak = a0 + (long long)k * nb;
        for (int t = ec_ptr[e]; t < ec_ptr[e + 1]; t++) {
            const int cl = ec_cell[t];
            const int cell = cl >> 4, li = cl & 15;
            double h[3];
            cell_h(xyz, nver, nver_stride, cell, h);
            const int mat = nvkat[cell];
            const double mult = (sig0[mat] - sig[mat]) * w;
            double gre = 0.0, gim = 0.0;
            for (int lj = 0; lj < 8; lj++) {   // x and y edges: A0 has no z part
                double b, c;
                brick_entry(li, lj, h, b, c);
                const double2 v = ak[ed[(long long)cell * ed_stride + lj]];
                gre = __dadd_rn(gre, __dmul_rn(c, v.x));
                gim = __dadd_rn(gim, __dmul_rn(c, v.y));
            }
            pre = __dadd_rn(pre, __dmul_rn(gim, -mult));
            pim = __dadd_rn(pim, __dmul_rn(gre, mult));
        }
    }
    const long long idx = interleaved ? (long long)e * S + k : (long long)k * rhs_stride + e;
    rhs[idx] = make_double2(pre, pim);
}

// complex values of A(omega) = K + i omega M
__global__ void k_form_a(long long len_c, long long len_r, const double *kc, const double *mc,
                         const double *kr, double omega, double2 *val_c, double *val_r)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len_c) val_c[i] = make_double2(kc[i], __dmul_rn(mc[i], omega));
    if (i < len_r) val_r[i] = kr[i];
}

__global__ void k_diag_slot(int nb, const int *nc, const long long *pc, const int *col_c,
                            int *diag_slot)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    int d = -1;
    for (int q = 0; q < nc[i]; q++)
        if (col_c[slot(pc, i, q)] == i) d = q;
    diag_slot[i] = d;
}

// lower-triangle block format of the reference: per row the number of
// columns below the diagonal, and the doubles they take
__global__ void k_lower_counts(int nb, const int *nc, const int *nr, const long long *pc,
                               const long long *pr, const int *col_c, const int *col_r,
                               int *cnt, int *dbl)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    int a = 0, b = 0;
    for (int q = 0; q < nc[i]; q++)
        if (col_c[slot(pc, i, q)] < i) { a++; b += 2; }
    for (int q = 0; q < nr[i]; q++)
        if (col_r[slot(pr, i, q)] < i) { a++; b += 1; }
    cnt[i] = a;
    dbl[i] = b;
}

__global__ void k_lower_fill(int nb, const int *nc, const int *nr, const long long *pc,
                             const long long *pr, const int *col_c, const int *col_r,
                             const double *kc, const double *mc, const double *kr,
                             double omega, const int *ig, const int *gofs, int *jg, int *ijg,
                             double *di, double *gg)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    int qc = 0, qr = 0, w = ig[i], o = gofs[i];
    const int ncc = nc[i], nrr = nr[i];
    while (qc < ncc || qr < nrr) {
        const int cc = qc < ncc ? col_c[slot(pc, i, qc)] : INT_MAX;
        const int cr = qr < nrr ? col_r[slot(pr, i, qr)] : INT_MAX;
        if (cc < cr) {
            const long long t = slot(pc, i, qc++);
            if (cc < i) {
                jg[w] = cc; ijg[w] = o; w++;
                gg[o] = kc[t];
                gg[o + 1] = __dmul_rn(mc[t], omega);
                o += 2;
            } else if (cc == i) {
                di[2 * i] = kc[t];
                di[2 * i + 1] = __dmul_rn(mc[t], omega);
            }
        } else {
            const long long t = slot(pr, i, qr++);
            if (cr < i) {
                jg[w] = cr; ijg[w] = o; w++;
                gg[o] = kr[t];
                o += 1;
            }
        }
    }
}

}  // namespace

int exclusive_scan_host(const int *d_in, int n, int *d_out, long long *total, cudaStream_t st)
{
    std::vector<int> h(n);
    if (n) MTGPU_TRY(cudaMemcpyAsync(h.data(), d_in, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    MTGPU_TRY(cudaStreamSynchronize(st));
    std::vector<int> o(n + 1);
    long long acc = 0;
    for (int i = 0; i < n; i++) {
        o[i] = (int)acc;
        acc += h[i];
    }
    o[n] = (int)acc;
    MTGPU_CHECK_ARG(acc < INT_MAX, "matrix too large for 32-bit offsets");
    MTGPU_TRY(cudaMemcpyAsync(d_out, o.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st));
    MTGPU_TRY(cudaStreamSynchronize(st));
    if (total) *total = acc;
    return MTGPU_OK;
}

template <class T>
static int up(T **d, const T *h, size_t n, cudaStream_t st)
{
    int rc = dev_alloc(d, n);
    if (rc) return rc;
    if (n) MTGPU_TRY(cudaMemcpyAsync(*d, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
    return MTGPU_OK;
}

int param_assemble(const mtgpu_fem_mesh &m, ParamMatrix &P, cudaStream_t st)
{
    P.release();
    MTGPU_CHECK_ARG(m.nb > 0 && m.kpar > 0 && m.kuzlov > 0 && m.n_materials > 0, "bad mesh sizes");
    MTGPU_CHECK_ARG(m.xyz && m.nver && m.ed && m.edges && m.nvkat && m.mu && m.sigma && m.sigma0,
                    "null mesh pointer");
    MTGPU_CHECK_ARG(m.nver_stride >= 8 && m.ed_stride >= 12, "bad strides");
    for (int i = 0; i < m.n_materials; i++) {
        MTGPU_CHECK_ARG(m.mu[i] > 0.0, "mu must be positive");
        if (m.mu0) MTGPU_CHECK_ARG(m.mu0[i] == m.mu[i], "mu0 != mu is not supported");
        if (m.dpr) MTGPU_CHECK_ARG(m.dpr[i] == 0.0, "displacement currents (dpr != 0) are not supported");
        if (m.dpr0) MTGPU_CHECK_ARG(m.dpr0[i] == 0.0, "displacement currents (dpr0 != 0) are not supported");
    }
    for (int c = 0; c < m.kpar; c++) {
        MTGPU_CHECK_ARG(m.nvkat[c] >= 0 && m.nvkat[c] < m.n_materials, "nvkat out of range");
        for (int l = 0; l < 12; l++) {
            const int e = m.ed[(size_t)c * m.ed_stride + l];
            MTGPU_CHECK_ARG(e >= 0 && e < m.nb, "cell edge out of range");
        }
        for (int l = 0; l < 8; l++) {
            const int v = m.nver[(size_t)c * m.nver_stride + l];
            MTGPU_CHECK_ARG(v >= 0 && v < m.kuzlov, "cell node out of range");
        }
    }
    for (int e = 0; e < m.nb; e++)
        MTGPU_CHECK_ARG(m.edges[2 * e] >= 0 && m.edges[2 * e] < m.kuzlov && m.edges[2 * e + 1] >= 0 &&
                            m.edges[2 * e + 1] < m.kuzlov, "edge node out of range");
    for (int i = 0; i < m.n_bound; i++)
        MTGPU_CHECK_ARG(m.bound_nodes[i] >= 0 && m.bound_nodes[i] < m.kuzlov, "boundary node out of range");

    const int nb = m.nb, kpar = m.kpar;
    P.nb = nb;
    P.kpar = kpar;
    P.kuzlov = m.kuzlov;
    P.n_materials = m.n_materials;
    P.ed_stride = m.ed_stride;
    P.nver_stride = m.nver_stride;
    P.nslices = ceil_div(nb, kSlice);
    int rc;
    if ((rc = up(&P.d_xyz, m.xyz, (size_t)m.kuzlov * 3, st)) ||
        (rc = up(&P.d_nver, m.nver, (size_t)kpar * m.nver_stride, st)) ||
        (rc = up(&P.d_ed, m.ed, (size_t)kpar * m.ed_stride, st)) ||
        (rc = up(&P.d_edges, m.edges, (size_t)nb * 2, st)) ||
        (rc = up(&P.d_nvkat, m.nvkat, (size_t)kpar, st)) ||
        (rc = up(&P.d_mu, m.mu, (size_t)m.n_materials, st)) ||
        (rc = up(&P.d_sig, m.sigma, (size_t)m.n_materials, st)) ||
        (rc = up(&P.d_sig0, m.sigma0, (size_t)m.n_materials, st)))
        return rc;
    unsigned char *bnode = nullptr;
    int *d_bnd = nullptr;
    if ((rc = dev_alloc(&bnode, m.kuzlov))) return rc;
    MTGPU_TRY(cudaMemsetAsync(bnode, 0, m.kuzlov, st));
    if (m.n_bound > 0) {
        if ((rc = up(&d_bnd, m.bound_nodes, (size_t)m.n_bound, st))) {
            dev_free(bnode);
            return rc;
        }
        k_bnode<<<ceil_div(m.n_bound, kThreads), kThreads, 0, st>>>(m.n_bound, d_bnd, bnode);
    }
    rc = param_build(P, bnode, st);
    P.d_bnode = bnode;   // kept for the solver set-up (preconditioner, matrix-free tables)
    dev_free(d_bnd);
    return rc;
}

// The device part of the assembly, from the mesh tables in P (d_xyz,
// d_nver, d_ed, d_edges, d_nvkat, the materials) and the Dirichlet node
// flags bnode[kuzlov]
int param_build(ParamMatrix &P, const unsigned char *bnode, cudaStream_t st)
{
    const int nb = P.nb, kpar = P.kpar;
    int rc;
    // Dirichlet edges: both nodes on the boundary (bound_cond_vec_harm.cpp:81-108)
    if ((rc = dev_alloc(&P.d_bedge, nb))) return rc;
    k_bedge<<<ceil_div(nb, kThreads), kThreads, 0, st>>>(nb, P.d_edges, bnode, P.d_bedge);
    // edge -> cells
    int *cnt = nullptr, *fill = nullptr, *overflow = nullptr;
    if ((rc = dev_alloc(&cnt, nb + 1)) || (rc = dev_alloc(&fill, nb)) ||
        (rc = dev_alloc(&P.d_ec_ptr, nb + 1)) || (rc = dev_alloc(&P.d_ec_cell, (size_t)kpar * 12)) ||
        (rc = dev_alloc(&overflow, 1)))
        return rc;
    MTGPU_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (nb + 1), st));
    MTGPU_TRY(cudaMemsetAsync(fill, 0, sizeof(int) * nb, st));
    MTGPU_TRY(cudaMemsetAsync(overflow, 0, sizeof(int), st));
    k_ec_count<<<ceil_div(kpar, kThreads), kThreads, 0, st>>>(kpar, P.d_ed, P.ed_stride, cnt);
    {
        // cnt[e+1] holds the count of edge e; ptr = inclusive scan
        std::vector<int> h(nb + 1);
        MTGPU_TRY(cudaMemcpyAsync(h.data(), cnt, sizeof(int) * (nb + 1), cudaMemcpyDeviceToHost, st));
        MTGPU_TRY(cudaStreamSynchronize(st));
        h[0] = 0;
        for (int e = 0; e < nb; e++) h[e + 1] += h[e];
        MTGPU_TRY(cudaMemcpyAsync(P.d_ec_ptr, h.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, st));
        MTGPU_TRY(cudaStreamSynchronize(st));
    }
    k_ec_fill<<<ceil_div(kpar, kThreads), kThreads, 0, st>>>(kpar, P.d_ed, P.ed_stride, P.d_ec_ptr,
                                                              fill, P.d_ec_cell);
    k_ec_sort<<<ceil_div(nb, kThreads), kThreads, 0, st>>>(nb, P.d_ec_ptr, P.d_ec_cell);
    // pattern
    unsigned long long *tot = nullptr;
    if ((rc = dev_alloc(&P.d_nc, nb)) || (rc = dev_alloc(&P.d_nr, nb)) ||
        (rc = dev_alloc(&P.d_wc, P.nslices)) || (rc = dev_alloc(&P.d_wr, P.nslices)) ||
        (rc = dev_alloc(&P.d_pc, P.nslices + 1)) || (rc = dev_alloc(&P.d_pr, P.nslices + 1)) ||
        (rc = dev_alloc(&tot, 2)))
        return rc;
    MTGPU_TRY(cudaMemsetAsync(tot, 0, 2 * sizeof(unsigned long long), st));
    k_row_counts<<<ceil_div(nb, 128), 128, 0, st>>>(nb, P.d_ec_ptr, P.d_ec_cell, P.d_ed,
                                                    P.ed_stride, P.d_nc, P.d_nr, overflow);
    k_widths2<<<ceil_div(P.nslices, kThreads), kThreads, 0, st>>>(nb, P.nslices, P.d_nc, P.d_nr,
                                                                   P.d_wc, P.d_wr, tot);
    MTGPU_TRY(cudaGetLastError());
    std::vector<int> wc(P.nslices), wr(P.nslices);
    unsigned long long htot[2];
    int hover = 0;
    MTGPU_TRY(cudaMemcpyAsync(wc.data(), P.d_wc, sizeof(int) * P.nslices, cudaMemcpyDeviceToHost, st));
    MTGPU_TRY(cudaMemcpyAsync(wr.data(), P.d_wr, sizeof(int) * P.nslices, cudaMemcpyDeviceToHost, st));
    MTGPU_TRY(cudaMemcpyAsync(htot, tot, sizeof(htot), cudaMemcpyDeviceToHost, st));
    MTGPU_TRY(cudaMemcpyAsync(&hover, overflow, sizeof(int), cudaMemcpyDeviceToHost, st));
    MTGPU_TRY(cudaStreamSynchronize(st));
    dev_free(cnt); dev_free(fill); dev_free(tot); dev_free(overflow);
    MTGPU_CHECK_ARG(hover == 0, "a matrix row has more than 64 distinct columns");
    std::vector<long long> pc(P.nslices + 1), pr(P.nslices + 1);
    pc[0] = pr[0] = 0;
    for (int s = 0; s < P.nslices; s++) {
        pc[s + 1] = pc[s] + (long long)wc[s] * kSlice;
        pr[s + 1] = pr[s] + (long long)wr[s] * kSlice;
    }
    P.len_c = pc[P.nslices];
    P.len_r = pr[P.nslices];
    P.nnz_c = (long long)htot[0];
    P.nnz_r = (long long)htot[1];
    MTGPU_TRY(cudaMemcpyAsync(P.d_pc, pc.data(), sizeof(long long) * (P.nslices + 1), cudaMemcpyHostToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(P.d_pr, pr.data(), sizeof(long long) * (P.nslices + 1), cudaMemcpyHostToDevice, st));
    if ((rc = dev_alloc(&P.d_col_c, P.len_c)) || (rc = dev_alloc(&P.d_kc, P.len_c)) ||
        (rc = dev_alloc(&P.d_mc, P.len_c)) || (rc = dev_alloc(&P.d_col_r, P.len_r)) ||
        (rc = dev_alloc(&P.d_kr, P.len_r)))
        return rc;
    k_row_fill<<<P.nslices * kSlice / 128 + 1, 128, 0, st>>>(
        nb, P.nslices, P.d_ec_ptr, P.d_ec_cell, P.d_ed, P.ed_stride, P.d_nver, P.nver_stride,
        P.d_xyz, P.d_nvkat, P.d_mu, P.d_sig, P.d_bedge, P.d_wc, P.d_wr, P.d_pc, P.d_pr,
        P.d_col_c, P.d_kc, P.d_mc, P.d_col_r, P.d_kr);
    MTGPU_TRY(cudaGetLastError());
    MTGPU_TRY(cudaStreamSynchronize(st));
    note_launches(9);
    return MTGPU_OK;
}

int param_rhs(const ParamMatrix &P, int S, const double *d_omega, const int *d_alfa, int n1d,
              const double *d_z1d, const double *d_usin, const double *d_ucos, double2 *d_rhs,
              long long rhs_stride, int interleaved, cudaStream_t st)
{
    dim3 grid(ceil_div(P.nb, 128), S);
    double2 *a0 = nullptr;
    int rc = dev_alloc(&a0, (size_t)S * P.nb);
    if (rc) return rc;
    k_a0<<<grid, 128, 0, st>>>(P.nb, S, d_alfa, n1d, d_z1d, d_usin, d_ucos, P.d_edges, P.d_xyz, a0);
    k_rhs<<<grid, 128, 0, st>>>(P.nb, S, d_omega, a0, P.d_ec_ptr, P.d_ec_cell, P.d_ed,
                                P.ed_stride, P.d_nver, P.nver_stride, P.d_xyz, P.d_nvkat, P.d_sig,
                                P.d_sig0, P.d_bedge, d_rhs, rhs_stride, interleaved);
    note_launches(2);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dev_free(a0);
    if (e != cudaSuccess) {
        set_last_error(e, "param_rhs", __FILE__, __LINE__);
        return MTGPU_ERR_CUDA;
    }
    return MTGPU_OK;
}

int param_to_sell(const ParamMatrix &P, double omega, SellMatrix &A, cudaStream_t st)
{
    A.release();
    A.nb = P.nb;
    A.nslices = P.nslices;
    A.nnz_c = P.nnz_c;
    A.nnz_r = P.nnz_r;
    A.len_c = P.len_c;
    A.len_r = P.len_r;
    int rc;
    if ((rc = dev_alloc(&A.d_wc, A.nslices)) || (rc = dev_alloc(&A.d_wr, A.nslices)) ||
        (rc = dev_alloc(&A.d_pc, A.nslices + 1)) || (rc = dev_alloc(&A.d_pr, A.nslices + 1)) ||
        (rc = dev_alloc(&A.d_nc, A.nb)) || (rc = dev_alloc(&A.d_nr, A.nb)) ||
        (rc = dev_alloc(&A.d_col_c, A.len_c)) || (rc = dev_alloc(&A.d_col_r, A.len_r)) ||
        (rc = dev_alloc(&A.d_val_c, A.len_c)) || (rc = dev_alloc(&A.d_val_r, A.len_r)) ||
        (rc = dev_alloc(&A.d_diag_slot, A.nb)))
        return rc;
    MTGPU_TRY(cudaMemcpyAsync(A.d_wc, P.d_wc, sizeof(int) * A.nslices, cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(A.d_wr, P.d_wr, sizeof(int) * A.nslices, cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(A.d_pc, P.d_pc, sizeof(long long) * (A.nslices + 1), cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(A.d_pr, P.d_pr, sizeof(long long) * (A.nslices + 1), cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(A.d_nc, P.d_nc, sizeof(int) * A.nb, cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(A.d_nr, P.d_nr, sizeof(int) * A.nb, cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(A.d_col_c, P.d_col_c, sizeof(int) * A.len_c, cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(A.d_col_r, P.d_col_r, sizeof(int) * A.len_r, cudaMemcpyDeviceToDevice, st));
    const long long len = std::max(A.len_c, A.len_r);
    k_form_a<<<(unsigned)((len + kThreads - 1) / kThreads), kThreads, 0, st>>>(
        A.len_c, A.len_r, P.d_kc, P.d_mc, P.d_kr, omega, A.d_val_c, A.d_val_r);
    k_diag_slot<<<ceil_div(A.nb, kThreads), kThreads, 0, st>>>(A.nb, A.d_nc, A.d_pc, A.d_col_c,
                                                               A.d_diag_slot);
    note_launches(2);
    MTGPU_TRY(cudaGetLastError());
    return MTGPU_OK;
}

int param_to_block2x2(const ParamMatrix &P, double omega, Block2x2Dev &B, cudaStream_t st)
{
    B.release();
    const int nb = P.nb;
    int rc;
    int *cnt = nullptr, *dbl = nullptr, *gofs = nullptr;
    if ((rc = dev_alloc(&cnt, nb)) || (rc = dev_alloc(&dbl, nb)) || (rc = dev_alloc(&gofs, nb + 1)) ||
        (rc = dev_alloc(&B.ig, nb + 1)) || (rc = dev_alloc(&B.idi, nb + 1)) ||
        (rc = dev_alloc(&B.di, (size_t)2 * nb)))
        return rc;
    k_lower_counts<<<ceil_div(nb, kThreads), kThreads, 0, st>>>(nb, P.d_nc, P.d_nr, P.d_pc, P.d_pr,
                                                                P.d_col_c, P.d_col_r, cnt, dbl);
    long long nnz = 0, ndbl = 0;
    if ((rc = exclusive_scan_host(cnt, nb, B.ig, &nnz, st)) ||
        (rc = exclusive_scan_host(dbl, nb, gofs, &ndbl, st)))
        return rc;
    B.nb = nb;
    B.nnz = (int)nnz;
    B.gg_len = ndbl;
    if ((rc = dev_alloc(&B.jg, nnz)) || (rc = dev_alloc(&B.ijg, nnz + 1)) ||
        (rc = dev_alloc(&B.gg, ndbl)))
        return rc;
    {
        std::vector<int> idi(nb + 1);
        for (int i = 0; i <= nb; i++) idi[i] = 2 * i;    // every diagonal block is complex
        MTGPU_TRY(cudaMemcpyAsync(B.idi, idi.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, st));
        const int last = (int)ndbl;
        MTGPU_TRY(cudaMemcpyAsync(B.ijg + nnz, &last, sizeof(int), cudaMemcpyHostToDevice, st));
        k_lower_fill<<<ceil_div(nb, kThreads), kThreads, 0, st>>>(
            nb, P.d_nc, P.d_nr, P.d_pc, P.d_pr, P.d_col_c, P.d_col_r, P.d_kc, P.d_mc, P.d_kr, omega,
            B.ig, gofs, B.jg, B.ijg, B.di, B.gg);
        MTGPU_TRY(cudaGetLastError());
        MTGPU_TRY(cudaStreamSynchronize(st));
    }
    note_launches(2);
    dev_free(cnt); dev_free(dbl); dev_free(gofs);
    return MTGPU_OK;
}

void Block2x2Dev::release()
{
    dev_free(ig); dev_free(jg); dev_free(idi); dev_free(ijg); dev_free(di); dev_free(gg);
    nb = nnz = 0;
    gg_len = 0;
}

}  // namespace mtgpu

namespace mtgpu {
namespace {
__global__ void k_split_complex(long long len_c, long long len_r, const double2 *val_c,
                                const double *val_r, double *kc, double *mc, double *kr)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < len_c) {
        kc[i] = val_c[i].x;
        mc[i] = val_c[i].y;
    }
    if (i < len_r) kr[i] = val_r[i];
}
}  // namespace

int param_from_sell(const SellMatrix &A, ParamMatrix &P, cudaStream_t st)
{
    P.release();
    P.nb = A.nb;
    P.nslices = A.nslices;
    P.nnz_c = A.nnz_c;
    P.nnz_r = A.nnz_r;
    P.len_c = A.len_c;
    P.len_r = A.len_r;
    int rc;
    if ((rc = dev_alloc(&P.d_wc, P.nslices)) || (rc = dev_alloc(&P.d_wr, P.nslices)) ||
        (rc = dev_alloc(&P.d_pc, P.nslices + 1)) || (rc = dev_alloc(&P.d_pr, P.nslices + 1)) ||
        (rc = dev_alloc(&P.d_nc, P.nb)) || (rc = dev_alloc(&P.d_nr, P.nb)) ||
        (rc = dev_alloc(&P.d_col_c, P.len_c)) || (rc = dev_alloc(&P.d_col_r, P.len_r)) ||
        (rc = dev_alloc(&P.d_kc, P.len_c)) || (rc = dev_alloc(&P.d_mc, P.len_c)) ||
        (rc = dev_alloc(&P.d_kr, P.len_r)))
        return rc;
    MTGPU_TRY(cudaMemcpyAsync(P.d_wc, A.d_wc, sizeof(int) * P.nslices, cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(P.d_wr, A.d_wr, sizeof(int) * P.nslices, cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(P.d_pc, A.d_pc, sizeof(long long) * (P.nslices + 1), cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(P.d_pr, A.d_pr, sizeof(long long) * (P.nslices + 1), cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(P.d_nc, A.d_nc, sizeof(int) * P.nb, cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(P.d_nr, A.d_nr, sizeof(int) * P.nb, cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(P.d_col_c, A.d_col_c, sizeof(int) * P.len_c, cudaMemcpyDeviceToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(P.d_col_r, A.d_col_r, sizeof(int) * P.len_r, cudaMemcpyDeviceToDevice, st));
    const long long len = std::max(P.len_c, P.len_r);
    k_split_complex<<<(unsigned)((len + kThreads - 1) / kThreads), kThreads, 0, st>>>(
        P.len_c, P.len_r, A.d_val_c, A.d_val_r, P.d_kc, P.d_mc, P.d_kr);
    note_launches(1);
    MTGPU_TRY(cudaGetLastError());
    return MTGPU_OK;
}
}  // namespace mtgpu
