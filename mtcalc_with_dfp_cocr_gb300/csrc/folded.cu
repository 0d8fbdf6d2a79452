// Folded preconditioner  M^{-1} = D_A + G^T D_S G  on the device.
//
// G is the discrete gradient restricted to the interior nodes of conductive
// cells, with -1/2 for an edge's first node and +1/2 for its second
// (Code/COCR_FP/FoldedPreconditioner.cpp:68-259), D_A = diag(A)^{-1} and
// D_S = diag(G A G^T)^{-1} (FoldedPreconditioner.cpp:473-574).  The apply
// (FoldedPreconditioner.cpp:578-630) is a node gather followed by an edge
// gather; the COCR loop fuses both into its own kernels, the generic form
// here serves the set-up stages and the stand-alone entry point.
#include "mtgpu_internal.cuh"

#include <climits>

namespace mtgpu {

void Folded::release()
{
    dev_free(d_gp); dev_free(d_gj); dev_free(d_gv);
    dev_free(d_tp); dev_free(d_tj); dev_free(d_tv); dev_free(d_tn);
    dev_free(d_da); dev_free(d_ds); dev_free(d_h);
    n = m = 0;
}

int folded_build_g(const mtgpu_mesh_desc &mesh, Folded &P, cudaStream_t st)
{
    P.release();
    const int ne = mesh.n_edges_c, nn = mesh.n_nodes_c;
    MTGPU_CHECK_ARG(ne > 0 && nn > 0, "empty mesh");
    std::vector<char> in_sigma(nn, 0);
    for (int c = 0; c < mesh.kpar; c++) {
        if (!(mesh.sigma3d[mesh.nvkat[c]] > 0.0)) continue;
        for (int j = 0; j < 8; j++) {
            const int v = mesh.nver14[(size_t)c * mesh.nver_stride + j];
            if (v >= 0 && v < nn && !mesh.is_node_bound[v]) in_sigma[v] = 1;
        }
    }
    std::vector<int> renum(nn, -1);
    int m = 0;
    for (int v = 0; v < nn; v++)
        if (in_sigma[v]) renum[v] = m++;
    // G^T rows: the edge's first node (-1/2) then its second (+1/2); nodes
    // beyond n_nodes_c are expanded through the T-matrix rows ig_t/jg_t/gg_t
    std::vector<int> tp(ne + 1, 0), tj;
    std::vector<double> tv;
    std::vector<int2> tn(ne, make_int2(-1, -1));
    bool compact = true;
    tj.reserve((size_t)ne * 2);
    tv.reserve((size_t)ne * 2);
    for (int e = 0; e < ne; e++) {
        for (int k = 0; k < 2; k++) {
            const int v = mesh.edges2[2 * e + k];
            const double sgn = k == 0 ? -0.5 : 0.5;
            if (v < nn) {
                if (v >= 0 && in_sigma[v]) {
                    tj.push_back(renum[v]);
                    tv.push_back(sgn);
                    (k == 0 ? tn[e].x : tn[e].y) = renum[v];
                }
            } else {
                compact = false;
                for (int t = mesh.ig_t[v]; t < mesh.ig_t[v + 1]; t++)
                    if (in_sigma[mesh.jg_t[t]]) {
                        tj.push_back(renum[mesh.jg_t[t]]);
                        tv.push_back(sgn * mesh.gg_t[t]);
                    }
            }
        }
        tp[e + 1] = (int)tj.size();
    }
    const int nnz = tp[ne];
    std::vector<int> gp(m + 1, 0), gj(nnz > 0 ? nnz : 1), fill;
    std::vector<double> gv(nnz > 0 ? nnz : 1);
    for (int t = 0; t < nnz; t++) gp[tj[t] + 1]++;
    for (int i = 0; i < m; i++) gp[i + 1] += gp[i];
    fill.assign(gp.begin(), gp.end() - 1);
    for (int e = 0; e < ne; e++)
        for (int t = tp[e]; t < tp[e + 1]; t++) {
            const int r = tj[t];
            gj[fill[r]] = e;
            gv[fill[r]] = tv[t];
            fill[r]++;
        }
    P.n = ne;
    P.m = m;
    int rc;
    if ((rc = dev_alloc(&P.d_gp, m + 1)) || (rc = dev_alloc(&P.d_gj, nnz)) ||
        (rc = dev_alloc(&P.d_gv, nnz)) || (rc = dev_alloc(&P.d_tp, ne + 1)) ||
        (rc = dev_alloc(&P.d_tj, nnz)) || (rc = dev_alloc(&P.d_tv, nnz)) ||
        (rc = dev_alloc(&P.d_da, ne)) || (rc = dev_alloc(&P.d_ds, m)) ||
        (rc = dev_alloc(&P.d_h, m)))
        return rc;
    MTGPU_TRY(cudaMemcpyAsync(P.d_gp, gp.data(), sizeof(int) * (m + 1), cudaMemcpyHostToDevice, st));
    if (nnz > 0) {
        MTGPU_TRY(cudaMemcpyAsync(P.d_gj, gj.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
        MTGPU_TRY(cudaMemcpyAsync(P.d_gv, gv.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
        MTGPU_TRY(cudaMemcpyAsync(P.d_tj, tj.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
        MTGPU_TRY(cudaMemcpyAsync(P.d_tv, tv.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
    }
    MTGPU_TRY(cudaMemcpyAsync(P.d_tp, tp.data(), sizeof(int) * (ne + 1), cudaMemcpyHostToDevice, st));
    if (compact) {
        if ((rc = dev_alloc(&P.d_tn, ne))) return rc;
        MTGPU_TRY(cudaMemcpyAsync(P.d_tn, tn.data(), sizeof(int2) * ne, cudaMemcpyHostToDevice, st));
    }
    // the host vectors go out of scope: wait for the copies
    MTGPU_TRY(cudaStreamSynchronize(st));
    return MTGPU_OK;
}

namespace {

__device__ inline long long slot(const long long *p, int row, int k)
{
    return p[row / kSlice] + (long long)k * kSlice + (row % kSlice);
}

__global__ void k_diag_a(int nb, const long long *pc, const int *col_c, const double2 *val_c,
                         const int *diag_slot, double2 *da)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const int k = diag_slot[i];
    const double2 d = k >= 0 ? val_c[slot(pc, i, k)] : make_double2(0.0, 0.0);
    da[i] = cdiv(make_double2(1.0, 0.0), d);
}

// D_S[v] = 1 / sum_{k,c in row v of G} g_k g_c A[k][c].
// Re diag(G A G^T) is a cancellation (the curl-curl part annihilates
// gradients) and in the air it is not small next to the tiny imaginary
// part, so D_S there depends on the summation order.  This kernel therefore
// adds in the reference's order — row k of A by increasing column, complex
// and real entries merged (FoldedPreconditioner.cpp:518-556 over the rows
// of From2x2ToCSR2x2_2) — with unfused multiply and add.
__global__ void k_diag_s(int m, const int *gp, const int *gj, const double *gv,
                         const int *nc_row, const int *nr_row, const long long *pc,
                         const long long *pr, const int *col_c, const double2 *val_c,
                         const int *col_r, const double *val_r, double2 *ds)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m) return;
    const int b = gp[v], e = gp[v + 1];
    double sr = 0.0, si = 0.0;
    for (int j = b; j < e; j++) {
        const int k = gj[j];
        const double gk = gv[j];
        const int nc = nc_row[k], nr = nr_row[k];
        double tr = 0.0, ti = 0.0;
        int qc = 0, qr = 0;
        while (qc < nc || qr < nr) {
            const int cc = qc < nc ? col_c[slot(pc, k, qc)] : INT_MAX;
            const int cr = qr < nr ? col_r[slot(pr, k, qr)] : INT_MAX;
            double ar, ai;
            int c;
            if (cc < cr) {
                const double2 a = val_c[slot(pc, k, qc++)];
                ar = a.x;
                ai = a.y;
                c = cc;
            } else {
                ar = val_r[slot(pr, k, qr++)];
                ai = 0.0;
                c = cr;
            }
            for (int u = b; u < e; u++)
                if (gj[u] == c) {
                    tr = __dadd_rn(tr, __dmul_rn(ar, gv[u]));
                    ti = __dadd_rn(ti, __dmul_rn(ai, gv[u]));
                }
        }
        sr = __dadd_rn(sr, __dmul_rn(tr, gk));
        si = __dadd_rn(si, __dmul_rn(ti, gk));
    }
    ds[v] = cdiv(make_double2(1.0, 0.0), make_double2(sr, si));
}

__global__ void k_node(int m, const int *__restrict__ gp, const int *__restrict__ gj,
                       const double *__restrict__ gv, const double2 *__restrict__ ds,
                       const double2 *__restrict__ x, double2 *__restrict__ h)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m) return;
    double hr = 0.0, hi = 0.0;
    for (int j = gp[v]; j < gp[v + 1]; j++) {
        const double2 xv = x[gj[j]];
        hr += gv[j] * xv.x;
        hi += gv[j] * xv.y;
    }
    h[v] = cmul(make_double2(hr, hi), ds[v]);
}

__global__ void k_edge(int n, const int *__restrict__ tp, const int *__restrict__ tj,
                       const double *__restrict__ tv, const double2 *__restrict__ da,
                       const double2 *__restrict__ h, const double2 *__restrict__ x,
                       double2 *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 acc = cmul(x[i], da[i]);
    for (int j = tp[i]; j < tp[i + 1]; j++) {
        const double2 hv = h[tj[j]];
        acc.x += tv[j] * hv.x;
        acc.y += tv[j] * hv.y;
    }
    y[i] = acc;
}

}  // namespace

int folded_build_diag(const SellMatrix &A, Folded &P, cudaStream_t st)
{
    k_diag_a<<<ceil_div(A.nb, kThreads), kThreads, 0, st>>>(A.nb, A.d_pc, A.d_col_c, A.d_val_c,
                                                            A.d_diag_slot, P.d_da);
    if (P.m > 0)
        k_diag_s<<<ceil_div(P.m, 128), 128, 0, st>>>(P.m, P.d_gp, P.d_gj, P.d_gv, A.d_nc, A.d_nr,
                                                     A.d_pc, A.d_pr, A.d_col_c, A.d_val_c,
                                                     A.d_col_r, A.d_val_r, P.d_ds);
    MTGPU_TRY(cudaGetLastError());
    return MTGPU_OK;
}

void folded_apply(const Folded &P, const double2 *x, double2 *y, cudaStream_t st)
{
    if (P.m > 0)
        k_node<<<ceil_div(P.m, kThreads), kThreads, 0, st>>>(P.m, P.d_gp, P.d_gj, P.d_gv, P.d_ds,
                                                             x, P.d_h);
    k_edge<<<ceil_div(P.n, kThreads), kThreads, 0, st>>>(P.n, P.d_tp, P.d_tj, P.d_tv, P.d_da,
                                                         P.d_h, x, y);
}

}  // namespace mtgpu
