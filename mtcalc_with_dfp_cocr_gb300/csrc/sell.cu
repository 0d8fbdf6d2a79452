// Device matrix: conversion of the reference lower-triangle 2x2-block SLAE
// to full SELL-32 storage, and the FP64 complex SpMV.
//
// The reference multiplies from its lower storage and scatters every stored
// block into two rows (Code/COCR_FP/block_2x2_solver.cpp:73-173).  A row-
// parallel GPU kernel instead reads each row whole, so the conversion mirrors
// every lower block into the upper triangle once, at setup.  Slots of a row
// are ordered by column, so every sum has a fixed order and results are
// reproducible run to run.
#include "mtgpu_internal.cuh"

#include <algorithm>

namespace mtgpu {

void SellMatrix::release()
{
    dev_free(d_wc); dev_free(d_wr); dev_free(d_pc); dev_free(d_pr);
    dev_free(d_col_c); dev_free(d_col_r); dev_free(d_val_c); dev_free(d_val_r);
    dev_free(d_diag_slot); dev_free(d_nc); dev_free(d_nr);
    nb = nslices = 0;
}

namespace {

// one thread per row: count complex / real entries of every full row
__global__ void k_count(int nb, const int *__restrict__ ig, const int *__restrict__ jg,
                        const int *__restrict__ ijg, int *cnt_c, int *cnt_r)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    atomicAdd(&cnt_c[i], 1);  // the diagonal always takes a complex slot
    for (int q = ig[i]; q < ig[i + 1]; q++) {
        const int j = jg[q];
        if (ijg[q + 1] - ijg[q] == 2) {
            atomicAdd(&cnt_c[i], 1);
            atomicAdd(&cnt_c[j], 1);
        } else {
            atomicAdd(&cnt_r[i], 1);
            atomicAdd(&cnt_r[j], 1);
        }
    }
}

// one thread per slice: slice widths and entry totals
__global__ void k_widths(int nb, int nslices, const int *cnt_c, const int *cnt_r, int *wc,
                         int *wr, unsigned long long *tot)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslices) return;
    int a = 0, b = 0;
    unsigned long long sa = 0, sb = 0;
    for (int l = 0; l < kSlice; l++) {
        const int i = s * kSlice + l;
        if (i < nb) {
            a = max(a, cnt_c[i]);
            b = max(b, cnt_r[i]);
            sa += cnt_c[i];
            sb += cnt_r[i];
        }
    }
    wc[s] = a;
    wr[s] = b;
    atomicAdd(&tot[0], sa);
    atomicAdd(&tot[1], sb);
}

// padding: every slot points at its own row with value 0
__global__ void k_pad(int nb, int nslices, const int *wc, const int *wr, const long long *pc,
                      const long long *pr, int *col_c, double2 *val_c, int *col_r,
                      double *val_r)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslices * kSlice) return;
    const int s = i / kSlice, l = i % kSlice;
    const int row = i < nb ? i : nb - 1;
    for (int k = 0; k < wc[s]; k++) {
        col_c[pc[s] + (long long)k * kSlice + l] = row;
        val_c[pc[s] + (long long)k * kSlice + l] = make_double2(0.0, 0.0);
    }
    for (int k = 0; k < wr[s]; k++) {
        col_r[pr[s] + (long long)k * kSlice + l] = row;
        val_r[pr[s] + (long long)k * kSlice + l] = 0.0;
    }
}

__device__ inline long long slot(const long long *p, int row, int k)
{
    return p[row / kSlice] + (long long)k * kSlice + (row % kSlice);
}

__global__ void k_fill(int nb, const int *__restrict__ ig, const int *__restrict__ jg,
                       const int *__restrict__ idi, const int *__restrict__ ijg,
                       const double *__restrict__ di, const double *__restrict__ gg,
                       const long long *pc, const long long *pr, int *fill_c, int *fill_r,
                       int *col_c, double2 *val_c, int *col_r, double *val_r)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    {
        const int k = atomicAdd(&fill_c[i], 1);
        const long long t = slot(pc, i, k);
        col_c[t] = i;
        val_c[t] = make_double2(di[idi[i]], idi[i + 1] - idi[i] == 2 ? di[idi[i] + 1] : 0.0);
    }
    for (int q = ig[i]; q < ig[i + 1]; q++) {
        const int j = jg[q];
        const int b = ijg[q];
        if (ijg[q + 1] - b == 2) {
            const double2 v = make_double2(gg[b], gg[b + 1]);
            long long t = slot(pc, i, atomicAdd(&fill_c[i], 1));
            col_c[t] = j;
            val_c[t] = v;
            t = slot(pc, j, atomicAdd(&fill_c[j], 1));
            col_c[t] = i;
            val_c[t] = v;
        } else {
            const double v = gg[b];
            long long t = slot(pr, i, atomicAdd(&fill_r[i], 1));
            col_r[t] = j;
            val_r[t] = v;
            t = slot(pr, j, atomicAdd(&fill_r[j], 1));
            col_r[t] = i;
            val_r[t] = v;
        }
    }
}

// sort every row's slots by column (insertion sort, rows are short) and
// record the diagonal's complex slot
__global__ void k_sort(int nb, const int *cnt_c, const int *cnt_r, const long long *pc,
                       const long long *pr, int *col_c, double2 *val_c, int *col_r,
                       double *val_r, int *diag_slot)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const int nc = cnt_c[i], nr = cnt_r[i];
    for (int a = 1; a < nc; a++) {
        const long long ta = slot(pc, i, a);
        const int c = col_c[ta];
        const double2 v = val_c[ta];
        int b = a - 1;
        while (b >= 0 && col_c[slot(pc, i, b)] > c) {
            col_c[slot(pc, i, b + 1)] = col_c[slot(pc, i, b)];
            val_c[slot(pc, i, b + 1)] = val_c[slot(pc, i, b)];
            b--;
        }
        col_c[slot(pc, i, b + 1)] = c;
        val_c[slot(pc, i, b + 1)] = v;
    }
    for (int a = 1; a < nr; a++) {
        const long long ta = slot(pr, i, a);
        const int c = col_r[ta];
        const double v = val_r[ta];
        int b = a - 1;
        while (b >= 0 && col_r[slot(pr, i, b)] > c) {
            col_r[slot(pr, i, b + 1)] = col_r[slot(pr, i, b)];
            val_r[slot(pr, i, b + 1)] = val_r[slot(pr, i, b)];
            b--;
        }
        col_r[slot(pr, i, b + 1)] = c;
        val_r[slot(pr, i, b + 1)] = v;
    }
    int d = -1;
    for (int a = 0; a < nc; a++)
        if (col_c[slot(pc, i, a)] == i) d = a;
    diag_slot[i] = d;
}

}  // namespace

int sell_from_block2x2_device(int nb, const int *d_ig, const int *d_jg, const int *d_idi,
                              const int *d_ijg, const double *d_di, const double *d_gg,
                              int nnz_lower, SellMatrix &A, cudaStream_t st)
{
    (void)nnz_lower;
    MTGPU_CHECK_ARG(nb > 0, "number of edges must be positive");
    A.release();
    A.nb = nb;
    A.nslices = ceil_div(nb, kSlice);
    int *fill_c = nullptr, *fill_r = nullptr;
    unsigned long long *tot = nullptr;
    int rc;
    if ((rc = dev_alloc(&A.d_nc, nb)) || (rc = dev_alloc(&A.d_nr, nb)) ||
        (rc = dev_alloc(&fill_c, nb)) || (rc = dev_alloc(&fill_r, nb)) ||
        (rc = dev_alloc(&tot, 2)) || (rc = dev_alloc(&A.d_wc, A.nslices)) ||
        (rc = dev_alloc(&A.d_wr, A.nslices)) || (rc = dev_alloc(&A.d_pc, A.nslices + 1)) ||
        (rc = dev_alloc(&A.d_pr, A.nslices + 1)) || (rc = dev_alloc(&A.d_diag_slot, nb)))
        return rc;
    int *cnt_c = A.d_nc, *cnt_r = A.d_nr;
    MTGPU_TRY(cudaMemsetAsync(cnt_c, 0, sizeof(int) * nb, st));
    MTGPU_TRY(cudaMemsetAsync(cnt_r, 0, sizeof(int) * nb, st));
    MTGPU_TRY(cudaMemsetAsync(fill_c, 0, sizeof(int) * nb, st));
    MTGPU_TRY(cudaMemsetAsync(fill_r, 0, sizeof(int) * nb, st));
    MTGPU_TRY(cudaMemsetAsync(tot, 0, sizeof(unsigned long long) * 2, st));
    k_count<<<ceil_div(nb, kThreads), kThreads, 0, st>>>(nb, d_ig, d_jg, d_ijg, cnt_c, cnt_r);
    k_widths<<<ceil_div(A.nslices, kThreads), kThreads, 0, st>>>(nb, A.nslices, cnt_c, cnt_r,
                                                                  A.d_wc, A.d_wr, tot);
    MTGPU_TRY(cudaGetLastError());
    std::vector<int> wc(A.nslices), wr(A.nslices);
    unsigned long long htot[2];
    MTGPU_TRY(cudaMemcpyAsync(wc.data(), A.d_wc, sizeof(int) * A.nslices, cudaMemcpyDeviceToHost, st));
    MTGPU_TRY(cudaMemcpyAsync(wr.data(), A.d_wr, sizeof(int) * A.nslices, cudaMemcpyDeviceToHost, st));
    MTGPU_TRY(cudaMemcpyAsync(htot, tot, sizeof(htot), cudaMemcpyDeviceToHost, st));
    MTGPU_TRY(cudaStreamSynchronize(st));
    std::vector<long long> pc(A.nslices + 1), pr(A.nslices + 1);
    pc[0] = pr[0] = 0;
    for (int s = 0; s < A.nslices; s++) {
        pc[s + 1] = pc[s] + (long long)wc[s] * kSlice;
        pr[s + 1] = pr[s] + (long long)wr[s] * kSlice;
    }
    A.len_c = pc[A.nslices];
    A.len_r = pr[A.nslices];
    A.nnz_c = (long long)htot[0];
    A.nnz_r = (long long)htot[1];
    MTGPU_TRY(cudaMemcpyAsync(A.d_pc, pc.data(), sizeof(long long) * (A.nslices + 1),
                              cudaMemcpyHostToDevice, st));
    MTGPU_TRY(cudaMemcpyAsync(A.d_pr, pr.data(), sizeof(long long) * (A.nslices + 1),
                              cudaMemcpyHostToDevice, st));
    if ((rc = dev_alloc(&A.d_col_c, A.len_c)) || (rc = dev_alloc(&A.d_val_c, A.len_c)) ||
        (rc = dev_alloc(&A.d_col_r, A.len_r)) || (rc = dev_alloc(&A.d_val_r, A.len_r)))
        return rc;
    k_pad<<<ceil_div((long long)A.nslices * kSlice, kThreads), kThreads, 0, st>>>(
        nb, A.nslices, A.d_wc, A.d_wr, A.d_pc, A.d_pr, A.d_col_c, A.d_val_c, A.d_col_r,
        A.d_val_r);
    k_fill<<<ceil_div(nb, kThreads), kThreads, 0, st>>>(nb, d_ig, d_jg, d_idi, d_ijg, d_di,
                                                        d_gg, A.d_pc, A.d_pr, fill_c, fill_r,
                                                        A.d_col_c, A.d_val_c, A.d_col_r,
                                                        A.d_val_r);
    k_sort<<<ceil_div(nb, kThreads), kThreads, 0, st>>>(nb, cnt_c, cnt_r, A.d_pc, A.d_pr,
                                                        A.d_col_c, A.d_val_c, A.d_col_r,
                                                        A.d_val_r, A.d_diag_slot);
    MTGPU_TRY(cudaGetLastError());
    MTGPU_TRY(cudaStreamSynchronize(st));
    dev_free(fill_c); dev_free(fill_r); dev_free(tot);
    return MTGPU_OK;
}

// ------------------------------------------------------------------ SpMV
// One thread per row; complex slots then real slots, both in column order.
template <bool kResidual>
__global__ void __launch_bounds__(kThreads)
k_spmv(int nb, const int *__restrict__ wc, const int *__restrict__ wr,
       const long long *__restrict__ pc, const long long *__restrict__ pr,
       const int *__restrict__ col_c, const double2 *__restrict__ val_c,
       const int *__restrict__ col_r, const double *__restrict__ val_r,
       const double2 *__restrict__ x, const double2 *__restrict__ b, double2 *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const int s = i / kSlice, l = i % kSlice;
    double ar = 0.0, ai = 0.0;
    {
        const long long base = pc[s] + l;
        const int w = wc[s];
#pragma unroll 4
        for (int k = 0; k < w; k++) {
            const double2 v = val_c[base + (long long)k * kSlice];
            const double2 xv = x[col_c[base + (long long)k * kSlice]];
            ar += v.x * xv.x - v.y * xv.y;
            ai += v.x * xv.y + v.y * xv.x;
        }
    }
    {
        const long long base = pr[s] + l;
        const int w = wr[s];
#pragma unroll 8
        for (int k = 0; k < w; k++) {
            const double v = val_r[base + (long long)k * kSlice];
            const double2 xv = x[col_r[base + (long long)k * kSlice]];
            ar += v * xv.x;
            ai += v * xv.y;
        }
    }
    if (kResidual) {
        const double2 bv = b[i];
        y[i] = make_double2(bv.x - ar, bv.y - ai);
    } else {
        y[i] = make_double2(ar, ai);
    }
}

void sell_spmv(const SellMatrix &A, const double2 *x, double2 *y, cudaStream_t st)
{
    k_spmv<false><<<ceil_div(A.nb, kThreads), kThreads, 0, st>>>(
        A.nb, A.d_wc, A.d_wr, A.d_pc, A.d_pr, A.d_col_c, A.d_val_c, A.d_col_r, A.d_val_r, x,
        nullptr, y);
}

void sell_residual(const SellMatrix &A, const double2 *b, const double2 *x, double2 *y,
                   cudaStream_t st)
{
    k_spmv<true><<<ceil_div(A.nb, kThreads), kThreads, 0, st>>>(
        A.nb, A.d_wc, A.d_wr, A.d_pc, A.d_pr, A.d_col_c, A.d_val_c, A.d_col_r, A.d_val_r, x, b,
        y);
}

}  // namespace mtgpu
