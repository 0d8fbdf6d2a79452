// Exclusive prefix sum of an int array on the device, for the set-up
// stages that turn per-row counts into CSR offsets.  Three launches:
// per-tile sums, one block scanning the tile sums (in chunks, with a
// carry), then every tile rescanned with its offset.
#include "mtgpu_internal.cuh"

#include <climits>

namespace mtgpu {
namespace {

constexpr int kScanT = 512;                     // threads per block
constexpr int kScanPer = 8;                     // elements per thread
constexpr int kScanTile = kScanT * kScanPer;    // elements per tile

// exclusive scan of v over the block; *total gets the block's sum
__device__ long long block_exclusive(long long v, long long *total)
{
    __shared__ long long warp_sum[kScanT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        long long w = lane < kScanT / 32 ? warp_sum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanT / 32) warp_sum[lane] = w;   // inclusive over warps
    }
    __syncthreads();
    const long long before = warp == 0 ? 0 : warp_sum[warp - 1];
    *total = warp_sum[kScanT / 32 - 1];
    __syncthreads();   // warp_sum is reused by the next call
    return before + x - v;
}

__global__ void __launch_bounds__(kScanT) k_tile_sums(const int *__restrict__ in, long long n,
                                                      long long *sums)
{
    const long long base = (long long)blockIdx.x * kScanTile;
    long long s = 0;
    for (int q = threadIdx.x; q < kScanTile; q += kScanT) {
        const long long i = base + q;
        if (i < n) s += in[i];
    }
    long long tot;
    block_exclusive(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// one block: sums[0..nt) -> exclusive offsets in place, sums[nt] = total
__global__ void __launch_bounds__(kScanT) k_scan_sums(long long *sums, long long nt)
{
    long long carry = 0;
    for (long long b = 0; b < nt; b += kScanT) {
        const long long i = b + threadIdx.x;
        const long long v = i < nt ? sums[i] : 0;
        long long tot;
        const long long ex = block_exclusive(v, &tot);
        if (i < nt) sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) sums[nt] = carry;
}

__global__ void __launch_bounds__(kScanT) k_scan_tiles(const int *__restrict__ in, long long n,
                                                       const long long *__restrict__ sums, int *out)
{
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanPer;
    int v[kScanPer];
    long long t = 0;
#pragma unroll
    for (int j = 0; j < kScanPer; j++) {
        v[j] = base + j < n ? in[base + j] : 0;
        t += v[j];
    }
    long long tot;
    long long ex = block_exclusive(t, &tot) + sums[blockIdx.x];
#pragma unroll
    for (int j = 0; j < kScanPer; j++) {
        if (base + j < n) out[base + j] = (int)ex;
        ex += v[j];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = (int)sums[gridDim.x];
}

}  // namespace

int dev_exclusive_scan(const int *d_in, long long n, int *d_out, long long *total, cudaStream_t st)
{
    MTGPU_CHECK_ARG(n >= 0, "negative scan length");
    if (n == 0) {
        MTGPU_TRY(cudaMemsetAsync(d_out, 0, sizeof(int), st));
        if (total) *total = 0;
        return MTGPU_OK;
    }
    const long long nt = (n + kScanTile - 1) / kScanTile;
    MTGPU_CHECK_ARG(nt < (1LL << 31), "scan too long");
    long long *sums = nullptr;
    int rc = dev_alloc(&sums, nt + 1);
    if (rc) return rc;
    k_tile_sums<<<(unsigned)nt, kScanT, 0, st>>>(d_in, n, sums);
    k_scan_sums<<<1, kScanT, 0, st>>>(sums, nt);
    k_scan_tiles<<<(unsigned)nt, kScanT, 0, st>>>(d_in, n, sums, d_out);
    note_launches(3);
    cudaError_t e = cudaGetLastError();
    long long tot = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tot, sums + nt, sizeof(long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dev_free(sums);
    if (e != cudaSuccess) {
        set_last_error(e, "dev_exclusive_scan", __FILE__, __LINE__);
        return MTGPU_ERR_CUDA;
    }
    MTGPU_CHECK_ARG(tot < INT_MAX, "scan total exceeds 32-bit offsets");
    if (total) *total = tot;
    return MTGPU_OK;
}

}  // namespace mtgpu
