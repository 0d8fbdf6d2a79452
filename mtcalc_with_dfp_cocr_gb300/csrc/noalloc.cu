// y = A x on device buffers without any device allocation.
//
// Who needs this: a host program or framework that owns all GPU memory
// through its own pool (a caching allocator that has reserved most of the
// device, or an application that sizes every buffer up front) cannot let a
// library call cudaMalloc/cudaFree: those calls synchronise the whole device,
// stalling the caller's other streams, and they fail once the pool holds the
// memory.  Such a caller keeps the SLAE and the vectors in its own buffers
// and calls mtgpu_mult_mv_block_2x2_noalloc, which uses only the scratch
// below.
//
// The scratch is a file-scope __device__ array: every GPU that loads the
// library holds it (16 MiB) until the process exits, and every call shares
// it.  It receives the upper-triangle contributions A_ij x_i of the lower
// storage; each call clears the part it uses first.  Calls whose kernels
// overlap on the GPU (for example on two streams at once) race on it.
//
// The index arrays live on the device, so the host cannot check them.  The
// kernels do: arrays that do not start at 0 (the reference's 1-based files
// passed without subtracting 1) are not read beyond their first element, and
// an entry whose column is not below its row or whose block is neither 1 nor
// 2 doubles is skipped.  Either case sets a bit of the call's status word.
#include "mtgpu_internal.cuh"

#include <mutex>

namespace mtgpu {
namespace {

constexpr int kNoAllocMaxEdges = 1 << 20;   // 1,048,576 edges (16 MiB of scratch)

__device__ __align__(256) double2 g_upper[kNoAllocMaxEdges];
// status of the latest call: MTGPU_NOALLOC_NOT_ZERO_BASED | MTGPU_NOALLOC_BAD_ENTRY
__device__ int g_status;

// device address of g_upper for every device, looked up once per device
std::mutex g_mu;
double2 *g_upper_addr[64] = {nullptr};

int scratch_address(double2 **out)
{
    int dev = 0;
    MTGPU_TRY(cudaGetDevice(&dev));
    MTGPU_CHECK_ARG(dev >= 0 && dev < 64, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_upper_addr[dev]) {
        void *p = nullptr;
        // with `dev` current: the symbol's address on this device
        MTGPU_TRY(cudaGetSymbolAddress(&p, g_upper));
        g_upper_addr[dev] = (double2 *)p;
    }
    *out = g_upper_addr[dev];
    return MTGPU_OK;
}

__global__ void k_na_clear(int nb, double2 *upper)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nb) upper[i] = make_double2(0.0, 0.0);
    if (i == 0) g_status = 0;
}

__device__ __forceinline__ double2 block_times(const double *a, int size, double2 x)
{
    return size == 2 ? make_double2(a[0] * x.x - a[1] * x.y, a[1] * x.x + a[0] * x.y)
                     : make_double2(a[0] * x.x, a[0] * x.y);
}

// row i: y_i = D_i x_i + sum_lower A_ij x_j (stored directly), and the
// mirrored A_ij x_i added into upper[j].  Nothing past the first element of
// an index array is read unless all three start at 0.
__global__ void k_na_rows(int nb, const int *__restrict__ ig, const int *__restrict__ jg,
                          const int *__restrict__ idi, const int *__restrict__ ijg,
                          const double *__restrict__ di, const double *__restrict__ gg,
                          const double2 *__restrict__ x, double2 *__restrict__ y, double2 *upper)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    if (__ldg(ig) != 0 || __ldg(idi) != 0 || __ldg(ijg) != 0) {
        if (i == 0) atomicOr(&g_status, MTGPU_NOALLOC_NOT_ZERO_BASED);
        return;
    }
    const double2 xi = x[i];
    const int d0 = idi[i], dsz = idi[i + 1] - d0;
    double2 acc = make_double2(0.0, 0.0);
    bool bad = false;
    if (dsz == 1 || dsz == 2) acc = block_times(&di[d0], dsz, xi);
    else bad = true;
    const int q0 = ig[i], q1 = ig[i + 1];
    for (int q = q0; q < q1; q++) {
        const int j = jg[q];
        const int a0 = ijg[q], size = ijg[q + 1] - a0;
        if (j < 0 || j >= i || (size != 1 && size != 2)) {
            bad = true;
            continue;
        }
        const double *a = &gg[a0];
        const double2 t = block_times(a, size, x[j]);
        acc.x += t.x;
        acc.y += t.y;
        const double2 u = block_times(a, size, xi);
        atomicAdd(&upper[j].x, u.x);
        atomicAdd(&upper[j].y, u.y);
    }
    if (bad) atomicOr(&g_status, MTGPU_NOALLOC_BAD_ENTRY);
    y[i] = acc;
}

// y += upper; the status word goes to the caller's d_status
__global__ void k_na_add(int nb, const double2 *upper, double2 *y, int *status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int st = *(volatile int *)&g_status;
    if (i == 0 && status) *status = st;
    if (i >= nb || (st & MTGPU_NOALLOC_NOT_ZERO_BASED)) return;
    const double2 u = upper[i];
    double2 v = y[i];
    v.x += u.x;
    v.y += u.y;
    y[i] = v;
}

}  // namespace
}  // namespace mtgpu

using namespace mtgpu;

extern "C" int mtgpu_mult_mv_block_2x2_noalloc(int nb, const int *d_ig, const int *d_jg,
                                               const int *d_idi, const int *d_ijg,
                                               const double *d_di, const double *d_gg,
                                               const double *d_x, double *d_y, int *d_status,
                                               void *stream)
{
    MTGPU_CHECK_ARG(nb > 0, "nb must be positive");
    MTGPU_CHECK_ARG(nb <= kNoAllocMaxEdges,
                    "mtgpu_mult_mv_block_2x2_noalloc handles at most 1048576 edges "
                    "(the size of its static scratch)");
    MTGPU_CHECK_ARG(d_ig && d_jg && d_idi && d_ijg && d_di && d_gg && d_x && d_y,
                    "null device pointer");
    MTGPU_CHECK_ARG(((uintptr_t)d_x % 16) == 0 && ((uintptr_t)d_y % 16) == 0,
                    "x and y must be 16-byte aligned");
    MTGPU_CHECK_ARG(((uintptr_t)d_status % sizeof(int)) == 0, "d_status must be int-aligned");
    double2 *upper = nullptr;
    int rc = scratch_address(&upper);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int blocks = ceil_div(nb, kThreads);
    k_na_clear<<<blocks, kThreads, 0, st>>>(nb, upper);
    k_na_rows<<<blocks, kThreads, 0, st>>>(nb, d_ig, d_jg, d_idi, d_ijg, d_di, d_gg,
                                           (const double2 *)d_x, (double2 *)d_y, upper);
    k_na_add<<<blocks, kThreads, 0, st>>>(nb, upper, (double2 *)d_y, d_status);
    note_launches(3);
    MTGPU_TRY(cudaGetLastError());
    return MTGPU_OK;
}
