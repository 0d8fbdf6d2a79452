// Mesh tables of a regular (tensor-product) hexahedral mesh generated on
// the device from its node lines, for the device assembly.
//
// The numbering is RegularMeshBuilder's (Code/RegularMeshBuilder/main.cpp):
// nodes x fastest, then y, then z; cells likewise with the reference's local
// node order (n0, n0+1, n0+nx, n0+nx+1, then the same one plane up); edges
// numbered by node, each node's +x, +y, +z edge in that order where present
// (the lexicographic (n1 < n2) order of the std::set the builder fills at
// :923-1032); the 12 edges of a cell in the reference's local order (4 x,
// 4 y, 4 z: mesh.py cell_edges); every node of the outer surface Dirichlet
// (:1706-1736).  The first edge of node (i, j, k) has a closed form, so every
// table is one pass of lattice arithmetic and none crosses PCIe.
#include "assemble.cuh"

namespace mtgpu {
namespace {

struct Lattice {
    int nx, ny, nz;
    // first edge of node (i, j, k): the planes below, the lines before, the
    // nodes before on the line (3 edges each where all three exist)
    __device__ __forceinline__ int first_edge(int i, int j, int k) const
    {
        const int plane = (ny - 1) * (3 * nx - 1) + (2 * nx - 1);
        const int line = k < nz - 1 ? 3 * nx - 1 : 2 * nx - 1;
        return k * plane + j * line + i * (1 + (j < ny - 1) + (k < nz - 1));
    }
    // the +d edge of node (i, j, k), -1 if absent
    __device__ __forceinline__ int edge(int d, int i, int j, int k) const
    {
        const int hx = i < nx - 1, hy = j < ny - 1, hz = k < nz - 1;
        const int e = first_edge(i, j, k);
        if (d == 0) return hx ? e : -1;
        if (d == 1) return hy ? e + hx : -1;
        return hz ? e + hx + hy : -1;
    }
};

__global__ void k_reg_nodes(Lattice L, const double *__restrict__ x, const double *__restrict__ y,
                            const double *__restrict__ z, double *xyz, unsigned char *bnode)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nn = (long long)L.nx * L.ny * L.nz;
    if (n >= nn) return;
    const int i = (int)(n % L.nx), j = (int)((n / L.nx) % L.ny), k = (int)(n / ((long long)L.nx * L.ny));
    xyz[3 * n] = x[i];
    xyz[3 * n + 1] = y[j];
    xyz[3 * n + 2] = z[k];
    bnode[n] = i == 0 || j == 0 || k == 0 || i == L.nx - 1 || j == L.ny - 1 || k == L.nz - 1;
}

__global__ void k_reg_edges(Lattice L, int *edges)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nn = (long long)L.nx * L.ny * L.nz;
    if (n >= nn) return;
    const int i = (int)(n % L.nx), j = (int)((n / L.nx) % L.ny), k = (int)(n / ((long long)L.nx * L.ny));
    const int step[3] = {1, L.nx, L.nx * L.ny};
    for (int d = 0; d < 3; d++) {
        const int e = L.edge(d, i, j, k);
        if (e < 0) continue;
        edges[2 * e] = (int)n;
        edges[2 * e + 1] = (int)n + step[d];
    }
}

__global__ void k_reg_cells(Lattice L, int *nver, int *ed)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int cx = L.nx - 1, cy = L.ny - 1;
    const long long nc = (long long)cx * cy * (L.nz - 1);
    if (c >= nc) return;
    const int i = (int)(c % cx), j = (int)((c / cx) % cy), k = (int)(c / ((long long)cx * cy));
    const int nx = L.nx, nxy = L.nx * L.ny;
    const int n0 = (k * L.ny + j) * nx + i;
    int *v = nver + 8 * c;
    v[0] = n0; v[1] = n0 + 1; v[2] = n0 + nx; v[3] = n0 + nx + 1;
    v[4] = n0 + nxy; v[5] = n0 + nxy + 1; v[6] = n0 + nxy + nx; v[7] = n0 + nxy + nx + 1;
    int *q = ed + 12 * c;
    q[0] = L.edge(0, i, j, k);      q[1] = L.edge(0, i, j + 1, k);
    q[2] = L.edge(0, i, j, k + 1);  q[3] = L.edge(0, i, j + 1, k + 1);
    q[4] = L.edge(1, i, j, k);      q[5] = L.edge(1, i, j, k + 1);
    q[6] = L.edge(1, i + 1, j, k);  q[7] = L.edge(1, i + 1, j, k + 1);
    q[8] = L.edge(2, i, j, k);      q[9] = L.edge(2, i + 1, j, k);
    q[10] = L.edge(2, i, j + 1, k); q[11] = L.edge(2, i + 1, j + 1, k);
}

}  // namespace

int param_assemble_regular(int nx, int ny, int nz, const double *x, const double *y,
                           const double *z, const int *cell_material, int n_materials,
                           const double *mu, const double *sigma, const double *sigma0,
                           ParamMatrix &P, cudaStream_t st)
{
    P.release();
    MTGPU_CHECK_ARG(nx >= 2 && ny >= 2 && nz >= 2, "a regular mesh needs two lines per axis");
    MTGPU_CHECK_ARG(x && y && z && cell_material && mu && sigma && sigma0, "null argument");
    for (int i = 1; i < nx; i++) MTGPU_CHECK_ARG(x[i] > x[i - 1], "x lines must ascend");
    for (int i = 1; i < ny; i++) MTGPU_CHECK_ARG(y[i] > y[i - 1], "y lines must ascend");
    for (int i = 1; i < nz; i++) MTGPU_CHECK_ARG(z[i] > z[i - 1], "z lines must ascend");
    const long long kuz = (long long)nx * ny * nz, kpar = (long long)(nx - 1) * (ny - 1) * (nz - 1);
    const long long nb = (long long)(nx - 1) * ny * nz + (long long)nx * (ny - 1) * nz +
                         (long long)nx * ny * (nz - 1);
    MTGPU_CHECK_ARG(2 * nb < (1LL << 31) && 12 * kpar < (1LL << 31) && 3 * kuz < (1LL << 31),
                    "mesh too large for 32-bit tables");
    MTGPU_CHECK_ARG(n_materials > 0, "no materials");
    for (long long c = 0; c < kpar; c++)
        MTGPU_CHECK_ARG(cell_material[c] >= 0 && cell_material[c] < n_materials,
                        "cell material out of range");
    for (int i = 0; i < n_materials; i++) MTGPU_CHECK_ARG(mu[i] > 0.0, "mu must be positive");
    P.nb = (int)nb;
    P.kpar = (int)kpar;
    P.kuzlov = (int)kuz;
    P.n_materials = n_materials;
    P.ed_stride = 12;
    P.nver_stride = 8;
    P.nslices = ceil_div(P.nb, kSlice);
    double *d_x = nullptr, *d_y = nullptr, *d_z = nullptr;
    unsigned char *bnode = nullptr;
    int rc;
    auto done = [&](int code) {
        dev_free(d_x); dev_free(d_y); dev_free(d_z); dev_free(bnode);
        return code;
    };
    if ((rc = dev_alloc(&d_x, nx)) || (rc = dev_alloc(&d_y, ny)) || (rc = dev_alloc(&d_z, nz)) ||
        (rc = dev_alloc(&bnode, kuz)) || (rc = dev_alloc(&P.d_xyz, 3 * kuz)) ||
        (rc = dev_alloc(&P.d_nver, 8 * kpar)) || (rc = dev_alloc(&P.d_ed, 12 * kpar)) ||
        (rc = dev_alloc(&P.d_edges, 2 * nb)) || (rc = dev_alloc(&P.d_nvkat, kpar)) ||
        (rc = dev_alloc(&P.d_mu, n_materials)) || (rc = dev_alloc(&P.d_sig, n_materials)) ||
        (rc = dev_alloc(&P.d_sig0, n_materials)))
        return done(rc);
    cudaError_t e = cudaSuccess;
    auto up = [&](void *d, const void *h, size_t bytes) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st);
    };
    up(d_x, x, sizeof(double) * nx);
    up(d_y, y, sizeof(double) * ny);
    up(d_z, z, sizeof(double) * nz);
    up(P.d_nvkat, cell_material, sizeof(int) * kpar);
    up(P.d_mu, mu, sizeof(double) * n_materials);
    up(P.d_sig, sigma, sizeof(double) * n_materials);
    up(P.d_sig0, sigma0, sizeof(double) * n_materials);
    if (e != cudaSuccess) {
        set_last_error(e, "param_assemble_regular upload", __FILE__, __LINE__);
        return done(MTGPU_ERR_CUDA);
    }
    const Lattice L{nx, ny, nz};
    const unsigned gn = (unsigned)((kuz + kThreads - 1) / kThreads);
    const unsigned gc = (unsigned)((kpar + kThreads - 1) / kThreads);
    k_reg_nodes<<<gn, kThreads, 0, st>>>(L, d_x, d_y, d_z, P.d_xyz, bnode);
    k_reg_edges<<<gn, kThreads, 0, st>>>(L, P.d_edges);
    k_reg_cells<<<gc, kThreads, 0, st>>>(L, P.d_nver, P.d_ed);
    note_launches(3);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(e, "param_assemble_regular tables", __FILE__, __LINE__);
        return done(MTGPU_ERR_CUDA);
    }
    rc = param_build(P, bnode, st);
    P.d_bnode = bnode;   // kept for the solver set-up (preconditioner, matrix-free tables)
    bnode = nullptr;
    return done(rc);
}

}  // namespace mtgpu
