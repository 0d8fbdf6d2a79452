// Tiled matrix-free SpMV of tensor meshes (SpMV variant 34), included by
// survey.cu after the matrix-free helpers (MF, Pos, SpmvTail).
//
// The operator is the one of k_mf_faces + k_mf_edges: A s = D^T F D s +
// i omega M s from six weights per cell.  Instead of writing every face
// circulation to global memory and gathering it back, a block owns a tile of
// TX x TY node columns and marches along z through a chunk of node planes.
// Per plane it stages in shared memory the edge values of the tile plus a
// one-node halo (the x- and y-edges of three planes, the z-edges of two
// layers), computes the face circulations it needs from them (z-faces of
// three planes, x- and y-faces of two layers; rings indexed by plane
// number), and then produces the rows of its own nodes' three edges.  Every
// edge value crosses HBM once per launch (plus the halo, an L2 hit), and no
// face value leaves the SM.
//
// The face sums and the row sums are accumulated in exactly the order of
// k_mf_faces / mf_row, so the result equals variant 32's bit for bit.
//
// Dirichlet edges (both nodes on the outer surface) enter the sums as 0 and
// their rows return s itself, as in the assembled matrix.  On a tensor mesh
// whose outer nodes are exactly the Dirichlet nodes this is the lattice rule
// "an x-edge is Dirichlet iff its node line has j or k on the surface"
// (likewise for y and z); the set-up enables the variant only when the
// mesh's Dirichlet edges follow it.

// systems per block: 2 (one 32-byte sector per edge) when the layout holds
// two or more, else 1; tile TX x TY node columns, one thread per
// (column, system of the block), one block per SM.  Shared arrays are
// system-major ([ring][system][slot]) so that a warp (32 columns of one
// system) reads nearly consecutive 16-byte slots.  The tile's shape is fitted
// to the mesh at set-up (at most TX x TY columns, its halo frame at most NS
// slots): c2's 97 node columns become 4 tiles of 25, not 3 of 32 and one of 1.  The x/y-edge ring holds four
// planes and the z-edge ring three layers: the copies of plane k + 2 are in
// flight (cp.async, zero-filled where an edge is absent or Dirichlet) while
// the faces of plane k + 1 and the rows of plane k are computed.
template <int SP>
struct MfTile {
    static constexpr int SB = SP >= 2 ? 2 : 1;
    static constexpr int TX = 32;
    static constexpr int TY = SB == 1 ? 16 : 8;
    static constexpr int NT = TX * TY * SB;
    static constexpr int NX = TX + 2, NY = TY + 2, NS = NX * NY;   // halo frame
    static constexpr int OFF_EXY = 0;                              // [4][2][SB][NS]
    static constexpr int OFF_EZ = OFF_EXY + 4 * 2 * SB * NS;       // [3][SB][NS]
    static constexpr int OFF_FZ = OFF_EZ + 3 * SB * NS;            // [3][SB][NS]
    static constexpr int OFF_FX = OFF_FZ + 3 * SB * NS;            // [2][SB][NS]
    static constexpr int OFF_FY = OFF_FX + 2 * SB * NS;            // [2][SB][NS]
    static constexpr int SLOTS = OFF_FY + 2 * SB * NS;
    static constexpr int SMEM = SLOTS * 16;   // the reduction staging reuses it at the end
    static_assert(NT * 2 * 8 <= SMEM, "staging fits");
};

// asynchronous 16-byte copy global -> shared; valid = false writes zeros
// (source size 0: nothing is read)
__device__ __forceinline__ void cp_async16_zfill(void *smem_dst, const void *gsrc, bool valid)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    const int n = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gsrc), "r"(n)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

struct MfTileGrid {
    int tiles_x, tiles_y, zchunks, groups, kz;   // kz planes per chunk
    int tx, ty;   // node columns of a tile: tx * ty <= TX * TY, (tx + 2) (ty + 2) <= NS
};

__device__ __forceinline__ float4 f4zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }

// the same sum as k_mf_faces: a + b - c - d, in that order
__device__ __forceinline__ float4 face_sum(float4 a, float4 b, float4 c, float4 d)
{
    acc fr, fi;
    fr.add(df{a.x, a.y}); fr.add(df{b.x, b.y}); fr.add(neg(df{c.x, c.y})); fr.add(neg(df{d.x, d.y}));
    fi.add(df{a.z, a.w}); fi.add(df{b.z, b.w}); fi.add(neg(df{c.z, c.w})); fi.add(neg(df{d.z, d.w}));
    return to4(dfc{fr.get(), fi.get()});
}

// one face group of mf_row: sg (wa fm + 2 (wa + wb) f0 + wb fp) into kr, ki
__device__ __forceinline__ void mf_group(acc &kr, acc &ki, df wa, df wb, float sg, float4 fm4,
                                         float4 f04, float4 fp4)
{
    const dfc fm = from4(fm4), f0 = from4(f04), fp = from4(fp4);
    const df ca = scale(wa, sg), cb = scale(wb, sg), c0 = scale(add(wa, wb), 2.f * sg);
    kr.mac(ca, fm.re); kr.mac(c0, f0.re); kr.mac(cb, fp.re);
    ki.mac(ca, fm.im); ki.mac(c0, f0.im); ki.mac(cb, fp.im);
}

// mass part of mf_row from the 4 cell weights wm[a][b] and the 3 x 3 parallel
// edges xe[A][B] (A along T1, B along T2), then y = K s + i omega M s
__device__ __forceinline__ dfc mf_mass(acc &kr, acc &ki, const df (&wm)[2][2],
                                       const float4 (&xe)[3][3], df om)
{
    acc mr, mi;
    const df s0_ = add(wm[0][0], wm[0][1]), s1_ = add(wm[1][0], wm[1][1]);
    const df r0_ = add(wm[0][0], wm[1][0]), r1_ = add(wm[0][1], wm[1][1]);
    const df cm[3][3] = {{wm[0][0], scale(s0_, 2.f), wm[0][1]},
                         {scale(r0_, 2.f), scale(add(s0_, s1_), 4.f), scale(r1_, 2.f)},
                         {wm[1][0], scale(s1_, 2.f), wm[1][1]}};
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const dfc x = from4(xe[a][b]);
            mr.mac(cm[a][b], x.re);
            mi.mac(cm[a][b], x.im);
        }
    const df mxr = mr.get(), mxi = mi.get();
    kr.mac(neg(om), mxi);
    ki.mac(om, mxr);
    return dfc{kr.get(), ki.get()};
}

template <int SP>
__global__ void __launch_bounds__(MfTile<SP>::NT, 1)
k_mf_tile(MF M, MfTileGrid G, const float2 *__restrict__ omega, const float4 *__restrict__ s,
          float4 *__restrict__ z,
          SysState *sys, double *partials, int mode)
{
    pdl_wait();
    using C = MfTile<SP>;
    constexpr int SB = C::SB, NT = C::NT, NS = C::NS;   // NS: the plane stride of the rings
    // this mesh's tile: TX x TY columns, halo frame NX x (TY + 2)
    const int TX = G.tx, TY = G.ty, NX = TX + 2, NF = NX * (TY + 2);
    extern __shared__ __align__(16) float4 sh[];
    float4 *const EXY = sh + C::OFF_EXY, *const EZ = sh + C::OFF_EZ, *const FZ = sh + C::OFF_FZ,
                 *const FX = sh + C::OFF_FX, *const FY = sh + C::OFF_FY;
    // rings by plane / layer number p >= -1
    auto at4 = [](int p) { return (p + 4) & 3; };
    auto at3 = [](int p) { return (p + 3) % 3; };
    auto at2 = [](int p) { return (p + 2) & 1; };
    auto exy = [&](int pl, int d, int ii, int jj, int u) -> float4 & {
        return EXY[((at4(pl) * 2 + d) * SB + u) * NS + jj * NX + ii];
    };
    auto ezs = [&](int ly, int ii, int jj, int u) -> float4 & {
        return EZ[(at3(ly) * SB + u) * NS + jj * NX + ii];
    };
    auto fz = [&](int pl, int ii, int jj, int u) -> float4 & {
        return FZ[(at3(pl) * SB + u) * NS + jj * NX + ii];
    };
    auto fx = [&](int ly, int ii, int jj, int u) -> float4 & {
        return FX[(at2(ly) * SB + u) * NS + jj * NX + ii];
    };
    auto fy = [&](int ly, int ii, int jj, int u) -> float4 & {
        return FY[(at2(ly) * SB + u) * NS + jj * NX + ii];
    };

    int b = blockIdx.x;
    const int grp = b % G.groups;
    b /= G.groups;
    const int tx = b % G.tiles_x;
    b /= G.tiles_x;
    const int ty = b % G.tiles_y;
    const int zc = b / G.tiles_y;
    const int i0 = tx * TX, j0 = ty * TY, sys0 = grp * SB;
    const int nx = M.nx, ny = M.ny, nz = M.nz;
    const int k0 = zc * G.kz, k1 = min(k0 + G.kz, nz);
    const int tid = threadIdx.x;
    constexpr int CPS = C::TX * C::TY;   // threads per system of the block
    const int u_me = tid / CPS, cme = tid % CPS, ti = cme % TX, tj = cme / TX;
    const int kme = sys0 + u_me;
    const bool on = sys[kme].status == kRun;
    const df om = d2f(omega[kme]);
    SpmvTail tail;
    const int nc = (int)M.ncell;

    // issue the copies of the edges owned by the nodes of plane P (x, y on
    // P; z of layer P); absent, Dirichlet and out-of-mesh slots become 0
    auto load_plane = [&](int P) {
        for (int q = tid; q < NF * 3 * SB; q += NT) {
            const int u = q % SB, d = (q / SB) % 3, slot = q / (3 * SB);
            const int ii = slot % NX, jj = slot / NX;
            const int i = i0 - 1 + ii, j = j0 - 1 + jj;
            const float4 *src = s;
            bool valid = false;
            if (P >= 0 && P < nz && i >= 0 && i < nx && j >= 0 && j < ny) {
                const int ex = i < nx - 1, ey = j < ny - 1, ezp = P < nz - 1;
                const bool has = d == 0 ? ex : (d == 1 ? ey : ezp);
                const bool dir = d == 0 ? (j == 0 || j == ny - 1 || P == 0 || P == nz - 1)
                               : d == 1 ? (i == 0 || i == nx - 1 || P == 0 || P == nz - 1)
                                        : (i == 0 || i == nx - 1 || j == 0 || j == ny - 1);
                if (has && !dir) {
                    int e = mf_line(M, j, P) + i * (1 + ey + ezp);
                    if (d >= 1) e += ex;
                    if (d == 2) e += ey;
                    src = s + (long long)e * SP + sys0 + u;
                    valid = true;
                }
            }
            cp_async16_zfill(d < 2 ? &exy(P, d, ii, jj, u) : &ezs(P, ii, jj, u), src, valid);
        }
        cp_async_commit();
    };
    // z-faces of plane P: lower corners ii in [0, TX], jj in [0, TY]
    auto faces_z = [&](int P) {
        const int n = (TX + 1) * (TY + 1);
        for (int q = tid; q < n * SB; q += NT) {
            const int u = q / n, c = q % n, ii = c % (TX + 1), jj = c / (TX + 1);
            fz(P, ii, jj, u) = face_sum(exy(P, 0, ii, jj, u), exy(P, 1, ii + 1, jj, u),
                                        exy(P, 0, ii, jj + 1, u), exy(P, 1, ii, jj, u));
        }
    };
    // x-faces (ii in [0, TX+1], jj in [0, TY]) and y-faces (ii in [0, TX],
    // jj in [0, TY+1]) of layer L (between planes L and L+1)
    auto faces_xy = [&](int L) {
        const int n1 = (TX + 2) * (TY + 1), n2 = (TX + 1) * (TY + 2);
        for (int q = tid; q < n1 * SB; q += NT) {
            const int u = q / n1, c = q % n1, ii = c % (TX + 2), jj = c / (TX + 2);
            fx(L, ii, jj, u) = face_sum(exy(L, 1, ii, jj, u), ezs(L, ii, jj + 1, u),
                                        exy(L + 1, 1, ii, jj, u), ezs(L, ii, jj, u));
        }
        for (int q = tid; q < n2 * SB; q += NT) {
            const int u = q / n2, c = q % n2, ii = c % (TX + 1), jj = c / (TX + 1);
            fy(L, ii, jj, u) = face_sum(ezs(L, ii, jj, u), exy(L + 1, 0, ii, jj, u),
                                        ezs(L, ii + 1, jj, u), exy(L, 0, ii, jj, u));
        }
    };
    // weight w (0-2: wF/3 of x, y, z; 3-5: sigma wM/9 of x, y, z) of cell (ci, cj, ck)
    auto wcell = [&](int w, int ci, int cj, int ck) {
        return d2f(__ldg(M.w + (long long)w * nc + (ck * (ny - 1) + cj) * (nx - 1) + ci));
    };

    // prologue: planes k0 - 1, k0 staged (k0 + 1 in flight), z-faces of both,
    // x/y faces of layer k0 - 1
    load_plane(k0 - 1);
    load_plane(k0);
    load_plane(k0 + 1);
    cp_async_wait<1>();
    __syncthreads();
    faces_z(k0 - 1);
    faces_z(k0);
    faces_xy(k0 - 1);
    __syncthreads();

    // this thread's node column in the halo frame
    const int ii = ti + 1, jj = tj + 1;
    const int i = i0 + ti, j = j0 + tj;
    const bool col = cme < TX * TY && i < nx && j < ny;
    for (int k = k0; k < k1; k++) {
        load_plane(k + 2);      // lands in the ring slots of plane k - 2 / layer k - 1
        cp_async_wait<1>();     // plane k + 1 has arrived (this thread's copies)
        __syncthreads();        // ... and everyone's
        faces_z(k + 1);
        faces_xy(k);
        __syncthreads();
        if (col && on) {
            const int ex = i < nx - 1, ey = j < ny - 1, ezp = k < nz - 1;
            const int base = mf_line(M, j, k) + i * (1 + ey + ezp);
            // x-edge (D = 0, T1 = y, T2 = z)
            if (ex) {
                const long long idx = (long long)base * SP + kme;
                const float4 sv4 = __ldg(s + idx);
                dfc y;
                if (j == 0 || j == ny - 1 || k == 0 || k == nz - 1) {
                    y = from4(sv4);
                } else {
                    df w1[2][2], w2[2][2], wm[2][2];
#pragma unroll
                    for (int a = 0; a < 2; a++)
#pragma unroll
                        for (int bb = 0; bb < 2; bb++) {
                            w1[a][bb] = wcell(1, i, j - 1 + a, k - 1 + bb);
                            w2[a][bb] = wcell(2, i, j - 1 + a, k - 1 + bb);
                            wm[a][bb] = wcell(3, i, j - 1 + a, k - 1 + bb);
                        }
                    acc kr, ki;
#pragma unroll
                    for (int bb = 0; bb < 2; bb++)   // y-faces of layers k - 1, k
                        mf_group(kr, ki, w1[0][bb], w1[1][bb], bb == 0 ? 1.f : -1.f,
                                 fy(k - 1 + bb, ii, jj - 1, u_me), fy(k - 1 + bb, ii, jj, u_me),
                                 fy(k - 1 + bb, ii, jj + 1, u_me));
#pragma unroll
                    for (int a = 0; a < 2; a++)      // z-faces of planes k - 1 .. k + 1
                        mf_group(kr, ki, w2[a][0], w2[a][1], a == 0 ? -1.f : 1.f,
                                 fz(k - 1, ii, jj - 1 + a, u_me), fz(k, ii, jj - 1 + a, u_me),
                                 fz(k + 1, ii, jj - 1 + a, u_me));
                    float4 xe[3][3];
#pragma unroll
                    for (int A = 0; A < 3; A++)
#pragma unroll
                        for (int B = 0; B < 3; B++) xe[A][B] = exy(k - 1 + B, 0, ii, jj - 1 + A, u_me);
                    y = mf_mass(kr, ki, wm, xe, om);
                }
                tail.row(idx, y, sv4, z);
            }
            // y-edge (D = 1, T1 = z, T2 = x)
            if (ey) {
                const long long idx = (long long)(base + ex) * SP + kme;
                const float4 sv4 = __ldg(s + idx);
                dfc y;
                if (i == 0 || i == nx - 1 || k == 0 || k == nz - 1) {
                    y = from4(sv4);
                } else {
                    df w1[2][2], w2[2][2], wm[2][2];
#pragma unroll
                    for (int a = 0; a < 2; a++)
#pragma unroll
                        for (int bb = 0; bb < 2; bb++) {
                            // offsets a - 1 along T1 = z, bb - 1 along T2 = x
                            w1[a][bb] = wcell(2, i - 1 + bb, j, k - 1 + a);
                            w2[a][bb] = wcell(0, i - 1 + bb, j, k - 1 + a);
                            wm[a][bb] = wcell(4, i - 1 + bb, j, k - 1 + a);
                        }
                    acc kr, ki;
#pragma unroll
                    for (int bb = 0; bb < 2; bb++)   // z-faces of planes k - 1 .. k + 1
                        mf_group(kr, ki, w1[0][bb], w1[1][bb], bb == 0 ? 1.f : -1.f,
                                 fz(k - 1, ii - 1 + bb, jj, u_me), fz(k, ii - 1 + bb, jj, u_me),
                                 fz(k + 1, ii - 1 + bb, jj, u_me));
#pragma unroll
                    for (int a = 0; a < 2; a++)      // x-faces of layers k - 1, k
                        mf_group(kr, ki, w2[a][0], w2[a][1], a == 0 ? -1.f : 1.f,
                                 fx(k - 1 + a, ii - 1, jj, u_me), fx(k - 1 + a, ii, jj, u_me),
                                 fx(k - 1 + a, ii + 1, jj, u_me));
                    float4 xe[3][3];
#pragma unroll
                    for (int A = 0; A < 3; A++)
#pragma unroll
                        for (int B = 0; B < 3; B++) xe[A][B] = exy(k - 1 + A, 1, ii - 1 + B, jj, u_me);
                    y = mf_mass(kr, ki, wm, xe, om);
                }
                tail.row(idx, y, sv4, z);
            }
            // z-edge of layer k (D = 2, T1 = x, T2 = y)
            if (ezp) {
                const long long idx = (long long)(base + ex + ey) * SP + kme;
                const float4 sv4 = __ldg(s + idx);
                dfc y;
                if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1) {
                    y = from4(sv4);
                } else {
                    df w1[2][2], w2[2][2], wm[2][2];
#pragma unroll
                    for (int a = 0; a < 2; a++)
#pragma unroll
                        for (int bb = 0; bb < 2; bb++) {
                            // offsets a - 1 along T1 = x, bb - 1 along T2 = y
                            w1[a][bb] = wcell(0, i - 1 + a, j - 1 + bb, k);
                            w2[a][bb] = wcell(1, i - 1 + a, j - 1 + bb, k);
                            wm[a][bb] = wcell(5, i - 1 + a, j - 1 + bb, k);
                        }
                    acc kr, ki;
#pragma unroll
                    for (int bb = 0; bb < 2; bb++)   // x-faces of layer k at x - 1 .. x + 1
                        mf_group(kr, ki, w1[0][bb], w1[1][bb], bb == 0 ? 1.f : -1.f,
                                 fx(k, ii - 1, jj - 1 + bb, u_me), fx(k, ii, jj - 1 + bb, u_me),
                                 fx(k, ii + 1, jj - 1 + bb, u_me));
#pragma unroll
                    for (int a = 0; a < 2; a++)      // y-faces of layer k at y - 1 .. y + 1
                        mf_group(kr, ki, w2[a][0], w2[a][1], a == 0 ? -1.f : 1.f,
                                 fy(k, ii - 1 + a, jj - 1, u_me), fy(k, ii - 1 + a, jj, u_me),
                                 fy(k, ii - 1 + a, jj + 1, u_me));
                    float4 xe[3][3];
#pragma unroll
                    for (int A = 0; A < 3; A++)
#pragma unroll
                        for (int B = 0; B < 3; B++) xe[A][B] = ezs(k, ii - 1 + A, jj - 1 + B, u_me);
                    y = mf_mass(kr, ki, wm, xe, om);
                }
                tail.row(idx, y, sv4, z);
            }
        }
        __syncthreads();   // the next plane's copies overwrite ring slots read above
    }
    cp_async_wait<0>();    // copies past the chunk's end, before the staging reuses the rings
    __syncthreads();
    // per-system sums in a fixed order (deterministic): thread t's partials
    // staged, then thread u < SB adds those of its system in thread order
    double *const red = reinterpret_cast<double *>(sh);
    red[tid] = tail.zsr.to_double();
    red[NT + tid] = tail.zsi.to_double();
    __syncthreads();
    double v[2] = {0.0, 0.0};
    if (tid < SP) {
        const int u = tid - sys0;
        if (u >= 0 && u < SB)
            for (int n = 0; n < 2; n++)
                for (int t = u * CPS; t < (u + 1) * CPS; t++) v[n] += red[n * NT + t];
    }
    SpmvTail::finish_v<SP, NT>(v, sys, partials, mode);
}
