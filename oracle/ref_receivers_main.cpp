// Harness around the reference's own receiver evaluation (direct path):
// OutputVect3d::OutputFieldAtReceivers, Code/OutputNu/OutputArbitrary.cpp:202-293,
// which locates every receiver in its element (FindElemForReceivers, :385-500)
// and evaluates T_Brick::VectorFieldOnPar / RotXOnPar / RotYOnPar / RotZOnPar
// (Code/OutputNu/T_Brick.cpp:1842-1918, 2133-2149).
//
// Test infrastructure only: compiled by oracle/build_ref.sh together with the
// reference sources, run by tests/golden/make_golden_receivers.py to pin the
// C restatement.  The product never links or runs it.
//
// stdin-free; usage: ref_receivers IN OUT
//   IN  (little-endian): int32 kuzlov, kpar, nb, nrec; f64 xyz[kuzlov][3];
//       int32 nver[kpar][14] (0-based); int32 ed[kpar][25] (0-based);
//       f64 rec[nrec][3]; f64 v3[nb][2] (re, im interleaved)
//   OUT f64 [2][6][nrec]: part (0 = re "sin", 1 = im "cos") x derive
//       (0 Ax, 1 Ay, 2 Az, 3 curl_z, 4 curl_x, 5 curl_y)
#include "stdafx.h"
#include "OutputArbitrary.h"

#include <cstdio>
#include <vector>

ofstream logfile;

static bool read_all(FILE *f, void *p, size_t bytes)
{
    return fread(p, 1, bytes, f) == bytes;
}

int main(int argc, char **argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s IN OUT\n", argv[0]);
        return 2;
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 3;
    int hdr[4];
    if (!read_all(f, hdr, sizeof hdr)) return 4;
    const long kuzlov = hdr[0], kpar = hdr[1], nb = hdr[2], nrec = hdr[3];
    std::vector<double> xyz(3 * kuzlov), rec(3 * nrec), v3(2 * nb);
    std::vector<int> nver32(14 * kpar), ed32(25 * kpar);
    if (!read_all(f, xyz.data(), 8 * xyz.size()) || !read_all(f, nver32.data(), 4 * nver32.size()) ||
        !read_all(f, ed32.data(), 4 * ed32.size()) || !read_all(f, rec.data(), 8 * rec.size()) ||
        !read_all(f, v3.data(), 8 * v3.size()))
        return 4;
    fclose(f);

    // the reference's element tables are arrays of `long`
    std::vector<long> nver(nver32.begin(), nver32.end()), ed(ed32.begin(), ed32.end());
    logfile.open("/dev/null");
    OutputVect3d out(0, 0, 0, kuzlov, kpar, nb, nrec, (double(*)[3])rec.data(),
                     (double(*)[3])xyz.data(), (long(*)[14])nver.data(), (long(*)[25])ed.data());

    std::vector<double> part(nb), res((size_t)2 * 6 * nrec, 0.0);
    for (int p = 0; p < 2; p++) {
        for (long i = 0; i < nb; i++) part[i] = v3[2 * i + p];
        for (int d = 0; d < 6; d++)
            out.OutputFieldAtReceivers(part.data(), &res[((size_t)p * 6 + d) * nrec], d);
    }
    FILE *g = fopen(argv[2], "wb");
    if (!g) return 5;
    fwrite(res.data(), 8, res.size(), g);
    fclose(g);
    return 0;
}
