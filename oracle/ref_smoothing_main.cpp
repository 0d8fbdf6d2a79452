// Harness around the reference's default receiver output: the subdomain
// L2-projection smoothing of Code/OutputNu (OutputResultant3d::Prepare and
// ::Output, OutputResultant3d.cpp:76-199, 293-450; Subdomain::Init,
// ::AsmGlobalMatrix, ::AsmGlobalVector, Subdomain.cpp:132-661), driven the way
// Give_out_vec_mt::Give_out_on_hex drives it (give_out_vec_mt.cpp:200-237):
// one subdomain for curl A (vtWithoutDiscontinuity), one per material for A
// (vtWithDiscontinuity), 5 neighbour levels.  The mesh interface
// (AbstractFEM3D) is implemented here over plain arrays; the element-centre
// values follow Give_out_vec_mt::GetValueInElementCenter
// (give_out_vec_mt.cpp:645-688) through the reference's own T_Brick.  The
// PARDISO solves go to oracle/ref_shim/pardiso_shim.cpp.
//
// Test infrastructure only: built by oracle/build_ref.sh with the reference
// sources, run by tests/golden/make_golden_smoothing.py.  The product never
// links or runs it.
//
// usage: ref_smoothing IN OUT   (run in a scratch directory: the reference
// reads the cell neighbour file "elem_neib" from the working directory,
// which this harness writes first)
//   IN  (little-endian): int32 ncx, ncy, ncz (cells per axis), kuzlov, kpar,
//       nb, nrec; f64 xyz[kuzlov][3]; int32 nver[kpar][14] (0-based);
//       int32 ed[kpar][25] (0-based); int32 nvkat[kpar] (0-based, 0 = air);
//       f64 rec[nrec][3]; f64 v3[nb][2] (re, im interleaved)
//   OUT f64 [12][nrec]: smoothed Ax, Ay, Az, curl_x, curl_y, curl_z, each as
//       (re = "Sin", im = "Cos") rows, in that order
#include "stdafx.h"
#include "OutputResultant3d.h"
#include "T_Brick.h"

#include <cstdio>
#include <vector>

ofstream logfile;

namespace {

bool read_all(FILE *f, void *p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

int row_of(Res3DValueType t)
{
    switch (t) {
    case vtAxSin: return 0;
    case vtAxCos: return 1;
    case vtAySin: return 2;
    case vtAyCos: return 3;
    case vtAzSin: return 4;
    case vtAzCos: return 5;
    case vtRotxASin: return 6;
    case vtRotxACos: return 7;
    case vtRotyASin: return 8;
    case vtRotyACos: return 9;
    case vtRotzASin: return 10;
    case vtRotzACos: return 11;
    default: return -1;
    }
}

class ArrayMesh : public AbstractFEM3D {
public:
    int kuzlov = 0, kpar = 0, nrec = 0;
    std::vector<double> xyz, rec, v3, out;
    std::vector<int> nver, ed, nvkat;

    int GetNumberOfNodes() override { return kuzlov; }
    int GetNumberOfElements() override { return kpar; }
    int GetElementNodesNumber() override { return 8; }
    const pv::Point3D GetNode(const int &i) override
    {
        return pv::Point3D(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    }
    const pv::Point3D GetNodeTrue(const int &i) override { return GetNode(i); }
    int GetNodeNumberOnElement(const int &e, const int &j) override { return nver[14 * e + j]; }
    int GetElementMaterial(const int &e) override { return nvkat[e]; }
    int GetTypeOfElement(const int &e) override { return nver[14 * e + 13]; }
    // the value of A or curl A at the element centre (local point (0,0,0)):
    // real parts for the "Sin" types, imaginary parts for the "Cos" types
    double GetValueInElementCenter(const int &e, const Res3DValueType &t) override
    {
        const int row = row_of(t);
        const int part = row & 1, comp = (row % 6) >> 1;
        double f[12], x[8], y[8], z[8], in[3] = {0.0, 0.0, 0.0}, o[3];
        for (int i = 0; i < 12; i++) f[i] = v3[2 * (size_t)ed[25 * e + i] + part];
        for (int i = 0; i < 8; i++) {
            const int n = nver[14 * e + i];
            x[i] = xyz[3 * n];
            y[i] = xyz[3 * n + 1];
            z[i] = xyz[3 * n + 2];
        }
        T_Brick L(x, y, z, nver[14 * e + 13]);
        if (row < 6)
            L.Calc_value_inside_hex(f, in, o);
        else
            L.Calc_rotor_inside_hex(f, in, o);
        return o[comp];
    }
    int GetNumberOfResPoints(const Res3DValueType &) override { return nrec; }
    pv::Point3D GetResPoint(const Res3DValueType &, const int &i) override
    {
        return pv::Point3D(rec[3 * i], rec[3 * i + 1], rec[3 * i + 2]);
    }
    int *GetPointerToRegular() override { return nullptr; }
    int GetXSize() override { return 0; }
    int GetYSize() override { return 0; }
    int GetZSize() override { return 0; }
    double *GetPointerToX() override { return nullptr; }
    double *GetPointerToY() override { return nullptr; }
    double *GetPointerToZ() override { return nullptr; }
    void SaveResult(const Res3DValueType &t, const double &v, const int &j, const int &) override
    {
        const int row = row_of(t);
        if (row >= 0) out[(size_t)row * nrec + j] = v;
    }
};

// the neighbour file RegularMeshBuilder writes for a tensor mesh
// (main.cpp:1480-1540 format): per cell and face (-x, -y, -z, +x, +y, +z)
// a count (0 or 1) and the 1-based neighbour
bool write_elem_neib(int ncx, int ncy, int ncz)
{
    FILE *f = fopen("elem_neib", "wb");
    if (!f) return false;
    const int nxy = ncx * ncy;
    int cell = 0;
    for (int iz = 0; iz < ncz; iz++)
        for (int iy = 0; iy < ncy; iy++)
            for (int ix = 0; ix < ncx; ix++, cell++) {
                const int nb[6] = {ix == 0 ? -1 : cell - 1,      iy == 0 ? -1 : cell - ncx,
                                   iz == 0 ? -1 : cell - nxy,    ix == ncx - 1 ? -1 : cell + 1,
                                   iy == ncy - 1 ? -1 : cell + ncx,
                                   iz == ncz - 1 ? -1 : cell + nxy};
                for (int i = 0; i < 6; i++) {
                    const int cnt = nb[i] >= 0, one = nb[i] + 1;
                    fwrite(&cnt, sizeof(int), 1, f);
                    if (cnt) fwrite(&one, sizeof(int), 1, f);
                }
            }
    fclose(f);
    return true;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s IN OUT\n", argv[0]);
        return 2;
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 3;
    int hdr[7];
    if (!read_all(f, hdr, sizeof hdr)) return 4;
    ArrayMesh m;
    const int ncx = hdr[0], ncy = hdr[1], ncz = hdr[2];
    m.kuzlov = hdr[3];
    m.kpar = hdr[4];
    const int nb = hdr[5];
    m.nrec = hdr[6];
    m.xyz.resize(3 * (size_t)m.kuzlov);
    m.nver.resize(14 * (size_t)m.kpar);
    m.ed.resize(25 * (size_t)m.kpar);
    m.nvkat.resize(m.kpar);
    m.rec.resize(3 * (size_t)m.nrec);
    m.v3.resize(2 * (size_t)nb);
    if (!read_all(f, m.xyz.data(), 8 * m.xyz.size()) ||
        !read_all(f, m.nver.data(), 4 * m.nver.size()) ||
        !read_all(f, m.ed.data(), 4 * m.ed.size()) ||
        !read_all(f, m.nvkat.data(), 4 * m.nvkat.size()) ||
        !read_all(f, m.rec.data(), 8 * m.rec.size()) || !read_all(f, m.v3.data(), 8 * m.v3.size()))
        return 4;
    fclose(f);
    if (!write_elem_neib(ncx, ncy, ncz)) return 5;
    m.out.assign((size_t)12 * m.nrec, 0.0);
    logfile.open("/dev/null");

    // give_out_vec_mt.cpp:200-237 and HarmVect3d.cpp:213-216
    OutputResultant3d resB(&m, vtWithoutDiscontinuity);
    resB.Prepare();
    OutputResultant3d resA(&m, vtWithDiscontinuity);
    resA.Prepare();
    const Res3DValueType tb[6] = {vtRotzASin, vtRotzACos, vtRotxASin,
                                  vtRotxACos, vtRotyASin, vtRotyACos};
    const Res3DValueType ta[6] = {vtAzSin, vtAzCos, vtAxSin, vtAxCos, vtAySin, vtAyCos};
    for (int i = 0; i < 6; i++) {
        resB.ValueType = tb[i];
        resB.Output(0);
    }
    for (int i = 0; i < 6; i++) {
        resA.ValueType = ta[i];
        resA.Output(0);
    }
    resB.StopSolvers();
    resA.StopSolvers();

    FILE *g = fopen(argv[2], "wb");
    if (!g) return 6;
    fwrite(m.out.data(), 8, m.out.size(), g);
    fclose(g);
    return 0;
}
