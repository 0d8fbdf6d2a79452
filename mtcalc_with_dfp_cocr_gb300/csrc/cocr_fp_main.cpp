// Drop-in replacement for the reference's COCR_FP.exe
// (Code/COCR_FP/HarmVect3d.cpp:118-365): run in a calculation directory, it
// reads the same files, solves on the GPU through mtgpu_pcocr_2x2_folded and
// writes the same outputs (v3.dat, kit, logharm3dCalc).
//
// Inputs (all in the current directory, formats of the reference):
//   kuslau (n eps maxiter), pr, ig, idi, jg, ijg, di, gg       the SLAE
//   inftry.dat, xyz.dat, nver.dat, nvkat.dat, l13d.dat          the mesh
//   sig3d, mu3d, dpr3d, tsize3d_.dat, tsize3d.dat,
//   nodesforedges.dat, edges.dat, nthreads.txt (read, unused)
// Exit status: 0 when the solve ran (whatever the solver's code, as the
// reference does, HarmVect3d.cpp:322,364); 1 on input or device errors.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "mtgpu.h"

namespace {

std::ofstream logfile;

[[noreturn]] void fail(const std::string &msg)
{
    logfile << "Error: " << msg << std::endl;
    std::fprintf(stderr, "COCR_FP (GPU): %s\n", msg.c_str());
    std::exit(1);
}

template <class T>
std::vector<T> read_bin(const char *name, size_t count)
{
    std::vector<T> v(count);
    FILE *f = std::fopen(name, "rb");
    if (!f) fail(std::string("cannot open ") + name);
    const size_t got = count ? std::fread(v.data(), sizeof(T), count, f) : 0;
    std::fclose(f);
    if (got != count) fail(std::string("cannot read binary file ") + name);
    return v;
}

std::vector<int> read_index(const char *name, size_t count)
{
    std::vector<int> v = read_bin<int>(name, count);
    for (int &x : v) x -= 1;
    return v;
}

std::vector<std::string> tokens(const char *name, bool required = true)
{
    std::ifstream in(name);
    std::vector<std::string> t;
    if (!in) {
        if (required) fail(std::string("cannot open ") + name);
        return t;
    }
    std::string s;
    while (in >> s) t.push_back(s);
    return t;
}

// "i a b" material table; returns column a (1-based material index i)
std::vector<double> read_material_column(const char *name, int n_materials)
{
    std::vector<std::string> t = tokens(name);
    std::vector<double> col(n_materials, 0.0);
    for (size_t k = 0; k + 2 < t.size(); k += 3) {
        const int i = std::atoi(t[k].c_str()) - 1;
        if (i >= 0 && i < n_materials) col[i] = std::atof(t[k + 1].c_str());
    }
    return col;
}

}  // namespace

int main()
{
    logfile.open("logharm3dCalc");
    logfile << "COCR_FP on the GPU (libmtgpu)" << std::endl;

    // materials (vec_prep_data.cpp:55-120): the number of materials is the
    // largest index in sig3d
    std::vector<std::string> st = tokens("sig3d");
    int n_materials = 0;
    for (size_t k = 0; k + 2 < st.size(); k += 3) n_materials = std::max(n_materials, std::atoi(st[k].c_str()));
    std::vector<double> sigma3d = read_material_column("sig3d", n_materials);

    // inftry.dat
    int kuzlov = -1, kpar = -1, kt1 = -1;
    {
        std::vector<std::string> t = tokens("inftry.dat");
        for (size_t k = 0; k + 1 < t.size(); k++) {
            if (t[k] == "KUZLOV=") kuzlov = std::atoi(t[k + 1].c_str());
            if (t[k] == "KPAR=") kpar = std::atoi(t[k + 1].c_str());
            if (t[k] == "KT1=") kt1 = std::atoi(t[k + 1].c_str());
        }
        if (kuzlov <= 0 || kpar <= 0 || kt1 < 0) fail("bad inftry.dat");
    }
    std::vector<int> nver = read_index("nver.dat", (size_t)kpar * 14);
    std::vector<int> nvkat = read_index("nvkat.dat", (size_t)kpar);
    std::vector<double> xyz = read_bin<double>("xyz.dat", (size_t)kuzlov * 3);
    std::vector<int> l13d = read_index("l13d.dat", (size_t)kt1);
    for (int m : nvkat)
        if (m < 0 || m >= n_materials) fail("nvkat.dat refers to an unknown material");

    // edges (HarmVect3d.cpp:36-112); non-conforming meshes are not handled
    int n_dep = 0, n_edges = 0;
    {
        std::vector<std::string> t = tokens("tsize3d_.dat");
        if (t.size() < 2) fail("bad tsize3d_.dat");
        n_dep = std::atoi(t[0].c_str());
        n_edges = std::atoi(t[1].c_str());
    }
    int tsize3d = 0;
    {
        std::vector<std::string> t = tokens("tsize3d.dat", false);
        if (!t.empty()) tsize3d = std::atoi(t[0].c_str());
    }
    if (n_dep != 0 || tsize3d != 0) fail("non-conforming meshes (T-matrix) are not supported");
    std::vector<int> edges = read_index("nodesforedges.dat", (size_t)n_edges * 2);

    // the SLAE (HarmVect3d.cpp:181-229)
    int n = 0, maxiter = 0;
    double eps = 0.0;
    {
        std::vector<std::string> t = tokens("kuslau");
        if (t.size() < 3) fail("bad kuslau");
        n = std::atoi(t[0].c_str());
        eps = std::atof(t[1].c_str());
        maxiter = std::atoi(t[2].c_str());
    }
    const int nb = n / 2;
    if (n <= 0 || n % 2 || nb != n_edges) fail("kuslau size does not match the mesh");
    std::vector<double> pr = read_bin<double>("pr", (size_t)n);
    std::vector<int> ig = read_index("ig", (size_t)nb + 1);
    std::vector<int> idi = read_index("idi", (size_t)nb + 1);
    std::vector<int> jg = read_index("jg", (size_t)ig[nb]);
    std::vector<int> ijg = read_index("ijg", (size_t)ig[nb] + 1);
    std::vector<double> di = read_bin<double>("di", (size_t)idi[nb]);
    std::vector<double> gg = read_bin<double>("gg", (size_t)ijg[ig[nb]]);

    // conductivity flags and boundary nodes (HarmVect3d.cpp:247-316)
    std::vector<double> sig(n_materials);
    for (int i = 0; i < n_materials; i++) sig[i] = sigma3d[i] == 0.0 ? 0.0 : 1.0;
    std::vector<int> bound(kuzlov, 0);
    for (int v : l13d) {
        if (v < 0 || v >= kuzlov) fail("l13d.dat refers to an unknown node");
        bound[v] = 1;
    }
    std::vector<int> ig_t(kuzlov + 1, 0), jg_t(1, 0);
    std::vector<double> gg_t(1, 0.0);
    std::vector<double> u(n, 0.0);

    logfile << "Solving SLAE" << std::endl;
    const int rc = mtgpu_pcocr_2x2_folded(
        n, ig.data(), jg.data(), idi.data(), ijg.data(), di.data(), gg.data(), pr.data(),
        u.data(), eps, maxiter, nullptr, kpar, nb, kuzlov, (double(*)[3])xyz.data(),
        nvkat.data(), (int(*)[14])nver.data(), sig.data(), (int(*)[2])edges.data(), ig_t.data(),
        jg_t.data(), gg_t.data(), bound.data());
    if (rc < -100) fail(std::string("GPU solve failed: ") + mtgpu_last_error());
    logfile << "solver status " << rc << std::endl;

    FILE *f = std::fopen("v3.dat", "wb");
    if (!f) fail("cannot write v3.dat");
    std::fwrite(u.data(), sizeof(double), u.size(), f);
    std::fclose(f);
    logfile << "All done" << std::endl;
    return 0;
}
