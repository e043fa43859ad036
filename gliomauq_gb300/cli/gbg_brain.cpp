// gbg_brain: the `brain -anatomy HGG_UQ` program on libgbglioma (and
// `-anatomy syntheticData`, below), with the reference's file contract
// (source/Glioma/Glioma_HG_UQ.cpp):
//   reads   HGG_InputParameters.txt  (Dw [cm^2/day], rho [1/day], tend [day])
//           HGG_TumorIC.bin          (tumour centre, float32, unit coordinates)
//           ../../Anatmoy/PatientNN/PNN_{GM,WM,CSF,T1,T2}.dat (Matrix::D3D)
//   writes  HGG_data.dat             (Matrix::D3D<double>, (bpd*16)^3)
// Command line: -anatomy HGG_UQ -pID N -adaptive 0|1 [-dumpfreq d -vtk 0
// -verbose 0 -nthreads k] plus -bpd (blocks per dimension, the reference's
// compile-time _BPD_, default 4), -maxlevel (its _MAXLEVEL_; default the
// initial grid's level log2(bpd), as the reference's makefile pairs them) and
// -precision f32ref|f64|f32 (default f32ref, the reference's default
// Real = float build).
//
// The initial state restates Glioma_HG_UQ::_ic_PatientCase (:67-225) in the
// chosen Real type. -adaptive 0: the time loop is gbg_run
// (Glioma_HG_UQ::run, :511-552) on the uniform grid. -adaptive 1: the same
// loop on the library's block grid (gbg_amr_run): regrids at every dump time
// and the refinement after the loop, tolerances 1e-4 / 1e-5
// (Glioma_Types.h:462-463). The dump is _dumpUQoutput (:309-372), with its
// replication rules for coarse blocks, on the (bpd * 16)^3 grid.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/gbglioma.h"
#include "matrix_file.hpp"
#include "patient_ic.hpp"

using gbgcli::Args;
using gbgcli::Matrix;

namespace {

int fail(const std::string &m, int code = 1) {
    std::fprintf(stderr, "gbg_brain: %s\n", m.c_str());
    return code;
}

// -anatomy syntheticData (Glioma_ProcessSyntheticData): HGG_data.dat ->
// PET_data.dat, T1_data.dat, T2_data.dat and HGG_TumorIC.bin (the centre of
// mass, 3 floats; the reference program writes 12 floats, of which the
// last 9 are whatever follows its 3-float buffer). -blockorder FILE gives
// the grid's block loop order (lines "level ix iy iz"), default x fastest;
// -seed48 the drand48 state before the first draw (default 0, glibc's
// unseeded state).
int synthetic_data(Args &args) {
    if (args.as_int("-adaptive", 0) != 0) return fail("syntheticData: only -adaptive 0 is supported");
    const int bpd = args.as_int("-bpd", 4);
    int level = 0;
    while ((1 << level) < bpd) ++level;
    if ((1 << level) != bpd) return fail("-bpd must be a power of two");
    const int n = bpd * 16;
    Matrix T;
    try {
        T = gbgcli::read_matrix("HGG_data.dat", 3);
    } catch (const std::exception &e) {
        return fail(e.what());
    }
    if (T.nx < n || T.ny < n || T.nz < n) return fail("HGG_data.dat is smaller than the grid");
    // the grid's cells read the file's [0, n)^3 corner, as the program does
    std::vector<double> u((size_t)n * n * n);
    for (int z = 0; z < n; ++z)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) u[(size_t)x + (size_t)n * ((size_t)y + (size_t)n * z)] = T(x, y, z);
    std::vector<gbg_block> order;
    const std::string of = args.as_string("-blockorder", "");
    if (!of.empty()) {
        std::ifstream in(of);
        gbg_block b;
        while (in >> b.level >> b.ix >> b.iy >> b.iz) order.push_back(b);
        if (order.empty()) return fail("cannot read the block order " + of);
    }
    gbg_synthetic_opts o = {0.8, 0.3, 0.02, (unsigned long long)std::strtoull(
                                               args.as_string("-seed48", "0").c_str(), nullptr, 0)};
    std::vector<double> pet(u.size()), t1(u.size()), t2(u.size());
    float com[3];
    if (gbg_synthetic_observations(n, u.data(), (int)order.size(), order.empty() ? nullptr : order.data(), &o,
                                   pet.data(), t1.data(), t2.data(), com) != GBG_OK)
        return fail(gbg_last_error(), 4);
    gbgcli::write_d3d("PET_data.dat", n, n, n, pet);
    gbgcli::write_d3d("T1_data.dat", n, n, n, t1);
    gbgcli::write_d3d("T2_data.dat", n, n, n, t2);
    FILE *f = std::fopen("HGG_TumorIC.bin", "wb");
    if (!f) return fail("cannot write HGG_TumorIC.bin");
    std::fwrite(com, sizeof(float), 3, f);
    std::fclose(f);
    if (args.as_int("-verbose", 0)) std::printf("centre of mass %f %f %f\n", com[0], com[1], com[2]);
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    Args args{argc, argv};
    if (args.as_string("-anatomy", "") == "syntheticData") return synthetic_data(args);
    if (args.as_string("-anatomy", "") != "HGG_UQ")
        return fail("only -anatomy HGG_UQ and syntheticData are supported");
    const bool adaptive = args.as_int("-adaptive", 0) != 0;
    const int pID = args.as_int("-pID", 0);
    const int bpd = args.as_int("-bpd", 4);
    int level0 = 0;
    while ((1 << level0) < bpd) ++level0;
    if ((1 << level0) != bpd) return fail("-bpd must be a power of two");
    const int max_level = args.as_int("-maxlevel", level0);
    if (max_level < level0 || max_level > 6) return fail("-maxlevel must lie in [log2(bpd), 6]");
    const double dumpfreq = args.as_double("-dumpfreq", 1000.0);
    if (adaptive && !(dumpfreq > 0)) return fail("-dumpfreq must be positive");
    const std::string prec = args.as_string("-precision", "f32ref");
    const int precision = prec == "f64" ? GBG_PREC_F64 : prec == "f32" ? GBG_PREC_F32 : GBG_PREC_F32REF;
    const bool verbose = args.as_int("-verbose", 0) != 0;

    char folder[256];
    std::snprintf(folder, sizeof(folder), "../../Anatmoy/Patient%02d/P%02d", pID, pID);
    const std::string base(folder);
    Matrix GM, WM, CSF, T1, T2;
    try {
        GM = gbgcli::read_matrix(base + "_GM.dat", 3);
        WM = gbgcli::read_matrix(base + "_WM.dat", 3);
        CSF = gbgcli::read_matrix(base + "_CSF.dat", 3);
        T1 = gbgcli::read_matrix(base + "_T1.dat", 3);
        T2 = gbgcli::read_matrix(base + "_T2.dat", 3);
    } catch (const std::exception &e) {
        return fail(e.what());
    }
    // HGG_TumorIC.bin: the first three floats (Glioma_HG_UQ.cpp:229-263)
    float ic[3];
    {
        FILE *f = std::fopen("HGG_TumorIC.bin", "rb");
        if (!f) return fail("File error", 1);
        if (std::fread(ic, sizeof(float), 3, f) != 3) {
            std::fclose(f);
            return fail("Reading error", 3);
        }
        std::fclose(f);
    }
    // HGG_InputParameters.txt: Dw, rho, tend (:519-529); a missing file leaves
    // the reference's values uninitialised -- here it is an error.
    double Dw, rho, tend;
    {
        std::ifstream in("HGG_InputParameters.txt");
        if (!(in >> Dw >> rho >> tend)) return fail("cannot read HGG_InputParameters.txt");
    }
    std::vector<double> pw, pg, phi;
    double L = 0;
    if (precision == GBG_PREC_F64) {
        const double t[3] = {ic[0], ic[1], ic[2]};
        gbgcli::initial_state<double>(bpd, GM, WM, CSF, T1, T2, t, pw, pg, phi, L);
    } else {
        const float t[3] = {ic[0], ic[1], ic[2]};
        gbgcli::initial_state<float>(bpd, GM, WM, CSF, T1, T2, t, pw, pg, phi, L);
    }
    const int n = bpd * 16;
    if (adaptive) {
        // the uniform initial state as the blocks of the initial grid (level
        // log2(bpd), ix fastest), block-major with x fastest inside a block
        const int nb = bpd * bpd * bpd;
        std::vector<gbg_block> blocks(nb);
        std::vector<double> bw((size_t)nb * 4096), bg(bw.size()), bp(bw.size());
        for (int bz = 0, b = 0; bz < bpd; ++bz)
            for (int by = 0; by < bpd; ++by)
                for (int bx = 0; bx < bpd; ++bx, ++b) {
                    blocks[b] = {level0, bx, by, bz};
                    for (int z = 0; z < 16; ++z)
                        for (int y = 0; y < 16; ++y)
                            for (int x = 0; x < 16; ++x) {
                                const size_t g = (size_t)(bx * 16 + x) +
                                                 (size_t)n * ((size_t)(by * 16 + y) + (size_t)n * (bz * 16 + z));
                                const size_t c = (size_t)b * 4096 + x + 16 * (y + 16 * z);
                                bw[c] = pw[g];
                                bg[c] = pg[g];
                                bp[c] = phi[g];
                            }
                }
        const int cap = 1 << (3 * max_level);
        gbg_amr_config acfg = {cap, precision, 0};
        gbg_handle *a = nullptr;
        if (gbg_amr_create(&acfg, &a) != GBG_OK) return fail(gbg_last_error(), 4);
        gbg_amr_run_opts o = {Dw, rho, tend, L, dumpfreq, bpd, 1, max_level, 1, 1e-4, 1e-5};
        long nsteps = 0;
        int regrids = 0;
        std::vector<double> out((size_t)n * n * n);
        if (gbg_amr_set_grid(a, nb, blocks.data(), bw.data(), bg.data(), bp.data()) != GBG_OK ||
            gbg_amr_run(a, &o, &nsteps, &regrids) != GBG_OK ||
            gbg_amr_dump_uniform(a, n, 1, out.data()) != GBG_OK) {
            const std::string m = gbg_last_error();
            gbg_destroy(a);
            return fail(m, 4);
        }
        int nbf = 0;
        gbg_amr_get_blocks(a, nullptr, 0, &nbf);
        gbg_destroy(a);
        if (verbose) std::printf("steps=%ld regrids=%d blocks=%d L=%f\n", nsteps, regrids, nbf, L);
        gbgcli::write_d3d("HGG_data.dat", n, n, n, out);
        return 0;
    }
    gbg_config cfg = {n, precision, 0, 0};
    gbg_handle *h = nullptr;
    if (gbg_create(&cfg, &h) != GBG_OK) return fail(gbg_last_error(), 4);
    long nsteps = 0;
    double dt = 0;
    if (gbg_set_anatomy(h, pw.data(), pg.data()) != GBG_OK || gbg_set_phi(h, phi.data()) != GBG_OK ||
        gbg_run(h, Dw, rho, tend, L, &nsteps, &dt) != GBG_OK || gbg_get_phi(h, phi.data()) != GBG_OK) {
        const std::string m = gbg_last_error();
        gbg_destroy(h);
        return fail(m, 4);
    }
    gbg_destroy(h);
    if (verbose) std::printf("dt=%f steps=%ld L=%f\n", dt, nsteps, L);
    gbgcli::write_d3d("HGG_data.dat", n, n, n, phi);
    return 0;
}
