// Test infrastructure only: a driver that runs GliomaUQ's own MRAG grid, block
// lab, block-processing back-end and Glioma operators, compiled in place from
// the reference sources (see oracle/Makefile). It never ships and nothing in the
// product links it. Its outputs pin the oracle restatement and fill the golden
// fixtures under tests/golden/.
//
// What it drives, all unmodified reference code:
//   Grid<W,B>                           source/MRAGcore/MRAGrid.h:44-186
//   BlockProcessing (TBB pipeline)      source/MRAGmultithreading/MRAGBlockProcessing_TBB.h:314-512
//   Glioma_ReactionDiffusionOperator<3> source/Glioma/Glioma_ReactionDiffusionOperator.h:12-222
//   UpdateTumor<3>                      source/Glioma/Glioma_ReactionDiffusionOperator.h:227-266
//   Glioma_MALAslopesRHS<3>, UpdateMALAslopes<3>
//                                       source/Glioma/Glioma_MALA_SlopesOperator.h:13-229
//   Science::AutomaticRefinement/Compression
//                                       source/MRAGscience/MRAGScienceCore.h:42-177
// The time loop is Glioma_HG_UQ::run (source/Glioma/Glioma_HG_UQ.cpp:511-588)
// restated with the anatomy and initial density taken from an input file
// instead of the patient files and the smoothed-sphere initial condition.
//
// Commands:
//   solve  <in> <out>   time loop; writes the final field resampled to the
//                       finest uniform grid plus every block of the final grid
//   ghosts <in> <out>   flattens Grid::getBoundaryInfo() of the (possibly
//                       regridded) grid: per block, per ghost cell, the
//                       (source block, source cell, weight) triples
//   fwt    <in> <out>   per-block detail maxima of BlockFWT on phi
//   state  <in> <out> [k]  adaptive fixtures: blocks + ghost tables + FWT
//                       maxima after the loop, blocks after k more steps,
//                       blocks after one more regrid
//   timing <in>         times steps only (no output), prints cell-steps/s
//   mala   <in> <out>   nsteps steps of Glioma_HG_UQ_MALA::_reactionDiffusionMALAStep
//                       (source/Glioma/Glioma_HG_UQ_MALA.cpp:575-591) from zero
//                       slopes; writes phi, sRho and sD on the uniform grid
//   dump   <in> <out> [regrid]   (builds with GBG_HARNESS_DUMP only) the time
//                       loop as `state` runs it, optionally one more regrid,
//                       then the blocks and the reference's own
//                       Glioma_HG_UQ::_dumpUQoutput of that grid
//                       (source/Glioma/Glioma_HG_UQ.cpp:309-372), which
//                       resamples to (blocksPerDimension * blockSize)^3 with
//                       its h / 2h / 3h / else-4h replication rules
//   dumpgrid <out> <r1> [r2 ...]  (GBG_HARNESS_DUMP builds) a grid of
//                       blocksPerDimension^3 blocks at the maximum level
//                       compressed once per radius by Grid::compress (blocks
//                       whose centre lies farther than r1, then r2, ... from
//                       the point (0.3, 0.35, 0.4) of the unit cube), its cells set to
//                       phi = ((7 gx + 13 gy + 29 gz + 101 level) mod 1009) / 1009
//                       (gx, gy, gz: the cell's index on its level), then the
//                       blocks, the grid's ghost tables (as `state` writes
//                       them) and _dumpUQoutput of that grid
#include "Glioma_Types.h"
#include "Glioma_MALA_SlopesOperator.h"
#ifdef GBG_HARNESS_DUMP
// _dumpUQoutput is a private member of Glioma_HG_UQ; this test-only
// translation unit lifts the access specifier for the class declaration so
// that the reference's own member function can be called on a grid of the
// harness's choosing (the definitions are compiled unmodified from
// Glioma_HG_UQ.cpp).
#define private public
#include "Glioma_HG_UQ.h"
#undef private
#endif

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <set>
#include <string>
#include <vector>

static int maxStencilH[2][3] = {{-1, -1, -1}, {+2, +2, +2}};

struct Input {
    int32_t n = 0;           // finest uniform cells per side of the input fields
    int32_t bpd = 0;         // blocks per dimension of the initial grid
    int32_t adaptive = 0;    // regrid at dump times (Glioma_HG_UQ -adaptive)
    int32_t nsteps = -1;     // >=0: run exactly nsteps steps, ignore tend
    double Dw_file = 0;      // cm^2/day as read from HGG_InputParameters.txt
    double rho = 0;
    double tend = 0;
    double L = 0;            // brain length (cm), Glioma_HG_UQ.cpp:104
    double dumpfreq = 0;     // -dumpfreq
    std::vector<double> pw, pg, phi;
};

static void die(const char *m) {
    fprintf(stderr, "ref_harness: %s\n", m);
    exit(2);
}

static Input readInput(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) die("cannot open input");
    char magic[8];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "GBGREF01", 8)) die("bad magic");
    Input in;
    int32_t ib[4];
    double db[5];
    if (fread(ib, 4, 4, f) != 4) die("short header");
    if (fread(db, 8, 5, f) != 5) die("short header");
    in.n = ib[0]; in.bpd = ib[1]; in.adaptive = ib[2]; in.nsteps = ib[3];
    in.Dw_file = db[0]; in.rho = db[1]; in.tend = db[2]; in.L = db[3]; in.dumpfreq = db[4];
    size_t N = (size_t)in.n * in.n * in.n;
    in.pw.resize(N); in.pg.resize(N); in.phi.resize(N);
    if (fread(in.pw.data(), 8, N, f) != N) die("short pw");
    if (fread(in.pg.data(), 8, N, f) != N) die("short pg");
    if (fread(in.phi.data(), 8, N, f) != N) die("short phi");
    fclose(f);
    return in;
}

// finest level spanned by the grid: cells per side n = 2^L * blockSize
static int finestLevel(int n) {
    int l = 0;
    while ((blockSize << l) < n) ++l;
    if ((blockSize << l) != n) die("n must be blockSize * 2^L");
    return l;
}

// Fill every block of the grid from the finest uniform input (point sampling of
// the fine cell at the block cell's lower corner, which is exact for the
// initial uniform grid at the finest level).
static void fillGrid(Grid<W, B> &grid, const Input &in) {
    const int Lf = finestLevel(in.n);
    std::vector<BlockInfo> vInfo = grid.getBlocksInfo();
    for (size_t i = 0; i < vInfo.size(); i++) {
        BlockInfo &info = vInfo[i];
        B &block = grid.getBlockCollection()[info.blockID];
        const int stride = 1 << (Lf - info.level);
        for (int iz = 0; iz < B::sizeZ; iz++)
            for (int iy = 0; iy < B::sizeY; iy++)
                for (int ix = 0; ix < B::sizeX; ix++) {
                    const size_t gx = (size_t)(info.index[0] * B::sizeX + ix) * stride;
                    const size_t gy = (size_t)(info.index[1] * B::sizeY + iy) * stride;
                    const size_t gz = (size_t)(info.index[2] * B::sizeZ + iz) * stride;
                    const size_t g = gx + in.n * (gy + in.n * gz);
                    block(ix, iy, iz).p_w = (Real)in.pw[g];
                    block(ix, iy, iz).p_g = (Real)in.pg[g];
                    block(ix, iy, iz).phi = (Real)in.phi[g];
                }
        grid.getBlockCollection().release(info.blockID);
    }
}

struct Sim {
    Grid<W, B> *grid;
    BlockProcessing blockProcessing;
    Refiner_SpaceExtension *refiner;
    Compressor *compressor;
    BlockFWT<W, B, RD_Projector_Wavelets> blockfwt;
    Profiler profiler;

    explicit Sim(int bpd) {
        // same construction as Glioma_HG_UQ::Glioma_HG_UQ (Glioma_HG_UQ.cpp:29-35)
        refiner = new Refiner_SpaceExtension(resJump, maxLevel);
        compressor = new Compressor(resJump);
        grid = new Grid<W, B>(bpd, bpd, bpd, maxStencilH);
        grid->setCompressor(compressor);
        grid->setRefiner(refiner);
    }
    // Glioma_HG_UQ::_reactionDiffusionStep (Glioma_HG_UQ.cpp:266-277)
    void step(BoundaryInfo *bi, int gran, Real Dw, Real Dg, Real rho, double dt) {
        vector<BlockInfo> vInfo = grid->getBlocksInfo();
        const BlockCollection<B> &coll = grid->getBlockCollection();
        Glioma_ReactionDiffusionOperator<_DIM> rhs(Dw, Dg, rho);
        UpdateTumor<_DIM> updateTumor(dt);
        blockProcessing.pipeline_process(vInfo, coll, *bi, rhs);
        BlockProcessing::process(vInfo, coll, updateTumor, gran);
    }
    // Glioma_HG_UQ_MALA::_reactionDiffusionMALAStep (Glioma_HG_UQ_MALA.cpp:575-591):
    // both right-hand sides from the state before the step, then both updates
    void malaStep(BoundaryInfo *bi, int gran, Real Dw, Real Dg, Real rho, double dt) {
        vector<BlockInfo> vInfo = grid->getBlocksInfo();
        const BlockCollection<B> &coll = grid->getBlockCollection();
        Glioma_ReactionDiffusionOperator<_DIM> rhs(Dw, Dg, rho);
        UpdateTumor<_DIM> updateTumor(dt);
        Glioma_MALAslopesRHS<_DIM> slopesRhs(Dw, Dg);
        UpdateMALAslopes<_DIM> updateSlopes(dt);
        blockProcessing.pipeline_process(vInfo, coll, *bi, rhs);
        blockProcessing.pipeline_process(vInfo, coll, *bi, slopesRhs);
        BlockProcessing::process(vInfo, coll, updateTumor, gran);
        BlockProcessing::process(vInfo, coll, updateSlopes, gran);
    }
    void regrid() {
        const int r = Science::AutomaticRefinement<0, 0>(*grid, blockfwt, refinement_tolerance, maxLevel, 1, &profiler);
        const int c = Science::AutomaticCompression<0, 0>(*grid, blockfwt, compression_tolerance, -1, &profiler);
        if (getenv("GBG_HARNESS_VERBOSE"))
            fprintf(stderr, "regrid: refined %d collapsed %d -> %zu blocks\n", r, c, grid->getBlocksInfo().size());
    }
};

struct RunInfo {
    double dt;
    long steps;
    int regrids;
    double Dw_unit, Dg_unit, rho;
};

// Glioma_HG_UQ::run time loop (Glioma_HG_UQ.cpp:511-575); returns step count.
static RunInfo runLoop(Sim &s, const Input &in, bool verbose, double *secs, bool final_refine = true) {
    const int gran = (s.grid->getBlocksInfo().size() <= 8 ? 1 : 4);
    BoundaryInfo *boundaryInfo = &s.grid->getBoundaryInfo();
    Real Dw = (Real)in.Dw_file, rho = (Real)in.rho, Dg;
    const double L = in.L;
    Dw = Dw / (L * L);
    Dg = 0.1 * Dw;
    double t = 0.0;
    double h = 1. / (blockSize * in.bpd);
    double dt = 0.99 * h * h / (2. * _DIM * std::max(Dw, Dg));
    double whenToWriteOffset = in.dumpfreq, whenToWrite = whenToWriteOffset;
    RunInfo ri{dt, 0, 0, (double)Dw, (double)Dg, (double)rho};
    auto t0 = std::chrono::steady_clock::now();
    if (in.nsteps >= 0) {
        for (long k = 0; k < in.nsteps; ++k) {
            s.step(boundaryInfo, gran, Dw, Dg, rho, dt);
            ri.steps++;
        }
    } else {
        while (t <= in.tend) {
            s.step(boundaryInfo, gran, Dw, Dg, rho, dt);
            t += dt;
            ri.steps++;
            if (t >= ((double)(whenToWrite))) {
                if (in.adaptive) {
                    s.regrid();
                    ri.regrids++;
                }
                whenToWrite = whenToWrite + whenToWriteOffset;
            }
        }
        if (in.adaptive && final_refine) {
            Science::AutomaticRefinement<0, 0>(*s.grid, s.blockfwt, refinement_tolerance, maxLevel, 1,
                                               &s.profiler);
            ri.regrids++;
        }
    }
    auto t1 = std::chrono::steady_clock::now();
    if (secs) *secs = std::chrono::duration<double>(t1 - t0).count();
    if (verbose)
        fprintf(stderr, "ref_harness: dt=%.17g steps=%ld regrids=%d\n", dt, ri.steps, ri.regrids);
    return ri;
}

static void writeBlocks(FILE *f, Grid<W, B> &grid) {
    std::vector<BlockInfo> vInfo = grid.getBlocksInfo();
    int32_t nb = (int32_t)vInfo.size();
    fwrite(&nb, 4, 1, f);
    std::vector<double> buf(3 * B::sizeX * B::sizeY * B::sizeZ);
    for (size_t i = 0; i < vInfo.size(); i++) {
        BlockInfo &info = vInfo[i];
        int32_t hdr[5] = {info.blockID, info.level, info.index[0], info.index[1], info.index[2]};
        fwrite(hdr, 4, 5, f);
        B &block = grid.getBlockCollection()[info.blockID];
        size_t c = 0, nc = (size_t)B::sizeX * B::sizeY * B::sizeZ;
        for (int iz = 0; iz < B::sizeZ; iz++)
            for (int iy = 0; iy < B::sizeY; iy++)
                for (int ix = 0; ix < B::sizeX; ix++, c++) {
                    buf[c] = block(ix, iy, iz).phi;
                    buf[nc + c] = block(ix, iy, iz).p_w;
                    buf[2 * nc + c] = block(ix, iy, iz).p_g;
                }
        grid.getBlockCollection().release(info.blockID);
        fwrite(buf.data(), 8, buf.size(), f);
    }
}

// Piecewise-constant resampling of every block to the finest uniform grid (the
// intent of Glioma_HG_UQ::_dumpUQoutput, Glioma_HG_UQ.cpp:309-372, for any level).
static std::vector<double> uniformPhi(Grid<W, B> &grid, int n) {
    const int Lf = finestLevel(n);
    std::vector<double> out((size_t)n * n * n, 0.0);
    std::vector<BlockInfo> vInfo = grid.getBlocksInfo();
    for (size_t i = 0; i < vInfo.size(); i++) {
        BlockInfo &info = vInfo[i];
        B &block = grid.getBlockCollection()[info.blockID];
        const int r = 1 << (Lf - info.level);
        for (int iz = 0; iz < B::sizeZ; iz++)
            for (int iy = 0; iy < B::sizeY; iy++)
                for (int ix = 0; ix < B::sizeX; ix++) {
                    const double v = block(ix, iy, iz).phi;
                    for (int cz = 0; cz < r; cz++)
                        for (int cy = 0; cy < r; cy++)
                            for (int cx = 0; cx < r; cx++) {
                                size_t gx = (size_t)(info.index[0] * B::sizeX + ix) * r + cx;
                                size_t gy = (size_t)(info.index[1] * B::sizeY + iy) * r + cy;
                                size_t gz = (size_t)(info.index[2] * B::sizeZ + iz) * r + cz;
                                out[gx + n * (gy + n * gz)] = v;
                            }
                }
        grid.getBlockCollection().release(info.blockID);
    }
    return out;
}

// One cell field of a uniform grid at the finest level (no regridding).
template <typename F>
static std::vector<double> uniformField(Grid<W, B> &grid, int n, F get) {
    std::vector<double> out((size_t)n * n * n, 0.0);
    std::vector<BlockInfo> vInfo = grid.getBlocksInfo();
    for (size_t i = 0; i < vInfo.size(); i++) {
        BlockInfo &info = vInfo[i];
        B &block = grid.getBlockCollection()[info.blockID];
        for (int iz = 0; iz < B::sizeZ; iz++)
            for (int iy = 0; iy < B::sizeY; iy++)
                for (int ix = 0; ix < B::sizeX; ix++) {
                    const size_t gx = (size_t)info.index[0] * B::sizeX + ix;
                    const size_t gy = (size_t)info.index[1] * B::sizeY + iy;
                    const size_t gz = (size_t)info.index[2] * B::sizeZ + iz;
                    out[gx + n * (gy + n * gz)] = get(block(ix, iy, iz));
                }
        grid.getBlockCollection().release(info.blockID);
    }
    return out;
}

// The MALA variant's loop (Glioma_HG_UQ_MALA::run, Glioma_HG_UQ_MALA.cpp:717-758:
// the same parameter rescale and step rule as Glioma_HG_UQ::run) for a fixed
// number of steps on a uniform grid.
static int cmdMala(const char *inp, const char *outp) {
    Input in = readInput(inp);
    if (in.nsteps < 0 || in.adaptive) die("mala: fixed nsteps, uniform grid");
    Sim s(in.bpd);
    fillGrid(*s.grid, in);
    const int gran = (s.grid->getBlocksInfo().size() <= 8 ? 1 : 4);
    BoundaryInfo *boundaryInfo = &s.grid->getBoundaryInfo();
    Real Dw = (Real)in.Dw_file, rho = (Real)in.rho, Dg;
    const double L = in.L;
    Dw = Dw / (L * L);
    Dg = 0.1 * Dw;
    double h = 1. / (blockSize * in.bpd);
    double dt = 0.99 * h * h / (2. * _DIM * std::max(Dw, Dg));
    for (long k = 0; k < in.nsteps; ++k) s.malaStep(boundaryInfo, gran, Dw, Dg, rho, dt);
    FILE *f = fopen(outp, "wb");
    if (!f) die("cannot open output");
    fwrite("GBGMAL01", 1, 8, f);
    int32_t hdr[4] = {in.n, (int32_t)sizeof(Real), (int32_t)in.nsteps, 0};
    fwrite(hdr, 4, 4, f);
    double dh[4] = {dt, (double)Dw, (double)Dg, (double)rho};
    fwrite(dh, 8, 4, f);
    std::vector<double> u = uniformField(*s.grid, in.n, [](const CCell_extended &c) { return (double)c.phi; });
    std::vector<double> sr = uniformField(*s.grid, in.n, [](const CCell_extended &c) { return (double)c.sRho; });
    std::vector<double> sd = uniformField(*s.grid, in.n, [](const CCell_extended &c) { return (double)c.sD; });
    fwrite(u.data(), 8, u.size(), f);
    fwrite(sr.data(), 8, sr.size(), f);
    fwrite(sd.data(), 8, sd.size(), f);
    fclose(f);
    return 0;
}

static int cmdSolve(const char *inp, const char *outp) {
    Input in = readInput(inp);
    Sim s(in.bpd);
    fillGrid(*s.grid, in);
    RunInfo ri = runLoop(s, in, true, nullptr);
    FILE *f = fopen(outp, "wb");
    if (!f) die("cannot open output");
    fwrite("GBGOUT01", 1, 8, f);
    int32_t hdr[4] = {in.n, (int32_t)sizeof(Real), (int32_t)ri.steps, ri.regrids};
    fwrite(hdr, 4, 4, f);
    double dh[4] = {ri.dt, ri.Dw_unit, ri.Dg_unit, ri.rho};
    fwrite(dh, 8, 4, f);
    std::vector<double> u = uniformPhi(*s.grid, in.n);
    fwrite(u.data(), 8, u.size(), f);
    writeBlocks(f, *s.grid);
    fclose(f);
    return 0;
}

// Runs the loop (which may regrid), then flattens the boundary info of the
// resulting grid. Per block: 27 region headers, then for every ghost cell in
// BlockLab::load order (MRAGBlockLab.h:256-295) its instruction list as
// (source blockID, source cell index, w0, w1, w2) with the weights already
// converted to Real as BlockLab does (MRAGBlockLab.h:250-251).
static int cmdGhosts(const char *inp, const char *outp) {
    Input in = readInput(inp);
    Sim s(in.bpd);
    fillGrid(*s.grid, in);
    runLoop(s, in, true, nullptr);
    BoundaryInfo &bi = s.grid->getBoundaryInfo();
    std::vector<BlockInfo> vInfo = s.grid->getBlocksInfo();
    FILE *f = fopen(outp, "wb");
    if (!f) die("cannot open output");
    fwrite("GBGGHO01", 1, 8, f);
    int32_t nb = (int32_t)vInfo.size();
    fwrite(&nb, 4, 1, f);
    for (size_t i = 0; i < vInfo.size(); i++) {
        const BlockInfo &info = vInfo[i];
        BoundaryInfoBlock &bb = *bi.boundaryInfoOfBlock.find(info.blockID)->second;
        bb.lock();
        const vector<PointIndex> &pool = bb.getIndexPool();
        const vector<vector<IndexWP> > &gh = bb.getGhosts();
        int32_t hdr[6] = {info.blockID, info.level, info.index[0], info.index[1], info.index[2],
                          (int32_t)gh.size()};
        fwrite(hdr, 4, 6, f);
        for (int c = 0; c < 27; c++) {
            int32_t r[2] = {(int32_t)bb.boundary[c].start, (int32_t)bb.boundary[c].nGhosts};
            fwrite(r, 4, 2, f);
        }
        for (size_t g = 0; g < gh.size(); g++) {
            int32_t cnt = (int32_t)gh[g].size();
            fwrite(&cnt, 4, 1, f);
            for (size_t k = 0; k < gh[g].size(); k++) {
                const IndexWP &w = gh[g][k];
                int32_t src[2] = {pool[w.point_index].blockID, pool[w.point_index].index};
                double wr[3] = {(double)(Real)bb.weightsPool[w.weights_index[0]],
                                (double)(Real)bb.weightsPool[w.weights_index[1]],
                                (double)(Real)bb.weightsPool[w.weights_index[2]]};
                fwrite(src, 4, 2, f);
                fwrite(wr, 8, 3, f);
            }
        }
        bb.release();
    }
    fclose(f);
    return 0;
}

// Per-block FWT detail maxima on the current field (BlockFWT::multichannel_fwt,
// MRAGBlockFWT.h:447-468, report FWTReport::getOverAll_DetailMaxMag :184-190).
static int cmdFwt(const char *inp, const char *outp) {
    Input in = readInput(inp);
    Sim s(in.bpd);
    fillGrid(*s.grid, in);
    runLoop(s, in, true, nullptr);
    std::vector<BlockInfo> vInfo = s.grid->getBlocksInfo();
    vector<FWTReport<1> > rep = BlockFWT<W, B, RD_Projector_Wavelets>::template multichannel_fwt<0, 0>(
        vInfo, s.grid->getBlockCollection(), s.grid->getBoundaryInfo());
    FILE *f = fopen(outp, "wb");
    if (!f) die("cannot open output");
    fwrite("GBGFWT01", 1, 8, f);
    int32_t nb = (int32_t)vInfo.size();
    fwrite(&nb, 4, 1, f);
    for (size_t i = 0; i < vInfo.size(); i++) {
        int32_t hdr[5] = {vInfo[i].blockID, vInfo[i].level, vInfo[i].index[0], vInfo[i].index[1],
                          vInfo[i].index[2]};
        fwrite(hdr, 4, 5, f);
        double d = rep[i].getOverAll_DetailMaxMag();
        fwrite(&d, 8, 1, f);
    }
    fclose(f);
    return 0;
}

static void writeGhostTables(FILE *f, Grid<W, B> &grid) {
    BoundaryInfo &bi = grid.getBoundaryInfo();
    std::vector<BlockInfo> vInfo = grid.getBlocksInfo();
    int32_t nb = (int32_t)vInfo.size();
    fwrite(&nb, 4, 1, f);
    for (size_t i = 0; i < vInfo.size(); i++) {
        const BlockInfo &info = vInfo[i];
        BoundaryInfoBlock &bb = *bi.boundaryInfoOfBlock.find(info.blockID)->second;
        bb.lock();
        const vector<PointIndex> &pool = bb.getIndexPool();
        const vector<vector<IndexWP> > &gh = bb.getGhosts();
        int32_t hdr[2] = {info.blockID, (int32_t)gh.size()};
        fwrite(hdr, 4, 2, f);
        for (int c = 0; c < 27; c++) {
            int32_t r[2] = {(int32_t)bb.boundary[c].start, (int32_t)bb.boundary[c].nGhosts};
            fwrite(r, 4, 2, f);
        }
        for (size_t g = 0; g < gh.size(); g++) {
            int32_t cnt = (int32_t)gh[g].size();
            fwrite(&cnt, 4, 1, f);
            for (size_t k = 0; k < gh[g].size(); k++) {
                const IndexWP &w = gh[g][k];
                // the weight product as BlockLab forms it, in Real (MRAGBlockLab.h:289)
                const Real w0 = (Real)bb.weightsPool[w.weights_index[0]];
                const Real w1 = (Real)bb.weightsPool[w.weights_index[1]];
                const Real w2 = (Real)bb.weightsPool[w.weights_index[2]];
                const Real wr = w0 * w1 * w2;
                int32_t src[2] = {pool[w.point_index].blockID, pool[w.point_index].index};
                double wd = (double)wr;
                fwrite(src, 4, 2, f);
                fwrite(&wd, 8, 1, f);
            }
        }
        bb.release();
    }
}

static void writeFwt(FILE *f, Grid<W, B> &grid) {
    std::vector<BlockInfo> vInfo = grid.getBlocksInfo();
    vector<FWTReport<1> > rep = BlockFWT<W, B, RD_Projector_Wavelets>::template multichannel_fwt<0, 0>(
        vInfo, grid.getBlockCollection(), grid.getBoundaryInfo());
    int32_t nb = (int32_t)vInfo.size();
    fwrite(&nb, 4, 1, f);
    for (size_t i = 0; i < vInfo.size(); i++) {
        double d = rep[i].getOverAll_DetailMaxMag();
        fwrite(&d, 8, 1, f);
    }
}

// Adaptive state for the AMR fixtures: run the time loop (regridding at dump
// times, without run()'s final refinement), then write S0 = blocks + ghost tables + FWT detail maxima; take
// `extra` more steps without regridding and write S1 = blocks; then a
// forced regrid (split every block below the maximum level, then collapse
// the complete sibling groups among the other blocks in the upper half of x)
// and write S2 = blocks.
static int cmdState(const char *inp, const char *outp, int extra) {
    Input in = readInput(inp);
    Sim s(in.bpd);
    fillGrid(*s.grid, in);
    RunInfo ri = runLoop(s, in, true, nullptr, false);
    FILE *f = fopen(outp, "wb");
    if (!f) die("cannot open output");
    fwrite("GBGSTA01", 1, 8, f);
    int32_t hdr[4] = {in.n, (int32_t)sizeof(Real), (int32_t)ri.steps, ri.regrids};
    fwrite(hdr, 4, 4, f);
    double dh[4] = {ri.dt, ri.Dw_unit, ri.Dg_unit, ri.rho};
    fwrite(dh, 8, 4, f);
    writeBlocks(f, *s.grid);
    writeGhostTables(f, *s.grid);
    writeFwt(f, *s.grid);
    const int gran = (s.grid->getBlocksInfo().size() <= 8 ? 1 : 4);
    for (int k = 0; k < extra; ++k)
        s.step(&s.grid->getBoundaryInfo(), gran, (Real)ri.Dw_unit, (Real)ri.Dg_unit, (Real)ri.rho, ri.dt);
    writeBlocks(f, *s.grid);
    // a forced regrid that both splits and collapses (Grid::refine with
    // BlockSplitter, Grid::compress with BlockCollapser): refine every block
    // below the maximum level, then offer for compression every block in the
    // upper half of x
    {
        std::vector<BlockInfo> v = s.grid->getBlocksInfo();
        std::set<int> toRefine, before;
        for (const BlockInfo &b : v) {
            before.insert(b.blockID);
            if (b.level < maxLevel) toRefine.insert(b.blockID);
        }
        if (!toRefine.empty()) s.grid->refine(toRefine);
        v = s.grid->getBlocksInfo();
        std::set<int> toCompress;
        for (const BlockInfo &b : v)
            if (before.count(b.blockID) && b.index[0] >= (1 << b.level) / 2) toCompress.insert(b.blockID);
        int nc = 0;
        s.grid->compress(toCompress, nc);
        if (getenv("GBG_HARNESS_VERBOSE"))
            fprintf(stderr, "forced regrid: refined %zu, collapsed %d -> %zu blocks\n", toRefine.size(), nc,
                    s.grid->getBlocksInfo().size());
    }
    writeBlocks(f, *s.grid);
    fclose(f);
    return 0;
}

#ifdef GBG_HARNESS_DUMP
// Glioma_HG_UQ's constructor reads the patient files; _dumpUQoutput reads no
// member of the object but bVerbose, so it runs on zeroed storage of the
// class's size and alignment (bVerbose = false) instead of a constructed
// object. It writes HGG_data.dat (MatrixD3D<double>) into the working
// directory.
static int cmdDump(const char *inp, const char *outp, int regrid) {
    Input in = readInput(inp);
    Sim s(in.bpd);
    fillGrid(*s.grid, in);
    RunInfo ri = runLoop(s, in, true, nullptr, false);
    if (regrid) {
        s.regrid();
        ri.regrids++;
    }
    alignas(Glioma_HG_UQ) static unsigned char storage[sizeof(Glioma_HG_UQ)];
    memset(storage, 0, sizeof storage);
    reinterpret_cast<Glioma_HG_UQ *>(storage)->_dumpUQoutput(*s.grid);
    FILE *f = fopen(outp, "wb");
    if (!f) die("cannot open output");
    fwrite("GBGDMP01", 1, 8, f);
    int32_t hdr[4] = {in.n, (int32_t)sizeof(Real), (int32_t)ri.steps, ri.regrids};
    fwrite(hdr, 4, 4, f);
    int32_t gpd = blocksPerDimension * blockSize;
    fwrite(&gpd, 4, 1, f);
    writeBlocks(f, *s.grid);
    fclose(f);
    return 0;
}
#endif

#ifdef GBG_HARNESS_DUMP
static int cmdDumpGrid(const char *outp, const std::vector<double> &radii) {
    Sim s(blocksPerDimension);
    const double c[3] = {0.3, 0.35, 0.4};
    for (double r : radii) {
        std::vector<BlockInfo> v = s.grid->getBlocksInfo();
        std::set<int> toCompress;
        for (const BlockInfo &b : v) {
            const double w = 1.0 / (1 << b.level);
            double d2 = 0;
            for (int k = 0; k < 3; k++) {
                const double x = (b.index[k] + 0.5) * w - c[k];
                d2 += x * x;
            }
            if (d2 > r * r) toCompress.insert(b.blockID);
        }
        int nc = 0;
        s.grid->compress(toCompress, nc);
    }
    std::vector<BlockInfo> vInfo = s.grid->getBlocksInfo();
    for (size_t i = 0; i < vInfo.size(); i++) {
        BlockInfo &info = vInfo[i];
        B &block = s.grid->getBlockCollection()[info.blockID];
        for (int iz = 0; iz < B::sizeZ; iz++)
            for (int iy = 0; iy < B::sizeY; iy++)
                for (int ix = 0; ix < B::sizeX; ix++) {
                    const long gx = (long)info.index[0] * B::sizeX + ix;
                    const long gy = (long)info.index[1] * B::sizeY + iy;
                    const long gz = (long)info.index[2] * B::sizeZ + iz;
                    block(ix, iy, iz).phi = (Real)((double)((7 * gx + 13 * gy + 29 * gz + 101 * info.level) % 1009) / 1009.0);
                }
        s.grid->getBlockCollection().release(info.blockID);
    }
    alignas(Glioma_HG_UQ) static unsigned char storage[sizeof(Glioma_HG_UQ)];
    memset(storage, 0, sizeof storage);
    reinterpret_cast<Glioma_HG_UQ *>(storage)->_dumpUQoutput(*s.grid);
    FILE *f = fopen(outp, "wb");
    if (!f) die("cannot open output");
    fwrite("GBGDMP03", 1, 8, f);
    int32_t hdr[2] = {blocksPerDimension * blockSize, (int32_t)vInfo.size()};
    fwrite(hdr, 4, 2, f);
    for (const BlockInfo &b : vInfo) {
        int32_t bh[5] = {b.blockID, b.level, b.index[0], b.index[1], b.index[2]};
        fwrite(bh, 4, 5, f);
    }
    writeGhostTables(f, *s.grid);
    fclose(f);
    return 0;
}
#endif

static int cmdTiming(const char *inp, int nthreads) {
    Environment::setup(nthreads);
    Input in = readInput(inp);
    Sim s(in.bpd);
    fillGrid(*s.grid, in);
    double secs = 0;
    RunInfo ri = runLoop(s, in, false, &secs);
    double cells = (double)in.n * in.n * in.n;
    printf("{\"steps\": %ld, \"seconds\": %.6f, \"cell_steps_per_s\": %.6e, \"threads\": %d, "
           "\"real_bytes\": %d}\n",
           ri.steps, secs, cells * ri.steps / secs, nthreads, (int)sizeof(Real));
    return 0;
}

int main(int argc, const char **argv) {
    if (argc < 3) die("usage: ref_harness solve|ghosts|fwt|state|mala|dump|dumpgrid|timing <in> [out|nthreads]");
    std::string cmd = argv[1];
    if (cmd == "timing") return cmdTiming(argv[2], argc > 3 ? atoi(argv[3]) : 1);
    Environment::setup(1);
    if (argc < 4) die("missing output path");
    if (cmd == "solve") return cmdSolve(argv[2], argv[3]);
    if (cmd == "ghosts") return cmdGhosts(argv[2], argv[3]);
    if (cmd == "fwt") return cmdFwt(argv[2], argv[3]);
    if (cmd == "state") return cmdState(argv[2], argv[3], argc > 4 ? atoi(argv[4]) : 10);
    if (cmd == "mala") return cmdMala(argv[2], argv[3]);
#ifdef GBG_HARNESS_DUMP
    if (cmd == "dump") return cmdDump(argv[2], argv[3], argc > 4 ? atoi(argv[4]) : 0);
    if (cmd == "dumpgrid") {
        if (argc < 4) die("dumpgrid <out> <r1> [r2 ...]");
        std::vector<double> radii;
        for (int i = 3; i < argc; i++) radii.push_back(atof(argv[i]));
        return cmdDumpGrid(argv[2], radii);
    }
#endif
    die("unknown command");
    return 2;
}
