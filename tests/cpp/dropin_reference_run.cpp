// CPU wiring check of the drop-in back-end on the reference's own types: two
// Grid<W,B> of 2^3 blocks filled alike; one steps through Glioma_HG_UQ's
// _reactionDiffusionStep body (Glioma_HG_UQ.cpp:266-277) with the reference's
// BlockProcessing (its TBB pipeline), the other through the same body with
// BlockProcessing_GPU over a CPU stand-in of the library
// (gbg_amr_cpu_stub.cpp). 5 steps, a functor the back-end does not know
// (run on the reference's pipeline after a host sync), 5 more steps, then the
// two grids' phi must be equal bit for bit. Prints "equal <cells> calls ...".
// With the argument "schedule": Glioma_HG_UQ::run's loop (t += dt, output
// times every 2.5 dt, tend = 9.5 dt) with HostSync::at_times on the drop-in
// grid; the grids must agree at every output time and at the end, with one
// read-back per output time.
#include "Glioma_Types.h"
#include "gbglioma_blockprocessing.hpp"

#include <cstdio>
#include <string>

extern "C" int stub_calls(int i);

typedef gbglioma::BlockProcessing_GPU<B, BlockProcessing> GpuBlockProcessing;

static int maxStencilH[2][3] = {{-1, -1, -1}, {+2, +2, +2}};

static void fill(Grid<W, B> &grid) {
    vector<BlockInfo> vInfo = grid.getBlocksInfo();
    for (size_t i = 0; i < vInfo.size(); i++) {
        BlockInfo &info = vInfo[i];
        B &b = grid.getBlockCollection()[info.blockID];
        for (int iz = 0; iz < B::sizeZ; iz++)
            for (int iy = 0; iy < B::sizeY; iy++)
                for (int ix = 0; ix < B::sizeX; ix++) {
                    const int gx = info.index[0] * 16 + ix, gy = info.index[1] * 16 + iy,
                              gz = info.index[2] * 16 + iz;
                    const double r2 = (gx - 15.3) * (gx - 15.3) + (gy - 16.2) * (gy - 16.2) +
                                      (gz - 14.7) * (gz - 14.7);
                    const bool brain = r2 < 14.0 * 14.0;
                    const double w = ((gx * 7 + gy * 13 + gz * 29) % 17) / 16.0;
                    b(ix, iy, iz).p_w = (Real)(brain ? w : 0.0);
                    b(ix, iy, iz).p_g = (Real)(brain ? 1.0 - w : 0.0);
                    b(ix, iy, iz).phi = (Real)(r2 < 9.0 ? 0.1 * (1.0 - r2 / 9.0) : 0.0);
                }
        grid.getBlockCollection().release(info.blockID);
    }
}

template <typename BP>
static void rd_step(Grid<W, B> &grid, BP &bp, Real Dw, Real Dg, Real rho, double dt) {
    vector<BlockInfo> vInfo = grid.getBlocksInfo();
    const BlockCollection<B> &collecton = grid.getBlockCollection();
    Glioma_ReactionDiffusionOperator<_DIM> rhs(Dw, Dg, rho);
    UpdateTumor<_DIM> updateTumor(dt);
    bp.pipeline_process(vInfo, collecton, grid.getBoundaryInfo(), rhs);
    BP::process(vInfo, collecton, updateTumor, 1);
}

template <typename BP>
static void other(Grid<W, B> &grid) {
    vector<BlockInfo> vInfo = grid.getBlocksInfo();
    const BlockCollection<B> &collecton = grid.getBlockCollection();
    UpdateTumor<_DIM> half(0.5);  // a plain update with the rates left in dphidt
    BP::process(vInfo, collecton, half, 1);
}

// phi of the two grids, blocks matched by level and position: the number of
// cells that differ (-1: the block sets differ); *cells and *maxphi set
static long compare(Grid<W, B> &ref, Grid<W, B> &mine, long *cells_out, double *maxphi_out) {
    vector<BlockInfo> a = ref.getBlocksInfo(), b = mine.getBlocksInfo();
    long cells = 0, diff = 0;
    double maxphi = 0;
    if (a.size() != b.size()) return -1;
    for (size_t i = 0; i < a.size(); i++) {
        size_t j = 0;
        while (j < b.size() && !(b[j].level == a[i].level && b[j].index[0] == a[i].index[0] &&
                                 b[j].index[1] == a[i].index[1] && b[j].index[2] == a[i].index[2]))
            ++j;
        if (j == b.size()) return -1;
        B &x = ref.getBlockCollection()[a[i].blockID];
        B &y = mine.getBlockCollection()[b[j].blockID];
        for (int iz = 0; iz < B::sizeZ; iz++)
            for (int iy = 0; iy < B::sizeY; iy++)
                for (int ix = 0; ix < B::sizeX; ix++) {
                    ++cells;
                    if (x(ix, iy, iz).phi != y(ix, iy, iz).phi) ++diff;
                    if (x(ix, iy, iz).phi > maxphi) maxphi = x(ix, iy, iz).phi;
                }
    }
    *cells_out = cells;
    *maxphi_out = maxphi;
    return diff;
}

int main(int argc, char **argv) {
    Environment::setup(1);
    Grid<W, B> ref(2, 2, 2, maxStencilH), mine(2, 2, 2, maxStencilH);
    fill(ref);
    fill(mine);
    const double L = 6.4, h = 1.0 / 32;
    const Real Dw = (Real)(0.0013 / (L * L)), Dg = (Real)(0.1 * Dw), rho = (Real)0.15;
    const double dt = 0.99 * h * h / (2. * _DIM * Dw);
    BlockProcessing ref_bp;
    GpuBlockProcessing gpu_bp;
    if (argc > 1 && std::string(argv[1]) == "schedule") {
        const double every = 2.5 * dt, tend = 9.5 * dt;
        double t = 0.0, whenToWrite = every;
        gpu_bp.sync_at(whenToWrite, every, tend);
        int outputs = 0;
        long cells = 0, bad = 0;
        double maxphi = 0;
        while (t <= tend) {
            rd_step(ref, ref_bp, Dw, Dg, rho, dt);
            rd_step(mine, gpu_bp, Dw, Dg, rho, dt);
            t += dt;
            if (t >= whenToWrite) {
                // where the run loop regrids and dumps: the host blocks are current
                if (compare(ref, mine, &cells, &maxphi) != 0) ++bad;
                ++outputs;
                whenToWrite = whenToWrite + every;
            }
        }
        if (compare(ref, mine, &cells, &maxphi) != 0) ++bad;  // _dumpUQoutput after the loop
        printf("%s outputs=%d syncs=%lld steps=%lld maxphi=%.9g\n", bad ? "differ" : "schedule ok", outputs,
               gpu_bp.host_syncs(), gpu_bp.gpu_steps(), maxphi);
        return bad ? 1 : 0;
    }
    for (int k = 0; k < 5; ++k) {
        rd_step(ref, ref_bp, Dw, Dg, rho, dt);
        rd_step(mine, gpu_bp, Dw, Dg, rho, dt);
    }
    // UpdateTumor outside the RD pair: the reference pipeline runs it on both
    // grids (the drop-in first syncs its blocks); dphidt holds the last
    // step's rates on the reference grid only, so zero it on both first
    for (Grid<W, B> *g : {&ref, &mine}) {
        vector<BlockInfo> vInfo = g->getBlocksInfo();
        for (size_t i = 0; i < vInfo.size(); i++) {
            B &b = g->getBlockCollection()[vInfo[i].blockID];
            for (int iz = 0; iz < B::sizeZ; iz++)
                for (int iy = 0; iy < B::sizeY; iy++)
                    for (int ix = 0; ix < B::sizeX; ix++) b(ix, iy, iz).dphidt = 0;
        }
    }
    other<BlockProcessing>(ref);
    other<GpuBlockProcessing>(mine);
    for (int k = 0; k < 5; ++k) {
        rd_step(ref, ref_bp, Dw, Dg, rho, dt);
        rd_step(mine, gpu_bp, Dw, Dg, rho, dt);
    }
    {
        vector<BlockInfo> vInfo = mine.getBlocksInfo();
        gpu_bp.sync_to_host(vInfo, mine.getBlockCollection());
    }
    long cells = 0;
    double maxphi = 0;
    const long diff = compare(ref, mine, &cells, &maxphi);
    printf("%s %ld diff=%ld maxphi=%.9g steps=%lld uploads=%lld calls=%d,%d,%d,%d real=%zu\n",
           diff ? "differ" : "equal", cells, diff, maxphi, gpu_bp.gpu_steps(), gpu_bp.uploads(), stub_calls(0),
           stub_calls(1), stub_calls(2), stub_calls(3), sizeof(Real));
    return diff ? 1 : 0;
}
