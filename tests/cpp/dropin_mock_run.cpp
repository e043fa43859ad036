// Runs the drop-in back-end at the reference's call-site shape on a mock MRAG
// grid (16^3 blocks at any levels, FP64).
//
//   dropin_mock_run Dw Dg rho dt < grid
//     grid on stdin: nb, then nb lines "level ix iy iz", then the block-major
//     p_w, p_g and phi (nb * 4096 values each, x fastest inside a block).
//     5 fused steps, a CPU functor (phi *= 2), 3 more fused steps; prints
//     the block-major phi, one double per line.
//   dropin_mock_run Dw Dg rho dt schedule < grid
//     Glioma_HG_UQ::run's loop (t += dt, output every `dt * 2.5` from
//     `dt * 2.5`, tend = 9.5 dt) with HostSync::every_step and with
//     HostSync::at_times: the host blocks at every output time and at the
//     end must agree; prints "schedule ok syncs=<at_times syncs>".
//   dropin_mock_run Dw Dg rho dt steps K < grid
//     K fused steps only; prints the block-major phi.
//   dropin_mock_run Dw Dg rho dt time bpd steps
//     a uniform bpd^3-block grid from the first block of the input, repeated;
//     ms per step with every_step and with at_times (no output time inside).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mock_mrag.h"
#include "gbglioma_blockprocessing.hpp"

typedef gbglioma::BlockProcessing_GPU<Block, MockCPUBackend> BP;

namespace {

struct Grid {
    std::vector<Block> blocks;
    std::vector<BlockInfo> vInfo;
};

bool read_grid(Grid &g) {
    int nb = 0;
    if (scanf("%d", &nb) != 1 || nb <= 0) return false;
    g.blocks.resize(nb);
    for (int b = 0; b < nb; ++b) {
        int l, x, y, z;
        if (scanf("%d %d %d %d", &l, &x, &y, &z) != 4) return false;
        BlockInfo bi;
        bi.blockID = b;
        bi.level = (short)l;
        bi.index[0] = (short)x;
        bi.index[1] = (short)y;
        bi.index[2] = (short)z;
        g.vInfo.push_back(bi);
    }
    for (int f = 0; f < 3; ++f)
        for (int b = 0; b < nb; ++b)
            for (int k = 0; k < 4096; ++k) {
                double v;
                if (scanf("%lf", &v) != 1) return false;
                Cell &c = g.blocks[b].data[k];
                (f == 0 ? c.p_w : f == 1 ? c.p_g : c.phi) = v;
            }
    return true;
}

void step(BP &bp, Grid &g, BlockCollection &coll, double Dw, double Dg, double rho, double dt) {
    BoundaryInfo binfo;
    Glioma_ReactionDiffusionOperator<3> rhs(Dw, Dg, rho);
    UpdateTumor<3> upd(dt);
    bp.pipeline_process(g.vInfo, coll, binfo, rhs);
    BP::process(g.vInfo, coll, upd, 4);
}

std::vector<double> host_phi(const Grid &g) {
    std::vector<double> out;
    for (const Block &b : g.blocks)
        for (const Cell &c : b.data) out.push_back(c.phi);
    return out;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 5) return 2;
    const double Dw = std::atof(argv[1]), Dg = std::atof(argv[2]), rho = std::atof(argv[3]),
                 dt = std::atof(argv[4]);
    const char *mode = argc > 5 ? argv[5] : "";
    Grid g;
    if (!read_grid(g)) return 3;
    if (!std::strcmp(mode, "schedule")) {
        // the run loop twice: host blocks synced every step, and only at the
        // loop's output times and end
        std::vector<std::vector<double>> seen[2];
        long long syncs = 0;
        for (int pass = 0; pass < 2; ++pass) {
            Grid w = g;
            BlockCollection coll{&w.blocks};
            BP bp;
            const double every = 2.5 * dt, tend = 9.5 * dt;
            double whenToWrite = every, t = 0.0;
            if (pass == 1) bp.sync_at(whenToWrite, every, tend);
            while (t <= tend) {
                step(bp, w, coll, Dw, Dg, rho, dt);
                t += dt;
                if (t >= whenToWrite) {
                    seen[pass].push_back(host_phi(w));
                    whenToWrite = whenToWrite + every;
                }
            }
            seen[pass].push_back(host_phi(w));
            if (pass == 1) syncs = bp.host_syncs();
        }
        if (seen[0] != seen[1]) {
            printf("schedule mismatch\n");
            return 1;
        }
        printf("schedule ok syncs=%lld outputs=%zu\n", syncs, seen[1].size());
        return 0;
    }
    if (!std::strcmp(mode, "time")) {
        const int bpd = argc > 6 ? std::atoi(argv[6]) : 8;
        const int steps = argc > 7 ? std::atoi(argv[7]) : 50;
        int level = 0;
        while ((1 << level) < bpd) ++level;
        Grid u;
        for (int z = 0, id = 0; z < bpd; ++z)
            for (int y = 0; y < bpd; ++y)
                for (int x = 0; x < bpd; ++x, ++id) {
                    BlockInfo bi;
                    bi.blockID = id;
                    bi.level = (short)level;
                    bi.index[0] = (short)x;
                    bi.index[1] = (short)y;
                    bi.index[2] = (short)z;
                    u.vInfo.push_back(bi);
                    u.blocks.push_back(g.blocks[0]);
                }
        for (int pass = 0; pass < 2; ++pass) {
            Grid w = u;
            BlockCollection coll{&w.blocks};
            BP bp(pass == 0 ? gbglioma::HostSync::every_step : gbglioma::HostSync::at_times);
            if (pass == 1) bp.sync_at(1e300, 1e300, 1e300);
            step(bp, w, coll, Dw, Dg, rho, dt);  // upload, ghost tables
            auto t0 = std::chrono::steady_clock::now();
            for (int k = 0; k < steps; ++k) step(bp, w, coll, Dw, Dg, rho, dt);
            bp.sync_to_host(w.vInfo, coll);
            auto t1 = std::chrono::steady_clock::now();
            printf("%s %.4f ms/step (%d^3 cells)\n", pass == 0 ? "every_step" : "at_times",
                   std::chrono::duration<double, std::milli>(t1 - t0).count() / steps, bpd * 16);
        }
        return 0;
    }
    BlockCollection coll{&g.blocks};
    BP bp;
    if (!std::strcmp(mode, "steps")) {
        const int K = argc > 6 ? std::atoi(argv[6]) : 1;
        for (int k = 0; k < K; ++k) step(bp, g, coll, Dw, Dg, rho, dt);
        bp.sync_to_host(g.vInfo, coll);
        for (double v : host_phi(g)) printf("%.17g\n", v);
        return 0;
    }
    for (int k = 0; k < 5; ++k) step(bp, g, coll, Dw, Dg, rho, dt);
    DoublePhi twice;
    BP::process(g.vInfo, coll, twice, 4);
    for (int k = 0; k < 3; ++k) step(bp, g, coll, Dw, Dg, rho, dt);
    fprintf(stderr, "gpu_steps=%lld cpu_calls=%d uploads=%lld\n", bp.gpu_steps(), MockCPUBackend::calls(),
            bp.uploads());
    for (double v : host_phi(g)) printf("%.17g\n", v);
    return 0;
}
