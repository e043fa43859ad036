// Runs the drop-in back-end at the reference's call-site shape on a mock MRAG
// grid (2^3 blocks of 16^3, FP64) and prints phi after: 5 fused steps, a CPU
// functor (phi *= 2), 3 more fused steps. Prints one double per line.
#include <cmath>
#include <cstdio>
#include <vector>

#include "mock_mrag.h"
#include "gbglioma_blockprocessing.hpp"

typedef gbglioma::BlockProcessing_GPU<Block, MockCPUBackend> BP;

int main(int argc, char **argv) {
    const int bpd = 2, n = 32;
    std::vector<Block> blocks(bpd * bpd * bpd);
    std::vector<BlockInfo> vInfo;
    for (int bz = 0; bz < bpd; bz++)
        for (int by = 0; by < bpd; by++)
            for (int bx = 0; bx < bpd; bx++) {
                BlockInfo bi;
                bi.blockID = bx + bpd * (by + bpd * bz);
                bi.index[0] = bx; bi.index[1] = by; bi.index[2] = bz;
                bi.level = 1;
                vInfo.push_back(bi);
            }
    // read the initial fields (x fastest) from stdin: p_w, p_g, phi
    std::vector<double> f(3 * n * n * n);
    for (auto &v : f)
        if (scanf("%lf", &v) != 1) return 3;
    for (auto &bi : vInfo)
        for (int iz = 0; iz < 16; iz++)
            for (int iy = 0; iy < 16; iy++)
                for (int ix = 0; ix < 16; ix++) {
                    size_t g = (bi.index[0] * 16 + ix) + n * ((bi.index[1] * 16 + iy) + (size_t)n * (bi.index[2] * 16 + iz));
                    Cell &c = blocks[bi.blockID](ix, iy, iz);
                    c.p_w = f[g];
                    c.p_g = f[n * n * n + g];
                    c.phi = f[2 * n * n * n + g];
                }
    BlockCollection coll{&blocks};
    BoundaryInfo binfo;
    BP bp;
    const double Dw = std::atof(argv[1]), Dg = std::atof(argv[2]), rho = std::atof(argv[3]),
                 dt = std::atof(argv[4]);
    auto step = [&]() {
        Glioma_ReactionDiffusionOperator<3> rhs(Dw, Dg, rho);
        UpdateTumor<3> upd(dt);
        bp.pipeline_process(vInfo, coll, binfo, rhs);
        BP::process(vInfo, coll, upd, 4);
    };
    for (int k = 0; k < 5; ++k) step();
    DoublePhi twice;
    BP::process(vInfo, coll, twice, 4);
    for (int k = 0; k < 3; ++k) step();
    fprintf(stderr, "gpu_steps=%lld cpu_calls=%d\n", bp.gpu_steps(), MockCPUBackend::calls());
    for (int gz = 0; gz < n; gz++)
        for (int gy = 0; gy < n; gy++)
            for (int gx = 0; gx < n; gx++) {
                const BlockInfo &bi = vInfo[(gx / 16) + bpd * ((gy / 16) + bpd * (gz / 16))];
                printf("%.17g\n", blocks[bi.blockID](gx % 16, gy % 16, gz % 16).phi);
            }
    return 0;
}
