// Test infrastructure only: the `-anatomy syntheticData` entry of
// source/Glioma/Glioma_main.cpp reduced to that one driver, so the reference's
// own Glioma_ProcessSyntheticData.cpp (synthetic observations from a tumour
// density: thresholds, PET statistics, noise, normalisation) links without
// the other drivers. Before running it writes `block_order.txt`: the grid's
// blocks (level, ix, iy, iz) in the order its loops visit them, which comes
// from MRAG's node map (ordered by node address) and decides which tumour
// cell receives which random number.
#define private public
#include "Glioma_ProcessSyntheticData.h"
#undef private

#include <cstdio>

int main(int argc, const char **argv) {
    ArgumentParser parser(argc, argv);
    Environment::setup(std::max(1, parser("-nthreads").asInt()));
    Glioma_ProcessSyntheticData *s = new Glioma_ProcessSyntheticData(argc, argv);
    {
        std::vector<BlockInfo> v = s->grid->getBlocksInfo();
        FILE *f = std::fopen("block_order.txt", "w");
        for (size_t i = 0; i < v.size(); ++i)
            std::fprintf(f, "%d %d %d %d\n", v[i].level, v[i].index[0], v[i].index[1], v[i].index[2]);
        std::fclose(f);
    }
    s->run();
    delete s;
    return 0;
}
