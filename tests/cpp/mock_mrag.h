// Minimal stand-ins for the MRAG types the drop-in back-end touches (BlockInfo,
// Block, BlockCollection, BoundaryInfo) and for the two Glioma operator
// templates, with the reference's member names. Used to run the back-end on a
// GPU where the reference tree is not available. The operator bodies are not
// needed: the GPU back-end only reads their parameters.
#pragma once
#include <vector>

struct Cell {
    double phi = 0, dphidt = 0, p_g = 0, p_w = 0;
};

struct BlockInfo {
    int blockID;
    short index[3];
    short level;
};

struct Block {
    static const int sizeX = 16, sizeY = 16, sizeZ = 16;
    Cell data[16 * 16 * 16];
    Cell &operator()(int ix, int iy, int iz) { return data[ix + 16 * (iy + 16 * iz)]; }
};

struct BlockCollection {
    std::vector<Block> *blocks;
    Block &operator[](int id) const { return (*blocks)[id]; }
};

struct BoundaryInfo {};

template <int nDim = 3>
struct Glioma_ReactionDiffusionOperator {
    int stencil_start[3], stencil_end[3];
    const double Dw, Dg, rho;
    Glioma_ReactionDiffusionOperator(double a, double b, double c) : Dw(a), Dg(b), rho(c) {}
};

template <int nDim = 3>
struct UpdateTumor {
    double dt;
    explicit UpdateTumor(double d) : dt(d) {}
};

// a functor the GPU back-end does not know: doubles phi
struct DoublePhi {};

// CPU back-end stand-in: runs DoublePhi on the host and counts its calls
struct MockCPUBackend {
    static int &calls() {
        static int c = 0;
        return c;
    }
    template <typename P>
    void pipeline_process(std::vector<BlockInfo> &, const BlockCollection &, BoundaryInfo &, P &) {
        ++calls();
    }
    template <typename P>
    static void process(std::vector<BlockInfo> &, const BlockCollection &, P &, int) {
        ++calls();
    }
    static void process(std::vector<BlockInfo> &vInfo, const BlockCollection &c, DoublePhi &, int) {
        ++calls();
        for (auto &info : vInfo)
            for (auto &cell : c[info.blockID].data) cell.phi *= 2.0;
    }
};
