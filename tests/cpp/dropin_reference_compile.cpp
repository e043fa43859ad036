// Compile-only check: the drop-in back-end instantiated at the reference's own
// call site types (MRAG Grid, BlockCollection, BoundaryInfo, Glioma operators),
// with the reference's TBB pipeline as the CPU back-end. Built against the
// reference headers where they are present; never run.
#include "Glioma_Types.h"
#include "gbglioma_blockprocessing.hpp"

typedef gbglioma::BlockProcessing_GPU<B, BlockProcessing> GpuBlockProcessing;

void reaction_diffusion_step(Grid<W, B> &grid, BoundaryInfo *boundaryInfo, GpuBlockProcessing &bp,
                             int gran, Real Dw, Real Dg, Real rho, double dt) {
    // the body of Glioma_HG_UQ::_reactionDiffusionStep (Glioma_HG_UQ.cpp:266-277)
    vector<BlockInfo> vInfo = grid.getBlocksInfo();
    const BlockCollection<B> &collecton = grid.getBlockCollection();
    Glioma_ReactionDiffusionOperator<_DIM> rhs(Dw, Dg, rho);
    UpdateTumor<_DIM> updateTumor(dt);
    bp.pipeline_process(vInfo, collecton, *boundaryInfo, rhs);
    GpuBlockProcessing::process(vInfo, collecton, updateTumor, gran);
    // a functor the GPU back-end does not know goes to the CPU back-end
    UpdatePressureSource<_DIM> other(rho);
    GpuBlockProcessing::process(vInfo, collecton, other, gran);
    bp.sync_to_host(vInfo, collecton);
}
