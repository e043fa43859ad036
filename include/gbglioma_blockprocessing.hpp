// Drop-in GPU back-end for MRAG's block processing on GliomaUQ's RD step.
//
// Replaces the type selected by the BlockProcessing typedef
// (source/Glioma/Glioma_Types.h:473-479) so that Glioma_HG_UQ's call site
// (source/Glioma/Glioma_HG_UQ.cpp:266-277)
//
//     blockProcessing.pipeline_process(vInfo, collection, *boundaryInfo, rhs);
//     BlockProcessing::process(vInfo, collection, updateTumor, granularity);
//
// stays as it is. The interface mirrors BlockProcessing_Pipeline_TBB
// (source/MRAGmultithreading/MRAGBlockProcessing_TBB.h:447-512): a member
// pipeline_process(vInfo, collection, boundaryInfo, functor) and a static
// process(vInfo, collection, functor, granularity).
//
// What runs where:
//  * pipeline_process with Glioma_ReactionDiffusionOperator<3> records Dw,
//    Dg and rho; the following process with UpdateTumor<3> runs both as one
//    step of the library's block grid (gbg_amr_step) in the precision of
//    Real: GBG_PREC_F64 for double, GBG_PREC_F32REF for float, bit-identical
//    to the CPU back-end either way, on a uniform grid or one with blocks at
//    several levels (the ghost cells of resolution jumps come from the
//    library's own ghost-table compiler, gbg_amr_build_ghosts).
//  * Any other functor runs on the CPU back-end given as the second template
//    argument, after the GPU state has been copied back into the blocks --
//    results never silently change.
//  * The fields live on the device block-major, the layout of the blocks
//    themselves: an upload or a read-back is one pass over each block's
//    cells, no reordering into a global array.
//  * When the host blocks get the device's phi (HostSync):
//      every_step  after every fused step (the default: correct for any
//                  caller, which may read the grid at any time);
//      at_times    only where the run loop reads the grid: after the step at
//                  which the loop's time reaches its next output time (where
//                  Glioma_HG_UQ::run regrids and dumps) and after the step
//                  that ends the loop (the final refinement and
//                  _dumpUQoutput). sync_at(whenToWrite, whenToWriteOffset,
//                  tend) mirrors the loop's own bookkeeping in the same
//                  double arithmetic (Glioma_HG_UQ.cpp:541-566);
//      on_demand   only by sync_to_host(), which the caller must call
//                  before reading the blocks.
//  * dphidt is not written back: the fused step keeps the rates on the GPU.
//  * The anatomy (p_w, p_g) and phi are uploaded at the first fused step and
//    again whenever the blocks change (their IDs, levels or positions) or a
//    CPU-run functor may have modified them; between fused steps the GPU copy
//    is authoritative, so code that writes the blocks directly calls
//    invalidate() afterwards.
//
// Requires gbglioma.h and linking libgbglioma. The operator templates are
// matched by name; they are declared (not defined) here so this header can be
// included before or after source/Glioma/Glioma_ReactionDiffusionOperator.h.
#pragma once

#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "gbglioma.h"

template <int nDim> struct Glioma_ReactionDiffusionOperator;
template <int nDim> struct UpdateTumor;

namespace gbglioma {

enum class HostSync { every_step, at_times, on_demand };

template <typename P> struct is_rd_rhs { static const bool value = false; };
template <> struct is_rd_rhs<Glioma_ReactionDiffusionOperator<3> > { static const bool value = true; };
template <> struct is_rd_rhs<const Glioma_ReactionDiffusionOperator<3> > { static const bool value = true; };
template <typename P> struct is_rd_update { static const bool value = false; };
template <> struct is_rd_update<UpdateTumor<3> > { static const bool value = true; };
template <> struct is_rd_update<const UpdateTumor<3> > { static const bool value = true; };

class GpuError : public std::runtime_error {
public:
    GpuError(int status, const std::string &what)
        : std::runtime_error(what + ": " + gbg_last_error()), status(status) {}
    int status;
};

template <typename BlockType, typename CPUBackend>
class BlockProcessing_GPU {
public:
    static const int kCells = BlockType::sizeX * BlockType::sizeY * BlockType::sizeZ;

    explicit BlockProcessing_GPU(HostSync sync = HostSync::every_step, int device = 0)
        : sync_(sync), device_(device) {}
    ~BlockProcessing_GPU() {
        if (current() == this) current() = nullptr;
        if (h_) gbg_destroy(h_);
    }
    BlockProcessing_GPU(const BlockProcessing_GPU &) = delete;
    BlockProcessing_GPU &operator=(const BlockProcessing_GPU &) = delete;

    // HostSync::at_times with the run loop's schedule: its first output time
    // (whenToWrite), the interval (whenToWriteOffset) and its end time (tend);
    // the loop's time starts at 0 here.
    void sync_at(double first, double every, double tend) {
        sync_ = HostSync::at_times;
        t_ = 0.0;
        next_ = first;
        every_ = every;
        tend_ = tend;
    }

    template <typename Processing, typename Collection, typename Info, typename Boundary>
    void pipeline_process(std::vector<Info> &vInfo, Collection &c, Boundary &b, Processing &p) {
        current() = this;
        if (is_rd_rhs<Processing>::value && !vInfo.empty()) {
            ensure_device(vInfo, c);
            pending_ = true;
            Dw_ = (double)rhs_Dw(p);
            Dg_ = (double)rhs_Dg(p);
            rho_ = (double)rhs_rho(p);
            return;
        }
        sync_to_host(vInfo, c);
        pending_ = false;
        cpu_.pipeline_process(vInfo, c, b, p);
        device_valid_ = false;
    }

    template <typename Processing, typename Collection, typename Info>
    static void process(std::vector<Info> &vInfo, Collection &c, Processing &p,
                        int nGranularity = -1) {
        BlockProcessing_GPU *self = current();
        if (self && is_rd_update<Processing>::value && self->pending_ && self->device_valid_ &&
            self->matches(vInfo)) {
            self->fused_step(vInfo, c, (double)update_dt(p));
            return;
        }
        if (self) {
            self->sync_to_host(vInfo, c);
            self->pending_ = false;
            self->device_valid_ = false;
        }
        CPUBackend::process(vInfo, c, p, nGranularity);
    }

    // Copy the GPU's phi into the blocks if the device is ahead of them.
    template <typename Collection, typename Info>
    void sync_to_host(std::vector<Info> &vInfo, Collection &c) {
        if (!host_stale_ || !device_valid_ || !matches(vInfo)) return;
        check(gbg_amr_get_phi(h_, phi_.data()), "gbg_amr_get_phi");
        scatter(vInfo, c);
        host_stale_ = false;
        ++syncs_;
    }

    // Call after changing the blocks' phi, p_w or p_g directly: the next fused
    // step uploads them again.
    void invalidate() { device_valid_ = false; host_stale_ = false; }

    long long gpu_steps() const { return steps_; }
    long long host_syncs() const { return syncs_; }
    long long uploads() const { return uploads_; }

private:
    // Member access kept in one place: Glioma_ReactionDiffusionOperator has
    // const Real Dw, Dg, rho; UpdateTumor has double dt.
    template <typename P> static auto rhs_Dw(const P &p) -> decltype(p.Dw) { return p.Dw; }
    template <typename P> static auto rhs_Dg(const P &p) -> decltype(p.Dg) { return p.Dg; }
    template <typename P> static auto rhs_rho(const P &p) -> decltype(p.rho) { return p.rho; }
    static double rhs_Dw(...) { return 0; }
    static double rhs_Dg(...) { return 0; }
    static double rhs_rho(...) { return 0; }
    template <typename P> static auto update_dt(const P &p) -> decltype(p.dt) { return p.dt; }
    static double update_dt(...) { return 0; }

    static BlockProcessing_GPU *&current() {
        static BlockProcessing_GPU *c = nullptr;
        return c;
    }

    static void check(int rc, const char *what) {
        if (rc != GBG_OK) throw GpuError(rc, what);
    }

    // the blocks the device holds, in the order of vInfo: IDs, levels and
    // positions must all agree (a regrid can reuse an ID elsewhere)
    template <typename Info>
    bool matches(const std::vector<Info> &vInfo) const {
        if (ids_.size() != vInfo.size()) return false;
        for (size_t i = 0; i < vInfo.size(); ++i) {
            const gbg_block &g = grid_[i];
            const Info &info = vInfo[i];
            if (ids_[i] != info.blockID || g.level != info.level || g.ix != info.index[0] ||
                g.iy != info.index[1] || g.iz != info.index[2])
                return false;
        }
        return true;
    }

    static size_t local(int ix, int iy, int iz) {
        return (size_t)ix + (size_t)BlockType::sizeX * ((size_t)iy + (size_t)BlockType::sizeY * iz);
    }

    template <typename Info, typename Collection>
    void gather(std::vector<Info> &vInfo, Collection &c) {
        for (size_t i = 0; i < vInfo.size(); ++i) {
            BlockType &b = c[vInfo[i].blockID];
            double *pw = pw_.data() + i * kCells, *pg = pg_.data() + i * kCells,
                   *phi = phi_.data() + i * kCells;
            for (int iz = 0; iz < BlockType::sizeZ; iz++)
                for (int iy = 0; iy < BlockType::sizeY; iy++)
                    for (int ix = 0; ix < BlockType::sizeX; ix++) {
                        const size_t k = local(ix, iy, iz);
                        pw[k] = (double)b(ix, iy, iz).p_w;
                        pg[k] = (double)b(ix, iy, iz).p_g;
                        phi[k] = (double)b(ix, iy, iz).phi;
                    }
        }
    }

    template <typename Info, typename Collection>
    void scatter(std::vector<Info> &vInfo, Collection &c) {
        typedef typename std::remove_reference<decltype(c[0](0, 0, 0).phi)>::type RealT;
        for (size_t i = 0; i < vInfo.size(); ++i) {
            BlockType &b = c[vInfo[i].blockID];
            const double *phi = phi_.data() + i * kCells;
            for (int iz = 0; iz < BlockType::sizeZ; iz++)
                for (int iy = 0; iy < BlockType::sizeY; iy++)
                    for (int ix = 0; ix < BlockType::sizeX; ix++)
                        b(ix, iy, iz).phi = (RealT)phi[local(ix, iy, iz)];
        }
    }

    template <typename Info, typename Collection>
    void ensure_device(std::vector<Info> &vInfo, Collection &c) {
        if (device_valid_ && matches(vInfo)) return;
        if (BlockType::sizeX != 16 || BlockType::sizeY != 16 || BlockType::sizeZ != 16)
            throw std::invalid_argument("BlockProcessing_GPU needs 16^3 blocks");
        typedef typename std::remove_reference<decltype(c[0](0, 0, 0).phi)>::type RealT;
        const int prec = sizeof(RealT) == sizeof(double) ? GBG_PREC_F64 : GBG_PREC_F32REF;
        const int nb = (int)vInfo.size();
        if (!h_ || nb > capacity_ || prec != prec_) {
            if (h_) gbg_destroy(h_);
            h_ = nullptr;
            const int cap = nb > 2 * capacity_ ? nb : 2 * capacity_;
            gbg_amr_config cfg = {cap, prec, device_};
            check(gbg_amr_create(&cfg, &h_), "gbg_amr_create");
            capacity_ = cap;
            prec_ = prec;
        }
        grid_.resize(nb);
        ids_.resize(nb);
        for (int i = 0; i < nb; ++i) {
            const Info &info = vInfo[i];
            grid_[i] = {(int)info.level, (int)info.index[0], (int)info.index[1], (int)info.index[2]};
            ids_[i] = info.blockID;
        }
        const size_t cells = (size_t)nb * kCells;
        pw_.resize(cells);
        pg_.resize(cells);
        phi_.resize(cells);
        gather(vInfo, c);
        check(gbg_amr_set_grid(h_, nb, grid_.data(), pw_.data(), pg_.data(), phi_.data()),
              "gbg_amr_set_grid");
        check(gbg_amr_build_ghosts(h_), "gbg_amr_build_ghosts");
        device_valid_ = true;
        host_stale_ = false;
        ++uploads_;
    }

    template <typename Info, typename Collection>
    void fused_step(std::vector<Info> &vInfo, Collection &c, double dt) {
        check(gbg_amr_step(h_, Dw_, Dg_, rho_, dt, 1), "gbg_amr_step");
        pending_ = false;
        host_stale_ = true;
        ++steps_;
        if (sync_ == HostSync::every_step) {
            sync_to_host(vInfo, c);
        } else if (sync_ == HostSync::at_times) {
            t_ += dt;  // the run loop's t += dt
            bool now = false;
            if (t_ >= next_) {
                now = true;
                next_ = next_ + every_;
            }
            if (!(t_ <= tend_)) now = true;  // the loop ends after this step
            if (now) sync_to_host(vInfo, c);
        }
    }

    CPUBackend cpu_;
    HostSync sync_;
    int device_;
    gbg_handle *h_ = nullptr;
    int capacity_ = 0, prec_ = -1;
    std::vector<int> ids_;
    std::vector<gbg_block> grid_;
    std::vector<double> pw_, pg_, phi_;
    bool device_valid_ = false, host_stale_ = false, pending_ = false;
    double Dw_ = 0, Dg_ = 0, rho_ = 0;
    double t_ = 0, next_ = 0, every_ = 0, tend_ = 0;
    long long steps_ = 0, syncs_ = 0, uploads_ = 0;
};

}  // namespace gbglioma
