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
//  * pipeline_process with Glioma_ReactionDiffusionOperator<3> on a uniform
//    grid (every block at one level) records Dw, Dg and rho; the following
//    process with UpdateTumor<3> runs both as one fused step on the GPU
//    (gbg_rd_step) in the precision of Real: GBG_PREC_F64 for double,
//    GBG_PREC_F32REF for float, bit-identical to the CPU back-end either way.
//  * Any other functor, or a grid with more than one level, runs on the CPU
//    back-end given as the second template argument, after the GPU state has
//    been copied back into the blocks -- results never silently change.
//  * After every fused step the new phi is copied back into the blocks
//    (HostSync::every_step, the default), so code that reads the grid
//    (regridding, dumps) sees current values. With HostSync::on_demand the
//    blocks are updated only by sync_to_host(), which the caller must call
//    before reading them; the device then keeps the state between steps.
//  * dphidt is not written back: the fused step keeps the rates on the GPU.
//  * The anatomy (p_w, p_g) and phi are uploaded at the first fused step and
//    again whenever the set of blocks changes or a CPU-run functor may have
//    modified them; between fused steps the GPU copy is authoritative, so code
//    that writes the blocks directly calls invalidate() afterwards.
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

enum class HostSync { every_step, on_demand };

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
    explicit BlockProcessing_GPU(HostSync sync = HostSync::every_step, int device = 0)
        : sync_(sync), device_(device) {}
    ~BlockProcessing_GPU() {
        if (current() == this) current() = nullptr;
        if (h_) gbg_destroy(h_);
    }
    BlockProcessing_GPU(const BlockProcessing_GPU &) = delete;
    BlockProcessing_GPU &operator=(const BlockProcessing_GPU &) = delete;

    template <typename Processing, typename Collection, typename Info, typename Boundary>
    void pipeline_process(std::vector<Info> &vInfo, Collection &c, Boundary &b, Processing &p) {
        current() = this;
        if (is_rd_rhs<Processing>::value && uniform(vInfo)) {
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
        check(gbg_get_phi(h_, phi_.data()), "gbg_get_phi");
        scatter(vInfo, c);
        host_stale_ = false;
    }

    // Call after changing the blocks' phi, p_w or p_g directly: the next fused
    // step uploads them again.
    void invalidate() { device_valid_ = false; host_stale_ = false; }

    long long gpu_steps() const { return steps_; }

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

    template <typename Info>
    static bool uniform(const std::vector<Info> &vInfo) {
        if (vInfo.empty()) return false;
        const int l = vInfo[0].level;
        for (size_t i = 1; i < vInfo.size(); ++i)
            if (vInfo[i].level != l) return false;
        const size_t side = (size_t)1 << l;
        return vInfo.size() == side * side * side;
    }

    template <typename Info>
    bool matches(const std::vector<Info> &vInfo) const {
        if (ids_.size() != vInfo.size()) return false;
        for (size_t i = 0; i < vInfo.size(); ++i)
            if (ids_[i] != vInfo[i].blockID) return false;
        return true;
    }

    template <typename Info>
    size_t cell(const Info &info, int ix, int iy, int iz) const {
        const size_t gx = (size_t)info.index[0] * BlockType::sizeX + ix;
        const size_t gy = (size_t)info.index[1] * BlockType::sizeY + iy;
        const size_t gz = (size_t)info.index[2] * BlockType::sizeZ + iz;
        return gx + (size_t)n_ * (gy + (size_t)n_ * gz);
    }

    template <typename Info, typename Collection>
    void gather(std::vector<Info> &vInfo, Collection &c) {
        for (const Info &info : vInfo) {
            BlockType &b = c[info.blockID];
            for (int iz = 0; iz < BlockType::sizeZ; iz++)
                for (int iy = 0; iy < BlockType::sizeY; iy++)
                    for (int ix = 0; ix < BlockType::sizeX; ix++) {
                        const size_t g = cell(info, ix, iy, iz);
                        pw_[g] = (double)b(ix, iy, iz).p_w;
                        pg_[g] = (double)b(ix, iy, iz).p_g;
                        phi_[g] = (double)b(ix, iy, iz).phi;
                    }
        }
    }

    template <typename Info, typename Collection>
    void scatter(std::vector<Info> &vInfo, Collection &c) {
        typedef typename std::remove_reference<decltype(c[0](0, 0, 0).phi)>::type RealT;
        for (const Info &info : vInfo) {
            BlockType &b = c[info.blockID];
            for (int iz = 0; iz < BlockType::sizeZ; iz++)
                for (int iy = 0; iy < BlockType::sizeY; iy++)
                    for (int ix = 0; ix < BlockType::sizeX; ix++)
                        b(ix, iy, iz).phi = (RealT)phi_[cell(info, ix, iy, iz)];
        }
    }

    template <typename Info, typename Collection>
    void ensure_device(std::vector<Info> &vInfo, Collection &c) {
        if (device_valid_ && matches(vInfo)) return;
        const int l = vInfo[0].level;
        const int n = (1 << l) * BlockType::sizeX;
        if (BlockType::sizeX != BlockType::sizeY || BlockType::sizeX != BlockType::sizeZ)
            throw std::invalid_argument("BlockProcessing_GPU needs cubic blocks");
        typedef typename std::remove_reference<decltype(c[0](0, 0, 0).phi)>::type RealT;
        const int prec = sizeof(RealT) == sizeof(double) ? GBG_PREC_F64 : GBG_PREC_F32REF;
        if (!h_ || n != n_ || prec != prec_) {
            if (h_) gbg_destroy(h_);
            h_ = nullptr;
            gbg_config cfg = {n, prec, device_, 0};
            check(gbg_create(&cfg, &h_), "gbg_create");
            n_ = n;
            prec_ = prec;
        }
        const size_t N = (size_t)n * n * n;
        pw_.assign(N, 0.0);
        pg_.assign(N, 0.0);
        phi_.assign(N, 0.0);
        gather(vInfo, c);
        check(gbg_set_anatomy(h_, pw_.data(), pg_.data()), "gbg_set_anatomy");
        check(gbg_set_phi(h_, phi_.data()), "gbg_set_phi");
        ids_.clear();
        for (const Info &info : vInfo) ids_.push_back(info.blockID);
        device_valid_ = true;
        host_stale_ = false;
    }

    template <typename Info, typename Collection>
    void fused_step(std::vector<Info> &vInfo, Collection &c, double dt) {
        check(gbg_rd_step(h_, Dw_, Dg_, rho_, dt, 1), "gbg_rd_step");
        pending_ = false;
        host_stale_ = true;
        ++steps_;
        if (sync_ == HostSync::every_step) sync_to_host(vInfo, c);
    }

    CPUBackend cpu_;
    HostSync sync_;
    int device_;
    gbg_handle *h_ = nullptr;
    int n_ = 0, prec_ = -1;
    std::vector<int> ids_;
    std::vector<double> pw_, pg_, phi_;
    bool device_valid_ = false, host_stale_ = false, pending_ = false;
    double Dw_ = 0, Dg_ = 0, rho_ = 0;
    long long steps_ = 0;
};

}  // namespace gbglioma
