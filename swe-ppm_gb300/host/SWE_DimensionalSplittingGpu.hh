/*
 * SWE_DimensionalSplittingGpu -- a block of the reference's class hierarchy
 * whose step runs on the GB300 through the C ABI (include/swe_gb300.h).
 *
 * Meant to sit in the reference's tree next to
 * src/blocks/SWE_DimensionalSplittingMpi.hh: it derives from the reference's
 * own SWE_Block<Float2DNative> (src/blocks/SWE_Block.hh:110-251) and keeps
 * its interface, so a driver's per-step sequence (setGhostLayer,
 * computeNumericalFluxes, getMaxTimestep, updateUnknowns;
 * src/examples/swe_mpi.cpp:307-316) is unchanged.  The block's Float2D arrays
 * are host mirrors: initScenario samples the scenario there (the reference's
 * own code) and uploads; synchBeforeRead refreshes them from the device
 * before the writer or computeMaxTimestep reads them.  Errors of the library
 * throw std::runtime_error.
 */
#ifndef SWE_DIMENSIONALSPLITTINGGPU_HH
#define SWE_DIMENSIONALSPLITTINGGPU_HH

#include <stdexcept>

#include "blocks/SWE_Block.hh"
#include "swe_gb300.h"
#include "tools/Float2DNative.hh"

class SWE_DimensionalSplittingGpu : public SWE_Block<Float2DNative> {
public:
    /// solver: SWE_SOLVER_*; semantics: SWE_SEMANTICS_UNSPLIT (the MPI blocks)
    /// or SWE_SEMANTICS_SPLIT (the serial block); arithmetic: SWE_ARITH_*
    SWE_DimensionalSplittingGpu(int nx, int ny, float dx, float dy, float originX, float originY,
                                int solver = SWE_SOLVER_HLLE, int semantics = SWE_SEMANTICS_UNSPLIT,
                                int arithmetic = SWE_ARITH_EXACT, int device = 0)
        : SWE_Block<Float2DNative>(nx, ny, dx, dy, originX, originY), solver_(solver), semantics_(semantics),
          arithmetic_(arithmetic), device_(device) {}
    ~SWE_DimensionalSplittingGpu() override {
        if (dom_) swe_gpu_domain_destroy(dom_);
    }

    /// samples the scenario on the host (SWE_Block::initScenario), then
    /// creates the device block and uploads the state and bathymetry
    void initScenario(SWE_Scenario &scenario, BoundaryType boundaries[]) override {
        SWE_Block<Float2DNative>::initScenario(scenario, boundaries);
        if (dom_) swe_gpu_domain_destroy(dom_);
        dom_ = nullptr;
        swe_gpu_desc d{};
        d.blocks_x = d.blocks_y = 1;
        d.nx_cols = &nx;
        d.ny_rows = &ny;
        d.dx = dx;
        d.dy = dy;
        for (int i = 0; i < 4; i++) d.boundary[i] = int(boundaryType[i]);
        d.solver = solver_;
        d.semantics = semantics_;
        d.arithmetic = arithmetic_;
        d.device = device_;
        check(swe_gpu_domain_create(&d, &dom_));
        upload();
    }

    /// the host arrays (after the caller changed them) back to the device
    void upload() {
        check(swe_gpu_upload_block(dom_, 0, h.getRawPointer(), hu.getRawPointer(), hv.getRawPointer(),
                                   b.getRawPointer(), ny + 2));
        check(swe_gpu_exchange_bathymetry(dom_));
    }

    void setGhostLayer() { check(swe_gpu_set_ghost_layer(dom_)); }

    void computeNumericalFluxes() override {
        check(swe_gpu_compute_fluxes(dom_));
        check(swe_gpu_get_max_timestep(dom_, &maxTimestep));
    }

    void updateUnknowns(float dt) override { check(swe_gpu_update_unknowns(dom_, dt)); }

    /// refreshes the host arrays (h, hu, hv with their ghosts) from the device
    void synchBeforeRead() {
        check(swe_gpu_download_block(dom_, 0, h.getRawPointer(), hu.getRawPointer(), hv.getRawPointer(), nullptr,
                                     ny + 2));
    }

    swe_gpu_domain *domain() { return dom_; }

private:
    static void check(int rc) {
        if (rc) throw std::runtime_error(swe_gpu_last_error());
    }
    swe_gpu_domain *dom_ = nullptr;
    int solver_, semantics_, arithmetic_, device_;
};

#endif
