/**
 * ORACLE — test infrastructure only.  Harness compiled TOGETHER WITH the
 * reference's own sources (see oracle/ref/Makefile; the sources stay where
 * they lie and nothing of them is copied): it drives the reference's
 * SWE_DimensionalSplittingMpi, SWE_DimensionalSplittingMPIOverdecomp and
 * SWE_DimensionalSplitting blocks and its SWE_Block::initScenario through a
 * small C interface, so tests can pin the oracle (and, through it, the CUDA
 * path) against the reference's compiled block code and write golden vectors.
 * The solver headers come from oracle/solvers (the original module is absent).
 *
 * Array exchange format: per block (nx+2)*(ny+2) floats in Float2D layout
 * a[x][y] = raw[x*(ny+2)+y]; blocks concatenated in rank order.
 */
#include <array>
#include <cstring>
#include <memory>
#include <vector>

#include "blocks/SWE_DimensionalSplitting.hh"
#include "blocks/SWE_DimensionalSplittingMPIOverdecomp.hh"
#include "blocks/SWE_DimensionalSplittingMpi.hh"
#include "scenarios/SWE_simple_scenarios.hh"

#include "scenarios.hpp"  // the library's synthetic scenarios (host code)

namespace {

/// Presents a library scenario through the reference's SWE_Scenario interface.
class Adapter : public SWE_Scenario {
public:
    explicit Adapter(swegb::Scenario *s) : s_(s) {}
    float getWaterHeight(float x, float y) override { return s_->getWaterHeight(x, y); }
    float getBathymetry(float x, float y) override { return s_->getBathymetry(x, y); }
    float getVeloc_u(float x, float y) override { return s_->getVeloc_u(x, y); }
    float getVeloc_v(float x, float y) override { return s_->getVeloc_v(x, y); }
    BoundaryType getBoundaryType(Boundary b) override { return BoundaryType(s_->getBoundaryType(swegb::Boundary(b))); }
    float getBoundaryPos(Boundary b) override { return s_->getBoundaryPos(swegb::Boundary(b)); }

private:
    swegb::Scenario *s_;
};

/// Scenario ids shared with the tests: 0..6 the reference's own classes,
/// 10.. the library's synthetic scenarios through the adapter.
std::unique_ptr<SWE_Scenario> makeScenario(int id, const double *p, std::unique_ptr<swegb::Scenario> &keep) {
    switch (id) {
    case 0: return std::unique_ptr<SWE_Scenario>(new SWE_RadialDamBreakScenario());
    case 1: return std::unique_ptr<SWE_Scenario>(new SWE_RadialBathymetryDamBreakScenario());
    case 2: return std::unique_ptr<SWE_Scenario>(new SWE_SeaAtRestScenario());
    case 3: return std::unique_ptr<SWE_Scenario>(new SWE_HalfDomainDry());
    case 4: return std::unique_ptr<SWE_Scenario>(new SWE_BathymetryDamBreakScenario());
    case 5: return std::unique_ptr<SWE_Scenario>(new SWE_SplashingPoolScenario());
    case 6: return std::unique_ptr<SWE_Scenario>(new SWE_SplashingConeScenario());
    case 10: keep.reset(new swegb::DamBreakScenario(float(p[0]), float(p[1]), float(p[2]), float(p[3]), float(p[4]))); break;
    case 11: keep.reset(new swegb::TsunamiScenario(int(p[0]), uint64_t(p[1]), p[2])); break;
    case 12: keep.reset(new swegb::ShorelineScenario(uint64_t(p[0]), p[1])); break;
    default: return nullptr;
    }
    return std::unique_ptr<SWE_Scenario>(new Adapter(keep.get()));
}

template <class B> void copyIn(B &blk, const float *h, const float *hu, const float *hv, const float *b) {
    const size_t n = size_t(blk.nx + 2) * size_t(blk.ny + 2);
    if (h) std::memcpy(blk.h.getRawPointer(), h, n * sizeof(float));
    if (hu) std::memcpy(blk.hu.getRawPointer(), hu, n * sizeof(float));
    if (hv) std::memcpy(blk.hv.getRawPointer(), hv, n * sizeof(float));
    if (b) std::memcpy(blk.b.getRawPointer(), b, n * sizeof(float));
}
template <class B> void copyOut(B &blk, float *h, float *hu, float *hv, float *b) {
    const size_t n = size_t(blk.nx + 2) * size_t(blk.ny + 2);
    if (h) std::memcpy(h, blk.h.getRawPointer(), n * sizeof(float));
    if (hu) std::memcpy(hu, blk.hu.getRawPointer(), n * sizeof(float));
    if (hv) std::memcpy(hv, blk.hv.getRawPointer(), n * sizeof(float));
    if (b) std::memcpy(b, blk.b.getRawPointer(), n * sizeof(float));
}

} // namespace

extern "C" {

/// WAVE_PROPAGATION_SOLVER this harness was compiled with
int ref_solver_macro() { return WAVE_PROPAGATION_SOLVER; }

/// SWE_Block::initScenario (src/blocks/SWE_Block.hh:650-682) of one block
int ref_init_block(int scenarioId, const double *params, int nx, int ny, float dx, float dy, float originX,
                   float originY, const int *bnd, float *h, float *hu, float *hv, float *b) {
    std::unique_ptr<swegb::Scenario> keep;
    std::unique_ptr<SWE_Scenario> sc = makeScenario(scenarioId, params, keep);
    if (!sc) return -1;
    SWE_DimensionalSplittingMpi blk(nx, ny, dx, dy, originX, originY, false);
    BoundaryType bt[4];
    for (int i = 0; i < 4; i++) bt[i] = BoundaryType(bnd[i]);
    blk.initScenario(*sc, bt);
    copyOut(blk, h, hu, hv, b);
    blk.freeMpiType();
    return 0;
}

/// the swe_mpi driver's domain geometry (src/examples/swe_mpi.cpp:153-156):
/// width/height truncated to int, dx = width / nx
int ref_domain_geometry(int scenarioId, const double *params, int nx, int ny, float *out) {
    std::unique_ptr<swegb::Scenario> keep;
    std::unique_ptr<SWE_Scenario> sc = makeScenario(scenarioId, params, keep);
    if (!sc) return -1;
    int widthScenario = sc->getBoundaryPos(BND_RIGHT) - sc->getBoundaryPos(BND_LEFT);
    int heightScenario = sc->getBoundaryPos(BND_TOP) - sc->getBoundaryPos(BND_BOTTOM);
    out[0] = (float)widthScenario / nx;
    out[1] = (float)heightScenario / ny;
    out[2] = sc->getBoundaryPos(BND_LEFT);
    out[3] = sc->getBoundaryPos(BND_BOTTOM);
    return 0;
}

/// `nsteps` steps of one SWE_DimensionalSplittingMpi block, one rank
/// (driver loop src/examples/swe_mpi.cpp:300-327); dts receives each dt
int ref_run_unsplit(int nx, int ny, float dx, float dy, const int *bnd, float *h, float *hu, float *hv,
                    const float *b, int nsteps, float *dts) {
    SWE_DimensionalSplittingMpi blk(nx, ny, dx, dy, 0.f, 0.f, false);
    for (int i = 0; i < 4; i++) blk.setBoundaryType(Boundary(i), BoundaryType(bnd[i]));
    copyIn(blk, h, hu, hv, b);
    for (int s = 0; s < nsteps; s++) {
        blk.setGhostLayer();
        blk.computeNumericalFluxes();
        float timestep = blk.getMaxTimestep();
        blk.updateUnknowns(timestep);
        if (dts) dts[s] = timestep;
    }
    copyOut(blk, h, hu, hv, nullptr);
    blk.freeMpiType();
    return 0;
}

/// `nsteps` steps of one serial SWE_DimensionalSplitting block (Hybrid solver,
/// driver loop src/examples/swe_simple.cpp:215-252)
int ref_run_split(int nx, int ny, float dx, float dy, const int *bnd, float *h, float *hu, float *hv,
                  const float *b, int nsteps, float *dts) {
    SWE_DimensionalSplitting blk(nx, ny, dx, dy, 0.f, 0.f);
    for (int i = 0; i < 4; i++) blk.setBoundaryType(Boundary(i), BoundaryType(bnd[i]));
    copyIn(blk, h, hu, hv, b);
    for (int s = 0; s < nsteps; s++) {
        blk.setGhostLayer();
        blk.computeNumericalFluxes();
        float timestep = blk.getMaxTimestep();
        blk.updateUnknowns(timestep);
        if (dts) dts[s] = timestep;
    }
    copyOut(blk, h, hu, hv, nullptr);
    return 0;
}

/// Overdecomposed run on one rank: blocksX x blocksY SWE_DimensionalSplittingMPIOverdecomp
/// blocks with CONNECT_WITHIN_RANK neighbours, the driver loop of
/// src/examples/swe_mpi_overdecomp.cpp:189-343 (global or local time stepping).
/// Arrays are the concatenation of all blocks; b ghosts of inner sides are
/// re-exchanged through sendBathymetry.  With ltsMaxTimestep > 0, `nsteps`
/// counts synchronisation intervals and dts receives the interval length;
/// blockSteps (may be NULL) receives each block's final step divisor.
int ref_run_overdecomp(int blocksX, int blocksY, const int *nxCols, const int *nyRows, float dx, float dy,
                       const int *outer, float *h, float *hu, float *hv, float *b, int nsteps, float *dts,
                       float ltsMaxTimestep, float duration, int *blockSteps) {
    const bool lts = ltsMaxTimestep > 0.f;
    std::vector<std::shared_ptr<SWE_DimensionalSplittingMPIOverdecomp>> blocks;
    const int total = blocksX * blocksY;
    for (int k = 0; k < total; k++) {
        const int px = k / blocksY, py = k % blocksY;
        blocks.push_back(std::make_shared<SWE_DimensionalSplittingMPIOverdecomp>(
            nxCols[px], nyRows[py], dx, dy, 0.f, 0.f, lts, std::string("ref"), false));
    }
    size_t off = 0;
    for (int k = 0; k < total; k++) {
        const int px = k / blocksY, py = k % blocksY;
        const int nb[4] = {px > 0 ? k - blocksY : -1, px < blocksX - 1 ? k + blocksY : -1, py > 0 ? k - 1 : -1,
                           py < blocksY - 1 ? k + 1 : -1};
        std::array<std::shared_ptr<SWE_DimensionalSplittingMPIOverdecomp>, 4> nbBlocks;
        int loc[4];
        for (int s = 0; s < 4; s++) {
            if (nb[s] >= 0) {
                blocks[k]->setBoundaryType(Boundary(s), CONNECT_WITHIN_RANK);
                nbBlocks[s] = blocks[nb[s]];
                loc[s] = -2;
            } else {
                blocks[k]->setBoundaryType(Boundary(s), BoundaryType(outer[s]));
                loc[s] = -1;
            }
        }
        blocks[k]->connectNeighbourLocalities(loc);
        blocks[k]->connectNeighbours(const_cast<int *>(nb));
        blocks[k]->connectLocalNeighbours(nbBlocks);
        blocks[k]->setRank(k);
        blocks[k]->setDuration(duration);
        copyIn(*blocks[k], h + off, hu + off, hv + off, b + off);
        off += size_t(nxCols[px] + 2) * size_t(nyRows[py] + 2);
    }
    for (auto &blk : blocks) blk->sendBathymetry();
    for (auto &blk : blocks) blk->recvBathymetry();
    if (lts)
        for (auto &blk : blocks) blk->setMaxLocalTimestep(ltsMaxTimestep);

    for (int s = 0; s < nsteps; s++) {
        bool synchronizedTimestep = true;
        float timestep = 0.f;
        do {
            for (auto &blk : blocks) blk->setGhostLayer();
            for (auto &blk : blocks) blk->receiveGhostLayer();
            for (auto &blk : blocks) blk->computeNumericalFluxes();
            if (!lts) {
                float minTimestep = blocks[0]->maxTimestep;
                for (auto &blk : blocks) minTimestep = std::min(minTimestep, blk->maxTimestep);
                timestep = minTimestep;  // MPI_Allreduce(MIN) over one rank
                for (auto &blk : blocks) blk->maxTimestep = timestep;
            } else {
                for (auto &blk : blocks)
                    if (blk->allGhostlayersInSync()) blk->maxTimestep = blk->getRoundTimestep(blk->maxTimestep);
            }
            for (auto &blk : blocks) blk->updateUnknowns(timestep);
            if (lts) {
                synchronizedTimestep = true;
                for (auto &blk : blocks)
                    if (!blk->hasMaxLocalTimestep()) synchronizedTimestep = false;
            }
        } while (lts && !synchronizedTimestep);
        if (dts) dts[s] = lts ? ltsMaxTimestep : timestep;
        if (lts) {
            if (blockSteps)
                for (int k = 0; k < total; k++) blockSteps[k] = blocks[k]->stepSize;
            for (auto &blk : blocks) blk->resetStepSizeCounter();
        }
    }
    off = 0;
    for (int k = 0; k < total; k++) {
        copyOut(*blocks[k], h + off, hu + off, hv + off, b + off);
        off += size_t(blocks[k]->nx + 2) * size_t(blocks[k]->ny + 2);
    }
    for (auto &blk : blocks) blk->freeMpiType();
    return 0;
}

/// per-edge calls of the solver object the MPI block owns (compile-time choice)
int ref_solve_edges(long n, const float *hL, const float *hR, const float *huL, const float *huR, const float *bL,
                    const float *bR, float *oHL, float *oHR, float *oHuL, float *oHuR, float *oS) {
#if WAVE_PROPAGATION_SOLVER == 0
    solver::HLLEFun<float> s;
#elif WAVE_PROPAGATION_SOLVER == 1
    solver::FWave<float> s;
#else
    solver::AugRie<float> s;
#endif
    for (long i = 0; i < n; i++)
        s.computeNetUpdates(hL[i], hR[i], huL[i], huR[i], bL[i], bR[i], oHL[i], oHR[i], oHuL[i], oHuR[i], oS[i]);
    return 0;
}

} // extern "C"
