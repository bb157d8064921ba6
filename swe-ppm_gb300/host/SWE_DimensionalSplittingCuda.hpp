/**
 * Drop-in block classes of the GB300 step, header-only C++ over the C ABI
 * (include/swe_gb300.h, include/swe_gb300_host.h).
 *
 * SWE_DimensionalSplittingCuda keeps the method names and meaning of the
 * reference's block interface SWE_Block<T, Buffer> (src/blocks/SWE_Block.hh:110-251)
 * and its subclasses (src/blocks/SWE_DimensionalSplittingMpi.hh:52-124,
 * src/blocks/SWE_DimensionalSplitting.hh:41-83): initScenario, setGhostLayer,
 * computeNumericalFluxes, getMaxTimestep, updateUnknowns, the getters of h, hu,
 * hv and b as Float2D, setBoundaryType, computeMaxTimestep.  The state lives in
 * HBM; the Float2D getters are host mirrors refreshed on demand
 * (synchBeforeRead), as the reference's memory model allows
 * (src/blocks/SWE_Block.hh:57-81).  SWE_DomainCuda holds a grid of blocks of
 * one simulation (the overdecomposed layout) in one device allocation.
 * Errors of the C ABI are thrown as std::runtime_error.
 */
#ifndef SWE_GB300_HOST_DIMSPLITCUDA_HPP
#define SWE_GB300_HOST_DIMSPLITCUDA_HPP

#include <algorithm>
#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/swe_gb300.h"
#include "../../include/swe_gb300_host.h"
#include "scenarios.hpp"

namespace swegb {

inline void check(int rc, const char *what) {
    if (rc != SWE_GPU_OK) throw std::runtime_error(std::string(what) + ": " + swe_gpu_last_error());
}

/// host array with the reference's Float2D accessor: a[x][y] = raw[x*rows + y]
/// (src/tools/Float2D.hh:74-80)
class Float2D {
public:
    Float2D(int cols = 0, int rows = 0) : cols_(cols), rows_(rows), v_(size_t(cols) * size_t(rows), 0.f) {}
    float *operator[](int x) { return v_.data() + size_t(x) * rows_; }
    const float *operator[](int x) const { return v_.data() + size_t(x) * rows_; }
    float *getRawPointer() { return v_.data(); }
    const float *getRawPointer() const { return v_.data(); }
    int getRows() const { return rows_; }
    int getCols() const { return cols_; }

private:
    int cols_, rows_;
    std::vector<float> v_;
};

/// A grid of blocks advanced together on the GPU (global time step).
class SWE_DomainCuda {
public:
    SWE_DomainCuda(const std::vector<int> &nxCols, const std::vector<int> &nyRows, float dx, float dy,
                   const BoundaryType outer[4], int solver = SWE_SOLVER_HLLE, int semantics = SWE_SEMANTICS_UNSPLIT,
                   int device = 0)
        : nxCols_(nxCols), nyRows_(nyRows), dx_(dx), dy_(dy) {
        swe_gpu_desc d{};
        d.blocks_x = int(nxCols.size());
        d.blocks_y = int(nyRows.size());
        d.nx_cols = nxCols_.data();
        d.ny_rows = nyRows_.data();
        d.dx = dx;
        d.dy = dy;
        for (int i = 0; i < 4; i++) d.boundary[i] = int(outer[i]);
        d.solver = solver;
        d.semantics = semantics;
        d.device = device;
        swe_gpu_domain *h = nullptr;
        check(swe_gpu_domain_create(&d, &h), "swe_gpu_domain_create");
        dom_.reset(h);
        for (int k = 0; k < blockCount(); k++) {
            int nx, ny;
            swe_gpu_block_shape(h, k, &nx, &ny);
            shapes_.push_back({nx, ny});
        }
    }
    int blockCount() const { return int(nxCols_.size() * nyRows_.size()); }
    int blockNx(int k) const { return shapes_[k].first; }
    int blockNy(int k) const { return shapes_[k].second; }
    swe_gpu_domain *handle() const { return dom_.get(); }

    /// uploads one block from host Float2D arrays (Float2D layout, stride ny+2)
    void upload(int k, const Float2D &h, const Float2D &hu, const Float2D &hv, const Float2D &b) {
        check(swe_gpu_upload_block(handle(), k, h.getRawPointer(), hu.getRawPointer(), hv.getRawPointer(),
                                   b.getRawPointer(), h.getRows()),
              "swe_gpu_upload_block");
    }
    void download(int k, Float2D &h, Float2D &hu, Float2D &hv, Float2D *b = nullptr) {
        check(swe_gpu_download_block(handle(), k, h.getRawPointer(), hu.getRawPointer(), hv.getRawPointer(),
                                     b ? b->getRawPointer() : nullptr, h.getRows()),
              "swe_gpu_download_block");
    }
    void exchangeBathymetry() { check(swe_gpu_exchange_bathymetry(handle()), "swe_gpu_exchange_bathymetry"); }
    void setGhostLayer() { check(swe_gpu_set_ghost_layer(handle()), "swe_gpu_set_ghost_layer"); }
    void computeNumericalFluxes() { check(swe_gpu_compute_fluxes(handle()), "swe_gpu_compute_fluxes"); }
    float getMaxTimestep() {
        float dt = 0.f;
        check(swe_gpu_get_max_timestep(handle(), &dt), "swe_gpu_get_max_timestep");
        return dt;
    }
    void updateUnknowns(float dt) { check(swe_gpu_update_unknowns(handle(), dt), "swe_gpu_update_unknowns"); }
    /// the drivers' `while (t < tEnd) step` loop on the device; returns the steps taken
    int advance(float tEnd, float *t) {
        int n = 0;
        check(swe_gpu_advance(handle(), tEnd, 1 << 30, &n, t), "swe_gpu_advance");
        return n;
    }

private:
    struct Destroy {
        void operator()(swe_gpu_domain *d) const { swe_gpu_domain_destroy(d); }
    };
    std::vector<int> nxCols_, nyRows_;
    float dx_, dy_;
    std::unique_ptr<swe_gpu_domain, Destroy> dom_;
    std::vector<std::pair<int, int>> shapes_;
};

/// One block with the reference's block interface.
class SWE_DimensionalSplittingCuda {
public:
    SWE_DimensionalSplittingCuda(int nx, int ny, float dx, float dy, float originX = 0, float originY = 0,
                                 int solver = SWE_SOLVER_HLLE, int semantics = SWE_SEMANTICS_UNSPLIT)
        : nx(nx), ny(ny), dx(dx), dy(dy), originX(originX), originY(originY), solver_(solver),
          semantics_(semantics), h(nx + 2, ny + 2), hu(nx + 2, ny + 2), hv(nx + 2, ny + 2), b(nx + 2, ny + 2) {
        for (int i = 0; i < 4; i++) boundaryType[i] = PASSIVE;
    }

    // ---- SWE_Block interface ----
    int getCellCountHorizontal() const { return nx; }
    int getCellCountVertical() const { return ny; }
    float getCellSizeHorizontal() const { return dx; }
    float getCellSizeVertical() const { return dy; }
    int getOriginX() const { return int(originX); }  // int, as the reference (src/blocks/SWE_Block.hh:584-592)
    int getOriginY() const { return int(originY); }
    void setBoundaryType(Boundary boundary, BoundaryType type) {
        boundaryType[boundary] = type;
        dom_.reset();
    }

    /// SWE_Block::initScenario (src/blocks/SWE_Block.hh:650-682)
    void initScenario(Scenario &scenario, const BoundaryType boundaries[4]) {
        for (int i = 0; i < 4; i++) boundaryType[i] = boundaries[i];
        sample(scenario);
    }
    void setGhostLayer() { domain().setGhostLayer(); }
    void computeNumericalFluxes() { domain().computeNumericalFluxes(); }
    float getMaxTimestep() { return maxTimestep = domain().getMaxTimestep(); }
    void updateUnknowns(float dt) { domain().updateUnknowns(dt); }

    /// host mirrors, refreshed from the device (synchBeforeRead)
    const Float2D &getWaterHeight() { synchBeforeRead(); return h; }
    const Float2D &getMomentumHorizontal() { synchBeforeRead(); return hu; }
    const Float2D &getMomentumVertical() { synchBeforeRead(); return hv; }
    const Float2D &getBathymetry() { return b; }
    Float2D &getModifiableWaterHeight() { synchBeforeRead(); return h; }
    Float2D &getModifiableMomentumHorizontal() { synchBeforeRead(); return hu; }
    Float2D &getModifiableMomentumVertical() { synchBeforeRead(); return hv; }
    Float2D &getModifiableBathymetry() { return b; }
    void synchBeforeRead() { domain().download(0, h, hu, hv); }
    /// pushes host-side edits of h, hu, hv, b to the device (synchAfterWrite)
    void synchAfterWrite() { domain().upload(0, h, hu, hv, b); }

    /// SWE_Block::computeMaxTimestep (src/blocks/SWE_Block.hh:693-717), on the host mirrors
    void computeMaxTimestep(float dryTol = 0.1f, float cflNumber = 0.4f) {
        synchBeforeRead();
        float maximumWaveSpeed = 0.f;
        const float g = 9.81f;
        for (int i = 1; i < nx + 1; i++)
            for (int j = 1; j < ny + 1; j++)
                if (h[i][j] > dryTol) {
                    const float momentum = std::max(std::abs(hu[i][j]), std::abs(hv[i][j]));
                    const float particleVelocity = momentum / h[i][j];
                    const float waveSpeed = particleVelocity + std::sqrt(g * h[i][j]);
                    maximumWaveSpeed = std::max(maximumWaveSpeed, waveSpeed);
                }
        maxTimestep = std::min(dx, dy) / maximumWaveSpeed;
        maxTimestep *= cflNumber;
    }

    int nx, ny;
    float dx, dy, originX, originY;
    float maxTimestep = 0.f;
    BoundaryType boundaryType[4];

private:
    /// scenario sampled on the host at every cell centre (ghosts included),
    /// then the boundary conditions and bathymetry ghosts applied on the device
    void sample(Scenario &scenario) {
        for (int i = 0; i < ny + 2; i++)
            for (int j = 0; j < nx + 2; j++) {
                const float x = float(double(originX) + (double(j) - 0.5) * double(dx));
                const float y = float(double(originY) + (double(i) - 0.5) * double(dy));
                b[j][i] = scenario.getBathymetry(x, y);
                h[j][i] = scenario.getWaterHeight(x, y);
                hu[j][i] = scenario.getVeloc_u(x, y) * h[j][i];
                hv[j][i] = scenario.getVeloc_v(x, y) * h[j][i];
            }
        dom_.reset();
        SWE_DomainCuda &D = domain();
        D.upload(0, h, hu, hv, b);
        D.exchangeBathymetry();
        D.setGhostLayer();
        D.download(0, h, hu, hv, &b);
    }
    SWE_DomainCuda &domain() {
        if (!dom_) dom_.reset(new SWE_DomainCuda({nx}, {ny}, dx, dy, boundaryType, solver_, semantics_));
        return *dom_;
    }
    int solver_, semantics_;
    Float2D h, hu, hv, b;
    std::unique_ptr<SWE_DomainCuda> dom_;
};

} // namespace swegb

#endif
