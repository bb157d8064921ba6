/**
 * ORACLE — test infrastructure only.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it, and only as the checker or the
 * timed CPU baseline; the product library never links it.
 *
 * CPU restatement (templated on float / double: the FP32 oracle and its FP64
 * twin) of the reference's block step:
 *   - storage: Float2D column layout a[x][y] = raw[x*(ny+2)+y]
 *     (src/tools/Float2D.hh:74-80), ghost ring at 0 and n+1;
 *   - applyBoundaryConditions / applyBoundaryBathymetry
 *     (src/blocks/SWE_Block.hh:757-911, 724-749);
 *   - semantics A, the unsplit step of SWE_DimensionalSplittingMpi /
 *     SWE_DimensionalSplittingMPIOverdecomp: computeNumericalFluxes
 *     (src/blocks/SWE_DimensionalSplittingMpi.cpp:383-476) and updateUnknowns
 *     with the dry clamp (:484-518);
 *   - semantics B, the serial SWE_DimensionalSplitting step
 *     (src/blocks/SWE_DimensionalSplitting.cpp:105-210);
 *   - intra-rank ghost copies between blocks (CONNECT_WITHIN_RANK,
 *     src/blocks/SWE_DimensionalSplittingMPIOverdecomp.cpp:208-235, 269-304)
 *     and the overdecomposed driver loop with the min-dt reduction
 *     (src/examples/swe_mpi_overdecomp.cpp:263-343);
 *   - local time stepping: getRoundTimestep, getTotalLocalTimestep,
 *     checkAllGhostlayers, interpolateGhostlayer, copyGhostlayer,
 *     hasMaxLocalTimestep, allGhostlayersInSync, isSendable/isReceivable
 *     (src/blocks/SWE_Block.hh:311-562).
 * Loops, index shifts and operation order follow the reference line by line so
 * that the float instantiation reproduces the reference's compiled block code
 * bit for bit (given the same solver and no -ffast-math).
 */
#ifndef ORACLE_BLOCK_HPP
#define ORACLE_BLOCK_HPP

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <vector>

#include "solvers/AugRie.hpp"
#include "solvers/FWave.hpp"
#include "solvers/HLLEFun.hpp"
#include "solvers/Hybrid.hpp"

namespace oracle {

enum Boundary { BND_LEFT = 0, BND_RIGHT = 1, BND_BOTTOM = 2, BND_TOP = 3 };
enum BoundaryType { OUTFLOW = 0, WALL = 1, INFLOW = 2, CONNECT = 3, CONNECT_WITHIN_RANK = 4, PASSIVE = 5 };
enum GhostlayerState { GL_DONE = 0, GL_UNVALID = 1, GL_INTER = 2, GL_SYNC = 3, GL_NEXT = 4 };
enum SolverId { SOLVER_FWAVE = 1, SOLVER_AUGRIE = 2, SOLVER_HYBRID = 3, SOLVER_HLLE = 4 };
enum Semantics { SEMANTICS_UNSPLIT = 0, SEMANTICS_SPLIT = 1 };
/// How the split block (semantics B) reduces its x-wave speed: the evident
/// intent (max over all x-edges) or what the reference computes with one
/// OpenMP thread (the solver overwrites the reduction variable, so the speed
/// of the last x-edge solved, x = nx, y = ny+1, remains).
enum SplitDtMode { SPLIT_DT_MAX = 0, SPLIT_DT_LAST_EDGE = 1 };

template <typename T> struct Array2D {
    int cols = 0, rows = 0;
    std::vector<T> v;
    Array2D() = default;
    Array2D(int c, int r) : cols(c), rows(r), v(size_t(c) * size_t(r), T(0)) {}
    T &operator()(int x, int y) { return v[size_t(x) * rows + y]; }
    const T &operator()(int x, int y) const { return v[size_t(x) * rows + y]; }
    T *col(int x) { return v.data() + size_t(x) * rows; }
};

template <typename T> struct Block {
    int nx = 0, ny = 0;
    T dx = 0, dy = 0;
    Array2D<T> h, hu, hv, b;
    // local-time-stepping receive buffers (alias of h/hu/hv without LTS)
    Array2D<T> bufH, bufHu, bufHv;
    int boundaryType[4] = {PASSIVE, PASSIVE, PASSIVE, PASSIVE};
    int neighbour[4] = {-1, -1, -1, -1};
    T maxTimestep = T(0);
    double clampMass = 0.0;  // depth the dry clamp added (sum of -h over clamped cells), test bookkeeping

    // LTS state (src/blocks/SWE_Block.hh:214-229)
    bool localTimestepping = false;
    T duration = T(0);
    T maxTimestepLocal = T(0);
    int maxDivisor = 1024;
    bool notifiedLastTimestep = false;
    int stepSize = 0, stepSizeCounter = 0, timestepCounter = 0;
    int receivedGhostlayer[4] = {GL_NEXT, GL_NEXT, GL_NEXT, GL_NEXT};
    T borderTimestep[4] = {0, 0, 0, 0};

    // semantics A net updates (src/blocks/SWE_DimensionalSplittingMpi.cpp:80-91)
    Array2D<T> hNL, hNR, huNL, huNR, hNB, hNA, hvNB, hvNA, hStar, huStar;

    Block(int nx_, int ny_, T dx_, T dy_, bool lts = false)
        : nx(nx_), ny(ny_), dx(dx_), dy(dy_), h(nx_ + 2, ny_ + 2), hu(nx_ + 2, ny_ + 2), hv(nx_ + 2, ny_ + 2),
          b(nx_ + 2, ny_ + 2), localTimestepping(lts), hNL(nx_ + 2, ny_ + 2), hNR(nx_ + 2, ny_ + 2),
          huNL(nx_ + 2, ny_ + 2), huNR(nx_ + 2, ny_ + 2), hNB(nx_ + 1, ny_ + 2), hNA(nx_ + 1, ny_ + 2),
          hvNB(nx_ + 1, ny_ + 2), hvNA(nx_ + 1, ny_ + 2), hStar(nx_ + 1, ny_ + 2), huStar(nx_ + 1, ny_ + 2) {
        if (lts) {
            bufH = Array2D<T>(nx + 2, ny + 2);
            bufHu = Array2D<T>(nx + 2, ny + 2);
            bufHv = Array2D<T>(nx + 2, ny + 2);
        }
    }
    Array2D<T> &BH() { return localTimestepping ? bufH : h; }
    Array2D<T> &BHu() { return localTimestepping ? bufHu : hu; }
    Array2D<T> &BHv() { return localTimestepping ? bufHv : hv; }

    /// src/blocks/SWE_Block.hh:757-911
    void applyBoundaryConditions() {
        switch (boundaryType[BND_LEFT]) {
        case WALL:
            for (int j = 1; j <= ny; j++) { h(0, j) = h(1, j); hu(0, j) = -hu(1, j); hv(0, j) = hv(1, j); }
            break;
        case OUTFLOW:
            for (int j = 1; j <= ny; j++) { h(0, j) = h(1, j); hu(0, j) = hu(1, j); hv(0, j) = hv(1, j); }
            break;
        default: break;
        }
        switch (boundaryType[BND_RIGHT]) {
        case WALL:
            for (int j = 1; j <= ny; j++) { h(nx + 1, j) = h(nx, j); hu(nx + 1, j) = -hu(nx, j); hv(nx + 1, j) = hv(nx, j); }
            break;
        case OUTFLOW:
            for (int j = 1; j <= ny; j++) { h(nx + 1, j) = h(nx, j); hu(nx + 1, j) = hu(nx, j); hv(nx + 1, j) = hv(nx, j); }
            break;
        default: break;
        }
        switch (boundaryType[BND_BOTTOM]) {
        case WALL:
            for (int i = 1; i <= nx; i++) { h(i, 0) = h(i, 1); hu(i, 0) = hu(i, 1); hv(i, 0) = -hv(i, 1); }
            break;
        case OUTFLOW:
            for (int i = 1; i <= nx; i++) { h(i, 0) = h(i, 1); hu(i, 0) = hu(i, 1); hv(i, 0) = hv(i, 1); }
            break;
        default: break;
        }
        switch (boundaryType[BND_TOP]) {
        case WALL:
            for (int i = 1; i <= nx; i++) { h(i, ny + 1) = h(i, ny); hu(i, ny + 1) = hu(i, ny); hv(i, ny + 1) = -hv(i, ny); }
            break;
        case OUTFLOW:
            for (int i = 1; i <= nx; i++) { h(i, ny + 1) = h(i, ny); hu(i, ny + 1) = hu(i, ny); hv(i, ny + 1) = hv(i, ny); }
            break;
        default: break;
        }
        h(0, 0) = h(1, 1); hu(0, 0) = hu(1, 1); hv(0, 0) = hv(1, 1);
        h(0, ny + 1) = h(1, ny); hu(0, ny + 1) = hu(1, ny); hv(0, ny + 1) = hv(1, ny);
        h(nx + 1, 0) = h(nx, 1); hu(nx + 1, 0) = hu(nx, 1); hv(nx + 1, 0) = hv(nx, 1);
        h(nx + 1, ny + 1) = h(nx, ny); hu(nx + 1, ny + 1) = hu(nx, ny); hv(nx + 1, ny + 1) = hv(nx, ny);
    }

    /// src/blocks/SWE_Block.hh:724-749
    void applyBoundaryBathymetry() {
        if (boundaryType[BND_LEFT] == OUTFLOW || boundaryType[BND_LEFT] == WALL)
            std::memcpy(b.col(0), b.col(1), sizeof(T) * (ny + 2));
        if (boundaryType[BND_RIGHT] == OUTFLOW || boundaryType[BND_RIGHT] == WALL)
            std::memcpy(b.col(nx + 1), b.col(nx), sizeof(T) * (ny + 2));
        if (boundaryType[BND_BOTTOM] == OUTFLOW || boundaryType[BND_BOTTOM] == WALL)
            for (int i = 0; i <= nx + 1; i++) b(i, 0) = b(i, 1);
        if (boundaryType[BND_TOP] == OUTFLOW || boundaryType[BND_TOP] == WALL)
            for (int i = 0; i <= nx + 1; i++) b(i, ny + 1) = b(i, ny);
        b(0, 0) = b(1, 1);
        b(0, ny + 1) = b(1, ny);
        b(nx + 1, 0) = b(nx, 1);
        b(nx + 1, ny + 1) = b(nx, ny);
    }

    /// dt from the block's maximum wave speed
    /// (src/blocks/SWE_DimensionalSplittingMpi.cpp:448-456)
    void timestepFromSpeed(T maxWaveSpeed) {
        if (double(maxWaveSpeed) > 0.00001) {
            maxTimestep = std::min(dx / maxWaveSpeed, dy / maxWaveSpeed);
            maxTimestep *= T(0.4);
        } else {
            maxTimestep = std::numeric_limits<T>::max();
        }
    }

    /// semantics A edge loops (src/blocks/SWE_DimensionalSplittingMpi.cpp:391-446); returns max speed
    template <class S> T computeFluxesUnsplit(const S &solver) {
        T maxWaveSpeed = T(0);
        for (int i = 1; i < nx + 2; i++) {
            for (int j = 1; j < ny + 1; ++j) {
                T maxEdgeSpeed;
                solver.computeNetUpdates(h(i - 1, j), h(i, j), hu(i - 1, j), hu(i, j), b(i - 1, j), b(i, j),
                                         hNL(i - 1, j - 1), hNR(i - 1, j - 1), huNL(i - 1, j - 1),
                                         huNR(i - 1, j - 1), maxEdgeSpeed);
                maxWaveSpeed = std::max(maxWaveSpeed, maxEdgeSpeed);
            }
        }
        for (int i = 1; i < nx + 1; i++) {
            for (int j = 1; j < ny + 2; j++) {
                T maxEdgeSpeed;
                solver.computeNetUpdates(h(i, j - 1), h(i, j), hv(i, j - 1), hv(i, j), b(i, j - 1), b(i, j),
                                         hNB(i - 1, j - 1), hNA(i - 1, j - 1), hvNB(i - 1, j - 1),
                                         hvNA(i - 1, j - 1), maxEdgeSpeed);
                maxWaveSpeed = std::max(maxWaveSpeed, maxEdgeSpeed);
            }
        }
        return maxWaveSpeed;
    }

    /// semantics A update + dry clamp (src/blocks/SWE_DimensionalSplittingMpi.cpp:484-518)
    void updateUnsplit() {
        const T dt = maxTimestep;
        for (int i = 1; i < nx + 1; i++) {
            for (int j = 1; j < ny + 1; j++) {
                h(i, j) -= dt / dx * (hNR(i - 1, j - 1) + hNL(i, j - 1)) + dt / dy * (hNA(i - 1, j - 1) + hNB(i - 1, j));
                hu(i, j) -= dt / dx * (huNR(i - 1, j - 1) + huNL(i, j - 1));
                hv(i, j) -= dt / dy * (hvNA(i - 1, j - 1) + hvNB(i - 1, j));
                if (h(i, j) < T(0)) {
                    clampMass -= double(h(i, j));
                    h(i, j) = hu(i, j) = hv(i, j) = T(0);
                } else if (double(h(i, j)) < 0.1) {
                    hu(i, j) = hv(i, j) = T(0);
                }
            }
        }
    }

    /// semantics B (src/blocks/SWE_DimensionalSplitting.cpp:105-179): x-sweep, dt, Q*, y-sweep
    template <class S> void computeFluxesSplit(const S &solver, int dtMode) {
        T maxHorizontalWaveSpeed = T(0);
        T lastEdgeSpeed = T(0);
        for (int x = 0; x < nx + 1; x++) {
            for (int y = 0; y < ny + 2; y++) {
                T s;
                solver.computeNetUpdates(h(x, y), h(x + 1, y), hu(x, y), hu(x + 1, y), b(x, y), b(x + 1, y),
                                         hNL(x, y), hNR(x + 1, y), huNL(x, y), huNR(x + 1, y), s);
                maxHorizontalWaveSpeed = std::max(maxHorizontalWaveSpeed, s);
                lastEdgeSpeed = s;
            }
        }
        const T speed = (dtMode == SPLIT_DT_LAST_EDGE) ? std::max(T(0), lastEdgeSpeed) : maxHorizontalWaveSpeed;
        maxTimestep = T(0.4) * (dx / speed);
        for (int x = 1; x < nx + 1; x++) {
            for (int y = 0; y < ny + 2; y++) {
                hStar(x, y) = h(x, y) - (maxTimestep / dx) * (hNL(x, y) + hNR(x, y));
                huStar(x, y) = hu(x, y) - (maxTimestep / dx) * (huNL(x, y) + huNR(x, y));
            }
        }
        for (int x = 1; x < nx + 1; x++) {
            for (int y = 0; y < ny + 1; y++) {
                T s;
                solver.computeNetUpdates(h(x, y), h(x, y + 1), hv(x, y), hv(x, y + 1), b(x, y), b(x, y + 1),
                                         hNB(x, y), hNA(x, y + 1), hvNB(x, y), hvNA(x, y + 1), s);
            }
        }
    }

    /// semantics B update (src/blocks/SWE_DimensionalSplitting.cpp:187-210)
    void updateSplit() {
        for (int x = 1; x < nx + 1; x++) {
            for (int y = 1; y < ny + 1; y++) {
                h(x, y) = hStar(x, y) - (maxTimestep / dx) * (hNB(x, y) + hNA(x, y));
                hu(x, y) = huStar(x, y);
                hv(x, y) = hv(x, y) - (maxTimestep / dx) * (hvNB(x, y) + hvNA(x, y));
            }
        }
    }

    // ---------------- local time stepping (src/blocks/SWE_Block.hh:311-562) ----------------
    bool allGhostlayersInSync() const {
        return receivedGhostlayer[BND_LEFT] != GL_UNVALID && receivedGhostlayer[BND_RIGHT] != GL_UNVALID &&
               receivedGhostlayer[BND_TOP] != GL_UNVALID && receivedGhostlayer[BND_BOTTOM] != GL_UNVALID &&
               (stepSizeCounter <= stepSize);
    }
    bool hasMaxLocalTimestep() const {
        return (stepSizeCounter >= stepSize && allGhostlayersInSync()) || notifiedLastTimestep;
    }
    bool isReceivable(int border) const {
        if (notifiedLastTimestep) return false;
        return receivedGhostlayer[border] == GL_NEXT || receivedGhostlayer[border] == GL_UNVALID ||
               receivedGhostlayer[border] == GL_SYNC;
    }
    T getTotalLocalTimestep() const {
        return T(maxTimestepLocal * timestepCounter) +
               (stepSize > 0 ? (T(maxTimestepLocal * stepSizeCounter) / T(stepSize)) : T(0));
    }
    T interpolateValue(T oldval, T newval, T remoteTimestep) const {
        return (oldval + (newval - oldval) * (getTotalLocalTimestep() / remoteTimestep));
    }
    void resetStepSizeCounter() {
        stepSizeCounter = 0;
        stepSize = 0;
        timestepCounter++;
    }
    T getRoundTimestep(T timestep) {
        if (stepSizeCounter <= 0) {
            if (timestep > maxTimestepLocal) timestep = maxTimestepLocal;
            if (timestep < T(maxTimestepLocal / maxDivisor)) timestep = T(maxTimestepLocal / maxDivisor);
            // log(float) is the float overload in the reference (libstdc++ math.h)
            const T logT = std::log(timestep);
            int divisor = int(std::pow(2.0, -(std::ceil(double(logT) / std::log(2.0)))));
            if (T(1) / T(divisor) > timestep) divisor *= 2;
            stepSize = divisor;
            if (stepSize > maxDivisor) stepSize = maxDivisor;
        }
        return T(maxTimestepLocal / stepSize);
    }
    void interpolateGhostlayer(int border, T remoteTimestep) {
        Array2D<T> &bH = BH(), &bHu = BHu(), &bHv = BHv();
        switch (border) {
        case BND_LEFT:
            for (int i = 1; i < ny + 1; i++) {
                h(0, i) = interpolateValue(h(0, i), bH(0, i), remoteTimestep);
                hu(0, i) = interpolateValue(hu(0, i), bHu(0, i), remoteTimestep);
                hv(0, i) = interpolateValue(hv(0, i), bHv(0, i), remoteTimestep);
            }
            break;
        case BND_RIGHT:
            for (int i = 1; i < ny + 1; i++) {
                h(nx + 1, i) = interpolateValue(h(nx + 1, i), bH(nx + 1, i), remoteTimestep);
                hu(nx + 1, i) = interpolateValue(hu(nx + 1, i), bHu(nx + 1, i), remoteTimestep);
                hv(nx + 1, i) = interpolateValue(hv(nx + 1, i), bHv(nx + 1, i), remoteTimestep);
            }
            break;
        case BND_BOTTOM:
            for (int i = 1; i < nx + 1; i++) {
                h(i, 0) = interpolateValue(h(i, 0), bH(i, 0), remoteTimestep);
                hu(i, 0) = interpolateValue(hu(i, 0), bHu(i, 0), remoteTimestep);
                hv(i, 0) = interpolateValue(hv(i, 0), bHv(i, 0), remoteTimestep);
            }
            break;
        case BND_TOP:
            for (int i = 1; i < nx + 1; i++) {
                h(i, ny + 1) = interpolateValue(h(i, ny + 1), bH(i, ny + 1), remoteTimestep);
                hu(i, ny + 1) = interpolateValue(hu(i, ny + 1), bHu(i, ny + 1), remoteTimestep);
                hv(i, ny + 1) = interpolateValue(hv(i, ny + 1), bHv(i, ny + 1), remoteTimestep);
            }
            break;
        }
    }
    void copyGhostlayer(int border) {
        Array2D<T> &bH = BH(), &bHu = BHu(), &bHv = BHv();
        switch (border) {
        case BND_LEFT:
            for (int i = 1; i < ny + 1; i++) { h(0, i) = bH(0, i); hu(0, i) = bHu(0, i); hv(0, i) = bHv(0, i); }
            break;
        case BND_RIGHT:
            for (int i = 1; i < ny + 1; i++) { h(nx + 1, i) = bH(nx + 1, i); hu(nx + 1, i) = bHu(nx + 1, i); hv(nx + 1, i) = bHv(nx + 1, i); }
            break;
        case BND_BOTTOM:
            for (int i = 1; i < nx + 1; i++) { h(i, 0) = bH(i, 0); hu(i, 0) = bHu(i, 0); hv(i, 0) = bHv(i, 0); }
            break;
        case BND_TOP:
            for (int i = 1; i < nx + 1; i++) { h(i, ny + 1) = bH(i, ny + 1); hu(i, ny + 1) = bHu(i, ny + 1); hv(i, ny + 1) = bHv(i, ny + 1); }
            break;
        }
    }
    /// src/blocks/SWE_Block.hh:375-436
    void checkAllGhostlayers() {
        if (!localTimestepping) return;
        for (int border = BND_LEFT; border <= BND_TOP; border++) {
            if (boundaryType[border] == CONNECT || boundaryType[border] == CONNECT_WITHIN_RANK) {
                const T local = getTotalLocalTimestep();
                if (std::fabs(double(borderTimestep[border] - local)) <= std::numeric_limits<double>::epsilon()) {
                    copyGhostlayer(border);
                    receivedGhostlayer[border] = GL_SYNC;
                } else if (borderTimestep[border] > local) {
                    interpolateGhostlayer(border, borderTimestep[border]);
                    receivedGhostlayer[border] = GL_INTER;
                } else {
                    receivedGhostlayer[border] = GL_UNVALID;
                }
                if (borderTimestep[border] >= duration) receivedGhostlayer[border] = GL_DONE;
            }
        }
        const T local = getTotalLocalTimestep();
        if (std::fabs(double(duration - local)) <= std::numeric_limits<double>::epsilon() || local >= duration)
            notifiedLastTimestep = true;
        if (allGhostlayersInSync()) {
            for (int bnd : {BND_LEFT, BND_RIGHT, BND_TOP, BND_BOTTOM})
                if (receivedGhostlayer[bnd] != GL_DONE)
                    receivedGhostlayer[bnd] = (receivedGhostlayer[bnd] == GL_INTER) ? GL_INTER : GL_NEXT;
        }
        if (allGhostlayersInSync()) {
            if (stepSizeCounter < stepSize) stepSizeCounter++;
        }
    }

    /// src/blocks/SWE_Block.hh:693-717
    void computeMaxTimestep(T dryTol, T cflNumber) {
        T maximumWaveSpeed = T(0);
        const T g = T(9.81);
        for (int i = 1; i < nx + 1; i++)
            for (int j = 1; j < ny + 1; j++)
                if (h(i, j) > dryTol) {
                    T momentum = std::max(std::abs(hu(i, j)), std::abs(hv(i, j)));
                    T particleVelocity = momentum / h(i, j);
                    T waveSpeed = particleVelocity + std::sqrt(g * h(i, j));
                    maximumWaveSpeed = std::max(maximumWaveSpeed, waveSpeed);
                }
        maxTimestep = std::min(dx, dy) / maximumWaveSpeed;
        maxTimestep *= cflNumber;
    }
};

/// A rectangular grid of blocks advanced together (one block = the single-rank
/// drivers; several = the overdecomposed driver with CONNECT_WITHIN_RANK ghost
/// copies, src/examples/swe_mpi_overdecomp.cpp:148-343).  Block k sits at
/// (k / blocksY, k % blocksY) like rank k in src/examples/swe_mpi.cpp:186-187.
template <typename T> struct Domain {
    int blocksX = 1, blocksY = 1;
    int solverId = SOLVER_HLLE;
    int semantics = SEMANTICS_UNSPLIT;
    int splitDtMode = SPLIT_DT_MAX;
    bool lts = false;
    std::vector<Block<T>> blocks;
    solver::FWave<T> fwave;
    solver::HLLEFun<T> hlle;
    solver::AugRie<T> augrie;
    solver::Hybrid<T> hybrid;

    Domain(int bx, int by, const int *nxCols, const int *nyRows, T dx, T dy, const int outer[4], int solver,
           int sem, int dtMode, bool localTimestepping = false)
        : blocksX(bx), blocksY(by), solverId(solver), semantics(sem), splitDtMode(dtMode), lts(localTimestepping) {
        for (int k = 0; k < bx * by; k++) {
            const int px = k / by, py = k % by;
            blocks.emplace_back(nxCols[px], nyRows[py], dx, dy, localTimestepping);
            Block<T> &B = blocks.back();
            const int nb[4] = {px > 0 ? k - by : -1, px < bx - 1 ? k + by : -1, py > 0 ? k - 1 : -1,
                               py < by - 1 ? k + 1 : -1};
            for (int s = 0; s < 4; s++) {
                B.neighbour[s] = nb[s];
                B.boundaryType[s] = nb[s] >= 0 ? CONNECT_WITHIN_RANK : outer[s];
            }
        }
    }

    /// intra-rank copy of the neighbours' copy layers into this block's ghost
    /// cells (or LTS buffers), src/blocks/SWE_DimensionalSplittingMPIOverdecomp.cpp:273-304
    void exchangeGhosts(int k) {
        Block<T> &B = blocks[k];
        Array2D<T> &bH = B.BH(), &bHu = B.BHu(), &bHv = B.BHv();
        if (B.boundaryType[BND_RIGHT] == CONNECT_WITHIN_RANK && B.isReceivable(BND_RIGHT)) {
            Block<T> &R = blocks[B.neighbour[BND_RIGHT]];
            B.borderTimestep[BND_RIGHT] = R.getTotalLocalTimestep();
            for (int i = 1; i < B.ny + 1; i++) { bH(B.nx + 1, i) = R.h(1, i); bHu(B.nx + 1, i) = R.hu(1, i); bHv(B.nx + 1, i) = R.hv(1, i); }
        }
        if (B.boundaryType[BND_LEFT] == CONNECT_WITHIN_RANK && B.isReceivable(BND_LEFT)) {
            Block<T> &L = blocks[B.neighbour[BND_LEFT]];
            B.borderTimestep[BND_LEFT] = L.getTotalLocalTimestep();
            for (int i = 1; i < B.ny + 1; i++) { bH(0, i) = L.h(L.nx, i); bHu(0, i) = L.hu(L.nx, i); bHv(0, i) = L.hv(L.nx, i); }
        }
        if (B.boundaryType[BND_TOP] == CONNECT_WITHIN_RANK && B.isReceivable(BND_TOP)) {
            Block<T> &U = blocks[B.neighbour[BND_TOP]];
            B.borderTimestep[BND_TOP] = U.getTotalLocalTimestep();
            for (int i = 1; i < B.nx + 1; i++) { bH(i, B.ny + 1) = U.h(i, 1); bHu(i, B.ny + 1) = U.hu(i, 1); bHv(i, B.ny + 1) = U.hv(i, 1); }
        }
        if (B.boundaryType[BND_BOTTOM] == CONNECT_WITHIN_RANK && B.isReceivable(BND_BOTTOM)) {
            Block<T> &D = blocks[B.neighbour[BND_BOTTOM]];
            B.borderTimestep[BND_BOTTOM] = D.getTotalLocalTimestep();
            for (int i = 1; i < B.nx + 1; i++) { bH(i, 0) = D.h(i, D.ny); bHu(i, 0) = D.hu(i, D.ny); bHv(i, 0) = D.hv(i, D.ny); }
        }
    }

    /// bathymetry ghosts from the neighbours, once at set-up
    /// (src/blocks/SWE_DimensionalSplittingMPIOverdecomp.cpp:208-235)
    void exchangeBathymetry() {
        for (auto &B : blocks) {
            if (B.boundaryType[BND_RIGHT] == CONNECT_WITHIN_RANK)
                for (int i = 1; i < B.ny + 1; i++) B.b(B.nx + 1, i) = blocks[B.neighbour[BND_RIGHT]].b(1, i);
            if (B.boundaryType[BND_LEFT] == CONNECT_WITHIN_RANK) {
                Block<T> &L = blocks[B.neighbour[BND_LEFT]];
                for (int i = 1; i < B.ny + 1; i++) B.b(0, i) = L.b(L.nx, i);
            }
            if (B.boundaryType[BND_TOP] == CONNECT_WITHIN_RANK)
                for (int i = 1; i < B.nx + 1; i++) B.b(i, B.ny + 1) = blocks[B.neighbour[BND_TOP]].b(i, 1);
            if (B.boundaryType[BND_BOTTOM] == CONNECT_WITHIN_RANK) {
                Block<T> &D = blocks[B.neighbour[BND_BOTTOM]];
                for (int i = 1; i < B.nx + 1; i++) B.b(i, 0) = D.b(i, D.ny);
            }
        }
    }

    /// setGhostLayer for every block: boundary conditions, then the copies
    void setGhostLayers() {
        for (auto &B : blocks) B.applyBoundaryConditions();
        for (size_t k = 0; k < blocks.size(); k++) exchangeGhosts(int(k));
        for (auto &B : blocks) B.checkAllGhostlayers();
    }

    T blockSpeed(Block<T> &B) {
        switch (solverId) {
        case SOLVER_FWAVE: return B.computeFluxesUnsplit(fwave);
        case SOLVER_AUGRIE: return B.computeFluxesUnsplit(augrie);
        case SOLVER_HYBRID: return B.computeFluxesUnsplit(hybrid);
        default: return B.computeFluxesUnsplit(hlle);
        }
    }
    void blockSplitFluxes(Block<T> &B) {
        switch (solverId) {
        case SOLVER_FWAVE: B.computeFluxesSplit(fwave, splitDtMode); break;
        case SOLVER_AUGRIE: B.computeFluxesSplit(augrie, splitDtMode); break;
        case SOLVER_HLLE: B.computeFluxesSplit(hlle, splitDtMode); break;
        default: B.computeFluxesSplit(hybrid, splitDtMode); break;
        }
    }

    /// One global time step; returns the dt used.  Unsplit: every block solves
    /// its edges and proposes dt, the minimum is applied to all blocks
    /// (src/examples/swe_mpi_overdecomp.cpp:269-323).  Split: the serial block.
    T step() {
        setGhostLayers();
        if (semantics == SEMANTICS_SPLIT) {
            Block<T> &B = blocks[0];
            blockSplitFluxes(B);
            B.updateSplit();
            return B.maxTimestep;
        }
        for (auto &B : blocks) B.timestepFromSpeed(blockSpeed(B));
        T dt = blocks[0].maxTimestep;
        for (auto &B : blocks) dt = std::min(dt, B.maxTimestep);
        for (auto &B : blocks) B.maxTimestep = dt;
        for (auto &B : blocks) B.updateUnsplit();
        return dt;
    }

    /// One inner iteration of the local-time-stepping loop
    /// (src/examples/swe_mpi_overdecomp.cpp:266-337 with localTimestepping):
    /// ghost exchange, fluxes on in-sync blocks, per-block rounded dt, update.
    /// Returns true once every block has reached its max local time step.
    bool ltsIteration() {
        setGhostLayers();
        for (auto &B : blocks)
            if (B.allGhostlayersInSync()) B.timestepFromSpeed(blockSpeed(B));
        for (auto &B : blocks)
            if (B.allGhostlayersInSync()) B.maxTimestep = B.getRoundTimestep(B.maxTimestep);
        for (auto &B : blocks)
            if (B.allGhostlayersInSync()) B.updateUnsplit();
        bool done = true;
        for (auto &B : blocks)
            if (!B.hasMaxLocalTimestep()) done = false;
        return done;
    }
};

} // namespace oracle

#endif
