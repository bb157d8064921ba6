/**
 * ORACLE — test infrastructure only.  C entry points (for ctypes) into the CPU
 * restatement in oracle_block.hpp; loaded by tests/, smoke() and the CPU
 * baseline leg of bench.py, never by the product library.
 *
 * Block state is exchanged as the concatenation over blocks k = 0..B-1 (block
 * k at grid position (k / blocksY, k % blocksY), the rank order of
 * src/examples/swe_mpi.cpp:186-187) of (nx_k+2)*(ny_k+2) values in Float2D
 * layout a[x][y] = raw[x*(ny_k+2)+y] (src/tools/Float2D.hh:74-76).
 */
#include <cstdint>
#include <memory>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_block.hpp"

using namespace oracle;

namespace {

struct Handle {
    int precision = 32;
    std::unique_ptr<Domain<float>> f;
    std::unique_ptr<Domain<double>> d;
    double t = 0.0;  // simulated time, accumulated in the domain's precision
};

template <typename T> void solveEdges(int solverId, int64_t n, const T *hL, const T *hR, const T *huL,
                                      const T *huR, const T *bL, const T *bR, T *oHL, T *oHR, T *oHuL,
                                      T *oHuR, T *oS) {
    solver::FWave<T> fw;
    solver::HLLEFun<T> hl;
    solver::AugRie<T> ar;
    solver::Hybrid<T> hy;
    for (int64_t i = 0; i < n; i++) {
        switch (solverId) {
        case SOLVER_FWAVE: fw.computeNetUpdates(hL[i], hR[i], huL[i], huR[i], bL[i], bR[i], oHL[i], oHR[i], oHuL[i], oHuR[i], oS[i]); break;
        case SOLVER_AUGRIE: ar.computeNetUpdates(hL[i], hR[i], huL[i], huR[i], bL[i], bR[i], oHL[i], oHR[i], oHuL[i], oHuR[i], oS[i]); break;
        case SOLVER_HYBRID: hy.computeNetUpdates(hL[i], hR[i], huL[i], huR[i], bL[i], bR[i], oHL[i], oHR[i], oHuL[i], oHuR[i], oS[i]); break;
        default: hl.computeNetUpdates(hL[i], hR[i], huL[i], huR[i], bL[i], bR[i], oHL[i], oHR[i], oHuL[i], oHuR[i], oS[i]); break;
        }
    }
}

template <typename T, typename U> void setState(Domain<T> &D, const U *h, const U *hu, const U *hv, const U *b) {
    size_t off = 0;
    for (auto &B : D.blocks) {
        const size_t n = B.h.v.size();
        for (size_t i = 0; i < n; i++) {
            if (h) B.h.v[i] = T(h[off + i]);
            if (hu) B.hu.v[i] = T(hu[off + i]);
            if (hv) B.hv.v[i] = T(hv[off + i]);
            if (b) B.b.v[i] = T(b[off + i]);
        }
        off += n;
    }
}

template <typename T, typename U> void getState(Domain<T> &D, U *h, U *hu, U *hv, U *b) {
    size_t off = 0;
    for (auto &B : D.blocks) {
        const size_t n = B.h.v.size();
        for (size_t i = 0; i < n; i++) {
            if (h) h[off + i] = U(B.h.v[i]);
            if (hu) hu[off + i] = U(B.hu.v[i]);
            if (hv) hv[off + i] = U(B.hv.v[i]);
            if (b) b[off + i] = U(B.b.v[i]);
        }
        off += n;
    }
}

/// Global time stepping until t >= target (the checkpoint loop of
/// src/examples/swe_mpi.cpp:300-327): t accumulates in T like the driver's float t.
template <typename T> int advance(Domain<T> &D, double &tIO, double target, int maxSteps, double *dts) {
    T t = T(tIO);
    const T tgt = T(target);
    int n = 0;
    while (t < tgt && n < maxSteps) {
        const T dt = D.step();
        if (dts) dts[n] = double(dt);
        t += dt;
        n++;
    }
    tIO = double(t);
    return n;
}

/// One synchronisation interval of local time stepping
/// (src/examples/swe_mpi_overdecomp.cpp:266-342): inner iterations until every
/// block reached maxTimestepLocal, then t += maxTimestepLocal and the counters reset.
template <typename T> int ltsInterval(Domain<T> &D, double &tIO, int maxIterations, int *blockSteps) {
    int it = 0;
    bool done = false;
    do {
        done = D.ltsIteration();
        it++;
    } while (!done && it < maxIterations);
    if (blockSteps)
        for (size_t k = 0; k < D.blocks.size(); k++) blockSteps[k] = D.blocks[k].stepSize;
    T t = T(tIO);
    t += D.blocks[0].maxTimestepLocal;
    tIO = double(t);
    for (auto &B : D.blocks) B.resetStepSizeCounter();
    return done ? it : -it;
}

} // namespace

/// CPU baseline: `nsteps` global steps of an unsplit multi-block domain with
/// one OpenMP thread per block (the overdecomposed driver's parallel loops,
/// src/examples/swe_mpi_overdecomp.cpp:269-323).  Returns the threads used.
template <typename T> int stepParallel(Domain<T> &D, int nsteps, double *dts) {
    const int nb = int(D.blocks.size());
    int threads = 1;
    for (int s = 0; s < nsteps; s++) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nb; k++) D.blocks[k].applyBoundaryConditions();
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nb; k++) D.exchangeGhosts(k);
#pragma omp parallel for schedule(dynamic, 1)
        for (int k = 0; k < nb; k++) D.blocks[k].timestepFromSpeed(D.blockSpeed(D.blocks[k]));
        T dt = D.blocks[0].maxTimestep;
        for (auto &B : D.blocks) dt = std::min(dt, B.maxTimestep);
        for (auto &B : D.blocks) B.maxTimestep = dt;
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nb; k++) D.blocks[k].updateUnsplit();
        if (dts) dts[s] = double(dt);
    }
#ifdef _OPENMP
    threads = omp_get_max_threads();
#endif
    return threads;
}

extern "C" {

int oracle_solve_edges_f32(int solverId, int64_t n, const float *hL, const float *hR, const float *huL,
                           const float *huR, const float *bL, const float *bR, float *oHL, float *oHR,
                           float *oHuL, float *oHuR, float *oS) {
    solveEdges<float>(solverId, n, hL, hR, huL, huR, bL, bR, oHL, oHR, oHuL, oHuR, oS);
    return 0;
}

int oracle_solve_edges_f64(int solverId, int64_t n, const double *hL, const double *hR, const double *huL,
                           const double *huR, const double *bL, const double *bR, double *oHL, double *oHR,
                           double *oHuL, double *oHuR, double *oS) {
    solveEdges<double>(solverId, n, hL, hR, huL, huR, bL, bR, oHL, oHR, oHuL, oHuR, oS);
    return 0;
}

void *oracle_domain_create(int precision, int blocksX, int blocksY, const int *nxCols, const int *nyRows,
                           double dx, double dy, const int *outer, int solverId, int semantics,
                           int splitDtMode, double ltsMaxTimestep, double duration) {
    auto *H = new Handle();
    H->precision = precision;
    const bool lts = ltsMaxTimestep > 0.0;
    if (precision == 64) {
        H->d.reset(new Domain<double>(blocksX, blocksY, nxCols, nyRows, dx, dy, outer, solverId, semantics,
                                      splitDtMode, lts));
        for (auto &B : H->d->blocks) { B.maxTimestepLocal = ltsMaxTimestep; B.duration = duration; }
    } else {
        H->f.reset(new Domain<float>(blocksX, blocksY, nxCols, nyRows, float(dx), float(dy), outer, solverId,
                                     semantics, splitDtMode, lts));
        for (auto &B : H->f->blocks) { B.maxTimestepLocal = float(ltsMaxTimestep); B.duration = float(duration); }
    }
    return H;
}

void oracle_domain_destroy(void *h) { delete static_cast<Handle *>(h); }

int oracle_domain_set_state_f32(void *h, const float *H_, const float *HU, const float *HV, const float *B) {
    auto *H = static_cast<Handle *>(h);
    if (H->f) setState(*H->f, H_, HU, HV, B); else setState(*H->d, H_, HU, HV, B);
    return 0;
}

int oracle_domain_get_state_f32(void *h, float *H_, float *HU, float *HV, float *B) {
    auto *H = static_cast<Handle *>(h);
    if (H->f) getState(*H->f, H_, HU, HV, B); else getState(*H->d, H_, HU, HV, B);
    return 0;
}

int oracle_domain_set_state_f64(void *h, const double *H_, const double *HU, const double *HV, const double *B) {
    auto *H = static_cast<Handle *>(h);
    if (H->f) setState(*H->f, H_, HU, HV, B); else setState(*H->d, H_, HU, HV, B);
    return 0;
}

int oracle_domain_get_state_f64(void *h, double *H_, double *HU, double *HV, double *B) {
    auto *H = static_cast<Handle *>(h);
    if (H->f) getState(*H->f, H_, HU, HV, B); else getState(*H->d, H_, HU, HV, B);
    return 0;
}

/// bathymetry ghosts of every block: boundary copies (applyBoundaryBathymetry)
/// and neighbour copies (sendBathymetry)
int oracle_domain_bathymetry_ghosts(void *h) {
    auto *H = static_cast<Handle *>(h);
    if (H->f) { for (auto &B : H->f->blocks) B.applyBoundaryBathymetry(); H->f->exchangeBathymetry(); }
    else { for (auto &B : H->d->blocks) B.applyBoundaryBathymetry(); H->d->exchangeBathymetry(); }
    return 0;
}

int oracle_domain_set_ghost_layers(void *h) {
    auto *H = static_cast<Handle *>(h);
    if (H->f) H->f->setGhostLayers(); else H->d->setGhostLayers();
    return 0;
}

/// runs `nsteps` global time steps; dts (may be NULL) receives each dt
int oracle_domain_step(void *h, int nsteps, double *dts) {
    auto *H = static_cast<Handle *>(h);
    for (int i = 0; i < nsteps; i++) {
        const double dt = H->f ? double(H->f->step()) : H->d->step();
        if (dts) dts[i] = dt;
    }
    return nsteps;
}

/// steps while t < target (driver checkpoint loop); returns the step count
int oracle_domain_advance(void *h, double target, int maxSteps, double *dts) {
    auto *H = static_cast<Handle *>(h);
    return H->f ? advance(*H->f, H->t, target, maxSteps, dts) : advance(*H->d, H->t, target, maxSteps, dts);
}

double oracle_domain_time(void *h) { return static_cast<Handle *>(h)->t; }

/// getRoundTimestep (src/blocks/SWE_Block.hh:536-555) of a block at the start
/// of an interval, for every entry of t: the step sizes it picks
int oracle_lts_round_timesteps(const float *t, int n, float tsync, int maxDivisor, int *stepSizes) {
    for (int i = 0; i < n; i++) {
        Block<float> B(1, 1, 1.f, 1.f);
        B.maxTimestepLocal = tsync;
        B.maxDivisor = maxDivisor;
        B.stepSizeCounter = 0;
        B.getRoundTimestep(t[i]);
        stepSizes[i] = B.stepSize;
    }
    return 0;
}

/// depth the dry clamp of updateUnknowns (src/blocks/SWE_DimensionalSplittingMpi.cpp:502-515)
/// has added over all blocks and steps: the sum of -h over cells it set from h < 0 to 0
double oracle_domain_clamp_mass(void *h) {
    auto *H = static_cast<Handle *>(h);
    double m = 0.0;
    if (H->f)
        for (auto &B : H->f->blocks) m += B.clampMass;
    else
        for (auto &B : H->d->blocks) m += B.clampMass;
    return m;
}

/// one local-time-stepping interval; blockSteps receives each block's step count
int oracle_domain_lts_interval(void *h, int maxIterations, int *blockSteps) {
    auto *H = static_cast<Handle *>(h);
    return H->f ? ltsInterval(*H->f, H->t, maxIterations, blockSteps)
                : ltsInterval(*H->d, H->t, maxIterations, blockSteps);
}

/// one inner iteration of local time stepping; when it completes the
/// interval, the interval end too (t += maxTimestepLocal, counters reset).
/// Returns 1 if the interval ended.
int oracle_domain_lts_iteration(void *h) {
    auto *H = static_cast<Handle *>(h);
    auto run = [&](auto &D) {
        const bool done = D.ltsIteration();
        if (done) {
            auto t = decltype(D.blocks[0].maxTimestepLocal)(H->t);
            t += D.blocks[0].maxTimestepLocal;
            H->t = double(t);
            for (auto &B : D.blocks) B.resetStepSizeCounter();
        }
        return done ? 1 : 0;
    };
    return H->f ? run(*H->f) : run(*H->d);
}

/// local-time-stepping state of every block: ints[8k..8k+7] = received[4],
/// stepSize, stepSizeCounter, timestepCounter, notified; border[4k..4k+3]
int oracle_domain_lts_blocks(void *h, int *ints, double *border) {
    auto *H = static_cast<Handle *>(h);
    auto fill = [&](auto &D) {
        for (size_t k = 0; k < D.blocks.size(); k++) {
            const auto &B = D.blocks[k];
            for (int s4 = 0; s4 < 4; s4++) {
                ints[8 * k + s4] = B.receivedGhostlayer[s4];
                border[4 * k + s4] = double(B.borderTimestep[s4]);
            }
            ints[8 * k + 4] = B.stepSize;
            ints[8 * k + 5] = B.stepSizeCounter;
            ints[8 * k + 6] = B.timestepCounter;
            ints[8 * k + 7] = B.notifiedLastTimestep ? 1 : 0;
        }
        return 0;
    };
    return H->f ? fill(*H->f) : fill(*H->d);
}

/// the float dt the blocks last applied (maxTimestep of block k)
double oracle_domain_block_max_timestep(void *h, int k) {
    auto *H = static_cast<Handle *>(h);
    return H->f ? double(H->f->blocks[k].maxTimestep) : H->d->blocks[k].maxTimestep;
}

/// stepParallel in the domain's precision
int oracle_domain_step_parallel(void *h, int nsteps, double *dts) {
    auto *H = static_cast<Handle *>(h);
    return H->f ? stepParallel(*H->f, nsteps, dts) : stepParallel(*H->d, nsteps, dts);
}

} // extern "C"
