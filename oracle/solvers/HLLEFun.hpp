/**
 * ORACLE — test infrastructure only (never linked into the product library).
 *
 * `solver::HLLEFun<T>`: CPU restatement of the HLLE solver that every
 * distributed block selects for WAVE_PROPAGATION_SOLVER==0 ("hybrid"; the
 * Hybrid include is commented out: src/blocks/SWE_DimensionalSplittingMpi.hh:42-45,78-81)
 * and that the CMake-built swe_benchmark_mpi therefore runs.
 *
 * Method: Einfeldt (1988) speeds
 *   s1 = min(uL - sqrt(g hL), uRoe - sqrt(g hRoe)),
 *   s2 = max(uR + sqrt(g hR), uRoe + sqrt(g hRoe)),
 * used as the two wave speeds of an f-wave decomposition of the flux jump
 * (including the bathymetry source term).  Wet/dry handling and the speed
 * output follow FWave.hpp.  Parity of this arithmetic is unpinned: the
 * original solver module is absent.
 */
#ifndef ORACLE_SOLVERS_HLLEFUN_HPP
#define ORACLE_SOLVERS_HLLEFUN_HPP

#include "WaveCommon.hpp"

namespace solver {

template <typename T> class HLLEFun {
public:
    explicit HLLEFun(T dryTol = T(0.01), T gravity = T(9.81), T zeroTol = T(1e-7))
        : dryTol_(dryTol), g_(gravity), zeroTol_(zeroTol), sqrtG_(std::sqrt(gravity)) {}

    void computeNetUpdates(T hL, T hR, T huL, T huR, T bL, T bR,
                           T &hUpdL, T &hUpdR, T &huUpdL, T &huUpdR, T &maxWaveSpeed) const {
        const bool dryL = hL < dryTol_;
        const bool dryR = hR < dryTol_;
        if (dryL && dryR) {
            hUpdL = hUpdR = huUpdL = huUpdR = T(0);
            maxWaveSpeed = T(0);
            return;
        }
        if (dryL) {
            hL = hR;
            huL = -huR;
            bL = bR;
        } else if (dryR) {
            hR = hL;
            huR = -huL;
            bR = bL;
        }
        // per-cell quantities: one division and one square root per cell
        const T uL = huL * (T(1) / hL);
        const T uR = huR * (T(1) / hR);
        const T sqL = std::sqrt(hL);
        const T sqR = std::sqrt(hR);
        const T cL = sqrtG_ * sqL;  // sqrt(g h) as sqrt(g) * sqrt(h)
        const T cR = sqrtG_ * sqR;
        const T uRoe = detail::roeVelocity(uL, uR, sqL, sqR);
        const T cRoe = std::sqrt(g_ * (T(0.5) * (hL + hR)));
        const T s1 = detail::vmin(uL - cL, uRoe - cRoe);
        const T s2 = detail::vmax(uR + cR, uRoe + cRoe);

        T df1, df2;
        detail::fluxJump(hL, hR, huL, huR, uL, uR, bL, bR, g_, df1, df2);
        detail::twoWaveFluctuations(s1, s2, df1, df2, zeroTol_, hUpdL, hUpdR, huUpdL, huUpdR);
        if (dryL) {
            hUpdL = T(0);
            huUpdL = T(0);
        }
        if (dryR) {
            hUpdR = T(0);
            huUpdR = T(0);
        }
        maxWaveSpeed = detail::vmax(std::fabs(s1), std::fabs(s2));
    }

private:
    T dryTol_, g_, zeroTol_, sqrtG_;
};

} // namespace solver

#endif
