/**
 * ORACLE — test infrastructure only (never linked into the product library).
 *
 * `solver::FWave<T>`: CPU restatement of the f-wave Riemann solver that the
 * reference selects with WAVE_PROPAGATION_SOLVER==1
 * (src/blocks/SWE_DimensionalSplittingMpi.hh:46-47,82-84) and calls at
 * src/blocks/SWE_DimensionalSplittingMpi.cpp:403-410,432-439.
 *
 * Method (Bale, LeVeque, Mitran, Rossmanith 2002): Roe eigenvalues
 * s1,2 = uRoe -+ sqrt(g hRoe); the flux jump including the bathymetry source is
 * split into two f-waves along (1, s1), (1, s2).  Wet/dry edges: a dry cell
 * (h < dryTol) is replaced by the reflection of its wet neighbour (a wall) and
 * receives no update.  maxWaveSpeed = max(|s1|, |s2|) (written, not accumulated).
 * Parity of this arithmetic is unpinned: the original solver module is absent.
 */
#ifndef ORACLE_SOLVERS_FWAVE_HPP
#define ORACLE_SOLVERS_FWAVE_HPP

#include "WaveCommon.hpp"

namespace solver {

template <typename T> class FWave {
public:
    explicit FWave(T dryTol = T(0.01), T gravity = T(9.81), T zeroTol = T(1e-7))
        : dryTol_(dryTol), g_(gravity), zeroTol_(zeroTol) {}

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
        const T uRoe = detail::roeVelocity(uL, uR, sqL, sqR);
        const T cRoe = std::sqrt(g_ * (T(0.5) * (hL + hR)));
        const T s1 = uRoe - cRoe;
        const T s2 = uRoe + cRoe;

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
    T dryTol_, g_, zeroTol_;
};

} // namespace solver

#endif
