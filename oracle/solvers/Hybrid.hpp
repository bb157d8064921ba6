/**
 * ORACLE — test infrastructure only (never linked into the product library).
 *
 * `solver::Hybrid<T>`: CPU restatement of the hybrid solver that the serial
 * split block uses (src/blocks/SWE_DimensionalSplitting.hh:39,60).  The
 * original (swe_solvers, absent) is not available.  Rule used here: the
 * augmented Riemann solver (AugRie.hpp) on edges where either cell is shallower
 * than `switchDepth` (default 0.1 m, the block's dry tolerance
 * defaultDryTol, src/Constants.hh:5), where wet/dry fronts and large
 * relative bathymetry steps occur; the f-wave solver (FWave.hpp) elsewhere.
 */
#ifndef ORACLE_SOLVERS_HYBRID_HPP
#define ORACLE_SOLVERS_HYBRID_HPP

#include "AugRie.hpp"
#include "FWave.hpp"

namespace solver {

template <typename T> class Hybrid {
public:
    explicit Hybrid(T dryTol = T(0.01), T gravity = T(9.81), T switchDepth = T(0.1))
        : fwave_(dryTol, gravity), augrie_(dryTol, gravity), switchDepth_(switchDepth) {}

    void computeNetUpdates(T hL, T hR, T huL, T huR, T bL, T bR,
                           T &hUpdL, T &hUpdR, T &huUpdL, T &huUpdR, T &maxWaveSpeed) const {
        if (hL < switchDepth_ || hR < switchDepth_)
            augrie_.computeNetUpdates(hL, hR, huL, huR, bL, bR, hUpdL, hUpdR, huUpdL, huUpdR, maxWaveSpeed);
        else
            fwave_.computeNetUpdates(hL, hR, huL, huR, bL, bR, hUpdL, hUpdR, huUpdL, huUpdR, maxWaveSpeed);
    }

private:
    FWave<T> fwave_;
    AugRie<T> augrie_;
    T switchDepth_;
};

} // namespace solver

#endif
