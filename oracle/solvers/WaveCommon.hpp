/**
 * ORACLE — test infrastructure only (never linked into the product library).
 *
 * Shared pieces of the CPU restatement of the edge Riemann solvers that the
 * reference's blocks call through `solver::X<T>::computeNetUpdates`
 * (call sites: src/blocks/SWE_DimensionalSplittingMpi.cpp:403-410,432-439,
 * src/blocks/SWE_DimensionalSplitting.cpp:122-129,152-159).
 *
 * The solver module itself (TUM-I5/swe_solvers, git submodule declared in
 * .gitmodules:1-3, version unpinned, directory empty in the reference) is not
 * available, so these headers restate the published methods:
 *   - f-wave:  Bale, LeVeque, Mitran, Rossmanith, SIAM J. Sci. Comput. 24 (2002)
 *   - HLLE:    Einfeldt, SIAM J. Numer. Anal. 25 (1988), in f-wave form
 *   - augmented Riemann solver: D. L. George, J. Comput. Phys. 227 (2008)
 * Parity of the solver arithmetic is therefore unpinned; the block code around
 * it is pinned bit-for-bit against the reference's own compiled sources.
 *
 * Per-cell quantities of the f-wave and HLLE solvers are formed as
 * u = hu * (1/h) and sqrt(g h) = sqrt(g) * sqrt(h): one division and one
 * square root per cell, so a GPU can share them between a cell's four edges.
 *
 * Floating-point contract: every multiply-add that is fused is written as an
 * explicit std::fma; everything else is a separate IEEE operation. Build with
 * -ffp-contract=off and without -ffast-math to get results that are identical
 * on x86-64 and aarch64 (and to the CUDA kernels, which follow the same order).
 */
#ifndef ORACLE_SOLVERS_WAVECOMMON_HPP
#define ORACLE_SOLVERS_WAVECOMMON_HPP

#include <algorithm>
#include <cmath>

namespace solver {
namespace detail {

/// min/max with the operand order of std::min/std::max (no NaNs occur here).
template <typename T> inline T vmin(T a, T b) { return (b < a) ? b : a; }
template <typename T> inline T vmax(T a, T b) { return (a < b) ? b : a; }

/// Adds one f-wave (zh, zhu) with speed `s` to the left- or right-going
/// fluctuation; a wave with |s| <= zeroTol is split evenly between both.
template <typename T>
inline void routeWave(T s, T zh, T zhu, T zeroTol, T &hL, T &hR, T &huL, T &huR) {
    if (s < -zeroTol) {
        hL += zh;
        huL += zhu;
    } else if (s > zeroTol) {
        hR += zh;
        huR += zhu;
    } else {
        const T a = T(0.5) * zh;
        const T c = T(0.5) * zhu;
        hL += a;
        huL += c;
        hR += a;
        huR += c;
    }
}

/// Jump of the flux (hu, hu^2 + g h^2 / 2) across the edge plus the
/// well-balanced bathymetry source term g * (hL + hR) / 2 * (bR - bL).
template <typename T>
inline void fluxJump(T hL, T hR, T huL, T huR, T uL, T uR, T bL, T bR, T g, T &df1, T &df2) {
    const T halfG = T(0.5) * g;
    df1 = huR - huL;
    const T phiL = std::fma(huL, uL, halfG * hL * hL);
    const T phiR = std::fma(huR, uR, halfG * hR * hR);
    df2 = (phiR - phiL) + halfG * (hL + hR) * (bR - bL);
}

/// Decomposes the flux jump into two f-waves along (1, s1) and (1, s2) and
/// sums them into left/right-going net updates (wave 1 first, then wave 2).
template <typename T>
inline void twoWaveFluctuations(T s1, T s2, T df1, T df2, T zeroTol,
                                T &hUpdL, T &hUpdR, T &huUpdL, T &huUpdR) {
    const T rd = T(1) / (s2 - s1);
    const T beta1 = std::fma(s2, df1, -df2) * rd;
    const T beta2 = std::fma(-s1, df1, df2) * rd;
    hUpdL = T(0);
    hUpdR = T(0);
    huUpdL = T(0);
    huUpdR = T(0);
    routeWave(s1, beta1, beta1 * s1, zeroTol, hUpdL, hUpdR, huUpdL, huUpdR);
    routeWave(s2, beta2, beta2 * s2, zeroTol, hUpdL, hUpdR, huUpdL, huUpdR);
}

/// Roe-averaged velocity (uL sqrt(hL) + uR sqrt(hR)) / (sqrt(hL) + sqrt(hR)).
template <typename T> inline T roeVelocity(T uL, T uR, T sqL, T sqR) {
    return std::fma(uL, sqL, uR * sqR) / (sqL + sqR);
}

} // namespace detail
} // namespace solver

#endif
