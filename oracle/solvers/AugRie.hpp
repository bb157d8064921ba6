/**
 * ORACLE — test infrastructure only (never linked into the product library).
 *
 * `solver::AugRie<T>`: CPU restatement of the augmented Riemann solver that the
 * reference selects with WAVE_PROPAGATION_SOLVER==2
 * (src/blocks/SWE_DimensionalSplittingMpi.hh:48-49,85-87).  The original
 * implementation (swe_solvers, absent) is not available; this follows the
 * published method of D. L. George, "Augmented Riemann solvers for the shallow
 * water equations over variable topography with steady states and
 * inundation", J. Comput. Phys. 227 (2008):
 *
 *  1. dry/dry edges give no update; a dry cell next to a wet one is either
 *     inundated (its state becomes h = hu = 0) or, when the wet side's water
 *     cannot rise above the dry cell's bathymetry, acts as a reflecting wall;
 *  2. a middle-state estimate (two-rarefaction closed form, otherwise Newton
 *     steps on the shock/rarefaction curves) gives the middle-state
 *     characteristic speeds s1m, s2m and the rarefaction flags;
 *  3. Einfeldt speeds widened by those middle speeds bound the solution:
 *     l1 = min(sE1, s1m), l3 = max(sE2, s2m);
 *  4. the jump (dh, dhu, dphi) minus the steady-state (bathymetry) wave
 *     (ddh, ddphi), with the sonic test and positivity bounds of George §4,
 *     is decomposed along r1 = (1, l1, l1^2), r2 = (0, 0, 1) (or the
 *     rarefaction corrector (1, l2, l2^2) for a transonic rarefaction) and
 *     r3 = (1, l3, l3^2) in closed form;
 *  5. f-waves (beta_p r_p[1], beta_p r_p[2]) are routed by the sign of l_p.
 *
 * By construction the h-fluctuations sum to huR - huL (mass conservation).
 * Parity of this arithmetic is unpinned: the original solver module is absent.
 */
#ifndef ORACLE_SOLVERS_AUGRIE_HPP
#define ORACLE_SOLVERS_AUGRIE_HPP

#include "WaveCommon.hpp"

namespace solver {

template <typename T> class AugRie {
public:
    // Defaults: the reference default-constructs its solver
    // (src/blocks/SWE_DimensionalSplittingMpi.hh:84-87) from the swe_solvers
    // module, absent from the reference checkout, so they are unpinned.  The
    // single Newton iteration with tolerance 1e-6 is George 2008's solver as
    // GeoClaw calls it (riemann_aug_JCP); dryTol 0.01 and zeroTol 1e-7 are the
    // module's default-construction values.
    explicit AugRie(T dryTol = T(0.01), T gravity = T(9.81), T newtonTol = T(1e-6),
                    int maxNewtonIterations = 1, T zeroTol = T(1e-7))
        : dryTol_(dryTol), g_(gravity), newtonTol_(newtonTol), maxNewton_(maxNewtonIterations),
          zeroTol_(zeroTol) {}

    void computeNetUpdates(T hL, T hR, T huL, T huR, T bL, T bR,
                           T &hUpdL, T &hUpdR, T &huUpdL, T &huUpdR, T &maxWaveSpeed) const {
        using detail::vmax;
        using detail::vmin;
        const bool dryL = hL < dryTol_;
        const bool dryR = hR < dryTol_;
        hUpdL = hUpdR = huUpdL = huUpdR = T(0);
        if (dryL && dryR) {
            maxWaveSpeed = T(0);
            return;
        }

        // 1. wet/dry: inundation or reflecting wall
        T uL = T(0), uR = T(0);
        bool wallL = false, wallR = false;
        if (dryR) {
            uL = huL / hL;
            T hm, s1m, s2m;
            bool r1, r2;
            middleState(hL, hL, uL, -uL, hm, s1m, s2m, r1, r2);
            const T hTest = vmax(hL, hm);
            if (hTest + bL < bR) {
                wallR = true;
                hR = hL;
                huR = -huL;
                uR = -uL;
                bR = bL;
            } else {
                hR = T(0);
                huR = T(0);
            }
        } else if (dryL) {
            uR = huR / hR;
            T hm, s1m, s2m;
            bool r1, r2;
            middleState(hR, hR, -uR, uR, hm, s1m, s2m, r1, r2);
            const T hTest = vmax(hR, hm);
            if (hTest + bR < bL) {
                wallL = true;
                hL = hR;
                huL = -huR;
                uL = -uR;
                bL = bR;
            } else {
                hL = T(0);
                huL = T(0);
            }
        } else {
            uL = huL / hL;
            uR = huR / hR;
        }

        // 2. middle state of the homogeneous problem
        T hm, s1m, s2m;
        bool rare1, rare2;
        middleState(hL, hR, uL, uR, hm, s1m, s2m, rare1, rare2);

        // 3. speeds
        const T cL = std::sqrt(g_ * hL);
        const T cR = std::sqrt(g_ * hR);
        const T sqL = std::sqrt(hL);
        const T sqR = std::sqrt(hR);
        const T uRoe = detail::roeVelocity(uL, uR, sqL, sqR);
        const T cRoe = std::sqrt(g_ * (T(0.5) * (hL + hR)));
        const T sE1 = vmin(uL - cL, uRoe - cRoe);
        const T sE2 = vmax(uR + cR, uRoe + cRoe);
        const T l1 = vmin(sE1, s1m);
        const T l3 = vmax(sE2, s2m);

        // HLL middle depth, used for the positivity bounds
        const T hStarHLL = vmax((huL - huR + l3 * hR - l1 * hL) / (l3 - l1), T(0));

        // middle wave: jump in momentum flux, or rarefaction corrector
        T l2 = T(0.5) * (l1 + l3);
        bool corrector = false;
        if (rare1 && l1 < T(0) && s1m > T(0)) {
            l2 = s1m;
            corrector = true;
        } else if (rare2 && s2m < T(0) && l3 > T(0)) {
            l2 = s2m;
            corrector = true;
        }
        if (corrector && !(l1 < l2 && l2 < l3)) corrector = false;
        if (corrector && vmin(hL, hR) < dryTol_) corrector = false;
        if (!corrector) l2 = T(0.5) * (l1 + l3);

        // 4. steady-state wave from the bathymetry jump
        const T halfG = T(0.5) * g_;
        const T dh = hR - hL;
        const T dhu = huR - huL;
        const T phiL = std::fma(huL, uL, halfG * hL * hL);
        const T phiR = std::fma(huR, uR, halfG * hR * hR);
        const T dphi = phiR - phiL;
        const T db = bR - bL;

        const T critTol = T(1e-6);
        const T hbar = vmax(T(0.5) * (hL + hR), T(0));
        const T uSum = uL + uR;
        const T s1s2bar = T(0.25) * uSum * uSum - g_ * hbar;
        const T s1s2tilde = vmax(T(0), uL * uR) - g_ * hbar;

        bool sonic = false;
        if (std::fabs(s1s2bar) <= critTol) sonic = true;
        if (s1s2bar * s1s2tilde <= critTol) sonic = true;
        if (s1s2bar * l1 * l3 <= critTol) sonic = true;
        if (vmin(std::fabs(l1), std::fabs(l3)) < critTol) sonic = true;
        if (l1 < T(0) && s1m > T(0)) sonic = true;
        if (l3 > T(0) && s2m < T(0)) sonic = true;
        if ((uL + cL) * (uR + cR) < T(0)) sonic = true;
        if ((uL - cL) * (uR - cR) < T(0)) sonic = true;

        T ddh = sonic ? -db : db * g_ * hbar / s1s2bar;
        const T width = l3 - l1;
        if (l1 < -critTol && l3 > critTol) {
            ddh = vmin(ddh, hStarHLL * width / l3);
            ddh = vmax(ddh, hStarHLL * width / l1);
        } else if (l1 >= critTol) {
            ddh = vmin(ddh, hStarHLL * width / l1);
            ddh = vmax(ddh, -hL);
        } else if (l3 <= -critTol) {
            ddh = vmin(ddh, hR);
            ddh = vmax(ddh, hStarHLL * width / l3);
        }
        T ddphi = sonic ? -g_ * hbar * db : -db * g_ * hbar * s1s2tilde / s1s2bar;
        const T pL = -hL * db;
        const T pR = -hR * db;
        ddphi = vmin(ddphi, g_ * vmax(pL, pR));
        ddphi = vmax(ddphi, g_ * vmin(pL, pR));

        const T d1 = dh - ddh;
        const T d2 = dhu;
        const T d3 = dphi - ddphi;

        // 5. closed-form decomposition and routing
        T beta1, beta2, beta3;
        if (!corrector) {
            const T rd = T(1) / width;
            beta1 = std::fma(l3, d1, -d2) * rd;
            beta3 = std::fma(-l1, d1, d2) * rd;
            beta2 = d3 - l1 * (l1 * beta1) - l3 * (l3 * beta3);
        } else {
            // Vandermonde system: beta_p = (lq lr d1 - (lq + lr) d2 + d3) / ((lp - lq)(lp - lr))
            beta1 = (l2 * l3 * d1 - (l2 + l3) * d2 + d3) / ((l1 - l2) * (l1 - l3));
            beta2 = (l1 * l3 * d1 - (l1 + l3) * d2 + d3) / ((l2 - l1) * (l2 - l3));
            beta3 = (l1 * l2 * d1 - (l1 + l2) * d2 + d3) / ((l3 - l1) * (l3 - l2));
        }
        detail::routeWave(l1, beta1 * l1, beta1 * l1 * l1, zeroTol_, hUpdL, hUpdR, huUpdL, huUpdR);
        if (corrector)
            detail::routeWave(l2, beta2 * l2, beta2 * l2 * l2, zeroTol_, hUpdL, hUpdR, huUpdL, huUpdR);
        else
            detail::routeWave(l2, T(0), beta2, zeroTol_, hUpdL, hUpdR, huUpdL, huUpdR);
        detail::routeWave(l3, beta3 * l3, beta3 * l3 * l3, zeroTol_, hUpdL, hUpdR, huUpdL, huUpdR);

        if (wallL) {
            hUpdL = T(0);
            huUpdL = T(0);
        }
        if (wallR) {
            hUpdR = T(0);
            huUpdR = T(0);
        }
        maxWaveSpeed = vmax(std::fabs(l1), std::fabs(l3));
    }

    /// Middle state of the Riemann problem without bathymetry: depth hm, the
    /// characteristic speeds um -+ sqrt(g hm) and whether each family is a
    /// rarefaction.  States with h < dryTol are dry (rarefaction into dry bed).
    void middleState(T hL, T hR, T uL, T uR, T &hm, T &s1m, T &s2m, bool &rare1, bool &rare2) const {
        using detail::vmax;
        using detail::vmin;
        if (hR < dryTol_) {
            hm = T(0);
            const T front = uL + T(2) * std::sqrt(g_ * hL);
            s1m = front;
            s2m = front;
            rare1 = true;
            rare2 = false;
            return;
        }
        if (hL < dryTol_) {
            hm = T(0);
            const T front = uR - T(2) * std::sqrt(g_ * hR);
            s1m = front;
            s2m = front;
            rare1 = false;
            rare2 = true;
            return;
        }
        const T cL = std::sqrt(g_ * hL);
        const T cR = std::sqrt(g_ * hR);
        const T cm = T(0.5) * (cL + cR) + T(0.25) * (uL - uR);
        if (cm <= T(0)) {  // the two rarefactions open a dry middle state
            hm = T(0);
            s1m = uL + T(2) * cL;
            s2m = uR - T(2) * cR;
            rare1 = true;
            rare2 = true;
            return;
        }
        const T hRR = cm * cm / g_;
        T um;
        if (hRR <= vmin(hL, hR)) {
            hm = hRR;
            um = uL + T(2) * (cL - cm);
            rare1 = true;
            rare2 = true;
        } else {
            T h = hRR;
            for (int it = 0; it < maxNewton_; ++it) {
                T fL, dfL, fR, dfR;
                waveCurve(h, hL, cL, fL, dfL);
                waveCurve(h, hR, cR, fR, dfR);
                const T F = fL + fR + (uR - uL);
                if (std::fabs(F) < newtonTol_) break;
                h = h - F / (dfL + dfR);
                if (h < dryTol_) {
                    h = dryTol_;
                    break;
                }
            }
            hm = h;
            // middle velocity seen from both sides, averaged (equal once the
            // iteration has converged; keeps the estimate mirror-symmetric)
            T fL, dfL, fR, dfR;
            waveCurve(hm, hL, cL, fL, dfL);
            waveCurve(hm, hR, cR, fR, dfR);
            um = T(0.5) * ((uL - fL) + (uR + fR));
            rare1 = hm <= hL;
            rare2 = hm <= hR;
        }
        const T cmid = std::sqrt(g_ * hm);
        s1m = um - cmid;
        s2m = um + cmid;
    }

private:
    /// Velocity change across a shock (h > hK) or rarefaction (h <= hK)
    /// connecting depth hK (wave speed cK) to depth h, and its derivative.
    void waveCurve(T h, T hK, T cK, T &f, T &df) const {
        if (h > hK) {
            const T s = std::sqrt(T(0.5) * g_ * (T(1) / h + T(1) / hK));
            f = (h - hK) * s;
            df = s - g_ * (h - hK) / (T(4) * h * h * s);
        } else {
            f = T(2) * (std::sqrt(g_ * h) - cK);
            df = std::sqrt(g_ / h);
        }
    }

    T dryTol_, g_, newtonTol_;
    int maxNewton_;
    T zeroTol_;
};

} // namespace solver

#endif
