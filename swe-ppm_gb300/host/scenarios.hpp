/**
 * Host-side scenario interface and scenarios.
 *
 * `Scenario` keeps the virtual interface of SWE_Scenario
 * (src/scenarios/SWE_Scenario.hh:42-66): pointwise water height, bathymetry,
 * velocities, boundary type and boundary position, evaluated on the host when
 * a block is initialised (sample -> upload).
 *
 * The first group restates the reference's simple scenarios
 * (src/scenarios/SWE_simple_scenarios.hh:37-284) with the same float/double
 * precision in each expression, so sampling them gives the reference's bits.
 * The second group are the synthetic workloads this library is measured on:
 * a 1000 m radial dam break, a 100 km tsunami over sinusoidal bathymetry with
 * seeded noise, a 50 km shoreline ramp and the ensemble dam breaks.  Seeded
 * noise is a counter-based hash of the global cell index (no global RNG state),
 * so any block can be sampled independently and reproducibly.
 */
#ifndef SWE_GB300_HOST_SCENARIOS_HPP
#define SWE_GB300_HOST_SCENARIOS_HPP

#include <cmath>
#include <cstdint>

namespace swegb {

enum Boundary { BND_LEFT = 0, BND_RIGHT = 1, BND_BOTTOM = 2, BND_TOP = 3 };
enum BoundaryType { OUTFLOW = 0, WALL = 1, INFLOW = 2, CONNECT = 3, CONNECT_WITHIN_RANK = 4, PASSIVE = 5 };

class Scenario {
public:
    virtual ~Scenario() {}
    virtual float getWaterHeight(float x, float y) { (void)x; (void)y; return 0; }
    virtual float getBathymetry(float x, float y) { (void)x; (void)y; return 0; }
    virtual float getVeloc_u(float x, float y) { (void)x; (void)y; return 0; }
    virtual float getVeloc_v(float x, float y) { (void)x; (void)y; return 0; }
    virtual BoundaryType getBoundaryType(Boundary boundary) { (void)boundary; return OUTFLOW; }
    virtual float getBoundaryPos(Boundary boundary) {
        return (boundary == BND_LEFT || boundary == BND_BOTTOM) ? 0.0f : 1.0f;
    }
    virtual float waterHeightAtRest() { return 0; }
    virtual float endSimulation() { return 0; }
};

namespace detail {
inline float box1000(Boundary boundary) { return (boundary == BND_LEFT || boundary == BND_BOTTOM) ? 0.f : 1000.f; }
} // namespace detail

// ---- reference scenarios (src/scenarios/SWE_simple_scenarios.hh) ----

/// :37-71 — radial bump of 15 m over 10 m, bathymetry -250, walls
class HalfDomainDryScenario : public Scenario {
public:
    float getBathymetry(float, float) override { return -250; }
    float getWaterHeight(float x, float y) override {
        return (std::sqrt((x - 250.f) * (x - 250.f) + (y - 250.f) * (y - 250.f)) < 100.f) ? 15.f : 10.0f;
    }
    float endSimulation() override { return 15.f; }
    BoundaryType getBoundaryType(Boundary) override { return WALL; }
    float getBoundaryPos(Boundary b) override { return detail::box1000(b); }
};

/// :77-108 — radial dam break around (250, 250), bathymetry 10
class RadialDamBreakScenario : public Scenario {
public:
    float getBathymetry(float, float) override { return 10.f; }
    float getWaterHeight(float x, float y) override {
        return (std::sqrt((x - 250.f) * (x - 250.f) + (y - 250.f) * (y - 250.f)) < 100.f) ? 15.f : 10.0f;
    }
    float endSimulation() override { return 15.f; }
    BoundaryType getBoundaryType(Boundary) override { return OUTFLOW; }
    float getBoundaryPos(Boundary b) override { return detail::box1000(b); }
};

/// :110-152 — the scenario swe_mpi.cpp:128 hard-codes: 2000 m box, bathymetry
/// step of radius 300 around (1000, 1000), water 40 m inside r < 300 of (500, 500)
class RadialBathymetryDamBreakScenario : public Scenario {
public:
    float getBathymetry(float x, float y) override {
        return (std::sqrt((x - 1000.f) * (x - 1000.f) + (y - 1000.f) * (y - 1000.f)) < 300.f) ? 20.f : 10.f;
    }
    float endSimulation() override { return 15.f; }
    BoundaryType getBoundaryType(Boundary) override { return OUTFLOW; }
    float getBoundaryPos(Boundary b) override {
        return (b == BND_LEFT || b == BND_BOTTOM) ? 0.f : 2000.f;
    }
    float getWaterHeight(float x, float y) override {
        return (std::sqrt((x - 500.f) * (x - 500.f) + (y - 500.f) * (y - 500.f)) < 300.f) ? 40.f : 15.0f;
    }
};

/// :157-196 — uniform 260 m water over a raised disc of bathymetry
class BathymetryDamBreakScenario : public Scenario {
public:
    float getBathymetry(float x, float y) override {
        return (std::sqrt((x - 500.f) * (x - 500.f) + (y - 500.f) * (y - 500.f)) < 50.f) ? -255.f : -260.f;
    }
    float endSimulation() override { return 15.f; }
    BoundaryType getBoundaryType(Boundary) override { return OUTFLOW; }
    float getBoundaryPos(Boundary b) override { return detail::box1000(b); }
    float getWaterHeight(float, float) override { return 260.f; }
};

/// :204-216 — flat surface over a bump: the lake-at-rest test (unit box)
class SeaAtRestScenario : public Scenario {
public:
    float getWaterHeight(float x, float y) override {
        return (std::sqrt((x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5)) < 0.1f) ? 9.9f : 10.0f;
    }
    float getBathymetry(float x, float y) override {
        return (std::sqrt((x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5)) < 0.1f) ? 0.1f : 0.0f;
    }
};

/// :222-253 — sloped initial surface
class SplashingPoolScenario : public Scenario {
public:
    float getBathymetry(float, float) override { return -250.f; }
    float getWaterHeight(float x, float y) override { return 250.0f + (5.0f - (x + y) / 200); }
    float endSimulation() override { return 15.f; }
    float getBoundaryPos(Boundary b) override { return detail::box1000(b); }
};

/// :261-284 — conical bathymetry with a raised centre (unit box)
class SplashingConeScenario : public Scenario {
public:
    float getWaterHeight(float x, float y) override {
        float r = std::sqrt((x - 0.5f) * (x - 0.5f) + (y - 0.5f) * (y - 0.5f));
        float h = 4.0f - 4.5f * (r / 0.5f);
        if (r < 0.1f) h = h + 1.0f;
        return (h > 0.0f) ? h : 0.0f;
    }
    float getBathymetry(float x, float y) override {
        float r = std::sqrt((x - 0.5f) * (x - 0.5f) + (y - 0.5f) * (y - 0.5f));
        return 1.0f + 9.0f * ((r < 0.5f) ? r : 0.5f);
    }
    float waterHeightAtRest() override { return 4.0f; }
    float endSimulation() override { return 0.5f; }
    BoundaryType getBoundaryType(Boundary) override { return OUTFLOW; }
};

// ---- synthetic workloads ----

namespace detail {
inline uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
/// Uniform in [0, 1) from a 64-bit hash (53 mantissa bits, exact in double).
inline double unit(uint64_t z) { return double(z >> 11) * (1.0 / 9007199254740992.0); }
/// Approximately standard-normal value for global cell (i, j): the sum of 12
/// uniforms minus 6 (Irwin-Hall); only additions, so bit-identical everywhere.
inline double cellNormal(uint64_t seed, int64_t i, int64_t j) {
    uint64_t key = splitmix64(seed ^ splitmix64(uint64_t(i) * 0x100000001B3ull ^ splitmix64(uint64_t(j))));
    double s = 0.0;
    for (int k = 0; k < 12; k++) {
        key = splitmix64(key);
        s += unit(key);
    }
    return s - 6.0;
}
inline double seededUnit(uint64_t seed, uint64_t salt) { return unit(splitmix64(seed * 0x9E3779B97F4A7C15ull + salt)); }
} // namespace detail

/// Radial dam break: one square box of side `length`, flat bathymetry `bottom`,
/// water `inner` m inside radius `radius` around the centre, `outer` m outside,
/// still water, outflow boundaries.  With the defaults it is the 256^2 / 1000 m
/// plain dam break (15 m inside r < 100 m, 10 m outside, b = 0).
class DamBreakScenario : public Scenario {
public:
    DamBreakScenario(float length = 1000.f, float radius = 100.f, float inner = 15.f, float outer = 10.f,
                     float bottom = 0.f, float centreX = -1.f, float centreY = -1.f)
        : L_(length), r_(radius), hi_(inner), ho_(outer), b_(bottom),
          cx_(centreX < 0 ? 0.5f * length : centreX), cy_(centreY < 0 ? 0.5f * length : centreY) {}
    float getBathymetry(float, float) override { return b_; }
    float getWaterHeight(float x, float y) override {
        return (std::sqrt((x - cx_) * (x - cx_) + (y - cy_) * (y - cy_)) < r_) ? hi_ : ho_;
    }
    BoundaryType getBoundaryType(Boundary) override { return OUTFLOW; }
    float getBoundaryPos(Boundary b) override { return (b == BND_LEFT || b == BND_BOTTOM) ? 0.f : L_; }
    float endSimulation() override { return 10.f; }

private:
    float L_, r_, hi_, ho_, b_, cx_, cy_;
};

/// Synthetic tsunami on a `length` square (default 100 km) resolved by n x n
/// cells: b = -2000 + 500 sin(2 pi x / L) cos(2 pi y / L) + N(0, 20^2) per cell
/// (seeded), still water h = -b plus a Gaussian surface bump (5 m, sigma 5 km)
/// at a seeded location in the middle half of the box; outflow boundaries.
class TsunamiScenario : public Scenario {
public:
    TsunamiScenario(int n, uint64_t seed = 20261203ull, double length = 100000.0)
        : n_(n), seed_(seed), L_(length) {
        cx_ = L_ * (0.25 + 0.5 * detail::seededUnit(seed_, 1));
        cy_ = L_ * (0.25 + 0.5 * detail::seededUnit(seed_, 2));
    }
    float getBathymetry(float x, float y) override { return float(bathy(x, y)); }
    float getWaterHeight(float x, float y) override {
        const double dxc = double(x) - cx_, dyc = double(y) - cy_;
        const double bump = 5.0 * std::exp(-(dxc * dxc + dyc * dyc) / (2.0 * 5000.0 * 5000.0));
        return float(-bathy(x, y) + bump);
    }
    BoundaryType getBoundaryType(Boundary) override { return OUTFLOW; }
    float getBoundaryPos(Boundary b) override { return (b == BND_LEFT || b == BND_BOTTOM) ? 0.f : float(L_); }
    float endSimulation() override { return 80.f; }

private:
    double bathy(float x, float y) const {
        const double pi = 3.14159265358979323846;
        const int64_t i = int64_t(std::floor(double(x) * n_ / L_));
        const int64_t j = int64_t(std::floor(double(y) * n_ / L_));
        return -2000.0 + 500.0 * std::sin(2.0 * pi * double(x) / L_) * std::cos(2.0 * pi * double(y) / L_) +
               20.0 * detail::cellNormal(seed_, i, j);
    }
    int n_;
    uint64_t seed_;
    double L_, cx_, cy_;
};

/// Shoreline ramp on a `length` square (default 50 km): bathymetry rises
/// linearly from -4000 m at x = 0 to +50 m at x = L, still water up to sea
/// level (h = max(0, -b)) plus a Gaussian bump (3 m, sigma 2 km) at a seeded
/// offshore location; the dry land on the right exercises wet/dry edges.
class ShorelineScenario : public Scenario {
public:
    ShorelineScenario(uint64_t seed = 20261203ull, double length = 50000.0) : seed_(seed), L_(length) {
        cx_ = L_ * (0.2 + 0.3 * detail::seededUnit(seed_, 3));
        cy_ = L_ * (0.3 + 0.4 * detail::seededUnit(seed_, 4));
    }
    float getBathymetry(float x, float) override { return float(bathy(x)); }
    float getWaterHeight(float x, float y) override {
        const double depth = -bathy(x);
        if (depth <= 0.0) return 0.f;
        const double dxc = double(x) - cx_, dyc = double(y) - cy_;
        return float(depth + 3.0 * std::exp(-(dxc * dxc + dyc * dyc) / (2.0 * 2000.0 * 2000.0)));
    }
    BoundaryType getBoundaryType(Boundary) override { return OUTFLOW; }
    float getBoundaryPos(Boundary b) override { return (b == BND_LEFT || b == BND_BOTTOM) ? 0.f : float(L_); }
    float endSimulation() override { return 200.f; }

private:
    double bathy(float x) const { return -4000.0 + 4050.0 * double(x) / L_; }
    uint64_t seed_;
    double L_, cx_, cy_;
};

} // namespace swegb

#endif
