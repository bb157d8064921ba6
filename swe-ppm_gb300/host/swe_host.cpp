// Host-side set-up of blocks (C ABI in include/swe_gb300_host.h):
//   - SWE_Block::initScenario (src/blocks/SWE_Block.hh:650-682): sample the
//     scenario at every cell centre of the (nx+2) x (ny+2) block, ghosts
//     included, hu = u h, hv = v h, then the boundary conditions
//     (src/blocks/SWE_Block.hh:757-911) and bathymetry ghosts (:724-749);
//   - the drivers' domain geometry and block decomposition
//     (src/examples/swe_mpi.cpp:153-156, 181-212).
#include <cmath>
#include <cstring>
#include <memory>

#include "../../include/swe_gb300_host.h"
#include "scenarios.hpp"

using namespace swegb;

namespace {

std::unique_ptr<Scenario> makeScenario(int id, const double *p) {
    double q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (p)
        for (int i = 0; i < 8; i++) q[i] = p[i];
    switch (id) {
    case SWE_SCENARIO_RADIAL_DAM_BREAK: return std::unique_ptr<Scenario>(new RadialDamBreakScenario());
    case SWE_SCENARIO_RADIAL_BATHYMETRY_DAM_BREAK: return std::unique_ptr<Scenario>(new RadialBathymetryDamBreakScenario());
    case SWE_SCENARIO_SEA_AT_REST: return std::unique_ptr<Scenario>(new SeaAtRestScenario());
    case SWE_SCENARIO_HALF_DOMAIN_DRY: return std::unique_ptr<Scenario>(new HalfDomainDryScenario());
    case SWE_SCENARIO_BATHYMETRY_DAM_BREAK: return std::unique_ptr<Scenario>(new BathymetryDamBreakScenario());
    case SWE_SCENARIO_SPLASHING_POOL: return std::unique_ptr<Scenario>(new SplashingPoolScenario());
    case SWE_SCENARIO_SPLASHING_CONE: return std::unique_ptr<Scenario>(new SplashingConeScenario());
    case SWE_SCENARIO_DAM_BREAK:
        return std::unique_ptr<Scenario>(new DamBreakScenario(q[0] > 0 ? float(q[0]) : 1000.f, q[1] > 0 ? float(q[1]) : 100.f,
                                                              q[2] > 0 ? float(q[2]) : 15.f, q[3] > 0 ? float(q[3]) : 10.f,
                                                              float(q[4]), q[5] > 0 ? float(q[5]) : -1.f,
                                                              q[6] > 0 ? float(q[6]) : -1.f));
    case SWE_SCENARIO_TSUNAMI:
        return std::unique_ptr<Scenario>(new TsunamiScenario(q[0] > 0 ? int(q[0]) : 2048, q[1] > 0 ? uint64_t(q[1]) : 20261203ull,
                                                             q[2] > 0 ? q[2] : 100000.0));
    case SWE_SCENARIO_SHORELINE:
        return std::unique_ptr<Scenario>(new ShorelineScenario(q[0] > 0 ? uint64_t(q[0]) : 20261203ull, q[1] > 0 ? q[1] : 50000.0));
    default: return nullptr;
    }
}

struct View {  // Float2D-style accessor a[x][y] = raw[x*ld + y]
    float *p;
    int ld;
    float &operator()(int x, int y) const { return p[size_t(x) * ld + y]; }
};

void boundaryConditions(int nx, int ny, const int bnd[4], View h, View hu, View hv) {
    for (int side = 0; side < 4; side++) {
        const int type = bnd[side];
        if (type != SWE_HOST_OUTFLOW && type != SWE_HOST_WALL) continue;
        const float sgn = type == SWE_HOST_WALL ? -1.f : 1.f;
        if (side < 2) {
            const int g = side == 0 ? 0 : nx + 1, s = side == 0 ? 1 : nx;
            for (int j = 1; j <= ny; j++) {
                h(g, j) = h(s, j);
                hu(g, j) = type == SWE_HOST_WALL ? -hu(s, j) : hu(s, j);
                hv(g, j) = hv(s, j);
            }
        } else {
            const int g = side == 2 ? 0 : ny + 1, s = side == 2 ? 1 : ny;
            for (int i = 1; i <= nx; i++) {
                h(i, g) = h(i, s);
                hu(i, g) = hu(i, s);
                hv(i, g) = type == SWE_HOST_WALL ? -hv(i, s) : hv(i, s);
            }
        }
        (void)sgn;
    }
    const int cx[4][4] = {{0, 0, 1, 1}, {0, ny + 1, 1, ny}, {nx + 1, 0, nx, 1}, {nx + 1, ny + 1, nx, ny}};
    for (auto &c : cx) {
        h(c[0], c[1]) = h(c[2], c[3]);
        hu(c[0], c[1]) = hu(c[2], c[3]);
        hv(c[0], c[1]) = hv(c[2], c[3]);
    }
}

void bathymetryGhosts(int nx, int ny, const int bnd[4], View b) {
    auto wallOrOut = [](int t) { return t == SWE_HOST_OUTFLOW || t == SWE_HOST_WALL; };
    if (wallOrOut(bnd[0])) std::memcpy(&b(0, 0), &b(1, 0), sizeof(float) * size_t(ny + 2));
    if (wallOrOut(bnd[1])) std::memcpy(&b(nx + 1, 0), &b(nx, 0), sizeof(float) * size_t(ny + 2));
    if (wallOrOut(bnd[2]))
        for (int i = 0; i <= nx + 1; i++) b(i, 0) = b(i, 1);
    if (wallOrOut(bnd[3]))
        for (int i = 0; i <= nx + 1; i++) b(i, ny + 1) = b(i, ny);
    b(0, 0) = b(1, 1);
    b(0, ny + 1) = b(1, ny);
    b(nx + 1, 0) = b(nx, 1);
    b(nx + 1, ny + 1) = b(nx, ny);
}

} // namespace

extern "C" {

int swe_host_scenario_geometry(int scenario, const double *params, int nx, int ny, float *out) {
    auto sc = makeScenario(scenario, params);
    if (!sc || !out || nx < 1 || ny < 1) return -1;
    // the drivers truncate the scenario extent to int before dividing
    const int width = int(sc->getBoundaryPos(BND_RIGHT) - sc->getBoundaryPos(BND_LEFT));
    const int height = int(sc->getBoundaryPos(BND_TOP) - sc->getBoundaryPos(BND_BOTTOM));
    out[0] = float(width) / float(nx);
    out[1] = float(height) / float(ny);
    out[2] = sc->getBoundaryPos(BND_LEFT);
    out[3] = sc->getBoundaryPos(BND_BOTTOM);
    return 0;
}

int swe_host_scenario_boundary(int scenario, const double *params, int *bnd) {
    auto sc = makeScenario(scenario, params);
    if (!sc || !bnd) return -1;
    for (int s = 0; s < 4; s++) bnd[s] = int(sc->getBoundaryType(Boundary(s)));
    return 0;
}

int swe_host_init_block(int scenario, const double *params, int nx, int ny, float dx, float dy, float originX,
                        float originY, const int *bnd, float *h, float *hu, float *hv, float *b, int ld) {
    auto sc = makeScenario(scenario, params);
    if (!sc || !bnd || !h || !hu || !hv || !b || ld < ny + 2) return -1;
    View H{h, ld}, HU{hu, ld}, HV{hv, ld}, B{b, ld};
    for (int i = 0; i < ny + 2; i++) {
        for (int j = 0; j < nx + 2; j++) {
            // cell centre of column j, row i; the ghost ring sits half a cell outside
            const float x = float(double(originX) + (double(j) - 0.5) * double(dx));
            const float y = float(double(originY) + (double(i) - 0.5) * double(dy));
            B(j, i) = sc->getBathymetry(x, y);
            H(j, i) = sc->getWaterHeight(x, y);
            HU(j, i) = sc->getVeloc_u(x, y) * H(j, i);
            HV(j, i) = sc->getVeloc_v(x, y) * H(j, i);
        }
    }
    boundaryConditions(nx, ny, bnd, H, HU, HV);
    bathymetryGhosts(nx, ny, bnd, B);
    return 0;
}

int swe_host_decompose(int nx, int ny, int nblocks, float dx, float dy, float originX, float originY, int *blocksX,
                       int *blocksY, int *nxCols, int *nyRows, float *originXCols, float *originYRows) {
    if (nblocks < 1 || nx < 1 || ny < 1) return -1;
    // near-square block grid, blocksX >= blocksY (src/examples/swe_mpi.cpp:181-183)
    int by = int(std::sqrt(double(nblocks)));
    while (nblocks % by != 0) by--;
    const int bx = nblocks / by;
    if (blocksX) *blocksX = bx;
    if (blocksY) *blocksY = by;
    // equal blocks, the last one in each direction takes the remainder (:192-198)
    const int nxBlock = nx / bx, nyBlock = ny / by;
    for (int i = 0; i < bx; i++) {
        if (nxCols) nxCols[i] = (i < bx - 1) ? nxBlock : nx - (bx - 1) * nxBlock;
        if (originXCols) originXCols[i] = originX + float(i) * dx * float(nxBlock);
    }
    for (int i = 0; i < by; i++) {
        if (nyRows) nyRows[i] = (i < by - 1) ? nyBlock : ny - (by - 1) * nyBlock;
        if (originYRows) originYRows[i] = originY + float(i) * dy * float(nyBlock);
    }
    return 0;
}

} // extern "C"
