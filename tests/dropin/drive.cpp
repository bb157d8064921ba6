// The reference's per-step driver sequence (src/examples/swe_mpi.cpp:295-343,
// one rank, no checkpoints) over SWE_DimensionalSplittingGpu, the library's
// drop-in block for the reference's class hierarchy.  Built against the
// reference's own headers (SWE_Block, Float2DNative, scenarios) and
// libswe_gb300.  Writes the initial state, every step's dt, the
// computeMaxTimestep estimate of the final state and the final state to
// <out> as raw floats for the test to compare with the oracle.
//   drive <out> <nx> <ny> <steps> <solver>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "SWE_DimensionalSplittingGpu.hh"
#include "scenarios/SWE_simple_scenarios.hh"

static void put(FILE *f, const Float2D &a, int n) { fwrite(a.getRawPointer(), sizeof(float), size_t(n), f); }

int main(int argc, char **argv) {
    if (argc < 6) {
        fprintf(stderr, "usage: drive out nx ny steps solver\n");
        return 2;
    }
    const int nx = atoi(argv[2]), ny = atoi(argv[3]), steps = atoi(argv[4]), solver = atoi(argv[5]);
    SWE_RadialDamBreakScenario scenario;
    const float dx = (scenario.getBoundaryPos(BND_RIGHT) - scenario.getBoundaryPos(BND_LEFT)) / nx;
    const float dy = (scenario.getBoundaryPos(BND_TOP) - scenario.getBoundaryPos(BND_BOTTOM)) / ny;
    SWE_DimensionalSplittingGpu block(nx, ny, dx, dy, scenario.getBoundaryPos(BND_LEFT),
                                      scenario.getBoundaryPos(BND_BOTTOM), solver);
    BoundaryType bnd[4] = {OUTFLOW, OUTFLOW, OUTFLOW, OUTFLOW};
    try {
        block.initScenario(scenario, bnd);
        const int n = (nx + 2) * (ny + 2);
        FILE *f = fopen(argv[1], "wb");
        if (!f) return 3;
        put(f, block.getWaterHeight(), n);
        put(f, block.getMomentumHorizontal(), n);
        put(f, block.getMomentumVertical(), n);
        put(f, block.getBathymetry(), n);
        std::vector<float> dts;
        float t = 0.f;
        for (int i = 0; i < steps; i++) {
            block.setGhostLayer();
            block.computeNumericalFluxes();
            const float dt = block.getMaxTimestep();
            block.updateUnknowns(dt);
            t += dt;
            dts.push_back(dt);
        }
        fwrite(dts.data(), sizeof(float), dts.size(), f);
        block.synchBeforeRead();
        block.computeMaxTimestep();  // the reference's host estimate on the mirrored state
        const float est = block.getMaxTimestep();
        fwrite(&est, sizeof(float), 1, f);
        put(f, block.getWaterHeight(), n);
        put(f, block.getMomentumHorizontal(), n);
        put(f, block.getMomentumVertical(), n);
        fclose(f);
        printf("%d steps, t = %g\n", steps, t);
    } catch (const std::exception &e) {
        fprintf(stderr, "drive: %s\n", e.what());
        return 1;
    }
    return 0;
}
