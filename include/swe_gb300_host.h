/*
 * swe_gb300_host.h -- host-side set-up helpers of the GB300 block step
 * (plain C ABI, host memory only, no CUDA calls).
 *
 * They replace the reference's host-side initialisation path:
 *   SWE_Block::initScenario              src/blocks/SWE_Block.hh:650-682
 *   SWE_Block::applyBoundaryConditions   src/blocks/SWE_Block.hh:757-911
 *   SWE_Block::applyBoundaryBathymetry   src/blocks/SWE_Block.hh:724-749
 *   domain geometry and decomposition    src/examples/swe_mpi.cpp:153-156, 181-212
 *   SWE_Scenario subclasses              src/scenarios/SWE_simple_scenarios.hh:37-284
 */
#ifndef SWE_GB300_HOST_H
#define SWE_GB300_HOST_H

#ifdef __cplusplus
extern "C" {
#endif

/* BoundaryType values (src/types/Boundary.hh:23-30) */
#define SWE_HOST_OUTFLOW 0
#define SWE_HOST_WALL 1

/* scenario ids: 0..6 the reference's simple scenarios, 10.. synthetic workloads */
#define SWE_SCENARIO_RADIAL_DAM_BREAK 0            /* SWE_RadialDamBreakScenario */
#define SWE_SCENARIO_RADIAL_BATHYMETRY_DAM_BREAK 1 /* SWE_RadialBathymetryDamBreakScenario (swe_mpi default) */
#define SWE_SCENARIO_SEA_AT_REST 2                 /* SWE_SeaAtRestScenario */
#define SWE_SCENARIO_HALF_DOMAIN_DRY 3             /* SWE_HalfDomainDry */
#define SWE_SCENARIO_BATHYMETRY_DAM_BREAK 4        /* SWE_BathymetryDamBreakScenario */
#define SWE_SCENARIO_SPLASHING_POOL 5              /* SWE_SplashingPoolScenario */
#define SWE_SCENARIO_SPLASHING_CONE 6              /* SWE_SplashingConeScenario */
#define SWE_SCENARIO_DAM_BREAK 10  /* params: length, radius, inner, outer, bottom, centre x, centre y */
#define SWE_SCENARIO_TSUNAMI 11    /* params: cells per side, seed, length */
#define SWE_SCENARIO_SHORELINE 12  /* params: seed, length */

/* dx, dy, origin x, origin y of an nx x ny discretisation of the scenario */
int swe_host_scenario_geometry(int scenario, const double *params, int nx, int ny, float *out4);
/* the scenario's boundary types, indexed LEFT, RIGHT, BOTTOM, TOP */
int swe_host_scenario_boundary(int scenario, const double *params, int *bnd4);
/* samples one block (incl. ghosts) into Float2D arrays with column stride ld
 * and applies the boundary conditions and bathymetry ghosts for bnd4 */
int swe_host_init_block(int scenario, const double *params, int nx, int ny, float dx, float dy, float origin_x,
                        float origin_y, const int *bnd4, float *h, float *hu, float *hv, float *b, int ld);
/* near-square decomposition of nx x ny cells into nblocks blocks */
int swe_host_decompose(int nx, int ny, int nblocks, float dx, float dy, float origin_x, float origin_y,
                       int *blocks_x, int *blocks_y, int *nx_cols, int *ny_rows, float *origin_x_cols,
                       float *origin_y_rows);

/* NetCDF snapshot files with the reference writer's variables and layout
 * (src/writer/NetCdfWriter.cpp:84-234: time, x, y, ah(time,y,x), hu, hv,
 * b(y,x)), written in the classic 64-bit-offset format without libnetcdf. */
typedef struct swe_nc_writer swe_nc_writer;
/* creates the file; b is the block's bathymetry in Float2D layout (stride ld) */
int swe_nc_open(const char *path, int nx, int ny, float dx, float dy, float origin_x, float origin_y, const float *b,
                int ld, swe_nc_writer **out);
/* appends time t from host Float2D arrays (NetCdfWriter::writeTimeStep) */
int swe_nc_write_step(swe_nc_writer *w, float t, const float *h, const float *hu, const float *hv, int ld);
/* appends time t from big-endian (y, x) slabs of the interior, as produced on
 * the device by swe_gpu_snapshot_slabs_async */
int swe_nc_write_step_slabs(swe_nc_writer *w, float t, const void *h, const void *hu, const void *hv);
int swe_nc_close(swe_nc_writer *w);

#ifdef __cplusplus
}
#endif

#endif
