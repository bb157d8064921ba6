/*
 * swe_gb300.h -- C ABI of the GB300 block step of the SWE-PPM finite-volume
 * shallow-water solver.
 *
 * Plain C: pointers, sizes and ints only; every function returns an int
 * status (0 = OK, negative = error, message via swe_gpu_last_error()); no
 * exception crosses the ABI.  One domain handle owns a set of blocks in one
 * device allocation plus a CUDA stream; calls on distinct handles are
 * thread-safe, a single handle is not re-entrant.
 *
 * The entry points replace the reference's block interface:
 *   SWE_Block<T, Buffer>                      src/blocks/SWE_Block.hh:110-251
 *   SWE_DimensionalSplittingMpi               src/blocks/SWE_DimensionalSplittingMpi.hh:52-124
 *   SWE_DimensionalSplittingMPIOverdecomp     src/blocks/SWE_DimensionalSplittingMPIOverdecomp.hh:50-117
 *   SWE_DimensionalSplitting (serial)         src/blocks/SWE_DimensionalSplitting.hh:41-83
 *   solver::{FWave,AugRie,HLLEFun,Hybrid}<float>::computeNetUpdates
 *                                             (call sites src/blocks/SWE_DimensionalSplittingMpi.cpp:403-410)
 * Block arrays use the reference's Float2D layout: a[x][y] = raw[x*ld + y]
 * with ld >= ny+2 (src/tools/Float2D.hh:74-80), ghost ring at 0 and n+1.
 */
#ifndef SWE_GB300_H
#define SWE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWE_GPU_OK 0
#define SWE_GPU_ERR_INVALID (-1)   /* bad argument or handle */
#define SWE_GPU_ERR_CUDA (-2)      /* CUDA runtime error */
#define SWE_GPU_ERR_DEVICE (-3)    /* device-side status flag set (e.g. NaN wave speed) */
#define SWE_GPU_ERR_NOMEM (-4)     /* device allocation failed */
#define SWE_GPU_INCOMPLETE 1       /* not an error: an iteration budget ran out first */

/* Riemann solvers.  The reference chooses at compile time with
 * WAVE_PROPAGATION_SOLVER (SConstruct:543-553, src/blocks/SWE_DimensionalSplittingMpi.hh:42-50):
 * 0 "hybrid" = HLLEFun in the distributed blocks and Hybrid in the serial
 * block, 1 = FWave, 2 = AugRie.  Here the choice is a runtime value. */
#define SWE_SOLVER_FWAVE 1
#define SWE_SOLVER_AUGRIE 2
#define SWE_SOLVER_HYBRID 3
#define SWE_SOLVER_HLLE 4

/* step semantics: UNSPLIT = SWE_DimensionalSplittingMpi / ...MPIOverdecomp
 * (src/blocks/SWE_DimensionalSplittingMpi.cpp:383-518), SPLIT = serial
 * SWE_DimensionalSplitting (src/blocks/SWE_DimensionalSplitting.cpp:105-210) */
#define SWE_SEMANTICS_UNSPLIT 0
#define SWE_SEMANTICS_SPLIT 1

/* how the split block reduces its x wave speed: MAX = max over all x-edges;
 * LAST_EDGE = the reference's one-thread result (the solver overwrites the
 * reduction variable, src/blocks/SWE_DimensionalSplitting.cpp:118-131) */
#define SWE_SPLIT_DT_MAX 0
#define SWE_SPLIT_DT_LAST_EDGE 1

/* BoundaryType values of src/types/Boundary.hh:23-30 */
#define SWE_OUTFLOW 0
#define SWE_WALL 1
#define SWE_INFLOW 2
#define SWE_CONNECT 3
#define SWE_CONNECT_WITHIN_RANK 4
#define SWE_PASSIVE 5

/* Boundary index values of src/types/Boundary.hh:5-10 */
#define SWE_BND_LEFT 0
#define SWE_BND_RIGHT 1
#define SWE_BND_BOTTOM 2
#define SWE_BND_TOP 3

typedef struct swe_gpu_domain swe_gpu_domain;

/* A blocks_x x blocks_y grid of blocks (one simulation, global time step):
 * the overdecomposed layout of src/examples/swe_mpi_overdecomp.cpp:148-225.
 * Block k sits at (k / blocks_y, k % blocks_y) like rank k in
 * src/examples/swe_mpi.cpp:186-187; neighbours get CONNECT_WITHIN_RANK, outer
 * sides `boundary[]`. */
typedef struct swe_gpu_desc {
    int blocks_x, blocks_y;
    const int *nx_cols;  /* blocks_x interior widths */
    const int *ny_rows;  /* blocks_y interior heights */
    float dx, dy;
    int boundary[4];     /* outer boundary types, indexed LEFT, RIGHT, BOTTOM, TOP */
    int solver;          /* SWE_SOLVER_* */
    int semantics;       /* SWE_SEMANTICS_* */
    int split_dt_mode;   /* SWE_SPLIT_DT_* (split semantics only) */
    int tile_rows;       /* rows per CTA (multiple of 32, <= 256); 0 = default */
    int tile_cols;       /* max columns per work segment (<= 128 for the tile mapping); 0 = default */
    int device;          /* CUDA device ordinal */
    int kernel_variant;  /* reserved, must be 0 (the sweep kernels' one thread
                            mapping: CTA tiles of tile_rows rows); any other
                            value is SWE_GPU_ERR_INVALID */
    int speed_pass;      /* 0 = bounded speed pass where available (f-wave or HLLE,
                            unsplit step, CTA tiles): exact wave speeds only where
                            the previous update's speed bounds can reach the
                            maximum; the augmented solver (unsplit, CTA tiles,
                            global time stepping) solves each edge once into edge
                            buffers and applies them; 1 = a speed pass over every
                            edge, then the update pass solving every edge again.
                            All give the same results bit for bit. */
    float lts_max_timestep; /* > 0: local time stepping with synchronisation
                            intervals of this length (the drivers' -l; unsplit
                            step only; advanced with swe_gpu_lts_advance) */
    float duration;      /* simulated duration (local time stepping's last-step notice) */
    int arithmetic;      /* SWE_ARITH_EXACT (0, default): IEEE division and square
                            root, no contraction -- every solver and mode, results
                            identical to the CPU restatement of the reference bit for
                            bit.  SWE_ARITH_FAST: approximate reciprocal / square root
                            and fused multiply-adds, results equal to FP32 round-off;
                            offered for the f-wave and HLLE unsplit step with global
                            time stepping (domains and ensembles), where a step is
                            one launch that also computes the next maxTimestep. */
} swe_gpu_desc;

#define SWE_ARITH_EXACT 0
#define SWE_ARITH_FAST 1

int swe_gpu_domain_create(const swe_gpu_desc *desc, swe_gpu_domain **out);

/* One independent simulation of an ensemble: a single block with its own
 * size, cell size and boundary types. */
typedef struct swe_gpu_instance {
    int nx, ny;          /* interior cells */
    float dx, dy;
    int boundary[4];     /* LEFT, RIGHT, BOTTOM, TOP (no CONNECT_WITHIN_RANK) */
} swe_gpu_instance;

/* An ensemble: `count` independent instances in one domain handle, each its
 * own dt group (own CFL time step, own clock), stepped together by the same
 * persistent launches (swe_gpu_step, swe_gpu_advance; graph replay).  Block k
 * is instance k for uploads, downloads and snapshots.  From `options` only
 * solver, semantics, split_dt_mode, tile_rows, tile_cols, device,
 * kernel_variant (0), speed_pass and arithmetic are used.  The reference runs independent
 * scenarios as separate processes; this has no counterpart there. */
int swe_gpu_ensemble_create(const swe_gpu_instance *instances, int count, const swe_gpu_desc *options,
                            swe_gpu_domain **out);
int swe_gpu_domain_destroy(swe_gpu_domain *dom);
int swe_gpu_block_count(const swe_gpu_domain *dom, int *count);
int swe_gpu_block_shape(const swe_gpu_domain *dom, int block, int *nx, int *ny);

/* Copies one block's state (incl. ghosts) from host arrays in Float2D layout
 * with column stride `ld` floats; NULL skips a field.  Replaces writing the
 * block's h/hu/hv/b (SWE_Block::getModifiable*, src/blocks/SWE_Block.hh:130-142). */
int swe_gpu_upload_block(swe_gpu_domain *dom, int block, const float *h, const float *hu, const float *hv,
                         const float *b, int ld);
/* Copies one block's current state to host arrays; returns when the data is there
 * (SWE_Block::getWaterHeight & co., src/blocks/SWE_Block.hh:128-142). */
int swe_gpu_download_block(swe_gpu_domain *dom, int block, float *h, float *hu, float *hv, float *b, int ld);

/* Whole-domain transfers: host arrays hold every block's (nx+2)*(ny+2) floats
 * in Float2D layout, blocks concatenated in rank order; NULL skips a field.
 * One contiguous copy per field through a device staging buffer (pinned host
 * memory reaches full link bandwidth).  Both return when the copy is done. */
int swe_gpu_upload_domain(swe_gpu_domain *dom, const float *h, const float *hu, const float *hv, const float *b);
int swe_gpu_download_domain(swe_gpu_domain *dom, float *h, float *hu, float *hv, float *b);
/* Asynchronous forms of the two, for pipelines that keep the link busy in both
 * directions -- no counterpart in the reference (its blocks live in host
 * memory).  The host arrays should be pinned; they are read / written after
 * the call returns, in stream order: an upload's inputs must stay unchanged
 * and a download's outputs unread until swe_gpu_sync.  Uploads and downloads
 * each go through two staging slots and a stream of their own, so the link
 * carries step k's results and step k+1's inputs at the same time as the
 * device computes.  The first call of each allocates its slots (8 floats per
 * cell): make both before any stream capture. */
int swe_gpu_upload_domain_async(swe_gpu_domain *dom, const float *h, const float *hu, const float *hv,
                                const float *b);
int swe_gpu_download_domain_async(swe_gpu_domain *dom, float *h, float *hu, float *hv, float *b);

/* Checkpoint snapshot of one block without stopping the simulation: a device
 * kernel writes the current interior of h, hu, hv as big-endian (y, x) slabs
 * (the NetCDF record layout of NetCdfWriter::writeTimeStep,
 * src/writer/NetCdfWriter.cpp:207-234) into a device staging area and
 * copies them to the three host buffers (nx*ny*4 bytes each; pinned memory
 * makes the copy asynchronous).  Returns at once; the data is there after
 * swe_gpu_snapshot_wait.  Steps queued after the call do not disturb it. */
int swe_gpu_snapshot_slabs_async(swe_gpu_domain *dom, int block, void *h, void *hu, void *hv);
int swe_gpu_snapshot_wait(swe_gpu_domain *dom);
/* page-locked host memory for snapshot and transfer buffers (cudaMallocHost) */
int swe_gpu_alloc_pinned(size_t bytes, void **out);
int swe_gpu_free_pinned(void *p);

/* bathymetry ghosts: OUTFLOW/WALL copies (SWE_Block::applyBoundaryBathymetry,
 * src/blocks/SWE_Block.hh:724-749) and neighbour copies (exchangeBathymetry,
 * src/blocks/SWE_DimensionalSplittingMpi.cpp:109-186; sendBathymetry,
 * src/blocks/SWE_DimensionalSplittingMPIOverdecomp.cpp:208-266) */
int swe_gpu_exchange_bathymetry(swe_gpu_domain *dom);

/* setGhostLayer (src/blocks/SWE_DimensionalSplittingMpi.cpp:188-376): boundary
 * conditions and on-device halo copies between blocks.  After an update pass
 * the ring already holds these values (the pass pushed them from the new rim
 * cells), and the call only marks it as the current state's; after an upload
 * it recomputes the ring. */
int swe_gpu_set_ghost_layer(swe_gpu_domain *dom);
/* computeNumericalFluxes (src/blocks/SWE_DimensionalSplittingMpi.cpp:383-476):
 * wave speeds of every edge and the group's maxTimestep, kept on the device */
int swe_gpu_compute_fluxes(swe_gpu_domain *dom);
/* updateUnknowns (src/blocks/SWE_DimensionalSplittingMpi.cpp:484-518); like the
 * reference it applies the maxTimestep of the preceding compute_fluxes and
 * ignores `dt` */
int swe_gpu_update_unknowns(swe_gpu_domain *dom, float dt);
/* getMaxTimestep (src/blocks/SWE_Block.hh:594-597); synchronises */
int swe_gpu_get_max_timestep(swe_gpu_domain *dom, float *dt);

/* `nsteps` fused steps (ghosts + fluxes + update) queued on the stream; no host
 * synchronisation */
int swe_gpu_step(swe_gpu_domain *dom, int nsteps);
/* the drivers' checkpoint loop `while (t < t_end) { step; t += dt; }`
 * (src/examples/swe_mpi.cpp:300-327) run on the device from a captured CUDA
 * graph; returns the executed steps and the float time reached */
int swe_gpu_advance(swe_gpu_domain *dom, float t_end, int max_steps, int *steps_done, float *t_now);
int swe_gpu_get_time(swe_gpu_domain *dom, float *t, int *steps);
/* Update steps every block has executed (one entry per block; under local
 * time stepping blocks step at different rates).  Synchronises. */
int swe_gpu_block_steps(swe_gpu_domain *dom, long long *steps);
/* Local time stepping (domains created with lts_max_timestep > 0): runs
 * synchronisation intervals of every block at its own power-of-two share of
 * the interval, with time-interpolated ghost layers (src/blocks/SWE_Block.hh:311-562,
 * src/examples/swe_mpi_overdecomp.cpp:266-343), until the interval start time
 * t reaches t_end or max_iterations inner iterations ran.  The iterations are
 * decided on the device and replayed from a captured graph of 8; the next
 * replay is queued before the host reads the last one's control block, and
 * iterations past t_end or the limit do nothing.  Returns the finished
 * intervals and t;
 * SWE_GPU_INCOMPLETE when exactly max_iterations inner iterations ran first. */
int swe_gpu_lts_advance(swe_gpu_domain *dom, float t_end, int max_iterations, int *intervals_done, float *t_now);
/* Local time stepping counters: t, finished intervals, inner iterations and,
 * when block_steps is not null, each block's number of steps (power-of-two
 * divisor) in the last finished interval. */
int swe_gpu_lts_state(swe_gpu_domain *dom, float *t, int *intervals, int *iterations, int *block_steps);
/* Ghost-layer state machine of every block: ints[8k..8k+7] = the state of the
 * LEFT, RIGHT, BOTTOM, TOP layers (0 done, 1 invalid, 2 interpolated, 3 in
 * sync, 4 next), stepSize, stepSizeCounter, timestepCounter, last-timestep
 * notice; border[4k..4k+3] = the neighbours' local times of the layers. */
int swe_gpu_lts_blocks(swe_gpu_domain *dom, int *ints, float *border);
/* getRoundTimestep (src/blocks/SWE_Block.hh:536-555) as the device applies it
 * at the start of an interval: for each of the n time steps t (host array),
 * the step size (power-of-two divisor of max_timestep_local, at most
 * max_divisor) a block with that maxTimestep takes.  Evaluated on `device`;
 * for tests and tools. */
int swe_gpu_lts_round_timesteps(const float *t, int n, float max_timestep_local, int max_divisor, int *step_sizes,
                                int device);
/* dt groups (1 for a grid of blocks, one per instance of an ensemble or per
 * block under local time stepping) and their clocks: time, last dt and steps
 * (arrays of group-count entries, any may be null).  Synchronises. */
int swe_gpu_group_count(const swe_gpu_domain *dom, int *count);
int swe_gpu_group_state(swe_gpu_domain *dom, float *time, float *dt, int *steps);

/* Re-partitions the step kernels' work for another tile shape (rows per CTA,
 * a multiple of 32 up to 256; cap on columns per work segment, 0 = balanced
 * default).  The state is untouched; results do not depend on the shape. */
int swe_gpu_retile(swe_gpu_domain *dom, int tile_rows, int tile_cols);
/* Tile-shape tuner: times `trial_steps` steps for each candidate shape on a
 * copy of the current state (restored after every trial), keeps the fastest
 * and reports it.  Needs room for one more copy of h, hu, hv. */
int swe_gpu_autotune(swe_gpu_domain *dom, int trial_steps, int *best_rows, int *best_cols, float *best_ms);

/* Kernels this domain has enqueued so far (a replay of the captured step
 * graph counts each of its kernel nodes); no synchronisation. */
int swe_gpu_launch_count(const swe_gpu_domain *dom, long long *count);
/* Bounded speed pass: bound tiles of the domain and how many of them the
 * last pass evaluated edge by edge (both 0 when the full speed pass is in
 * use).  Synchronises the domain's stream. */
int swe_gpu_speed_pass_stats(swe_gpu_domain *dom, int *tiles, int *evaluated);

/* The fast step's pieces (SWE_ARITH_FAST): runs of next-state edges whose
 * two cells are written by different work segments, evaluated for the next
 * maxTimestep by the last of those segments to finish.  Five ints per piece:
 * block, dir (0: x-edges (x0-1|x0) of rows y0 .. y0+len-1; 1: y-edges
 * (y0-1|y0) of columns x0 .. x0+len-1), x0, y0, len.  Writes at most `cap`
 * pieces to `out` (may be NULL with cap 0); *count = the number of pieces.
 * Introspection for tests and tools; no counterpart in the reference. */
int swe_gpu_fast_pieces(const swe_gpu_domain *dom, int *out, int cap, int *count);
int swe_gpu_set_time(swe_gpu_domain *dom, float t);

/* waits for everything queued on the domain (steps, transfers, async downloads) */
int swe_gpu_sync(swe_gpu_domain *dom);
/* device-side status bits (bit 0: NaN wave speed); 0 when healthy */
int swe_gpu_status(swe_gpu_domain *dom, int *status);
/* the CUDA stream the handle launches on (a cudaStream_t) */
int swe_gpu_get_stream(swe_gpu_domain *dom, void **stream);
/* launch on a caller's CUDA stream (a cudaStream_t of the handle's device,
 * e.g. a framework's current stream); NULL returns to the handle's own stream */
int swe_gpu_set_stream(swe_gpu_domain *dom, void *stream);
/* message of the last failed call on this thread */
const char *swe_gpu_last_error(void);
int swe_gpu_version(void);

/* Per-edge solver on device arrays (solver::X<float>::computeNetUpdates over n
 * edges): inputs hL, hR, huL, huR, bL, bR; outputs hUpdL, hUpdR, huUpdL,
 * huUpdR, maxWaveSpeed.  All pointers are device memory; `stream` may be NULL. */
int swe_gpu_solve_edges(int solver, long long n, const float *hL, const float *hR, const float *huL,
                        const float *huR, const float *bL, const float *bR, float *hUpdL, float *hUpdR,
                        float *huUpdL, float *huUpdR, float *maxWaveSpeed, void *stream);

/* Allocation-free step of one block -- no counterpart in the reference.
 * For callers that cannot allocate device memory: hosts whose GPU memory
 * belongs to another allocator (a framework's caching pool, a fixed arena)
 * and latency-critical loops that cannot take cudaMalloc's implicit device
 * synchronisation.  Runs setGhostLayer + computeNumericalFluxes +
 * updateUnknowns of one block (solver, semantics as above; split semantics
 * reduce dt with SWE_SPLIT_DT_MAX) on caller-owned DEVICE arrays in Float2D
 * layout with column stride ld >= ny+2: h, hu, hv hold Q^n (their ghost cells
 * are written, like setGhostLayer), b the bathymetry with its ghosts,
 * h_out/hu_out/hv_out receive Q^{n+1} with its ghost ring already set for
 * the next step, and must not alias the inputs.  If dt_out (host) is not NULL the call waits for the
 * stream and stores the step's dt there.  Nothing is allocated: the scratch
 * (dt control block, block descriptor, CTA work list) is a fixed array of
 * about 82 KB that every GPU loading the library holds until exit, so the
 * block may need at most 4096 work units, ceil(ny/256) * ceil(nx/32); larger
 * blocks are rejected with SWE_GPU_ERR_INVALID.  The first call on a device
 * looks the array's device address up (cudaGetSymbolAddress); make that first
 * call before any stream capture.  A call that meets a CUDA error forgets the
 * address, so the next call looks it up again (after a cudaDeviceReset).  Every call on a device shares the array and
 * clears it when it starts: calls that overlap on the GPU race. */
int swe_gpu_step_block_noalloc(int solver, int semantics, int nx, int ny, float dx, float dy, const int *boundary4,
                               int ld, float *h, float *hu, float *hv, const float *b, float *h_out, float *hu_out,
                               float *hv_out, float *dt_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif
