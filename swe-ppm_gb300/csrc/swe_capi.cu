// C ABI of the GB300 block step (include/swe_gb300.h): domain set-up, state
// transfer, the ghost-layer and bathymetry kernels, and the step drivers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/swe_gb300.h"
#include "../../include/swe_gb300_mlp.h"
#include "swe_device.cuh"
#include "swe_fast.hpp"
#include "swe_launch.hpp"
#include "swe_mlp_launch.hpp"


using namespace swegb;

namespace {

thread_local std::string g_lastError;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_lastError = buf;
    return code;
}

#define CUDA_TRY(call)                                                                            \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(SWE_GPU_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// ---------------------------------------------------------------------------
// setGhostLayer: boundary conditions (src/blocks/SWE_Block.hh:757-911) and the
// intra-rank copies of the neighbours' copy layers
// (src/blocks/SWE_DimensionalSplittingMPIOverdecomp.cpp:273-304).  One thread
// per ghost cell of one block (blockIdx.y); reads touch only interior cells,
// writes only ghost cells, so blocks never race.
// ---------------------------------------------------------------------------
/// mode 0: state ghosts of the groups still stepping; 1: bathymetry ghosts;
/// 2: the next step's state ghosts of the groups whose update just finished
/// (ghostsAhead set), as the two-pass update pass pushes them -- the previous
/// ring stays in the other buffer for downloads; 3: the ring is already the
/// one mode 0 would write (the update pass pushed it): only hand it to the
/// current state, as mode 0 does
__global__ void ghostKernel(const DomainDev d, int mode) {
    const bool bathymetry = mode == 1;
    const BlockDesc B = d.blocks[blockIdx.y];
    const GroupState *G = d.groups + B.group;
    if ((mode == 0 || mode == 3) && !(*((volatile const float *)&G->time) < *((volatile const float *)&G->target))) return;
    if (mode == 3) {
        if (threadIdx.x == 0) const_cast<GroupState *>(G)->ghostsAhead = 0;
        return;
    }
    if (mode == 2 && !*((volatile const int *)&G->ghostsAhead)) return;
    const int cur = G->cur;
    const int nx = B.nx, ny = B.ny;
    const size_t P = size_t(B.pitch);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    // the ghost ring of the current buffer now belongs to the current state
    if (mode == 0 && threadIdx.x == 0) const_cast<GroupState *>(G)->ghostsAhead = 0;
    float *fields[3];
    int nf;
    if (bathymetry) {
        fields[0] = d.b;
        nf = 1;
    } else {
        fields[0] = cur ? d.h[1] : d.h[0];
        fields[1] = cur ? d.hu[1] : d.hu[0];
        fields[2] = cur ? d.hv[1] : d.hv[0];
        nf = 3;
    }
    int side, pos;
    if (i < ny) { side = 0; pos = i + 1; }
    else if (i < 2 * ny) { side = 1; pos = i - ny + 1; }
    else if (i < 2 * ny + nx) { side = 2; pos = i - 2 * ny + 1; }
    else if (i < 2 * ny + 2 * nx) { side = 3; pos = i - 2 * ny - nx + 1; }
    else if (i < 2 * ny + 2 * nx + 4) { side = 4; pos = i - 2 * ny - 2 * nx; }
    else return;

    if (side == 4) {  // corners from the diagonal interior cell
        const int gx = (pos & 1) ? nx + 1 : 0, gy = (pos & 2) ? ny + 1 : 0;
        const int sx = (pos & 1) ? nx : 1, sy = (pos & 2) ? ny : 1;
        for (int f = 0; f < nf; f++) {
            float *F = fields[f] + B.base;
            F[size_t(gx) * P + gy] = F[size_t(sx) * P + sy];
        }
        return;
    }
    const int type = B.bnd[side];
    // ghost cell and its source inside this block
    int gx, gy, sx, sy, negate;
    switch (side) {
    case 0: gx = 0; gy = pos; sx = 1; sy = pos; negate = 1; break;
    case 1: gx = nx + 1; gy = pos; sx = nx; sy = pos; negate = 1; break;
    case 2: gx = pos; gy = 0; sx = pos; sy = 1; negate = 2; break;
    default: gx = pos; gy = ny + 1; sx = pos; sy = ny; negate = 2; break;
    }
    long long srcBase = B.base;
    size_t srcP = P;
    if (type == CONNECT_WITHIN_RANK) {
        const BlockDesc N = d.blocks[B.nbr[side]];
        srcBase = N.base;
        srcP = size_t(N.pitch);
        switch (side) {
        case 0: sx = N.nx; break;
        case 1: sx = 1; break;
        case 2: sy = N.ny; break;
        default: sy = 1; break;
        }
        negate = 0;
    } else if (type == OUTFLOW) {
        negate = 0;
    } else if (type != WALL) {
        return;  // CONNECT, INFLOW, PASSIVE: set elsewhere
    }
    if (bathymetry) negate = 0;
    for (int f = 0; f < nf; f++) {
        const float v = fields[f][srcBase + size_t(sx) * srcP + sy];
        fields[f][B.base + size_t(gx) * P + gy] = (negate == f && f > 0) ? -v : v;
    }
}

/// the target time of every group (steps run while time < target)
__global__ void setTargetsKernel(GroupState *g, int n, float target) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) g[i].target = target;
}

/// per-edge solver over arrays (solver::X<float>::computeNetUpdates)
template <int S>
__global__ void solveEdgesKernel(long long n, const float *hL, const float *hR, const float *huL, const float *huR,
                                 const float *bL, const float *bR, float *oHL, float *oHR, float *oHuL, float *oHuR,
                                 float *oS) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float a = hL[i], c = hR[i], e = huL[i], f = huR[i];
    Cell L, R;
    L.h = a; L.hn = e; L.b = bL[i];
    R.h = c; R.hn = f; R.b = bR[i];
    // per-cell quantities as the sweep kernels form them
    L.u = (a < kDryTol) ? 0.f : e * (1.f / a);
    R.u = (c < kDryTol) ? 0.f : f * (1.f / c);
    L.sq = sqrtf(a); R.sq = sqrtf(c);
    L.c = kSqrtG * L.sq; R.c = kSqrtG * R.sq;
    edgeSolve<S>(L, R, oHL[i], oHR[i], oHuL[i], oHuR[i], oS[i]);
}

/// Copies between the contiguous host-order layout (blocks concatenated, each
/// (nx+2)*(ny+2) floats, a[x][y] = raw[x*(ny+2)+y]) in `stage` and the padded
/// device layout of the current buffer; one CTA per column of one block.
/// fieldMask bit f selects h, hu, hv, b; stage holds field f at f*stageElems.
__global__ void repackKernel(const DomainDev d, float *stage, long long stageElems, int toDevice, int fieldMask,
                             int blockOffset) {
    const int k = blockIdx.y + blockOffset;
    const BlockDesc B = d.blocks[k];
    const int x = blockIdx.x;
    if (x > B.nx + 1) return;
    GroupState *G = d.groups + B.group;
    const int cur = G->cur;
    // After an update pass the current buffer's ghost ring already holds the
    // next step's boundary values; the block's state as the reference shows
    // it (ghosts set at the start of the last step) has them in the other buffer.
    const bool ahead = !toDevice && G->ghostsAhead;
    if (toDevice && x == 0 && threadIdx.x == 0) {
        G->ghostsAhead = 0;
        if (fieldMask & 7) {
            G->boundsValid[0] = 0;
            G->boundsValid[1] = 0;
        }
    }
    float *fields[4] = {cur ? d.h[1] : d.h[0], cur ? d.hu[1] : d.hu[0], cur ? d.hv[1] : d.hv[0], d.b};
    float *other[4] = {cur ? d.h[0] : d.h[1], cur ? d.hu[0] : d.hu[1], cur ? d.hv[0] : d.hv[1], d.b};
    const int rows = B.ny + 2;
    const bool ghostColumn = (x == 0) || (x == B.nx + 1);
    for (int f = 0; f < 4; f++) {
        if (!(fieldMask & (1 << f))) continue;
        float *dev = fields[f] + B.base + size_t(x) * size_t(B.pitch);
        float *oth = other[f] + B.base + size_t(x) * size_t(B.pitch);
        float *st = stage + size_t(f) * size_t(stageElems) + size_t(B.stage) + size_t(x) * size_t(rows);
        for (int y = threadIdx.x; y < rows; y += blockDim.x) {
            if (toDevice) {
                dev[y] = st[y];
            } else {
                const bool ghost = ghostColumn || y == 0 || y == rows - 1;
                st[y] = (ahead && ghost) ? oth[y] : dev[y];
            }
        }
    }
}

/// interior of the current state of block k as big-endian (y, x) slabs:
/// out[f][j*nx + i] = field_f(i+1, j+1); 32 x 32 tiles transposed through
/// shared memory so both the column reads and the row writes are coalesced
__global__ void snapshotKernel(const DomainDev d, int k, uint32_t *out) {
    __shared__ float tile[32][33];
    const BlockDesc B = d.blocks[k];
    const int cur = d.groups[B.group].cur;
    const float *fields[3] = {cur ? d.h[1] : d.h[0], cur ? d.hu[1] : d.hu[0], cur ? d.hv[1] : d.hv[0]};
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    const size_t slab = size_t(B.nx) * size_t(B.ny);
    for (int f = 0; f < 3; f++) {
        const float *F = fields[f] + B.base;
        for (int r = threadIdx.y; r < 32; r += blockDim.y) {
            const int i = i0 + r, j = j0 + threadIdx.x;
            if (i < B.nx && j < B.ny) tile[r][threadIdx.x] = F[size_t(i + 1) * size_t(B.pitch) + size_t(j + 1)];
        }
        __syncthreads();
        for (int r = threadIdx.y; r < 32; r += blockDim.y) {
            const int j = j0 + r, i = i0 + threadIdx.x;
            if (i < B.nx && j < B.ny) {
                const uint32_t u = __float_as_uint(tile[threadIdx.x][r]);
                out[size_t(f) * slab + size_t(j) * size_t(B.nx) + size_t(i)] = __byte_perm(u, 0, 0x0123);
            }
        }
        __syncthreads();
    }
}

} // namespace

struct swe_gpu_domain {
    int device = 0;
    cudaStream_t stream = nullptr;     // stream launches go to
    cudaStream_t ownStream = nullptr;  // the handle's own stream
    int solver = SOLVER_HLLE, semantics = SEM_UNSPLIT, splitDtMode = SPLIT_DT_MAX;
    int tileRows = 256, tileCols = 32;
    int tileColsArg = 0;              // segment-length cap asked for (0: default)
    std::vector<BlockDesc> blocks;
    std::vector<WorkUnit> units;
    std::vector<GroupState> groupsInit;
    int ngroups = 1;
    int maxPerimeter = 0;
    size_t fieldElems = 0;
    float *h[2] = {nullptr, nullptr}, *hu[2] = {nullptr, nullptr}, *hv[2] = {nullptr, nullptr}, *b = nullptr;
    BlockDesc *dBlocks = nullptr;
    WorkUnit *dUnits = nullptr;
    int *dCtaSeg = nullptr;
    GroupState *dGroups = nullptr;
    std::vector<int> ctaSeg;      // speed pass: worker c owns segments [ctaSeg[c], ctaSeg[c+1])
    int grid = 0;                 // CTAs of the speed pass
    std::vector<WorkUnit> unitsU; // update pass segments and owners
    std::vector<int> ctaSegU;
    int gridU = 0;
    WorkUnit *dUnitsU = nullptr;
    int *dCtaSegU = nullptr;
    bool ghostsValid = false;     // the current buffer's ghost ring matches its interior
    DomainDev dev{};
    float *stage = nullptr;       // host-order staging for transfers (4 fields)
    long long stageElems = 0;     // floats per field in the staging layout
    int maxCols = 0;              // max nx+2 over blocks
    cudaGraphExec_t graph = nullptr;
    int graphSteps = 0;
    cudaEvent_t snapEvent = nullptr;  // completion of the last snapshot copy
    bool bounded = false;             // bounded speed pass (f-wave / HLLE, unsplit, CTA tiles)
    std::vector<TileInfo> tiles;      // bound tiles of all blocks
    TileInfo *dTiles = nullptr;
    unsigned int *dTileW = nullptr;   // 2 parities x tiles
    unsigned long long *dTileKey = nullptr;
    int gridB = 0;                    // CTAs of the bounded speed pass
    long long launches = 0;           // kernels enqueued (graph replays: per kernel node)
    long long graphKernels = 0;       // kernel nodes of the captured step graph
    // local time stepping
    bool lts = false;
    LtsBlock *dLts = nullptr;
    LtsControl *dLtsCtl = nullptr;
    int *dLtsWork = nullptr;     // work lists of the running iteration
    float *dLtsLocal = nullptr;  // published total local time per block
    float *dRing[3] = {nullptr, nullptr, nullptr};
    long long ringElems = 0;
    cudaGraphExec_t ltsGraph = nullptr;
    long long ltsGraphKernels = 0;
    // the control block after each of two replays in flight (pinned) and
    // the events that mark its copy
    LtsControl *ltsCtlHost = nullptr;
    cudaEvent_t ltsCtlReady[2] = {nullptr, nullptr};
    // surrogate step and edge logger: edge tiles and the stored net updates
    std::vector<mlp::EdgeTile> edgeTiles;
    mlp::EdgeTile *dEdgeTiles = nullptr;
    float *edgeBuf = nullptr;             // 8 fields: x-edge then y-edge net updates
    unsigned long long *dUsed = nullptr;  // edges the surrogate solved
    // augmented solver, unsplit, CTA tiles, global time stepping: the step
    // solves every edge once into the edge buffers (computeNumericalFluxes)
    // and applies them (updateUnknowns) instead of solving each edge in both
    // the speed and the update pass
    bool edgeBuffered = false;
    // asynchronous downloads: two staging slots (4 fields each), copied out on
    // a second stream so one step's download overlaps the next one's upload
    float *stageDown[2] = {nullptr, nullptr};
    cudaStream_t copyStream = nullptr;
    cudaEvent_t downReady[2] = {nullptr, nullptr}, downDone[2] = {nullptr, nullptr};
    int downSlot = 0;
    bool downUsed[2] = {false, false};
    // asynchronous uploads: two staging slots filled on a third stream
    float *stageUp[2] = {nullptr, nullptr};
    cudaStream_t upStream = nullptr;
    cudaEvent_t upReady[2] = {nullptr, nullptr}, upConsumed[2] = {nullptr, nullptr};
    int upSlot = 0;
    bool upUsed[2] = {false, false};
    // fast-arithmetic step (SWE_ARITH_FAST): one launch per step that also
    // computes the next maxTimestep; dtValid = the groups' dt describes the
    // current state (false after an upload or a bathymetry change, until a
    // speed pass or a fast step has run)
    bool fast = false;
    bool dtValid = false;
    std::vector<fast::Unit> unitsF;
    std::vector<int> ctaSegF;
    std::vector<fast::Piece> pieces;
    std::vector<int> arrF;
    int gridF = 0;
    int tileRowsF = 256;          // rows per segment of the fast step (>= 64)
    fast::Unit *dUnitsF = nullptr;
    int *dCtaSegF = nullptr;
    fast::Piece *dPieces = nullptr;
    unsigned *dPieceCnt = nullptr;
    int *dArrF = nullptr;
};

namespace {

/// ghost kernel launch; mode as ghostKernel's
int enqueueGhost(swe_gpu_domain *D, int mode) {
    const int threads = mode == 3 ? 32 : 128;
    dim3 grid(mode == 3 ? 1 : (D->maxPerimeter + threads - 1) / threads, unsigned(D->blocks.size()));
    ghostKernel<<<grid, threads, 0, D->stream>>>(D->dev, mode);
    CUDA_TRY(cudaGetLastError());
    D->launches++;
    return SWE_GPU_OK;
}

mlp::EdgeUpdates edgeUpdates(const swe_gpu_domain *D) {
    mlp::EdgeUpdates u;
    for (int k = 0; k < 4; k++) {
        u.x[k] = D->edgeBuf + size_t(k) * D->fieldElems;
        u.y[k] = D->edgeBuf + size_t(4 + k) * D->fieldElems;
    }
    return u;
}

long long maxBlockCells(const swe_gpu_domain *D) {
    long long m = 0;
    for (const BlockDesc &B : D->blocks) m = std::max(m, (long long)B.nx * B.ny);
    return m;
}

int enqueueSpeed(swe_gpu_domain *D) {
    DomainDev d = D->dev;
    if (D->edgeBuffered) {
        CUDA_TRY(mlp::launchSurrogateEdges(d, nullptr, D->dEdgeTiles, int(D->edgeTiles.size()), edgeUpdates(D), D->dUsed,
                                           D->stream));
        CUDA_TRY(mlp::launchSurrogateDt(d, D->ngroups, D->stream));
        D->launches += 2;
        return SWE_GPU_OK;
    }
    if (D->bounded) {
        CUDA_TRY(launchSpeedBound(d, D->gridB, D->stream));
        D->launches++;
        return SWE_GPU_OK;
    }
    d.units = D->dUnits;
    d.ctaSeg = D->dCtaSeg;
    // local time stepping: most iterations list no block for the speed pass
    // (a block needs it only at the start of its interval); two CTAs per SM
    // measured 1% faster per iteration than the full grid, one or three slower
    int grid = D->grid;
    if (D->lts) {
        int sms = 148;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, D->device);
        grid = std::min(grid, 2 * sms);
    }
    CUDA_TRY(launchSpeed(d, grid, D->tileRows, D->stream));
    D->launches++;
    return SWE_GPU_OK;
}

int enqueueUpdate(swe_gpu_domain *D) {
    DomainDev d = D->dev;
    if (D->edgeBuffered) {
        CUDA_TRY(mlp::launchSurrogateApply(d, edgeUpdates(D), int(D->blocks.size()), maxBlockCells(D), D->stream));
        CUDA_TRY(mlp::launchSurrogateFinish(d, D->ngroups, D->stream));
        D->launches += 2;
        // the new state's ghost ring, as the two-pass update leaves it
        int rc = enqueueGhost(D, 2);
        if (rc) return rc;
        D->ghostsValid = true;
        return SWE_GPU_OK;
    }
    d.units = D->dUnitsU;
    d.ctaSeg = D->dCtaSegU;
    CUDA_TRY(launchUpdate(d, D->gridU, D->tileRows, D->stream));
    D->launches++;
    D->ghostsValid = true;  // the update pass pushed the next ghost ring
    return SWE_GPU_OK;
}

/// the fast step's launch
int enqueueFast(swe_gpu_domain *D) {
    fast::FastDev f;
    f.d = D->dev;
    f.units = D->dUnitsF;
    f.ctaSeg = D->dCtaSegF;
    f.pieces = D->dPieces;
    f.pieceCnt = D->dPieceCnt;
    f.arr = D->dArrF;
    CUDA_TRY(fast::launchFastStep(f, D->solver, D->gridF, D->tileRowsF, D->stream));
    D->launches++;
    D->ghostsValid = true;  // the step pushed the next ghost ring
    D->dtValid = true;      // and computed the next maxTimestep
    return SWE_GPU_OK;
}

/// fast arithmetic: the speed pass runs only when the groups' dt does not
/// describe the current state (first step, after an upload)
int enqueueFastPrologue(swe_gpu_domain *D) {
    if (!D->ghostsValid) {
        int rc = enqueueGhost(D, 0);
        if (rc) return rc;
        D->ghostsValid = true;
    }
    if (!D->dtValid) {
        DomainDev d = D->dev;
        d.units = D->dUnits;
        d.ctaSeg = D->dCtaSeg;
        CUDA_TRY(launchSpeed(d, D->grid, D->tileRows, D->stream));
        D->launches++;
        D->dtValid = true;
    }
    return SWE_GPU_OK;
}

/// one fused step; the ghost kernel runs only when the ghost ring is stale
/// (after an upload), every update pass leaves a valid one behind
int enqueueStep(swe_gpu_domain *D) {
    if (D->fast) {
        int rc = enqueueFastPrologue(D);
        if (rc) return rc;
        return enqueueFast(D);
    }
    if (!D->ghostsValid) {
        int rc = enqueueGhost(D, 0);
        if (rc) return rc;
        D->ghostsValid = true;
    }
    int rc = enqueueSpeed(D);
    if (rc) return rc;
    return enqueueUpdate(D);
}

/// one inner iteration of local time stepping (see swe_lts.cu): check
/// (with the exchange), speed pass of the blocks at an interval start
/// (unless the check runs it, DomainDev::ltsCheckSpeed), update pass of the
/// enabled blocks (with the iteration's end)
int enqueueLtsIteration(swe_gpu_domain *D) {
    int sidePositions = 0;  // positions of a side pair (LEFT + RIGHT or BOTTOM + TOP)
    for (const BlockDesc &B : D->blocks) sidePositions = std::max(sidePositions, 2 * std::max(B.nx, B.ny));
    CUDA_TRY(launchLtsCheck(D->dev, D->stream, !D->dev.ltsCheckSpeed, sidePositions));
    D->launches++;
    if (!D->dev.ltsCheckSpeed) {  // (else the check computed the interval starts' dt)
        int rc = enqueueSpeed(D);
        if (rc) return rc;
    }
    return enqueueUpdate(D);
}

int readGroups(swe_gpu_domain *D, std::vector<GroupState> &g) {
    g.resize(D->ngroups);
    CUDA_TRY(cudaStreamSynchronize(D->stream));
    CUDA_TRY(cudaMemcpy(g.data(), D->dGroups, sizeof(GroupState) * D->ngroups, cudaMemcpyDeviceToHost));
    return SWE_GPU_OK;
}

int setTargets(swe_gpu_domain *D, float target) {
    setTargetsKernel<<<(D->ngroups + 255) / 256, 256, 0, D->stream>>>(D->dGroups, D->ngroups, target);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(D->stream));
    return SWE_GPU_OK;
}

void freeDomain(swe_gpu_domain *D) {
    if (D->graph) cudaGraphExecDestroy(D->graph);
    if (D->ltsGraph) cudaGraphExecDestroy(D->ltsGraph);
    cudaFree(D->dLts);
    cudaFree(D->dLtsCtl);
    cudaFree(D->dLtsWork);
    cudaFree(D->dLtsLocal);
    for (int f = 0; f < 3; f++) cudaFree(D->dRing[f]);
    if (D->ltsCtlHost) cudaFreeHost(D->ltsCtlHost);
    for (int j = 0; j < 2; j++)
        if (D->ltsCtlReady[j]) cudaEventDestroy(D->ltsCtlReady[j]);
    if (D->snapEvent) cudaEventDestroy(D->snapEvent);
    for (int i = 0; i < 2; i++) {
        cudaFree(D->h[i]);
        cudaFree(D->hu[i]);
        cudaFree(D->hv[i]);
    }
    cudaFree(D->b);
    cudaFree(D->stage);
    cudaFree(D->dBlocks);
    cudaFree(D->dUnits);
    cudaFree(D->dCtaSeg);
    cudaFree(D->dUnitsU);
    cudaFree(D->dCtaSegU);
    cudaFree(D->dUnitsF);
    cudaFree(D->dCtaSegF);
    cudaFree(D->dPieces);
    cudaFree(D->dPieceCnt);
    cudaFree(D->dArrF);
    cudaFree(D->dGroups);
    cudaFree(D->dTiles);
    cudaFree(D->dTileW);
    cudaFree(D->dTileKey);
    cudaFree(D->dEdgeTiles);
    cudaFree(D->edgeBuf);
    cudaFree(D->dUsed);
    for (int j = 0; j < 2; j++) {
        cudaFree(D->stageDown[j]);
        if (D->downReady[j]) cudaEventDestroy(D->downReady[j]);
        if (D->downDone[j]) cudaEventDestroy(D->downDone[j]);
    }
    if (D->copyStream) {
        cudaStreamSynchronize(D->copyStream);
        cudaStreamDestroy(D->copyStream);
    }
    for (int j = 0; j < 2; j++) {
        cudaFree(D->stageUp[j]);
        if (D->upReady[j]) cudaEventDestroy(D->upReady[j]);
        if (D->upConsumed[j]) cudaEventDestroy(D->upConsumed[j]);
    }
    if (D->upStream) {
        cudaStreamSynchronize(D->upStream);
        cudaStreamDestroy(D->upStream);
    }
    if (D->ownStream) cudaStreamDestroy(D->ownStream);
    delete D;
}

int checkBlock(const swe_gpu_domain *D, int block) {
    if (!D) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    if (block < 0 || block >= int(D->blocks.size()))
        return fail(SWE_GPU_ERR_INVALID, "block %d out of range [0, %d)", block, int(D->blocks.size()));
    return SWE_GPU_OK;
}

} // namespace

extern "C" {

const char *swe_gpu_last_error(void) { return g_lastError.c_str(); }

int swe_gpu_version(void) { return 1; }

namespace {

/// one block before layout: interior size, cell size, sides, dt group
struct BlockSpec {
    int nx, ny;
    float dx, dy;
    int bnd[4];  // boundary types; CONNECT_WITHIN_RANK where nbr >= 0
    int nbr[4];
    int group;
};

struct DomainOptions {
    int device, solver, semantics, splitDtMode, tileRows, tileCols, speedPass, arithmetic;
    float ltsMaxTimestep, duration;
    int ngroups;
};

/// Balanced persistent partitions of both passes for the domain's current
/// tile shape; tileColsArg > 0 caps the segment length.
void buildPartitions(swe_gpu_domain *D, int tileColsArg) {
    D->units.clear();
    D->unitsU.clear();
    D->ctaSeg.clear();
    D->ctaSegU.clear();
    // Balanced persistent partitions, one per pass (the two kernels differ in
    // registers and therefore in resident CTAs): the (row tile, column) pairs
    // of all blocks in order, split into `workers` equal runs, one per CTA; a
    // run that crosses a tile or a block boundary becomes several segments.  tile_cols,
    // when given, caps the segment length and raises the number of workers.
    for (int pass = 0; pass < 2; pass++) {
        int sms = 148;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, D->device);
        const int rowsPerTile = D->tileRows;
        const int occ = passOccupancy(D->solver, D->semantics, pass == 1, D->tileRows);
        const long long perSM = std::max(1, std::min(16, occ));
        long long total = 0;
        for (const BlockDesc &B : D->blocks) total += (long long)((B.ny + rowsPerTile - 1) / rowsPerTile) * B.nx;
        long long workers = (long long)sms * perSM;
        if (tileColsArg > 0) workers = std::max(workers, (total + tileColsArg - 1) / tileColsArg);
        workers = std::max(1LL, std::min(total, workers));
        std::vector<WorkUnit> &units = pass ? D->unitsU : D->units;
        std::vector<int> &ctaSeg = pass ? D->ctaSegU : D->ctaSeg;
        (pass ? D->gridU : D->grid) = int(workers);
        ctaSeg.assign(1, 0);
        long long pos = 0;  // global (tile, column) index
        int k = 0, tile = 0, col = 1;
        auto tiles = [&](int kk) { return (D->blocks[kk].ny + rowsPerTile - 1) / rowsPerTile; };
        for (long long c = 0; c < workers; c++) {
            const long long end = total * (c + 1) / workers;
            while (pos < end) {
                const BlockDesc &B = D->blocks[k];
                const long long take = std::min<long long>(end - pos, (long long)(B.nx + 1 - col));
                const int cap = tileColsArg > 0 ? tileColsArg : kMaxTileCols;
                const int len = int(std::min<long long>(take, cap));
                units.push_back(WorkUnit{k, 1 + tile * rowsPerTile, col, col + len});
                pos += len;
                col += len;
                if (col > B.nx) {
                    col = 1;
                    if (++tile >= tiles(k)) {
                        tile = 0;
                        k++;
                    }
                }
            }
            ctaSeg.push_back(int(units.size()));
        }
    }
}

/// Partition and pieces of the fast step (swe_fast.cu).  Segments: the
/// (row tile, column) pairs of all blocks split evenly over a persistent
/// grid sized from the kernel's occupancy, as for the update pass.  Pieces:
/// each segment's left edge column (x0-1 | x0) and bottom edge row
/// (y0-1 | y0) where the cell across belongs to another segment (the
/// neighbouring segment of the tile, the tile below, or the neighbour block
/// that fills this block's ghost column / row); every segment writing one of
/// the piece's cells arrives on it.  Returns false when blocks that share a
/// side differ in the length of that side (the pieces would not line up).
bool buildFastPlan(swe_gpu_domain *D) {
    D->unitsF.clear();
    D->ctaSegF.clear();
    D->pieces.clear();
    D->arrF.clear();
    // whole warps of fastRows() rows per thread
    const int rowsPerWarp = 32 * fast::fastRows();
    const int TY = std::min(kMaxTileRows, (std::max(rowsPerWarp, D->tileRows) + rowsPerWarp - 1) / rowsPerWarp * rowsPerWarp);
    D->tileRowsF = TY;
    int sms = 148;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, D->device);
    const int occ = std::max(1, std::min(16, fast::fastOccupancy(D->solver, TY)));
    long long total = 0;
    for (const BlockDesc &B : D->blocks) total += (long long)((B.ny + TY - 1) / TY) * B.nx;
    long long workers = (long long)sms * occ;
    if (D->tileColsArg > 0) workers = std::max(workers, (total + D->tileColsArg - 1) / D->tileColsArg);
    workers = std::max(1LL, std::min(total, workers));
    D->gridF = int(workers);
    const int cap = D->tileColsArg > 0 ? std::min(D->tileColsArg, kMaxTileCols) : kMaxTileCols;
    D->ctaSegF.assign(1, 0);
    long long pos = 0;
    int k = 0, tile = 0, col = 1;
    auto tilesOf = [&](int kk) { return (D->blocks[kk].ny + TY - 1) / TY; };
    for (long long c = 0; c < workers; c++) {
        const long long end = total * (c + 1) / workers;
        while (pos < end) {
            const BlockDesc &B = D->blocks[k];
            const long long take = std::min<long long>(end - pos, (long long)(B.nx + 1 - col));
            const int len = int(std::min<long long>(take, cap));
            D->unitsF.push_back(fast::Unit{k, 1 + tile * TY, col, col + len, 0, 0});
            pos += len;
            col += len;
            if (col > B.nx) {
                col = 1;
                if (++tile >= tilesOf(k)) {
                    tile = 0;
                    k++;
                }
            }
        }
        D->ctaSegF.push_back(int(D->unitsF.size()));
    }
    // segments of every (block, tile) in column order
    std::vector<std::vector<std::vector<int>>> segsOf(D->blocks.size());
    for (size_t b = 0; b < D->blocks.size(); b++) segsOf[b].resize(tilesOf(int(b)));
    for (int s = 0; s < int(D->unitsF.size()); s++) {
        const fast::Unit &u = D->unitsF[s];
        segsOf[u.block][(u.y0 - 1) / TY].push_back(s);
    }
    auto covering = [&](int blk, int ti, int xa, int xb, std::vector<int> &out) {
        for (int s : segsOf[blk][ti]) {
            const fast::Unit &u = D->unitsF[s];
            if (u.x0 < xb && xa < u.x1) out.push_back(s);
        }
    };
    std::vector<std::vector<int>> arrOf(D->unitsF.size());
    for (int s = 0; s < int(D->unitsF.size()); s++) {
        const fast::Unit u = D->unitsF[s];
        const BlockDesc &B = D->blocks[u.block];
        const int ti = (u.y0 - 1) / TY;
        const int yTop = std::min(u.y0 + TY - 1, B.ny);
        if (u.x0 > 1 || B.bnd[0] == CONNECT_WITHIN_RANK) {
            std::vector<int> c{s};
            if (u.x0 > 1) {
                covering(u.block, ti, u.x0 - 1, u.x0, c);
            } else {
                const int nb = B.nbr[0];
                if (D->blocks[nb].ny != B.ny) return false;
                covering(nb, ti, D->blocks[nb].nx, D->blocks[nb].nx + 1, c);
            }
            const int id = int(D->pieces.size());
            D->pieces.push_back(fast::Piece{u.block, 0, u.x0, u.y0, yTop - u.y0 + 1, int(c.size())});
            for (int x : c) arrOf[x].push_back(id);
        }
        if (u.y0 > 1 || B.bnd[2] == CONNECT_WITHIN_RANK) {
            std::vector<int> c{s};
            if (u.y0 > 1) {
                covering(u.block, ti - 1, u.x0, u.x1, c);
            } else {
                const int nb = B.nbr[2];
                if (D->blocks[nb].nx != B.nx) return false;
                covering(nb, tilesOf(nb) - 1, u.x0, u.x1, c);
            }
            const int id = int(D->pieces.size());
            D->pieces.push_back(fast::Piece{u.block, 1, u.x0, u.y0, u.x1 - u.x0, int(c.size())});
            for (int x : c) arrOf[x].push_back(id);
        }
    }
    for (int s = 0; s < int(D->unitsF.size()); s++) {
        if (int(arrOf[s].size()) > std::min(fast::kMaxArrivals, TY / fast::fastRows())) return false;
        D->unitsF[s].arrBegin = int(D->arrF.size());
        D->arrF.insert(D->arrF.end(), arrOf[s].begin(), arrOf[s].end());
        D->unitsF[s].arrEnd = int(D->arrF.size());
    }
    return true;
}

/// device copies of the fast step's plan (replacing earlier ones)
int uploadFastPlan(swe_gpu_domain *D) {
    cudaFree(D->dUnitsF);
    cudaFree(D->dCtaSegF);
    cudaFree(D->dPieces);
    cudaFree(D->dPieceCnt);
    cudaFree(D->dArrF);
    D->dUnitsF = nullptr;
    D->dCtaSegF = nullptr;
    D->dPieces = nullptr;
    D->dPieceCnt = nullptr;
    D->dArrF = nullptr;
    const size_t np = std::max<size_t>(1, D->pieces.size()), na = std::max<size_t>(1, D->arrF.size());
    CUDA_TRY(cudaMalloc(&D->dUnitsF, sizeof(fast::Unit) * D->unitsF.size()));
    CUDA_TRY(cudaMalloc(&D->dCtaSegF, sizeof(int) * D->ctaSegF.size()));
    CUDA_TRY(cudaMalloc(&D->dPieces, sizeof(fast::Piece) * np));
    CUDA_TRY(cudaMalloc(&D->dPieceCnt, sizeof(unsigned) * np));
    CUDA_TRY(cudaMalloc(&D->dArrF, sizeof(int) * na));
    CUDA_TRY(cudaMemcpy(D->dUnitsF, D->unitsF.data(), sizeof(fast::Unit) * D->unitsF.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(D->dCtaSegF, D->ctaSegF.data(), sizeof(int) * D->ctaSegF.size(), cudaMemcpyHostToDevice));
    if (!D->pieces.empty())
        CUDA_TRY(cudaMemcpy(D->dPieces, D->pieces.data(), sizeof(fast::Piece) * D->pieces.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(D->dPieceCnt, 0, sizeof(unsigned) * np));
    if (!D->arrF.empty()) CUDA_TRY(cudaMemcpy(D->dArrF, D->arrF.data(), sizeof(int) * D->arrF.size(), cudaMemcpyHostToDevice));
    return SWE_GPU_OK;
}

/// per-group work counts of the passes
void groupCounts(swe_gpu_domain *D, std::vector<GroupState> &g) {
    for (GroupState &x : g) {
        x.units = 0;
        x.unitsUpd = 0;
        x.tiles = 0;
    }
    for (const WorkUnit &u : D->units) g[D->blocks[u.block].group].units++;
    for (const WorkUnit &u : D->unitsU) g[D->blocks[u.block].group].unitsUpd++;
    for (GroupState &x : g) x.unitsFast = 0;
    for (const fast::Unit &u : D->unitsF) g[D->blocks[u.block].group].unitsFast++;
    for (const TileInfo &t : D->tiles) g[t.group].tiles++;
}

int buildDomain(const std::vector<BlockSpec> &spec, const DomainOptions &o, swe_gpu_domain **out) {
    auto *D = new swe_gpu_domain();
    D->device = o.device;
    D->lts = o.ltsMaxTimestep > 0.f;
    D->solver = o.solver;
    D->semantics = o.semantics;
    D->splitDtMode = o.splitDtMode;
    D->tileColsArg = o.tileCols;
    int maxNy = 0;
    for (const BlockSpec &b : spec) maxNy = std::max(maxNy, b.ny);
    D->tileRows = std::min(o.tileRows > 0 ? o.tileRows : 256, ((maxNy + 31) / 32) * 32);
    D->tileCols = o.tileCols > 0 ? o.tileCols : 32;
    const int tileColsArg = o.tileCols;

    cudaError_t e = cudaSetDevice(D->device);
    if (e != cudaSuccess) {
        delete D;
        return fail(SWE_GPU_ERR_CUDA, "cudaSetDevice(%d): %s", o.device, cudaGetErrorString(e));
    }
    e = cudaStreamCreateWithFlags(&D->ownStream, cudaStreamNonBlocking);
    D->stream = D->ownStream;
    if (e != cudaSuccess) {
        delete D;
        return fail(SWE_GPU_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }

    // block descriptors and field layout
    size_t elems = 0;
    for (const BlockSpec &bs : spec) {
        BlockDesc B{};
        B.nx = bs.nx;
        B.ny = bs.ny;
        B.pitch = ((B.ny + 2 + kColPad) + 31) / 32 * 32;
        B.group = bs.group;
        B.base = (long long)elems + kColPad;
        B.ring = D->ringElems;
        D->ringElems += 2LL * (B.nx + B.ny);
        B.dx = bs.dx;
        B.dy = bs.dy;
        for (int s = 0; s < 4; s++) {
            B.nbr[s] = bs.nbr[s];
            B.bnd[s] = bs.bnd[s];
        }
        elems += size_t(B.nx + 2) * size_t(B.pitch);
        B.stage = D->stageElems;
        D->stageElems += (long long)(B.nx + 2) * (long long)(B.ny + 2);
        D->maxCols = std::max(D->maxCols, B.nx + 2);
        D->maxPerimeter = std::max(D->maxPerimeter, 2 * B.nx + 2 * B.ny + 4);
        D->blocks.push_back(B);
    }
    elems += 32;  // slack so the last column's padding (and the fast step's strip copies) stays inside the allocation
    D->fieldElems = elems;
    buildPartitions(D, tileColsArg);
    D->fast = o.arithmetic == SWE_ARITH_FAST;
    if (D->fast && !buildFastPlan(D)) {
        if (D->ownStream) cudaStreamDestroy(D->ownStream);
        delete D;
        return fail(SWE_GPU_ERR_INVALID, "fast arithmetic: neighbouring blocks must share the length of their common side");
    }
    // Bounded speed pass: bound tiles of 32 x 32 cells per block, numbered
    // block by block, column of tiles by column of tiles
    bool smallBlocks = true;
    for (const BlockDesc &B : D->blocks) smallBlocks = smallBlocks && B.nx < 65535 && B.ny < 65535;
    // (not under local time stepping: with one dt group per block every block's
    // own maximum needs exact edges, so many tiles are candidates and the full
    // pass, one streaming read of every edge, is faster)
    D->bounded = D->semantics == SEM_UNSPLIT &&
                 (D->solver == SOLVER_FWAVE || D->solver == SOLVER_HLLE) && o.speedPass == 0 && smallBlocks &&
                 !D->lts && !D->fast;
    if (D->bounded) {
        int base = 0;
        for (BlockDesc &B : D->blocks) {
            B.tileBase = base;
            B.tilesY = (B.ny + kBoundTile - 1) / kBoundTile;
            base += B.tilesY * ((B.nx + kBoundTile - 1) / kBoundTile);
        }
        auto tileId = [&](int k, int i, int j) { return D->blocks[k].tileBase + i * D->blocks[k].tilesY + j; };
        auto tilesX = [&](int k) { return (D->blocks[k].nx + kBoundTile - 1) / kBoundTile; };
        auto ghostSide = [&](const BlockDesc &B, int side, int nbTile) {
            const int type = B.bnd[side];
            // local time stepping time-interpolates these ghosts: no bound
            if (type == CONNECT_WITHIN_RANK) return D->lts ? kNbrUnbounded : nbTile;
            return (type == OUTFLOW || type == WALL) ? kNbrSelf : kNbrUnbounded;
        };
        for (int k = 0; k < int(D->blocks.size()); k++) {
            const BlockDesc &B = D->blocks[k];
            for (int i = 0; i < tilesX(k); i++)
                for (int j = 0; j < B.tilesY; j++) {
                    TileInfo T{};
                    T.base = B.base;
                    T.pitch = B.pitch;
                    T.group = B.group;
                    T.x0 = 1 + i * kBoundTile;
                    T.x1 = std::min(T.x0 + kBoundTile, B.nx + 1);
                    T.y0 = 1 + j * kBoundTile;
                    T.y1 = std::min(T.y0 + kBoundTile, B.ny + 1);
                    T.nx = B.nx;
                    T.ny = B.ny;
                    const int nL = B.nbr[0], nR = B.nbr[1], nB = B.nbr[2], nT = B.nbr[3];
                    T.nbr[0] = i > 0 ? tileId(k, i - 1, j) : ghostSide(B, 0, nL >= 0 ? tileId(nL, tilesX(nL) - 1, j) : 0);
                    T.nbr[1] = j > 0 ? tileId(k, i, j - 1)
                                     : ghostSide(B, 2, nB >= 0 ? tileId(nB, i, D->blocks[nB].tilesY - 1) : 0);
                    T.nbr[2] = T.x1 <= B.nx ? kNbrSelf : ghostSide(B, 1, nR >= 0 ? tileId(nR, 0, j) : 0);
                    T.nbr[3] = T.y1 <= B.ny ? kNbrSelf : ghostSide(B, 3, nT >= 0 ? tileId(nT, i, 0) : 0);
                    D->tiles.push_back(T);
                }
        }
        if (D->tiles.size() >= (size_t(1) << 19)) {  // edge codes hold 19 bits of tile id
            D->bounded = false;
            D->tiles.clear();
        }
        int sms = 148;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, D->device);
        const long long want = ((long long)D->tiles.size() + 7) / 8;
        D->gridB = int(std::max(1LL, std::min(want, (long long)sms * std::max(1, occupancyBound(D->solver)))));
    }
    // dt groups
    D->ngroups = o.ngroups;
    {
        GroupState g0{};
        g0.target = INFINITY;
        g0.enabled = D->lts ? 0 : 1;
        D->groupsInit.assign(D->ngroups, g0);
        for (int k = int(D->blocks.size()) - 1; k >= 0; k--) D->groupsInit[D->blocks[k].group].firstBlock = k;
        groupCounts(D, D->groupsInit);
    }

    bool ok = true;
    const size_t bytes = elems * sizeof(float);
    for (int i = 0; i < 2 && ok; i++)
        ok = cudaMalloc(&D->h[i], bytes) == cudaSuccess && cudaMalloc(&D->hu[i], bytes) == cudaSuccess &&
             cudaMalloc(&D->hv[i], bytes) == cudaSuccess;
    ok = ok && cudaMalloc(&D->b, bytes) == cudaSuccess;
    ok = ok && cudaMalloc(&D->stage, sizeof(float) * 4 * size_t(D->stageElems)) == cudaSuccess;
    ok = ok && cudaMalloc(&D->dBlocks, sizeof(BlockDesc) * D->blocks.size()) == cudaSuccess;
    ok = ok && cudaMalloc(&D->dUnits, sizeof(WorkUnit) * D->units.size()) == cudaSuccess;
    ok = ok && cudaMalloc(&D->dCtaSeg, sizeof(int) * D->ctaSeg.size()) == cudaSuccess;
    ok = ok && cudaMalloc(&D->dUnitsU, sizeof(WorkUnit) * D->unitsU.size()) == cudaSuccess;
    ok = ok && cudaMalloc(&D->dCtaSegU, sizeof(int) * D->ctaSegU.size()) == cudaSuccess;
    ok = ok && cudaMalloc(&D->dGroups, sizeof(GroupState) * D->ngroups) == cudaSuccess;
    if (D->lts) {
        ok = ok && cudaMalloc(&D->dLts, sizeof(LtsBlock) * D->blocks.size()) == cudaSuccess;
        ok = ok && cudaMalloc(&D->dLtsCtl, sizeof(LtsControl)) == cudaSuccess;
        ok = ok && cudaMalloc(&D->dLtsWork, sizeof(int) * ltsWorkInts(int(D->blocks.size()))) == cudaSuccess;
        ok = ok && cudaMalloc(&D->dLtsLocal, sizeof(float) * D->blocks.size()) == cudaSuccess;
        for (int f = 0; f < 3 && ok; f++)
            ok = cudaMalloc(&D->dRing[f], sizeof(float) * std::max(1LL, D->ringElems)) == cudaSuccess;
    }
    D->edgeBuffered = D->solver == SOLVER_AUGRIE && D->semantics == SEM_UNSPLIT && !D->lts &&
                      o.speedPass == 0;
    if (D->edgeBuffered) {
        D->edgeTiles = mlp::buildEdgeTiles(D->blocks);
        ok = ok && cudaMalloc(&D->edgeBuf, 8 * bytes) == cudaSuccess;
        ok = ok && cudaMalloc(&D->dUsed, sizeof(unsigned long long)) == cudaSuccess;
        ok = ok && cudaMalloc(&D->dEdgeTiles, sizeof(mlp::EdgeTile) * std::max<size_t>(1, D->edgeTiles.size())) == cudaSuccess;
    }
    if (D->bounded) {
        ok = ok && cudaMalloc(&D->dTiles, sizeof(TileInfo) * D->tiles.size()) == cudaSuccess;
        ok = ok && cudaMalloc(&D->dTileW, sizeof(unsigned int) * 2 * D->tiles.size()) == cudaSuccess;
        ok = ok && cudaMalloc(&D->dTileKey, sizeof(unsigned long long) * 2 * D->tiles.size()) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        freeDomain(D);
        return fail(SWE_GPU_ERR_NOMEM, "device allocation of %.1f MB failed", 7.0 * bytes / 1e6);
    }
    for (int i = 0; i < 2; i++) {
        cudaMemsetAsync(D->h[i], 0, bytes, D->stream);
        cudaMemsetAsync(D->hu[i], 0, bytes, D->stream);
        cudaMemsetAsync(D->hv[i], 0, bytes, D->stream);
    }
    cudaMemsetAsync(D->b, 0, bytes, D->stream);
    cudaMemcpyAsync(D->dBlocks, D->blocks.data(), sizeof(BlockDesc) * D->blocks.size(), cudaMemcpyHostToDevice, D->stream);
    if (D->edgeBuffered && !D->edgeTiles.empty())
        cudaMemcpyAsync(D->dEdgeTiles, D->edgeTiles.data(), sizeof(mlp::EdgeTile) * D->edgeTiles.size(),
                        cudaMemcpyHostToDevice, D->stream);
    cudaMemcpyAsync(D->dUnits, D->units.data(), sizeof(WorkUnit) * D->units.size(), cudaMemcpyHostToDevice, D->stream);
    cudaMemcpyAsync(D->dCtaSeg, D->ctaSeg.data(), sizeof(int) * D->ctaSeg.size(), cudaMemcpyHostToDevice, D->stream);
    cudaMemcpyAsync(D->dUnitsU, D->unitsU.data(), sizeof(WorkUnit) * D->unitsU.size(), cudaMemcpyHostToDevice, D->stream);
    cudaMemcpyAsync(D->dCtaSegU, D->ctaSegU.data(), sizeof(int) * D->ctaSegU.size(), cudaMemcpyHostToDevice, D->stream);
    cudaMemcpyAsync(D->dGroups, D->groupsInit.data(), sizeof(GroupState) * D->ngroups, cudaMemcpyHostToDevice, D->stream);
    std::vector<LtsBlock> ltsInit;
    LtsControl ctlInit{};
    if (D->lts) {
        LtsBlock l0{};
        for (int s4 = 0; s4 < 4; s4++) l0.received[s4] = GL_NEXT;
        ltsInit.assign(D->blocks.size(), l0);
        ctlInit.t = 0.f;
        ctlInit.target = 0.f;  // nothing runs before swe_gpu_lts_advance
        ctlInit.maxTimestepLocal = o.ltsMaxTimestep;
        ctlInit.duration = o.duration;
        ctlInit.maxDivisor = 1024;  // src/blocks/SWE_Block.hh:221
        cudaMemcpyAsync(D->dLts, ltsInit.data(), sizeof(LtsBlock) * ltsInit.size(), cudaMemcpyHostToDevice, D->stream);
        cudaMemcpyAsync(D->dLtsCtl, &ctlInit, sizeof(LtsControl), cudaMemcpyHostToDevice, D->stream);
        for (int f = 0; f < 3; f++)
            cudaMemsetAsync(D->dRing[f], 0, sizeof(float) * std::max(1LL, D->ringElems), D->stream);
        // empty work lists, every block at local time 0
        cudaMemsetAsync(D->dLtsWork, 0, sizeof(int) * ltsWorkInts(int(D->blocks.size())), D->stream);
        cudaMemsetAsync(D->dLtsLocal, 0, sizeof(float) * D->blocks.size(), D->stream);
    }
    if (D->bounded) {
        cudaMemcpyAsync(D->dTiles, D->tiles.data(), sizeof(TileInfo) * D->tiles.size(), cudaMemcpyHostToDevice,
                        D->stream);
        cudaMemsetAsync(D->dTileW, 0, sizeof(unsigned int) * 2 * D->tiles.size(), D->stream);
        cudaMemsetAsync(D->dTileKey, 0, sizeof(unsigned long long) * 2 * D->tiles.size(), D->stream);
    }
    e = cudaStreamSynchronize(D->stream);
    if (e != cudaSuccess) {
        freeDomain(D);
        return fail(SWE_GPU_ERR_CUDA, "domain initialisation: %s", cudaGetErrorString(e));
    }
    if (D->fast) {
        const int rcF = uploadFastPlan(D);
        if (rcF) {
            freeDomain(D);
            return rcF;
        }
    }
    for (int i = 0; i < 2; i++) {
        D->dev.h[i] = D->h[i];
        D->dev.hu[i] = D->hu[i];
        D->dev.hv[i] = D->hv[i];
    }
    D->dev.b = D->b;
    D->dev.blocks = D->dBlocks;
    D->dev.units = D->dUnits;
    D->dev.ctaSeg = D->dCtaSeg;
    D->dev.groups = D->dGroups;
    D->dev.nblocks = int(D->blocks.size());
    D->dev.solver = D->solver;
    D->dev.semantics = D->semantics;
    D->dev.splitDtMode = D->splitDtMode;
    D->dev.tileRows = D->tileRows;
    D->dev.lts = D->dLts;
    D->dev.ltsCtl = D->dLtsCtl;
    D->dev.ltsWork = D->dLtsWork;
    D->dev.ltsLocal = D->dLtsLocal;
    {
        long long maxCells = 0;
        for (const BlockDesc &B : D->blocks) maxCells = std::max(maxCells, (long long)B.nx * B.ny);
        D->dev.ltsCheckSpeed = D->lts && (D->solver == SOLVER_FWAVE || D->solver == SOLVER_HLLE) &&
                               maxCells <= kLtsCheckSpeedCells;
    }
    for (int f = 0; f < 3; f++) D->dev.ring[f] = D->dRing[f];
    D->dev.tileW = D->dTileW;
    D->dev.tileKey = D->dTileKey;
    D->dev.tileInfo = D->dTiles;
    D->dev.ntiles = int(D->tiles.size());
    {  // a multiplier coprime to the tile count spreads neighbouring tiles over CTAs
        const unsigned long long n = std::max<unsigned long long>(1, D->tiles.size());
        unsigned long long m = 2654435761ull % n;
        auto gcd = [](unsigned long long a, unsigned long long b) {
            while (b) { const unsigned long long t = a % b; a = b; b = t; }
            return a;
        };
        while (m == 0 || gcd(m, n) != 1) m++;
        D->dev.tileHashMul = n == 1 ? 1 : m;
    }
    *out = D;
    return SWE_GPU_OK;
}

int checkCommon(int solver, int semantics, const int boundary[4]) {
    if (solver < SWE_SOLVER_FWAVE || solver > SWE_SOLVER_HLLE) return fail(SWE_GPU_ERR_INVALID, "unknown solver %d", solver);
    if (semantics != SWE_SEMANTICS_UNSPLIT && semantics != SWE_SEMANTICS_SPLIT)
        return fail(SWE_GPU_ERR_INVALID, "unknown semantics %d", semantics);
    for (int i = 0; i < 4; i++)
        if (boundary[i] < SWE_OUTFLOW || boundary[i] > SWE_PASSIVE)
            return fail(SWE_GPU_ERR_INVALID, "unknown boundary type %d", boundary[i]);
    return SWE_GPU_OK;
}

int checkArithmetic(int arithmetic, int solver, int semantics, bool lts) {
    if (arithmetic == SWE_ARITH_EXACT) return SWE_GPU_OK;
    if (arithmetic != SWE_ARITH_FAST) return fail(SWE_GPU_ERR_INVALID, "unknown arithmetic %d", arithmetic);
    if (solver != SWE_SOLVER_FWAVE && solver != SWE_SOLVER_HLLE)
        return fail(SWE_GPU_ERR_INVALID, "fast arithmetic is offered for the f-wave and HLLE solvers");
    if (semantics != SWE_SEMANTICS_UNSPLIT)
        return fail(SWE_GPU_ERR_INVALID, "fast arithmetic is offered for the unsplit step");
    if (lts) return fail(SWE_GPU_ERR_INVALID, "fast arithmetic is offered with global time stepping");
    return SWE_GPU_OK;
}

int checkVariant(int kernelVariant) {
    if (kernelVariant != 0)
        return fail(SWE_GPU_ERR_INVALID, "kernel_variant %d: the sweep kernels have one thread mapping (0, CTA tiles)",
                    kernelVariant);
    return SWE_GPU_OK;
}

int checkTiles(int tileRows, int tileCols) {
    const int tr = tileRows > 0 ? tileRows : 256;
    if (tr % 32 != 0 || tr > kMaxTileRows) return fail(SWE_GPU_ERR_INVALID, "tile_rows must be a multiple of 32 <= %d", kMaxTileRows);
    if (tileCols > kMaxTileCols) return fail(SWE_GPU_ERR_INVALID, "tile_cols must be <= %d", kMaxTileCols);
    return SWE_GPU_OK;
}

} // namespace

int swe_gpu_domain_create(const swe_gpu_desc *desc, swe_gpu_domain **out) {
    if (!desc || !out) return fail(SWE_GPU_ERR_INVALID, "null descriptor or output pointer");
    *out = nullptr;
    const int bx = desc->blocks_x, by = desc->blocks_y;
    if (bx < 1 || by < 1 || !desc->nx_cols || !desc->ny_rows)
        return fail(SWE_GPU_ERR_INVALID, "need at least one block and the block sizes");
    if (!(desc->dx > 0.f) || !(desc->dy > 0.f)) return fail(SWE_GPU_ERR_INVALID, "dx, dy must be positive");
    int rc = checkCommon(desc->solver, desc->semantics, desc->boundary);
    if (rc) return rc;
    if (desc->semantics == SWE_SEMANTICS_SPLIT && bx * by != 1)
        return fail(SWE_GPU_ERR_INVALID, "the split step is defined for a single block");
    if (desc->lts_max_timestep > 0.f && desc->semantics != SWE_SEMANTICS_UNSPLIT)
        return fail(SWE_GPU_ERR_INVALID, "local time stepping is defined for the unsplit step");
    for (int i = 0; i < bx; i++)
        if (desc->nx_cols[i] < 1) return fail(SWE_GPU_ERR_INVALID, "block width must be >= 1");
    for (int i = 0; i < by; i++)
        if (desc->ny_rows[i] < 1) return fail(SWE_GPU_ERR_INVALID, "block height must be >= 1");
    rc = checkTiles(desc->tile_rows, desc->tile_cols);
    if (rc) return rc;
    const bool lts = desc->lts_max_timestep > 0.f;
    rc = checkArithmetic(desc->arithmetic, desc->solver, desc->semantics, lts);
    if (rc) return rc;
    rc = checkVariant(desc->kernel_variant);
    if (rc) return rc;
    std::vector<BlockSpec> spec;
    for (int k = 0; k < bx * by; k++) {
        const int px = k / by, py = k % by;
        BlockSpec b{};
        b.nx = desc->nx_cols[px];
        b.ny = desc->ny_rows[py];
        b.dx = desc->dx;
        b.dy = desc->dy;
        const int nb[4] = {px > 0 ? k - by : -1, px < bx - 1 ? k + by : -1, py > 0 ? k - 1 : -1,
                           py < by - 1 ? k + 1 : -1};
        for (int s = 0; s < 4; s++) {
            b.nbr[s] = nb[s];
            b.bnd[s] = nb[s] >= 0 ? CONNECT_WITHIN_RANK : desc->boundary[s];
        }
        b.group = lts ? k : 0;  // local time stepping: every block its own dt group
        spec.push_back(b);
    }
    DomainOptions o{};
    o.device = desc->device;
    o.solver = desc->solver;
    o.semantics = desc->semantics;
    o.splitDtMode = desc->split_dt_mode;
    o.tileRows = desc->tile_rows;
    o.tileCols = desc->tile_cols;
    o.speedPass = desc->speed_pass;
    o.ltsMaxTimestep = desc->lts_max_timestep;
    o.duration = desc->duration;
    o.arithmetic = desc->arithmetic;
    o.ngroups = lts ? bx * by : 1;
    return buildDomain(spec, o, out);
}

int swe_gpu_ensemble_create(const swe_gpu_instance *inst, int count, const swe_gpu_desc *options,
                            swe_gpu_domain **out) {
    if (!inst || count < 1 || !options || !out) return fail(SWE_GPU_ERR_INVALID, "need instances, options and output");
    *out = nullptr;
    if (options->lts_max_timestep > 0.f)
        return fail(SWE_GPU_ERR_INVALID, "ensembles step globally per instance (no local time stepping)");
    int rc = checkTiles(options->tile_rows, options->tile_cols);
    if (rc) return rc;
    rc = checkArithmetic(options->arithmetic, options->solver, options->semantics, false);
    if (rc) return rc;
    rc = checkVariant(options->kernel_variant);
    if (rc) return rc;
    std::vector<BlockSpec> spec;
    for (int i = 0; i < count; i++) {
        rc = checkCommon(options->solver, options->semantics, inst[i].boundary);
        if (rc) return rc;
        if (inst[i].nx < 1 || inst[i].ny < 1 || !(inst[i].dx > 0.f) || !(inst[i].dy > 0.f))
            return fail(SWE_GPU_ERR_INVALID, "instance %d: sizes must be positive", i);
        for (int s = 0; s < 4; s++)
            if (inst[i].boundary[s] == SWE_CONNECT_WITHIN_RANK)
                return fail(SWE_GPU_ERR_INVALID, "instance %d: an instance is one block without neighbours", i);
        BlockSpec b{};
        b.nx = inst[i].nx;
        b.ny = inst[i].ny;
        b.dx = inst[i].dx;
        b.dy = inst[i].dy;
        for (int s = 0; s < 4; s++) {
            b.bnd[s] = inst[i].boundary[s];
            b.nbr[s] = -1;
        }
        b.group = i;
        spec.push_back(b);
    }
    DomainOptions o{};
    o.device = options->device;
    o.solver = options->solver;
    o.semantics = options->semantics;
    o.splitDtMode = options->split_dt_mode;
    o.tileRows = options->tile_rows;
    o.tileCols = options->tile_cols;
    o.speedPass = options->speed_pass;
    o.arithmetic = options->arithmetic;
    o.ngroups = count;
    return buildDomain(spec, o, out);
}

int swe_gpu_domain_destroy(swe_gpu_domain *dom) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    cudaSetDevice(dom->device);
    cudaStreamSynchronize(dom->stream);
    freeDomain(dom);
    return SWE_GPU_OK;
}

int swe_gpu_block_count(const swe_gpu_domain *dom, int *count) {
    if (!dom || !count) return fail(SWE_GPU_ERR_INVALID, "null argument");
    *count = int(dom->blocks.size());
    return SWE_GPU_OK;
}

int swe_gpu_block_shape(const swe_gpu_domain *dom, int block, int *nx, int *ny) {
    int rc = checkBlock(dom, block);
    if (rc) return rc;
    if (nx) *nx = dom->blocks[block].nx;
    if (ny) *ny = dom->blocks[block].ny;
    return SWE_GPU_OK;
}

// Host <-> device transfers go through the staging buffer: large contiguous
// copies at full link bandwidth, then a repack kernel that reads the current
// buffer index on the device (so transfers need no host synchronisation
// with queued steps).
static int stageTransfer(swe_gpu_domain *D, int firstBlock, int nblocks, float *const host[4], int ld, bool up,
                         bool wait) {
    CUDA_TRY(cudaSetDevice(D->device));
    int mask = 0;
    for (int f = 0; f < 4; f++)
        if (host[f]) mask |= 1 << f;
    if (!mask) return SWE_GPU_OK;
    const BlockDesc &F = D->blocks[firstBlock];
    const BlockDesc &L = D->blocks[firstBlock + nblocks - 1];
    const long long n0 = F.stage;
    const long long n = L.stage + (long long)(L.nx + 2) * (L.ny + 2) - n0;
    const bool contiguous = (nblocks > 1) || ld == F.ny + 2;
    const dim3 grid(unsigned(D->maxCols), unsigned(nblocks));
    if (!up) {
        repackKernel<<<grid, 256, 0, D->stream>>>(D->dev, D->stage, D->stageElems, 0, mask, firstBlock);
        CUDA_TRY(cudaGetLastError());
        D->launches++;
    }
    for (int f = 0; f < 4; f++) {
        if (!host[f]) continue;
        float *st = D->stage + size_t(f) * size_t(D->stageElems) + size_t(n0);
        if (contiguous) {
            if (up)
                CUDA_TRY(cudaMemcpyAsync(st, host[f], size_t(n) * 4, cudaMemcpyHostToDevice, D->stream));
            else
                CUDA_TRY(cudaMemcpyAsync(host[f], st, size_t(n) * 4, cudaMemcpyDeviceToHost, D->stream));
        } else {
            const size_t w = size_t(F.ny + 2) * 4;
            if (up)
                CUDA_TRY(cudaMemcpy2DAsync(st, w, host[f], size_t(ld) * 4, w, size_t(F.nx + 2), cudaMemcpyHostToDevice, D->stream));
            else
                CUDA_TRY(cudaMemcpy2DAsync(host[f], size_t(ld) * 4, st, w, w, size_t(F.nx + 2), cudaMemcpyDeviceToHost, D->stream));
        }
    }
    if (up) {
        repackKernel<<<grid, 256, 0, D->stream>>>(D->dev, D->stage, D->stageElems, 1, mask, firstBlock);
        CUDA_TRY(cudaGetLastError());
        D->launches++;
        D->ghostsValid = false;
        D->dtValid = false;
    }
    if (wait) CUDA_TRY(cudaStreamSynchronize(D->stream));
    return SWE_GPU_OK;
}

int swe_gpu_upload_block(swe_gpu_domain *dom, int block, const float *h, const float *hu, const float *hv,
                         const float *b, int ld) {
    int rc = checkBlock(dom, block);
    if (rc) return rc;
    if (ld < dom->blocks[block].ny + 2) return fail(SWE_GPU_ERR_INVALID, "ld %d < ny+2", ld);
    float *const host[4] = {const_cast<float *>(h), const_cast<float *>(hu), const_cast<float *>(hv),
                            const_cast<float *>(b)};
    // the staging buffer is reused by the next transfer: wait for the copy
    return stageTransfer(dom, block, 1, host, ld, true, true);
}

int swe_gpu_download_block(swe_gpu_domain *dom, int block, float *h, float *hu, float *hv, float *b, int ld) {
    int rc = checkBlock(dom, block);
    if (rc) return rc;
    if (ld < dom->blocks[block].ny + 2) return fail(SWE_GPU_ERR_INVALID, "ld %d < ny+2", ld);
    float *const host[4] = {h, hu, hv, b};
    return stageTransfer(dom, block, 1, host, ld, false, true);
}

int swe_gpu_upload_domain(swe_gpu_domain *dom, const float *h, const float *hu, const float *hv, const float *b) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    float *const host[4] = {const_cast<float *>(h), const_cast<float *>(hu), const_cast<float *>(hv),
                            const_cast<float *>(b)};
    return stageTransfer(dom, 0, int(dom->blocks.size()), host, dom->blocks[0].ny + 2, true, true);
}

int swe_gpu_download_domain(swe_gpu_domain *dom, float *h, float *hu, float *hv, float *b) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    float *const host[4] = {h, hu, hv, b};
    return stageTransfer(dom, 0, int(dom->blocks.size()), host, dom->blocks[0].ny + 2, false, true);
}

int swe_gpu_upload_domain_async(swe_gpu_domain *dom, const float *h, const float *hu, const float *hv,
                                const float *b) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    const float *host[4] = {h, hu, hv, b};
    int mask = 0;
    for (int f = 0; f < 4; f++)
        if (host[f]) mask |= 1 << f;
    if (!mask) return SWE_GPU_OK;
    if (!dom->upStream) {
        CUDA_TRY(cudaStreamCreateWithFlags(&dom->upStream, cudaStreamNonBlocking));
        for (int j = 0; j < 2; j++) {
            CUDA_TRY(cudaMalloc(&dom->stageUp[j], sizeof(float) * 4 * size_t(dom->stageElems)));
            CUDA_TRY(cudaEventCreateWithFlags(&dom->upReady[j], cudaEventDisableTiming));
            CUDA_TRY(cudaEventCreateWithFlags(&dom->upConsumed[j], cudaEventDisableTiming));
        }
    }
    const int j = dom->upSlot;
    dom->upSlot ^= 1;
    // slot j is free once the repack of its previous use has read it
    if (dom->upUsed[j]) CUDA_TRY(cudaStreamWaitEvent(dom->upStream, dom->upConsumed[j], 0));
    const size_t n = size_t(dom->stageElems);
    for (int f = 0; f < 4; f++)
        if (host[f])
            CUDA_TRY(cudaMemcpyAsync(dom->stageUp[j] + size_t(f) * n, host[f], n * sizeof(float), cudaMemcpyHostToDevice,
                                     dom->upStream));
    CUDA_TRY(cudaEventRecord(dom->upReady[j], dom->upStream));
    CUDA_TRY(cudaStreamWaitEvent(dom->stream, dom->upReady[j], 0));
    const dim3 grid(unsigned(dom->maxCols), unsigned(dom->blocks.size()));
    repackKernel<<<grid, 256, 0, dom->stream>>>(dom->dev, dom->stageUp[j], dom->stageElems, 1, mask, 0);
    CUDA_TRY(cudaGetLastError());
    dom->launches++;
    CUDA_TRY(cudaEventRecord(dom->upConsumed[j], dom->stream));
    dom->upUsed[j] = true;
    dom->ghostsValid = false;
    dom->dtValid = false;
    return SWE_GPU_OK;
}

int swe_gpu_download_domain_async(swe_gpu_domain *dom, float *h, float *hu, float *hv, float *b) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    float *const host[4] = {h, hu, hv, b};
    int mask = 0;
    for (int f = 0; f < 4; f++)
        if (host[f]) mask |= 1 << f;
    if (!mask) return SWE_GPU_OK;
    if (!dom->copyStream) {
        CUDA_TRY(cudaStreamCreateWithFlags(&dom->copyStream, cudaStreamNonBlocking));
        for (int j = 0; j < 2; j++) {
            CUDA_TRY(cudaMalloc(&dom->stageDown[j], sizeof(float) * 4 * size_t(dom->stageElems)));
            CUDA_TRY(cudaEventCreateWithFlags(&dom->downReady[j], cudaEventDisableTiming));
            CUDA_TRY(cudaEventCreateWithFlags(&dom->downDone[j], cudaEventDisableTiming));
        }
    }
    const int j = dom->downSlot;
    dom->downSlot ^= 1;
    // slot j is free once the copies out of its previous use have finished
    if (dom->downUsed[j]) CUDA_TRY(cudaStreamWaitEvent(dom->stream, dom->downDone[j], 0));
    const dim3 grid(unsigned(dom->maxCols), unsigned(dom->blocks.size()));
    repackKernel<<<grid, 256, 0, dom->stream>>>(dom->dev, dom->stageDown[j], dom->stageElems, 0, mask, 0);
    CUDA_TRY(cudaGetLastError());
    dom->launches++;
    CUDA_TRY(cudaEventRecord(dom->downReady[j], dom->stream));
    CUDA_TRY(cudaStreamWaitEvent(dom->copyStream, dom->downReady[j], 0));
    const size_t n = size_t(dom->stageElems);
    for (int f = 0; f < 4; f++)
        if (host[f])
            CUDA_TRY(cudaMemcpyAsync(host[f], dom->stageDown[j] + size_t(f) * n, n * sizeof(float),
                                     cudaMemcpyDeviceToHost, dom->copyStream));
    CUDA_TRY(cudaEventRecord(dom->downDone[j], dom->copyStream));
    dom->downUsed[j] = true;
    return SWE_GPU_OK;
}

int swe_gpu_snapshot_slabs_async(swe_gpu_domain *dom, int block, void *h, void *hu, void *hv) {
    int rc = checkBlock(dom, block);
    if (rc) return rc;
    if (!h || !hu || !hv) return fail(SWE_GPU_ERR_INVALID, "null snapshot buffer");
    CUDA_TRY(cudaSetDevice(dom->device));
    const BlockDesc &B = dom->blocks[block];
    // the staging area holds 4 fields of the whole domain; 3 interior slabs fit
    uint32_t *out = reinterpret_cast<uint32_t *>(dom->stage);
    const dim3 grid(unsigned((B.nx + 31) / 32), unsigned((B.ny + 31) / 32));
    snapshotKernel<<<grid, dim3(32, 8), 0, dom->stream>>>(dom->dev, block, out);
    CUDA_TRY(cudaGetLastError());
    dom->launches++;
    const size_t slab = size_t(B.nx) * size_t(B.ny) * 4;
    CUDA_TRY(cudaMemcpyAsync(h, out, slab, cudaMemcpyDeviceToHost, dom->stream));
    CUDA_TRY(cudaMemcpyAsync(hu, reinterpret_cast<char *>(out) + slab, slab, cudaMemcpyDeviceToHost, dom->stream));
    CUDA_TRY(cudaMemcpyAsync(hv, reinterpret_cast<char *>(out) + 2 * slab, slab, cudaMemcpyDeviceToHost, dom->stream));
    if (!dom->snapEvent) CUDA_TRY(cudaEventCreateWithFlags(&dom->snapEvent, cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(dom->snapEvent, dom->stream));
    return SWE_GPU_OK;
}

int swe_gpu_snapshot_wait(swe_gpu_domain *dom) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    if (!dom->snapEvent) return SWE_GPU_OK;
    CUDA_TRY(cudaSetDevice(dom->device));
    CUDA_TRY(cudaEventSynchronize(dom->snapEvent));
    return SWE_GPU_OK;
}

int swe_gpu_alloc_pinned(size_t bytes, void **out) {
    if (!out) return fail(SWE_GPU_ERR_INVALID, "null output pointer");
    cudaError_t e = cudaMallocHost(out, bytes);
    if (e != cudaSuccess) return fail(SWE_GPU_ERR_NOMEM, "cudaMallocHost(%zu): %s", bytes, cudaGetErrorString(e));
    return SWE_GPU_OK;
}

int swe_gpu_free_pinned(void *p) {
    CUDA_TRY(cudaFreeHost(p));
    return SWE_GPU_OK;
}

int swe_gpu_exchange_bathymetry(swe_gpu_domain *dom) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    dom->dtValid = false;
    return enqueueGhost(dom, 1);
}

int swe_gpu_set_ghost_layer(swe_gpu_domain *dom) {
    if (dom && dom->lts) return fail(SWE_GPU_ERR_INVALID, "local-time-stepping domain: use swe_gpu_lts_advance");
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    // after an update pass the ring already holds what setGhostLayer computes
    // (the pass pushed it from the new rim cells): only mark it current
    int rc = enqueueGhost(dom, dom->ghostsValid ? 3 : 0);
    if (!rc) dom->ghostsValid = true;
    return rc;
}

int swe_gpu_compute_fluxes(swe_gpu_domain *dom) {
    if (dom && dom->lts) return fail(SWE_GPU_ERR_INVALID, "local-time-stepping domain: use swe_gpu_lts_advance");
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    // fast arithmetic: the previous step already computed this state's
    // maxTimestep; a speed pass runs only when it did not
    if (dom->fast) return enqueueFastPrologue(dom);
    return enqueueSpeed(dom);
}

int swe_gpu_update_unknowns(swe_gpu_domain *dom, float dt) {
    (void)dt;
    if (dom && dom->lts) return fail(SWE_GPU_ERR_INVALID, "local-time-stepping domain: use swe_gpu_lts_advance");
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    if (dom->fast) {
        int rc = enqueueFastPrologue(dom);
        if (rc) return rc;
        return enqueueFast(dom);
    }
    return enqueueUpdate(dom);
}

int swe_gpu_get_max_timestep(swe_gpu_domain *dom, float *dt) {
    if (!dom || !dt) return fail(SWE_GPU_ERR_INVALID, "null argument");
    CUDA_TRY(cudaSetDevice(dom->device));
    std::vector<GroupState> g;
    int rc = readGroups(dom, g);
    if (rc) return rc;
    *dt = g[0].dt;
    return SWE_GPU_OK;
}

int swe_gpu_step(swe_gpu_domain *dom, int nsteps) {
    if (dom && dom->lts) return fail(SWE_GPU_ERR_INVALID, "local-time-stepping domain: use swe_gpu_lts_advance");
    if (!dom || nsteps < 0) return fail(SWE_GPU_ERR_INVALID, "bad argument");
    CUDA_TRY(cudaSetDevice(dom->device));
    for (int i = 0; i < nsteps; i++) {
        int rc = enqueueStep(dom);
        if (rc) return rc;
    }
    return SWE_GPU_OK;
}

int swe_gpu_advance(swe_gpu_domain *dom, float t_end, int max_steps, int *steps_done, float *t_now) {
    if (!dom || max_steps < 0) return fail(SWE_GPU_ERR_INVALID, "bad argument");
    if (dom->lts) return fail(SWE_GPU_ERR_INVALID, "local-time-stepping domain: use swe_gpu_lts_advance");
    CUDA_TRY(cudaSetDevice(dom->device));
    const int batch = 16;
    if (dom->fast) {  // fast step: ghost ring and dt of the current state first, outside the graph
        int rc0 = enqueueFastPrologue(dom);
        if (rc0) return rc0;
    }
    if (!dom->graph) {  // capture `batch` steps once; replays are identical
        cudaGraph_t g;
        CUDA_TRY(cudaStreamBeginCapture(dom->stream, cudaStreamCaptureModeThreadLocal));
        int rc = SWE_GPU_OK;
        const long long before = dom->launches;
        for (int i = 0; i < batch && rc == SWE_GPU_OK; i++) rc = enqueueStep(dom);
        cudaError_t e = cudaStreamEndCapture(dom->stream, &g);
        dom->graphKernels = dom->launches - before;  // captured, not launched
        dom->launches = before;
        if (rc) return rc;
        if (e != cudaSuccess) return fail(SWE_GPU_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&dom->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(SWE_GPU_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
        dom->graphSteps = batch;
    }
    std::vector<GroupState> g;
    int rc = readGroups(dom, g);
    if (rc) return rc;
    std::vector<int> startSteps(g.size());
    for (size_t i = 0; i < g.size(); i++) startSteps[i] = g[i].steps;
    rc = setTargets(dom, t_end);
    if (rc) return rc;
    // steps taken (the most any group took) and whether every group reached t_end
    auto progress = [&](int &steps) {
        steps = 0;
        bool all = true;
        for (size_t i = 0; i < g.size(); i++) {
            steps = std::max(steps, g[i].steps - startSteps[i]);
            all = all && !(g[i].time < t_end);
        }
        return all;
    };
    int done = 0;
    while (done < max_steps) {
        const int remaining = max_steps - done;
        if (remaining >= dom->graphSteps) {
            CUDA_TRY(cudaGraphLaunch(dom->graph, dom->stream));
            dom->launches += dom->graphKernels;
        } else {
            for (int i = 0; i < remaining; i++) {
                rc = enqueueStep(dom);
                if (rc) return rc;
            }
        }
        rc = readGroups(dom, g);
        if (rc) return rc;
        if (progress(done)) break;
    }
    rc = setTargets(dom, INFINITY);
    if (rc) return rc;
    if (steps_done) *steps_done = done;
    float tmin = g[0].time;
    int status = 0;
    for (const GroupState &x : g) {
        tmin = std::min(tmin, x.time);
        status |= x.status;
    }
    if (t_now) *t_now = tmin;
    if (status) return fail(SWE_GPU_ERR_DEVICE, "device status 0x%x (NaN wave speed)", status);
    return SWE_GPU_OK;
}

int swe_gpu_lts_advance(swe_gpu_domain *dom, float t_end, int max_iterations, int *intervals_done, float *t_now) {
    if (!dom || max_iterations < 0) return fail(SWE_GPU_ERR_INVALID, "bad argument");
    if (!dom->lts) return fail(SWE_GPU_ERR_INVALID, "not a local-time-stepping domain");
    CUDA_TRY(cudaSetDevice(dom->device));
    const int batch = 8;  // inner iterations per graph replay
    if (!dom->ltsGraph) {
        cudaGraph_t g;
        CUDA_TRY(cudaStreamBeginCapture(dom->stream, cudaStreamCaptureModeThreadLocal));
        int rc = SWE_GPU_OK;
        const long long before = dom->launches;
        for (int i = 0; i < batch && rc == SWE_GPU_OK; i++) rc = enqueueLtsIteration(dom);
        cudaError_t e = cudaStreamEndCapture(dom->stream, &g);
        dom->ltsGraphKernels = dom->launches - before;
        dom->launches = before;
        if (rc) return rc;
        if (e != cudaSuccess) return fail(SWE_GPU_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&dom->ltsGraph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(SWE_GPU_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
    if (!dom->ltsCtlHost) {
        cudaError_t e = cudaMallocHost(&dom->ltsCtlHost, 2 * sizeof(LtsControl));
        if (e != cudaSuccess) {
            dom->ltsCtlHost = nullptr;
            return fail(SWE_GPU_ERR_NOMEM, "cudaMallocHost: %s", cudaGetErrorString(e));
        }
        for (int j = 0; j < 2; j++) CUDA_TRY(cudaEventCreateWithFlags(&dom->ltsCtlReady[j], cudaEventDisableTiming));
    }
    LtsControl c{};
    CUDA_TRY(cudaMemcpyAsync(&c, dom->dLtsCtl, sizeof(LtsControl), cudaMemcpyDeviceToHost, dom->stream));
    CUDA_TRY(cudaStreamSynchronize(dom->stream));
    const int startIntervals = c.intervals, startIterations = c.iterations;
    const int limit = int(std::min<long long>(INT32_MAX, (long long)c.iterations + max_iterations));
    CUDA_TRY(cudaMemcpyAsync(&dom->dLtsCtl->target, &t_end, sizeof(float), cudaMemcpyHostToDevice, dom->stream));
    CUDA_TRY(cudaMemcpyAsync(&dom->dLtsCtl->iterLimit, &limit, sizeof(int), cudaMemcpyHostToDevice, dom->stream));
    // replays of `batch` iterations with the next one queued before the
    // host reads the last one's control block: the device does not wait for
    // the host between replays.  Iterations queued past the target or the
    // limit do nothing (the kernels test the control block).
    auto replay = [&](int slot) -> int {
        CUDA_TRY(cudaGraphLaunch(dom->ltsGraph, dom->stream));
        dom->launches += dom->ltsGraphKernels;
        CUDA_TRY(cudaMemcpyAsync(dom->ltsCtlHost + slot, dom->dLtsCtl, sizeof(LtsControl), cudaMemcpyDeviceToHost,
                                 dom->stream));
        CUDA_TRY(cudaEventRecord(dom->ltsCtlReady[slot], dom->stream));
        return SWE_GPU_OK;
    };
    if (c.t < t_end && c.iterations < limit) {
        int rc = replay(0);
        if (rc) return rc;
        for (int slot = 0;; slot ^= 1) {
            rc = replay(slot ^ 1);
            if (rc) return rc;
            CUDA_TRY(cudaEventSynchronize(dom->ltsCtlReady[slot]));
            c = dom->ltsCtlHost[slot];
            if (!(c.t < t_end && c.iterations < limit)) break;
        }
        CUDA_TRY(cudaStreamSynchronize(dom->stream));
        c = dom->ltsCtlHost[0].iterations > dom->ltsCtlHost[1].iterations ? dom->ltsCtlHost[0] : dom->ltsCtlHost[1];
    }
    // the update passes push no ghosts: a check with the run over carries the
    // last ring into the current buffer, as the reference's single array holds it
    CUDA_TRY(launchLtsCheck(dom->dev, dom->stream, false));
    dom->launches++;
    // stop: no kernel runs until the next call sets a new target
    const float stop = -INFINITY;
    CUDA_TRY(cudaMemcpyAsync(&dom->dLtsCtl->target, &stop, sizeof(float), cudaMemcpyHostToDevice, dom->stream));
    CUDA_TRY(cudaStreamSynchronize(dom->stream));
    if (intervals_done) *intervals_done = c.intervals - startIntervals;
    if (t_now) *t_now = c.t;
    std::vector<GroupState> g;
    int rc = readGroups(dom, g);
    if (rc) return rc;
    int status = 0;
    for (const GroupState &s : g) status |= s.status;
    if (status) return fail(SWE_GPU_ERR_DEVICE, "device status 0x%x", status);
    if (c.t < t_end && c.iterations - startIterations >= max_iterations)
        return SWE_GPU_INCOMPLETE;  // the iteration budget ran out first
    return SWE_GPU_OK;
}

int swe_gpu_lts_state(swe_gpu_domain *dom, float *t, int *intervals, int *iterations, int *block_steps) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    if (!dom->lts) return fail(SWE_GPU_ERR_INVALID, "not a local-time-stepping domain");
    CUDA_TRY(cudaSetDevice(dom->device));
    LtsControl c{};
    std::vector<LtsBlock> L(dom->blocks.size());
    CUDA_TRY(cudaMemcpyAsync(&c, dom->dLtsCtl, sizeof(LtsControl), cudaMemcpyDeviceToHost, dom->stream));
    CUDA_TRY(cudaMemcpyAsync(L.data(), dom->dLts, sizeof(LtsBlock) * L.size(), cudaMemcpyDeviceToHost, dom->stream));
    CUDA_TRY(cudaStreamSynchronize(dom->stream));
    if (t) *t = c.t;
    if (intervals) *intervals = c.intervals;
    if (iterations) *iterations = c.iterations;
    if (block_steps)
        for (size_t k = 0; k < L.size(); k++) block_steps[k] = L[k].lastStepSize;
    return SWE_GPU_OK;
}

int swe_gpu_block_steps(swe_gpu_domain *dom, long long *steps) {
    if (!dom || !steps) return fail(SWE_GPU_ERR_INVALID, "null argument");
    CUDA_TRY(cudaSetDevice(dom->device));
    std::vector<GroupState> g;
    int rc = readGroups(dom, g);
    if (rc) return rc;
    for (size_t k = 0; k < dom->blocks.size(); k++) steps[k] = g[dom->blocks[k].group].steps;
    return SWE_GPU_OK;
}

int swe_gpu_lts_blocks(swe_gpu_domain *dom, int *ints, float *border) {
    if (!dom || !ints || !border) return fail(SWE_GPU_ERR_INVALID, "null argument");
    if (!dom->lts) return fail(SWE_GPU_ERR_INVALID, "not a local-time-stepping domain");
    CUDA_TRY(cudaSetDevice(dom->device));
    std::vector<LtsBlock> L(dom->blocks.size());
    CUDA_TRY(cudaMemcpyAsync(L.data(), dom->dLts, sizeof(LtsBlock) * L.size(), cudaMemcpyDeviceToHost, dom->stream));
    CUDA_TRY(cudaStreamSynchronize(dom->stream));
    for (size_t k = 0; k < L.size(); k++) {
        for (int s4 = 0; s4 < 4; s4++) {
            ints[8 * k + s4] = L[k].received[s4];
            border[4 * k + s4] = L[k].borderTimestep[s4];
        }
        ints[8 * k + 4] = L[k].stepSize;
        ints[8 * k + 5] = L[k].stepSizeCounter;
        ints[8 * k + 6] = L[k].timestepCounter;
        ints[8 * k + 7] = L[k].notified;
    }
    return SWE_GPU_OK;
}

int swe_gpu_group_count(const swe_gpu_domain *dom, int *count) {
    if (!dom || !count) return fail(SWE_GPU_ERR_INVALID, "null argument");
    *count = dom->ngroups;
    return SWE_GPU_OK;
}

int swe_gpu_group_state(swe_gpu_domain *dom, float *time, float *dt, int *steps) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    std::vector<GroupState> g;
    int rc = readGroups(dom, g);
    if (rc) return rc;
    for (size_t i = 0; i < g.size(); i++) {
        if (time) time[i] = g[i].time;
        if (dt) dt[i] = g[i].dt;
        if (steps) steps[i] = g[i].steps;
    }
    return SWE_GPU_OK;
}

int swe_gpu_retile(swe_gpu_domain *dom, int tile_rows, int tile_cols) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    int rc = checkTiles(tile_rows, tile_cols);
    if (rc) return rc;
    CUDA_TRY(cudaSetDevice(dom->device));
    CUDA_TRY(cudaStreamSynchronize(dom->stream));
    int maxNy = 0;
    for (const BlockDesc &B : dom->blocks) maxNy = std::max(maxNy, B.ny);
    dom->tileRows = std::min(tile_rows > 0 ? tile_rows : 256, ((maxNy + 31) / 32) * 32);
    dom->tileColsArg = tile_cols;
    dom->tileCols = tile_cols > 0 ? tile_cols : 32;
    buildPartitions(dom, tile_cols);
    // device copies of the new partitions; per-group segment counts
    cudaFree(dom->dUnits);
    cudaFree(dom->dCtaSeg);
    cudaFree(dom->dUnitsU);
    cudaFree(dom->dCtaSegU);
    dom->dUnits = nullptr;
    dom->dCtaSeg = nullptr;
    dom->dUnitsU = nullptr;
    dom->dCtaSegU = nullptr;
    CUDA_TRY(cudaMalloc(&dom->dUnits, sizeof(WorkUnit) * dom->units.size()));
    CUDA_TRY(cudaMalloc(&dom->dCtaSeg, sizeof(int) * dom->ctaSeg.size()));
    CUDA_TRY(cudaMalloc(&dom->dUnitsU, sizeof(WorkUnit) * dom->unitsU.size()));
    CUDA_TRY(cudaMalloc(&dom->dCtaSegU, sizeof(int) * dom->ctaSegU.size()));
    CUDA_TRY(cudaMemcpy(dom->dUnits, dom->units.data(), sizeof(WorkUnit) * dom->units.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dom->dCtaSeg, dom->ctaSeg.data(), sizeof(int) * dom->ctaSeg.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dom->dUnitsU, dom->unitsU.data(), sizeof(WorkUnit) * dom->unitsU.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dom->dCtaSegU, dom->ctaSegU.data(), sizeof(int) * dom->ctaSegU.size(), cudaMemcpyHostToDevice));
    std::vector<GroupState> g;
    rc = readGroups(dom, g);
    if (rc) return rc;
    groupCounts(dom, g);
    CUDA_TRY(cudaMemcpy(dom->dGroups, g.data(), sizeof(GroupState) * g.size(), cudaMemcpyHostToDevice));
    dom->dev.units = dom->dUnits;
    dom->dev.ctaSeg = dom->dCtaSeg;
    dom->dev.tileRows = dom->tileRows;
    if (dom->fast) {
        if (!buildFastPlan(dom)) return fail(SWE_GPU_ERR_INVALID, "fast arithmetic: pieces do not line up");
        rc = uploadFastPlan(dom);
        if (rc) return rc;
        groupCounts(dom, g);
        CUDA_TRY(cudaMemcpy(dom->dGroups, g.data(), sizeof(GroupState) * g.size(), cudaMemcpyHostToDevice));
    }
    // captured step graphs hold the old launch shapes
    if (dom->graph) cudaGraphExecDestroy(dom->graph);
    if (dom->ltsGraph) cudaGraphExecDestroy(dom->ltsGraph);
    dom->graph = nullptr;
    dom->ltsGraph = nullptr;
    return SWE_GPU_OK;
}

int swe_gpu_autotune(swe_gpu_domain *dom, int trial_steps, int *best_rows, int *best_cols, float *best_ms) {
    if (!dom || trial_steps < 1) return fail(SWE_GPU_ERR_INVALID, "bad argument");
    if (dom->lts) return fail(SWE_GPU_ERR_INVALID, "the tuner times global steps; not for local time stepping");
    CUDA_TRY(cudaSetDevice(dom->device));
    CUDA_TRY(cudaStreamSynchronize(dom->stream));
    // save the state the trials run on, restore it after each
    const size_t bytes = dom->fieldElems * sizeof(float);
    std::vector<float *> save(6, nullptr);
    float *live[6] = {dom->h[0], dom->h[1], dom->hu[0], dom->hu[1], dom->hv[0], dom->hv[1]};
    GroupState *gsave = nullptr;
    unsigned int *wsave = nullptr;
    unsigned long long *ksave = nullptr;
    const size_t nt = dom->tiles.size();
    auto release = [&]() {
        for (float *p : save) cudaFree(p);
        cudaFree(gsave);
        cudaFree(wsave);
        cudaFree(ksave);
    };
    bool ok = true;
    for (int i = 0; i < 6 && ok; i++) ok = cudaMalloc(&save[i], bytes) == cudaSuccess;
    ok = ok && cudaMalloc(&gsave, sizeof(GroupState) * dom->ngroups) == cudaSuccess;
    if (nt) {
        ok = ok && cudaMalloc(&wsave, sizeof(unsigned int) * 2 * nt) == cudaSuccess;
        ok = ok && cudaMalloc(&ksave, sizeof(unsigned long long) * 2 * nt) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        release();
        return fail(SWE_GPU_ERR_NOMEM, "tuner: no room for a copy of the state");
    }
    const bool ghostsValid = dom->ghostsValid, dtValid = dom->dtValid;
    auto copyState = [&](bool toSave) -> cudaError_t {
        for (int i = 0; i < 6; i++) {
            cudaError_t e = cudaMemcpyAsync(toSave ? save[i] : live[i], toSave ? live[i] : save[i], bytes,
                                            cudaMemcpyDeviceToDevice, dom->stream);
            if (e != cudaSuccess) return e;
        }
        cudaError_t e = cudaMemcpyAsync(toSave ? gsave : dom->dGroups, toSave ? dom->dGroups : gsave,
                                        sizeof(GroupState) * dom->ngroups, cudaMemcpyDeviceToDevice, dom->stream);
        if (e == cudaSuccess && nt) {
            e = cudaMemcpyAsync(toSave ? wsave : dom->dTileW, toSave ? dom->dTileW : wsave, sizeof(unsigned int) * 2 * nt,
                                cudaMemcpyDeviceToDevice, dom->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(toSave ? ksave : dom->dTileKey, toSave ? dom->dTileKey : ksave,
                                    sizeof(unsigned long long) * 2 * nt, cudaMemcpyDeviceToDevice, dom->stream);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(dom->stream);
        dom->ghostsValid = ghostsValid;
        dom->dtValid = dtValid;
        if (e == cudaSuccess && !toSave) {
            // the saved group states carry the saved partition's segment counts
            std::vector<GroupState> g(dom->ngroups);
            e = cudaMemcpy(g.data(), dom->dGroups, sizeof(GroupState) * g.size(), cudaMemcpyDeviceToHost);
            groupCounts(dom, g);
            if (e == cudaSuccess)
                e = cudaMemcpy(dom->dGroups, g.data(), sizeof(GroupState) * g.size(), cudaMemcpyHostToDevice);
        }
        return e;
    };
    cudaError_t e = copyState(true);
    if (e != cudaSuccess) {
        release();
        return fail(SWE_GPU_ERR_CUDA, "tuner: %s", cudaGetErrorString(e));
    }
    int maxNy = 0;
    for (const BlockDesc &B : dom->blocks) maxNy = std::max(maxNy, B.ny);
    const int rowCands[4] = {32, 64, 128, 256}, colCands[4] = {0, 8, 32, 128};
    const int origRows = dom->tileRows, origCols = dom->tileColsArg;
    int bestR = origRows, bestC = origCols;
    float bestT = INFINITY;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = SWE_GPU_OK;
    for (int r : rowCands) {
        if (r > ((maxNy + 31) / 32) * 32 && r != 32) continue;
        for (int c : colCands) {
            if ((rc = swe_gpu_retile(dom, r, c))) break;
            if ((e = copyState(false)) != cudaSuccess) break;
            for (int i = 0; i < 2 && !rc; i++) rc = enqueueStep(dom);  // warm-up
            cudaEventRecord(e0, dom->stream);
            for (int i = 0; i < trial_steps && !rc; i++) rc = enqueueStep(dom);
            cudaEventRecord(e1, dom->stream);
            if (rc || (e = cudaEventSynchronize(e1)) != cudaSuccess) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms /= float(trial_steps);
            if (ms < bestT) {
                bestT = ms;
                bestR = dom->tileRows;
                bestC = c;
            }
        }
        if (rc || e != cudaSuccess) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // the best shape, on the original state
    const bool failed = rc || e != cudaSuccess;
    const int rc2 = swe_gpu_retile(dom, failed ? origRows : bestR, failed ? origCols : bestC);
    const cudaError_t e2 = copyState(false);
    release();
    if (rc) return rc;
    if (e != cudaSuccess) return fail(SWE_GPU_ERR_CUDA, "tuner: %s", cudaGetErrorString(e));
    if (rc2) return rc2;
    if (e2 != cudaSuccess) return fail(SWE_GPU_ERR_CUDA, "tuner: %s", cudaGetErrorString(e2));
    if (best_rows) *best_rows = bestR;
    if (best_cols) *best_cols = bestC;
    if (best_ms) *best_ms = bestT;
    return SWE_GPU_OK;
}

int swe_gpu_speed_pass_stats(swe_gpu_domain *dom, int *tiles, int *evaluated) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    std::vector<GroupState> g;
    int rc = readGroups(dom, g);
    if (rc) return rc;
    int t = 0, e = 0;
    for (const GroupState &s : g) {
        t += s.tiles;
        e += s.lastCandidates;
    }
    if (tiles) *tiles = dom->bounded ? t : 0;
    if (evaluated) *evaluated = dom->bounded ? e : 0;
    return SWE_GPU_OK;
}

int swe_gpu_lts_round_timesteps(const float *t, int n, float max_timestep_local, int max_divisor, int *step_sizes,
                                int device) {
    if (n < 0 || (n > 0 && (!t || !step_sizes)) || !(max_timestep_local > 0.f) || max_divisor < 1)
        return fail(SWE_GPU_ERR_INVALID, "bad argument");
    if (n == 0) return SWE_GPU_OK;
    CUDA_TRY(cudaSetDevice(device));
    float *dt = nullptr;
    int *ds = nullptr;
    cudaError_t e = cudaMalloc(&dt, sizeof(float) * size_t(n));
    if (e == cudaSuccess) e = cudaMalloc(&ds, sizeof(int) * size_t(n));
    if (e == cudaSuccess) e = cudaMemcpy(dt, t, sizeof(float) * size_t(n), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launchLtsRound(dt, n, max_timestep_local, max_divisor, ds, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(step_sizes, ds, sizeof(int) * size_t(n), cudaMemcpyDeviceToHost);
    cudaFree(dt);
    cudaFree(ds);
    if (e != cudaSuccess) return fail(SWE_GPU_ERR_CUDA, "lts rounding: %s", cudaGetErrorString(e));
    return SWE_GPU_OK;
}

int swe_gpu_fast_pieces(const swe_gpu_domain *dom, int *out, int cap, int *count) {
    if (!dom || !count || cap < 0 || (cap > 0 && !out)) return fail(SWE_GPU_ERR_INVALID, "bad argument");
    if (!dom->fast) return fail(SWE_GPU_ERR_INVALID, "not a fast-arithmetic domain");
    *count = int(dom->pieces.size());
    for (int i = 0; i < std::min(cap, *count); i++) {
        const fast::Piece &p = dom->pieces[i];
        const int v[5] = {p.block, p.dir, p.x0, p.y0, p.len};
        for (int j = 0; j < 5; j++) out[5 * i + j] = v[j];
    }
    return SWE_GPU_OK;
}

int swe_gpu_launch_count(const swe_gpu_domain *dom, long long *count) {
    if (!dom || !count) return fail(SWE_GPU_ERR_INVALID, "null argument");
    *count = dom->launches;
    return SWE_GPU_OK;
}

int swe_gpu_get_time(swe_gpu_domain *dom, float *t, int *steps) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    std::vector<GroupState> g;
    int rc = readGroups(dom, g);
    if (rc) return rc;
    if (t) *t = g[0].time;
    if (steps) *steps = g[0].steps;
    return SWE_GPU_OK;
}

int swe_gpu_set_time(swe_gpu_domain *dom, float t) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    for (int gi = 0; gi < dom->ngroups; gi++)
        CUDA_TRY(cudaMemcpyAsync(&dom->dGroups[gi].time, &t, sizeof(float), cudaMemcpyHostToDevice, dom->stream));
    CUDA_TRY(cudaStreamSynchronize(dom->stream));
    return SWE_GPU_OK;
}

int swe_gpu_sync(swe_gpu_domain *dom) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    CUDA_TRY(cudaStreamSynchronize(dom->stream));
    if (dom->copyStream) CUDA_TRY(cudaStreamSynchronize(dom->copyStream));
    if (dom->upStream) CUDA_TRY(cudaStreamSynchronize(dom->upStream));
    return SWE_GPU_OK;
}

int swe_gpu_status(swe_gpu_domain *dom, int *status) {
    if (!dom || !status) return fail(SWE_GPU_ERR_INVALID, "null argument");
    CUDA_TRY(cudaSetDevice(dom->device));
    std::vector<GroupState> g;
    int rc = readGroups(dom, g);
    if (rc) return rc;
    int s = 0;
    for (auto &x : g) s |= x.status;
    *status = s;
    return SWE_GPU_OK;
}

int swe_gpu_get_stream(swe_gpu_domain *dom, void **stream) {
    if (!dom || !stream) return fail(SWE_GPU_ERR_INVALID, "null argument");
    *stream = dom->stream;
    return SWE_GPU_OK;
}

int swe_gpu_set_stream(swe_gpu_domain *dom, void *stream) {
    if (!dom) return fail(SWE_GPU_ERR_INVALID, "null domain handle");
    CUDA_TRY(cudaSetDevice(dom->device));
    CUDA_TRY(cudaStreamSynchronize(dom->stream));
    dom->stream = stream ? static_cast<cudaStream_t>(stream) : dom->ownStream;
    return SWE_GPU_OK;
}

int swe_gpu_solve_edges(int solver, long long n, const float *hL, const float *hR, const float *huL,
                        const float *huR, const float *bL, const float *bR, float *hUpdL, float *hUpdR,
                        float *huUpdL, float *huUpdR, float *maxWaveSpeed, void *stream) {
    if (n < 0) return fail(SWE_GPU_ERR_INVALID, "negative edge count");
    if (n == 0) return SWE_GPU_OK;
    const int th = 256;
    const unsigned blocks = unsigned((n + th - 1) / th);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (solver) {
    case SWE_SOLVER_FWAVE: solveEdgesKernel<SOLVER_FWAVE><<<blocks, th, 0, s>>>(n, hL, hR, huL, huR, bL, bR, hUpdL, hUpdR, huUpdL, huUpdR, maxWaveSpeed); break;
    case SWE_SOLVER_AUGRIE: solveEdgesKernel<SOLVER_AUGRIE><<<blocks, th, 0, s>>>(n, hL, hR, huL, huR, bL, bR, hUpdL, hUpdR, huUpdL, huUpdR, maxWaveSpeed); break;
    case SWE_SOLVER_HYBRID: solveEdgesKernel<SOLVER_HYBRID><<<blocks, th, 0, s>>>(n, hL, hR, huL, huR, bL, bR, hUpdL, hUpdR, huUpdL, huUpdR, maxWaveSpeed); break;
    case SWE_SOLVER_HLLE: solveEdgesKernel<SOLVER_HLLE><<<blocks, th, 0, s>>>(n, hL, hR, huL, huR, bL, bR, hUpdL, hUpdR, huUpdL, huUpdR, maxWaveSpeed); break;
    default: return fail(SWE_GPU_ERR_INVALID, "unknown solver %d", solver);
    }
    CUDA_TRY(cudaGetLastError());
    return SWE_GPU_OK;
}


// ---------------------------------------------------------------------------
// MLP surrogate on a domain (include/swe_gb300_mlp.h)
// ---------------------------------------------------------------------------
static int ensureEdgeTiles(swe_gpu_domain *D) {
    if (D->dEdgeTiles) return SWE_GPU_OK;
    D->edgeTiles = mlp::buildEdgeTiles(D->blocks);
    CUDA_TRY(cudaMalloc(&D->dEdgeTiles, D->edgeTiles.size() * sizeof(mlp::EdgeTile)));
    CUDA_TRY(cudaMemcpy(D->dEdgeTiles, D->edgeTiles.data(), D->edgeTiles.size() * sizeof(mlp::EdgeTile),
                        cudaMemcpyHostToDevice));
    return SWE_GPU_OK;
}

int swe_gpu_surrogate_step(swe_gpu_domain *dom, swe_mlp *m, int nsteps, long long *surrogate_edges) {
    if (!dom || nsteps < 0) return fail(SWE_GPU_ERR_INVALID, "bad argument");
    if (dom->lts) return fail(SWE_GPU_ERR_INVALID, "local-time-stepping domain: the surrogate step is global");
    if (dom->semantics != SEM_UNSPLIT) return fail(SWE_GPU_ERR_INVALID, "the surrogate step is the unsplit step (semantics 0)");
    if (m && mlp::deviceOf(m) != dom->device)
        return fail(SWE_GPU_ERR_INVALID, "surrogate on device %d, domain on device %d", mlp::deviceOf(m), dom->device);
    CUDA_TRY(cudaSetDevice(dom->device));
    int rc = ensureEdgeTiles(dom);
    if (rc) return rc;
    if (!dom->edgeBuf) CUDA_TRY(cudaMalloc(&dom->edgeBuf, 8 * dom->fieldElems * sizeof(float)));
    if (!dom->dUsed) CUDA_TRY(cudaMalloc(&dom->dUsed, sizeof(unsigned long long)));
    mlp::EdgeUpdates u;
    for (int k = 0; k < 4; k++) {
        u.x[k] = dom->edgeBuf + size_t(k) * dom->fieldElems;
        u.y[k] = dom->edgeBuf + size_t(4 + k) * dom->fieldElems;
    }
    long long maxCells = 0;
    for (const BlockDesc &B : dom->blocks) maxCells = std::max(maxCells, (long long)B.nx * B.ny);
    CUDA_TRY(cudaMemsetAsync(dom->dUsed, 0, sizeof(unsigned long long), dom->stream));
    const int ntiles = int(dom->edgeTiles.size());
    for (int i = 0; i < nsteps; i++) {
        if (i > 0 || !dom->ghostsValid) {
            if ((rc = enqueueGhost(dom, 0))) return rc;
        }
        CUDA_TRY(mlp::launchSurrogateEdges(dom->dev, m, dom->dEdgeTiles, ntiles, u, dom->dUsed, dom->stream));
        CUDA_TRY(mlp::launchSurrogateDt(dom->dev, dom->ngroups, dom->stream));
        CUDA_TRY(mlp::launchSurrogateApply(dom->dev, u, int(dom->blocks.size()), maxCells, dom->stream));
        CUDA_TRY(mlp::launchSurrogateFinish(dom->dev, dom->ngroups, dom->stream));
        dom->launches += 4;
    }
    // the ghost ring of the new state, as the regular update pass leaves it
    if (nsteps > 0) {
        if ((rc = enqueueGhost(dom, 2))) return rc;
    }
    dom->ghostsValid = true;
    if (surrogate_edges) {
        unsigned long long used = 0;
        CUDA_TRY(cudaStreamSynchronize(dom->stream));
        CUDA_TRY(cudaMemcpy(&used, dom->dUsed, sizeof(used), cudaMemcpyDeviceToHost));
        *surrogate_edges = (long long)used;
    }
    if (m) {
        CUDA_TRY(cudaStreamSynchronize(dom->stream));
        if (mlp::checkDeviceError(m, "surrogate step")) return fail(SWE_GPU_ERR_DEVICE, "%s", swe_mlp_last_error());
    }
    return SWE_GPU_OK;
}

int swe_gpu_surrogate_edge_count(swe_gpu_domain *dom, long long *edges) {
    if (!dom || !edges) return fail(SWE_GPU_ERR_INVALID, "null argument");
    long long n = 0;
    for (const BlockDesc &B : dom->blocks) n += (long long)(B.nx + 1) * B.ny + (long long)B.nx * (B.ny + 1);
    *edges = n;
    return SWE_GPU_OK;
}

int swe_gpu_log_edges(swe_gpu_domain *dom, int stride, int capacity, float *edges, float *targets, int *count) {
    if (!dom || stride < 1 || capacity < 0 || !count || (capacity > 0 && (!edges || !targets)))
        return fail(SWE_GPU_ERR_INVALID, "bad argument");
    if (dom->lts) return fail(SWE_GPU_ERR_INVALID, "local-time-stepping domain");
    CUDA_TRY(cudaSetDevice(dom->device));
    int rc = ensureEdgeTiles(dom);
    if (rc) return rc;
    if ((rc = enqueueGhost(dom, 0))) return rc;
    dom->ghostsValid = true;
    const int ntiles = int(dom->edgeTiles.size());
    const long long nslots = ((long long)ntiles * 128 + stride - 1) / stride;
    float *dSlots = nullptr;
    CUDA_TRY(cudaMalloc(&dSlots, size_t(11) * nslots * sizeof(float)));
    std::vector<float> hs(size_t(11) * nslots);
    cudaError_t e = mlp::launchLogEdges(dom->dev, dom->dEdgeTiles, ntiles, stride, dSlots, nslots, dom->stream);
    dom->launches++;
    if (e == cudaSuccess) e = cudaStreamSynchronize(dom->stream);
    if (e == cudaSuccess) e = cudaMemcpy(hs.data(), dSlots, hs.size() * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dSlots);
    if (e != cudaSuccess) return fail(SWE_GPU_ERR_CUDA, "log edges: %s", cudaGetErrorString(e));
    int c = 0;
    for (long long k = 0; k < nslots && c < capacity; k++) {
        if (hs[size_t(10) * nslots + k] == 0.f) continue;
        for (int f = 0; f < 6; f++) edges[size_t(f) * capacity + c] = hs[size_t(f) * nslots + k];
        for (int f = 0; f < 4; f++) targets[size_t(f) * capacity + c] = hs[size_t(6 + f) * nslots + k];
        c++;
    }
    // rows of length c (packed in place; row f moves down from f * capacity)
    for (int f = 1; f < 6; f++) memmove(edges + size_t(f) * c, edges + size_t(f) * capacity, size_t(c) * sizeof(float));
    for (int f = 1; f < 4; f++) memmove(targets + size_t(f) * c, targets + size_t(f) * capacity, size_t(c) * sizeof(float));
    *count = c;
    return SWE_GPU_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free single-block step.
//
// Some callers cannot allocate device memory: hosts whose GPU memory is owned
// by another allocator (a framework's caching pool or a pre-sized arena that
// must not grow), and latency-critical loops that cannot afford cudaMalloc's
// implicit device-wide synchronisation.  swe_gpu_step_block_noalloc runs one
// step of one block on the caller's device arrays and keeps the little scratch
// the step kernels need (the dt control block, the block descriptor and the
// CTA work list) in the file-scope array below instead of allocating it.
// ---------------------------------------------------------------------------
namespace {

constexpr int kNoAllocMaxUnits = 4096;  // CTA work units: (ny/256 rounded up) * (nx/32 rounded up)
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocScratch {
    GroupState group;
    BlockDesc block;
    WorkUnit units[kNoAllocMaxUnits];
    int ctaSeg[kNoAllocMaxUnits + 1];
};

} // namespace

// One copy per GPU that loads the library, held until the process exits
// (about 82 KB).  Every call on a device reuses it: the set-up kernel below
// clears the control block at the start of each call, and calls that overlap
// on the GPU (different streams, or several host threads) race on it.
static __device__ __align__(256) NoAllocScratch g_noallocScratch;

namespace {

std::mutex g_noallocMutex;
NoAllocScratch *g_noallocPtr[kNoAllocMaxDevices] = {};

/// Device address of the scratch array for `device` (current device), looked
/// up once per device; in host code the symbol itself is only a stand-in.
int noallocScratch(int device, NoAllocScratch **out) {
    if (device < 0 || device >= kNoAllocMaxDevices)
        return fail(SWE_GPU_ERR_INVALID, "device %d beyond the %d supported", device, kNoAllocMaxDevices);
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocPtr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess)
            return fail(SWE_GPU_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        g_noallocPtr[device] = static_cast<NoAllocScratch *>(p);
    }
    *out = g_noallocPtr[device];
    return SWE_GPU_OK;
}

/// writes the block descriptor and work list and clears the control block
__global__ void noallocSetupKernel(NoAllocScratch *s, BlockDesc b, int tileRows, int tileCols, int nunits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        GroupState g{};
        g.enabled = 1;
        g.speedBits = 0u;
        g.arrived = 0u;
        g.units = nunits;
        g.unitsUpd = nunits;
        g.firstBlock = 0;
        g.dt = 0.f;
        g.speed = 0.f;
        g.time = 0.f;
        g.target = INFINITY;
        g.steps = 0;
        g.cur = 0;
        g.status = 0;
        g.ghostsAhead = 0;
        s->group = g;
        s->block = b;
    }
    const int xChunks = (b.nx + tileCols - 1) / tileCols;
    for (int u = i; u < nunits; u += gridDim.x * blockDim.x) {
        const int ty = u / xChunks, xc = u % xChunks;
        s->units[u] = WorkUnit{0, 1 + ty * tileRows, 1 + xc * tileCols, min(1 + (xc + 1) * tileCols, b.nx + 1)};
        s->ctaSeg[u] = u;  // one segment per CTA
    }
    if (i == 0) s->ctaSeg[nunits] = nunits;
}

} // namespace

extern "C" int swe_gpu_step_block_noalloc(int solver, int semantics, int nx, int ny, float dx, float dy,
                                          const int *boundary, int ld, float *h, float *hu, float *hv,
                                          const float *b, float *h_out, float *hu_out, float *hv_out,
                                          float *dt_out, void *stream) {
    if (solver < SWE_SOLVER_FWAVE || solver > SWE_SOLVER_HLLE) return fail(SWE_GPU_ERR_INVALID, "unknown solver %d", solver);
    if (semantics != SWE_SEMANTICS_UNSPLIT && semantics != SWE_SEMANTICS_SPLIT)
        return fail(SWE_GPU_ERR_INVALID, "unknown semantics %d", semantics);
    if (nx < 1 || ny < 1) return fail(SWE_GPU_ERR_INVALID, "block size %d x %d", nx, ny);
    if (!(dx > 0.f) || !(dy > 0.f)) return fail(SWE_GPU_ERR_INVALID, "dx, dy must be positive");
    if (ld < ny + 2) return fail(SWE_GPU_ERR_INVALID, "ld %d < ny+2 = %d", ld, ny + 2);
    if (!boundary || !h || !hu || !hv || !b || !h_out || !hu_out || !hv_out)
        return fail(SWE_GPU_ERR_INVALID, "null array argument");
    for (int i = 0; i < 4; i++)
        if (boundary[i] < SWE_OUTFLOW || boundary[i] > SWE_PASSIVE || boundary[i] == SWE_CONNECT_WITHIN_RANK)
            return fail(SWE_GPU_ERR_INVALID, "boundary %d: type %d is not valid for a single block", i, boundary[i]);
    const int tileRows = std::min(256, ((ny + 31) / 32) * 32);
    const int tileCols = 32;
    const long long nunits = (long long)((ny + tileRows - 1) / tileRows) * ((nx + tileCols - 1) / tileCols);
    if (nunits > kNoAllocMaxUnits)
        return fail(SWE_GPU_ERR_INVALID,
                    "block %d x %d needs %lld work units; the allocation-free step supports at most %d "
                    "(ceil(ny/256) * ceil(nx/32))", nx, ny, nunits, kNoAllocMaxUnits);
    int device = 0;
    CUDA_TRY(cudaGetDevice(&device));
    NoAllocScratch *scr = nullptr;
    int rc = noallocScratch(device, &scr);
    if (rc) return rc;

    BlockDesc B{};
    B.nx = nx;
    B.ny = ny;
    B.pitch = ld;
    B.group = 0;
    B.base = 0;
    B.dx = dx;
    B.dy = dy;
    B.stage = 0;
    for (int i = 0; i < 4; i++) {
        B.bnd[i] = boundary[i];
        B.nbr[i] = -1;
    }
    DomainDev d{};
    d.h[0] = h; d.h[1] = h_out;
    d.hu[0] = hu; d.hu[1] = hu_out;
    d.hv[0] = hv; d.hv[1] = hv_out;
    d.b = const_cast<float *>(b);
    d.blocks = &scr->block;
    d.units = scr->units;
    d.ctaSeg = scr->ctaSeg;
    d.groups = &scr->group;
    d.nblocks = 1;
    d.solver = solver;
    d.semantics = semantics;
    d.splitDtMode = SPLIT_DT_MAX;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // any CUDA error drops the device's cached scratch address, so a call
    // after the context was torn down (cudaDeviceReset) looks it up again
    // instead of handing the kernels a stale pointer
    auto check = [&](cudaError_t e, const char *what) {
        if (e == cudaSuccess) return SWE_GPU_OK;
        std::lock_guard<std::mutex> lock(g_noallocMutex);
        g_noallocPtr[device] = nullptr;
        return fail(SWE_GPU_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    };
    noallocSetupKernel<<<(unsigned)std::max<long long>(1, std::min<long long>(64, (nunits + 255) / 256)), 256, 0, s>>>(
        scr, B, tileRows, tileCols, int(nunits));
    if ((rc = check(cudaGetLastError(), "set-up kernel"))) return rc;
    const int threads = 128;
    ghostKernel<<<dim3((2 * nx + 2 * ny + 4 + threads - 1) / threads, 1), threads, 0, s>>>(d, 0);
    if ((rc = check(cudaGetLastError(), "ghost kernel"))) return rc;
    if ((rc = check(launchSpeed(d, int(nunits), tileRows, s), "speed pass"))) return rc;
    if ((rc = check(launchUpdate(d, int(nunits), tileRows, s), "update pass"))) return rc;
    if (dt_out) {
        if ((rc = check(cudaMemcpyAsync(dt_out, &scr->group.dt, sizeof(float), cudaMemcpyDeviceToHost, s), "dt copy")))
            return rc;
        if ((rc = check(cudaStreamSynchronize(s), "stream synchronize"))) return rc;
    }
    return SWE_GPU_OK;
}
