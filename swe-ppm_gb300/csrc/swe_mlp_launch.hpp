// Launchers of the surrogate's domain kernels (swe_mlp.cu), called by the
// domain entry points of swe_capi.cu.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "swe_device.cuh"

struct swe_mlp;

namespace swegb {
namespace mlp {

/// up to 128 consecutive edges of one column of one block: x-edges
/// (col | col+1) of rows j0 .. j0+count-1 (dir 0), or y-edges (j | j+1) of
/// column col for j = j0 .. j0+count-1 (dir 1).  Both sides of every edge are
/// contiguous in the column layout, so a tile's loads coalesce.
struct EdgeTile {
    int block, dir, col, j0, count;
};

/// net updates of every edge (hUpdL, hUpdR, huUpdL, huUpdR with the normal
/// momentum), stored at the element offset of the edge's left / lower cell
struct EdgeUpdates {
    float *x[4];
    float *y[4];
};

/// x-edges (0|1) .. (nx|nx+1) of rows 1..ny and y-edges (0|1) .. (ny|ny+1) of
/// columns 1..nx of every block: the edges one unsplit step solves
/// (src/blocks/SWE_DimensionalSplittingMpi.cpp:382-412), in tiles
inline std::vector<EdgeTile> buildEdgeTiles(const std::vector<BlockDesc> &blocks) {
    std::vector<EdgeTile> t;
    for (int k = 0; k < int(blocks.size()); k++) {
        const BlockDesc &B = blocks[k];
        for (int col = 0; col <= B.nx; col++)
            for (int j0 = 1; j0 <= B.ny; j0 += 128) t.push_back({k, 0, col, j0, std::min(128, B.ny - j0 + 1)});
        for (int col = 1; col <= B.nx; col++)
            for (int j0 = 0; j0 <= B.ny; j0 += 128) t.push_back({k, 1, col, j0, std::min(128, B.ny + 1 - j0)});
    }
    return t;
}

/// the edge pass: every edge's net updates and the groups' max wave speed
/// (m null: the augmented Riemann solver on every edge, through the same
/// kernels); *used counts the edges the surrogate solved
cudaError_t launchSurrogateEdges(const DomainDev &d, const swe_mlp *m, const EdgeTile *tiles, int ntiles, EdgeUpdates u,
                                 unsigned long long *used, cudaStream_t s);
/// dt of every group from its max wave speed (unsplit step)
cudaError_t launchSurrogateDt(const DomainDev &d, int ngroups, cudaStream_t s);
/// the unsplit update of every interior cell from the stored net updates
cudaError_t launchSurrogateApply(const DomainDev &d, EdgeUpdates u, int nblocks, long long maxCells, cudaStream_t s);
/// time, step count and current buffer of every group
cudaError_t launchSurrogateFinish(const DomainDev &d, int ngroups, cudaStream_t s);
/// edge-state logger: slot e / stride of every stride-th edge gets the edge's
/// six inputs, its augmented-solver net updates and a wet flag (11 x nslots)
cudaError_t launchLogEdges(const DomainDev &d, const EdgeTile *tiles, int ntiles, int stride, float *slots,
                           long long nslots, cudaStream_t s);

/// SWE_GPU_ERR_DEVICE (message set) when a tensor-core wait of the surrogate
/// ran out of its iteration limit since the last check; waits for the device
int checkDeviceError(swe_mlp *m, const char *what);
/// the CUDA device the surrogate's state lives on
int deviceOf(const swe_mlp *m);

} // namespace mlp
} // namespace swegb
