// Host-visible types and launchers of the fast-arithmetic step (swe_fast.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

#include "swe_device.cuh"

namespace swegb {
namespace fast {

/// work segment of the fast step: rows [y0, y0 + tile rows) of one block,
/// columns [x0, x1); arr[arrBegin, arrEnd) lists the pieces whose cells it writes
struct Unit {
    int block, y0, x0, x1;
    int arrBegin, arrEnd;
};

/// A run of next-state edges whose two cells are written by different
/// segments.  dir 0: x-edges (x0-1 | x0) of rows y0 .. y0+len-1; dir 1: y-edges
/// (y0-1 | y0) of columns x0 .. x0+len-1; both cells in `block`'s output
/// buffer (a ghost column / row there is filled by the neighbour block's
/// pushes).  The last of the `need` segments writing its cells evaluates it.
struct Piece {
    int block, dir, x0, y0, len, need;
};

struct FastDev {
    DomainDev d;          // fields, block descriptors, dt groups
    const Unit *units;    // segments of the fast step
    const int *ctaSeg;    // CTA c owns segments [ctaSeg[c], ctaSeg[c+1])
    const Piece *pieces;
    unsigned *pieceCnt;   // arrivals per piece in the running step (reset by the evaluator)
    const int *arr;       // piece ids, indexed by Unit::arrBegin .. arrEnd
};

/// most pieces one segment writes into (shared-memory list of a CTA)
constexpr int kMaxArrivals = 32;

/// rows per thread of the fast step kernel
int fastRows();

/// one fast step of every active group (one launch, programmatic dependent
/// launch); tileRows = rows per segment (multiple of 32, <= 256)
cudaError_t launchFastStep(const FastDev &f, int solver, int grid, int tileRows, cudaStream_t s);
/// resident CTAs per SM of the fast step kernel
int fastOccupancy(int solver, int tileRows);

} // namespace fast
} // namespace swegb
