// Device-side data layout and Riemann solvers of the GB300 block step.
//
// Layout (HBM): every block owns (nx+2) columns of `pitch` floats per field,
// column x at base + x*pitch, element (x, y) at base + x*pitch + y -- the
// Float2D order of the reference (a[x][y], y contiguous; src/tools/Float2D.hh:74-76)
// with each column shifted by kColPad floats so the first interior row y = 1
// starts on a 128-byte boundary (pitch is a multiple of 32 floats).  h, hu, hv
// are double-buffered (a step reads buffer p and writes buffer p^1, so tiles
// can read their neighbours' halo without racing the update); b is single.
//
// Solvers: the f-wave, HLLE and augmented Riemann solvers restated from the
// published methods (Bale et al. 2002; Einfeldt 1988; George 2008) with the
// swe_solvers argument convention of the reference's call sites
// (src/blocks/SWE_DimensionalSplittingMpi.cpp:403-410).  Every fused
// multiply-add is an explicit fmaf; the library is compiled with -fmad=false,
// IEEE division and square root, so results are reproducible bit for bit.
#pragma once

#include <cfloat>
#include <cstdint>

namespace swegb {

constexpr float kG = 9.81f;
constexpr float kHalfG = 0.5f * 9.81f;  // exact in float
constexpr float kSqrtG = 0x1.90e864p+1f;  // sqrtf(9.81f), correctly rounded
constexpr float kDryTol = 0.01f;        // solver dry tolerance (swe_solvers' default; see AugRieParams)
constexpr float kZeroTol = 1e-7f;       // |s| below this: wave split evenly (the same)
constexpr int kColPad = 31;             // y = 0 sits at offset 31 of a column
constexpr int kMaxTileRows = 256;       // threads per CTA (one row each)
constexpr int kMaxTileCols = 128;       // columns per x-chunk

enum SolverId { SOLVER_FWAVE = 1, SOLVER_AUGRIE = 2, SOLVER_HYBRID = 3, SOLVER_HLLE = 4 };
enum Semantics { SEM_UNSPLIT = 0, SEM_SPLIT = 1 };
enum BoundaryType { OUTFLOW = 0, WALL = 1, INFLOW = 2, CONNECT = 3, CONNECT_WITHIN_RANK = 4, PASSIVE = 5 };
enum SplitDtMode { SPLIT_DT_MAX = 0, SPLIT_DT_LAST_EDGE = 1 };
// states of a received ghost layer under local time stepping (src/blocks/SWE_Block.hh)
enum GhostlayerState { GL_DONE = 0, GL_UNVALID = 1, GL_INTER = 2, GL_SYNC = 3, GL_NEXT = 4 };

struct BlockDesc {
    int nx, ny;       // interior cells
    int pitch;        // floats per column
    int group;        // dt group (one per independent simulation)
    long long base;   // element offset of cell (0, 0)
    int bnd[4];       // boundary types LEFT, RIGHT, BOTTOM, TOP
    int nbr[4];       // neighbour block ids (CONNECT_WITHIN_RANK) or -1
    float dx, dy;
    long long stage;  // offset of the block in the contiguous host-order layout
    int tileBase;     // first bound tile of the block (bounded speed pass)
    int tilesY;       // bound tiles per column of tiles: ceil(ny / 32)
    long long ring;   // local time stepping: offset of the block's receive ring
                      // (LEFT ny, RIGHT ny, BOTTOM nx, TOP nx values per field)
};

// Per-block state of local time stepping (src/blocks/SWE_Block.hh:214-229).
struct __align__(16) LtsBlock {
    int received[4];          // GhostlayerState per side
    float borderTimestep[4];  // the neighbour's total local time when its layer was received
    int stepSize, stepSizeCounter, timestepCounter, notified;
    int lastStepSize;         // stepSize of the last finished interval
    int pad[3];
};

// Interval control of local time stepping (the drivers' outer loop,
// src/examples/swe_mpi_overdecomp.cpp:308-343).
struct LtsControl {
    float t;                  // time at the start of the running interval
    float target;             // intervals run while t < target
    float maxTimestepLocal;   // length of a synchronisation interval (-l)
    float duration;           // simulated duration (last-timestep detection)
    int maxDivisor;           // finest subdivision of an interval
    int intervals;            // finished intervals
    int iterations;           // inner iterations run
    int iterLimit;            // inner iterations run while iterations < iterLimit
};

// work unit of the sweep kernels: one block, rows [y0, y0+TY) x columns [x0, x1)
struct WorkUnit {
    int block, y0, x0, x1;
};

// Per dt-group control block, device-resident.  Kernels of a step skip the
// group once time >= target (so a batch of steps can be queued ahead and stops
// where the reference's `while (t < checkpoint)` loop stops); the last CTA of
// each pass (arrival counter) finishes the pass: dt after the speed pass,
// time/steps/current buffer after the update pass.
struct __align__(128) GroupState {
    // --- updated by atomics while a pass runs (a cache line of their own) ---
    unsigned int speedBits;  // max wave speed of the running step (float bits)
    unsigned int arrived;    // segments / tiles of the running pass that have finished
    // the fastest edge found by the running bounded speed pass:
    // (speed bits << 32) | edge code (bound tile << 13 | dir << 12 | lx << 6 | ly)
    unsigned long long maxEdge;
    int candidates;          // tiles evaluated edge by edge in the running pass
    int hotPad[27];
    // --- read by every CTA of a pass, written by the pass's last CTA ---
    int units;               // segments of the speed pass in this group
    int unitsUpd;            // segments of the update pass in this group
    int firstBlock;          // the group's first block (its dx, dy)
    float dt;                // maxTimestep of the last speed pass
    float speed;             // max wave speed of the last speed pass
    float time;              // simulated time (float, like the drivers' t)
    float target;            // steps run only while time < target
    int steps;               // executed steps
    int cur;                 // buffer (0/1) holding the current state
    int status;              // bit 0: NaN wave speed, bit 1: non-finite water height produced
    int ghostsAhead;         // 1: the current buffer's ghost ring already holds the next
                             // step's boundary values (pushed by the update pass)
    // Bounded speed pass: boundsValid[p] = 1 when the bound tiles' speed
    // bounds and sample keys of parity p describe the state in buffer p
    int boundsValid[2];
    int tiles;               // bound tiles of the group's blocks
    int enabled;             // 0: the group sits this step out (local time stepping)
    // the fastest edge of the last bounded speed pass as element offsets of
    // its two cells (lower, upper) and direction (0: x-edge, 1: y-edge);
    // its speed in the next state is a lower bound of the next maximum
    long long prevA, prevB;
    int prevDir, prevValid;
    int lastCandidates;      // tiles the last bounded speed pass evaluated edge by edge
    int unitsFast;           // segments of the fast-arithmetic step in this group
    int ringStale;           // local time stepping: the update flipped the buffers; the
                             // current buffer's ghost ring is still in the other one
    int ltsStep;             // local time stepping, set by the check: 0 when the block is at
                             // the start of its interval, else its stepSize
};

// Bound tile of the bounded speed pass: 32 x 32 interior cells of a block,
// cells [x0, x1) x [y0, y1) (block coordinates, ends exclusive).  It owns the
// x-edges (x-1|x), x0 <= x < x1, and y-edges (y-1|y), y0 <= y < y1, plus the
// block's right (nx|nx+1) and top (ny|ny+1) edges where x1 = nx+1 or
// y1 = ny+1.  nbr[side] (LEFT, BOTTOM, RIGHT, TOP) names whose speed bound
// covers the cells across the tile's side that these edges touch: a tile id,
// kNbrSelf (the tile's own cells: a copy or mirror ghost, or no edge on that
// side) or kNbrUnbounded (ghosts set elsewhere).
struct TileInfo {
    long long base;
    int pitch, group;
    int x0, x1, y0, y1;
    int nx, ny;
    int nbr[4];
};
constexpr int kNbrSelf = -1;
constexpr int kNbrUnbounded = -2;
constexpr int kBoundTile = 32;

struct DomainDev {
    float *h[2], *hu[2], *hv[2];
    float *b;
    const BlockDesc *blocks;
    const WorkUnit *units;   // segments: block, rows [y0, y0+TY), columns [x0, x1)
    const int *ctaSeg;       // CTA c owns segments [ctaSeg[c], ctaSeg[c+1])
    GroupState *groups;
    int nblocks;
    int solver, semantics, splitDtMode;
    int tileRows;            // TY of the CTA-tile mapping
    // bounded speed pass (null when the full speed pass is used), two
    // parities of ntiles entries each, parity p describing the state written
    // into buffer p: tileW = float bits of the largest cell speed bound of the
    // tile, tileKey = (those bits << 32) | x << 16 | y of a cell attaining it
    // (block coordinates), 0 if none
    unsigned int *tileW;
    unsigned long long *tileKey;
    const TileInfo *tileInfo;
    int ntiles;
    unsigned long long tileHashMul;  // coprime to ntiles: slot -> tile permutation
    // local time stepping (null without): one group per block
    LtsBlock *lts;
    LtsControl *ltsCtl;
    float *ring[3];                  // receive rings of h, hu, hv
    int *ltsWork;                    // the iteration's work lists (layout: kLw* below)
    float *ltsLocal;                 // every block's total local time at the end of the last iteration
    int ltsCheckSpeed;               // 1: the check computes an interval start's dt itself
                                     // (f-wave / HLLE, blocks up to kLtsCheckSpeedCells cells)
};

// Largest block whose interval-start speed pass the check kernel's one CTA
// runs itself (128^2 cells); larger blocks keep the grid-wide speed pass.
// The separate pass costs a launch in every inner iteration, the check's
// one CTA a block-sized speed pass on one SM in the first iteration of an
// interval: on 8 x 8 blocks at 16 to 32 steps per interval the check won at
// 128^2 blocks (1024^2: 40.2 -> 38.4 us per iteration) and lost at 256^2
// (2048^2: 74.9 -> 76.5 us).
constexpr long long kLtsCheckSpeedCells = 128LL * 128LL;

// Work lists of a local-time-stepping iteration (DomainDev::ltsWork, ints),
// built by the last CTA of the check kernel: the enabled blocks (update pass)
// and the enabled blocks at the start of their interval (speed pass), each
// with the prefix sums of their (row tile, column) pairs, over which the
// pass's CTAs split the work evenly.  Arrival counters of the check and the
// update kernel in front.
constexpr int kLwArrCheck = 0, kLwArrUpd = 1, kLwNUpd = 2, kLwTotUpd = 3, kLwNSpd = 4, kLwTotSpd = 5, kLwHead = 8;
__host__ __device__ constexpr int ltsWorkInts(int nblocks) { return kLwHead + 4 * nblocks + 2; }
__host__ __device__ inline int *lwList(int *w, int nblocks, bool update) {
    return w + kLwHead + (update ? 0 : 2 * nblocks + 1);
}
__host__ __device__ inline int *lwPrefix(int *w, int nblocks, bool update) {
    return lwList(w, nblocks, update) + nblocks;
}

__device__ __forceinline__ float vmin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float vmax(float a, float b) { return (a < b) ? b : a; }

// ---------------------------------------------------------------------------
// Per-cell quantities shared by the four edges of a cell (f-wave / HLLE):
// h, normal momentum hn, b, u = hn/h, sqrt(h), sqrt(g h).  Dry cells keep
// their raw values; their derived values are never used.
// ---------------------------------------------------------------------------
struct Cell {
    float h, hn, b, u, sq, c;
};

__device__ __forceinline__ Cell makeCell(float h, float hn, float b, float u, float sq, float c) {
    Cell q;
    q.h = h; q.hn = hn; q.b = b; q.u = u; q.sq = sq; q.c = c;
    return q;
}

__device__ __forceinline__ void routeWave(float s, float zh, float zhu, float &hL, float &hR, float &huL, float &huR) {
    if (s < -kZeroTol) {
        hL += zh;
        huL += zhu;
    } else if (s > kZeroTol) {
        hR += zh;
        huR += zhu;
    } else {
        const float a = 0.5f * zh;
        const float c = 0.5f * zhu;
        hL += a;
        huL += c;
        hR += a;
        huR += c;
    }
}

// wet/dry pre-step of the f-wave and HLLE solvers: a dry side becomes the
// reflection of the wet side (a wall).  Returns false for a dry/dry edge.
__device__ __forceinline__ bool reflectDry(Cell &L, Cell &R, bool dryL, bool dryR) {
    if (dryL && dryR) return false;
    if (dryL) {
        L.h = R.h; L.hn = -R.hn; L.u = -R.u; L.sq = R.sq; L.c = R.c; L.b = R.b;
    } else if (dryR) {
        R.h = L.h; R.hn = -L.hn; R.u = -L.u; R.sq = L.sq; R.c = L.c; R.b = L.b;
    }
    return true;
}

/// wave speeds; fminf/fmaxf equal the (b < a ? b : a) selection of the CPU
/// restatement for every non-NaN input up to the sign of a zero, which no
/// later operation can observe
template <int S>
__device__ __forceinline__ void waveSpeeds(const Cell &L, const Cell &R, float &s1, float &s2) {
    const float uRoe = fmaf(L.u, L.sq, R.u * R.sq) / (L.sq + R.sq);
    const float cRoe = sqrtf(kG * (0.5f * (L.h + R.h)));
    if (S == SOLVER_FWAVE) {
        s1 = uRoe - cRoe;
        s2 = uRoe + cRoe;
    } else {
        s1 = fminf(L.u - L.c, uRoe - cRoe);
        s2 = fmaxf(R.u + R.c, uRoe + cRoe);
    }
}

/// share of a wave with speed s that goes to the left cell: 1, 0 or 1/2
/// (|s| <= zeroTol); the right cell gets 1 minus that.  Products with these
/// weights are exact, and a share of 0 adds a signed zero to a sum that
/// started at +0 (so never -0), which leaves it unchanged: the weighted sums
/// (0 + w1 z1) + w2 z2 equal the routing of the two waves in turn, bit for bit.
__device__ __forceinline__ float leftShare(float s) {
    return (s < -kZeroTol) ? 1.f : ((s > kZeroTol) ? 0.f : 0.5f);
}

/// the two f-waves of an edge with both sides wet (or a dry side reflected):
/// wave speeds, decomposition of the flux jump and routing.  SWEEP: the caller
/// only ever adds a left-going part to a right-going one (never -0: every such
/// sum starts at +0) or to +0, so a subsonic edge may hand out its left-going
/// parts without the + 0 that only turns -0 into +0
template <int S, bool SWEEP = false>
__device__ __forceinline__ void fhWaves(const Cell &L, const Cell &R, float &hUpdL, float &hUpdR, float &huUpdL,
                                        float &huUpdR, float &speed) {
    float s1, s2;
    waveSpeeds<S>(L, R, s1, s2);
    const float df1 = R.hn - L.hn;
    const float phiL = fmaf(L.hn, L.u, kHalfG * L.h * L.h);
    const float phiR = fmaf(R.hn, R.u, kHalfG * R.h * R.h);
    const float df2 = (phiR - phiL) + kHalfG * (L.h + R.h) * (R.b - L.b);
    const float rd = 1.f / (s2 - s1);
    const float beta1 = fmaf(s2, df1, -df2) * rd;
    const float beta2 = fmaf(-s1, df1, df2) * rd;
    const float z1u = beta1 * s1, z2u = beta2 * s2;
    // the routing of wave 1, then wave 2, into sums that start at +0
    if (s1 < -kZeroTol && s2 > kZeroTol) {  // subsonic: wave 1 left, wave 2 right
        hUpdL = SWEEP ? beta1 : 0.f + beta1;
        huUpdL = SWEEP ? z1u : 0.f + z1u;
        hUpdR = 0.f + beta2;
        huUpdR = 0.f + z2u;
    } else {
        const float w1 = leftShare(s1), w2 = leftShare(s2);
        hUpdL = (0.f + w1 * beta1) + w2 * beta2;
        hUpdR = (0.f + (1.f - w1) * beta1) + (1.f - w2) * beta2;
        huUpdL = (0.f + w1 * z1u) + w2 * z2u;
        huUpdR = (0.f + (1.f - w1) * z1u) + (1.f - w2) * z2u;
    }
    speed = fmaxf(fabsf(s1), fabsf(s2));
}

/// f-wave (S = SOLVER_FWAVE) or HLLE (S = SOLVER_HLLE) net updates of one
/// edge.  Wet/wet edges run straight through; an edge with a dry side takes
/// the (warp-uniform away from shorelines) reflection branch.
template <int S, bool SWEEP = false>
__device__ __forceinline__ void edgeFH(Cell L, Cell R, float &hUpdL, float &hUpdR, float &huUpdL, float &huUpdR,
                                       float &speed) {
    const bool dryL = L.h < kDryTol, dryR = R.h < kDryTol;
    if (!(dryL || dryR)) {
        fhWaves<S, SWEEP>(L, R, hUpdL, hUpdR, huUpdL, huUpdR, speed);
        return;
    }
    if (!reflectDry(L, R, dryL, dryR)) {
        hUpdL = 0.f; hUpdR = 0.f; huUpdL = 0.f; huUpdR = 0.f;
        speed = 0.f;
        return;
    }
    fhWaves<S>(L, R, hUpdL, hUpdR, huUpdL, huUpdR, speed);
    if (dryL) { hUpdL = 0.f; huUpdL = 0.f; }
    if (dryR) { hUpdR = 0.f; huUpdR = 0.f; }
}

/// max wave speed of one edge, bit-identical to edgeFH's `speed`
template <int S> __device__ __forceinline__ float edgeSpeedFH(Cell L, Cell R) {
    const bool dryL = L.h < kDryTol, dryR = R.h < kDryTol;
    if (dryL || dryR) {
        if (!reflectDry(L, R, dryL, dryR)) return 0.f;
    }
    float s1, s2;
    waveSpeeds<S>(L, R, s1, s2);
    return fmaxf(fabsf(s1), fabsf(s2));
}

// ---------------------------------------------------------------------------
// Augmented Riemann solver (George 2008): per-edge, same operation order as
// the CPU restatement it is tested against.
// ---------------------------------------------------------------------------
// The reference default-constructs its solvers (src/blocks/SWE_DimensionalSplittingMpi.hh:84-87)
// from the swe_solvers module, which is not part of the reference checkout,
// so these values cannot be checked against it.  They are those of the
// published augmented solver: George 2008's method as GeoClaw calls it
// (riemann_aug_JCP with a single Newton iteration for the middle state,
// tolerance 1e-6), with zeroTol (1e-7) and dryTol (0.01) above as the
// default-construction values of swe_solvers' solver classes.
struct AugRieParams {
    static constexpr float newtonTol = 1e-6f;
    static constexpr int maxNewton = 1;
    static constexpr float critTol = 1e-6f;
};

__device__ __forceinline__ void waveCurve(float h, float hK, float cK, float &f, float &df) {
    if (h > hK) {
        const float s = sqrtf(0.5f * kG * (1.f / h + 1.f / hK));
        f = (h - hK) * s;
        df = s - kG * (h - hK) / (4.f * h * h * s);
    } else {
        f = 2.f * (sqrtf(kG * h) - cK);
        df = sqrtf(kG / h);
    }
}

/// cL, cR: sqrt(g hL), sqrt(g hR), computed once by the caller
static __device__ __forceinline__ void middleState(float hL, float hR, float uL, float uR, float cL, float cR, float &hm,
                                                float &s1m, float &s2m, bool &rare1, bool &rare2) {
    if (hR < kDryTol) {
        hm = 0.f;
        const float front = uL + 2.f * cL;
        s1m = front; s2m = front; rare1 = true; rare2 = false;
        return;
    }
    if (hL < kDryTol) {
        hm = 0.f;
        const float front = uR - 2.f * cR;
        s1m = front; s2m = front; rare1 = false; rare2 = true;
        return;
    }
    const float cm = 0.5f * (cL + cR) + 0.25f * (uL - uR);
    if (cm <= 0.f) {
        hm = 0.f;
        s1m = uL + 2.f * cL; s2m = uR - 2.f * cR; rare1 = true; rare2 = true;
        return;
    }
    const float hRR = cm * cm / kG;
    float um;
    if (hRR <= vmin(hL, hR)) {
        hm = hRR;
        um = uL + 2.f * (cL - cm);
        rare1 = true; rare2 = true;
    } else {
        float h = hRR;
        for (int it = 0; it < AugRieParams::maxNewton; ++it) {
            float fL, dfL, fR, dfR;
            waveCurve(h, hL, cL, fL, dfL);
            waveCurve(h, hR, cR, fR, dfR);
            const float F = fL + fR + (uR - uL);
            if (fabsf(F) < AugRieParams::newtonTol) break;
            h = h - F / (dfL + dfR);
            if (h < kDryTol) {
                h = kDryTol;
                break;
            }
        }
        hm = h;
        float fL, dfL, fR, dfR;
        waveCurve(hm, hL, cL, fL, dfL);
        waveCurve(hm, hR, cR, fR, dfR);
        um = 0.5f * ((uL - fL) + (uR + fR));
        rare1 = hm <= hL;
        rare2 = hm <= hR;
    }
    const float cmid = sqrtf(kG * hm);
    s1m = um - cmid;
    s2m = um + cmid;
}

static __device__ __forceinline__ void edgeAugRie(float hL, float hR, float huL, float huR, float bL, float bR, float &hUpdL,
                                        float &hUpdR, float &huUpdL, float &huUpdR, float &speed) {
    const bool dryL = hL < kDryTol;
    const bool dryR = hR < kDryTol;
    hUpdL = 0.f; hUpdR = 0.f; huUpdL = 0.f; huUpdR = 0.f;
    if (dryL && dryR) {
        speed = 0.f;
        return;
    }
    float uL = 0.f, uR = 0.f;
    bool wallL = false, wallR = false;
    if (dryR) {
        uL = huL / hL;
        float hm, s1m, s2m;
        bool r1, r2;
        const float c = sqrtf(kG * hL);
        middleState(hL, hL, uL, -uL, c, c, hm, s1m, s2m, r1, r2);
        const float hTest = vmax(hL, hm);
        if (hTest + bL < bR) {
            wallR = true;
            hR = hL; huR = -huL; uR = -uL; bR = bL;
        } else {
            hR = 0.f; huR = 0.f;
        }
    } else if (dryL) {
        uR = huR / hR;
        float hm, s1m, s2m;
        bool r1, r2;
        const float c = sqrtf(kG * hR);
        middleState(hR, hR, -uR, uR, c, c, hm, s1m, s2m, r1, r2);
        const float hTest = vmax(hR, hm);
        if (hTest + bR < bL) {
            wallL = true;
            hL = hR; huL = -huR; uL = -uR; bL = bR;
        } else {
            hL = 0.f; huL = 0.f;
        }
    } else {
        uL = huL / hL;
        uR = huR / hR;
    }

    const float cL = sqrtf(kG * hL);
    const float cR = sqrtf(kG * hR);
    float hm, s1m, s2m;
    bool rare1, rare2;
    middleState(hL, hR, uL, uR, cL, cR, hm, s1m, s2m, rare1, rare2);

    const float sqL = sqrtf(hL);
    const float sqR = sqrtf(hR);
    const float uRoe = fmaf(uL, sqL, uR * sqR) / (sqL + sqR);
    const float cRoe = sqrtf(kG * (0.5f * (hL + hR)));
    const float sE1 = vmin(uL - cL, uRoe - cRoe);
    const float sE2 = vmax(uR + cR, uRoe + cRoe);
    const float l1 = vmin(sE1, s1m);
    const float l3 = vmax(sE2, s2m);

    const float hStarHLL = vmax((huL - huR + l3 * hR - l1 * hL) / (l3 - l1), 0.f);

    float l2 = 0.5f * (l1 + l3);
    bool corrector = false;
    if (rare1 && l1 < 0.f && s1m > 0.f) {
        l2 = s1m;
        corrector = true;
    } else if (rare2 && s2m < 0.f && l3 > 0.f) {
        l2 = s2m;
        corrector = true;
    }
    if (corrector && !(l1 < l2 && l2 < l3)) corrector = false;
    if (corrector && vmin(hL, hR) < kDryTol) corrector = false;
    if (!corrector) l2 = 0.5f * (l1 + l3);

    const float dh = hR - hL;
    const float dhu = huR - huL;
    const float phiL = fmaf(huL, uL, kHalfG * hL * hL);
    const float phiR = fmaf(huR, uR, kHalfG * hR * hR);
    const float dphi = phiR - phiL;
    const float db = bR - bL;

    const float critTol = AugRieParams::critTol;
    const float hbar = vmax(0.5f * (hL + hR), 0.f);
    const float uSum = uL + uR;
    const float s1s2bar = 0.25f * uSum * uSum - kG * hbar;
    const float s1s2tilde = vmax(0.f, uL * uR) - kG * hbar;

    bool sonic = false;
    if (fabsf(s1s2bar) <= critTol) sonic = true;
    if (s1s2bar * s1s2tilde <= critTol) sonic = true;
    if (s1s2bar * l1 * l3 <= critTol) sonic = true;
    if (vmin(fabsf(l1), fabsf(l3)) < critTol) sonic = true;
    if (l1 < 0.f && s1m > 0.f) sonic = true;
    if (l3 > 0.f && s2m < 0.f) sonic = true;
    if ((uL + cL) * (uR + cR) < 0.f) sonic = true;
    if ((uL - cL) * (uR - cR) < 0.f) sonic = true;

    float ddh = sonic ? -db : db * kG * hbar / s1s2bar;
    const float width = l3 - l1;
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
    float ddphi = sonic ? -kG * hbar * db : -db * kG * hbar * s1s2tilde / s1s2bar;
    const float pL = -hL * db;
    const float pR = -hR * db;
    ddphi = vmin(ddphi, kG * vmax(pL, pR));
    ddphi = vmax(ddphi, kG * vmin(pL, pR));

    const float d1 = dh - ddh;
    const float d2 = dhu;
    const float d3 = dphi - ddphi;

    float beta1, beta2, beta3;
    if (!corrector) {
        const float rd = 1.f / width;
        beta1 = fmaf(l3, d1, -d2) * rd;
        beta3 = fmaf(-l1, d1, d2) * rd;
        beta2 = d3 - l1 * (l1 * beta1) - l3 * (l3 * beta3);
    } else {
        beta1 = (l2 * l3 * d1 - (l2 + l3) * d2 + d3) / ((l1 - l2) * (l1 - l3));
        beta2 = (l1 * l3 * d1 - (l1 + l3) * d2 + d3) / ((l2 - l1) * (l2 - l3));
        beta3 = (l1 * l2 * d1 - (l1 + l2) * d2 + d3) / ((l3 - l1) * (l3 - l2));
    }
    routeWave(l1, beta1 * l1, beta1 * l1 * l1, hUpdL, hUpdR, huUpdL, huUpdR);
    if (corrector)
        routeWave(l2, beta2 * l2, beta2 * l2 * l2, hUpdL, hUpdR, huUpdL, huUpdR);
    else
        routeWave(l2, 0.f, beta2, hUpdL, hUpdR, huUpdL, huUpdR);
    routeWave(l3, beta3 * l3, beta3 * l3 * l3, hUpdL, hUpdR, huUpdL, huUpdR);

    if (wallL) { hUpdL = 0.f; huUpdL = 0.f; }
    if (wallR) { hUpdR = 0.f; huUpdR = 0.f; }
    speed = vmax(fabsf(l1), fabsf(l3));
}

/// the switch of the hybrid solver: augmented solver where either side is
/// shallower than 0.1 m, f-wave elsewhere
constexpr float kHybridSwitchDepth = 0.1f;

/// Full edge solve for any solver from per-cell quantities (SWEEP: see fhWaves).
template <int S, bool SWEEP = false>
__device__ __forceinline__ void edgeSolve(const Cell &L, const Cell &R, float &hUpdL, float &hUpdR, float &huUpdL,
                                          float &huUpdR, float &speed) {
    if (S == SOLVER_FWAVE || S == SOLVER_HLLE) {
        edgeFH<S, SWEEP>(L, R, hUpdL, hUpdR, huUpdL, huUpdR, speed);
    } else if (S == SOLVER_AUGRIE) {
        edgeAugRie(L.h, R.h, L.hn, R.hn, L.b, R.b, hUpdL, hUpdR, huUpdL, huUpdR, speed);
    } else {
        if (L.h < kHybridSwitchDepth || R.h < kHybridSwitchDepth)
            edgeAugRie(L.h, R.h, L.hn, R.hn, L.b, R.b, hUpdL, hUpdR, huUpdL, huUpdR, speed);
        else
            edgeFH<SOLVER_FWAVE, SWEEP>(L, R, hUpdL, hUpdR, huUpdL, huUpdR, speed);
    }
}

template <int S> __device__ __forceinline__ float edgeSpeed(const Cell &L, const Cell &R) {
    if (S == SOLVER_FWAVE || S == SOLVER_HLLE) {
        return edgeSpeedFH<S>(L, R);
    } else {
        float a, b, c, d, s;
        edgeSolve<S>(L, R, a, b, c, d, s);
        return s;
    }
}

} // namespace swegb
