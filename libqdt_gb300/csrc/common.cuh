// Shared device-side types of the GB300 batch triangulation engine.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace qdtg {

// One undirected edge of the planar map (the reference's quad-edge record,
// builder.hxx:82-86, holds onext of its four rotations). Here the map is kept
// as two directed half-edges per record, each linked into the ring of edges
// around its origin in both directions: next = onext (counter-clockwise),
// prev = oprev (clockwise). That is the same planar map: every query the
// builder makes -- onext, oprev, lnext = oprev(sym), rprev = onext(sym), org,
// dest -- has the same answer, but the dual (face) rings are implicit, so
// making and deleting an edge are ring insertions and removals of a couple of
// dependent loads instead of four-way splices over the rotations.
// Half-edge id = 2 * record + direction; sym(e) = e ^ 1.
// A record is 64 bytes, aligned, and also carries the coordinates of its two
// origins: a vertex never moves and an edge's origin is set once, when the
// edge is made, so the copies stay valid; they spare the merge a dependent
// load of the vertex array after every record load.
struct __align__(16) Rec
{
    int     next[2];   // onext of half-edges 2k, 2k+1
    int     prev[2];   // oprev of half-edges 2k, 2k+1
    int     org[2];    // origins; org[0] = -1 marks a dead record
    int     link;      // free-list link while the record is dead
    int     pad;
    double2 p[2];      // coordinates of org[0], org[1]
};

// Per-node state handed from a level to its parent level: the two hull edges
// the reference's build() returns (builder.hxx:303-348), and the node's free
// list of dead records (head, tail; -1 when empty). le2, re2: the same two
// edges in the other frame (the one the node itself merged in), from which
// the parent finds its own extremes without walking its hull.
struct __align__(16) NodeOut
{
    int le, re;
    int fhead, ftail;
    int le2, re2;
    int pad0, pad1;
};

// Device status word: bit flags; 0 means fine.
enum StatusBits : unsigned
{
    ST_NOT_FINITE = 1u,      // an input coordinate is NaN or infinite
    ST_POOL_EMPTY = 2u,      // a node's free list ran dry (cannot happen with a sound 3n bound)
    ST_GUARD = 4u,           // a loop exceeded its iteration guard (internal error)
    ST_BAD_INDEX = 8u,       // an index left its node's range (internal error)
    ST_SPLIT = 16u,          // a split merge could not finish: the call runs again without them
};

// Predicate statistics of one stage of a call ([0] orient2d, [1] in-circle):
// calls, calls the float pre-filter left undecided, calls the double filter
// left undecided as well (the exact evaluation ran). They are counted only
// when the kernel passes its pointer tagged (bit 0 set, pred_stage()).
// `wide` is set by a predicate that needed the widest exact tier in kernels
// built without it (predicates.cuh).
struct PredCounters
{
    unsigned long long calls[2], f32_undecided[2], exact[2];
    unsigned           wide, pad;
};

// The stages the statistics are split by: leaves (2-3 points), merges of a
// thread per node (and shared-memory cells), merges of a warp per node, and
// the extraction's orientation test.
enum PredStage : int
{
    kStageLeaf = 0,
    kStageThread = 1,
    kStageWarp = 2,
    kStageExtract = 3,
    kPredStages = 4,
};

struct DevStatus
{
    unsigned     flags;
    unsigned     pad;
    PredCounters pc[kPredStages];
};

// The counters of one stage, tagged when the call counts
__host__ __device__ inline PredCounters* pred_stage(DevStatus* st, int stage, int count)
{
    return reinterpret_cast<PredCounters*>(reinterpret_cast<uintptr_t>(&st->pc[stage]) | (count ? 1u : 0u));
}

// Depths whose seams (cut coordinates) are recorded during the split, and whose
// seam records are prefetched into L2 before they merge.
constexpr int kSeamDepth = 10;

// Split merges (seam_split.cuh): at most these depths (their children's cuts
// are recorded), nodes of at least kSplitFloor points.
constexpr int kSplitMaxDepth = 9;
constexpr int kSplitFloor = 256;
constexpr int kSplitDefaultDepth = 7;
constexpr int kSplitDefaultPoints = 1024;
// segments of one split merge's seam at most (two walkers each), and the
// default node size per added segment (floor kSplitSegFloor). The block of
// a split merge is its walker warps and an inserter warp; an SM's four
// sub-partitions hold 16,384 registers each and a block's warps are spread
// over them, so its 11 warps (3 on a sub-partition) get 168 registers a
// thread (k_build_split's cap). Measured against 3 segments at 232
// registers (7 warps, no spills): 2.6 M uniform 24.94 -> 23.71 ms a call
// with 4 segments despite the spills, 22.78 ms with 5.
constexpr int kSplitMaxSegs = 5;
constexpr int kSplitSegPoints = 16384;
constexpr int kSplitSegFloor = 1024;
// deletion lists (and spare-record ranges) of one split merge: one a
// walker, and with more than one segment one for the edges deleted before
// the walkers start
__host__ __device__ inline int split_lists(int segs) { return 2 * segs + (segs > 1 ? 1 : 0); }
// bins of the records near a split merge's seam, along it (where its two
// walkers meet)
constexpr int kSeamBins = 64;

// The split merges of one call: depths 0..depth, each walker of a node of
// depth d with per[d] spare records (ids spare0 + base[d] + 2 per[d] k + w
// per[d], w = 0 rising, 1 falling) and as many deletion-list entries (lists
// + the same offset); spare records in all.
struct SplitPlan
{
    int       depth = -1;
    int       spare0 = 0;
    int       spare = 0;
    int       per[kSplitMaxDepth + 1] = {};    // spare records (and deletion-list entries) of one walker
    int       segs[kSplitMaxDepth + 1] = {};   // seam segments of a merge at most (2 walkers each)
    long long base[kSplitMaxDepth + 1] = {};
    int*      lists = nullptr;
};

// Largest cell (points) built in shared memory: 6 * kCellMax half-edge ids
// fit in the 16-bit ids of the cell's records.
constexpr int kCellMax = 1024;

// The Dwyer split tree depends only on the number m of distinct points: the
// root covers [0, m); a node [lo, hi) of at least 4 points splits at
// lo + (hi - lo) / 2 (reference builder.hxx:306-308). Depth d, heap-style
// index k (bit d-1-l of k = the branch taken at depth l).
// Returns false when the node does not exist (an ancestor is a leaf).
__host__ __device__ inline bool node_range(int m, int d, long long k, int& lo, int& hi)
{
    lo = 0;
    hi = m;
    for (int l = 0; l < d; ++l)
    {
        if (hi - lo < 4) return false;
        const int mid = lo + (hi - lo) / 2;
        if ((k >> (d - 1 - l)) & 1) lo = mid;
        else hi = mid;
    }
    return true;
}

// The node at depth <= d that contains position i: stops early at a leaf.
// Returns the depth reached.
__host__ __device__ inline int node_of(int m, int d, int i, int& lo, int& hi)
{
    lo = 0;
    hi = m;
    for (int l = 0; l < d; ++l)
    {
        if (hi - lo < 4) return l;
        const int mid = lo + (hi - lo) / 2;
        if (i < mid) hi = mid;
        else lo = mid;
    }
    return d;
}

// Kernels launched by the calling host thread (the engine resets it per call
// and reports it).
inline int& launch_counter()
{
    static thread_local int c = 0;
    return c;
}

}  // namespace qdtg
