// Host-side launchers of the engine's kernel stages (one translation unit per
// stage group, compiled in parallel).
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "common.cuh"
#include "mesh_layout.hpp"
#include "mesh_mirror.hpp"

namespace qdtg {

struct PrepBuffers
{
    const double2* pts = nullptr;       // n input points (device)
    uint64_t*      kx[2] = { nullptr, nullptr };
    uint64_t*      ky[2] = { nullptr, nullptr };
    uint32_t*      val[2] = { nullptr, nullptr };
    int            sorted = 0;          // which ping-pong half holds sort 1's result
    uint32_t*      counts = nullptr;    // radix digit counts, 256 per tile
    uint32_t*      offs = nullptr;
    uint32_t*      scratch = nullptr;   // scan scratch
    uint32_t*      uexcl = nullptr;     // n: exclusive scans (unique numbering, split ranks)
    uint32_t*      head = nullptr;      // m: sorted position of each distinct point's first copy
    uint32_t*      uid = nullptr;       // m: input index of each distinct point
    double2*       ucoord = nullptr;    // m: coordinates of each distinct point, (x, y) order
    uint32_t*      rep = nullptr;       // n
    uint32_t*      A[2] = { nullptr, nullptr };
    uint32_t*      B[2] = { nullptr, nullptr };
    int            acur = 0, bcur = 0;
    bool           split_tail = true;   // the depths of small nodes in one shared-memory launch
    uint8_t*       side = nullptr;      // m
    double*        seam = nullptr;      // 2^(kSeamDepth+1): cut coordinate per upper node
    unsigned long long* box = nullptr;  // 4: bounding box of the points as order keys (min x, min y, max x, max y)
    double2*       V = nullptr;         // m, leaf order
    uint32_t*      vid = nullptr;       // m
    DevStatus*     status = nullptr;
    uint32_t*      status_u32 = nullptr;   // [0] = number of distinct points
};

struct BuildBuffers
{
    Rec*           recs = nullptr;      // 3 m records, then the split merges' spare ones
    const double2* V = nullptr;
    const uint32_t* vid = nullptr;
    NodeOut*       node[2] = { nullptr, nullptr };   // ping-pong per level, 2^D entries
    uint8_t*       tri_mask = nullptr;  // 3 m
    uint32_t*      tri_off = nullptr;   // 3 m
    uint32_t*      scratch = nullptr;
    uint32_t*      tris = nullptr;      // 3 * (2 m) output indices
    uint32_t*      tri_count = nullptr; // device word
    DevStatus*     status = nullptr;
    const double*  seam = nullptr;      // cut coordinates of the upper nodes (PrepBuffers::seam)
    const unsigned long long* box = nullptr;   // PrepBuffers::box
    int            count_filter = 0;    // count filter failures in status
    int            cell_points = 0;     // largest cell built in shared memory (0: no cells)
    int            warp_nodes = 4096;   // depths with at most this many nodes: a warp per node
    int            window = 2;          // the warp merges' candidate window (1 or 2)
    // a second stream for the seam prefetch of the next depth beside the
    // merges of this one (none: the prefetch runs in line)
    cudaStream_t   side = nullptr;
    cudaEvent_t    fork = nullptr, join = nullptr;
    SplitPlan      split;               // the top merges as split merges (depth -1: none)
    unsigned long long* seam_hist = nullptr; // kSeamBins per node of the split depths (2^(kSplitMaxDepth+1) nodes)
    // per node of the split depths, bin along the seam and side: the
    // half-edge leaving the vertex nearest to the cut (distance as float
    // bits above, half-edge below; all ones: none)
    unsigned long long* seam_near = nullptr;
};

// The split merges of m points: depths 0.. at most max_depth whose nodes
// hold at least min_points (>= kSplitFloor); plan.spare0 = 3 m, lists left
// to the caller. Returns the spare records (also plan.spare).
int split_plan(int m, int max_depth, int min_points, int max_segs, int seg_points, SplitPlan& plan);

// Distinct points sharing x with their predecessor in (x, y) order above
// this fraction (in 1/16) make the warp merges use a window of one
// candidate (integer lattices, snapped grids).
constexpr int kTieWindow = 8;

// Single-set build: depths whose nodes hold at least this many points merge
// with a warp per node whatever the warp-node threshold (m >> d points).
constexpr int kWarpMinPoints = 192;

size_t sort_count_words(size_t n);
int    split_levels(int m);

void launch_keys(const PrepBuffers& b, size_t n, cudaStream_t s);
void launch_sort_points(PrepBuffers& b, size_t n, cudaStream_t s);
void launch_unique(const PrepBuffers& b, size_t n, cudaStream_t s);
void launch_frames(PrepBuffers& b, size_t m, cudaStream_t s);
void launch_split(PrepBuffers& b, int m, cudaStream_t s);
void launch_finalize(const PrepBuffers& b, int m, cudaStream_t s);

// the half-edge mesh of T triangles (3 T point indices) over n points, both on
// the device, into host arrays (k_mesh.cu); the vertices and half-edges stay
// in the mirror as well. 0 or a negative value
int mesh_build_device(const uint32_t* tris, const double2* pts, size_t n, size_t T, cudaStream_t s,
    MeshMirror& mir, MeshVec<int>& o2l, MeshVec<MeshVertex>& v, MeshVec<MeshHalfEdge>& h);

// builds every level from the deepest to the root, then extracts the
// triangles: narrow, the kernels without the widest exact tier (every call);
// wide, with it (a call whose predicates needed it, run again)
namespace narrow {
void launch_build(const BuildBuffers& b, int m, cudaStream_t s);
void launch_extract(const BuildBuffers& b, int m, cudaStream_t s);
}  // namespace narrow
namespace wide {
void launch_build(const BuildBuffers& b, int m, cudaStream_t s);
void launch_extract(const BuildBuffers& b, int m, cudaStream_t s);
}  // namespace wide

}  // namespace qdtg
