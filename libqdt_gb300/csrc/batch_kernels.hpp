// Launchers of the batch engine's predicate kernels (batch_build.cu), built
// twice: qdtg::narrow without the widest exact tier (every call) and
// qdtg::wide with it (a batch run again when a predicate needed it).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace qdtg {

// heights of a set's tree (sets of at most 1e8 points)
constexpr int kMaxHeights = 28;

// the set of an element, from the offsets (binary search)
__host__ __device__ __forceinline__ uint32_t find_set(const uint32_t* __restrict__ off, int S, uint32_t i)
{
    int lo = 0, hi = S;   // off[lo] <= i < off[hi]
    while (hi - lo > 1)
    {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= i) lo = mid;
        else hi = mid;
    }
    return (uint32_t)lo;
}

// The persistent build's schedule: its work units, heights in increasing
// order (32 node slots a unit at the thread heights, one at the warp
// heights), and where each height's entries are.
struct PersistPlan
{
    int      nh;                          // heights
    uint32_t unit_off[kMaxHeights + 1];   // first unit of each height
    uint32_t ent0[kMaxHeights], eoff0[kMaxHeights];
    int      nent[kMaxHeights];
    uint8_t  warp[kMaxHeights];
};

// The device buffers the build and extraction kernels of a batch read and
// write (all owned by the batch engine's workspace).
struct BatchBuildArgs
{
    Rec*            recs = nullptr;
    int             nrec = 0;
    const double2*  V = nullptr;
    NodeOut*        nodes = nullptr;
    const uint32_t* noff = nullptr;
    const uint32_t* ents = nullptr;
    const uint32_t* eoffs = nullptr;
    const uint32_t* u_off = nullptr;
    const uint32_t* cell_off = nullptr;
    int             S = 0;
    int             cell_points = 0;
    uint32_t        ncells = 0;
    DevStatus*      status = nullptr;
    int             count = 0;   // count filter failures
    uint32_t*       counter = nullptr;   // persistent form: unit counter
    uint32_t*       done = nullptr;      // persistent form: per node slot
    const uint32_t* useg = nullptr;
    const uint8_t*  skip = nullptr;
    uint8_t*        mask = nullptr;
};

#define QDTG_BATCH_LAUNCHERS                                                                                   \
    void launch_bbuild_cells(const BatchBuildArgs& a, cudaStream_t s);                                         \
    void launch_bbuild_height(const BatchBuildArgs& a, int h, const uint32_t* en, const uint32_t* eo, int nent, \
        long long slots, bool warp, cudaStream_t s);                                                           \
    void launch_bbuild_persist(const BatchBuildArgs& a, const PersistPlan* plan, int grid, cudaStream_t s);    \
    int  persist_blocks_per_sm();                                                                              \
    void launch_btri_mask(const BatchBuildArgs& a, cudaStream_t s);

namespace narrow {
QDTG_BATCH_LAUNCHERS
}
namespace wide {
QDTG_BATCH_LAUNCHERS
}
#undef QDTG_BATCH_LAUNCHERS

}  // namespace qdtg
