// The GB300 batch triangulation engine: owns one CUDA stream and the device
// workspace of one context, runs the kernel stages, and leaves the result in
// host buffers of the context.
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <memory>
#include <new>
#include <map>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "common.cuh"
#include "mesh_layout.hpp"
#include "mesh_mirror.hpp"

namespace qdtg {

// Allocator for host buffers that the GPU copies to and from: page-locked
// memory (cudaHostAlloc), and default-initialisation so that resize() does not
// clear memory that a copy overwrites anyway. Where page-locked memory cannot
// be had (no usable GPU: a context that only holds a loaded triangulation and
// edits it on the host) it falls back to ordinary heap memory; a 64-byte
// header in front of each block records which.
template <class T>
struct PinnedAllocator
{
    using value_type = T;
    static constexpr size_t kHeader = 64;
    PinnedAllocator() = default;
    template <class U>
    PinnedAllocator(const PinnedAllocator<U>&) noexcept
    {
    }
    T* allocate(size_t n)
    {
        if (n > (SIZE_MAX - kHeader) / sizeof(T)) throw std::bad_alloc();
        const size_t bytes = kHeader + (n ? n : 1) * sizeof(T);
        void*        p = nullptr;
        unsigned char kind = 1;
        if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) != cudaSuccess)
        {
            cudaGetLastError();
            p = std::aligned_alloc(kHeader, (bytes + kHeader - 1) / kHeader * kHeader);
            if (!p) throw std::bad_alloc();
            kind = 2;
        }
        *static_cast<unsigned char*>(p) = kind;
        return reinterpret_cast<T*>(static_cast<unsigned char*>(p) + kHeader);
    }
    void deallocate(T* p, size_t) noexcept
    {
        if (!p) return;
        unsigned char* base = reinterpret_cast<unsigned char*>(p) - kHeader;
        if (*base == 1) cudaFreeHost(base);
        else std::free(base);
    }
    template <class U>
    void construct(U* p) noexcept
    {
        ::new (static_cast<void*>(p)) U;
    }
    template <class U, class... A>
    void construct(U* p, A&&... a)
    {
        ::new (static_cast<void*>(p)) U(static_cast<A&&>(a)...);
    }
    template <class U>
    bool operator==(const PinnedAllocator<U>&) const noexcept
    {
        return true;
    }
    template <class U>
    bool operator!=(const PinnedAllocator<U>&) const noexcept
    {
        return false;
    }
};

template <class T>
using PinnedVec = std::vector<T, PinnedAllocator<T>>;

struct StageTimes
{
    float h2d = 0, keys_sort = 0, unique = 0, split = 0, build = 0, extract = 0, d2h = 0, total = 0;
};

// Predicate statistics of one stage (common.cuh PredCounters)
struct PredStats
{
    unsigned long long calls[2] = { 0, 0 }, f32_undecided[2] = { 0, 0 }, exact[2] = { 0, 0 };
};

struct RunInfo
{
    size_t                 n = 0, unique_points = 0, ntri = 0;
    unsigned long long     orient_exact = 0, incircle_exact = 0;   // sums over the stages
    PredStats              stage[kPredStages];
    StageTimes             ms;
    int                    device_status = 0;
    int                    launches = 0;
    int                    window = 0;   // warp merges' candidate window of the last call
    int                    wide = 0;     // the build ran again with the widest exact tier
    int                    split_depth = -1;   // deepest depth merged as split merges (-1: none)
    int                    split_rerun = 0;    // a split merge failed and the build ran again (fewer segments, or without them)
    int                    split_segments = 0; // the most seam segments of a split merge in the last pass
};

struct DeviceWork;

// copies the predicate statistics of a call's device status into its RunInfo
inline void take_pred_stats(RunInfo& info, const DevStatus& st)
{
    info.orient_exact = info.incircle_exact = 0;
    for (int s = 0; s < kPredStages; ++s)
    {
        for (int k = 0; k < 2; ++k)
        {
            info.stage[s].calls[k] = st.pc[s].calls[k];
            info.stage[s].f32_undecided[k] = st.pc[s].f32_undecided[k];
            info.stage[s].exact[k] = st.pc[s].exact[k];
        }
        info.orient_exact += st.pc[s].exact[0];
        info.incircle_exact += st.pc[s].exact[1];
    }
}

// device bytes of a many-set workspace for N points in S sets (batch.cu)
size_t bcarve_bytes(size_t N, size_t S);

// Process-wide defaults of the schedule knobs, read when a context, batch or
// server is created (qdtg_set_defaults; the autotuner sets them).
// Atomic fields: a thread may set the defaults while another creates a
// context.
struct Tuning
{
    std::atomic<int> cell_points{ 0 };              // single set: shared-memory cells (0: none)
    std::atomic<int> batch_cell_points{ 0 };        // many sets: the same
    std::atomic<int> single_warp_nodes{ 4096 };     // single set: depths of at most this many nodes merge with a warp per node
    std::atomic<int> batch_warp_min_points{ 512 };  // many sets: heights whose nodes have at least this many points, a warp per node
    std::atomic<int> batch_warp_nodes{ 4096 };      // many sets: also heights with at most this many nodes
    std::atomic<int> server_large_workers{ 4 };     // serving: engines for large requests
};
Tuning& tuning();

class Engine
{
public:
    // nullptr when no usable CUDA device is present
    static Engine* create(int* cuda_error);
    ~Engine();

    // Triangulates n host points (already validated for count and NULL).
    // Copies them into `points` (the context's copy), uploads them, runs the
    // stages and downloads triangles and representatives.
    // Returns a qdt_status value (QDT_OK, QDT_ERR_NOT_FINITE,
    // QDT_ERR_OUT_OF_MEMORY, QDT_ERR_INTERNAL).
    int run_host(const double* xy, size_t n, PinnedVec<double>& points, PinnedVec<uint32_t>& tris,
        size_t* ntri, PinnedVec<uint32_t>& rep, size_t* unique_points);

    // Triangulates n points already resident on the device. Triangles stay on
    // the device (device_triangles()). Returns a qdt_status value.
    int run_device(const double* d_xy, size_t n, cudaStream_t user_stream);

    // Device bytes of the workspace for n points, and the bytes the
    // workspace would hold after run_host / run_device on n points (it grows
    // by at least a quarter when it grows).
    static size_t workspace_bytes(size_t n);
    size_t        bytes_after(size_t n) const;
    size_t        workspace_bytes() const;
    // frees the workspace (the next call allocates it again)
    void          release_workspace();
    // caps the workspace's device bytes (0: none); a call that needs more
    // returns QDT_ERR_OUT_OF_MEMORY; a workspace above a new cap is freed
    void          set_workspace_limit(size_t bytes);

    // The half-edge mesh of the last run_host result (n points, T triangles),
    // built on the device (k_mesh.cu). Returns 0, or a negative value when
    // the device no longer holds that result or the build failed (the caller
    // then builds the mesh on the host).
    int build_mesh(size_t n, size_t T, MeshVec<int>& o2l, MeshVec<MeshVertex>& v, MeshVec<MeshHalfEdge>& h);

    // The device copy of the handle's mesh for batch point location
    // (mesh_mirror.hpp); build_mesh fills it. Calls on it run on stream().
    MeshMirror& mirror() { return *mirror_; }
    // makes this engine's device current; false on failure
    bool        activate();

    const uint32_t* device_triangles() const;
    const uint32_t* device_rep() const;
    size_t          last_ntri() const { return info_.ntri; }
    size_t          last_unique() const { return info_.unique_points; }
    const RunInfo&  info() const { return info_; }
    cudaStream_t    stream() const { return stream_; }
    void            set_count_filter(bool on) { count_filter_ = on; }
    void            set_timing(bool on) { timing_ = on; }
    void            set_cell_points(int c) { cell_points_ = c; }
    int             cell_points() const { return cell_points_; }
    void            set_warp_nodes(int n) { warp_nodes_ = n; }
    // 0: chosen per call from the input (lattice-like: 1, else 2); 1 or 2: fixed
    void            set_merge_window(int w) { window_ = w; }
    // replay the stages after the distinct-point count from a CUDA graph per
    // (count, knobs) (default on)
    void            set_use_graphs(bool on) { use_graphs_ = on; }
    // run the split depths of nodes of at most 4,096 points in one
    // shared-memory launch (default on)
    void            set_split_tail(bool on) { split_tail_ = on; }
    // the build's seam prefetch on a second stream beside the merges, when
    // no other engine is running a call (default on)
    void            set_side_prefetch(bool on) { side_prefetch_ = on; }
    // merges of depth at most max_depth whose nodes hold at least min_points
    // points run as split merges (seam_split.cuh); max_depth -1: none
    void            set_split(int max_depth, int min_points)
    {
        split_depth_ = max_depth;
        split_min_ = min_points;
    }
    // seam segments of one split merge at most (1..kSplitMaxSegs), one more
    // per seg_points points of the node: segments beyond the first begin at
    // cross edges found before the merge
    void            set_split_segments(int segs, int seg_points)
    {
        split_segs_ = segs;
        split_seg_points_ = seg_points;
    }
    int             warp_nodes() const { return warp_nodes_; }

private:
    Engine() = default;
    int  ensure(size_t n);
    int  pipeline(size_t n, bool host_io, uint32_t* host_tris, size_t host_tri_cap, uint32_t* host_rep);
    void post_sync_work(size_t m, bool wide);
    void clear_graphs() noexcept;
    // runs work() on stream(): replayed from the graph cached under key, or
    // captured into one first; launch by launch when graphs are off or fail
    template <class F>
    void run_graph(std::pair<uint64_t, uint64_t> key, F&& work);
    void mark(int i);   // records stage-timing event i when timing is on

    struct GraphEntry
    {
        cudaGraphExec_t exec;
        int             launches;
    };

    int             device_ = 0;
    cudaStream_t    stream_ = nullptr;
    cudaStream_t    side_ = nullptr;   // the build's seam prefetch beside the merges
    cudaEvent_t     fork_ = nullptr, join_ = nullptr;
    DeviceWork*     w_ = nullptr;
    RunInfo         info_;
    bool            count_filter_ = false;
    bool            timing_ = false;
    int             cell_points_ = 0;
    int             warp_nodes_ = 4096;
    int             window_ = 0;
    bool            mesh_source_ = false;   // the device holds the last run_host's points and triangles
    size_t          mesh_n_ = 0, mesh_t_ = 0;
    MeshMirror*     mirror_ = nullptr;
    bool            use_graphs_ = true;
    bool            split_tail_ = true;
    bool            side_prefetch_ = true;
    int             split_depth_ = kSplitDefaultDepth;
    int             split_min_ = kSplitDefaultPoints;
    int             split_segs_ = kSplitMaxSegs;
    int             split_seg_points_ = kSplitSegPoints;
    size_t          limit_ = 0;   // workspace bytes cap (0: none)
    bool            capturing_ = false;   // run_graph is recording stream_
    bool            launch_error_ = false; // a launch of this call failed (the call reports QDT_ERR_INTERNAL)
    std::map<std::pair<uint64_t, uint64_t>, GraphEntry> graphs_;   // for the current workspace
    cudaEvent_t     ev_[10] = {};
};

}  // namespace qdtg
