// Host orchestration of the GB300 batch triangulation engine: device
// workspace, the stage sequence on the context's stream, and the transfers.
#include <cmath>
#include <cstring>
#include <new>
#include <thread>

#include "engine.hpp"
#include "engine_kernels.hpp"
#include "host_copy.hpp"
#include "scan.cuh"

namespace qdtg {

// status codes (qdt.h)
enum
{
    S_OK = 0,
    S_NOT_FINITE = -4,
    S_OOM = -10,
    S_INTERNAL = -11
};

struct HostSmall
{
    DevStatus st;
    uint32_t  words[8];   // [0] distinct points, [1] triangles
};

struct DeviceWork
{
    void*        block = nullptr;
    size_t       bytes = 0;
    size_t       cap = 0;      // capacity in points
    size_t       spare_cap = 0;   // spare records of the split merges
    PrepBuffers  prep;
    BuildBuffers build;
    double2*     pts = nullptr;
    uint32_t*    words = nullptr;   // device u32 words: [0] distinct, [1] triangles
    HostSmall*   hsmall = nullptr;  // pinned
};

namespace {

struct Carver
{
    char*  base;
    size_t off = 0;
    template <class T>
    T* take(size_t count)
    {
        off = (off + 255) & ~(size_t)255;
        T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
        off += count * sizeof(T);
        return p;
    }
};

// spare records (and deletion-list entries) of the split merges of N
// points: the default plan (seam segments included), and one segment a
// merge at every depth and node size the knobs allow. A call whose plan
// needs more (segments on deeper depths or smaller nodes) runs its merges
// with one segment.
size_t split_capacity(size_t N)
{
    SplitPlan  plan;
    const int  n = (int)std::min<size_t>(N, (size_t)INT32_MAX / 4);
    const auto a = (size_t)split_plan(n, kSplitDefaultDepth, kSplitDefaultPoints, kSplitMaxSegs, kSplitSegPoints, plan);
    const auto b = (size_t)split_plan(n, kSplitMaxDepth, kSplitFloor, 1, kSplitSegFloor, plan);
    return std::max(a, b);
}

size_t carve(DeviceWork& w, char* base, size_t N)
{
    Carver c{ base };
    const size_t tiles_words = sort_count_words(N);
    const int    D = split_levels((int)std::max<size_t>(N, 4));
    const size_t nodes = (size_t)1 << D;
    PrepBuffers& p = w.prep;
    BuildBuffers& b = w.build;
    w.pts = c.take<double2>(N);
    p.pts = w.pts;
    for (int i = 0; i < 2; ++i)
    {
        p.kx[i] = c.take<uint64_t>(N);
        p.ky[i] = c.take<uint64_t>(N);
        p.val[i] = c.take<uint32_t>(N);
        p.A[i] = c.take<uint32_t>(N);
        p.B[i] = c.take<uint32_t>(N);
        b.node[i] = c.take<NodeOut>(nodes);
    }
    p.counts = c.take<uint32_t>(tiles_words);
    p.offs = c.take<uint32_t>(tiles_words);
    const size_t sw = std::max(scan_scratch_words(3 * N), scan_scratch_words(tiles_words));
    p.scratch = c.take<uint32_t>(sw);
    p.uexcl = c.take<uint32_t>(N);
    p.head = c.take<uint32_t>(N);
    p.uid = c.take<uint32_t>(N);
    p.ucoord = c.take<double2>(N);
    p.rep = c.take<uint32_t>(N);
    p.side = c.take<uint8_t>(N);
    p.seam = c.take<double>((size_t)2 << kSeamDepth);
    b.seam = p.seam;
    p.box = c.take<unsigned long long>(4);
    b.box = p.box;
    p.V = c.take<double2>(N);
    p.vid = c.take<uint32_t>(N);
    p.status = c.take<DevStatus>(1);
    w.words = c.take<uint32_t>(8);
    p.status_u32 = w.words;
    const size_t spare = split_capacity(N);
    w.spare_cap = spare;
    b.recs = c.take<Rec>(3 * N + spare);
    b.V = p.V;
    b.vid = p.vid;
    b.tri_mask = c.take<uint8_t>(3 * N + spare);
    b.tri_off = c.take<uint32_t>(3 * N + spare);
    b.split.lists = c.take<int>(spare);
    b.seam_hist = c.take<unsigned long long>(((size_t)2 << kSplitMaxDepth) * kSeamBins);
    b.seam_near = c.take<unsigned long long>(((size_t)2 << kSplitMaxDepth) * kSeamBins * 2);
    b.scratch = p.scratch;
    b.tris = c.take<uint32_t>(6 * N + 3);
    b.tri_count = w.words + 1;
    b.status = p.status;
    return c.off + 256;
}

}  // namespace

int split_plan(int m, int max_depth, int min_points, int max_segs, int seg_points, SplitPlan& plan)
{
    plan.depth = -1;
    plan.spare0 = 3 * m;
    plan.spare = 0;
    min_points = std::max(min_points, kSplitFloor);
    long long base = 0;
    for (int d = 0; d <= std::min(max_depth, kSplitMaxDepth); ++d)
    {
        // the largest node of depth d
        const long long n = ((long long)m + (1ll << d) - 1) >> d;
        if (n < min_points) break;
        // one more segment (two more walkers) per seg_points points
        const int segs = (int)std::max<long long>(1, std::min<long long>(std::min(max_segs, kSplitMaxSegs),
                                                         1 + n / std::max(seg_points, kSplitSegFloor)));
        // each walker's records and deletion-list entries: about half the
        // seam's cross edges (3 sqrt(n) leaves room for clustered points; a
        // walker that runs out stops or frees its deleted edges first), and
        // with several segments twice that: a rising walker above the first
        // segment cannot free records while the others run, and a long seam
        // (heavy-tailed points: 4 times 3 sqrt(n)) would otherwise stop both
        // walkers of a segment
        const int per = ((int)(3.0 * std::sqrt((double)n)) + 128) * (segs > 1 ? 2 : 1);
        plan.per[d] = per;
        plan.segs[d] = segs;
        plan.base[d] = base;
        base += (long long)split_lists(segs) * per * (1ll << d);
        plan.depth = d;
    }
    plan.spare = (int)base;
    return plan.spare;
}

Engine* Engine::create(int* cuda_error)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
    {
        int count = 0;
        e = cudaGetDeviceCount(&count);
        if (e == cudaSuccess && count == 0) e = cudaErrorNoDevice;
    }
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        if (cuda_error) *cuda_error = (int)e;
        return nullptr;
    }
    Engine* g = new (std::nothrow) Engine();
    if (!g) return nullptr;
    g->device_ = dev;
    g->cell_points_ = tuning().cell_points;
    g->warp_nodes_ = tuning().single_warp_nodes;
    if (cudaStreamCreateWithFlags(&g->stream_, cudaStreamNonBlocking) != cudaSuccess)
    {
        cudaGetLastError();
        delete g;
        return nullptr;
    }
    for (auto& ev : g->ev_)
        cudaEventCreate(&ev);
    // the build's prefetch stream; without it the prefetch runs in line
    if (cudaStreamCreateWithFlags(&g->side_, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&g->fork_, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&g->join_, cudaEventDisableTiming) != cudaSuccess)
    {
        cudaGetLastError();
        if (g->side_) cudaStreamDestroy(g->side_);
        if (g->fork_) cudaEventDestroy(g->fork_);
        if (g->join_) cudaEventDestroy(g->join_);
        g->side_ = nullptr;
        g->fork_ = g->join_ = nullptr;
    }
    g->w_ = new (std::nothrow) DeviceWork();
    g->mirror_ = new (std::nothrow) MeshMirror();
    if (!g->w_ || !g->mirror_)
    {
        delete g;
        return nullptr;
    }
    if (cudaHostAlloc((void**)&g->w_->hsmall, sizeof(HostSmall), cudaHostAllocPortable) != cudaSuccess)
    {
        cudaGetLastError();
        delete g;
        return nullptr;
    }
    return g;
}

Engine::~Engine()
{
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    if (side_) cudaStreamSynchronize(side_);
    clear_graphs();
    if (w_)
    {
        if (w_->block) cudaFree(w_->block);
        if (w_->hsmall) cudaFreeHost(w_->hsmall);
        delete w_;
    }
    if (mirror_)
    {
        mirror_free(*mirror_);
        delete mirror_;
    }
    for (auto& ev : ev_)
        if (ev) cudaEventDestroy(ev);
    if (fork_) cudaEventDestroy(fork_);
    if (join_) cudaEventDestroy(join_);
    if (side_) cudaStreamDestroy(side_);
    if (stream_) cudaStreamDestroy(stream_);
}

Tuning& tuning()
{
    static Tuning t;
    return t;
}

size_t Engine::workspace_bytes(size_t n)
{
    DeviceWork w;
    return carve(w, nullptr, std::max<size_t>(n, 1024));
}

size_t Engine::bytes_after(size_t n) const
{
    if (w_->block && n <= w_->cap) return w_->bytes;
    size_t N = std::max<size_t>(n, 1024);
    if (w_->cap) N = std::max(N, w_->cap + w_->cap / 4);
    if (limit_ && workspace_bytes(N) > limit_) N = std::max<size_t>(n, 1024);
    return workspace_bytes(N);
}

size_t Engine::workspace_bytes() const { return w_->block ? w_->bytes : 0; }

void Engine::release_workspace()
{
    if (!w_->block) return;
    cudaSetDevice(device_);
    cudaStreamSynchronize(stream_);
    clear_graphs();
    cudaFree(w_->block);
    w_->block = nullptr;
    w_->cap = 0;
    w_->bytes = 0;
}

void Engine::set_workspace_limit(size_t bytes)
{
    limit_ = bytes;
    if (limit_ && w_->block && w_->bytes > limit_) release_workspace();
}

int Engine::ensure(size_t n)
{
    if (n <= w_->cap && w_->block) return S_OK;
    size_t N = std::max<size_t>(n, 1024);
    if (w_->cap) N = std::max(N, w_->cap + w_->cap / 4);
    if (limit_ && workspace_bytes(N) > limit_)
    {
        // grow to the exact size instead, or fail with the old workspace kept
        N = std::max<size_t>(n, 1024);
        if (workspace_bytes(N) > limit_) return S_OOM;
    }
    if (w_->block)
    {
        cudaStreamSynchronize(stream_);
        cudaFree(w_->block);
        w_->block = nullptr;
        w_->cap = 0;
    }
    clear_graphs();   // they hold pointers into the old workspace
    const size_t bytes = carve(*w_, nullptr, N);
    void*        blk = nullptr;
    if (cudaMalloc(&blk, bytes) != cudaSuccess)
    {
        cudaGetLastError();
        // retry at the exact size
        N = std::max<size_t>(n, 1024);
        const size_t b2 = carve(*w_, nullptr, N);
        if (cudaMalloc(&blk, b2) != cudaSuccess)
        {
            cudaGetLastError();
            return S_OOM;
        }
        w_->bytes = b2;
    }
    else
        w_->bytes = bytes;
    w_->block = blk;
    w_->cap = N;
    carve(*w_, static_cast<char*>(blk), N);
    return S_OK;
}

int Engine::build_mesh(size_t n, size_t T, MeshVec<int>& o2l, MeshVec<MeshVertex>& v, MeshVec<MeshHalfEdge>& h)
{
    if (!mesh_source_ || n != mesh_n_ || T != mesh_t_ || !w_ || !w_->block) return -1;
    if (cudaSetDevice(device_) != cudaSuccess)
    {
        cudaGetLastError();
        return -1;
    }
    return mesh_build_device(w_->build.tris, w_->pts, n, T, stream_, *mirror_, o2l, v, h);
}

bool Engine::activate()
{
    if (cudaSetDevice(device_) == cudaSuccess) return true;
    cudaGetLastError();
    return false;
}

const uint32_t* Engine::device_triangles() const { return w_ ? w_->build.tris : nullptr; }
const uint32_t* Engine::device_rep() const { return w_ ? w_->prep.rep : nullptr; }

// frames, split levels, leaf order, build, extraction: the stages after the
// host has read the distinct-point count m (stream order only, no host work)
void Engine::post_sync_work(size_t m, bool wide)
{
    cudaStream_t  s = stream_;
    PrepBuffers&  p = w_->prep;
    BuildBuffers& b = w_->build;
    // the bits of the stages before (read by the host already) or of a first
    // pass of the same call
    cudaMemsetAsync(&p.status->flags, 0, sizeof(unsigned), s);
    // the predicates' counters (the narrow pass's, for a wide one)
    cudaMemsetAsync(&p.status->pc[0], 0, sizeof(p.status->pc), s);
    launch_frames(p, m, s);
    launch_split(p, (int)m, s);
    launch_finalize(p, (int)m, s);
    mark(4);
    if (wide) wide::launch_build(b, (int)m, s);
    else narrow::launch_build(b, (int)m, s);
    mark(5);
    if (wide) wide::launch_extract(b, (int)m, s);
    else narrow::launch_extract(b, (int)m, s);
}

void Engine::clear_graphs() noexcept
{
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second.exec);
    graphs_.clear();
}

// A stage-timing event. Recorded on a capturing stream, a plain
// cudaEventRecord only orders the capture and is not replayed: the external
// flag makes it an event-record node of the graph.
void Engine::mark(int i)
{
    if (!timing_) return;
    if (capturing_)
        cudaEventRecordWithFlags(ev_[i], stream_, cudaEventRecordExternal);
    else
        cudaEventRecord(ev_[i], stream_);
}

template <class F>
void Engine::run_graph(std::pair<uint64_t, uint64_t> key, F&& work)
{
    cudaStream_t s = stream_;
    if (use_graphs_)
    {
        auto it = graphs_.find(key);
        if (it == graphs_.end())
        {
            if (graphs_.size() >= 32) clear_graphs();
            cudaGraph_t graph = nullptr;
            cudaGetLastError();   // an error left by an earlier call is not this one's
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess)
            {
                const int before = launch_counter();
                capturing_ = true;
                work();
                capturing_ = false;
                // a launch refused while recording: no graph, the launches
                // run directly below and report it
                const bool recorded = cudaGetLastError() == cudaSuccess;
                const int  added = launch_counter() - before;
                if (cudaStreamEndCapture(s, &graph) == cudaSuccess && graph)
                {
                    cudaGraphExec_t exec = nullptr;
                    if (recorded && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess)
                        it = graphs_.emplace(key, GraphEntry{ exec, added }).first;
                    cudaGraphDestroy(graph);
                }
                cudaGetLastError();
                launch_counter() = before;   // nothing ran during the capture
            }
            else
                cudaGetLastError();
        }
        if (it != graphs_.end())
        {
            if (cudaGraphLaunch(it->second.exec, s) == cudaSuccess)
            {
                launch_counter() += it->second.launches;   // the kernels recorded in the graph
                return;
            }
            cudaGetLastError();
        }
    }
    cudaGetLastError();
    work();
    if (cudaGetLastError() != cudaSuccess) launch_error_ = true;
}

// Engines running a call at this moment, process-wide. The build's seam
// prefetch beside the merges pays when one call has the GPU; beside other
// engines' calls (the server runs several) its full-GPU scans take SMs from
// their merges (serving at 800 requests/s: 89 -> 57 Mpts/s), so it then runs
// in line.
static std::atomic<int>& busy_engines()
{
    static std::atomic<int> n{ 0 };
    return n;
}

int Engine::pipeline(size_t n, bool host_io, uint32_t* host_tris, size_t host_tri_cap, uint32_t* host_rep)
{
    cudaStream_t s = stream_;
    PrepBuffers& p = w_->prep;
    BuildBuffers& b = w_->build;
    HostSmall*   hs = w_->hsmall;
    info_ = RunInfo();
    launch_error_ = false;
    info_.n = n;
    launch_counter() = 0;
    struct Busy
    {
        int others = busy_engines().fetch_add(1);
        ~Busy() { busy_engines().fetch_sub(1); }
    } busy;
    // keys, sort, distinct points: one graph per (input size, input array),
    // as run_device reads the caller's array in place. The array is 16-byte
    // aligned, so bit 0 set keeps these keys apart from the later stages'
    // (whose second word has its low four bits clear). The sort's pass count
    // is fixed, so the buffer it leaves the keys in (p.sorted, set at
    // capture) is the same on every replay.
    auto pre_sync = [&] {
        mark(1);
        cudaMemsetAsync(p.status, 0, sizeof(DevStatus), s);
        cudaMemsetAsync(w_->words, 0, 8 * sizeof(uint32_t), s);
        launch_keys(p, n, s);
        launch_sort_points(p, n, s);
        mark(2);
        launch_unique(p, n, s);
        mark(3);
    };
    run_graph({ ((uint64_t)n << 1) | (timing_ ? 1u : 0u), (uint64_t)(uintptr_t)p.pts | 1u }, pre_sync);
    cudaMemcpyAsync(&hs->st, p.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hs->words, w_->words, 8 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return S_INTERNAL;
    if (hs->st.flags & ST_NOT_FINITE) return S_NOT_FINITE;
    const size_t m = hs->words[0];
    info_.unique_points = m;
    b.count_filter = count_filter_ ? 1 : 0;
    b.cell_points = cell_points_;
    b.warp_nodes = warp_nodes_;
    b.side = (side_prefetch_ && busy.others == 0) ? side_ : nullptr;
    b.fork = fork_;
    b.join = join_;
    p.split_tail = split_tail_;
    // lattice-like input (most distinct points share x with another): the
    // narrow window (builder.cuh, kWinDefault)
    b.window = window_ ? window_ : (16ull * hs->words[2] > (unsigned long long)kTieWindow * m ? 1 : 2);
    info_.window = b.window;
    info_.wide = 0;
    info_.split_rerun = 0;
    // the top merges as split merges, except on lattice-like input (the
    // window-1 test above): there nearly every in-circle test is a tie, a
    // falling walker stops at its first, and the rising ones walk alone
    {
        int* lists = b.split.lists;
        if (split_depth_ >= 0 && b.window != 1)
        {
            split_plan((int)m, split_depth_, split_min_, split_segs_, split_seg_points_, b.split);
            // a plan beyond the workspace's spare records: one segment a merge
            if ((size_t)b.split.spare > w_->spare_cap)
                split_plan((int)m, split_depth_, split_min_, 1, split_seg_points_, b.split);
            if ((size_t)b.split.spare > w_->spare_cap) b.split.depth = -1;
        }
        else b.split.depth = -1;
        b.split.lists = lists;
    }
    info_.split_depth = b.split.depth;
    // the most seam segments of a split merge in the plan
    auto plan_segs = [&] {
        int sg = 0;
        for (int d = 0; d <= b.split.depth && d <= kSplitMaxDepth; ++d) sg = std::max(sg, b.split.segs[d]);
        return sg;
    };
    info_.split_segments = plan_segs();
    // the graph key's first word: m, and above it the plan's segments a
    // depth (3 bits each)
    static_assert(kSplitMaxSegs < 8 && 32 + 3 * (kSplitMaxDepth + 1) <= 64, "segments fit the graph key");
    auto key_of_m = [&] {
        uint64_t k = (uint64_t)m;
        for (int d = 0; d <= b.split.depth && d <= kSplitMaxDepth; ++d)
            k |= (uint64_t)(b.split.segs[d] & 7) << (32 + 3 * d);
        return k;
    };
    // the stages after the count depend only on m and the knobs: one CUDA
    // graph per such key (about 250 launches at 2.6 M points)
    auto knobs_of = [&](bool wide_kernels) {
        return ((uint64_t)(b.cell_points & 0x7FF) << 4) | ((uint64_t)b.window << 15) |
               ((uint64_t)b.count_filter << 17) | ((uint64_t)(timing_ ? 1 : 0) << 18) |
               ((uint64_t)(p.split_tail ? 1 : 0) << 19) | ((uint64_t)(uint32_t)b.warp_nodes << 20) |
               ((uint64_t)(b.side ? 1 : 0) << 52) | ((uint64_t)((b.split.depth + 1) & 0xF) << 53) |
               (wide_kernels ? (1ull << 57) : 0ull) | ((uint64_t)(plan_segs() & 7) << 58);
    };
    if (m >= 3)
    {
        // a counting call runs the kernels that count every predicate call
        // (the wide ones) from the start
        const bool counting = b.count_filter != 0;
        run_graph({ key_of_m(), knobs_of(counting) }, [&] { post_sync_work(m, counting); });
        info_.wide = counting ? 1 : 0;
    }
    else
    {
        if (timing_)
        {
            cudaEventRecord(ev_[4], s);
            cudaEventRecord(ev_[5], s);
        }
    }
    auto finish = [&] {
        if (timing_) cudaEventRecord(ev_[6], s);
        cudaMemcpyAsync(&hs->st, p.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hs->words, w_->words, 8 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        if (host_io)
        {
            // the triangle count is at most 2 m - 5: copy that bound, not a
            // round trip for the exact count
            const size_t bound = m >= 3 ? std::min<size_t>(2 * m, host_tri_cap) : 0;
            if (bound) cudaMemcpyAsync(host_tris, b.tris, 3 * bound * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
            if (n) cudaMemcpyAsync(host_rep, p.rep, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        }
        if (timing_) cudaEventRecord(ev_[7], s);
        return cudaStreamSynchronize(s) == cudaSuccess;
    };
    if (!finish()) return S_INTERNAL;
    // a split merge that could not finish: the stages after the count once
    // more, with one seam segment a merge when there were more (a walker
    // above the first segment met a zero predicate), else with one walker a
    // merge
    auto split_retry = [&] {
        info_.split_rerun = 1;
        if (plan_segs() > 1)
            for (int d = 0; d <= kSplitMaxDepth; ++d) b.split.segs[d] = std::min(b.split.segs[d], 1);
        else
        {
            b.split.depth = -1;
            info_.split_depth = -1;
        }
        info_.split_segments = plan_segs();
    };
    for (int tries = 0; m >= 3 && (hs->st.flags & ST_SPLIT) && b.split.depth >= 0 && tries < 2; ++tries)
    {
        split_retry();
        const bool w = info_.wide != 0;
        run_graph({ key_of_m(), knobs_of(w) }, [&] { post_sync_work(m, w); });
        if (!finish()) return S_INTERNAL;
    }
    bool wide = false;
    for (int sg = 0; sg < kPredStages; ++sg) wide = wide || hs->st.pc[sg].wide;
    if (m >= 3 && wide && !info_.wide)
    {
        // a predicate needed the widest exact tier, which the default
        // kernels leave out: the stages after the count once more with the
        // kernels that have it
        info_.wide = 1;
        run_graph({ key_of_m(), knobs_of(true) }, [&] { post_sync_work(m, true); });
        if (!finish()) return S_INTERNAL;
    }
    for (int tries = 0; m >= 3 && (hs->st.flags & ST_SPLIT) && b.split.depth >= 0 && tries < 2; ++tries)
    {
        // (a wide pass whose split merge failed)
        split_retry();
        run_graph({ key_of_m(), knobs_of(true) }, [&] { post_sync_work(m, true); });
        if (!finish()) return S_INTERNAL;
    }
    info_.launches = launch_counter();
    info_.device_status = (int)hs->st.flags;
    take_pred_stats(info_, hs->st);
    info_.ntri = m >= 3 ? hs->words[1] : 0;
    if (launch_error_ || (hs->st.flags & (ST_POOL_EMPTY | ST_GUARD | ST_BAD_INDEX | ST_SPLIT))) return S_INTERNAL;
    if (timing_)
    {
        auto el = [&](int a, int z) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev_[a], ev_[z]);
            return ms;
        };
        info_.ms.keys_sort = el(1, 2);
        info_.ms.unique = el(2, 3);
        info_.ms.split = el(3, 4);
        info_.ms.build = el(4, 5);
        info_.ms.extract = el(5, 6);
        info_.ms.d2h = el(6, 7);
    }
    return S_OK;
}

int Engine::run_host(const double* xy, size_t n, PinnedVec<double>& points, PinnedVec<uint32_t>& tris, size_t* ntri,
    PinnedVec<uint32_t>& rep, size_t* unique_points)
{
    if (cudaSetDevice(device_) != cudaSuccess)
    {
        cudaGetLastError();
        return S_INTERNAL;
    }
    mesh_source_ = false;
    int st = ensure(n);
    if (st != S_OK) return st;
    // host copies the caller's points into the context (pinned) in chunks; the
    // upload of a chunk overlaps the copy of the next one
    // room for later insertions: growing a page-locked vector reallocates
    // and re-pins it
    const size_t room = n + std::max<size_t>(n / 16, 1024);
    if (points.capacity() < 2 * n) points.reserve(2 * room);
    if (rep.capacity() < n) rep.reserve(room);
    points.resize(2 * n);
    rep.resize(n);
    tris.resize(6 * n + 3);
    if (timing_) cudaEventRecord(ev_[0], stream_);
    const size_t chunk = (size_t)1 << 20;   // points per chunk (16 MiB), each copied by the host pool
    for (size_t off = 0; off < n; off += chunk)
    {
        const size_t c = std::min(chunk, n - off);
        parallel_copy(points.data() + 2 * off, xy + 2 * off, c * 2 * sizeof(double));
        cudaMemcpyAsync(w_->pts + off, points.data() + 2 * off, c * sizeof(double2), cudaMemcpyHostToDevice,
            stream_);
    }
    st = pipeline(n, true, tris.data(), (6 * n + 3) / 3, rep.data());
    if (st != S_OK) return st;
    if (timing_)
    {
        float ms = 0;
        cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
        info_.ms.h2d = ms;
        cudaEventElapsedTime(&ms, ev_[0], ev_[7]);
        info_.ms.total = ms;
    }
    *ntri = info_.ntri;
    *unique_points = info_.unique_points;
    tris.resize(3 * info_.ntri);
    // the points and triangles stay on the device until the next call: the
    // first insertion or constraint builds its mesh from them
    mesh_source_ = true;
    mesh_n_ = n;
    mesh_t_ = info_.ntri;
    return S_OK;
}

int Engine::run_device(const double* d_xy, size_t n, cudaStream_t user_stream)
{
    mesh_source_ = false;
    if (cudaSetDevice(device_) != cudaSuccess)
    {
        cudaGetLastError();
        return S_INTERNAL;
    }
    int st = ensure(n);
    if (st != S_OK) return st;
    if (user_stream)
    {
        // order after the caller's work on its stream
        cudaEventRecord(ev_[8], user_stream);
        cudaStreamWaitEvent(stream_, ev_[8], 0);
    }
    if (timing_) cudaEventRecord(ev_[0], stream_);
    // read the caller's device array in place when it allows 16-byte loads
    if (((uintptr_t)d_xy & 15) == 0)
        w_->prep.pts = reinterpret_cast<const double2*>(d_xy);
    else if (n)
        cudaMemcpyAsync(w_->pts, d_xy, n * sizeof(double2), cudaMemcpyDeviceToDevice, stream_);
    st = pipeline(n, false, nullptr, 0, nullptr);
    w_->prep.pts = w_->pts;
    if (st == S_OK && timing_)
    {
        float ms = 0;
        cudaEventElapsedTime(&ms, ev_[0], ev_[7]);
        info_.ms.total = ms;
    }
    return st;
}

}  // namespace qdtg
