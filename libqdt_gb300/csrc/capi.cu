// The C interface (include/qdt.h, include/qdt_gpu.h): input checks, status
// codes, reset-on-failure, queries. Mirrors the reference shim
// (libqdt/qdt.cpp) function by function; no C++ exception crosses it.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <iterator>
#include <new>
#include <vector>

#include <cuda_runtime.h>

#include "common.cuh"
#include "context.hpp"
#include "predicates.cuh"
#include "qdt.h"
#include "qdt_gpu.h"

using qdtg::Context;

namespace qdtg {

void Context::reset() noexcept
{
    points.clear();
    rep.clear();
    tris.clear();
    unique_points = 0;
    if (mesh)
    {
        mesh_destroy(mesh);
        mesh = nullptr;
    }
}

void Context::reset_release() noexcept
{
    reset();
    PinnedVec<double>().swap(points);
    PinnedVec<uint32_t>().swap(rep);
    PinnedVec<uint32_t>().swap(tris);
}

Context::~Context()
{
    if (mesh) mesh_destroy(mesh);
    delete engine;
}

static int ensure_engine(Context& c)
{
    if (c.engine) return QDT_OK;
    int err = 0;
    c.engine = Engine::create(&err);
    if (!c.engine)
    {
        c.last_cuda_error = err ? err : -1;
        return QDT_ERR_INTERNAL;
    }
    return QDT_OK;
}

int rebuild_from_points(Context& c)
{
    const int e = ensure_engine(c);
    if (e != QDT_OK) return e;
    // the engine reads from the caller's array while it fills `points`:
    // hand it a separate copy
    PinnedVec<double> src(c.points);
    size_t            ntri = 0, uniq = 0;
    const int         st = c.engine->run_host(src.data(), src.size() / 2, c.points, c.tris, &ntri, c.rep, &uniq);
    if (st != QDT_OK) return st;
    c.unique_points = uniq;
    if (c.mesh)
    {
        mesh_destroy(c.mesh);
        c.mesh = nullptr;
    }
    return QDT_OK;
}

}  // namespace qdtg

namespace {

inline Context* ctx(qdt_t* p) { return reinterpret_cast<Context*>(p); }
inline const Context* ctx(const qdt_t* p) { return reinterpret_cast<const Context*>(p); }

inline bool point_ok(double x, double y) { return std::isfinite(x) && std::isfinite(y); }

// reference qdt.cpp:63-77
qdt_status status_from_current_exception() noexcept
{
    try
    {
        throw;
    }
    catch (const std::bad_alloc&)
    {
        return QDT_ERR_OUT_OF_MEMORY;
    }
    catch (...)
    {
        return QDT_ERR_INTERNAL;
    }
}

void fill_results(qdt_status* results, size_t n, qdt_status st) noexcept
{
    if (!results) return;
    for (size_t i = 0; i < n; ++i) results[i] = st;
}

// reference qdt.cpp:29-43 and :88-113. The finiteness scan of the input runs
// on the GPU, fused into the key transform (same order of checks: the count
// and NULL are tested first, on the host).
qdt_status execute_impl(qdt_t* ptr, const qdt_vec2d* pts, size_t n)
{
    Context* c = ctx(ptr);
    if (!c) return QDT_ERR_NULL_CONTEXT;
    try
    {
        if (n > qdtg::kMaxPoints)
        {
            c->reset();
            return QDT_ERR_TOO_MANY_POINTS;
        }
        if (n > 0 && !pts)
        {
            c->reset();
            return QDT_ERR_NULL_ARGUMENT;
        }
        c->reset();
        if (n == 0) return QDT_OK;
        int st = qdtg::ensure_engine(*c);
        if (st != QDT_OK)
        {
            c->reset();
            return (qdt_status)st;
        }
        size_t ntri = 0, uniq = 0;
        st = c->engine->run_host(reinterpret_cast<const double*>(pts), n, c->points, c->tris, &ntri, c->rep, &uniq);
        if (st != QDT_OK)
        {
            c->reset();
            return (qdt_status)st;
        }
        c->unique_points = uniq;
        return QDT_OK;
    }
    catch (...)
    {
        const qdt_status st = status_from_current_exception();
        c->reset_release();
        return st;
    }
}

// reference qdt.cpp:116-142
qdt_status insert_point_impl(qdt_t* ptr, const qdt_vec2d& pt, size_t* index, bool parallel)
{
    Context* c = ctx(ptr);
    if (!c) return QDT_ERR_NULL_CONTEXT;
    try
    {
        if (!point_ok(pt.x, pt.y)) return QDT_ERR_NOT_FINITE;
        if (c->npoints() >= qdtg::kMaxPoints) return QDT_ERR_TOO_MANY_POINTS;
        const int st = qdtg::mesh_insert_point(*c, pt.x, pt.y, parallel);
        if (st != QDT_OK)
        {
            c->reset();
            return (qdt_status)st;
        }
        if (index) *index = c->npoints() - 1;
        return QDT_OK;
    }
    catch (...)
    {
        const qdt_status st = status_from_current_exception();
        c->reset_release();
        return st;
    }
}

}  // namespace

extern "C" {

QDT_API const char* qdt_status_string(qdt_status status)
{
    switch (status)
    {
    case QDT_OK: return "success";
    case QDT_ERR_NULL_CONTEXT: return "the context is NULL";
    case QDT_ERR_NULL_ARGUMENT: return "a required pointer argument is NULL";
    case QDT_ERR_TOO_MANY_POINTS: return "more than 100000000 points";
    case QDT_ERR_NOT_FINITE: return "a coordinate is NaN or infinite";
    case QDT_ERR_INVALID_INDEX: return "an end point index is not a point of the context";
    case QDT_ERR_SAME_POINT: return "both end points are the same point";
    case QDT_ERR_NO_TRIANGLES: return "the context has no triangles";
    case QDT_ERR_CROSSES_CONSTRAINT: return "the segment crosses an existing constraint";
    case QDT_ERR_THROUGH_POINT: return "the segment passes through another point";
    case QDT_ERR_OUT_OF_MEMORY: return "out of memory";
    case QDT_ERR_INTERNAL: return "internal error";
    }
    return "unknown status";
}

QDT_API qdt_t* qdt_create(void) { return reinterpret_cast<qdt_t*>(new (std::nothrow) Context()); }

QDT_API qdt_status qdt_execute(qdt_t* ptr, const qdt_vec2d* pts, size_t n) { return execute_impl(ptr, pts, n); }

QDT_API qdt_status qdt_execute_parallel(qdt_t* ptr, const qdt_vec2d* pts, size_t n)
{
    return execute_impl(ptr, pts, n);
}

QDT_API qdt_status qdt_insert_point(qdt_t* ptr, qdt_vec2d pt, size_t* index)
{
    return insert_point_impl(ptr, pt, index, false);
}

QDT_API qdt_status qdt_insert_point_parallel(qdt_t* ptr, qdt_vec2d pt, size_t* index)
{
    return insert_point_impl(ptr, pt, index, true);
}

// reference qdt.cpp:193-212
QDT_API qdt_status qdt_insert_constraint(qdt_t* ptr, size_t v0, size_t v1)
{
    Context* c = ctx(ptr);
    if (!c) return QDT_ERR_NULL_CONTEXT;
    try
    {
        const qdt_status st = (qdt_status)qdtg::mesh_insert_constraint(*c, v0, v1);
        if (st == QDT_ERR_INTERNAL) c->reset();
        return st;
    }
    catch (...)
    {
        const qdt_status st = status_from_current_exception();
        c->reset_release();
        return st;
    }
}

// reference qdt.cpp:214-244 with Wrapper.cpp:1264-1285
QDT_API qdt_status qdt_insert_constraints_batch(qdt_t* ptr, const qdt_edge* edges, size_t num_edges,
    qdt_status* results)
{
    Context* c = ctx(ptr);
    if (!c)
    {
        fill_results(results, num_edges, QDT_ERR_NULL_CONTEXT);
        return QDT_ERR_NULL_CONTEXT;
    }
    if (num_edges == 0) return QDT_OK;
    if (!edges)
    {
        fill_results(results, num_edges, QDT_ERR_NULL_ARGUMENT);
        return QDT_ERR_NULL_ARGUMENT;
    }
    try
    {
        qdt_status first = QDT_OK;
        for (size_t i = 0; i < num_edges; ++i)
        {
            const qdt_status st = (qdt_status)qdtg::mesh_insert_constraint(*c, edges[i].v0, edges[i].v1);
            if (st == QDT_ERR_INTERNAL)
            {
                c->reset();
                fill_results(results, num_edges, QDT_ERR_INTERNAL);
                return QDT_ERR_INTERNAL;
            }
            if (results) results[i] = st;
            if (st != QDT_OK && first == QDT_OK) first = st;
        }
        return first;
    }
    catch (...)
    {
        const qdt_status st = status_from_current_exception();
        c->reset_release();
        fill_results(results, num_edges, st);
        return st;
    }
}

QDT_API size_t qdt_triangles_size(const qdt_t* ptr)
{
    const Context* c = ctx(ptr);
    return c ? c->ntris() : 0;
}

QDT_API size_t qdt_get_triangle(const qdt_t* ptr, size_t T[3], size_t id)
{
    const Context* c = ctx(ptr);
    if (!c || !T) return 0;
    if (id >= c->ntris()) return 0;
    const uint32_t* t = c->tris.data() + 3 * id;
    T[0] = t[0];
    T[1] = t[1];
    T[2] = t[2];
    return 1;
}

QDT_API size_t qdt_points_size(const qdt_t* ptr)
{
    const Context* c = ctx(ptr);
    return c ? c->npoints() : 0;
}

QDT_API size_t qdt_get_point(const qdt_t* ptr, qdt_vec2d* pt, size_t id)
{
    const Context* c = ctx(ptr);
    if (!c || !pt) return 0;
    if (id >= c->npoints()) return 0;
    pt->x = c->points[2 * id];
    pt->y = c->points[2 * id + 1];
    return 1;
}

// reference qdt.cpp:285-298
QDT_API size_t qdt_point_is_used(const qdt_t* ptr, size_t id)
{
    const Context* c = ctx(ptr);
    if (!c) return 0;
    if (id >= c->npoints() || id >= c->rep.size()) return 0;
    if (c->tris.empty()) return 0;
    return c->rep[id] == id ? 1 : 0;
}

QDT_API void qdt_destroy(qdt_t* ptr) { delete ctx(ptr); }

// ---------------------------------------------------------------------------
// qdt_gpu.h
// ---------------------------------------------------------------------------

QDT_API void qdtg_set_options(qdt_t* ptr, int count_filter_failures, int stage_timing)
{
    Context* c = ctx(ptr);
    if (!c) return;
    if (qdtg::ensure_engine(*c) != QDT_OK) return;
    c->engine->set_count_filter(count_filter_failures != 0);
    c->engine->set_timing(stage_timing != 0);
}

QDT_API size_t qdtg_workspace_bytes(size_t n) { return qdtg::Engine::workspace_bytes(n); }

QDT_API int qdtg_device_name(char* out, size_t cap)
{
    if (!out || cap == 0) return 0;
    out[0] = 0;
    int dev = 0, count = 0;
    cudaDeviceProp prop;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0 || cudaGetDevice(&dev) != cudaSuccess ||
        cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    std::strncpy(out, prop.name, cap - 1);
    out[cap - 1] = 0;
    return 1;
}

QDT_API int qdtg_set_defaults(int cell_points, int batch_cell_points, int single_warp_nodes,
    int batch_warp_min_points, int batch_warp_nodes, int server_large_workers)
{
    auto bad_cells = [](int c) { return c > qdtg::kCellMax || (c > 0 && c < 4); };
    if (bad_cells(cell_points) || bad_cells(batch_cell_points) || server_large_workers > 64) return 0;
    qdtg::Tuning& t = qdtg::tuning();
    if (cell_points >= 0) t.cell_points = cell_points;
    if (batch_cell_points >= 0) t.batch_cell_points = batch_cell_points;
    if (single_warp_nodes > 0) t.single_warp_nodes = single_warp_nodes;
    if (batch_warp_min_points > 0) t.batch_warp_min_points = batch_warp_min_points;
    if (batch_warp_nodes > 0) t.batch_warp_nodes = batch_warp_nodes;
    if (server_large_workers > 0) t.server_large_workers = server_large_workers;
    return 1;
}

QDT_API void qdtg_get_defaults(int* cell_points, int* batch_cell_points, int* single_warp_nodes,
    int* batch_warp_min_points, int* batch_warp_nodes, int* server_large_workers)
{
    const qdtg::Tuning& t = qdtg::tuning();
    if (cell_points) *cell_points = t.cell_points;
    if (batch_cell_points) *batch_cell_points = t.batch_cell_points;
    if (single_warp_nodes) *single_warp_nodes = t.single_warp_nodes;
    if (batch_warp_min_points) *batch_warp_min_points = t.batch_warp_min_points;
    if (batch_warp_nodes) *batch_warp_nodes = t.batch_warp_nodes;
    if (server_large_workers) *server_large_workers = t.server_large_workers;
}

QDT_API int qdtg_set_mesh_on_gpu(qdt_t* ptr, int on_gpu)
{
    Context* c = ctx(ptr);
    if (!c) return 0;
    c->mesh_on_gpu = on_gpu != 0;
    return 1;
}

QDT_API qdt_status qdtg_locate_points(qdt_t* ptr, const qdt_vec2d* pts, size_t k, int64_t* tri, int32_t* where)
{
    Context* c = ctx(ptr);
    if (!c) return QDT_ERR_NULL_CONTEXT;
    if (k == 0) return QDT_OK;
    if (!pts || !tri) return QDT_ERR_NULL_ARGUMENT;
    for (size_t i = 0; i < k; ++i)
        if (!point_ok(pts[i].x, pts[i].y)) return QDT_ERR_NOT_FINITE;
    try
    {
        std::vector<int> t(k), w(k);
        const int        st = qdtg::mesh_locate(*c, &pts[0].x, k, t.data(), w.data(), nullptr);
        if (st != QDT_OK) return (qdt_status)st;
        for (size_t i = 0; i < k; ++i)
        {
            tri[i] = t[i];
            if (where) where[i] = w[i];
        }
        return QDT_OK;
    }
    catch (...)
    {
        return status_from_current_exception();
    }
}

QDT_API qdt_status qdtg_trace_constraints(qdt_t* ptr, const qdt_edge* edges, size_t k, qdt_status* status,
    int64_t* crossed)
{
    Context* c = ctx(ptr);
    if (!c) return QDT_ERR_NULL_CONTEXT;
    if (k == 0) return QDT_OK;
    if (!edges || !status) return QDT_ERR_NULL_ARGUMENT;
    static_assert(sizeof(qdt_edge) == 2 * sizeof(size_t), "qdt_edge is two size_t");
    try
    {
        std::vector<int>     st(k);
        std::vector<int64_t> cr(k);
        const int            rc = qdtg::mesh_trace_segments(*c, &edges[0].v0, k, st.data(), cr.data());
        if (rc != QDT_OK) return (qdt_status)rc;
        for (size_t i = 0; i < k; ++i)
        {
            status[i] = (qdt_status)st[i];
            if (crossed) crossed[i] = cr[i];
        }
        return QDT_OK;
    }
    catch (...)
    {
        return status_from_current_exception();
    }
}

QDT_API qdt_status qdtg_insert_points(qdt_t* ptr, const qdt_vec2d* pts, size_t k, size_t* indices,
    qdt_status* results)
{
    Context* c = ctx(ptr);
    auto     fail_all = [&](qdt_status st) {
        fill_results(results, k, st);
        if (indices)
            for (size_t i = 0; i < k; ++i) indices[i] = (size_t)-1;
        return st;
    };
    if (!c) return fail_all(QDT_ERR_NULL_CONTEXT);
    if (k == 0) return QDT_OK;
    if (!pts) return fail_all(QDT_ERR_NULL_ARGUMENT);
    try
    {
        const std::vector<int> hints = qdtg::mesh_insert_hints(*c, &pts[0].x, k);
        qdt_status             first = QDT_OK;
        for (size_t i = 0; i < k; ++i)
        {
            qdt_status st;
            if (!point_ok(pts[i].x, pts[i].y))
                st = QDT_ERR_NOT_FINITE;
            else if (c->npoints() >= qdtg::kMaxPoints)
                st = QDT_ERR_TOO_MANY_POINTS;
            else
            {
                st = (qdt_status)qdtg::mesh_insert_point(*c, pts[i].x, pts[i].y, false, hints[i]);
                if (st != QDT_OK)
                {
                    // as qdt_insert_point: a failed rebuild leaves the context empty
                    c->reset();
                    fill_results(results ? results + i : nullptr, k - i, st);
                    if (indices)
                        for (size_t j = i; j < k; ++j) indices[j] = (size_t)-1;
                    return st;
                }
            }
            if (results) results[i] = st;
            if (indices) indices[i] = st == QDT_OK ? c->npoints() - 1 : (size_t)-1;
            if (st != QDT_OK && first == QDT_OK) first = st;
        }
        return first;
    }
    catch (...)
    {
        const qdt_status st = status_from_current_exception();
        c->reset_release();
        return fail_all(st);
    }
}

QDT_API int qdtg_set_warp_nodes(qdt_t* ptr, int warp_nodes)
{
    Context* c = ctx(ptr);
    if (!c || warp_nodes < 1) return 0;
    if (qdtg::ensure_engine(*c) != QDT_OK) return 0;
    c->engine->set_warp_nodes(warp_nodes);
    return 1;
}

QDT_API int qdtg_set_cell_points(qdt_t* ptr, int cell_points)
{
    Context* c = ctx(ptr);
    if (!c) return 0;
    if (cell_points != 0 && (cell_points < 4 || cell_points > qdtg::kCellMax)) return 0;
    if (qdtg::ensure_engine(*c) != QDT_OK) return 0;
    c->engine->set_cell_points(cell_points);
    return 1;
}

namespace qdtg {
// RunInfo's per-stage predicate statistics into the C struct
void fill_filter_stats(const RunInfo& r, qdtg_filter_stats* out)
{
    *out = qdtg_filter_stats{};
    for (int s = 0; s < kPredStages && s < 4; ++s)
        for (int k = 0; k < 2; ++k)
        {
            out->calls[s][k] = r.stage[s].calls[k];
            out->f32_undecided[s][k] = r.stage[s].f32_undecided[k];
            out->exact[s][k] = r.stage[s].exact[k];
        }
}
}  // namespace qdtg

// No counterpart in the reference (qdt_gpu.h).
QDT_API int qdtg_get_filter_stats(const qdt_t* ptr, qdtg_filter_stats* stats)
{
    const Context* c = ctx(ptr);
    if (!c || !stats) return 0;
    *stats = qdtg_filter_stats{};
    if (c->engine) qdtg::fill_filter_stats(c->engine->info(), stats);
    return 1;
}

QDT_API int qdtg_get_run_info(const qdt_t* ptr, qdtg_run_info* info)
{
    const Context* c = ctx(ptr);
    if (!c || !info) return 0;
    *info = qdtg_run_info{};
    if (!c->engine) return 1;
    const qdtg::RunInfo& r = c->engine->info();
    info->n = r.n;
    info->unique_points = r.unique_points;
    info->triangles = r.ntri;
    info->orient_exact = r.orient_exact;
    info->incircle_exact = r.incircle_exact;
    info->ms_h2d = r.ms.h2d;
    info->ms_sort = r.ms.keys_sort;
    info->ms_unique = r.ms.unique;
    info->ms_split = r.ms.split;
    info->ms_build = r.ms.build;
    info->ms_extract = r.ms.extract;
    info->ms_d2h = r.ms.d2h;
    info->ms_total = r.ms.total;
    info->device_flags = r.device_status;
    info->kernel_launches = r.launches;
    info->merge_window = r.window;
    info->wide_exact = r.wide;
    info->split_depth = r.split_depth;
    info->split_rerun = r.split_rerun;
    info->split_segments = r.split_segments;
    return 1;
}

QDT_API int qdtg_set_graphs(qdt_t* ptr, int use_graphs)
{
    Context* c = ctx(ptr);
    if (!c) return 0;
    if (qdtg::ensure_engine(*c) != QDT_OK) return 0;
    c->engine->set_use_graphs(use_graphs != 0);
    return 1;
}

QDT_API int qdtg_set_split_tail(qdt_t* ptr, int on)
{
    Context* c = ctx(ptr);
    if (!c) return 0;
    if (qdtg::ensure_engine(*c) != QDT_OK) return 0;
    c->engine->set_split_tail(on != 0);
    return 1;
}

QDT_API int qdtg_set_side_prefetch(qdt_t* ptr, int on)
{
    Context* c = ctx(ptr);
    if (!c) return 0;
    if (qdtg::ensure_engine(*c) != QDT_OK) return 0;
    c->engine->set_side_prefetch(on != 0);
    return 1;
}

QDT_API int qdtg_set_split_merges(qdt_t* ptr, int max_depth, int min_points)
{
    Context* c = ctx(ptr);
    if (!c || max_depth < -1 || max_depth > qdtg::kSplitMaxDepth || min_points < qdtg::kSplitFloor) return 0;
    if (qdtg::ensure_engine(*c) != QDT_OK) return 0;
    c->engine->set_split(max_depth, min_points);
    return 1;
}

QDT_API int qdtg_set_split_segments(qdt_t* ptr, int max_segments, int segment_points)
{
    Context* c = ctx(ptr);
    if (!c || max_segments < 1 || max_segments > qdtg::kSplitMaxSegs || segment_points < qdtg::kSplitSegFloor)
        return 0;
    if (qdtg::ensure_engine(*c) != QDT_OK) return 0;
    c->engine->set_split_segments(max_segments, segment_points);
    return 1;
}

QDT_API int qdtg_set_workspace_limit(qdt_t* ptr, size_t bytes)
{
    Context* c = ctx(ptr);
    if (!c) return 0;
    if (qdtg::ensure_engine(*c) != QDT_OK) return 0;
    c->engine->set_workspace_limit(bytes);
    return 1;
}

QDT_API size_t qdtg_context_workspace_bytes(const qdt_t* ptr)
{
    const Context* c = ctx(ptr);
    return (c && c->engine) ? c->engine->workspace_bytes() : 0;
}

QDT_API int qdtg_set_merge_window(qdt_t* ptr, int window)
{
    Context* c = ctx(ptr);
    if (!c || window < 0 || window > 2) return 0;
    if (qdtg::ensure_engine(*c) != QDT_OK) return 0;
    c->engine->set_merge_window(window);
    return 1;
}

QDT_API void* qdtg_stream(const qdt_t* ptr)
{
    const Context* c = ctx(ptr);
    return (c && c->engine) ? reinterpret_cast<void*>(c->engine->stream()) : nullptr;
}

QDT_API qdt_status qdtg_execute_device(qdt_t* ptr, const qdt_vec2d* d_pts, size_t n, void* cuda_stream)
{
    Context* c = ctx(ptr);
    if (!c) return QDT_ERR_NULL_CONTEXT;
    try
    {
        c->reset();
        if (n > qdtg::kMaxPoints) return QDT_ERR_TOO_MANY_POINTS;
        if (n > 0 && !d_pts) return QDT_ERR_NULL_ARGUMENT;
        int st = qdtg::ensure_engine(*c);
        if (st != QDT_OK) return (qdt_status)st;
        st = c->engine->run_device(reinterpret_cast<const double*>(d_pts), n,
            reinterpret_cast<cudaStream_t>(cuda_stream));
        return (qdt_status)st;
    }
    catch (...)
    {
        const qdt_status st = status_from_current_exception();
        c->reset_release();
        return st;
    }
}

QDT_API size_t qdtg_device_triangles(const qdt_t* ptr, const uint32_t** d_tris)
{
    const Context* c = ctx(ptr);
    if (!c || !c->engine) return 0;
    if (d_tris) *d_tris = c->engine->device_triangles();
    return c->engine->last_ntri();
}

QDT_API size_t qdtg_download_device_triangles(const qdt_t* ptr, uint32_t* out, size_t cap)
{
    const Context* c = ctx(ptr);
    if (!c || !c->engine || !out) return 0;
    const size_t k = std::min(cap, c->engine->last_ntri());
    if (k == 0) return 0;
    if (cudaMemcpy(out, c->engine->device_triangles(), 3 * k * sizeof(uint32_t), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    return k;
}

QDT_API size_t qdtg_copy_triangles(const qdt_t* ptr, uint32_t* out, size_t cap)
{
    const Context* c = ctx(ptr);
    if (!c || !out) return 0;
    const size_t k = std::min(cap, c->ntris());
    std::copy(c->tris.data(), c->tris.data() + 3 * k, out);
    return k;
}

QDT_API size_t qdtg_copy_rep(const qdt_t* ptr, uint32_t* out, size_t cap)
{
    const Context* c = ctx(ptr);
    if (!c || !out) return 0;
    const size_t k = std::min(cap, c->rep.size());
    std::copy(c->rep.data(), c->rep.data() + k, out);
    return k;
}

// No counterpart in the reference: loads a saved triangulation (qdt_gpu.h).
QDT_API qdt_status qdtg_set_triangulation(qdt_t* ptr, const qdt_vec2d* pts, size_t n, const uint32_t* rep,
    const uint32_t* tris, size_t ntri)
{
    Context* c = ctx(ptr);
    if (!c) return QDT_ERR_NULL_CONTEXT;
    try
    {
        c->reset();
        if (n > qdtg::kMaxPoints || ntri > 2 * qdtg::kMaxPoints) return QDT_ERR_TOO_MANY_POINTS;
        if ((n && !pts) || (ntri && !tris)) return QDT_ERR_NULL_ARGUMENT;
        for (size_t i = 0; i < n; ++i)
            if (!point_ok(pts[i].x, pts[i].y)) return QDT_ERR_NOT_FINITE;
        // representatives: the lowest index with the same coordinates (-0.0
        // equals +0.0)
        size_t uniq = 0;
        {
            auto bits = [](double v) {
                uint64_t b;
                v = v == 0.0 ? 0.0 : v;
                std::memcpy(&b, &v, sizeof b);
                return b;
            };
            std::vector<std::pair<std::pair<uint64_t, uint64_t>, uint32_t>> order(n);
            for (size_t i = 0; i < n; ++i) order[i] = { { bits(pts[i].x), bits(pts[i].y) }, (uint32_t)i };
            std::sort(order.begin(), order.end());
            for (size_t k = 0; k < n;)
            {
                size_t j = k;
                const uint32_t lowest = order[k].second;
                for (; j < n && order[j].first == order[k].first; ++j)
                {
                    const uint32_t i = order[j].second;
                    if ((rep ? rep[i] : i) != lowest) return QDT_ERR_INVALID_INDEX;
                }
                ++uniq;
                k = j;
            }
        }
        // triangles: representatives as corners, strictly counter-clockwise,
        // every directed edge once
        std::vector<uint64_t> edges;
        edges.reserve(3 * ntri);
        for (size_t t = 0; t < ntri; ++t)
        {
            const uint32_t* T = tris + 3 * t;
            for (int k = 0; k < 3; ++k)
                if (T[k] >= n || (rep && rep[T[k]] != T[k])) return QDT_ERR_INVALID_INDEX;
            const qdt_vec2d &a = pts[T[0]], &b = pts[T[1]], &d = pts[T[2]];
            if (qdtg::orient2d_sign(a.x, a.y, b.x, b.y, d.x, d.y) <= 0) return QDT_ERR_INVALID_INDEX;
            for (int k = 0; k < 3; ++k) edges.push_back(((uint64_t)T[k] << 32) | T[(k + 1) % 3]);
        }
        std::sort(edges.begin(), edges.end());
        if (std::adjacent_find(edges.begin(), edges.end()) != edges.end()) return QDT_ERR_INVALID_INDEX;
        // the triangles cover the convex hull of the distinct points once:
        // every distinct point is a corner; the edges without a reverse form
        // one cycle that turns left or runs straight at every corner; and the
        // triangles' areas add up to the area inside it (not twice as much)
        if (ntri)
        {
            std::vector<uint8_t> corner(n, 0);
            for (size_t i = 0; i < 3 * ntri; ++i) corner[tris[i]] = 1;
            for (size_t i = 0; i < n; ++i)
                if ((rep ? rep[i] : i) == i && !corner[i]) return QDT_ERR_INVALID_INDEX;
            std::vector<uint64_t> rev(edges.size());
            for (size_t i = 0; i < edges.size(); ++i) rev[i] = (edges[i] << 32) | (edges[i] >> 32);
            std::sort(rev.begin(), rev.end());
            std::vector<uint64_t> hull;   // a -> b with no b -> a, sorted by a
            std::set_difference(edges.begin(), edges.end(), rev.begin(), rev.end(), std::back_inserter(hull));
            for (size_t i = 1; i < hull.size(); ++i)
                if ((hull[i] >> 32) == (hull[i - 1] >> 32)) return QDT_ERR_INVALID_INDEX;
            auto after = [&](uint32_t a) -> int64_t {
                const auto it = std::lower_bound(hull.begin(), hull.end(), (uint64_t)a << 32);
                return (it != hull.end() && (*it >> 32) == a) ? (int64_t)(uint32_t)*it : -1;
            };
            if (hull.empty()) return QDT_ERR_INVALID_INDEX;
            const uint32_t first = (uint32_t)(hull[0] >> 32);
            const double   ox = pts[first].x, oy = pts[first].y;
            double         inside = 0.0, covered = 0.0;   // twice the areas
            size_t         steps = 0;
            for (uint32_t a = first;;)
            {
                const int64_t b = after(a);
                const int64_t d = b < 0 ? -1 : after((uint32_t)b);
                if (d < 0 || ++steps > hull.size()) return QDT_ERR_INVALID_INDEX;
                const qdt_vec2d &A = pts[a], &B = pts[b], &D = pts[d];
                if (qdtg::orient2d_sign(A.x, A.y, B.x, B.y, D.x, D.y) < 0) return QDT_ERR_INVALID_INDEX;
                inside += (A.x - ox) * (B.y - oy) - (B.x - ox) * (A.y - oy);
                a = (uint32_t)b;
                if (a == first) break;
            }
            if (steps != hull.size()) return QDT_ERR_INVALID_INDEX;   // more than one cycle
            for (size_t t = 0; t < ntri; ++t)
            {
                const qdt_vec2d &a = pts[tris[3 * t]], &b = pts[tris[3 * t + 1]], &d = pts[tris[3 * t + 2]];
                covered += (b.x - a.x) * (d.y - a.y) - (b.y - a.y) * (d.x - a.x);
            }
            if (covered > 1.5 * inside) return QDT_ERR_INVALID_INDEX;   // a region covered twice
        }
        c->points.resize(2 * n);
        for (size_t i = 0; i < n; ++i)
        {
            c->points[2 * i] = pts[i].x;
            c->points[2 * i + 1] = pts[i].y;
        }
        c->rep.resize(n);
        for (size_t i = 0; i < n; ++i) c->rep[i] = rep ? rep[i] : (uint32_t)i;
        c->tris.assign(tris, tris + 3 * ntri);
        c->unique_points = uniq;
        return QDT_OK;
    }
    catch (...)
    {
        const qdt_status st = status_from_current_exception();
        c->reset_release();
        return st;
    }
}

QDT_API int qdtg_last_cuda_error(const qdt_t* ptr)
{
    const Context* c = ctx(ptr);
    return c ? c->last_cuda_error : 0;
}

QDT_API const char* qdtg_version(void) { return "qdt-gb300 0.1 (sm_103a)"; }

}  // extern "C"
