/*
 * qdt_gpu.h -- GPU-specific additions to the qdt.h interface.
 *
 * qdt.h is the drop-in boundary and stays as the reference has it. The
 * functions here are additive: they have no counterpart in the reference and
 * expose what only a GPU implementation can offer -- input that already lives
 * in device memory, results read in bulk instead of one triangle per call,
 * per-stage timing, and the filter-failure counters of the exact predicates.
 */
#if !defined(_LIB_QDT_GPU_H_)
#define _LIB_QDT_GPU_H_

#include <stddef.h>
#include <stdint.h>

#include "qdt.h"

#if __cplusplus
extern "C"
{
#endif

/* What the last batch call of a context did. Times are milliseconds measured
   with CUDA events on the context's stream (0 unless timing is enabled with
   qdtg_set_options). */
typedef struct qdtg_run_info
{
    size_t             n;               /* input points */
    size_t             unique_points;   /* distinct points */
    size_t             triangles;
    unsigned long long orient_exact;    /* orient2d calls that needed the exact path (if counted) */
    unsigned long long incircle_exact;  /* in-circle calls that needed the exact path (if counted) */
    float              ms_h2d, ms_sort, ms_unique, ms_split, ms_build, ms_extract, ms_d2h, ms_total;
    int                device_flags;    /* device status bits; 0 = clean */
    int                kernel_launches; /* kernels the call launched */
    int                merge_window;    /* candidate window of the warp merges (1 or 2; 0 = none ran) */
    int                wide_exact;      /* 1: a predicate needed the widest exact tier and the build ran
                                           again with the kernels that have it */
    int                split_depth;     /* deepest depth whose merges ran as split merges (-1: none) */
    int                split_rerun;     /* 1: a split merge could not finish and the build ran again
                                           (with one seam segment a merge, else one walker) */
    int                split_segments;  /* the most seam segments of a split merge in the last pass */
} qdtg_run_info;

/* Options of a context: count_filter_failures != 0 counts the predicate calls
   that fall back to exact arithmetic (adds atomics on that rare path);
   stage_timing != 0 records CUDA events between the stages. */
QDT_API void qdtg_set_options(qdt_t* ptr, int count_filter_failures, int stage_timing);

/* The largest subtree (in points, 4..1024) that the context builds in
   on-chip shared memory before the levels above it run out of HBM; 0 builds
   every level out of HBM. Default 256. Returns 1, or 0 for a NULL context,
   a value out of range or no usable GPU. The triangulation does not depend
   on it. */
QDT_API int qdtg_set_cell_points(qdt_t* ptr, int cell_points);

/* The candidate window of the context's warp merges: 0 (default) chooses per
   call from the input -- 1 when most distinct points share their x with
   another (integer lattices, snapped grids), else 2; 1 or 2 fix it. The
   triangulation does not depend on it. Returns 1, or 0 for a NULL context,
   a value out of range or no usable GPU. */
QDT_API int qdtg_set_merge_window(qdt_t* ptr, int window);

/* The stages before the distinct-point count (keys, sort, distinct points)
   are captured once per (point count, input array) and the stages after it
   (split levels, build, extraction: about 250 launches at 2.6 M points)
   once per (distinct count, knobs) into CUDA graphs and replayed
   (use_graphs != 0, the default), or launched one by one. The result is
   the same. Returns 1, or 0 for a NULL context or no usable GPU. */
QDT_API int qdtg_set_graphs(qdt_t* ptr, int use_graphs);

/* The Dwyer split levels below the first depth whose nodes hold at most
   4,096 points run in one launch, a thread block per node working in shared
   memory (on != 0, the default), or one level at a time. The result is the
   same. Returns 1, or 0 for a NULL context or no usable GPU. */
QDT_API int qdtg_set_split_tail(qdt_t* ptr, int on);

/* Before each upper depth of the build, the records near that depth's
   seams are pulled into L2. With on != 0 (the default) that selection and
   prefetch runs on a second stream beside the previous depth's merges when
   no other engine is running a call, else in line. The prefetch reads only
   record numbers it selected and never writes a record, so the result is
   the same either way. Returns 1, or 0 for a NULL context or no usable GPU. */
QDT_API int qdtg_set_side_prefetch(qdt_t* ptr, int on);

/* The merges at the top of the build -- depths 0..max_depth (at most 9)
   whose nodes hold at least min_points points (at least 256) -- run as
   split merges: their seam is cut into segments (qdtg_set_split_segments),
   each walked by two walkers, the reference's rising merge from the
   segment's lower end and its mirror image from its upper end, which meet
   at a point of the seam. A falling walker that meets cocircular or
   collinear points hands its part to the rising one, so the triangulation
   is the same as with one walker per merge (max_depth -1). Defaults 7 and
   1,024.
   Returns 1, or 0 for a NULL context, values out of range or no usable
   GPU. No counterpart in the reference, whose merges are sequential. */
QDT_API int qdtg_set_split_merges(qdt_t* ptr, int max_depth, int min_points);

/* Seam segments of one split merge at most (1..5, default 5; a node gets
   one more segment per segment_points points, at least 1,024, default
   16,384; on calls of at least 65,536 points).
   Segments beyond the first begin at cross edges found before the merge:
   pairs of mutually nearest vertices of the two halves, which are edges of
   every Delaunay triangulation of the merged points; each segment is walked
   by a rising and a falling walker. The triangulation is the same for
   every value: a call whose walkers above the first segment meet a
   cocircular or collinear configuration runs its build again with one
   segment a merge (qdtg_run_info.split_rerun). Returns 1, or 0 for a NULL
   context, a value out of range or no usable GPU. No counterpart in the
   reference, whose merges are sequential. */
QDT_API int qdtg_set_split_segments(qdt_t* ptr, int max_segments, int segment_points);

/* Caps the device bytes of the context's workspace (0: no cap, the
   default). A batch call whose workspace would exceed the cap returns
   QDT_ERR_OUT_OF_MEMORY and leaves the context empty, as when cudaMalloc
   fails; a workspace already above a new cap is freed. The device copy of
   the mesh (qdtg_locate_points) is not counted. Returns 1, or 0 for a NULL
   context or no usable GPU. */
QDT_API int qdtg_set_workspace_limit(qdt_t* ptr, size_t bytes);

/* Device bytes the context's workspace holds now (0 when none). */
QDT_API size_t qdtg_context_workspace_bytes(const qdt_t* ptr);

/* Device bytes of a context's workspace for a batch call on n points (the
   workspace is kept between calls and grows when a call needs more). */
QDT_API size_t qdtg_workspace_bytes(size_t n);

/* The name of the current CUDA device into out (cap bytes, terminated);
   returns 0 (and an empty string) when no device is usable. */
QDT_API int qdtg_device_name(char* out, size_t cap);

/* The first insertion or constraint after a batch call builds the context's
   half-edge mesh; with on_gpu != 0 (the default) it is built on the GPU from
   the batch result the device still holds, else on the host. The mesh and
   every later result are the same either way. Returns 1, or 0 for a NULL
   context. */
QDT_API int qdtg_set_mesh_on_gpu(qdt_t* ptr, int on_gpu);

/* Batch point location (extends the reference's single-point locate_,
   GuibasStolfiDwyer_Wrapper.cpp:423-486, which qdt_insert_point runs): for
   each of the k points, tri[i] = the smallest index (qdt_get_triangle order)
   of a triangle that contains it, border included, or -1 beyond the hull or
   with no triangles; where[i] (may be NULL) = -1 outside, 0 inside a
   triangle, 1 on an edge, 2 on a vertex. The result depends only on the
   current triangulation and the point. The walks run on the GPU over a device
   copy of the mesh (built with it, uploaded again after insertions or
   constraints changed it). Checks: QDT_ERR_NULL_CONTEXT, QDT_ERR_NULL_ARGUMENT
   (pts or tri NULL with k > 0), QDT_ERR_NOT_FINITE (any coordinate; nothing
   is written); QDT_ERR_OUT_OF_MEMORY when the device copy cannot be made. */
QDT_API qdt_status qdtg_locate_points(qdt_t* ptr, const qdt_vec2d* pts, size_t k, int64_t* tri, int32_t* where);

/* qdt_insert_point() for each of the k points in order, with the same
   results (points, representatives, triangles in the same order). The
   points are located on the GPU first, so every insertion's walk starts next
   to its point instead of at the previous insertion. results[i] (may be NULL)
   = each entry's status; indices[i] (may be NULL) = the new point's index, or
   (size_t)-1 when the entry was rejected. Returns the first non-OK status,
   or QDT_OK. A rejected point (QDT_ERR_NOT_FINITE, QDT_ERR_TOO_MANY_POINTS)
   changes nothing; a failure that empties the context (as in
   qdt_insert_point) stops the loop and is reported for the remaining entries. */
QDT_API qdt_status qdtg_insert_points(qdt_t* ptr, const qdt_vec2d* pts, size_t k, size_t* indices,
    qdt_status* results);

/* Constraint tracing for a validation pass (the reference's trace_segment_,
   GuibasStolfiDwyer_Wrapper.cpp:1050-1106, and the checks before it,
   :1158-1165 and :1246-1261): for each of the k edges, on its
   own against the current triangulation (nothing is inserted), status[i] =
   what qdt_insert_constraint() would return for it as the next call
   (QDT_OK, QDT_ERR_INVALID_INDEX, QDT_ERR_SAME_POINT, QDT_ERR_NO_TRIANGLES,
   QDT_ERR_THROUGH_POINT, QDT_ERR_CROSSES_CONSTRAINT) and crossed[i] (may be
   NULL) = the number of edges its segment crosses before that decision (0
   when the edge exists; for QDT_OK, the edges the insertion flips away).
   Entries do not see each other: use qdt_insert_constraints_batch() to apply
   them in order. The traces run on the GPU over the device copy of the mesh
   (see qdtg_locate_points). Returns QDT_ERR_NULL_CONTEXT,
   QDT_ERR_NULL_ARGUMENT (edges or status NULL with k > 0),
   QDT_ERR_OUT_OF_MEMORY, or QDT_OK. */
QDT_API qdt_status qdtg_trace_constraints(qdt_t* ptr, const qdt_edge* edges, size_t k, qdt_status* status,
    int64_t* crossed);

/* The context's build merges with a whole warp per node at the depths that
   have at most warp_nodes nodes (few merges: each one's latency counts) or
   whose nodes hold at least 192 points, and with one thread per node below
   (many small merges); default 4096. Returns 1, or
   0 for a NULL context, a value below 1 or no usable GPU. The triangulation
   does not depend on it. */
QDT_API int qdtg_set_warp_nodes(qdt_t* ptr, int warp_nodes);

/* Process-wide defaults of the schedule knobs, taken by every context, batch
   and server created afterwards (the autotuner of the Python package sets
   them from its per-GPU cache): shared-memory cell size of the single-set
   and of the many-set builds (0: none), the single-set warp threshold
   (qdtg_set_warp_nodes), the many-set thresholds (qdtg_batch_set_options,
   qdtg_batch_set_warp_nodes) and the serving engines. A negative value (0
   for the last four) keeps the current one. Returns 0 and changes nothing
   for a value out of range. Call before creating contexts; not synchronised
   with concurrent creation. */
QDT_API int  qdtg_set_defaults(int cell_points, int batch_cell_points, int single_warp_nodes,
    int batch_warp_min_points, int batch_warp_nodes, int server_large_workers);
QDT_API void qdtg_get_defaults(int* cell_points, int* batch_cell_points, int* single_warp_nodes,
    int* batch_warp_min_points, int* batch_warp_nodes, int* server_large_workers);

/* Fills *info for the last batch call of the context. Returns 1, or 0 when
   ptr or info is NULL. */
QDT_API int qdtg_get_run_info(const qdt_t* ptr, qdtg_run_info* info);

/* Predicate statistics of the last batch call, when it counted
   (qdtg_set_options with count_filter_failures != 0; all zero otherwise),
   per stage of the build -- [0] leaves (2 or 3 points), [1] merges of a
   thread per node and shared-memory cells, [2] merges of a warp per node,
   [3] the extraction's orientation test -- and per predicate ([0]
   orient2d, [1] in-circle): the calls, the calls the single-precision
   pre-filter left undecided, and those the double filter left undecided as
   well (the exact evaluation ran). No counterpart in the reference, which
   counts nothing. */
typedef struct qdtg_filter_stats
{
    unsigned long long calls[4][2];
    unsigned long long f32_undecided[4][2];
    unsigned long long exact[4][2];
} qdtg_filter_stats;

/* Fills *stats for the last batch call of the context. Returns 1, or 0 when
   ptr or stats is NULL. */
QDT_API int qdtg_get_filter_stats(const qdt_t* ptr, qdtg_filter_stats* stats);

/* Batch triangulation of n points that are already in device memory (d_pts,
   16-byte aligned for the fastest path). The work is ordered after the work
   already queued on cuda_stream (a cudaStream_t; NULL for none) and the call
   returns when it is done. The triangles stay in device memory:
   qdtg_device_triangles() gives them. The host side of the context is left
   empty (no points, no triangles), as after a rejected batch call. Input
   checks and status codes are those of qdt_execute(). */
QDT_API qdt_status qdtg_execute_device(qdt_t* ptr, const qdt_vec2d* d_pts, size_t n, void* cuda_stream);

/* After qdtg_execute_device(): the number of triangles, and in *d_tris (if
   not NULL) a device pointer to 3 * count uint32 point indices, valid until
   the next batch call or qdt_destroy(). */
QDT_API size_t qdtg_device_triangles(const qdt_t* ptr, const uint32_t** d_tris);

/* After qdtg_execute_device(): copies min(cap, count) device triangles (3
   indices each) to host memory out and returns how many. */
QDT_API size_t qdtg_download_device_triangles(const qdt_t* ptr, uint32_t* out, size_t cap);

/* Bulk copies of the host results of the last batch call (or of the current
   triangulation after insertions and constraints). qdtg_copy_triangles
   writes min(cap, qdt_triangles_size) triangles (3 indices each) and returns
   how many; qdtg_copy_rep writes min(cap, qdt_points_size) representatives
   (the lowest index with the same coordinates) and returns how many. */
QDT_API size_t qdtg_copy_triangles(const qdt_t* ptr, uint32_t* out, size_t cap);
QDT_API size_t qdtg_copy_rep(const qdt_t* ptr, uint32_t* out, size_t cap);

/* Loads a triangulation made earlier into the context in place of a batch
   call: pts (n points), rep (the representatives qdtg_copy_rep wrote; NULL
   when all points are distinct) and tris (ntri triangles as
   qdtg_copy_triangles wrote them). The context then holds what that batch
   call left, and insertions, constraints and queries go on from there: a
   saved triangulation is resumed without triangulating again. Constraints
   are not part of the saved state. No counterpart in the reference; runs
   on the host and needs no GPU. The arrays are copied. Checks, in order:
   NULL context (QDT_ERR_NULL_CONTEXT); n > 1e8 or ntri > 2e8
   (QDT_ERR_TOO_MANY_POINTS); NULL arrays with n or ntri > 0
   (QDT_ERR_NULL_ARGUMENT); a NaN or infinite coordinate
   (QDT_ERR_NOT_FINITE); a representative that is not the lowest index of
   equal coordinates, a triangle corner out of range or not its own
   representative, a triangle not strictly counter-clockwise, a directed
   edge used twice, or triangles that do not cover the convex hull of the
   distinct points once (a distinct point that is no corner, a boundary
   that is not one cycle turning left or running straight at every corner,
   or a region covered twice) (QDT_ERR_INVALID_INDEX). Any rejection leaves
   the context empty. */
QDT_API qdt_status qdtg_set_triangulation(qdt_t* ptr, const qdt_vec2d* pts, size_t n, const uint32_t* rep,
    const uint32_t* tris, size_t ntri);

/* The CUDA stream (a cudaStream_t) on which the context's GPU work runs;
   NULL before the context's first batch call. Lets a caller order its own
   work or time the calls with CUDA events on that stream. */
QDT_API void* qdtg_stream(const qdt_t* ptr);

/* The CUDA error code of the last failed GPU call of the context (0 if
   none), e.g. when qdt_execute() returned QDT_ERR_INTERNAL because no GPU is
   present. */
QDT_API int qdtg_last_cuda_error(const qdt_t* ptr);

/* The exact predicates of the engine, on the host: the sign (-1, 0, +1) of
   orient2d(a, b, c) (> 0: counter-clockwise) and of incircle(a, b, c, d)
   (> 0: d inside the circle through a, b, c, taken counter-clockwise). Each
   point is two doubles. Exact for every finite input. */
QDT_API int qdtg_orient2d(const double* a, const double* b, const double* c);
QDT_API int qdtg_incircle(const double* a, const double* b, const double* c, const double* d);

/* The same predicates evaluated for count items, on the GPU (on_device != 0;
   allocates device memory for the call) or on the host: kind 0 =
   orient2d (6 doubles per item: ax ay bx by cx cy), kind 1 = incircle (8
   doubles). mode 0 = the full predicate, 1 = only the single-precision
   pre-filter (0 when it cannot decide), 2 = only the exact integer
   evaluation. Signs go to out. Returns 0, or a negative code on a CUDA
   failure or bad arguments. */
QDT_API int qdtg_eval_predicates(int kind, int mode, int on_device, const double* coords, size_t count,
    int8_t* out);

/* Distinct points and representatives of n device-resident points, with no
   device allocation at all. This entry point has no counterpart in the
   reference. It is meant for callers that cannot call cudaMalloc: plug-ins
   whose host application owns every device allocation, real-time loops that
   may not take the allocator's locks or latency. It computes the batch
   path's first stage (the reference's load_unique_points): d_rep[i]
   receives the lowest index j with the same coordinates as point i (-0.0
   equals +0.0), and *unique_points the number of distinct points.
   Limit: n <= 65536; larger n returns QDT_ERR_TOO_MANY_POINTS and does
   nothing. QDT_ERR_NULL_ARGUMENT for NULL pointers, QDT_ERR_NOT_FINITE for a
   NaN or infinite coordinate (d_rep is then not written), QDT_ERR_INTERNAL
   for a CUDA failure or a stream of another device than the current one.
   The work runs on cuda_stream (a cudaStream_t of the current device, NULL
   for the default stream); the call copies its status into host memory and
   waits for the stream before it returns.
   Its working memory (2.6 MB) is a static array of the library on each GPU,
   kept until the process exits and shared by every call: calls that overlap
   on the GPU race, so serialise them. The first call on a device looks up
   the array's device address; make that first call before any stream
   capture begins. */
QDT_API qdt_status qdtg_unique_points_noalloc(const qdt_vec2d* d_pts, size_t n, uint32_t* d_rep,
    size_t* unique_points, void* cuda_stream);

/* ------------------------------------------------------------------------
   Many sets in one call. The reference triangulates one point set per
   qdt_execute() call; a caller with thousands of independent sets (tiles,
   frames, meshes of many parts) makes thousands of calls. A qdtg_batch
   triangulates all of them in one GPU pipeline: set i is points
   [offsets[i], offsets[i + 1]) of pts, and its result is the one
   qdt_execute() gives for those points alone (triangles with indices local
   to the set, the same representatives and distinct count).
   ------------------------------------------------------------------------ */
typedef struct qdtg_batch qdtg_batch;

/* NULL when no GPU is usable. The batch keeps its device workspace, CUDA
   stream and recorded CUDA graphs between calls. */
QDT_API qdtg_batch* qdtg_batch_create(void);
QDT_API void        qdtg_batch_destroy(qdtg_batch* b);

/* Triangulates nsets sets of host points; offsets has nsets + 1 entries,
   offsets[0] = 0, non-decreasing, offsets[nsets] = total points
   (<= 100,000,000). Returns QDT_OK when the call ran (a set with a NaN or
   infinite coordinate then has status QDT_ERR_NOT_FINITE and no result,
   the others are complete), QDT_ERR_NULL_CONTEXT / QDT_ERR_NULL_ARGUMENT /
   QDT_ERR_TOO_MANY_POINTS for bad arguments, QDT_ERR_OUT_OF_MEMORY or
   QDT_ERR_INTERNAL otherwise (the batch is then empty). */
QDT_API qdt_status qdtg_batch_execute(qdtg_batch* b, const qdt_vec2d* pts, const size_t* offsets, size_t nsets);

/* The same for points resident on the device; the work waits for what is
   queued on cuda_stream. Triangles and representatives stay on the device:
   qdtg_batch_device_triangles(). */
QDT_API qdt_status qdtg_batch_execute_device(qdtg_batch* b, const qdt_vec2d* d_pts, const size_t* offsets,
    size_t nsets, void* cuda_stream);

/* Results of the last call, per set. */
QDT_API size_t     qdtg_batch_set_count(const qdtg_batch* b);
QDT_API qdt_status qdtg_batch_set_status(const qdtg_batch* b, size_t set);
/* Number of triangles of the set; *tris (if not NULL) points at 3 * count
   host indices local to the set (NULL after qdtg_batch_execute_device). */
QDT_API size_t qdtg_batch_triangles(const qdtg_batch* b, size_t set, const uint32_t** tris);
QDT_API size_t qdtg_batch_unique_points(const qdtg_batch* b, size_t set);
/* Representatives of the set's points (local indices), host memory. */
QDT_API const uint32_t* qdtg_batch_rep(const qdtg_batch* b, size_t set);
/* All triangles on the device: *d_tris = 3 * total indices (each set's
   local), *d_offsets = nsets + 1 triangle offsets. Returns the total. */
QDT_API size_t qdtg_batch_device_triangles(const qdtg_batch* b, const uint32_t** d_tris,
    const uint32_t** d_offsets);
/* Copies min(cap, total) device triangles to host memory out (3 indices
   each) and, if offsets_out is not NULL, the nsets + 1 triangle offsets;
   returns how many triangles it copied. */
QDT_API size_t qdtg_batch_download_device_triangles(const qdtg_batch* b, uint32_t* out, size_t cap,
    uint32_t* offsets_out);
/* Counting of filter failures, per-stage timing (CUDA events), CUDA graph
   replay of the launches after the distinct count (default on), and the
   smallest merge (in points) that runs one node per warp instead of one
   node per thread (0 keeps the current value; default 512). */
QDT_API void qdtg_batch_set_options(qdtg_batch* b, int count_filter_failures, int stage_timing, int use_graphs,
    int warp_min_points);
/* The heights (node sizes) merged with a warp per node are those whose nodes
   have at least warp_min_points points (qdtg_batch_set_options) or whose
   launch has at most warp_nodes nodes (default 4096). Returns 1, or 0 for a
   NULL batch or a negative value. */
QDT_API int qdtg_batch_set_warp_nodes(qdtg_batch* b, int warp_nodes);

/* The build of every set's tree as one persistent launch (on != 0): warps
   of blocks resident on every SM take work units (32 small nodes, or one
   large node) from a device counter, heights in increasing order, and a
   merge waits (bounded) for its children's done flags instead of for the
   end of a launch per height (the default, on == 0; faster on large
   batches). A batch with shared-memory cells runs per height. The result
   is the same. Returns 1, or 0 for a NULL batch or no usable GPU. No
   counterpart in the reference, which builds sets on host threads. */
QDT_API int qdtg_batch_set_persistent(qdtg_batch* b, int on);
/* The largest subtree (points, 4..1024; 0 = none) built in shared memory,
   as qdtg_set_cell_points(). Returns 1, or 0 for a bad value. */
QDT_API int   qdtg_batch_set_cell_points(qdtg_batch* b, int cell_points);
QDT_API int   qdtg_batch_get_run_info(const qdtg_batch* b, qdtg_run_info* info);
/* The same statistics as qdtg_get_filter_stats, for the last call of b. */
QDT_API int   qdtg_batch_get_filter_stats(const qdtg_batch* b, qdtg_filter_stats* stats);
QDT_API void* qdtg_batch_stream(const qdtg_batch* b);

/* Pre-allocates the batch's device workspace for up to `points` points in
   `sets` sets (the workspace otherwise grows on demand), and reports the
   device bytes it holds. */
QDT_API qdt_status qdtg_batch_reserve(qdtg_batch* b, size_t points, size_t sets);
QDT_API size_t     qdtg_batch_workspace_bytes(const qdtg_batch* b);

/* ------------------------------------------------------------------------
   Serving: a request loop in front of resident GPU engines. No reference
   counterpart (the reference has only the synchronous per-call API).
   Requests of at least small_threshold points run on large_workers engines,
   each with its own CUDA stream and a device workspace kept between
   requests; smaller requests are coalesced, whenever the batching engine is
   free, into one many-set call (continuous batching). The device bytes of all
   workspaces stay within hbm_budget_bytes: a request waits until its
   engine's workspace fits (idle workspaces are freed to make room); one that
   cannot fit alone, or that finds max_queue requests waiting, is rejected.
   Each result is the one qdt_execute() gives for the request alone.
   ------------------------------------------------------------------------ */
typedef struct qdtg_server qdtg_server;

typedef struct qdtg_server_config
{
    size_t hbm_budget_bytes;   /* default 150 GiB */
    int    large_workers;      /* engines for large requests, 1..64; default 4 */
    size_t small_threshold;    /* requests below this many points are coalesced; default 65536 (0: none) */
    size_t batch_max_points;   /* points per coalesced batch; default 8 Mi */
    size_t batch_max_sets;     /* requests per coalesced batch; default 4096 */
    size_t max_queue;          /* waiting requests beyond which new ones are rejected; default 4096 */
    int    cell_points;        /* engines: as qdtg_set_cell_points; default from qdtg_set_defaults */
    int    batch_cell_points;  /* batching engine: as qdtg_batch_set_cell_points; likewise */
} qdtg_server_config;

typedef struct qdtg_server_stats
{
    unsigned long long submitted, completed, rejected, queued;
    unsigned long long batches, batched_requests, pool_releases;
    size_t             resident_bytes, peak_resident_bytes, hbm_budget_bytes;
    size_t             waiting;     /* requests not yet started */
} qdtg_server_stats;

QDT_API void qdtg_server_default_config(qdtg_server_config* config);
/* Starts the worker threads; NULL on bad configuration or no usable GPU. */
QDT_API qdtg_server* qdtg_server_create(const qdtg_server_config* config);
/* Finishes every accepted request, then stops the workers and frees all. */
QDT_API void qdtg_server_destroy(qdtg_server* srv);
/* Queues a request for n points. The points are read while the request runs:
   keep them unchanged until it is done. *ticket identifies the request (also
   a rejected one). Returns QDT_OK when accepted, QDT_ERR_OUT_OF_MEMORY when
   rejected by the budget or the queue limit, or an argument error (then
   *ticket is 0). */
QDT_API qdt_status qdtg_server_submit(qdtg_server* srv, const qdt_vec2d* pts, size_t n, uint64_t* ticket);
/* Waits until the request is done: 1 done, 0 timed out (timeout_s < 0 waits
   without limit), -1 unknown ticket. */
QDT_API int qdtg_server_wait(qdtg_server* srv, uint64_t ticket, double timeout_s);
/* The request's status (its qdt_execute() status) and results: triangles (3
   indices each), representatives, distinct count; valid until released. */
QDT_API qdt_status qdtg_server_result(qdtg_server* srv, uint64_t ticket, const uint32_t** tris, size_t* ntri,
    const uint32_t** rep, size_t* unique_points);
/* Milliseconds from submission to start, start to done, submission to done;
   path 0 = own engine, 1 = coalesced batch. Returns 0 unless done. */
QDT_API int qdtg_server_timing(qdtg_server* srv, uint64_t ticket, double* queue_ms, double* run_ms,
    double* total_ms, int* path);
/* Frees a done request's results; returns 1, or 0 if unknown or not done. */
QDT_API int  qdtg_server_release(qdtg_server* srv, uint64_t ticket);
QDT_API void qdtg_server_get_stats(qdtg_server* srv, qdtg_server_stats* stats);

/* Library version string. */
QDT_API const char* qdtg_version(void);

#if __cplusplus
}
#endif

#endif
