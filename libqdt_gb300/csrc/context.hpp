// The object behind qdt_t: what the reference keeps in wrapper::Triangulation
// (wrapper.hxx:17-23 -- triangles, rep, unique_points, input_points), stored
// as 32-bit indices in page-locked host memory so that the GPU results land
// there directly, plus the engine and the lazily built mesh used by the
// incremental insertion and the constraints.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

#include "engine.hpp"

namespace qdtg {

constexpr size_t kMaxPoints = 100000000;   // reference wrapper.hxx:15

struct Mesh;

struct Context
{
    PinnedVec<double>   points;     // 2 per point: x, y (input order, then insertions)
    PinnedVec<uint32_t> rep;        // lowest index with the same coordinates
    PinnedVec<uint32_t> tris;       // 3 per triangle, counter-clockwise
    size_t              unique_points = 0;
    Engine*             engine = nullptr;
    int                 last_cuda_error = 0;
    Mesh*               mesh = nullptr;    // built on the first insertion or constraint
    bool                mesh_on_gpu = true;   // build that mesh on the GPU when the engine holds the result

    size_t npoints() const { return points.size() / 2; }
    size_t ntris() const { return tris.size() / 3; }

    // The empty state: no points, no triangles, no constraints, no mesh.
    // Does not allocate and does not throw.
    void reset() noexcept;
    // reset() and release host memory (after an allocation failure)
    void reset_release() noexcept;

    ~Context();
};

// Runs the batch engine on the context's own points (used by the insertion
// when it rebuilds). Returns a qdt_status value.
int rebuild_from_points(Context& c);

// mesh.cu -- incremental insertion and constrained edges on the host.
// Both may throw std::bad_alloc; they return a qdt_status value otherwise.
// hint: a half-edge to start the point location from (-1: the last insertion)
int  mesh_insert_point(Context& c, double x, double y, bool parallel_build, int hint = -1);
int  mesh_insert_constraint(Context& c, size_t v0, size_t v1);
// Locates k points (x, y pairs, finite) in the current triangulation: per
// point the smallest index of a triangle containing it (border included) or
// -1, its class (mesh_walk.cuh LocClass: -1 outside, 0 inside, 1 on an edge,
// 2 on a vertex), and, if he is not NULL, a half-edge next to it (a start
// for the walk of a later insertion). Runs on the GPU when the context has
// an engine; walks the device gives up on finish on the host.
int  mesh_locate(Context& c, const double* xy, size_t k, int* tri, int* where, int* he);
// Walk starts for inserting k points in order (-1: none): their locations in
// the current mesh, found on the GPU when that pays. A hint only shortens the
// walk; the insertion result does not depend on it.
std::vector<int> mesh_insert_hints(Context& c, const double* xy, size_t k);
// For k constraints (v0, v1 pairs), each on its own against the current
// triangulation: the status mesh_insert_constraint would return for it as
// the next call, and the number of edges its segment crosses before the
// decision (the edges the insertion would flip when it is accepted). The
// traces run on the GPU. Returns QDT_OK or the status of a device failure.
int mesh_trace_segments(Context& c, const size_t* v01, size_t k, int* status, int64_t* crossed);
void mesh_destroy(Mesh* m) noexcept;

}  // namespace qdtg
