// A device copy of the handle's half-edge mesh, used to locate many points at
// once (k_locate.cu). The GPU mesh build leaves its arrays here; after the
// host changes the mesh (insertions, constraints) the next location uploads
// it again. A uniform grid of seeds (per cell, an alive half-edge whose
// origin lies in the cell) gives every walk a start next to its point.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "mesh_layout.hpp"

namespace qdtg {

struct MeshMirror
{
    MeshVertex*         v = nullptr;
    MeshHalfEdge*       h = nullptr;
    int*                seed = nullptr;   // per grid cell, -1 when no vertex lies in it
    unsigned long long* box = nullptr;    // 4 order keys: min x, min y, max x, max y; then [4] = any alive half-edge
    double2*            q = nullptr;      // query points
    int4*               out = nullptr;    // per query: triangle, class, half-edge
    size_t              cap_v = 0, cap_h = 0, cap_seed = 0, cap_q = 0;
    size_t              nv = 0, nh = 0;
    int                 gx = 0, gy = 0;
    double              x0 = 0, y0 = 0, ix = 0, iy = 0;   // grid origin and cells per unit length
    bool                indexed = false;
    uint64_t            mesh_id = 0, mesh_version = ~0ull;   // the host mesh state it holds
};

// Grows the vertex and half-edge arrays to hold nv and nh entries (contents
// are not kept). 0 or -1.
int  mirror_reserve(MeshMirror& m, size_t nv, size_t nh);
void mirror_free(MeshMirror& m) noexcept;
// Copies a host mesh in and marks it unindexed. 0 or -1.
int  mirror_upload(MeshMirror& m, const MeshVertex* v, size_t nv, const MeshHalfEdge* h, size_t nh, cudaStream_t s);
// Locates k points (x, y pairs, all finite) in the mirrored mesh: per point
// the canonical triangle, its class (LocClass) and the half-edge the walk
// ended on. Points the device walk gives up on come back as kLocUnresolved.
// 0 or -1.
int  mirror_locate(MeshMirror& m, const double* xy, size_t k, int* tri, int* where, int* he, cudaStream_t s);
// Traces k constraint segments (mesh vertex pairs u, w; u != w) through the
// mirrored mesh: per segment the TraceClass (mesh_walk.cuh) and the edges
// crossed. Segments the device gives up on come back as kTraceUnresolved.
// 0 or -1.
int  mirror_trace(MeshMirror& m, const int* uw, size_t k, int* outcome, int* crossed, cudaStream_t s);

}  // namespace qdtg
