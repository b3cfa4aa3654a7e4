// The half-edge mesh of a triangulation, as the handle operations use it
// (mesh.cu) and as the GPU builds it (k_mesh.cu): one layout for both, so that
// the device result is copied into the host mesh as it is.
#pragma once

#include <cstdint>
#include <memory>
#include <new>
#include <utility>
#include <vector>

namespace qdtg {

// An allocator whose resize() leaves new elements uninitialised: the mesh
// arrays are filled by a device copy right after they are sized.
template <class T>
struct NoInitAllocator : std::allocator<T>
{
    template <class U>
    struct rebind
    {
        using other = NoInitAllocator<U>;
    };
    NoInitAllocator() = default;
    template <class U>
    NoInitAllocator(const NoInitAllocator<U>&) noexcept
    {
    }
    template <class U>
    void construct(U* p) noexcept
    {
        ::new (static_cast<void*>(p)) U;
    }
    template <class U, class... A>
    void construct(U* p, A&&... a)
    {
        ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
    }
};

template <class T>
using MeshVec = std::vector<T, NoInitAllocator<T>>;

struct MeshVertex
{
    double   x, y;
    uint32_t orig;   // point index in the context
    int      he;     // an outgoing half-edge (after a build the first one in triangle order)
};

struct MeshHalfEdge
{
    int org;    // mesh vertex
    int twin;   // -1 on the hull
    int next;   // next half-edge of the same triangle (counter-clockwise)
    int tri;    // triangle index in the context's list
    int cons;   // nonzero: a constrained edge
};

static_assert(sizeof(MeshVertex) == 24, "mesh vertex layout");
static_assert(sizeof(MeshHalfEdge) == 20, "mesh half-edge layout");

}  // namespace qdtg
