/*
 * Bulk read-back of a qdt.h context through its public query functions
 * (qdt_triangles_size, qdt_get_triangle, qdt_points_size,
 * qdt_point_is_used). TEST INFRASTRUCTURE: it lets the fixture generator read
 * millions of triangles from the reference library without a Python call
 * per triangle. It is linked against whichever library implements qdt.h.
 */
#include <stddef.h>
#include <stdint.h>

typedef struct qdt_t qdt_t;
size_t qdt_triangles_size(const qdt_t* ptr);
size_t qdt_get_triangle(const qdt_t* ptr, size_t T[3], size_t id);
size_t qdt_points_size(const qdt_t* ptr);
size_t qdt_point_is_used(const qdt_t* ptr, size_t id);

/* Writes 3 * qdt_triangles_size(q) indices; returns the triangle count. */
size_t qdt_dump_triangles(const qdt_t* q, int64_t* out)
{
    const size_t n = qdt_triangles_size(q);
    for (size_t i = 0; i < n; ++i)
    {
        size_t T[3] = { 0, 0, 0 };
        qdt_get_triangle(q, T, i);
        out[3 * i + 0] = (int64_t)T[0];
        out[3 * i + 1] = (int64_t)T[1];
        out[3 * i + 2] = (int64_t)T[2];
    }
    return n;
}

/* Writes qdt_points_size(q) flags; returns the point count. */
size_t qdt_dump_used(const qdt_t* q, uint8_t* out)
{
    const size_t n = qdt_points_size(q);
    for (size_t i = 0; i < n; ++i) out[i] = (uint8_t)qdt_point_is_used(q, i);
    return n;
}
