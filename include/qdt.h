/*
 * qdt.h -- the C interface of the GB300 implementation of libqdt.
 *
 * Drop-in for the reference's public header (libqdt/qdt.h): the same types,
 * the same 14 functions with the same signatures, the same status codes and
 * the same error and reset semantics. Programs written against the reference
 * header compile and link against this library unchanged.
 *
 * What differs is the engine behind qdt_execute() and qdt_execute_parallel():
 * the batch triangulation runs on the GPU (CUDA, sm_103a). Both functions
 * produce the same set of triangles as the reference's qdt_execute().
 * Additional GPU-specific entry points live in qdt_gpu.h; this header is not
 * extended.
 */
#if !defined(_LIB_QDT_H_)
#define _LIB_QDT_H_

#include <stddef.h>

/* reference qdt.h:12-20 */
#if defined(_WIN32)
#if defined(QDT_DLL)
#define QDT_API __declspec(dllexport)
#else
#define QDT_API __declspec(dllimport)
#endif
#else
#define QDT_API __attribute__((visibility("default")))
#endif

#if __cplusplus
extern "C"
{
#endif

/* A point with double coordinates (reference qdt.h:38-43). Coordinates must
   be finite. The geometric decisions are exact for every finite double input,
   subnormal numbers included. */
struct qdt_vec2d
{
    double x;
    double y;
};
typedef struct qdt_vec2d qdt_vec2d;

/* The end points of a constraint, as point indices (reference qdt.h:48-53). */
struct qdt_edge
{
    size_t v0;
    size_t v1;
};
typedef struct qdt_edge qdt_edge;

/* Result codes (reference qdt.h:79-93). 0 is success, errors are negative.
   What an error does to the context is the same as in the reference:
   - unchanged: QDT_ERR_NULL_CONTEXT from any function; QDT_ERR_NOT_FINITE and
     QDT_ERR_TOO_MANY_POINTS from the point insertions; QDT_ERR_NULL_ARGUMENT
     from qdt_insert_constraints_batch(); every rejection of a constraint;
   - emptied: QDT_ERR_TOO_MANY_POINTS, QDT_ERR_NULL_ARGUMENT and
     QDT_ERR_NOT_FINITE from the batch calls, and QDT_ERR_OUT_OF_MEMORY and
     QDT_ERR_INTERNAL from any function. */
typedef enum qdt_status
{
    QDT_OK = 0,
    QDT_ERR_NULL_CONTEXT = -1,
    QDT_ERR_NULL_ARGUMENT = -2,
    QDT_ERR_TOO_MANY_POINTS = -3,
    QDT_ERR_NOT_FINITE = -4,
    QDT_ERR_INVALID_INDEX = -5,
    QDT_ERR_SAME_POINT = -6,
    QDT_ERR_NO_TRIANGLES = -7,
    QDT_ERR_CROSSES_CONSTRAINT = -8,
    QDT_ERR_THROUGH_POINT = -9,
    QDT_ERR_OUT_OF_MEMORY = -10,
    QDT_ERR_INTERNAL = -11
} qdt_status;

/* Short English description of a status; "unknown status" for other values
   (reference qdt.h:102, qdt.cpp:145-163). */
QDT_API const char* qdt_status_string(qdt_status status);

/* Opaque triangulation context (reference qdt.h:125). One context must not be
   used by several threads at once; different contexts are independent. A NULL
   context is safe everywhere: status functions return QDT_ERR_NULL_CONTEXT,
   queries return 0. No C++ exception crosses this interface. */
typedef struct qdt_t qdt_t;

/* A new empty context, or NULL when its memory cannot be allocated
   (reference qdt.h:133). No GPU resource is taken before the first batch
   call. */
QDT_API qdt_t* qdt_create(void);

/* Delaunay triangulation of pts[0..n) (reference qdt.h:160). Replaces the
   context's contents. Input checks in order: more than 100000000 points
   (QDT_ERR_TOO_MANY_POINTS), pts NULL with n > 0 (QDT_ERR_NULL_ARGUMENT), a
   NaN or infinite coordinate (QDT_ERR_NOT_FINITE); a rejected call leaves the
   context empty. Indices refer to positions in pts; of several points with
   equal coordinates only the lowest index is used; fewer than three distinct
   points or all points collinear give no triangles. pts is copied. */
QDT_API qdt_status qdt_execute(qdt_t* ptr, const qdt_vec2d* pts, size_t n);

/* Same result set as qdt_execute() (reference qdt.h:181). On this
   implementation both run the same GPU engine. */
QDT_API qdt_status qdt_execute_parallel(qdt_t* ptr, const qdt_vec2d* pts, size_t n);

/* Inserts one point incrementally (reference qdt.h:219). Rejected points
   (QDT_ERR_NOT_FINITE, QDT_ERR_TOO_MANY_POINTS) change nothing. index, if not
   NULL, receives the new point's index on success. */
QDT_API qdt_status qdt_insert_point(qdt_t* ptr, qdt_vec2d pt, size_t* index);

/* Same as qdt_insert_point() (reference qdt.h:234). */
QDT_API qdt_status qdt_insert_point_parallel(qdt_t* ptr, qdt_vec2d pt, size_t* index);

/* Makes the segment v0-v1 a constrained edge (reference qdt.h:282). Checks in
   order: QDT_ERR_INVALID_INDEX, QDT_ERR_SAME_POINT, QDT_ERR_NO_TRIANGLES,
   then QDT_ERR_CROSSES_CONSTRAINT or QDT_ERR_THROUGH_POINT. A rejection
   changes nothing. */
QDT_API qdt_status qdt_insert_constraint(qdt_t* ptr, size_t v0, size_t v1);

/* qdt_insert_constraint() for each entry in order (reference qdt.h:312).
   results, if not NULL, receives each entry's status. */
QDT_API qdt_status qdt_insert_constraints_batch(qdt_t* ptr, const qdt_edge* edges, size_t num_edges,
    qdt_status* results);

/* Number of triangles; 0 for NULL (reference qdt.h:325). */
QDT_API size_t qdt_triangles_size(const qdt_t* ptr);

/* Copies triangle id's three point indices, counter-clockwise, into T and
   returns 1; returns 0 (T untouched) for a bad id or NULL arguments
   (reference qdt.h:349). */
QDT_API size_t qdt_get_triangle(const qdt_t* ptr, size_t T[3], size_t id);

/* Number of points, duplicates included; 0 for NULL (reference qdt.h:364). */
QDT_API size_t qdt_points_size(const qdt_t* ptr);

/* Copies point id's coordinates and returns 1, or returns 0 (reference
   qdt.h:377). */
QDT_API size_t qdt_get_point(const qdt_t* ptr, qdt_vec2d* pt, size_t id);

/* 1 if a triangle references point id (reference qdt.h:394). */
QDT_API size_t qdt_point_is_used(const qdt_t* ptr, size_t id);

/* Releases the context and its host and device resources; NULL is allowed
   (reference qdt.h:401). */
QDT_API void qdt_destroy(qdt_t* ptr);

#if __cplusplus
}
#endif

#endif
