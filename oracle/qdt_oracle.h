/*
 * CPU oracle for the batch Delaunay path -- TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference's batch triangulation
 * (libqdt: load_unique_points, the Guibas-Stolfi/Dwyer builder, the robust
 * predicates, the serial and the threaded drivers). It exists to check the
 * CUDA path and to time the reference's algorithm on the host cores. Only the
 * test-suite, the smoke check and the CPU-baseline leg of the benchmark may
 * load it; the product library never links or calls it.
 *
 * Parity of this restatement is pinned against the reference itself
 * (compiled from its own sources into oracle/_ref by oracle/build_ref.sh) and
 * against the reference's published known answers; see tests/test_oracle.py.
 */
#ifndef QDT_ORACLE_H_
#define QDT_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Counters of one triangulation (filter failures = calls that took the exact
   fallback). */
typedef struct qdo_stats
{
    uint64_t orient_calls;
    uint64_t orient_exact;
    uint64_t incircle_calls;
    uint64_t incircle_exact;
    uint64_t records_used;   /* quad-edge records handed out (high-water) */
    int      threaded_used;  /* 1 if the threaded builder ran */
    int      fell_back;      /* 1 if the threaded builder fell back to serial */
} qdo_stats;

typedef struct qdo_result
{
    uint32_t* tris;          /* 3 * ntri original point indices, CCW */
    size_t    ntri;
    uint32_t* rep;           /* n entries: lowest index with equal coordinates */
    size_t    n;
    size_t    unique_points;
    qdo_stats stats;
} qdo_result;

/* Status codes follow qdt.h (0 = OK, negative = error). */
int qdo_check_input(const double* xy, size_t n);

/* Triangulates n points given as interleaved (x, y) doubles. threaded = 0
   follows the serial driver, 1 the threaded one (pthreads, nthreads workers,
   0 = hardware concurrency capped at 64). Returns a qdt_status value. */
int  qdo_triangulate(const double* xy, size_t n, int threaded, int nthreads, qdo_result* out);
void qdo_result_free(qdo_result* r);

/* The robust predicates (sign only: -1, 0, +1), as used by the builder. */
int qdo_orient2d(const double* a, const double* b, const double* c);
int qdo_incircle(const double* a, const double* b, const double* c, const double* d);
/* Same, but always through the exact expansion path. */
int qdo_orient2d_exact(const double* a, const double* b, const double* c);
int qdo_incircle_exact(const double* a, const double* b, const double* c, const double* d);

/* Batched exact signs (used by the Delaunay checker). */
void qdo_orient_batch(const double* xy, const int64_t* idx, size_t k, int8_t* out);
void qdo_incircle_batch(const double* xy, const int64_t* idx, size_t k, int8_t* out);

#ifdef __cplusplus
}
#endif

#endif
