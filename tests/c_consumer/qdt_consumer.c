/*
 * A C client of the qdt.h interface, compiled with a C compiler against
 * include/qdt.h and linked against the GB300 library exactly as a program
 * written for the reference library links against it. TEST INFRASTRUCTURE:
 * tests/test_c_consumer.py builds and runs it.
 *
 * It checks the interface contract a caller relies on (the reference
 * header's documentation, qdt.h:38-401): NULL handling, status strings,
 * queries on const contexts, duplicate handling, what empties a context,
 * the constraint rules, that the caller's array is neither kept nor
 * modified, a known triangulation (the six-point listing of the reference
 * README), and independent contexts used from several threads at once.
 *
 *   qdt_consumer            all checks (needs a GPU for the batch calls)
 *   qdt_consumer --no-gpu   only the checks that make no batch call
 *
 * Prints one line per failed check and "qdt_consumer: N checks, M failed";
 * exits 0 when none failed.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "qdt.h"

static int g_checks = 0, g_failed = 0;

static void check(int ok, const char* what)
{
    ++g_checks;
    if (!ok)
    {
        ++g_failed;
        printf("FAILED: %s\n", what);
    }
}

static void no_context(void)
{
    size_t    idx = 41;
    qdt_vec2d p = { 1.0, 2.0 };
    check(qdt_execute(NULL, NULL, 0) == QDT_ERR_NULL_CONTEXT, "execute on NULL context");
    check(qdt_execute_parallel(NULL, NULL, 0) == QDT_ERR_NULL_CONTEXT, "execute_parallel on NULL context");
    check(qdt_insert_point(NULL, p, &idx) == QDT_ERR_NULL_CONTEXT && idx == 41, "insert_point on NULL context");
    check(qdt_insert_point_parallel(NULL, p, &idx) == QDT_ERR_NULL_CONTEXT && idx == 41,
        "insert_point_parallel on NULL context");
    check(qdt_insert_constraint(NULL, 0, 1) == QDT_ERR_NULL_CONTEXT, "insert_constraint on NULL context");
    {
        qdt_edge   e[3] = { { 0, 1 }, { 1, 2 }, { 2, 0 } };
        qdt_status r[3] = { QDT_OK, QDT_OK, QDT_OK };
        check(qdt_insert_constraints_batch(NULL, e, 3, r) == QDT_ERR_NULL_CONTEXT && r[0] == QDT_ERR_NULL_CONTEXT &&
                  r[1] == QDT_ERR_NULL_CONTEXT && r[2] == QDT_ERR_NULL_CONTEXT,
            "constraints_batch on NULL context fills every result");
    }
    {
        size_t    t[3] = { 5, 6, 7 };
        qdt_vec2d q = { 3.0, 4.0 };
        check(qdt_triangles_size(NULL) == 0 && qdt_points_size(NULL) == 0, "sizes of NULL context");
        check(qdt_get_triangle(NULL, t, 0) == 0 && t[0] == 5 && t[2] == 7, "get_triangle on NULL context");
        check(qdt_get_point(NULL, &q, 0) == 0 && q.x == 3.0 && q.y == 4.0, "get_point on NULL context");
        check(qdt_point_is_used(NULL, 0) == 0, "point_is_used on NULL context");
    }
    qdt_destroy(NULL);
}

static void statuses(void)
{
    int s, t, distinct = 1;
    for (s = QDT_ERR_INTERNAL; s <= QDT_OK; ++s)
    {
        const char* a = qdt_status_string((qdt_status)s);
        distinct = distinct && a && strcmp(a, "unknown status") != 0;
        for (t = QDT_ERR_INTERNAL; t < s; ++t) distinct = distinct && strcmp(a, qdt_status_string((qdt_status)t)) != 0;
    }
    check(distinct, "every status has its own text");
    check(strcmp(qdt_status_string((qdt_status)4242), "unknown status") == 0, "text of an undefined status");
}

static void fresh_context(void)
{
    qdt_t*     q = qdt_create();
    qdt_edge   e = { 0, 1 };
    qdt_status r[2] = { QDT_OK, QDT_OK };
    qdt_vec2d  one = { 0.0, 0.0 };
    check(q != NULL, "create");
    check(qdt_triangles_size(q) == 0 && qdt_points_size(q) == 0, "a new context is empty");
    check(qdt_insert_constraint(q, 0, 1) == QDT_ERR_INVALID_INDEX, "constraint on an empty context");
    check(qdt_insert_constraints_batch(q, &e, 1, r) == QDT_ERR_INVALID_INDEX && r[0] == QDT_ERR_INVALID_INDEX,
        "constraints_batch on an empty context");
    r[0] = r[1] = QDT_OK;
    check(qdt_insert_constraints_batch(q, NULL, 2, r) == QDT_ERR_NULL_ARGUMENT && r[0] == QDT_ERR_NULL_ARGUMENT &&
              r[1] == QDT_ERR_NULL_ARGUMENT,
        "constraints_batch with NULL edges");
    r[0] = QDT_ERR_INTERNAL;
    check(qdt_insert_constraints_batch(q, NULL, 0, r) == QDT_OK && r[0] == QDT_ERR_INTERNAL,
        "constraints_batch with no edges writes nothing");
    /* checks made before any batch work */
    check(qdt_execute(q, NULL, 3) == QDT_ERR_NULL_ARGUMENT, "execute with NULL points");
    check(qdt_execute(q, &one, (size_t)100000001) == QDT_ERR_TOO_MANY_POINTS, "execute with more than 1e8 points");
    check(qdt_execute(q, NULL, (size_t)100000001) == QDT_ERR_TOO_MANY_POINTS, "the count is checked before NULL");
    check(qdt_triangles_size(q) == 0 && qdt_points_size(q) == 0, "a rejected batch leaves the context empty");
    qdt_destroy(q);
}

static size_t find_triangle(const qdt_t* q, size_t a, size_t b, size_t c)
{
    size_t i, n = qdt_triangles_size(q), t[3];
    for (i = 0; i < n; ++i)
    {
        int k;
        if (!qdt_get_triangle(q, t, i)) return 0;
        for (k = 0; k < 3; ++k)
            if (t[k] == a && t[(k + 1) % 3] == b && t[(k + 2) % 3] == c) return 1;
    }
    return 0;
}

static void batch_contract(void)
{
    const qdt_vec2d quad[4] = { { 0, 0 }, { 4, 0 }, { 3, 1 }, { 1, 1 } };
    qdt_vec2d       mine[4];
    qdt_t*          q = qdt_create();
    const qdt_t*    cq = q;
    size_t          t[3] = { 9, 9, 9 }, i, idx = 0;
    qdt_vec2d       got = { -1, -1 };
    int             all = 1;

    memcpy(mine, quad, sizeof mine);
    check(qdt_execute(q, mine, 4) == QDT_OK, "execute on a quadrilateral");
    check(memcmp(mine, quad, sizeof mine) == 0, "the caller's array is not modified");
    mine[0].x = 100.0;   /* the context keeps its own copy */
    check(qdt_get_point(cq, &got, 0) == 1 && got.x == 0.0 && got.y == 0.0, "points are copied, not kept");
    check(qdt_triangles_size(cq) == 2 && qdt_points_size(cq) == 4, "two triangles, four points");
    check(qdt_get_triangle(cq, t, 0) == 1 && qdt_get_triangle(cq, NULL, 0) == 0, "get_triangle");
    check(qdt_get_triangle(cq, t, 2) == 0, "get_triangle out of range");
    check(qdt_get_point(cq, &got, 2) == 1 && got.x == 3.0 && got.y == 1.0, "get_point");
    got.x = got.y = -7.0;
    check(qdt_get_point(cq, &got, 4) == 0 && got.x == -7.0 && qdt_get_point(cq, NULL, 0) == 0, "get_point out of range");
    for (i = 0; i < 4; ++i) all = all && qdt_point_is_used(cq, i) == 1;
    check(all && qdt_point_is_used(cq, 4) == 0, "point_is_used on the quadrilateral");

    /* the constraint rules, and their replacement by the next batch call */
    check(qdt_insert_constraint(q, 0, 77) == QDT_ERR_INVALID_INDEX, "constraint with an invalid index");
    check(qdt_insert_constraint(q, (size_t)-1, 0) == QDT_ERR_INVALID_INDEX, "constraint with index SIZE_MAX");
    check(qdt_insert_constraint(q, 1, 1) == QDT_ERR_SAME_POINT, "constraint between one point");
    check(qdt_insert_constraint(q, 0, 2) == QDT_OK, "constraint across the quadrilateral");
    check(find_triangle(cq, 2, 0, 1) && find_triangle(cq, 0, 2, 3), "the quadrilateral after its constraint");
    check(qdt_insert_constraint(q, 2, 0) == QDT_OK, "the same constraint reversed");
    check(qdt_insert_constraint(q, 1, 3) == QDT_ERR_CROSSES_CONSTRAINT, "a crossing constraint is refused");
    check(qdt_execute(q, quad, 4) == QDT_OK && qdt_insert_constraint(q, 1, 3) == QDT_OK,
        "a batch call discards earlier constraints");

    /* duplicates: the lowest index represents them */
    {
        const qdt_vec2d dup[5] = { { 0, 0 }, { 1, 0 }, { 0, 0 }, { 0, 1 }, { 1, 0 } };
        const size_t    want[5] = { 1, 1, 0, 1, 0 };
        int             ok = 1;
        check(qdt_execute(q, dup, 5) == QDT_OK && qdt_points_size(q) == 5 && qdt_triangles_size(q) == 1,
            "duplicates: one triangle over five points");
        for (i = 0; i < 5; ++i) ok = ok && qdt_point_is_used(q, i) == want[i];
        check(ok, "duplicates: used flags");
        check(qdt_insert_point(q, (qdt_vec2d){ 0.0, 1.0 }, &idx) == QDT_OK && idx == 5 && qdt_point_is_used(q, 5) == 0,
            "inserting a duplicate returns a new, unused index");
        check(qdt_insert_constraint(q, 5, 3) == QDT_ERR_SAME_POINT, "a constraint between duplicates");
        check(qdt_insert_point(q, (qdt_vec2d){ 2.0, 2.0 }, &idx) == QDT_OK && idx == 6 && qdt_point_is_used(q, 6) == 1,
            "inserting a new point");
        check(qdt_insert_constraint(q, 6, 5) == QDT_OK, "a constraint through a duplicate's index");
    }

    /* degenerate inputs: no triangles, so no constraints */
    {
        const qdt_vec2d line[3] = { { 0, 0 }, { 1, 1 }, { 2, 2 } };
        const qdt_edge  e = { 0, 2 };
        qdt_status      r = QDT_OK;
        check(qdt_execute(q, line, 3) == QDT_OK && qdt_triangles_size(q) == 0 && qdt_points_size(q) == 3,
            "collinear points give no triangles");
        check(qdt_insert_constraint(q, 0, 2) == QDT_ERR_NO_TRIANGLES &&
                  qdt_insert_constraints_batch(q, &e, 1, &r) == QDT_ERR_NO_TRIANGLES && r == QDT_ERR_NO_TRIANGLES,
            "constraints on collinear points");
        check(qdt_point_is_used(q, 0) == 0, "no point of a collinear input is used");
    }

    /* a rejected batch empties the context */
    {
        qdt_vec2d bad[4] = { { 0, 0 }, { 1, 0 }, { 0, 1 }, { 0.5, 0.5 } };
        bad[3].y = NAN;
        check(qdt_execute(q, quad, 4) == QDT_OK && qdt_triangles_size(q) == 2, "a good batch");
        check(qdt_execute(q, bad, 4) == QDT_ERR_NOT_FINITE, "a NaN coordinate is refused");
        check(qdt_triangles_size(q) == 0 && qdt_points_size(q) == 0, "and the context is empty after it");
        check(qdt_execute(q, quad, 4) == QDT_OK && qdt_triangles_size(q) == 2, "and usable again");
        check(qdt_execute(q, NULL, 0) == QDT_OK && qdt_points_size(q) == 0, "an empty batch");
    }

    /* the six-point listing of the reference README: four corners, then
       (0.5, 0.5) and (0.25, 0.75) inserted */
    {
        const qdt_vec2d sq[4] = { { 0, 0 }, { 1, 0 }, { 0, 1 }, { 1, 1 } };
        const size_t    want[6][3] = { { 1, 3, 4 }, { 0, 1, 4 }, { 2, 0, 5 }, { 0, 4, 5 }, { 4, 3, 5 }, { 3, 2, 5 } };
        size_t          a = 0, b = 0;
        int             ok = 1;
        check(qdt_execute(q, sq, 4) == QDT_OK, "the unit square");
        check(qdt_insert_point(q, (qdt_vec2d){ 0.5, 0.5 }, &a) == QDT_OK && a == 4, "insert (0.5, 0.5)");
        check(qdt_insert_point_parallel(q, (qdt_vec2d){ 0.25, 0.75 }, &b) == QDT_OK && b == 5, "insert (0.25, 0.75)");
        for (i = 0; i < 6; ++i) ok = ok && find_triangle(q, want[i][0], want[i][1], want[i][2]);
        check(ok && qdt_triangles_size(q) == 6, "the six-point listing");
    }
    qdt_destroy(q);
}

/* independent contexts from several threads at once */
struct job
{
    unsigned seed;
    size_t   n, triangles;
    int      status, parallel;
};

static double next_unit(unsigned long long* s)
{
    unsigned long long z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

static void* run_job(void* arg)
{
    struct job*        j = (struct job*)arg;
    unsigned long long s = j->seed;
    qdt_vec2d*         p = (qdt_vec2d*)malloc(j->n * sizeof(qdt_vec2d));
    qdt_t*             q = qdt_create();
    size_t             i;
    for (i = 0; i < j->n; ++i)
    {
        p[i].x = next_unit(&s);
        p[i].y = next_unit(&s);
    }
    j->status = j->parallel ? qdt_execute_parallel(q, p, j->n) : qdt_execute(q, p, j->n);
    j->triangles = qdt_triangles_size(q);
    qdt_destroy(q);
    free(p);
    return NULL;
}

static void threads(void)
{
    enum { T = 6 };
    pthread_t  th[T];
    struct job jobs[T], again[T];
    int        i, ok = 1;
    for (i = 0; i < T; ++i)
    {
        jobs[i].seed = 1000u + (unsigned)i;
        jobs[i].n = 20000 + 7919 * (size_t)i;
        jobs[i].parallel = i & 1;
        pthread_create(&th[i], NULL, run_job, &jobs[i]);
    }
    for (i = 0; i < T; ++i) pthread_join(th[i], NULL);
    for (i = 0; i < T; ++i)
    {
        again[i] = jobs[i];
        run_job(&again[i]);   /* the same input alone */
        ok = ok && jobs[i].status == QDT_OK && jobs[i].triangles == again[i].triangles && jobs[i].triangles > 0;
    }
    check(ok, "contexts used from six threads at once give what each gives alone");
}

int main(int argc, char** argv)
{
    const int no_gpu = argc > 1 && strcmp(argv[1], "--no-gpu") == 0;
    no_context();
    statuses();
    fresh_context();
    if (!no_gpu)
    {
        batch_contract();
        threads();
    }
    printf("qdt_consumer: %d checks, %d failed\n", g_checks, g_failed);
    return g_failed ? 1 : 0;
}
