/*
 * oracle_bench.c -- TEST INFRASTRUCTURE ONLY (CPU baseline driver).
 *
 * Runs the CPU restatement over independent frame pairs on several host
 * threads, one estimator state per thread, the way a multi-stream encoder
 * would use the reference (which has no internal threading).
 */
#include <pthread.h>
#include <stdlib.h>
#include "oracle_internal.h"

typedef struct {
    const short* const* srcs;
    const short* const* refs;
    int nframes, w, h, motion_range, rc;
    int* next;  /* shared work counter: pairs are taken in order as threads free up */
    short* mv_out;
} me_job;

static void* me_worker(void* arg)
{
    me_job* j = (me_job*)arg;
    int nmb = vo_num_mbs(j->w, j->h);
    for (int f = __atomic_fetch_add(j->next, 1, __ATOMIC_RELAXED); f < j->nframes;
         f = __atomic_fetch_add(j->next, 1, __ATOMIC_RELAXED)) {
        long avg;
        int rc = vo_me_full(j->srcs[f], j->refs[f], j->w, j->h, j->motion_range, NULL, NULL,
                            j->mv_out + (size_t)f * 2 * nmb, NULL, &avg);
        if (rc) j->rc = rc;
    }
    return NULL;
}

int vo_bench_me_full(const short* const* srcs, const short* const* refs, int nframes,
                     int w, int h, int motion_range, int nthreads, short* mv_out)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    me_job jobs[256];
    int next = 0;
    for (int t = 0; t < nthreads; t++) {
        me_job jb = {srcs, refs, nframes, w, h, motion_range, 0, &next, mv_out};
        jobs[t] = jb;
        if (pthread_create(&th[t], NULL, me_worker, &jobs[t]) != 0) {
            jobs[t].rc = -3;
            me_worker(&jobs[t]);
            th[t] = 0;
        }
    }
    int rc = 0;
    for (int t = 0; t < nthreads; t++) {
        if (th[t]) pthread_join(th[t], NULL);
        if (jobs[t].rc && jobs[t].rc != -3) rc = jobs[t].rc;
    }
    return rc;
}
