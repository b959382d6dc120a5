/*
 * c2a_port_batch.c -- many independent queries through the oracle port,
 * spread over host threads (each query is independent and the port keeps no
 * global state).  Used by the tests and by the bench's CPU-baseline leg.
 * Test infrastructure only.
 */
#define _POSIX_C_SOURCE 200809L
#include <pthread.h>
#include <stdlib.h>
#include "c2a_port.h"

typedef struct batch_job {
    const c2a_port_model *models;
    int num_models;
    const int *qint;      /* n x 4: model_a, model_b, seed_a, seed_b */
    const double *poses;  /* n x 48: R0a T0a R1a T1a R0b T0b R1b T1b */
    int n;
    const c2a_port_params *prm;
    c2a_port_result *res;
    c2a_port_contact *contacts;
    int per_query;
    int next;             /* next unclaimed query */
    int bad;
} batch_job;

static void run_one(batch_job *j, int q)
{
    const int *qi = j->qint + 4 * q;
    const double *p = j->poses + 48 * q;
    if (qi[0] < 0 || qi[0] >= j->num_models || qi[1] < 0 || qi[1] >= j->num_models) {
        __sync_fetch_and_add(&j->bad, 1);
        return;
    }
    if (c2a_port_solve(&j->models[qi[0]], &j->models[qi[1]], p, p + 9, p + 12, p + 21, p + 24, p + 33, p + 36,
                       p + 45, qi[2], qi[3], j->prm, &j->res[q],
                       j->contacts ? j->contacts + (size_t)q * (size_t)j->per_query : NULL, j->per_query) != 0)
        __sync_fetch_and_add(&j->bad, 1);
}

static void *worker(void *arg)
{
    batch_job *j = (batch_job *)arg;
    for (;;) {
        int q = __sync_fetch_and_add(&j->next, 1);
        if (q >= j->n) break;
        run_one(j, q);
    }
    return NULL;
}

int c2a_port_solve_batch(const c2a_port_model *models, int num_models, const int *qint, const double *poses, int n,
                         const c2a_port_params *prm, c2a_port_result *res, c2a_port_contact *contacts,
                         int contacts_per_query, int num_threads)
{
    batch_job j;
    int t;
    pthread_t *th;
    j.models = models; j.num_models = num_models; j.qint = qint; j.poses = poses; j.n = n;
    j.prm = prm; j.res = res; j.contacts = contacts; j.per_query = contacts_per_query;
    j.next = 0; j.bad = 0;
    if (num_threads <= 1) {
        worker(&j);
        return j.bad;
    }
    th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)num_threads);
    if (!th) return -1;
    for (t = 0; t < num_threads; t++)
        if (pthread_create(&th[t], NULL, worker, &j) != 0) { num_threads = t; break; }
    for (t = 0; t < num_threads; t++) pthread_join(th[t], NULL);
    free(th);
    if (num_threads == 0) worker(&j);
    return j.bad;
}

/* the deterministic sin/cos/acos the oracle uses, exported for the tests */
#include "../c2a_gb300/csrc/common/c2a_detmath.h"
double c2a_port_det_sin(double x) { return c2a_det_sin(x); }
double c2a_port_det_cos(double x) { return c2a_det_cos(x); }
double c2a_port_det_acos(double x) { return c2a_det_acos(x); }
