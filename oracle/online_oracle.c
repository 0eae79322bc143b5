/* online_oracle.c -- TEST INFRASTRUCTURE: the reference's online discretiser
 * (code/pipeline/online_discretize.py) restated in C for streams too long for
 * the pure-Python restatement in online.py.  Only the tests and the CPU
 * baseline of the online transactionisation call it.
 *
 *   P2Quantile   :22-71   five-marker estimator (setup from the first five
 *                         samples, the reference's marker update, value)
 *   OnlineBinner :74-103  n_bins-1 estimators at i/n_bins; edges from their
 *                         sorted values (3-bin re-centring / push-up rule)
 *   bin_index    :106-108 searchsorted(edges, v, "right") - 1, clamped
 *   run_file     :111-128 every row of every window fed in window order (rows
 *                         of overlapping windows fed again), then the window
 *                         median binned with the edges of that moment
 *
 * Sensors are independent: one thread handles a contiguous range of them.
 * Built with -ffp-contract=off, so every operation rounds as the reference's
 * Python floats do.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double q;
    double init[5];
    int n_init;
    double n[5], qv[5];
} p2_t;

static void sort_small(double *a, int m) {
    for (int i = 1; i < m; ++i) {
        double v = a[i];
        int j = i;
        while (j > 0 && a[j - 1] > v) {
            a[j] = a[j - 1];
            --j;
        }
        a[j] = v;
    }
}

static void p2_add(p2_t *p, double x) {
    if (p->n_init < 5) {
        p->init[p->n_init++] = x;
        if (p->n_init == 5) {
            memcpy(p->qv, p->init, sizeof p->qv);
            sort_small(p->qv, 5);
            p->n[0] = 0.0;
            p->n[1] = 1.0 + 2.0 * p->q;
            p->n[2] = 1.0 + 4.0 * p->q;
            p->n[3] = 3.0 + 2.0 * p->q;
            p->n[4] = 4.0;
        }
        return;
    }
    double *qv = p->qv, *n = p->n;
    int k;
    if (x < qv[0]) {
        qv[0] = x;
        k = 0;
    } else if (x < qv[1]) {
        k = 0;
    } else if (x < qv[2]) {
        k = 1;
    } else if (x < qv[3]) {
        k = 2;
    } else if (x <= qv[4]) {
        k = 3;
    } else {
        qv[4] = x;
        k = 3;
    }
    for (int i = 0; i < 5; ++i) n[i] = n[i] + 1.0;
    for (int i = 1; i <= k; ++i) n[i] = n[i] + 1.0;
    for (int i = 1; i <= 3; ++i) {
        const double d = n[i] - n[i - 1];
        const double span = n[i + 1] - n[i - 1];
        if (d >= 1.0 && span > 1.0) {
            const double qp = (d + 1.0) * (qv[i + 1] - qv[i - 1]) / span;
            const double moved = qv[i] + qp;
            if (qv[i - 1] < moved && moved < qv[i + 1]) qv[i] = moved;
        }
    }
}

static double p2_value(const p2_t *p) {
    if (p->n_init >= 5) return p->qv[2];
    if (p->n_init == 0) return 0.0;
    double a[5];
    memcpy(a, p->init, sizeof(double) * (size_t)p->n_init);
    sort_small(a, p->n_init);
    const int m = p->n_init;
    return (m & 1) ? a[m / 2] : (a[m / 2 - 1] + a[m / 2]) / 2.0;
}

/* edges (n_bins + 1 values) from the estimators' values q[0 .. n_bins-2] */
static void binner_edges(double *q, uint32_t n_bins, double *edges) {
    const uint32_t m = n_bins - 1;
    sort_small(q, (int)m);
    double span = q[m - 1] - q[0];
    if (1e-9 > span) span = 1e-9;
    const double min_gap = 0.05 * span;
    if (n_bins == 3) {
        if (q[1] - q[0] < min_gap) {
            const double mid = (q[0] + q[1]) / 2.0;
            q[0] = mid - min_gap / 2.0;
            q[1] = mid + min_gap / 2.0;
        }
    } else {
        for (uint32_t i = 1; i < m; ++i)
            if (q[i] < q[i - 1] + min_gap) q[i] = q[i - 1] + min_gap;
    }
    edges[0] = q[0] - span;
    for (uint32_t i = 0; i < m; ++i) edges[1 + i] = q[i];
    edges[n_bins] = q[m - 1] + span;
}

typedef struct {
    const double *values;
    uint64_t n_rows;
    uint32_t S, window, stride, n_bins, s_lo, s_hi;
    uint64_t n_win;
    double *edges_out;
    uint32_t *items_out;
    int status;
} job_t;

static void *run_sensors(void *arg) {
    job_t *j = (job_t *)arg;
    const uint32_t m = j->n_bins - 1, ne = j->n_bins + 1;
    p2_t *est = (p2_t *)calloc(m, sizeof(p2_t));
    double *q = (double *)malloc(sizeof(double) * m);
    double *buf = (double *)malloc(sizeof(double) * j->window);
    if (!est || !q || !buf) {
        j->status = -1;
        free(est);
        free(q);
        free(buf);
        return NULL;
    }
    for (uint32_t s = j->s_lo; s < j->s_hi; ++s) {
        for (uint32_t e = 0; e < m; ++e) {
            memset(&est[e], 0, sizeof(p2_t));
            est[e].q = (double)(e + 1) / (double)j->n_bins;
        }
        for (uint64_t w = 0; w < j->n_win; ++w) {
            const uint64_t start = w * j->stride;
            for (uint64_t t = start; t < start + j->window; ++t) {
                const double x = j->values[t * j->S + s];
                for (uint32_t e = 0; e < m; ++e) p2_add(&est[e], x);
            }
            for (uint32_t e = 0; e < m; ++e) q[e] = p2_value(&est[e]);
            double *ed = j->edges_out + ((size_t)w * j->S + s) * ne;
            binner_edges(q, j->n_bins, ed);
            for (uint32_t i = 0; i < j->window; ++i) buf[i] = j->values[(start + i) * j->S + s];
            sort_small(buf, (int)j->window);
            const uint32_t W = j->window;
            const double med = (W & 1) ? buf[W / 2] : (buf[W / 2 - 1] + buf[W / 2]) / 2.0;
            uint32_t cnt = 0;
            for (uint32_t i = 0; i < ne; ++i) cnt += ed[i] <= med;
            int32_t b = (int32_t)cnt - 1;
            if (b < 0) b = 0;
            if (b > (int32_t)ne - 2) b = (int32_t)ne - 2;
            j->items_out[w * j->S + s] = s * j->n_bins + (uint32_t)b;
        }
    }
    free(est);
    free(q);
    free(buf);
    return NULL;
}

/* values: row-major [n_rows, S]; writes edges_out [n_win, S, n_bins+1] and
 * items_out [n_win, S] (sensor * n_bins + bin).  Returns the window count, or
 * -1 on bad arguments / allocation failure. */
int64_t orc_online_bins(const double *values, uint64_t n_rows, uint32_t S, uint32_t window, uint32_t stride,
                        uint32_t n_bins, int n_threads, double *edges_out, uint32_t *items_out) {
    if (S == 0 || window == 0 || stride == 0 || n_bins < 2) return -1;
    const uint64_t n_win = n_rows >= window ? (n_rows - window) / stride + 1 : 0;
    if (n_win == 0) return 0;
    if (n_threads < 1) n_threads = 1;
    if ((uint32_t)n_threads > S) n_threads = (int)S;
    job_t *jobs = (job_t *)calloc((size_t)n_threads, sizeof(job_t));
    pthread_t *th = (pthread_t *)calloc((size_t)n_threads, sizeof(pthread_t));
    if (!jobs || !th) {
        free(jobs);
        free(th);
        return -1;
    }
    for (int t = 0; t < n_threads; ++t) {
        job_t *j = &jobs[t];
        j->values = values;
        j->n_rows = n_rows;
        j->S = S;
        j->window = window;
        j->stride = stride;
        j->n_bins = n_bins;
        j->s_lo = (uint32_t)((uint64_t)S * t / n_threads);
        j->s_hi = (uint32_t)((uint64_t)S * (t + 1) / n_threads);
        j->n_win = n_win;
        j->edges_out = edges_out;
        j->items_out = items_out;
        pthread_create(&th[t], NULL, run_sensors, j);
    }
    int bad = 0;
    for (int t = 0; t < n_threads; ++t) {
        pthread_join(th[t], NULL);
        bad |= jobs[t].status;
    }
    free(jobs);
    free(th);
    return bad ? -1 : (int64_t)n_win;
}
