/*
 * mdref.c — CPU oracle (test infrastructure only) for the MDcraft MD hot path.
 *
 * Each function cites the reference routine it restates. Arithmetic follows
 * the reference's FP64 operation order; compile with -ffp-contract=off.
 * Threads: mdcraft::tools::Threads restated (a kept pool of workers and the
 * reference's cut of each loop into bins, threads.h:214-347), so the timed
 * CPU baseline runs the reference's threading scheme on every host core.
 */
#define _GNU_SOURCE
#include "mdref.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------------ */
/* parallel-for: tools::Threads with its thread pool                        */
/* ------------------------------------------------------------------------ */

typedef void (*range_fn)(void* ctx, size_t b, size_t e, int tid);

/* tools::Threads (mdcraft/tools/threads.h:214-347, threads.cxx:32-74,
 * thread-pool.h): `count` workers made once and kept; every parallel loop
 * is cut into n_tasks = max(1, min(10 * count, n / 500)) bins of n / n_tasks
 * elements (the last bin takes the remainder), handed to the workers in
 * order through one queue while the caller waits for all of them; with
 * count < 2 the loop runs serially on the caller (Threads::disabled). */
typedef struct {
    int count;
    pid_t pid; /* the process whose threads these are (a fork keeps none) */
    pthread_t th[256];
    pthread_mutex_t mu;
    pthread_cond_t work, done;
    range_fn fn;
    void* ctx;
    size_t n, bin;
    int n_tasks, next_task, done_tasks;
    int stop;
} md_pool;

typedef struct {
    md_pool* pool;
    int tid;
} md_worker;

static md_pool* g_pool = NULL;
static md_worker g_workers[256];

static void* pool_worker(void* p) {
    md_worker* w = (md_worker*)p;
    md_pool* q = w->pool;
    pthread_mutex_lock(&q->mu);
    for (;;) {
        while (!q->stop && q->next_task >= q->n_tasks) pthread_cond_wait(&q->work, &q->mu);
        if (q->stop) break;
        const int t = q->next_task++;
        const size_t b = (size_t)t * q->bin;
        const size_t e = t == q->n_tasks - 1 ? q->n : b + q->bin;
        pthread_mutex_unlock(&q->mu);
        q->fn(q->ctx, b, e, w->tid);
        pthread_mutex_lock(&q->mu);
        if (++q->done_tasks == q->n_tasks) pthread_cond_signal(&q->done);
    }
    pthread_mutex_unlock(&q->mu);
    return NULL;
}

static void pool_stop(md_pool* q) {
    pthread_mutex_lock(&q->mu);
    q->stop = 1;
    pthread_cond_broadcast(&q->work);
    pthread_mutex_unlock(&q->mu);
    for (int t = 0; t < q->count; ++t) pthread_join(q->th[t], NULL);
    pthread_mutex_destroy(&q->mu);
    pthread_cond_destroy(&q->work);
    pthread_cond_destroy(&q->done);
    free(q);
}

/* The pool of `count` workers (Threads::resize makes a new ThreadPool). */
static md_pool* pool_get(int count) {
    if (g_pool && g_pool->pid != getpid()) g_pool = NULL; /* inherited by a fork: no threads behind it */
    if (g_pool && g_pool->count == count) return g_pool;
    if (g_pool) pool_stop(g_pool);
    md_pool* q = (md_pool*)calloc(1, sizeof(md_pool));
    q->count = count;
    q->pid = getpid();
    pthread_mutex_init(&q->mu, NULL);
    pthread_cond_init(&q->work, NULL);
    pthread_cond_init(&q->done, NULL);
    for (int t = 0; t < count; ++t) {
        g_workers[t].pool = q;
        g_workers[t].tid = t;
        pthread_create(&q->th[t], NULL, pool_worker, &g_workers[t]);
    }
    g_pool = q;
    return q;
}

static void parallel_for(int nthreads, size_t n, range_fn fn, void* ctx) {
    if (n == 0) return;
    if (nthreads > 256) nthreads = 256;
    if (nthreads < 2) {
        fn(ctx, 0, n, 0);
        return;
    }
    md_pool* q = pool_get(nthreads);
    size_t per = n / 500;
    size_t want = (size_t)10 * (size_t)nthreads;
    int n_tasks = (int)(per < want ? per : want);
    if (n_tasks < 1) n_tasks = 1;
    pthread_mutex_lock(&q->mu);
    q->fn = fn;
    q->ctx = ctx;
    q->n = n;
    q->bin = n / (size_t)n_tasks;
    q->done_tasks = 0;
    q->next_task = 0;
    q->n_tasks = n_tasks;
    pthread_cond_broadcast(&q->work);
    while (q->done_tasks < q->n_tasks) pthread_cond_wait(&q->done, &q->mu);
    q->n_tasks = 0; /* nothing left to hand out */
    q->next_task = 0;
    pthread_mutex_unlock(&q->mu);
}

int md_hardware_threads(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

/* ------------------------------------------------------------------------ */
/* Domain — mdcraft/lattice/domain.cxx:9-66                                 */
/* ------------------------------------------------------------------------ */

void md_domain_init(md_domain* d, double xmin, double xmax, double ymin,
                    double ymax, double zmin, double zmax) {
    /* Domain::Domain (domain.cxx:9-20) */
    d->bmin[0] = xmin; d->bmin[1] = ymin; d->bmin[2] = zmin;
    d->bmax[0] = xmax; d->bmax[1] = ymax; d->bmax[2] = zmax;
    d->size[0] = xmax - xmin; d->size[1] = ymax - ymin; d->size[2] = zmax - zmin;
    d->periodic[0] = d->periodic[1] = d->periodic[2] = 0;
    d->dim = fabs(zmin - zmax) > 1e-15 ? 3 : fabs(ymin - ymax) > 1e-15 ? 2 : 1;
}

int md_domain_belong(const md_domain* d, const double v[3]) {
    /* Domain::belong (domain.cxx:33-39) */
    int inside = 1;
    for (int i = 0; i < 3; i++)
        inside = inside && (d->bmin[i] <= v[i] && v[i] <= d->bmax[i]);
    return inside;
}

void md_domain_fit_in_period(const md_domain* d, double v[3]) {
    /* Domain::fit_in_period (domain.cxx:41-47): one wrap per axis */
    for (int i = 0; i < 3; i++) {
        if (d->periodic[i])
            v[i] = v[i] < d->bmin[i] ? v[i] + d->size[i]
                 : v[i] > d->bmax[i] ? v[i] - d->size[i] : v[i];
    }
}

double md_domain_nearest_distance(const md_domain* d, const double v[3],
                                  int axis) {
    /* Domain::nearest_distance (domain.cxx:49-57) */
    double dist = 1.7976931348623157e308;
    if (d->periodic[axis]) {
        double dmin = fabs(v[axis] - d->bmin[axis]);
        double dmax = fabs(v[axis] - d->bmax[axis]);
        dist = dmin < dmax ? dmin : dmax;
    }
    return dist;
}

void md_domain_shortest(const md_domain* d, double v[3]) {
    /* Domain::shortest (domain.cxx:59-66) */
    for (int i = 0; i < 3; ++i) {
        if (!d->periodic[i]) continue;
        v[i] = fabs(v[i] + d->size[i]) < fabs(v[i]) ? v[i] + d->size[i] : v[i];
        v[i] = fabs(v[i] - d->size[i]) < fabs(v[i]) ? v[i] - d->size[i] : v[i];
    }
}

/* ------------------------------------------------------------------------ */
/* Grid — mdcraft/neibs/grid.cxx:43-243                                     */
/* ------------------------------------------------------------------------ */

static void grid_global_index3D(const md_grid* g, const md_domain* d,
                                const double v[3], int c[3]) {
    /* Grid::global_index3D (grid.cxx:107-112) */
    c[0] = c[1] = c[2] = 0;
    for (int i = 0; i < d->dim; ++i)
        c[i] = (int)floor((v[i] - d->bmin[i]) / g->cell_sizes[i]);
}

void md_grid_local_index3D(const md_grid* g, const md_domain* d,
                           const double v[3], int c[3]) {
    /* Grid::local_index3D (grid.cxx:114-119) */
    grid_global_index3D(g, d, v, c);
    for (int i = 0; i < d->dim; ++i) c[i] -= g->grid_offset[i];
}

int md_grid_cell_index(const md_grid* g, const int ijk[3]) {
    /* Grid::cell_index (grid.cxx:134-136) */
    return ijk[0] + g->num_cells[0] * (ijk[1] + g->num_cells[1] * ijk[2]);
}

int md_grid_cells_number(const md_grid* g) {
    return g->num_cells[0] * g->num_cells[1] * g->num_cells[2];
}

double md_grid_cell_size(const md_grid* g) {
    double m = g->cell_sizes[0];
    if (g->cell_sizes[1] > m) m = g->cell_sizes[1];
    if (g->cell_sizes[2] > m) m = g->cell_sizes[2];
    return m;
}

void md_grid_build(md_grid* g, const md_domain* d, const md_atom* atoms,
                   size_t n) {
    if (n == 0) {
        /* Grid::initialize_empty (grid.cxx:28-40) */
        for (int i = 0; i < 3; ++i) {
            g->cell_sizes[i] = d->size[i];
            g->domain_num_cells[i] = 1;
            g->grid_offset[i] = 1;
            g->min_coords[i] = NAN;
            g->max_coords[i] = NAN;
            g->num_cells[i] = 0;
        }
        return;
    }
    /* Grid::find_bounds (grid.cxx:209-243): min/max of r and max rns */
    double bmin[3] = {1.7976931348623157e308, 1.7976931348623157e308,
                      1.7976931348623157e308};
    double bmax[3] = {-1.7976931348623157e308, -1.7976931348623157e308,
                      -1.7976931348623157e308};
    double max_rns = 0.0;
    for (size_t k = 0; k < n; ++k) {
        const md_atom* a = &atoms[k];
        if (max_rns < a->rns) max_rns = a->rns;
        for (int i = 0; i < 3; ++i) {
            if (a->r[i] < bmin[i]) bmin[i] = a->r[i];
            if (a->r[i] > bmax[i]) bmax[i] = a->r[i];
        }
    }
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int i = 0; i < d->dim; ++i) {
        lo[i] = bmin[i];
        hi[i] = bmax[i];
    }
    double cell_size = max_rns;
    /* Grid::build (grid.cxx:43-95) */
    for (int i = 0; i < 3; ++i) g->domain_num_cells[i] = 1;
    for (int i = 0; i < d->dim; ++i) {
        int c = (int)floor(d->size[i] / cell_size);
        g->domain_num_cells[i] = c > 1 ? c : 1;
    }
    for (int i = 0; i < 3; ++i) g->cell_sizes[i] = d->size[i];
    for (int i = 0; i < d->dim; ++i) g->cell_sizes[i] /= g->domain_num_cells[i];
    grid_global_index3D(g, d, lo, g->grid_offset);
    int upper[3];
    grid_global_index3D(g, d, hi, upper);
    for (int i = 0; i < d->dim; ++i) {
        int u = upper[i] + 1;
        upper[i] = u < g->domain_num_cells[i] ? u : g->domain_num_cells[i];
    }
    for (int i = 0; i < 3; ++i) g->num_cells[i] = 1;
    for (int i = 0; i < d->dim; ++i) g->num_cells[i] = upper[i] - g->grid_offset[i];
    for (int i = 0; i < 3; ++i) {
        g->min_coords[i] = d->bmin[i];
        g->max_coords[i] = d->bmax[i];
    }
    for (int i = 0; i < d->dim; ++i) {
        g->min_coords[i] = d->bmin[i] + g->cell_sizes[i] * g->grid_offset[i];
        g->max_coords[i] = d->bmin[i] + g->cell_sizes[i] * upper[i];
    }
}

int md_grid_adjacent_cells(const md_grid* g, const md_domain* d,
                           const double r[3], int cells[27], int is_edge[3]) {
    /* Grid::adjacent_cells (grid.cxx:138-207) */
    int cell[3];
    grid_global_index3D(g, d, r, cell);
    int n_x = g->domain_num_cells[0], n_y = g->domain_num_cells[1],
        n_z = g->domain_num_cells[2];
    int cnt = 0;
    for (int x = -1; x <= 1; ++x) {
        if (d->periodic[0]) {
            if (n_x == 1 && x != 0) continue;
            if (n_x == 2 && x == 1) continue;
        }
        for (int y = -1; y <= 1; ++y) {
            if (d->periodic[1]) {
                if (n_y == 1 && y != 0) continue;
                if (n_y == 2 && y == 1) continue;
            }
            for (int z = -1; z <= 1; ++z) {
                if (d->periodic[2]) {
                    if (n_z == 1 && z != 0) continue;
                    if (n_z == 2 && z == 1) continue;
                }
                int nb[3] = {cell[0] + x, cell[1] + y, cell[2] + z};
                if (d->periodic[0]) nb[0] = (nb[0] + n_x) % n_x;
                if (d->periodic[1]) nb[1] = (nb[1] + n_y) % n_y;
                if (d->periodic[2]) nb[2] = (nb[2] + n_z) % n_z;
                nb[0] -= g->grid_offset[0];
                nb[1] -= g->grid_offset[1];
                nb[2] -= g->grid_offset[2];
                if (0 <= nb[0] && nb[0] < g->num_cells[0] && 0 <= nb[1] &&
                    nb[1] < g->num_cells[1] && 0 <= nb[2] &&
                    nb[2] < g->num_cells[2])
                    cells[cnt++] = md_grid_cell_index(g, nb);
            }
        }
    }
    for (int i = cnt; i < 27; ++i) cells[i] = -1;
    is_edge[0] = is_edge[1] = is_edge[2] = 0;
    for (int i = 0; i < d->dim; ++i)
        is_edge[i] = cell[i] == 0 || cell[i] == g->num_cells[i] - 1;
    return cnt;
}

/* ------------------------------------------------------------------------ */
/* VerletList — mdcraft/neibs/verlet-list.cxx                               */
/* ------------------------------------------------------------------------ */

struct md_nlist {
    size_t n;
    int half, nthreads;
    uint64_t** lists;
    uint32_t* counts;
    uint32_t* caps;
    md_grid grid;
    int have_cells;
    int* head;
    int* next;
    size_t head_cap, next_cap;
    double* saved_r;
    double* saved_rcut;
    double* saved_rns;
    uint32_t* saved_uid;
    size_t nsaved;
    int snapshot_valid;
};

md_nlist* md_nlist_create(size_t n, int half, int nthreads, int* status) {
    /* VerletList::VerletList (verlet-list.cxx:11-39): half lists are
     * rejected with an active thread pool. */
    if (status) *status = MDREF_OK;
    if (half && nthreads > 1) {
        if (status) *status = MDREF_ERR_INVALID;
        return NULL;
    }
    md_nlist* nl = (md_nlist*)calloc(1, sizeof(md_nlist));
    nl->half = half;
    nl->nthreads = nthreads < 1 ? 1 : nthreads;
    return nl;
}

static void nlist_resize(md_nlist* nl, size_t n) {
    if (n > nl->n) {
        nl->lists = (uint64_t**)realloc(nl->lists, n * sizeof(uint64_t*));
        nl->counts = (uint32_t*)realloc(nl->counts, n * sizeof(uint32_t));
        nl->caps = (uint32_t*)realloc(nl->caps, n * sizeof(uint32_t));
        for (size_t i = nl->n; i < n; ++i) {
            nl->caps[i] = 128; /* ListOne reserve(128), verlet-list.cxx:36 */
            nl->lists[i] = (uint64_t*)malloc(128 * sizeof(uint64_t));
            nl->counts[i] = 0;
        }
    } else {
        for (size_t i = n; i < nl->n; ++i) free(nl->lists[i]);
    }
    nl->n = n;
}

void md_nlist_destroy(md_nlist* nl) {
    if (!nl) return;
    for (size_t i = 0; i < nl->n; ++i) free(nl->lists[i]);
    free(nl->lists);
    free(nl->counts);
    free(nl->caps);
    free(nl->head);
    free(nl->next);
    free(nl->saved_r);
    free(nl->saved_rcut);
    free(nl->saved_rns);
    free(nl->saved_uid);
    free(nl);
}

static inline void list_push(md_nlist* nl, size_t i, uint64_t j) {
    if (nl->counts[i] == nl->caps[i]) {
        nl->caps[i] *= 2;
        nl->lists[i] = (uint64_t*)realloc(nl->lists[i], nl->caps[i] * sizeof(uint64_t));
    }
    nl->lists[i][nl->counts[i]++] = j;
}

/* VerletList::are_neibs (verlet-list.cxx:357-400) */
static inline int are_neibs(const md_domain* d, const double ra[3],
                            double radius_x, const double rb[3],
                            double radius_y, const int is_edge[3]) {
    double dd = radius_x < radius_y ? radius_y : radius_x; /* std::max */
    double d2 = dd * dd;
    double drx = ra[0] - rb[0];
    double dry = ra[1] - rb[1];
    double drz = ra[2] - rb[2];
    double xs = d->size[0], ys = d->size[1], zs = d->size[2];
    if (is_edge[0] && d->periodic[0] && (2 * drx < -xs)) drx += xs;
    if (is_edge[0] && d->periodic[0] && (2 * drx > xs)) drx -= xs;
    if (is_edge[1] && d->periodic[1] && (2 * dry < -ys)) dry += ys;
    if (is_edge[1] && d->periodic[1] && (2 * dry > ys)) dry -= ys;
    if (is_edge[2] && d->periodic[2] && (2 * drz < -zs)) drz += zs;
    if (is_edge[2] && d->periodic[2] && (2 * drz > zs)) drz -= zs;
    return drx * drx + dry * dry + drz * drz <= d2;
}

typedef struct {
    md_nlist* nl;
    const md_domain* d;
    md_atom* atoms;
    double kbuf;
} nl_ctx;

static void fit_range(void* p, size_t b, size_t e, int tid) {
    (void)tid;
    nl_ctx* c = (nl_ctx*)p;
    for (size_t i = b; i < e; ++i) md_domain_fit_in_period(c->d, c->atoms[i].r);
}

static void build_range(void* p, size_t b, size_t e, int tid) {
    /* build_one lambda of build_linked_cells (verlet-list.cxx:334-352) */
    (void)tid;
    nl_ctx* c = (nl_ctx*)p;
    md_nlist* nl = c->nl;
    for (size_t i = b; i < e; ++i) {
        const md_atom* a = &c->atoms[i];
        int cells[27], is_edge[3];
        int cnt = md_grid_adjacent_cells(&nl->grid, c->d, a->r, cells, is_edge);
        for (int k = 0; k < cnt; ++k) {
            for (int j = nl->head[cells[k]]; j != -1; j = nl->next[j]) {
                if (nl->half && (size_t)j < i) continue;
                const md_atom* nb = &c->atoms[j];
                if (are_neibs(c->d, a->r, a->rns, nb->r, nb->rns, is_edge))
                    list_push(nl, i, (uint64_t)j);
            }
        }
    }
}

static void optimize_range(void* p, size_t b, size_t e, int tid) {
    /* VerletList::optimize_search_radius (verlet-list.cxx:72-92) */
    (void)tid;
    nl_ctx* c = (nl_ctx*)p;
    md_nlist* nl = c->nl;
    for (size_t i = b; i < e; ++i) {
        md_atom* a = &c->atoms[i];
        double hmax = 0.0;
        for (uint32_t k = 0; k < nl->counts[i]; ++k) {
            const md_atom* nb = &c->atoms[nl->lists[i][k]];
            double h = a->rcut + nb->rcut;
            hmax = hmax < h ? h : hmax;
        }
        a->rns = c->kbuf * hmax;
    }
}

static void snapshot(md_nlist* nl, const md_atom* atoms, size_t n) {
    /* VerletList::snapshot_atoms (verlet-list.cxx:160-175) */
    nl->saved_r = (double*)realloc(nl->saved_r, (n ? n : 1) * 3 * sizeof(double));
    nl->saved_rcut = (double*)realloc(nl->saved_rcut, (n ? n : 1) * sizeof(double));
    nl->saved_rns = (double*)realloc(nl->saved_rns, (n ? n : 1) * sizeof(double));
    nl->saved_uid = (uint32_t*)realloc(nl->saved_uid, (n ? n : 1) * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) {
        memcpy(&nl->saved_r[3 * i], atoms[i].r, 3 * sizeof(double));
        nl->saved_rcut[i] = atoms[i].rcut;
        nl->saved_rns[i] = atoms[i].rns;
        nl->saved_uid[i] = atoms[i].uid;
    }
    nl->nsaved = n;
    nl->snapshot_valid = 1;
}

int md_nlist_update(md_nlist* nl, const md_domain* d, md_atom* atoms,
                    size_t n, double kbuf) {
    /* VerletList::update (verlet-list.cxx:41-55) */
    nl_ctx c = {nl, d, atoms, kbuf};
    int status = MDREF_OK;
    if (n == 0) {
        nlist_resize(nl, 0);
        snapshot(nl, atoms, 0);
        return MDREF_OK;
    }
    if (kbuf > 0.0 && nl->n == n) parallel_for(nl->nthreads, n, optimize_range, &c);
    else if (kbuf > 0.0) {
        for (size_t i = 0; i < n; ++i) atoms[i].rns = 0.0; /* empty lists */
    }
    nlist_resize(nl, n);
    for (size_t i = 0; i < n; ++i) nl->counts[i] = 0;
    /* build_linked_cells (verlet-list.cxx:306-355) */
    parallel_for(nl->nthreads, n, fit_range, &c);
    md_grid_build(&nl->grid, d, atoms, n);
    size_t n_cells = (size_t)md_grid_cells_number(&nl->grid);
    nl->have_cells = 0;
    if (n_cells == 0) {
        snapshot(nl, atoms, n);
        return MDREF_OK;
    }
    if (nl->head_cap < n_cells) {
        nl->head = (int*)realloc(nl->head, n_cells * sizeof(int));
        nl->head_cap = n_cells;
    }
    if (nl->next_cap < n) {
        nl->next = (int*)realloc(nl->next, n * sizeof(int));
        nl->next_cap = n;
    }
    for (size_t k = 0; k < n_cells; ++k) nl->head[k] = -1;
    for (size_t i = 0; i < n; ++i) nl->next[i] = -1;
    for (size_t i = 0; i < n; ++i) {
        int ijk[3];
        md_grid_local_index3D(&nl->grid, d, atoms[i].r, ijk);
        /* Outside the local grid the reference indexes head[] out of
         * bounds; clamp and report instead. */
        for (int a = 0; a < 3; ++a) {
            if (ijk[a] < 0) { ijk[a] = 0; status = MDREF_ERR_RANGE; }
            if (ijk[a] >= nl->grid.num_cells[a]) {
                ijk[a] = nl->grid.num_cells[a] - 1;
                status = MDREF_ERR_RANGE;
            }
        }
        int cell = md_grid_cell_index(&nl->grid, ijk);
        nl->next[i] = nl->head[cell];
        nl->head[cell] = (int)i;
    }
    nl->have_cells = 1;
    parallel_for(nl->half ? 1 : nl->nthreads, n, build_range, &c);
    snapshot(nl, atoms, n);
    return status;
}

typedef struct {
    const md_nlist* nl;
    const md_domain* d;
    const md_atom* atoms;
    atomic_int need;
} decide_ctx;

static void decide_range(void* p, size_t b, size_t e, int tid) {
    /* VerletList::decide body (verlet-list.cxx:127-155) */
    (void)tid;
    decide_ctx* c = (decide_ctx*)p;
    const md_nlist* nl = c->nl;
    for (size_t i = b; i < e; ++i) {
        if (atomic_load_explicit(&c->need, memory_order_relaxed)) return;
        const md_atom* a = &c->atoms[i];
        if (a->uid != nl->saved_uid[i] || a->rcut != nl->saved_rcut[i] ||
            a->rns != nl->saved_rns[i]) {
            atomic_store(&c->need, 1);
            return;
        }
        double skin = nl->saved_rns[i] - nl->saved_rcut[i];
        if (skin <= 0.0) {
            atomic_store(&c->need, 1);
            return;
        }
        double dr[3] = {a->r[0] - nl->saved_r[3 * i], a->r[1] - nl->saved_r[3 * i + 1],
                        a->r[2] - nl->saved_r[3 * i + 2]};
        md_domain_shortest(c->d, dr);
        double trigger2 = 0.25 * skin * skin;
        if (dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2] > trigger2)
            atomic_store(&c->need, 1);
    }
}

int md_nlist_decide(const md_nlist* nl, const md_domain* d,
                    const md_atom* atoms, size_t n) {
    /* VerletList::decide (verlet-list.cxx:110-158) */
    if (!nl->snapshot_valid || n != nl->nsaved) return 1;
    if (n == 0) return 0;
    decide_ctx c;
    c.nl = nl;
    c.d = d;
    c.atoms = atoms;
    atomic_init(&c.need, 0);
    parallel_for(nl->nthreads, n, decide_range, &c);
    return atomic_load(&c.need);
}

size_t md_nlist_count(const md_nlist* nl, size_t i) {
    return i < nl->n ? nl->counts[i] : 0;
}

const uint64_t* md_nlist_list(const md_nlist* nl, size_t i) {
    return i < nl->n ? nl->lists[i] : NULL;
}

size_t md_nlist_total(const md_nlist* nl) {
    size_t t = 0;
    for (size_t i = 0; i < nl->n; ++i) t += nl->counts[i];
    return t;
}

void md_nlist_export(const md_nlist* nl, uint64_t* offsets, uint64_t* idx) {
    uint64_t o = 0;
    for (size_t i = 0; i < nl->n; ++i) {
        offsets[i] = o;
        memcpy(idx + o, nl->lists[i], nl->counts[i] * sizeof(uint64_t));
        o += nl->counts[i];
    }
    offsets[nl->n] = o;
}

void md_nlist_grid(const md_nlist* nl, md_grid* out) { *out = nl->grid; }

size_t md_nlist_list_for(const md_nlist* nl, const md_domain* d,
                         const md_atom* atoms, const double x[3],
                         uint64_t* out, size_t cap) {
    /* VerletList::list_for (verlet-list.cxx:251-276): radius = cell_size() */
    if (!nl->have_cells) return 0;
    int cells[27], is_edge[3];
    int cnt = md_grid_adjacent_cells(&nl->grid, d, x, cells, is_edge);
    double rad = md_grid_cell_size(&nl->grid);
    size_t m = 0;
    for (int k = 0; k < cnt; ++k) {
        for (int j = nl->head[cells[k]]; j != -1; j = nl->next[j]) {
            if (are_neibs(d, x, rad, atoms[j].r, atoms[j].rns, is_edge)) {
                if (m < cap) out[m] = (uint64_t)j;
                ++m;
            }
        }
    }
    return m;
}

int md_sort_atoms(const md_domain* d, md_atom* atoms, size_t n, md_atom* sorted) {
    /* VerletList::sort (verlet-list.cxx:237-249): put_atoms_in_cells
     * (verlet-list.cxx:176-199) wraps the atoms in place and builds the grid
     * from them; the copy lists them by Grid::cell_index (grid.cxx:134-136).
     * The reference compares cells only (grid.h:31-33), so its order inside a
     * cell is unspecified; here it is ascending index (a stable counting
     * sort). Cells outside the local grid are clamped, as in update(). */
    if (n == 0) return MDREF_OK;
    int status = MDREF_OK;
    for (size_t i = 0; i < n; ++i) md_domain_fit_in_period(d, atoms[i].r);
    md_grid g;
    md_grid_build(&g, d, atoms, n);
    size_t nc = (size_t)md_grid_cells_number(&g);
    size_t* start = (size_t*)calloc(nc + 1, sizeof(size_t));
    int* cell = (int*)malloc(n * sizeof(int));
    for (size_t i = 0; i < n; ++i) {
        int ijk[3];
        md_grid_local_index3D(&g, d, atoms[i].r, ijk);
        for (int a = 0; a < 3; ++a) {
            if (ijk[a] < 0) { ijk[a] = 0; status = MDREF_ERR_RANGE; }
            if (ijk[a] >= g.num_cells[a]) { ijk[a] = g.num_cells[a] - 1; status = MDREF_ERR_RANGE; }
        }
        cell[i] = md_grid_cell_index(&g, ijk);
        start[cell[i] + 1]++;
    }
    for (size_t c = 0; c < nc; ++c) start[c + 1] += start[c];
    for (size_t i = 0; i < n; ++i) sorted[start[cell[i]]++] = atoms[i];
    free(cell);
    free(start);
    return status;
}

/* ------------------------------------------------------------------------ */
/* Potentials — mdcraft/solver/potential/{LJs-cut,EAM}.cxx                  */
/* ------------------------------------------------------------------------ */

struct md_pot {
    int type;
    double R1cut, R2cut;
    /* LJsCut (LJs-cut.cxx:8-20) */
    double a, s, s6, lj1, lj2, factor;
    /* EAM (EAM.cxx:15-53); tables carry one padding element at [N] */
    int Nr1, Nrh1;
    double dr, drh, dr1, drh1;
    double *Femb, *Rho, *Vpar, *dFemb, *dRho, *dVpar;
    /* LJs (LJs.cxx:7-29, LJs.h:41) */
    double aVr, aVr2, rVr, rVr1, rVr2, aLJ, aLJ3, bLJ, bLJ2;
};

md_pot* md_pot_ljcut_create(double a, double s, double rcut) {
    md_pot* p = (md_pot*)calloc(1, sizeof(md_pot));
    p->type = MD_POT_PAIR;
    p->R1cut = rcut;
    p->R2cut = rcut * rcut;
    p->a = a;
    p->s = s;
    p->s6 = pow(s, 6);
    p->lj1 = 2 * p->s6;
    p->lj2 = 1.;
    p->factor = 48. * p->a * p->s6;
    return p;
}

void md_eam_init_spline(const double* y, double* z, double H1, size_t N,
                        int ib) {
    /* EAM::init_spline (EAM.cxx:603-686), Shikin & Plis sweep. The final
     * loop reads z[i] before writing it; z is zero on entry, as the
     * reference's value-initialised vectors are. */
    double* a = (double*)malloc(N * sizeof(double));
    double* b = (double*)malloc(N * sizeof(double));
    double* c = (double*)malloc(N * sizeof(double));
    double* d = (double*)malloc(N * sizeof(double));
    double* s = (double*)malloc((N + 1) * sizeof(double));
    double* t = (double*)malloc((N + 1) * sizeof(double));
    double* u = (double*)malloc((N + 1) * sizeof(double));
    double* v = (double*)malloc((N + 1) * sizeof(double));
    double* w = (double*)malloc((N + 1) * sizeof(double));
    for (size_t i = 0; i < N; ++i) { a[i] = 2.0; b[i] = 0.0; c[i] = 0.0; d[i] = 0.0; }
    for (size_t i = 0; i <= N; ++i) { s[i] = t[i] = u[i] = v[i] = w[i] = 0.0; }
    b[0] = 1.0;
    c[0] = 0.0;
    d[0] = 3.0 * H1 * (y[1] - y[0]);
    b[N - 1] = 0.0;
    if (ib == 1) {
        c[N - 1] = 0.0;
        d[N - 1] = 0.0;
    } else if (ib == 2) {
        c[N - 1] = 1.0;
        d[N - 1] = 3.0 * H1 * (y[N - 1] - y[N - 2]);
    }
    for (size_t i = 1; i < N - 1; i++) {
        c[i] = 0.5;
        b[i] = 0.5;
        d[i] = 1.5 * H1 * (y[i + 1] - y[i - 1]);
    }
    u[0] = 0.0;
    v[0] = 0.0;
    w[0] = 1.0;
    for (size_t i = 0; i < N; i++) {
        double rp = -1.0 / (a[i] + c[i] * v[i]);
        v[i + 1] = rp * b[i];
        u[i + 1] = rp * (c[i] * u[i] - d[i]);
        w[i + 1] = rp * c[i] * w[i];
    }
    s[N - 1] = 1.0;
    t[N - 1] = 0.0;
    for (long i = (long)N - 2; i >= 0; i--) {
        s[i] = v[i + 1] * s[i + 1] + w[i + 1];
        t[i] = v[i + 1] * t[i + 1] + u[i + 1];
    }
    for (size_t i = 0; i < N; ++i) z[i] = 0.0;
    z[N - 1] = (d[N - 1] - b[N - 1] * t[0] - c[N - 1] * t[N - 2]) /
               (a[N - 1] + b[N - 1] * s[0] + c[N - 1] * s[N - 2]);
    for (size_t i = 0; i < N - 1; i++) z[i] = s[i] * z[i] + t[i];
    free(a); free(b); free(c); free(d);
    free(s); free(t); free(u); free(v); free(w);
}

static double* padded_copy(const double* src, int n) {
    double* p = (double*)malloc(((size_t)n + 1) * sizeof(double));
    memcpy(p, src, (size_t)n * sizeof(double));
    p[n] = src[n - 1];
    return p;
}

md_pot* md_pot_eam_create(double rcut, const double* Femb, const double* Rho,
                          const double* Vpar, int Nr1, double dr, int Nrh1,
                          double drh) {
    /* EAM::EAM(arrays) (EAM.cxx:15-53) */
    if (Nr1 < 3 || Nrh1 < 3) return NULL;
    md_pot* p = (md_pot*)calloc(1, sizeof(md_pot));
    p->type = MD_POT_EAM;
    p->R1cut = rcut;
    p->R2cut = rcut * rcut;
    p->Nr1 = Nr1;
    p->Nrh1 = Nrh1;
    p->dr = dr;
    p->drh = drh;
    p->dr1 = 1.0 / dr;
    p->drh1 = 1.0 / drh;
    p->Rho = padded_copy(Rho, Nr1);
    p->Vpar = padded_copy(Vpar, Nr1);
    p->Femb = padded_copy(Femb, Nrh1);
    p->dRho = (double*)calloc((size_t)Nr1 + 1, sizeof(double));
    p->dVpar = (double*)calloc((size_t)Nr1 + 1, sizeof(double));
    p->dFemb = (double*)calloc((size_t)Nrh1 + 1, sizeof(double));
    md_eam_init_spline(p->Vpar, p->dVpar, p->dr1, (size_t)Nr1, 1);
    md_eam_init_spline(p->Rho, p->dRho, p->dr1, (size_t)Nr1, 1);
    md_eam_init_spline(p->Femb, p->dFemb, p->drh1, (size_t)Nrh1, 2);
    p->dVpar[Nr1] = p->dVpar[Nr1 - 1];
    p->dRho[Nr1] = p->dRho[Nr1 - 1];
    p->dFemb[Nrh1] = p->dFemb[Nrh1 - 1];
    return p;
}

md_pot* md_pot_pair_create(double rcut, const double* Vpar, int Nr1,
                           double dr) {
    /* Pair::Pair(arrays) (pair.cxx:15-33). The reference's table has Nr1
     * entries and its spline reads entry N1+1 for N1 < Nr1 (one past the
     * end at the last interval); the copy here carries the last value as
     * padding, as for the EAM tables. */
    if (Nr1 < 3) return NULL;
    md_pot* p = (md_pot*)calloc(1, sizeof(md_pot));
    p->type = MD_POT_TAB;
    p->R1cut = rcut;
    p->R2cut = rcut * rcut;
    p->Nr1 = Nr1;
    p->dr = dr;
    p->dr1 = 1.0 / dr;
    p->Vpar = padded_copy(Vpar, Nr1);
    p->dVpar = (double*)calloc((size_t)Nr1 + 1, sizeof(double));
    md_eam_init_spline(p->Vpar, p->dVpar, p->dr1, (size_t)Nr1, 1);
    p->dVpar[Nr1] = p->dVpar[Nr1 - 1];
    return p;
}

md_pot* md_pot_ljs_create(double aVr, double rVr, double rcut) {
    /* LJs::LJs (LJs.cxx:7-29), same operation order */
    const double X2min = 1.2599210498948732;
    md_pot* p = (md_pot*)calloc(1, sizeof(md_pot));
    p->type = MD_POT_LJS;
    p->R1cut = rcut;
    p->R2cut = rcut * rcut;
    double R2cut = p->R2cut;
    p->rVr = rVr;
    p->rVr2 = rVr * rVr;
    p->rVr1 = 1.0 / p->rVr2;
    p->aVr2 = R2cut / p->rVr2 - X2min;
    p->aLJ3 = (p->rVr2 / R2cut) * (p->rVr2 / R2cut) * (p->rVr2 / R2cut);
    p->bLJ2 = (p->aLJ3 - 0.5) * p->aVr2 * p->rVr2 / R2cut;
    p->aLJ = (p->aLJ3 - 1.0 + 2.0 * p->bLJ2) * p->aLJ3 / (p->aVr2 * p->aVr2);
    p->bLJ = -(p->aLJ3 - 1.0 + 3.0 * p->bLJ2) * p->aLJ3 / (p->aVr2 * p->aVr2 * p->aVr2);
    p->aLJ3 = 3.0 * p->aLJ;
    p->bLJ2 = 2.0 * p->bLJ;
    p->aVr2 = -48.0 * aVr / p->rVr2;
    p->aVr = 2.0 * aVr;
    return p;
}

void md_pot_destroy(md_pot* p) {
    if (!p) return;
    free(p->Femb); free(p->Rho); free(p->Vpar);
    free(p->dFemb); free(p->dRho); free(p->dVpar);
    free(p);
}

double md_pot_rcut(const md_pot* p) { return p->R1cut; }
int md_pot_type(const md_pot* p) { return p->type; }

void md_eam_slopes(const md_pot* p, double* dVpar, double* dRho, double* dFemb) {
    memcpy(dVpar, p->dVpar, (size_t)p->Nr1 * sizeof(double));
    memcpy(dRho, p->dRho, (size_t)p->Nr1 * sizeof(double));
    memcpy(dFemb, p->dFemb, (size_t)p->Nrh1 * sizeof(double));
}

/* EAM::embeddingEnergy for one value (EAM.cxx:562-601). dF holds the
 * caller's initial value (zero in every reference caller). */
static void eam_embed(const md_pot* p, double nr, double* EF, double* dF) {
    double RN = nr * p->drh1;
    int N1 = (int)trunc(RN);
    if (RN >= 0.0 && N1 < p->Nrh1) {
        double VR = N1;
        double DV = RN - VR;
        RN = nr - VR * p->drh;
        VR = (p->Femb[N1 + 1] - p->Femb[N1]) * p->drh1;
        double aa = (p->dFemb[N1 + 1] - VR) - (VR - p->dFemb[N1]);
        double bb = aa - (VR - p->dFemb[N1]);
        aa = aa * DV;
        *EF = p->Femb[N1] + RN * (p->dFemb[N1] + DV * (aa - bb));
        *dF = p->dFemb[N1] + 2.0 * DV * (1.5 * aa - bb);
    } else {
        if (N1 >= p->Nrh1) {
            *EF = p->Femb[p->Nrh1] + p->dFemb[p->Nrh1] * (*dF - p->Nrh1 * p->drh);
            *dF = p->dFemb[p->Nrh1];
        } else {
            *EF = p->Femb[0] - p->dFemb[0] * (*dF);
            *dF = p->dFemb[0];
        }
    }
}

void md_eam_embedding(const md_pot* p, double rho, double* F, double* dF) {
    *dF = 0.0;
    eam_embed(p, rho, F, dF);
}

/* Neighbour view handed to the potentials: positions, densities and (for
 * half lists) pointers to the neighbour atoms. */
typedef struct {
    size_t nn;
    const double (*rj)[3];
    const double* ncj;
    md_atom** nbp; /* non-NULL only for half lists */
} nview;

/* LJsCut::force (LJs-cut.cxx:22-68) */
static void ljcut_force(const md_pot* p, md_atom* a, const nview* v) {
    if (v->nn == 0) return;
    double x = a->r[0], y = a->r[1], z = a->r[2];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (size_t i = 0; i < v->nn; i++) {
        double drx = v->rj[i][0] - x;
        double dry = v->rj[i][1] - y;
        double drz = v->rj[i][2] - z;
        double r2ij = drx * drx + dry * dry + drz * drz;
        if ((r2ij > p->R2cut) || (r2ij < 1e-15)) continue;
        double r2inv = 1.0 / r2ij;
        double r6inv = r2inv * r2inv * r2inv;
        double prefact = -0.5 * p->factor * (p->lj1 * r6inv - p->lj2) * r6inv * r2inv;
        fx += drx * prefact;
        fy += dry * prefact;
        fz += drz * prefact;
        if (v->nbp) {
            v->nbp[i]->f[0] -= drx * prefact;
            v->nbp[i]->f[1] -= dry * prefact;
            v->nbp[i]->f[2] -= drz * prefact;
        }
    }
    a->f[0] += fx;
    a->f[1] += fy;
    a->f[2] += fz;
}

/* LJsCut::virial (LJs-cut.cxx:70-131) */
static void ljcut_virial(const md_pot* p, md_atom* a, const nview* v) {
    if (v->nn == 0) return;
    double x = a->r[0], y = a->r[1], z = a->r[2];
    double Vxx = 0.0, Vyy = 0.0, Vzz = 0.0, Vxy = 0.0, Vxz = 0.0, Vyz = 0.0;
    for (size_t i = 0; i < v->nn; i++) {
        double drx = v->rj[i][0] - x;
        double dry = v->rj[i][1] - y;
        double drz = v->rj[i][2] - z;
        double r2ij = drx * drx + dry * dry + drz * drz;
        if ((r2ij > p->R2cut) || (r2ij < 1e-15)) continue;
        double r2inv = 1.0 / r2ij;
        double r6inv = r2inv * r2inv * r2inv;
        double prefact = -0.5 * p->factor * (p->lj1 * r6inv - p->lj2) * r6inv * r2inv;
        double fx = prefact * drx, fy = prefact * dry, fz = prefact * drz;
        Vxx += fx * drx;
        Vyy += fy * dry;
        Vzz += fz * drz;
        Vxy += fx * dry;
        Vxz += fx * drz;
        Vyz += fy * drz;
        double tmp = p->s6 * r6inv;
        double add_Ep = 0.5 * 4 * p->a * tmp * (tmp - 1);
        a->Ep += add_Ep;
        if (v->nbp) {
            md_atom* nb = v->nbp[i];
            double M[9] = {fx * drx, fy * drx, fz * drx, fx * dry, fy * dry,
                           fz * dry, fx * drz, fy * drz, fz * drz};
            for (int k = 0; k < 9; ++k) nb->V[k] += 0.5 * M[k];
            nb->Ep += add_Ep;
        }
    }
    /* column-major symmetric matrix {{Vxx,Vxy,Vxz},{Vxy,Vyy,Vyz},{Vxz,Vyz,Vzz}} */
    double M[9] = {Vxx, Vxy, Vxz, Vxy, Vyy, Vyz, Vxz, Vyz, Vzz};
    for (int k = 0; k < 9; ++k) a->V[k] += 0.5 * M[k];
}

/* Per-thread scratch for the EAM per-atom passes. */
typedef struct {
    size_t cap;
    double (*rall)[3];
    double* r2;
    double* nCharge;
    double* dFemb;
    double* Femb;
    /* ghost / multi split */
    double (*gr)[3];
    double* gnc;
    md_atom** gnb;
    uint16_t* gkind;
    double (*kr)[3];
    double* knc;
    md_atom** knb;
} scratch;

static void scratch_reserve(scratch* s, size_t n) {
    if (n + 1 <= s->cap) return;
    size_t c = n + 1 < 256 ? 256 : n + 1;
    s->rall = realloc(s->rall, c * sizeof(*s->rall));
    s->r2 = realloc(s->r2, c * sizeof(double));
    s->nCharge = realloc(s->nCharge, c * sizeof(double));
    s->dFemb = realloc(s->dFemb, c * sizeof(double));
    s->Femb = realloc(s->Femb, c * sizeof(double));
    s->gr = realloc(s->gr, c * sizeof(*s->gr));
    s->gnc = realloc(s->gnc, c * sizeof(double));
    s->gnb = realloc(s->gnb, c * sizeof(md_atom*));
    s->gkind = realloc(s->gkind, c * sizeof(uint16_t));
    s->kr = realloc(s->kr, c * sizeof(*s->kr));
    s->knc = realloc(s->knc, c * sizeof(double));
    s->knb = realloc(s->knb, c * sizeof(md_atom*));
    s->cap = c;
}

static void scratch_free(scratch* s) {
    free(s->rall); free(s->r2); free(s->nCharge); free(s->dFemb); free(s->Femb);
    free(s->gr); free(s->gnc); free(s->gnb); free(s->gkind);
    free(s->kr); free(s->knc); free(s->knb);
}

/* EAM::density(self, ...) (EAM.cxx:532-560) + density(r2, size) (499-530) */
static void eam_density(const md_pot* p, md_atom* a, const nview* v, scratch* s) {
    if (v->nn == 0) return;
    double* r2 = s->r2;
    for (size_t i = 0; i < v->nn; i++) {
        double rx = v->rj[i][0] - a->r[0];
        double ry = v->rj[i][1] - a->r[1];
        double rz = v->rj[i][2] - a->r[2];
        r2[i] = rx * rx + ry * ry + rz * rz;
    }
    size_t natoms = 0;
    for (size_t i = 0; i < v->nn; i++) {
        if (r2[i] > p->R2cut) continue;
        if (r2[i] < 1e-15) continue;
        r2[natoms] = r2[i];
        ++natoms;
    }
    double SD = 0.0;
    for (size_t k = 0; k < natoms; k++) {
        double R1 = sqrt(r2[k]);
        double RN = R1 * p->dr1;
        int N1 = (int)trunc(RN);
        if (N1 < p->Nr1) {
            double VR = N1;
            double DV = RN - VR;
            RN = R1 - VR * p->dr;
            VR = (p->Rho[N1 + 1] - p->Rho[N1]) * p->dr1;
            double aa = (p->dRho[N1 + 1] - VR) - (VR - p->dRho[N1]);
            double bb = aa - (VR - p->dRho[N1]);
            double nr = p->Rho[N1] + RN * (p->dRho[N1] + DV * (DV * aa - bb));
            SD = SD + nr;
        }
    }
    a->nc += SD;
}

/* Shared per-pair spline of EAM::force / EAM::virial (EAM.cxx:417-463) */
static inline double eam_pair_ff(const md_pot* p, double R2, double AdF) {
    double R1 = sqrt(R2);
    double RN = R1 * p->dr1;
    int N1 = (int)trunc(RN);
    double FF, VR, DV;
    if (N1 < p->Nr1) {
        VR = N1;
        DV = RN - VR;
        RN = R1 - VR * p->dr;
        VR = (p->Rho[N1 + 1] - p->Rho[N1]) * p->dr1;
        double aa = (p->dRho[N1 + 1] - VR) - (VR - p->dRho[N1]);
        double bb = aa - (VR - p->dRho[N1]);
        FF = p->dRho[N1] + 2.0 * DV * (1.5 * DV * aa - bb);
        VR = (p->Vpar[N1 + 1] - p->Vpar[N1]) * p->dr1;
        aa = (p->dVpar[N1 + 1] - VR) - (VR - p->dVpar[N1]);
        bb = aa - (VR - p->dVpar[N1]);
        aa = aa * DV;
        VR = p->Vpar[N1] + RN * (p->dVpar[N1] + DV * (aa - bb));
        DV = p->dVpar[N1] + 2.0 * DV * (1.5 * aa - bb);
    } else {
        FF = 0.0;
        VR = 0.0;
        DV = 0.0;
    }
    return (AdF * FF + (DV * R1 - VR) / R2) / R1;
}

/* EAM::value(r2, size) (EAM.cxx:237-270): sum of V(r)/(2r) */
static double eam_value(const md_pot* p, const double* r2, size_t size) {
    double Utot = 0.0;
    for (size_t k = 0; k < size; k++) {
        double R1 = sqrt(r2[k]);
        double RN = R1 * p->dr1;
        int N1 = (int)trunc(RN);
        double VR;
        if (N1 < p->Nr1) {
            VR = N1;
            double DV = RN - VR;
            RN = R1 - VR * p->dr;
            VR = (p->Vpar[N1 + 1] - p->Vpar[N1]) * p->dr1;
            double aa = (p->dVpar[N1 + 1] - VR) - (VR - p->dVpar[N1]);
            double bb = aa - (VR - p->dVpar[N1]);
            aa = aa * DV;
            VR = p->Vpar[N1] + RN * (p->dVpar[N1] + DV * (aa - bb));
        } else {
            VR = 0.0;
        }
        Utot += 0.5 * VR / R1;
    }
    return Utot;
}

/* Gather + embedding + cut filter shared by EAM::force and EAM::virial
 * (EAM.cxx:465-497 and 367-415). Returns the number of cut pairs. */
static size_t eam_gather(const md_pot* p, const md_atom* a, const nview* v,
                         scratch* s) {
    size_t n = v->nn;
    for (size_t i = 0; i < n; i++) {
        double rx = v->rj[i][0] - a->r[0];
        double ry = v->rj[i][1] - a->r[1];
        double rz = v->rj[i][2] - a->r[2];
        s->r2[i] = rx * rx + ry * ry + rz * rz;
        s->rall[i][0] = rx;
        s->rall[i][1] = ry;
        s->rall[i][2] = rz;
        s->nCharge[i] = v->ncj[i];
    }
    s->nCharge[n] = a->nc;
    for (size_t i = 0; i <= n; ++i) {
        s->dFemb[i] = 0.0;
        s->Femb[i] = 0.0;
        eam_embed(p, s->nCharge[i], &s->Femb[i], &s->dFemb[i]);
    }
    size_t natoms = 0;
    for (size_t i = 0; i < n; i++) {
        if (s->r2[i] > p->R2cut) continue;
        if (s->r2[i] < 1e-15) continue;
        s->r2[natoms] = s->r2[i];
        s->rall[natoms][0] = s->rall[i][0];
        s->rall[natoms][1] = s->rall[i][1];
        s->rall[natoms][2] = s->rall[i][2];
        s->dFemb[natoms] = s->dFemb[i] + s->dFemb[n];
        ++natoms;
    }
    return natoms;
}

static void eam_force(const md_pot* p, md_atom* a, const nview* v, scratch* s) {
    if (v->nn == 0) return;
    size_t natoms = eam_gather(p, a, v, s);
    double F[3] = {0.0, 0.0, 0.0};
    for (size_t k = 0; k < natoms; k++) {
        double FF = eam_pair_ff(p, s->r2[k], s->dFemb[k]);
        F[0] += FF * s->rall[k][0];
        F[1] += FF * s->rall[k][1];
        F[2] += FF * s->rall[k][2];
    }
    a->f[0] += F[0];
    a->f[1] += F[1];
    a->f[2] += F[2];
}

static void eam_virial(const md_pot* p, md_atom* a, const nview* v, scratch* s) {
    if (v->nn == 0) return;
    size_t n = v->nn;
    size_t natoms = eam_gather(p, a, v, s);
    a->Em = s->Femb[n];
    double Vt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (size_t k = 0; k < natoms; k++) {
        double FF = eam_pair_ff(p, s->r2[k], s->dFemb[k]);
        double h = 0.5 * FF;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r)
                Vt[r + 3 * c] += h * s->rall[k][r] * s->rall[k][c];
    }
    for (int k = 0; k < 9; ++k) a->V[k] += Vt[k];
    a->Ep += eam_value(p, s->r2, natoms);
}

/* Pair spline of one cut pair (pair.cxx:316-346): force/r, and V(r) */
static inline double tab_pair_ff(const md_pot* p, double R2, double* VRout) {
    double R1 = sqrt(R2);
    double RN = R1 * p->dr1;
    int N1 = (int)trunc(RN);
    double VR = 0.0, DV = 0.0;
    if (N1 < p->Nr1) {
        VR = N1;
        DV = RN - VR;
        RN = R1 - VR * p->dr;
        VR = (p->Vpar[N1 + 1] - p->Vpar[N1]) * p->dr1;
        double aa = (p->dVpar[N1 + 1] - VR) - (VR - p->dVpar[N1]);
        double bb = aa - (VR - p->dVpar[N1]);
        aa = aa * DV;
        VR = p->Vpar[N1] + RN * (p->dVpar[N1] + DV * (aa - bb));
        DV = p->dVpar[N1] + 2.0 * DV * (1.5 * aa - bb);
    }
    if (VRout) *VRout = VR;
    return ((DV * R1 - VR) / R2) / R1;
}

/* Pair::force(self, ...) (pair.cxx:387-462): half lists push the pair
 * force onto both atoms; full lists sum the cut pairs from zero, then add. */
static void tab_force(const md_pot* p, md_atom* a, const nview* v) {
    double F[3] = {0.0, 0.0, 0.0};
    for (size_t i = 0; i < v->nn; i++) {
        double rx = v->rj[i][0] - a->r[0];
        double ry = v->rj[i][1] - a->r[1];
        double rz = v->rj[i][2] - a->r[2];
        double r2 = rx * rx + ry * ry + rz * rz;
        if (r2 > p->R2cut || r2 < 1e-15) continue;
        double FF = tab_pair_ff(p, r2, NULL);
        if (v->nbp) {
            double G[3] = {FF * rx, FF * ry, FF * rz};
            for (int k = 0; k < 3; ++k) {
                a->f[k] += G[k];
                v->nbp[i]->f[k] -= G[k];
            }
        } else {
            F[0] += FF * rx;
            F[1] += FF * ry;
            F[2] += FF * rz;
        }
    }
    if (!v->nbp) {
        a->f[0] += F[0];
        a->f[1] += F[1];
        a->f[2] += F[2];
    }
}

/* Pair::virial(self, ...) (pair.cxx:228-314): V += 1/2 FF d d^T and
 * Ep += V(r)/(2r) per cut pair (both atoms for half lists). */
static void tab_virial(const md_pot* p, md_atom* a, const nview* v) {
    double Vt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double Ut = 0.0;
    for (size_t i = 0; i < v->nn; i++) {
        double d[3] = {v->rj[i][0] - a->r[0], v->rj[i][1] - a->r[1],
                       v->rj[i][2] - a->r[2]};
        double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (r2 > p->R2cut || r2 < 1e-15) continue;
        double VR;
        double FF = tab_pair_ff(p, r2, &VR);
        double E = 0.5 * VR / sqrt(r2);
        if (v->nbp) {
            double M[9];
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) M[r + 3 * c] = 0.5 * (FF * d[r]) * d[c];
            for (int k = 0; k < 9; ++k) {
                a->V[k] += M[k];
                v->nbp[i]->V[k] += M[k];
            }
            a->Ep += E;
            v->nbp[i]->Ep += E;
        } else {
            double h = 0.5 * FF;
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) Vt[r + 3 * c] += h * d[r] * d[c];
            Ut += E;
        }
    }
    if (!v->nbp) {
        for (int k = 0; k < 9; ++k) a->V[k] += Vt[k];
        a->Ep += Ut;
    }
}

/* LJs pair terms (LJs.cxx:153-166 force/r, 90-101 energy V(r)/2) */
static inline double ljs_ff(const md_pot* p, double r2, double* E) {
    const double X2min = 1.2599210498948732;
    double XX = p->rVr1 * r2 - X2min;
    double FV = p->rVr2 / r2;
    double Ur = FV * FV * FV;
    if (E) *E = p->aVr * (Ur * (Ur - 1.0) - (p->aLJ3 + p->bLJ2 * XX) * XX * XX);
    return p->aVr2 * (Ur * (Ur - 0.5) * FV + (p->aLJ + p->bLJ * XX) * XX);
}

void md_pot_values(const md_pot* p, const double* r2, size_t n, double* u) {
    /* Potential::value(r2[], U[], n): EAM.cxx:141-174 and pair.cxx:81-114
     * (V(r)/2r from the Vpar spline, 0 past the table), LJs.cxx:61-71;
     * LJsCut keeps Base::value (base.cxx:19), which leaves U alone: 0 here. */
    for (size_t k = 0; k < n; ++k) {
        double e = 0.0;
        if (p->type == MD_POT_EAM || p->type == MD_POT_TAB) {
            e = eam_value(p, &r2[k], 1);
        } else if (p->type == MD_POT_LJS) {
            ljs_ff(p, r2[k], &e);
        }
        u[k] = e;
    }
}

/* LJs::force(self, ...) (LJs.cxx:196-256) */
static void ljs_force(const md_pot* p, md_atom* a, const nview* v) {
    double F[3] = {0.0, 0.0, 0.0};
    for (size_t i = 0; i < v->nn; i++) {
        double d[3] = {v->rj[i][0] - a->r[0], v->rj[i][1] - a->r[1], v->rj[i][2] - a->r[2]};
        double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (r2 > p->R2cut || r2 < 1e-15) continue;
        double FF = ljs_ff(p, r2, NULL);
        if (v->nbp) {
            for (int k = 0; k < 3; ++k) {
                double G = FF * d[k];
                a->f[k] += G;
                v->nbp[i]->f[k] -= G;
            }
        } else {
            F[0] += FF * d[0];
            F[1] += FF * d[1];
            F[2] += FF * d[2];
        }
    }
    if (!v->nbp) {
        a->f[0] += F[0];
        a->f[1] += F[1];
        a->f[2] += F[2];
    }
}

/* LJs::virial(self, ...) (LJs.cxx:103-151) */
static void ljs_virial(const md_pot* p, md_atom* a, const nview* v) {
    double Vt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double Ut = 0.0;
    for (size_t i = 0; i < v->nn; i++) {
        double d[3] = {v->rj[i][0] - a->r[0], v->rj[i][1] - a->r[1], v->rj[i][2] - a->r[2]};
        double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (r2 > p->R2cut || r2 < 1e-15) continue;
        double E;
        double FF = ljs_ff(p, r2, &E);
        double G[3] = {FF * d[0], FF * d[1], FF * d[2]};
        if (v->nbp) {
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) {
                    double m = 0.5 * G[r] * d[c];
                    a->V[r + 3 * c] += m;
                    v->nbp[i]->V[r + 3 * c] += m;
                }
            a->Ep += E;
            v->nbp[i]->Ep += E;
        } else {
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) Vt[r + 3 * c] += 0.5 * G[r] * d[c];
            Ut += E;
        }
    }
    if (!v->nbp) {
        for (int k = 0; k < 9; ++k) a->V[k] += Vt[k];
        a->Ep += Ut;
    }
}

/* ------------------------------------------------------------------------ */
/* Langevin thermostat — mdcraft/solver/thermostat/langevin.cxx:8-42        */
/* ------------------------------------------------------------------------ */

#define MD_MAXTHERMO 8

struct md_thermo {
    int n;
    md_langevin term[MD_MAXTHERMO];
};

md_thermo* md_thermo_create(void) { return (md_thermo*)calloc(1, sizeof(md_thermo)); }

int md_thermo_add(md_thermo* t, const md_langevin* term) {
    if (!t || !term || t->n >= MD_MAXTHERMO) return MDREF_ERR_INVALID;
    t->term[t->n++] = *term;
    return MDREF_OK;
}

void md_thermo_destroy(md_thermo* t) { free(t); }

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11): ten rounds of two 32x32->64 multiplications
 * with a Weyl-sequence key schedule. */
void md_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                      uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* Two Box-Muller pairs from one Philox block; the first three normals. */
void md_langevin_normals(uint64_t seed, uint32_t atom, uint32_t call,
                         uint32_t term, double z[3]) {
    const uint32_t ctr[4] = {atom, call, term, 0u};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t x[4];
    md_philox4x32_10(ctr, key, x);
    const double k32 = 2.3283064365386962890625e-10; /* 2^-32 */
    const double two_pi = 6.283185307179586476925;
    double u0 = ((double)x[0] + 0.5) * k32, u1 = ((double)x[1] + 0.5) * k32;
    double u2 = ((double)x[2] + 0.5) * k32, u3 = ((double)x[3] + 0.5) * k32;
    double ra = sqrt(-2.0 * log(u0)), rb = sqrt(-2.0 * log(u2));
    z[0] = ra * cos(two_pi * u1);
    z[1] = ra * sin(two_pi * u1);
    z[2] = rb * cos(two_pi * u3);
}

/* Langevin::apply_one (langevin.cxx:29-42) for every term, in order. */
static void thermo_apply(const md_thermo* t, md_atom* a, uint32_t atom,
                         uint32_t call) {
    for (int q = 0; q < t->n; ++q) {
        const md_langevin* L = &t->term[q];
        if (a->r[0] < L->xmin || a->r[0] > L->xmax) continue;
        /* sigma = sqrt(2 beta Kb T / dt) (langevin.cxx:24), Kb of base.h:10 */
        double sigma = sqrt(2.0 * L->beta * 0.008314462175 * L->temperature / L->time_step);
        double z[3];
        md_langevin_normals(L->seed, atom, call, (uint32_t)q, z);
        double sqrt_mass = sqrt(a->m);
        for (int k = 0; k < 3; ++k) {
            double tf = (z[k] * sigma + 0.0) * sqrt_mass;
            tf -= (a->v[k] - L->U[k]) * L->beta * a->m;
            tf = tf * L->heat[k];
            a->f[k] += tf;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Solvers — mdcraft/solver/{pair,single,multi}.cxx + boundary/periodic.cxx */
/* ------------------------------------------------------------------------ */

#define MD_MAXK 8
enum { STAGE_CHARGE = 0, STAGE_FORCES = 1 };

struct md_solver {
    int multi, nkinds, nthreads;
    md_pot* pot[MD_MAXK][MD_MAXK];
    int nstages, stages[2];
    int periodic;
    md_domain dom;
    scratch* scr;
    int nscr;
    const md_thermo* thermo;
    uint32_t thermo_calls;
};

void md_solver_set_thermostat(md_solver* s, md_thermo* t, uint32_t calls) {
    s->thermo = t;
    s->thermo_calls = calls;
}

uint32_t md_solver_thermo_calls(const md_solver* s) { return s->thermo_calls; }

static int pair_type(const md_pot* p) {
    return p->type == MD_POT_PAIR || p->type == MD_POT_TAB || p->type == MD_POT_LJS;
}

static md_solver* solver_new(const md_domain* pd, int nthreads) {
    md_solver* s = (md_solver*)calloc(1, sizeof(md_solver));
    s->nthreads = nthreads < 1 ? 1 : nthreads;
    if (pd) {
        s->periodic = 1;
        s->dom = *pd;
    }
    s->nscr = s->nthreads;
    s->scr = (scratch*)calloc((size_t)s->nscr, sizeof(scratch));
    return s;
}

md_solver* md_solver_single(md_pot* p, const md_domain* pd, int nthreads) {
    /* Single::Single (single.cxx:11-28) */
    md_solver* s = solver_new(pd, nthreads);
    s->nkinds = 1;
    s->pot[0][0] = p;
    if (pair_type(p)) {
        s->nstages = 1;
        s->stages[0] = STAGE_FORCES;
    } else if (p->type == MD_POT_EAM) {
        s->nstages = 2;
        s->stages[0] = STAGE_CHARGE;
        s->stages[1] = STAGE_FORCES;
    }
    return s;
}

md_solver* md_solver_multi(int nkinds, const md_domain* pd, int nthreads) {
    if (nkinds < 1 || nkinds > MD_MAXK) return NULL;
    md_solver* s = solver_new(pd, nthreads);
    s->multi = 1;
    s->nkinds = nkinds;
    return s;
}

int md_solver_add_potential(md_solver* s, int i, int j, md_pot* p) {
    /* Multi::add_potential (multi.cxx:28-49) */
    if (!s->multi || i < 0 || j < 0 || i >= s->nkinds || j >= s->nkinds)
        return MDREF_ERR_INVALID;
    s->pot[i][j] = p;
    s->pot[j][i] = p;
    if (s->nstages == 0) {
        if (pair_type(p)) {
            s->nstages = 1;
            s->stages[0] = STAGE_FORCES;
        } else if (p->type == MD_POT_EAM) {
            s->nstages = 2;
            s->stages[0] = STAGE_CHARGE;
            s->stages[1] = STAGE_FORCES;
        }
    } else if (p->type == MD_POT_EAM && s->nstages == 1) {
        s->nstages = 2;
        s->stages[0] = STAGE_CHARGE;
        s->stages[1] = STAGE_FORCES;
    }
    return MDREF_OK;
}

void md_solver_destroy(md_solver* s) {
    if (!s) return;
    for (int t = 0; t < s->nscr; ++t) scratch_free(&s->scr[t]);
    free(s->scr);
    free(s);
}

int md_solver_num_stages(const md_solver* s) { return s->nstages; }

typedef struct {
    md_solver* s;
    md_atom* atoms;
    size_t n;
    const md_nlist* nl;
    int op; /* 0 charge, 1 force, 2 virial */
} st_ctx;

/* Potential dispatch on one neighbour view. */
static void pot_apply(md_pot* p, int op, md_atom* a, const nview* v, scratch* s) {
    if (!p) return;
    if (p->type == MD_POT_PAIR) {
        if (op == 1) ljcut_force(p, a, v);
        else if (op == 2) ljcut_virial(p, a, v);
        /* Base::density is a no-op for pair potentials */
    } else if (p->type == MD_POT_TAB) {
        if (op == 1) tab_force(p, a, v);
        else if (op == 2) tab_virial(p, a, v);
    } else if (p->type == MD_POT_LJS) {
        if (op == 1) ljs_force(p, a, v);
        else if (op == 2) ljs_virial(p, a, v);
    } else if (p->type == MD_POT_EAM) {
        if (op == 0) eam_density(p, a, v, s);
        else if (op == 1) eam_force(p, a, v, s);
        else eam_virial(p, a, v, s);
    }
}

/* Single::*_one / Multi::*_one on one neighbour view (single.cxx:55-83,
 * multi.cxx:65-151). `kinds` gives the neighbours' kinds (Multi split). */
static void solver_one(md_solver* s, int op, md_atom* a, const nview* v,
                       const uint16_t* kinds, scratch* sc) {
    if (a->tag == 0) return;
    if (!s->multi) {
        pot_apply(s->pot[0][0], op, a, v, sc);
        return;
    }
    /* Multi: split the list by neighbour kind, keeping list order */
    int ki = a->kind;
    for (int kj = 0; kj < s->nkinds; ++kj) {
        size_t m = 0;
        for (size_t i = 0; i < v->nn; ++i) {
            if (kinds[i] != kj) continue;
            sc->kr[m][0] = v->rj[i][0];
            sc->kr[m][1] = v->rj[i][1];
            sc->kr[m][2] = v->rj[i][2];
            sc->knc[m] = v->ncj[i];
            sc->knb[m] = v->nbp ? v->nbp[i] : NULL;
            ++m;
        }
        nview sub = {m, (const double(*)[3])sc->kr, sc->knc, v->nbp ? sc->knb : NULL};
        if (ki < s->nkinds) pot_apply(s->pot[ki][kj], op, a, &sub, sc);
    }
}

static void stage_range(void* pctx, size_t b, size_t e, int tid) {
    /* Pair::charge / Pair::forces / Pair::virials per-atom lambda
     * (pair.cxx:44-114) with the Periodic ghost pass (periodic.cxx:36-102) */
    st_ctx* c = (st_ctx*)pctx;
    md_solver* s = c->s;
    scratch* sc = &s->scr[tid];
    const md_nlist* nl = c->nl;
    for (size_t i = b; i < e; ++i) {
        md_atom* a = &c->atoms[i];
        size_t nn = i < nl->n ? nl->counts[i] : 0;
        const uint64_t* L = i < nl->n ? nl->lists[i] : NULL;
        scratch_reserve(sc, nn);
        /* main pass over the Verlet list */
        double (*rj)[3] = sc->gr;
        for (size_t k = 0; k < nn; ++k) {
            const md_atom* nb = &c->atoms[L[k]];
            rj[k][0] = nb->r[0];
            rj[k][1] = nb->r[1];
            rj[k][2] = nb->r[2];
            sc->gnc[k] = nb->nc;
            sc->gkind[k] = nb->kind;
            sc->gnb[k] = &c->atoms[L[k]];
        }
        nview v = {nn, (const double(*)[3])rj, sc->gnc, nl->half ? sc->gnb : NULL};
        /* The potentials reuse rall/r2; they do not touch gr/gnc/gkind. */
        solver_one(s, c->op, a, &v, sc->gkind, sc);
        /* thermostat.apply_one, for every atom (pair.cxx:81) */
        if (c->op == 1 && s->thermo) thermo_apply(s->thermo, a, (uint32_t)i, s->thermo_calls);
        if (!a->bc) continue;
        /* Periodic::prepare_ghosts (periodic.cxx:36-60) */
        size_t g = 0;
        for (size_t k = 0; k < nn; ++k) {
            const md_atom* nb = &c->atoms[L[k]];
            double dist[3] = {nb->r[0] - a->r[0], nb->r[1] - a->r[1], nb->r[2] - a->r[2]};
            double r2rns = nb->rns < a->rns ? a->rns : nb->rns;
            r2rns *= r2rns;
            if (dist[0] * dist[0] + dist[1] * dist[1] + dist[2] * dist[2] < r2rns) continue;
            md_domain_shortest(&s->dom, dist);
            if (dist[0] * dist[0] + dist[1] * dist[1] + dist[2] * dist[2] > r2rns) continue;
            rj[g][0] = a->r[0] + dist[0];
            rj[g][1] = a->r[1] + dist[1];
            rj[g][2] = a->r[2] + dist[2];
            sc->gnc[g] = nb->nc;
            sc->gkind[g] = nb->kind;
            ++g;
        }
        if (g == 0) continue;
        nview gv = {g, (const double(*)[3])rj, sc->gnc, NULL};
        solver_one(s, c->op, a, &gv, sc->gkind, sc);
    }
}

static void run_stage(md_solver* s, md_atom* atoms, size_t n,
                      const md_nlist* nl, int op) {
    st_ctx c = {s, atoms, n, nl, op};
    parallel_for(nl->half ? 1 : s->nthreads, n, stage_range, &c);
    if (op == 1 && s->thermo) s->thermo_calls += 1;
}

typedef struct {
    md_solver* s;
    md_atom* atoms;
} prep_ctx;

static void prepare_range(void* pctx, size_t b, size_t e, int tid) {
    /* Pair::prepare (pair.cxx:16-29) with Single::prepare_one
     * (single.cxx:38-53) / Multi::prepare_one (multi.cxx:51-63) and
     * Periodic::prepare_one (periodic.cxx:9-34) */
    (void)tid;
    prep_ctx* c = (prep_ctx*)pctx;
    md_solver* s = c->s;
    for (size_t i = b; i < e; ++i) {
        md_atom* a = &c->atoms[i];
        if (a->tag != 0) {
            a->f[0] = a->f[1] = a->f[2] = 0.0;
            for (int k = 0; k < 9; ++k) a->V[k] = 0.0;
            a->Ep = 0.0;
            if (s->multi) {
                a->Em = 0.0;
                a->nc = 0.0;
            } else {
                if (s->pot[0][0]->type == MD_POT_EAM) {
                    a->Em = 0.0;
                    a->nc = 0.0;
                }
                a->rcut = s->pot[0][0]->R1cut;
            }
        }
        a->bc = 0;
        if (s->periodic && a->tag != 0) {
            int need = 0;
            for (int d = 0; d < 3; ++d)
                need = need || md_domain_nearest_distance(&s->dom, a->r, d) < a->rns;
            a->bc += need ? 1 : 0;
        }
    }
}

void md_solver_prepare(md_solver* s, md_atom* atoms, size_t n) {
    prep_ctx c = {s, atoms};
    parallel_for(s->nthreads, n, prepare_range, &c);
}

void md_solver_charge(md_solver* s, md_atom* atoms, size_t n, const md_nlist* nl) {
    run_stage(s, atoms, n, nl, 0);
}

void md_solver_forces(md_solver* s, md_atom* atoms, size_t n, const md_nlist* nl) {
    run_stage(s, atoms, n, nl, 1);
}

void md_solver_virials(md_solver* s, md_atom* atoms, size_t n, const md_nlist* nl) {
    run_stage(s, atoms, n, nl, 2);
}

void md_solver_stages(md_solver* s, md_atom* atoms, size_t n, const md_nlist* nl) {
    for (int k = 0; k < s->nstages; ++k) {
        if (s->stages[k] == STAGE_CHARGE) md_solver_charge(s, atoms, n, nl);
        else md_solver_forces(s, atoms, n, nl);
    }
}

/* ------------------------------------------------------------------------ */
/* Verlet stepper — mdcraft/solver/stepper/verlet.cxx:36-85                 */
/* ------------------------------------------------------------------------ */

typedef struct {
    md_atom* atoms;
    double dt;
} vv_ctx;

static void coords_range(void* p, size_t b, size_t e, int tid) {
    /* Verlet::step_one_coords (verlet.cxx:71-78) */
    (void)tid;
    vv_ctx* c = (vv_ctx*)p;
    double dt = c->dt;
    for (size_t i = b; i < e; ++i) {
        md_atom* a = &c->atoms[i];
        if (a->tag == 0) continue;
        for (int k = 0; k < 3; ++k) {
            double acc = a->f[k] / a->m;
            double v = a->v[k] + acc * dt * 0.5;
            a->r[k] = a->r[k] + v * dt;
            a->v[k] = v;
        }
    }
}

static void velocities_range(void* p, size_t b, size_t e, int tid) {
    /* Verlet::step_one_velocities (verlet.cxx:80-85) */
    (void)tid;
    vv_ctx* c = (vv_ctx*)p;
    double dt = c->dt;
    for (size_t i = b; i < e; ++i) {
        md_atom* a = &c->atoms[i];
        if (a->tag == 0) continue;
        for (int k = 0; k < 3; ++k) {
            double acc = a->f[k] / a->m;
            a->v[k] = a->v[k] + acc * 0.5 * dt;
        }
    }
}

void md_verlet_make_step(md_solver* s, md_atom* atoms, size_t n,
                         const md_nlist* nl, double dt) {
    /* Verlet::make_step (verlet.cxx:36-48) */
    vv_ctx c = {atoms, dt};
    parallel_for(s->nthreads, n, coords_range, &c);
    md_solver_prepare(s, atoms, n);
    md_solver_stages(s, atoms, n, nl);
    parallel_for(s->nthreads, n, velocities_range, &c);
}

long md_run(md_solver* s, md_atom* atoms, size_t n, md_nlist* nl,
            const md_domain* d, double dt, long steps) {
    long rebuilds = 0;
    for (long k = 0; k < steps; ++k) {
        md_verlet_make_step(s, atoms, n, nl, dt);
        if (md_nlist_decide(nl, d, atoms, n)) {
            int st = md_nlist_update(nl, d, atoms, n, -1.0);
            if (st != MDREF_OK && st != MDREF_ERR_RANGE) return st;
            ++rebuilds;
        }
    }
    return rebuilds;
}

void md_measure_state(const md_atom* atoms, size_t n, double out[8]) {
    /* measure_state (test/cxx/support/md_test_utils.h:214-239) */
    double Ep = 0.0, Em = 0.0, vir = 0.0, tm = 0.0;
    double com[3] = {0.0, 0.0, 0.0};
    for (size_t i = 0; i < n; ++i) {
        const md_atom* a = &atoms[i];
        Ep += a->Ep;
        Em += a->Em;
        vir += a->V[0] + a->V[4] + a->V[8];
        for (int k = 0; k < 3; ++k) com[k] += a->m * a->v[k];
        tm += a->m;
    }
    if (tm > 0.0) {
        for (int k = 0; k < 3; ++k) com[k] /= tm;
    } else {
        com[0] = com[1] = com[2] = 0.0;
    }
    double KE = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const md_atom* a = &atoms[i];
        double rv[3] = {a->v[0] - com[0], a->v[1] - com[1], a->v[2] - com[2]};
        KE += 0.5 * a->m * (rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    }
    out[0] = Ep;
    out[1] = Em;
    out[2] = KE;
    out[3] = Ep + Em + KE;
    out[4] = vir;
    out[5] = com[0];
    out[6] = com[1];
    out[7] = com[2];
}
