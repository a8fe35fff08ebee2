/*
 * boids_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle; see boids_oracle.h).
 *
 * A plain-C restatement of the reference's per-timestep boid update.  Every
 * floating-point expression follows the reference's C++ types operation by
 * operation: Vector3D is float (src/vector3D.h:33), the parameters are double
 * (src/dtype.h:39-49), and the mixed expressions promote to double exactly
 * where the reference's do.  The file must be compiled with
 * -ffp-contract=off (GCC contracts a*b+c into FMA by default on aarch64,
 * which the reference's x86 build never does) and without -ffast-math.
 */
#include "boids_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ rng */

/* srand48: X = (seed & 0xffffffff) << 16 | 0x330e (POSIX; glibc masks the
 * long seed to 32 bits on LP64). */
void orc_srand48(uint64_t *state, long seed)
{
    uint64_t v = (uint64_t)seed & 0xffffffffULL;
    *state = (v << 16) | 0x330eULL;
}

/* drand48: X <- (0x5deece66d * X + 0xb) mod 2^48, result X * 2^-48. */
double orc_drand48(uint64_t *state)
{
    *state = (0x5deece66dULL * *state + 0xbULL) & 0xffffffffffffULL;
    return (double)*state * (1.0 / 281474976710656.0);
}

/* ------------------------------------------------------------------ init */

int orc_init(const orc_params *p, int kind, int seeded, int seed, float *pos, float *vel)
{
    /* glibc's drand48 state before any srand48 call is X = 0. */
    uint64_t X = 0;
    const double F = p->field;
    if (seeded) orc_srand48(&X, (long)seed);
    if (kind != 0 && kind != 1) return -1;
    for (uint32_t i = 0; i < p->n; i++) {
        if (kind == 1) {
            /* "test", src/boid_simulation_grid.cpp:100-108 */
            pos[3 * i + 0] = (float)(F * 3 / 8 + orc_drand48(&X) * F / 4);
            pos[3 * i + 1] = (float)(F * 3 / 8 + orc_drand48(&X) * F / 4);
            if (orc_drand48(&X) > 0.5) {
                pos[3 * i + 2] = (float)(orc_drand48(&X) * F / 4 + F * 3 / 4);
            } else {
                pos[3 * i + 2] = (float)(orc_drand48(&X) * F / 4);
            }
        } else {
            /* "random_uniform", src/boid_simulation_grid.cpp:123-126 */
            pos[3 * i + 0] = (float)(F * orc_drand48(&X));
            pos[3 * i + 1] = (float)(F * orc_drand48(&X));
            pos[3 * i + 2] = (float)(F * orc_drand48(&X));
        }
        /* speed and angles, src/boid_simulation_grid.cpp:127-132 */
        double v = orc_drand48(&X) * (p->vmax - p->vmin) + p->vmin;
        double th1 = orc_drand48(&X) * M_PI;
        double th2 = orc_drand48(&X) * 2.0 * M_PI;
        vel[3 * i + 0] = (float)(v * sin(th1) * cos(th2));
        vel[3 * i + 1] = (float)(v * sin(th1) * sin(th2));
        vel[3 * i + 2] = (float)(v * cos(th1));
    }
    return 0;
}

/* ------------------------------------------------------------------ pair logic */

typedef struct { float x, y, z; } v3;

static inline v3 ld3(const float *a, uint32_t i)
{
    v3 r = { a[3 * i], a[3 * i + 1], a[3 * i + 2] };
    return r;
}

/* Vector3D::norm, src/vector3D.cpp:64-67: float d = x*x + y*y + z*z; sqrt(d). */
static inline float norm3(v3 a)
{
    float d = a.x * a.x + a.y * a.y + a.z * a.z;
    return sqrtf(d);
}

/* Minimum-image copy of boid j as seen from boid i,
 * src/boid_simulation_grid.cpp:200-214.  The difference is a float, the
 * comparison promotes it to double against field/2, and the shift is done in
 * double and rounded back to float (compound assignment float -= double). */
static inline float image1(float xj, float xi, double F)
{
    if ((double)(xj - xi) > F / 2) {
        xj = (float)((double)xj - F);
    } else if ((double)(xi - xj) > F / 2) {
        xj = (float)((double)xj + F);
    }
    return xj;
}

static inline v3 image_of(v3 pj, v3 pi, double F)
{
    v3 r = { image1(pj.x, pi.x, F), image1(pj.y, pi.y, F), image1(pj.z, pi.z, F) };
    return r;
}

/* Boid::isInsideArea, src/boid.cpp:27-42, with this = boid i (position pi,
 * velocity vi) and _b = the imaged target (position pj). */
static inline int inside_area(v3 pi, v3 vi, v3 pj, double r, double a)
{
    v3 d = { pi.x - pj.x, pi.y - pj.y, pi.z - pj.z };
    if ((double)norm3(d) < r) {
        if (a >= 1.0) return 1;
        v3 rel = { pj.x - pi.x, pj.y - pi.y, pj.z - pi.z };
        float dot = vi.x * rel.x + vi.y * rel.y + vi.z * rel.z;   /* operator*(u, v) */
        float den = norm3(vi) * norm3(rel);
        double th = (double)acosf(dot / den);
        return th <= M_PI * a;
    }
    return 0;
}

/* rule flags: bit 0 cohesion, bit 1 separation, bit 2 alignment
 * (the order of the tests at src/boid_simulation_grid.cpp:220-238). */
static inline int pair_flags(const orc_params *p, v3 pi, v3 vi, v3 pj_img)
{
    int f = 0;
    if (inside_area(pi, vi, pj_img, p->coh_r, p->coh_a)) f |= 1;
    if (inside_area(pi, vi, pj_img, p->sep_r, p->sep_a)) f |= 2;
    if (inside_area(pi, vi, pj_img, p->ali_r, p->ali_a)) f |= 4;
    return f;
}

typedef struct {
    v3 coh, sep, ali;
    int ncoh, nsep, nali;
} acc_t;

static inline void acc_zero(acc_t *a) { memset(a, 0, sizeof(*a)); }

/* The body of the candidate loop for one candidate j,
 * src/boid_simulation_grid.cpp:197-239. */
static inline void acc_pair(const orc_params *p, acc_t *a, v3 pi, v3 vi, v3 pj, v3 vj)
{
    v3 t = image_of(pj, pi, p->field);
    int f = pair_flags(p, pi, vi, t);
    if (f & 1) {
        a->ncoh++;
        a->coh.x += t.x; a->coh.y += t.y; a->coh.z += t.z;
    }
    if (f & 2) {
        a->nsep++;
        v3 d = { pi.x - t.x, pi.y - t.y, pi.z - t.z };
        float n = norm3(d);                                     /* Vector3D::normalized */
        a->sep.x += d.x / n; a->sep.y += d.y / n; a->sep.z += d.z / n;
    }
    if (f & 4) {
        a->nali++;
        a->ali.x += vj.x; a->ali.y += vj.y; a->ali.z += vj.z;   /* un-imaged velocity */
    }
}

/* After the candidate loop, src/boid_simulation_grid.cpp:243-252.  Writes the
 * velocity increment and, when asked, get_force's nine floats
 * (src/boid_simulation_grid.cpp:319-334). */
static inline void acc_finish(const orc_params *p, acc_t *a, v3 pi, v3 vi, float *dv, float *f9)
{
    if (a->ncoh != 0) {
        float k = (float)a->ncoh;                               /* operator/(v, float) */
        a->coh.x = a->coh.x / k - pi.x;
        a->coh.y = a->coh.y / k - pi.y;
        a->coh.z = a->coh.z / k - pi.z;
    }
    if (a->nali != 0) {
        float k = (float)a->nali;
        a->ali.x = a->ali.x / k - vi.x;
        a->ali.y = a->ali.y / k - vi.y;
        a->ali.z = a->ali.z / k - vi.z;
    }
    /* double * Vector3D resolves to operator*(float, const Vector3D&). */
    const float cc = (float)p->coh_c, cs = (float)p->sep_c, ca = (float)p->ali_c;
    v3 fc = { a->coh.x * cc, a->coh.y * cc, a->coh.z * cc };
    v3 fs = { a->sep.x * cs, a->sep.y * cs, a->sep.z * cs };
    v3 fa = { a->ali.x * ca, a->ali.y * ca, a->ali.z * ca };
    dv[0] = fc.x + fs.x + fa.x;
    dv[1] = fc.y + fs.y + fa.y;
    dv[2] = fc.z + fs.z + fa.z;
    if (f9) {
        f9[0] = fc.x; f9[1] = fc.y; f9[2] = fc.z;
        f9[3] = fs.x; f9[4] = fs.y; f9[5] = fs.z;
        f9[6] = fa.x; f9[7] = fa.y; f9[8] = fa.z;
    }
}

/* Integration of one boid, src/boid_simulation_grid.cpp:262-289. */
static inline void integrate1(const orc_params *p, float *x, float *v, const float *dv)
{
    const double F = p->field;
    v3 vel = { v[0] + dv[0], v[1] + dv[1], v[2] + dv[2] };
    float n = norm3(vel);
    if ((double)n > 0. && (double)n > p->vmax) {
        float k = (float)p->vmax;
        vel.x = vel.x / n * k; vel.y = vel.y / n * k; vel.z = vel.z / n * k;
    } else if ((double)n > 0. && (double)n < p->vmin) {
        float k = (float)p->vmin;
        vel.x = vel.x / n * k; vel.y = vel.y / n * k; vel.z = vel.z / n * k;
    }
    v[0] = vel.x; v[1] = vel.y; v[2] = vel.z;
    for (int c = 0; c < 3; c++) {
        float xc = x[c] + v[c];
        if ((double)xc < 0.0) {
            xc = (float)(F + (double)xc);
        } else if ((double)xc > F) {
            xc = (float)((double)xc - F);
        }
        x[c] = xc;
    }
}

static void set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* ------------------------------------------------------------------ all-pairs */

void orc_step_allpairs(const orc_params *p, float *pos, float *vel, float *force9, int nthreads)
{
    const uint32_t N = p->n;
    float *dv = (float *)malloc(sizeof(float) * 3 * (size_t)(N ? N : 1));
    set_threads(nthreads);
    /* rule loop, src/boid_simulation.cpp:153-213 */
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)N; i++) {
        acc_t a;
        acc_zero(&a);
        v3 pi = ld3(pos, (uint32_t)i), vi = ld3(vel, (uint32_t)i);
        for (uint32_t j = 0; j < N; j++) {
            if ((uint32_t)i == j) continue;
            acc_pair(p, &a, pi, vi, ld3(pos, j), ld3(vel, j));
        }
        acc_finish(p, &a, pi, vi, dv + 3 * i, force9 ? force9 + 9 * i : NULL);
    }
    /* integration loop, src/boid_simulation.cpp:218-248 (serial in the
     * reference: its omp for is outside the parallel region) */
    for (uint32_t i = 0; i < N; i++) integrate1(p, pos + 3 * i, vel + 3 * i, dv + 3 * i);
    free(dv);
}

/* ------------------------------------------------------------------ reference grid */

struct orc_grid {
    orc_params p;
    float R, GS;
    unsigned G;
    int32_t *gi;         /* 8 per boid: Boid::grid_index */
    int32_t *start;      /* G^3 + 1 */
    int32_t *items;      /* CSR cell lists, push_back order */
    size_t items_cap;
    float *dv;
};

/* BoidSimulation::setup grid sizing, src/boid_simulation_grid.cpp:80-89.
 * Returns 0, or -1 where the reference would abort ("Invalid GRID_NUM!!!")
 * or divide by a zero GRID_NUM. */
int orc_grid_geometry(const orc_params *p, float *range, int *grid_num, float *grid_size)
{
    double m = (p->coh_r < p->ali_r) ? p->ali_r : p->coh_r;   /* std::max */
    m = (m < p->sep_r) ? p->sep_r : m;
    float R = (float)m;
    int gn = (int)(p->field / (double)(R * 2));               /* INTERACTION_RANGE*2 is float */
    unsigned G = (unsigned)gn;
    if (G == 0 || gn < 0) return -1;
    float GS = (float)(p->field / (double)G);
    if (R * 2 >= GS) return -1;
    if (range) *range = R;
    if (grid_num) *grid_num = (int)G;
    if (grid_size) *grid_size = GS;
    return 0;
}

/* Boid::grid_index of one boid, src/boid_simulation_grid.cpp:400-443. */
static void ref_cells1(float R, float GS, unsigned G, v3 x, int32_t *gi)
{
    int g[3][2];
    float c[3] = { x.x, x.y, x.z };
    for (int d = 0; d < 3; d++) {
        g[d][0] = (int)(c[d] / GS);
        if ((unsigned)g[d][0] == G) g[d][0] = (int)G - 1;
    }
    for (int d = 0; d < 3; d++) {
        float pig = c[d] - (float)g[d][0] * GS;
        if (pig <= R) {
            g[d][1] = (int)(((unsigned)(g[d][0] - 1) + G) % G);
        } else if (pig >= GS - R) {
            g[d][1] = (int)(((unsigned)g[d][0] + 1) % G);
        } else {
            g[d][1] = -1;
        }
    }
    unsigned n = 0;
    for (int i = 0; i < 2; i++) {
        if (g[0][i] == -1) continue;
        for (int j = 0; j < 2; j++) {
            if (g[1][j] == -1) continue;
            for (int k = 0; k < 2; k++) {
                if (g[2][k] == -1) continue;
                gi[n++] = (int32_t)((unsigned)g[0][i] + (unsigned)g[1][j] * G + (unsigned)g[2][k] * G * G);
            }
        }
    }
    while (n < 8) gi[n++] = -1;
}

int orc_ref_cells(const orc_params *p, const float *pos, int32_t *grid_index8)
{
    float R, GS;
    int G;
    if (orc_grid_geometry(p, &R, &G, &GS) != 0) return -1;
    for (uint32_t i = 0; i < p->n; i++) ref_cells1(R, GS, (unsigned)G, ld3(pos, i), grid_index8 + 8 * i);
    return 0;
}

orc_grid *orc_grid_create(const orc_params *p)
{
    orc_grid *g = (orc_grid *)calloc(1, sizeof(orc_grid));
    int G;
    if (!g) return NULL;
    g->p = *p;
    if (orc_grid_geometry(p, &g->R, &G, &g->GS) != 0) { free(g); return NULL; }
    g->G = (unsigned)G;
    size_t ncell = (size_t)g->G * g->G * g->G;
    size_t n = p->n ? p->n : 1;
    g->gi = (int32_t *)malloc(sizeof(int32_t) * 8 * n);
    g->start = (int32_t *)calloc(ncell + 1, sizeof(int32_t));
    g->items_cap = 8 * n;
    g->items = (int32_t *)malloc(sizeof(int32_t) * g->items_cap);
    g->dv = (float *)malloc(sizeof(float) * 3 * n);
    if (!g->gi || !g->start || !g->items || !g->dv) { orc_grid_destroy(g); return NULL; }
    return g;
}

void orc_grid_destroy(orc_grid *g)
{
    if (!g) return;
    free(g->gi); free(g->start); free(g->items); free(g->dv);
    free(g);
}

/* clear_list_grid + update_list_grid for every boid in index order
 * (src/boid_simulation_grid.cpp:255, :291, :445-450): each cell's list is in
 * push_back order, i.e. ascending boid index. */
void orc_grid_bin(orc_grid *g, const float *pos)
{
    const uint32_t N = g->p.n;
    size_t ncell = (size_t)g->G * g->G * g->G;
    memset(g->start, 0, sizeof(int32_t) * (ncell + 1));
    for (uint32_t i = 0; i < N; i++) {
        ref_cells1(g->R, g->GS, g->G, ld3(pos, i), g->gi + 8 * i);
        for (int k = 0; k < 8; k++) {
            int32_t c = g->gi[8 * i + k];
            if (c >= 0) g->start[c + 1]++;
        }
    }
    for (size_t c = 0; c < ncell; c++) g->start[c + 1] += g->start[c];
    int32_t *fill = (int32_t *)malloc(sizeof(int32_t) * (ncell ? ncell : 1));
    memcpy(fill, g->start, sizeof(int32_t) * ncell);
    for (uint32_t i = 0; i < N; i++) {
        for (int k = 0; k < 8; k++) {
            int32_t c = g->gi[8 * i + k];
            if (c >= 0) g->items[fill[c]++] = (int32_t)i;
        }
    }
    free(fill);
}

void orc_grid_step(orc_grid *g, float *pos, float *vel, float *force9, int nthreads)
{
    const orc_params *p = &g->p;
    const uint32_t N = p->n;
    set_threads(nthreads);
    /* rule loop over the primary cell's list, src/boid_simulation_grid.cpp:174-253 */
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)N; i++) {
        acc_t a;
        acc_zero(&a);
        v3 pi = ld3(pos, (uint32_t)i), vi = ld3(vel, (uint32_t)i);
        int32_t c = g->gi[8 * i];
        for (int32_t s = g->start[c]; s < g->start[c + 1]; s++) {
            uint32_t j = (uint32_t)g->items[s];
            if (j == (uint32_t)i) continue;                       /* id test, :217 */
            acc_pair(p, &a, pi, vi, ld3(pos, j), ld3(vel, j));
        }
        acc_finish(p, &a, pi, vi, g->dv + 3 * i, force9 ? force9 + 9 * i : NULL);
    }
    /* integration and rebinning, serial as in the reference (:255-292) */
    for (uint32_t i = 0; i < N; i++) integrate1(p, pos + 3 * i, vel + 3 * i, g->dv + 3 * i);
    orc_grid_bin(g, pos);
}

/* ------------------------------------------------------------------ neighbour sets */

uint64_t orc_id_hash(uint32_t id)
{
    uint64_t z = (uint64_t)id + 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

/* A private bucket grid for enumerating candidate pairs quickly.  Buckets
 * are at least 1% wider than the largest radius, so every pair the
 * reference's distance test can accept lies in adjacent buckets whatever the
 * rounding; the exact test is then applied to every candidate. */
typedef struct {
    int G;                 /* 0: no bucketing, scan all pairs */
    double inv;
    int32_t *start, *items;
} bucket_t;

static int bucket_of(const bucket_t *b, float x)
{
    int c = (int)((double)x * b->inv);
    if (c < 0) c = 0;
    if (c >= b->G) c = b->G - 1;
    return c;
}

static void bucket_build(bucket_t *b, const orc_params *p, const float *pos)
{
    double m = p->coh_r;
    if (p->ali_r > m) m = p->ali_r;
    if (p->sep_r > m) m = p->sep_r;
    int G = (int)floor(p->field / (m * 1.01));
    b->G = 0; b->start = b->items = NULL;
    if (G < 3) return;
    for (uint32_t i = 0; i < p->n; i++) {                 /* positions must lie in [0, F] */
        for (int d = 0; d < 3; d++) {
            float x = pos[3 * i + d];
            if (!((double)x >= 0.0 && (double)x <= p->field * (1.0 + 1e-6))) return;
        }
    }
    b->G = G;
    b->inv = G / p->field;
    size_t nc = (size_t)G * G * G;
    b->start = (int32_t *)calloc(nc + 1, sizeof(int32_t));
    b->items = (int32_t *)malloc(sizeof(int32_t) * (p->n ? p->n : 1));
    int32_t *key = (int32_t *)malloc(sizeof(int32_t) * (p->n ? p->n : 1));
    for (uint32_t i = 0; i < p->n; i++) {
        int cx = bucket_of(b, pos[3 * i]), cy = bucket_of(b, pos[3 * i + 1]), cz = bucket_of(b, pos[3 * i + 2]);
        key[i] = cx + G * (cy + G * cz);
        b->start[key[i] + 1]++;
    }
    for (size_t c = 0; c < nc; c++) b->start[c + 1] += b->start[c];
    int32_t *fill = (int32_t *)malloc(sizeof(int32_t) * nc);
    memcpy(fill, b->start, sizeof(int32_t) * nc);
    for (uint32_t i = 0; i < p->n; i++) b->items[fill[key[i]]++] = (int32_t)i;
    free(fill);
    free(key);
}

static void bucket_free(bucket_t *b) { free(b->start); free(b->items); }

/* Calls fn(ctx, i, j) for every candidate j != i (all pairs, or the 27
 * buckets around i); order is unspecified. */
typedef void (*pair_fn)(void *ctx, uint32_t i, uint32_t j);

static void for_candidates(const bucket_t *b, const orc_params *p, const float *pos, uint32_t i,
                           pair_fn fn, void *ctx)
{
    if (b->G == 0) {
        for (uint32_t j = 0; j < p->n; j++) if (j != i) fn(ctx, i, j);
        return;
    }
    const int G = b->G;
    int cx = bucket_of(b, pos[3 * i]), cy = bucket_of(b, pos[3 * i + 1]), cz = bucket_of(b, pos[3 * i + 2]);
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                int c = ((cx + dx + G) % G) + G * (((cy + dy + G) % G) + G * ((cz + dz + G) % G));
                for (int32_t s = b->start[c]; s < b->start[c + 1]; s++) {
                    uint32_t j = (uint32_t)b->items[s];
                    if (j != i) fn(ctx, i, j);
                }
            }
}

typedef struct {
    const orc_params *p;
    const float *pos, *vel;
    int32_t cnt[3];
    uint64_t h[3];
} nbr_ctx;

static void nbr_visit(void *vctx, uint32_t i, uint32_t j)
{
    nbr_ctx *c = (nbr_ctx *)vctx;
    v3 pi = ld3(c->pos, i), vi = ld3(c->vel, i);
    v3 t = image_of(ld3(c->pos, j), pi, c->p->field);
    int f = pair_flags(c->p, pi, vi, t);
    uint64_t h = f ? orc_id_hash(j) : 0;
    for (int r = 0; r < 3; r++) {
        if (f & (1 << r)) { c->cnt[r]++; c->h[r] += h; }
    }
}

void orc_neighbor_sets_ex(const orc_params *p, const float *pos, const float *vel,
                          int32_t *count3, uint64_t *hash3, int nthreads, int bucketed)
{
    bucket_t b;
    if (bucketed) {
        bucket_build(&b, p, pos);
    } else {
        b.G = 0;
        b.start = b.items = NULL;
    }
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)p->n; i++) {
        nbr_ctx c;
        memset(&c, 0, sizeof(c));
        c.p = p; c.pos = pos; c.vel = vel;
        for_candidates(&b, p, pos, (uint32_t)i, nbr_visit, &c);
        for (int r = 0; r < 3; r++) { count3[3 * i + r] = c.cnt[r]; hash3[3 * i + r] = c.h[r]; }
    }
    bucket_free(&b);
}

void orc_neighbor_sets(const orc_params *p, const float *pos, const float *vel,
                       int32_t *count3, uint64_t *hash3, int nthreads)
{
    orc_neighbor_sets_ex(p, pos, vel, count3, hash3, nthreads, 1);
}

/* ------------------------------------------------------------------ FP64 forces */

typedef struct {
    const orc_params *p;
    const float *pos, *vel;
    double coh[3], sep[3], ali[3];
    int ncoh, nsep, nali;
} f64_ctx;

static void f64_visit(void *vctx, uint32_t i, uint32_t j)
{
    f64_ctx *c = (f64_ctx *)vctx;
    const double F = c->p->field;
    v3 pi = ld3(c->pos, i), vi = ld3(c->vel, i);
    v3 pj = ld3(c->pos, j);
    int f = pair_flags(c->p, pi, vi, image_of(pj, pi, F));
    if (!f) return;
    /* the same image in exact double arithmetic */
    double xi[3] = { pi.x, pi.y, pi.z }, xj[3] = { pj.x, pj.y, pj.z };
    for (int d = 0; d < 3; d++) {
        if ((double)((float)xj[d] - (float)xi[d]) > F / 2) xj[d] -= F;
        else if ((double)((float)xi[d] - (float)xj[d]) > F / 2) xj[d] += F;
    }
    if (f & 1) {
        c->ncoh++;
        for (int d = 0; d < 3; d++) c->coh[d] += xj[d];
    }
    if (f & 2) {
        c->nsep++;
        double dd[3] = { xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2] };
        double n = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
        for (int d = 0; d < 3; d++) c->sep[d] += dd[d] / n;
    }
    if (f & 4) {
        c->nali++;
        c->ali[0] += c->vel[3 * j]; c->ali[1] += c->vel[3 * j + 1]; c->ali[2] += c->vel[3 * j + 2];
    }
}

void orc_forces_f64(const orc_params *p, const float *pos, const float *vel, double *force9, int nthreads)
{
    bucket_t b;
    bucket_build(&b, p, pos);
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)p->n; i++) {
        f64_ctx c;
        memset(&c, 0, sizeof(c));
        c.p = p; c.pos = pos; c.vel = vel;
        for_candidates(&b, p, pos, (uint32_t)i, f64_visit, &c);
        double *o = force9 + 9 * i;
        for (int d = 0; d < 3; d++) {
            double coh = c.ncoh ? c.coh[d] / c.ncoh - (double)pos[3 * i + d] : 0.0;
            double ali = c.nali ? c.ali[d] / c.nali - (double)vel[3 * i + d] : 0.0;
            o[d] = p->coh_c * coh;
            o[3 + d] = p->sep_c * c.sep[d];
            o[6 + d] = p->ali_c * ali;
        }
    }
    bucket_free(&b);
}
