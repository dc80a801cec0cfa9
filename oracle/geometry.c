/*
 * Oracle (test infrastructure only): exact CPU restatement of the reference's
 * neighbor search pair geometry. It is used by the tests, by the smoke check and
 * by the CPU baseline leg of the benchmark as the checker; the product never
 * links or calls it.
 *
 * Restates, in the same fp32 operation order as the reference's torch CPU code:
 *   getPeriodicPosition  src/diffSPH/v2/modules/neighborhood.py:406-431
 *       p = remainder(x - min, max - min) + min            (periodic axes only)
 *   mod                  src/diffSPH/v2/math.py:5-6
 *       where(|x| > (max-min)/2, sgn(x) * ((|x| + min) % (max-min) + min), x)
 *   computeNeighborhood  src/diffSPH/v2/modules/neighborhood.py:433-460
 *       x_ij = mod(p_i - p_j); r = ||x_ij||; xhat = x_ij / (r + 1e-7);
 *       q = r / h_j (scatter mode); keep q <= 1
 *
 * torch's CPU vector 2-norm of a 2-vector evaluates sqrt(fma(y, y, x*x)) in
 * fp32 (checked bit for bit against torch.linalg.norm on 6M random pairs),
 * hence the explicit fmaf below. Build with -ffp-contract=off so that the
 * compiler adds no other contraction.
 *
 * Torch's float remainder is fmod followed by a sign fix-up
 * (mod != 0 && (b < 0) != (mod < 0) -> mod += b), which is what rem_f32 does.
 *
 * Parity of this file is pinned by tests/test_oracle_golden.py against vectors
 * produced by running the reference itself (tests/golden/make_golden.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double min[2];
    double max[2];
    int periodic[2];
} domain_t;

static inline float rem_f32(float a, float b) {
    float m = fmodf(a, b);
    if (m != 0.0f && ((b < 0.0f) != (m < 0.0f))) m += b;
    return m;
}

static inline double rem_f64(double a, double b) {
    double m = fmod(a, b);
    if (m != 0.0 && ((b < 0.0) != (m < 0.0))) m += b;
    return m;
}

static inline float sgn_f32(float x) { return (float)((x > 0.0f) - (x < 0.0f)); }
static inline double sgn_f64(double x) { return (double)((x > 0.0) - (x < 0.0)); }

/* periodic position (neighborhood.py:431), fp32 */
static inline float wrap_f32(float x, float mn, float ext) { return rem_f32(x - mn, ext) + mn; }
static inline double wrap_f64(double x, double mn, double ext) { return rem_f64(x - mn, ext) + mn; }

/* math.py:5-6 with the python-float arguments min, max cast to the tensor dtype */
static inline float mod_f32(float x, float mn, float ext, float half) {
    float a = fabsf(x);
    if (a > half) return sgn_f32(x) * (rem_f32(a + mn, ext) + mn);
    return x;
}
static inline double mod_f64(double x, double mn, double ext, double half) {
    double a = fabs(x);
    if (a > half) return sgn_f64(x) * (rem_f64(a + mn, ext) + mn);
    return x;
}

/* Periodic wrap of a position array in place of the reference's getPeriodicPosition. */
void oracle_wrap_positions_f32(const float* x, float* out, int64_t n, const domain_t* d) {
    for (int64_t i = 0; i < n; ++i) {
        for (int a = 0; a < 2; ++a) {
            float v = x[2 * i + a];
            if (d->periodic[a]) {
                float mn = (float)d->min[a];
                float ext = (float)(d->max[a] - d->min[a]);
                v = wrap_f32(v, mn, ext);
            }
            out[2 * i + a] = v;
        }
    }
}

void oracle_wrap_positions_f64(const double* x, double* out, int64_t n, const domain_t* d) {
    for (int64_t i = 0; i < n; ++i) {
        for (int a = 0; a < 2; ++a) {
            double v = x[2 * i + a];
            if (d->periodic[a]) v = wrap_f64(v, d->min[a], d->max[a] - d->min[a]);
            out[2 * i + a] = v;
        }
    }
}

/* cell grid over the (wrapped) reference positions */
typedef struct {
    int ncx, ncy;
    double cell;
    int64_t* start;  /* ncx*ncy+1 */
    int64_t* order;  /* nr */
} grid_t;

static int cell_coord(double v, double mn, double cell, int nc) {
    double c = floor((v - mn) / cell);
    if (c < 0) c = 0;
    if (c > nc - 1) c = nc - 1;
    return (int)c;
}

static void grid_build(grid_t* g, const double* pr, int64_t nr, const domain_t* d, double cell) {
    g->cell = cell;
    g->ncx = (int)floor((d->max[0] - d->min[0]) / cell);
    g->ncy = (int)floor((d->max[1] - d->min[1]) / cell);
    if (g->ncx < 1) g->ncx = 1;
    if (g->ncy < 1) g->ncy = 1;
    int64_t nc = (int64_t)g->ncx * g->ncy;
    g->start = (int64_t*)calloc((size_t)nc + 1, sizeof(int64_t));
    g->order = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nr > 0 ? nr : 1));
    int64_t* key = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nr > 0 ? nr : 1));
    for (int64_t j = 0; j < nr; ++j) {
        int cx = cell_coord(pr[2 * j], d->min[0], cell, g->ncx);
        int cy = cell_coord(pr[2 * j + 1], d->min[1], cell, g->ncy);
        key[j] = (int64_t)cy * g->ncx + cx;
        g->start[key[j] + 1]++;
    }
    for (int64_t c = 0; c < nc; ++c) g->start[c + 1] += g->start[c];
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)nc);
    memcpy(cur, g->start, sizeof(int64_t) * (size_t)nc);
    for (int64_t j = 0; j < nr; ++j) g->order[cur[key[j]]++] = j; /* stable: ascending j per cell */
    free(cur);
    free(key);
}

static void grid_free(grid_t* g) {
    free(g->start);
    free(g->order);
}

static int cmp_i64(const void* a, const void* b) {
    int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return (x > y) - (x < y);
}

/*
 * Exact neighbor list, scatter mode (h_ij = h_j), rows ordered by i, columns by j.
 * Returns the number of pairs; if it exceeds cap, nothing beyond cap is written
 * and the caller retries with a larger buffer.
 * Outputs per pair: i, j, q = r/h_j, xhat (2), h_j.
 */
int64_t oracle_neighbors_f32(const float* xq, const float* hq, int64_t nq,
                             const float* xr, const float* hr, int64_t nr,
                             const domain_t* d, int64_t cap,
                             int64_t* oi, int64_t* oj, float* oq, float* ox, float* oh) {
    (void)hq;
    float* pq = (float*)malloc(sizeof(float) * 2 * (size_t)(nq > 0 ? nq : 1));
    float* pr = (float*)malloc(sizeof(float) * 2 * (size_t)(nr > 0 ? nr : 1));
    oracle_wrap_positions_f32(xq, pq, nq, d);
    oracle_wrap_positions_f32(xr, pr, nr, d);
    double hmax = 0.0;
    for (int64_t j = 0; j < nr; ++j) hmax = hr[j] > hmax ? hr[j] : hmax;
    double* prd = (double*)malloc(sizeof(double) * 2 * (size_t)(nr > 0 ? nr : 1));
    for (int64_t j = 0; j < 2 * nr; ++j) prd[j] = pr[j];
    grid_t g;
    grid_build(&g, prd, nr, d, hmax * 1.0001 + 1e-12);
    float mn[2], ext[2], half[2];
    for (int a = 0; a < 2; ++a) {
        mn[a] = (float)d->min[a];
        ext[a] = (float)(d->max[a] - d->min[a]);
        half[a] = (float)((d->max[a] - d->min[a]) / 2.0);
    }
    int64_t* rowbuf = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nr > 0 ? nr : 1));
    int64_t count = 0;
    for (int64_t i = 0; i < nq; ++i) {
        int cx = cell_coord(pq[2 * i], d->min[0], g.cell, g.ncx);
        int cy = cell_coord(pq[2 * i + 1], d->min[1], g.cell, g.ncy);
        int64_t nrow = 0;
        for (int dy = -1; dy <= 1; ++dy) {
            int yy = cy + dy;
            if (d->periodic[1]) yy = (yy % g.ncy + g.ncy) % g.ncy;
            else if (yy < 0 || yy >= g.ncy) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                int xx = cx + dx;
                if (d->periodic[0]) xx = (xx % g.ncx + g.ncx) % g.ncx;
                else if (xx < 0 || xx >= g.ncx) continue;
                int64_t c = (int64_t)yy * g.ncx + xx;
                for (int64_t s = g.start[c]; s < g.start[c + 1]; ++s) rowbuf[nrow++] = g.order[s];
            }
        }
        /* a small periodic grid can visit one cell twice: dedupe after sorting */
        qsort(rowbuf, (size_t)nrow, sizeof(int64_t), cmp_i64);
        int64_t prev = -1;
        for (int64_t t = 0; t < nrow; ++t) {
            int64_t j = rowbuf[t];
            if (j == prev) continue;
            prev = j;
            float x0 = pq[2 * i] - pr[2 * j];
            float x1 = pq[2 * i + 1] - pr[2 * j + 1];
            if (d->periodic[0]) x0 = mod_f32(x0, mn[0], ext[0], half[0]);
            if (d->periodic[1]) x1 = mod_f32(x1, mn[1], ext[1], half[1]);
            float r = sqrtf(fmaf(x1, x1, x0 * x0));
            float den = r + 1e-7f;
            float h = hr[j];
            float q = r / h;
            if (q <= 1.0f) {
                if (count < cap) {
                    oi[count] = i;
                    oj[count] = j;
                    oq[count] = q;
                    ox[2 * count] = x0 / den;
                    ox[2 * count + 1] = x1 / den;
                    oh[count] = h;
                }
                ++count;
            }
        }
    }
    free(rowbuf);
    grid_free(&g);
    free(prd);
    free(pq);
    free(pr);
    return count;
}

/* Same in float64 (used for the FP64 reference runs of the same scheme). */
int64_t oracle_neighbors_f64(const double* xq, const double* hq, int64_t nq,
                             const double* xr, const double* hr, int64_t nr,
                             const domain_t* d, int64_t cap,
                             int64_t* oi, int64_t* oj, double* oq, double* ox, double* oh) {
    (void)hq;
    double* pq = (double*)malloc(sizeof(double) * 2 * (size_t)(nq > 0 ? nq : 1));
    double* pr = (double*)malloc(sizeof(double) * 2 * (size_t)(nr > 0 ? nr : 1));
    oracle_wrap_positions_f64(xq, pq, nq, d);
    oracle_wrap_positions_f64(xr, pr, nr, d);
    double hmax = 0.0;
    for (int64_t j = 0; j < nr; ++j) hmax = hr[j] > hmax ? hr[j] : hmax;
    grid_t g;
    grid_build(&g, pr, nr, d, hmax * 1.0001 + 1e-12);
    double mn[2], ext[2], half[2];
    for (int a = 0; a < 2; ++a) {
        mn[a] = d->min[a];
        ext[a] = d->max[a] - d->min[a];
        half[a] = (d->max[a] - d->min[a]) / 2.0;
    }
    int64_t* rowbuf = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nr > 0 ? nr : 1));
    int64_t count = 0;
    for (int64_t i = 0; i < nq; ++i) {
        int cx = cell_coord(pq[2 * i], d->min[0], g.cell, g.ncx);
        int cy = cell_coord(pq[2 * i + 1], d->min[1], g.cell, g.ncy);
        int64_t nrow = 0;
        for (int dy = -1; dy <= 1; ++dy) {
            int yy = cy + dy;
            if (d->periodic[1]) yy = (yy % g.ncy + g.ncy) % g.ncy;
            else if (yy < 0 || yy >= g.ncy) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                int xx = cx + dx;
                if (d->periodic[0]) xx = (xx % g.ncx + g.ncx) % g.ncx;
                else if (xx < 0 || xx >= g.ncx) continue;
                int64_t c = (int64_t)yy * g.ncx + xx;
                for (int64_t s = g.start[c]; s < g.start[c + 1]; ++s) rowbuf[nrow++] = g.order[s];
            }
        }
        qsort(rowbuf, (size_t)nrow, sizeof(int64_t), cmp_i64);
        int64_t prev = -1;
        for (int64_t t = 0; t < nrow; ++t) {
            int64_t j = rowbuf[t];
            if (j == prev) continue;
            prev = j;
            double x0 = pq[2 * i] - pr[2 * j];
            double x1 = pq[2 * i + 1] - pr[2 * j + 1];
            if (d->periodic[0]) x0 = mod_f64(x0, mn[0], ext[0], half[0]);
            if (d->periodic[1]) x1 = mod_f64(x1, mn[1], ext[1], half[1]);
            double r = sqrt(fma(x1, x1, x0 * x0));
            double den = r + 1e-7;
            double h = hr[j];
            double q = r / h;
            if (q <= 1.0) {
                if (count < cap) {
                    oi[count] = i;
                    oj[count] = j;
                    oq[count] = q;
                    ox[2 * count] = x0 / den;
                    ox[2 * count + 1] = x1 / den;
                    oh[count] = h;
                }
                ++count;
            }
        }
    }
    free(rowbuf);
    grid_free(&g);
    free(pq);
    free(pr);
    return count;
}
