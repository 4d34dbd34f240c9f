/*
 * freud_oracle.c -- CPU restatement of freud's neighbour-query -> pair-reduction
 * path, used as the parity oracle and as the timed CPU ("port") baseline.
 *
 * TEST INFRASTRUCTURE ONLY. The product (freud_gb300/) never links or calls this
 * file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do.
 *
 * Every float32 operation that decides a neighbour set, a distance or an RDF bin
 * is written in the same order as the reference and must be compiled with
 * -ffp-contract=off (no FMA), so results are bit-identical to freud's x86 build.
 * Steinhardt quantities are computed in FP64 from the float32 pair vectors.
 *
 * Reference (glotzerlab/freud 3.5.0) lines restated here:
 *   box maths ............ freud/box/Box.h:212-222 (makeAbsolute), :243-255
 *                          (makeFractional), :307-329 (wrap), :489-497
 *                          (getNearestPlaneDistance), :503-518 (getLatticeVector);
 *                          freud/util/utils.h:29-32 (modulusPositive)
 *   periodic images ...... freud/locality/NeighborQuery.h:496-564 (updateImageVectors)
 *   AABB ball pair test .. freud/locality/AABBQuery.cc:77-150 (r_ij = p_j - (q + image))
 *   LinkCell pair test ... freud/locality/LinkCell.cc:496-573 (r_ij = wrap(p_j - q))
 *   kNN selection ........ freud/locality/AABBQuery.cc:152-281, LinkCell.cc:575-679
 *   bond order ........... freud/locality/NeighborBond.h:80-117 (less_as_tuple /
 *                          less_as_distance), NeighborQuery.h:434-481
 *   histogram bin ........ freud/util/Histogram.h:123-174 (RegularAxis)
 *   RDF normalisation .... freud/density/RDF.cc:25-64, :73-99
 *   Steinhardt ........... freud/order/Steinhardt.cc:120-359, Wigner3j.cc:17-57
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OFG_ARITH_AABB 0 /* r = p_j - (q + image)  (AABBQuery / RawPoints) */
#define OFG_ARITH_WRAP 1 /* r = wrap(p_j - q)      (LinkCell) */
#define OFG_ARITH_GHOST 2 /* r = g_j - q, g_j the point or a ghost copy (CellQuery) */

typedef struct
{
    float L[3];
    float xy, xz, yz;
    int is2d;
    float lo[3];
} obox;

static void box_init(obox* b, const float* box7)
{
    b->L[0] = box7[0];
    b->L[1] = box7[1];
    b->L[2] = box7[6] != 0.0f ? 0.0f : box7[2];
    b->xy = box7[3];
    b->xz = box7[4];
    b->yz = box7[5];
    b->is2d = box7[6] != 0.0f;
    for (int d = 0; d < 3; ++d)
    {
        b->lo[d] = -(b->L[d] / 2.0f); /* m_hi = m_L / 2; m_lo = -m_hi (Box.h:101-116) */
    }
}

/* Box.h:243-255 */
static void make_fractional(const obox* b, const float* v, float* f)
{
    float dx = v[0] - b->lo[0];
    float dy = v[1] - b->lo[1];
    float dz = v[2] - b->lo[2];
    const float t1 = b->yz * b->xy;
    const float t2 = b->xz - t1;
    const float t3 = t2 * v[2];
    const float t4 = b->xy * v[1];
    dx = dx - (t3 + t4);
    dy = dy - b->yz * v[2];
    f[0] = dx / b->L[0];
    f[1] = dy / b->L[1];
    f[2] = b->is2d ? 0.0f : dz / b->L[2];
}

/* Box.h:212-222 */
static void make_absolute(const obox* b, const float* f, float* v)
{
    float x = b->lo[0] + f[0] * b->L[0];
    float y = b->lo[1] + f[1] * b->L[1];
    float z = b->lo[2] + f[2] * b->L[2];
    x = x + (b->xy * y + b->xz * z);
    y = y + b->yz * z;
    v[0] = x;
    v[1] = y;
    v[2] = b->is2d ? 0.0f : z;
}

/* utils.h:29-32 with b = 1 */
static float mod_pos1(float a)
{
    return fmodf(fmodf(a, 1.0f) + 1.0f, 1.0f);
}

/* Box.h:307-329 (all periodic) */
static void box_wrap(const obox* b, const float* v, float* out)
{
    float f[3];
    make_fractional(b, v, f);
    f[0] = mod_pos1(f[0]);
    f[1] = mod_pos1(f[1]);
    f[2] = mod_pos1(f[2]);
    make_absolute(b, f, out);
}

/* Box.h:489-497 */
static void nearest_plane(const obox* b, float* d)
{
    const float t = b->xy * b->yz - b->xz;
    d[0] = b->L[0] / sqrtf(1.0f + b->xy * b->xy + t * t);
    d[1] = b->L[1] / sqrtf(1.0f + b->yz * b->yz);
    d[2] = b->L[2];
}

/* NeighborQuery.h:496-564 (all periodic). Returns the number of images. */
static int image_vectors(const obox* b, float img[27][3])
{
    const float a1[3] = {b->L[0], 0.0f, 0.0f};
    const float a2[3] = {b->L[1] * b->xy, b->L[1], 0.0f};
    float a3[3] = {0.0f, 0.0f, 0.0f};
    if (!b->is2d)
    {
        a3[0] = b->L[2] * b->xz;
        a3[1] = b->L[2] * b->yz;
        a3[2] = b->L[2];
    }
    const int n_images = b->is2d ? 9 : 27;
    img[0][0] = img[0][1] = img[0][2] = 0.0f;
    int n = 1;
    for (int i = -1; i <= 1 && n < n_images; ++i)
    {
        for (int j = -1; j <= 1 && n < n_images; ++j)
        {
            for (int k = -1; k <= 1 && n < n_images; ++k)
            {
                if (i == 0 && j == 0 && k == 0)
                {
                    continue;
                }
                if (k != 0 && b->is2d)
                {
                    continue;
                }
                for (int d = 0; d < 3; ++d)
                {
                    img[n][d] = ((float) i * a1[d] + (float) j * a2[d]) + (float) k * a3[d];
                }
                ++n;
            }
        }
    }
    return n;
}

/* vec3 dot, VectorMath.h:270-273: (x*x + y*y) + z*z */
static float dot3(const float* r)
{
    return (r[0] * r[0] + r[1] * r[1]) + r[2] * r[2];
}

/* ------------------------------------------------------------------------- */
/* Cell grid used only to enumerate candidates (the reference's tree / linked */
/* list is an accelerator; the accepted set is defined by the pair test).     */
/* ------------------------------------------------------------------------- */
typedef struct
{
    int dim[3];
    uint32_t* start; /* ncell + 1 */
    uint32_t* idx;   /* point indices sorted by cell */
    int ncell;
} ogrid;

static int cell_coord(const obox* b, const ogrid* g, const float* p, int* c)
{
    float f[3];
    make_fractional(b, p, f);
    for (int d = 0; d < 3; ++d)
    {
        double w = (double) f[d] - floor((double) f[d]);
        int cc = (int) floor(w * g->dim[d]);
        if (cc < 0)
        {
            cc = 0;
        }
        if (cc >= g->dim[d])
        {
            cc = g->dim[d] - 1;
        }
        c[d] = cc;
    }
    return c[0] + g->dim[0] * (c[1] + g->dim[1] * c[2]);
}

static void grid_build(const obox* b, ogrid* g, const float* pts, uint32_t n, float width)
{
    float pd[3];
    nearest_plane(b, pd);
    for (int d = 0; d < 3; ++d)
    {
        int dm = (int) floor((double) pd[d] / ((double) width * 1.0001));
        if (dm < 1)
        {
            dm = 1;
        }
        if (dm > 512)
        {
            dm = 512;
        }
        g->dim[d] = dm;
    }
    if (b->is2d)
    {
        g->dim[2] = 1;
    }
    /* keep the grid at most ~8 cells per point (wider cells stay correct) */
    while ((double) g->dim[0] * g->dim[1] * g->dim[2] > 8.0 * n + 64.0)
    {
        for (int d = 0; d < (b->is2d ? 2 : 3); ++d)
        {
            g->dim[d] = g->dim[d] > 1 ? (g->dim[d] * 3) / 4 : 1;
        }
    }
    g->ncell = g->dim[0] * g->dim[1] * g->dim[2];
    g->start = (uint32_t*) calloc((size_t) g->ncell + 1, sizeof(uint32_t));
    g->idx = (uint32_t*) malloc((size_t) (n ? n : 1) * sizeof(uint32_t));
    uint32_t* cell_of = (uint32_t*) malloc((size_t) (n ? n : 1) * sizeof(uint32_t));
    int c[3];
    for (uint32_t i = 0; i < n; ++i)
    {
        cell_of[i] = (uint32_t) cell_coord(b, g, pts + 3 * (size_t) i, c);
        g->start[cell_of[i] + 1]++;
    }
    for (int k = 0; k < g->ncell; ++k)
    {
        g->start[k + 1] += g->start[k];
    }
    uint32_t* cursor = (uint32_t*) malloc(((size_t) g->ncell + 1) * sizeof(uint32_t));
    memcpy(cursor, g->start, ((size_t) g->ncell + 1) * sizeof(uint32_t));
    for (uint32_t i = 0; i < n; ++i)
    {
        g->idx[cursor[cell_of[i]]++] = i;
    }
    free(cursor);
    free(cell_of);
}

static void grid_free(ogrid* g)
{
    free(g->start);
    free(g->idx);
}

/* Distinct wrapped cell indices along one axis within +-s of c. */
static int axis_cells(int c, int s, int dim, int* out)
{
    int n = 0;
    if (2 * s + 1 >= dim)
    {
        for (int k = 0; k < dim; ++k)
        {
            out[n++] = k;
        }
        return n;
    }
    for (int d = -s; d <= s; ++d)
    {
        out[n++] = ((c + d) % dim + dim) % dim;
    }
    return n;
}

/* ------------------------------------------------------------------------- */
/* Bond lists                                                                */
/* ------------------------------------------------------------------------- */
typedef struct
{
    uint32_t i, j;
    float d;
    float v[3];
} obond;

typedef struct
{
    obond* b;
    size_t n, cap;
} obonds;

static void bonds_push(obonds* l, uint32_t i, uint32_t j, float d, const float* v)
{
    if (l->n == l->cap)
    {
        l->cap = l->cap ? 2 * l->cap : 256;
        l->b = (obond*) realloc(l->b, l->cap * sizeof(obond));
    }
    obond* x = &l->b[l->n++];
    x->i = i;
    x->j = j;
    x->d = d;
    x->v[0] = v[0];
    x->v[1] = v[1];
    x->v[2] = v[2];
}

/* NeighborBond.h:80-95 less_as_tuple (weights are all 1) */
static int cmp_tuple(const void* pa, const void* pb)
{
    const obond* a = (const obond*) pa;
    const obond* b = (const obond*) pb;
    if (a->i != b->i)
        return a->i < b->i ? -1 : 1;
    if (a->j != b->j)
        return a->j < b->j ? -1 : 1;
    if (a->d != b->d)
        return a->d < b->d ? -1 : 1;
    return 0;
}

/* NeighborBond.h:97-117 less_as_distance */
static int cmp_dist(const void* pa, const void* pb)
{
    const obond* a = (const obond*) pa;
    const obond* b = (const obond*) pb;
    if (a->i != b->i)
        return a->i < b->i ? -1 : 1;
    if (a->d != b->d)
        return a->d < b->d ? -1 : 1;
    if (a->j != b->j)
        return a->j < b->j ? -1 : 1;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Query driver (threads over query points)                                  */
/* ------------------------------------------------------------------------- */
typedef struct
{
    const obox* box;
    const ogrid* grid;
    const float* pts;
    const float* qpts;
    uint32_t nq;
    float r_max, r_min;
    int exclude_ii;
    int arith;
    uint32_t k; /* 0 => ball query */
    float img[27][3];
    int n_img;
    /* output */
    obonds* per_thread;
    int nthreads;
    /* fused RDF (bins > 0) */
    uint32_t bins;
    float h_min, h_max, h_inv;
    uint64_t** hist;
} qctx;

typedef struct
{
    qctx* ctx;
    int tid;
} qarg;

/* Histogram.h:152-174 RegularAxis::bin; returns -1 for out of range */
static int64_t hist_bin(float value, float mn, float mx, float inv, uint32_t nbins)
{
    if (value < mn || value >= mx)
    {
        return -1;
    }
    const float val = (value - mn) * inv;
    int64_t b = (int64_t) val;
    if (b == (int64_t) nbins)
    {
        return (int64_t) nbins - 1;
    }
    return b;
}

/* Pair test for one (query, point). Returns 1 and fills r/r_sq when accepted by the
 * reference ball test r_sq < r_max^2 && r_sq >= r_min^2 (AABBQuery.cc:125-131,
 * LinkCell.cc:520-529). In AABB arithmetic each image is tried in reference order;
 * at most one image can pass because 2*r_max < nearest plane distance. */
static int pair_test(const qctx* c, const float* q, uint32_t j, float rmax_sq, float rmin_sq, float* r,
                     float* rsq)
{
    const float* p = c->pts + 3 * (size_t) j;
    if (c->arith == OFG_ARITH_WRAP)
    {
        float dv[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
        box_wrap(c->box, dv, r);
        *rsq = dot3(r);
        return *rsq < rmax_sq && *rsq >= rmin_sq;
    }
    float pj[3] = {p[0], p[1], c->box->is2d ? 0.0f : p[2]};
    float qi[3] = {q[0], q[1], c->box->is2d ? 0.0f : q[2]};
    for (int m = 0; m < c->n_img; ++m)
    {
        float qimg[3] = {qi[0] + c->img[m][0], qi[1] + c->img[m][1], qi[2] + c->img[m][2]};
        float rr[3] = {pj[0] - qimg[0], pj[1] - qimg[1], pj[2] - qimg[2]};
        float s = dot3(rr);
        if (s < rmax_sq && s >= rmin_sq)
        {
            r[0] = rr[0];
            r[1] = rr[1];
            r[2] = rr[2];
            *rsq = s;
            return 1;
        }
    }
    return 0;
}

/* kNN distance for one candidate: the image with the smallest r_sq (AABB
 * arithmetic, AABBQuery.cc:196-213) or the wrapped vector (LinkCell.cc:620-627).
 * Returns r_sq; the distance is sqrtf(r_sq). */
static float knn_rsq(const qctx* c, const float* q, uint32_t j, float* r)
{
    const float* p = c->pts + 3 * (size_t) j;
    if (c->arith == OFG_ARITH_WRAP)
    {
        float dv[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
        box_wrap(c->box, dv, r);
        return dot3(r);
    }
    float pj[3] = {p[0], p[1], c->box->is2d ? 0.0f : p[2]};
    float qi[3] = {q[0], q[1], c->box->is2d ? 0.0f : q[2]};
    float best = INFINITY;
    for (int m = 0; m < c->n_img; ++m)
    {
        float qimg[3] = {qi[0] + c->img[m][0], qi[1] + c->img[m][1], qi[2] + c->img[m][2]};
        float rr[3] = {pj[0] - qimg[0], pj[1] - qimg[1], pj[2] - qimg[2]};
        float s = dot3(rr);
        if (s < best)
        {
            best = s;
            r[0] = rr[0];
            r[1] = rr[1];
            r[2] = rr[2];
        }
    }
    return best;
}

static int cmp_knn(const void* pa, const void* pb)
{
    const obond* a = (const obond*) pa;
    const obond* b = (const obond*) pb;
    if (a->d != b->d)
        return a->d < b->d ? -1 : 1;
    if (a->j != b->j)
        return a->j < b->j ? -1 : 1;
    return 0;
}

static void* query_worker(void* varg)
{
    qarg* a = (qarg*) varg;
    qctx* c = a->ctx;
    obonds* out = &c->per_thread[a->tid];
    const ogrid* g = c->grid;
    const float rmax_sq = c->r_max * c->r_max;
    const float rmin_sq = c->r_min * c->r_min;
    int xs[1024], ys[1024], zs[1024];
    obonds cand = {0, 0, 0};
    const uint32_t chunk = (c->nq + (uint32_t) c->nthreads - 1) / (uint32_t) c->nthreads;
    const uint32_t i0 = (uint32_t) a->tid * chunk;
    const uint32_t i1 = i0 + chunk < c->nq ? i0 + chunk : c->nq;
    for (uint32_t i = i0; i < i1; ++i)
    {
        const float* q = c->qpts + 3 * (size_t) i;
        int cc[3];
        cell_coord(c->box, g, q, cc);
        if (c->k == 0)
        {
            const int nx = axis_cells(cc[0], 1, g->dim[0], xs);
            const int ny = axis_cells(cc[1], 1, g->dim[1], ys);
            const int nz = c->box->is2d ? 1 : axis_cells(cc[2], 1, g->dim[2], zs);
            if (c->box->is2d)
            {
                zs[0] = 0;
            }
            for (int z = 0; z < nz; ++z)
                for (int y = 0; y < ny; ++y)
                    for (int x = 0; x < nx; ++x)
                    {
                        const int cell = xs[x] + g->dim[0] * (ys[y] + g->dim[1] * zs[z]);
                        for (uint32_t t = g->start[cell]; t < g->start[cell + 1]; ++t)
                        {
                            const uint32_t j = g->idx[t];
                            if (c->exclude_ii && j == i)
                            {
                                continue;
                            }
                            float r[3], rsq;
                            if (pair_test(c, q, j, rmax_sq, rmin_sq, r, &rsq))
                            {
                                const float d = sqrtf(rsq);
                                if (c->bins > 0)
                                {
                                    int64_t bb = hist_bin(d, c->h_min, c->h_max, c->h_inv, c->bins);
                                    if (bb >= 0)
                                    {
                                        c->hist[a->tid][bb]++;
                                    }
                                }
                                else
                                {
                                    bonds_push(out, i, j, d, r);
                                }
                            }
                        }
                    }
            continue;
        }
        /* kNN: grow shells until k candidates lie strictly inside the covered radius. */
        float pd[3];
        nearest_plane(c->box, pd);
        double cw = 1e300;
        for (int d = 0; d < (c->box->is2d ? 2 : 3); ++d)
        {
            double w = (double) pd[d] / g->dim[d];
            if (w < cw)
                cw = w;
        }
        for (int s = 1;; ++s)
        {
            cand.n = 0;
            const int nx = axis_cells(cc[0], s, g->dim[0], xs);
            const int ny = axis_cells(cc[1], s, g->dim[1], ys);
            const int nz = c->box->is2d ? 1 : axis_cells(cc[2], s, g->dim[2], zs);
            if (c->box->is2d)
            {
                zs[0] = 0;
            }
            const int all = nx == g->dim[0] && ny == g->dim[1] && nz == (c->box->is2d ? 1 : g->dim[2]);
            for (int z = 0; z < nz; ++z)
                for (int y = 0; y < ny; ++y)
                    for (int x = 0; x < nx; ++x)
                    {
                        const int cell = xs[x] + g->dim[0] * (ys[y] + g->dim[1] * zs[z]);
                        for (uint32_t t = g->start[cell]; t < g->start[cell + 1]; ++t)
                        {
                            const uint32_t j = g->idx[t];
                            if (c->exclude_ii && j == i)
                            {
                                continue;
                            }
                            float r[3];
                            const float rsq = knn_rsq(c, q, j, r);
                            const float d = sqrtf(rsq);
                            /* AABB kNN: ball test r_sq < r_max^2 then distance >= r_min
                             * (AABBQuery.cc:180-205); LinkCell kNN: r_sq window
                             * (LinkCell.cc:624-628). */
                            if (!(rsq < rmax_sq))
                            {
                                continue;
                            }
                            if (c->arith == OFG_ARITH_WRAP ? !(rsq >= rmin_sq) : !(d >= c->r_min))
                            {
                                continue;
                            }
                            bonds_push(&cand, i, j, d, r);
                        }
                    }
            const double covered = (double) s * cw;
            size_t inside = 0;
            for (size_t t = 0; t < cand.n; ++t)
            {
                if ((double) cand.b[t].d < covered)
                {
                    inside++;
                }
            }
            if (all || inside >= c->k)
            {
                qsort(cand.b, cand.n, sizeof(obond), cmp_knn);
                const size_t take = cand.n < c->k ? cand.n : c->k;
                for (size_t t = 0; t < take; ++t)
                {
                    bonds_push(out, i, cand.b[t].j, cand.b[t].d, cand.b[t].v);
                }
                break;
            }
        }
    }
    free(cand.b);
    return NULL;
}

typedef struct
{
    obond* b;
    size_t n;
} ofg_nlist;

static void run_query(qctx* c, int nthreads)
{
    if (nthreads < 1)
    {
        nthreads = 1;
    }
    c->nthreads = nthreads;
    pthread_t* th = (pthread_t*) malloc(sizeof(pthread_t) * (size_t) nthreads);
    qarg* args = (qarg*) malloc(sizeof(qarg) * (size_t) nthreads);
    for (int t = 0; t < nthreads; ++t)
    {
        args[t].ctx = c;
        args[t].tid = t;
        pthread_create(&th[t], NULL, query_worker, &args[t]);
    }
    for (int t = 0; t < nthreads; ++t)
    {
        pthread_join(th[t], NULL);
    }
    free(th);
    free(args);
}

/* ------------------------------------------------------------------------- */
/* CellQuery: ghost copies on a padded axis-aligned grid                      */
/* ------------------------------------------------------------------------- */

typedef struct
{
    float fr[3];     /* r_cut / nearest-plane distance (CellQuery.cc:94) */
    float lat[3][3]; /* Box::getLatticeVector (Box.h:503-518) */
    float minp[3];   /* CellQuery::setupGrid (CellQuery.h:143-167) */
    float inv;
    int dim[3];
} oghost;

static void ghost_setup(const obox* b, float r_cut, oghost* G)
{
    G->inv = 1.0f / r_cut;
    const float wx = (b->L[0] + b->L[1] * fabsf(b->xy)) + b->L[2] * fabsf(b->xz);
    const float wy = b->L[1] + b->L[2] * fabsf(b->yz);
    const float wz = b->L[2];
    G->dim[0] = (int) (wx * G->inv) + 3;
    G->dim[1] = (int) (wy * G->inv) + 3;
    G->dim[2] = (int) (wz * G->inv) + 3;
    const float bmx = b->L[1] * fminf(0.0f, b->xy) + b->L[2] * fminf(0.0f, b->xz);
    const float bmy = b->L[2] * fminf(0.0f, b->yz);
    const float zero[3] = {0.0f, 0.0f, 0.0f};
    float a[3];
    make_absolute(b, zero, a);
    G->minp[0] = (bmx - r_cut) + a[0];
    G->minp[1] = (bmy - r_cut) + a[1];
    G->minp[2] = -r_cut + a[2];
    float pd[3];
    nearest_plane(b, pd);
    for (int d = 0; d < 3; ++d)
        G->fr[d] = r_cut / pd[d];
    G->lat[0][0] = b->L[0];
    G->lat[0][1] = 0.0f;
    G->lat[0][2] = 0.0f;
    G->lat[1][0] = b->L[1] * b->xy;
    G->lat[1][1] = b->L[1];
    G->lat[1][2] = 0.0f;
    G->lat[2][0] = b->is2d ? 0.0f : b->L[2] * b->xz;
    G->lat[2][1] = b->is2d ? 0.0f : b->L[2] * b->yz;
    G->lat[2][2] = b->is2d ? 0.0f : b->L[2];
}

/* cell_idx_xyz + getCellIdxSafe (CellQuery.h:53-75); 0 outside the grid */
static int ghost_cell(const oghost* G, const float* p, int* c)
{
    for (int d = 0; d < 3; ++d)
    {
        const float f = floorf((p[d] - G->minp[d]) * G->inv);
        if (!(f >= 0.0f && f < (float) G->dim[d]))
            return 0;
        c[d] = (int) f;
    }
    return 1;
}

/* The copies of point p: ghosts (faces, edges, corner; CellQuery.h:218-299),
 * then p itself. Returns the count (<= 8). */
static int ghost_copies(const obox* b, const oghost* G, const float* p, float out[8][3])
{
    int n = 0;
    float f[3];
    make_fractional(b, p, f);
    const int dx = (int) (f[0] <= G->fr[0]) - (int) ((double) f[0] >= 1.0 - (double) G->fr[0]);
    const int dy = (int) (f[1] <= G->fr[1]) - (int) ((double) f[1] >= 1.0 - (double) G->fr[1]);
    int dz = (int) (f[2] <= G->fr[2]) - (int) ((double) f[2] >= 1.0 - (double) G->fr[2]);
    if (b->is2d)
        dz = 0;
    if (dx != 0 || dy != 0 || dz != 0)
    {
        const int sites[7][3] = {{dx, 0, 0}, {0, dy, 0}, {0, 0, dz}, {dx, dy, 0}, {dx, 0, dz}, {0, dy, dz}, {dx, dy, dz}};
        const int use[7] = {dx != 0, dy != 0, dz != 0, dx != 0 && dy != 0, dx != 0 && dz != 0, dy != 0 && dz != 0,
                            dx != 0 && dy != 0 && dz != 0};
        for (int s = 0; s < 7; ++s)
        {
            if (!use[s])
                continue;
            float sh[3] = {0.0f, 0.0f, 0.0f};
            for (int a = 0; a < 3; ++a)
            {
                if (sites[s][a] != 0)
                {
                    for (int c = 0; c < 3; ++c)
                        sh[c] += sites[s][a] == 1 ? G->lat[a][c] : -G->lat[a][c];
                }
            }
            for (int c = 0; c < 3; ++c)
                out[n][c] = p[c] + sh[c];
            ++n;
        }
    }
    out[n][0] = p[0];
    out[n][1] = p[1];
    out[n][2] = p[2];
    return n + 1;
}

/* CellQueryBallIterator (CellIterator.h:35-185): the copies in the 27 cells around
 * the query's cell (clipped to the grid; no bonds for a query outside it), pair
 * vector g - q, the reference ball test, exclude_ii on the real index. */
static void ghost_bonds(const obox* b, const float* pts, uint32_t n, const float* qpts, uint32_t nq, float r_max,
                        float r_min, int exclude_ii, obonds* out)
{
    oghost G;
    ghost_setup(b, r_max, &G);
    const size_t ncell = (size_t) G.dim[0] * G.dim[1] * G.dim[2];
    uint32_t* cnt = (uint32_t*) calloc(ncell + 1, sizeof(uint32_t));
    float (*cp)[3] = (float (*)[3]) malloc(sizeof(float) * 3 * 8 * (size_t) (n ? n : 1));
    uint32_t* cj = (uint32_t*) malloc(sizeof(uint32_t) * 8 * (size_t) (n ? n : 1));
    uint32_t* cc = (uint32_t*) malloc(sizeof(uint32_t) * 8 * (size_t) (n ? n : 1));
    size_t nc = 0;
    for (uint32_t i = 0; i < n; ++i)
    {
        float copies[8][3];
        const int k = ghost_copies(b, &G, pts + 3 * (size_t) i, copies);
        for (int t = 0; t < k; ++t)
        {
            int c[3];
            if (!ghost_cell(&G, copies[t], c))
                continue;
            const size_t cell = ((size_t) c[2] * G.dim[1] + c[1]) * G.dim[0] + c[0];
            memcpy(cp[nc], copies[t], sizeof(float) * 3);
            cj[nc] = i;
            cc[nc] = (uint32_t) cell;
            cnt[cell + 1]++;
            ++nc;
        }
    }
    for (size_t c = 0; c < ncell; ++c)
        cnt[c + 1] += cnt[c];
    uint32_t* fill = (uint32_t*) malloc(sizeof(uint32_t) * (ncell ? ncell : 1));
    memcpy(fill, cnt, sizeof(uint32_t) * ncell);
    uint32_t* order = (uint32_t*) malloc(sizeof(uint32_t) * (nc ? nc : 1));
    for (size_t t = 0; t < nc; ++t)
        order[fill[cc[t]]++] = (uint32_t) t;
    const float rmax_sq = r_max * r_max;
    const float rmin_sq = r_min * r_min;
    for (uint32_t i = 0; i < nq; ++i)
    {
        const float* q = qpts + 3 * (size_t) i;
        int qc[3];
        if (!ghost_cell(&G, q, qc))
            continue;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx)
                {
                    const int x = qc[0] + dx, y = qc[1] + dy, z = qc[2] + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= G.dim[0] || y >= G.dim[1] || z >= G.dim[2])
                        continue;
                    const size_t cell = ((size_t) z * G.dim[1] + y) * G.dim[0] + x;
                    for (uint32_t u = cnt[cell]; u < cnt[cell + 1]; ++u)
                    {
                        const uint32_t t = order[u];
                        if (exclude_ii && cj[t] == i)
                            continue;
                        float r[3] = {cp[t][0] - q[0], cp[t][1] - q[1], cp[t][2] - q[2]};
                        const float rsq = dot3(r);
                        if (rsq < rmax_sq && rsq >= rmin_sq)
                            bonds_push(out, i, cj[t], sqrtf(rsq), r);
                    }
                }
    }
    free(cnt);
    free(cp);
    free(cj);
    free(cc);
    free(fill);
    free(order);
}

/* Neighbour query producing a NeighborList in reference order
 * (NeighborQuery.h:434-481): sorted by (i, j, weight, distance), or by
 * (i, distance, j, weight) when sort_by_distance. k == 0 selects a ball query.
 * box7 = (Lx, Ly, Lz, xy, xz, yz, is2D). Returns 0 on success. */
int ofg_query(const float* box7, const float* pts, uint32_t n, const float* qpts, uint32_t nq, uint32_t k,
              float r_max, float r_min, int exclude_ii, int arith, int sort_by_distance, int nthreads,
              uint64_t* nbonds_out, void** handle_out)
{
    obox box;
    box_init(&box, box7);
    if (arith == OFG_ARITH_GHOST)
    {
        obonds all = {0, 0, 0};
        ghost_bonds(&box, pts, n, qpts, nq, r_max, r_min, exclude_ii, &all);
        ofg_nlist* nl = (ofg_nlist*) malloc(sizeof(ofg_nlist));
        nl->n = all.n;
        nl->b = all.b ? all.b : (obond*) malloc(sizeof(obond));
        qsort(nl->b, nl->n, sizeof(obond), sort_by_distance ? cmp_dist : cmp_tuple);
        *nbonds_out = nl->n;
        *handle_out = nl;
        return 0;
    }
    qctx c;
    memset(&c, 0, sizeof(c));
    c.box = &box;
    c.pts = pts;
    c.qpts = qpts;
    c.nq = nq;
    c.r_max = r_max;
    c.r_min = r_min;
    c.exclude_ii = exclude_ii;
    c.arith = arith;
    c.k = k;
    c.n_img = image_vectors(&box, c.img);
    ogrid g;
    float width = r_max;
    if (k > 0)
    {
        /* density-based cell width giving ~k points per cell */
        float vol = box.is2d ? box.L[0] * box.L[1] : box.L[0] * box.L[1] * box.L[2];
        double per = (double) vol / (n > 0 ? n : 1) * (k > 4 ? k : 4);
        width = (float) (box.is2d ? sqrt(per) : cbrt(per));
    }
    grid_build(&box, &g, pts, n, width);
    c.grid = &g;
    if (nthreads < 1)
        nthreads = 1;
    c.per_thread = (obonds*) calloc((size_t) nthreads, sizeof(obonds));
    run_query(&c, nthreads);
    size_t total = 0;
    for (int t = 0; t < nthreads; ++t)
    {
        total += c.per_thread[t].n;
    }
    ofg_nlist* nl = (ofg_nlist*) malloc(sizeof(ofg_nlist));
    nl->n = total;
    nl->b = (obond*) malloc((total ? total : 1) * sizeof(obond));
    size_t off = 0;
    for (int t = 0; t < nthreads; ++t)
    {
        if (c.per_thread[t].n)
        {
            memcpy(nl->b + off, c.per_thread[t].b, c.per_thread[t].n * sizeof(obond));
        }
        off += c.per_thread[t].n;
        free(c.per_thread[t].b);
    }
    free(c.per_thread);
    grid_free(&g);
    qsort(nl->b, nl->n, sizeof(obond), sort_by_distance ? cmp_dist : cmp_tuple);
    *nbonds_out = nl->n;
    *handle_out = nl;
    return 0;
}

void ofg_nlist_copy(void* h, uint32_t* ij, float* dist, float* vec)
{
    ofg_nlist* nl = (ofg_nlist*) h;
    for (size_t b = 0; b < nl->n; ++b)
    {
        ij[2 * b] = nl->b[b].i;
        ij[2 * b + 1] = nl->b[b].j;
        dist[b] = nl->b[b].d;
        vec[3 * b] = nl->b[b].v[0];
        vec[3 * b + 1] = nl->b[b].v[1];
        vec[3 * b + 2] = nl->b[b].v[2];
    }
}

void ofg_nlist_free(void* h)
{
    ofg_nlist* nl = (ofg_nlist*) h;
    free(nl->b);
    free(nl);
}

/* Fused ball query + RDF histogram (the reference's RDF.compute((box, points)) path,
 * RDF.cc:101-110 over AABBQuery.cc:77-150). Adds into counts (uint64). */
int ofg_rdf_query(const float* box7, const float* pts, uint32_t n, const float* qpts, uint32_t nq, float q_r_max,
                  float q_r_min, int exclude_ii, int arith, uint32_t bins, float r_min, float r_max, int nthreads,
                  uint64_t* counts)
{
    obox box;
    box_init(&box, box7);
    if (arith == OFG_ARITH_GHOST)
    {
        obonds all = {0, 0, 0};
        ghost_bonds(&box, pts, n, qpts, nq, q_r_max, q_r_min, exclude_ii, &all);
        const float bw = (r_max - r_min) / (float) bins;
        const float inv = 1.0f / bw;
        for (size_t t = 0; t < all.n; ++t)
        {
            const int64_t bb = hist_bin(all.b[t].d, r_min, r_max, inv, bins);
            if (bb >= 0)
                counts[bb]++;
        }
        free(all.b);
        return 0;
    }
    qctx c;
    memset(&c, 0, sizeof(c));
    c.box = &box;
    c.pts = pts;
    c.qpts = qpts;
    c.nq = nq;
    c.r_max = q_r_max;
    c.r_min = q_r_min;
    c.exclude_ii = exclude_ii;
    c.arith = arith;
    c.n_img = image_vectors(&box, c.img);
    c.bins = bins;
    c.h_min = r_min;
    c.h_max = r_max;
    /* Histogram.h:130-131 */
    const float bw = (r_max - r_min) / (float) bins;
    c.h_inv = 1.0f / bw;
    ogrid g;
    grid_build(&box, &g, pts, n, q_r_max);
    c.grid = &g;
    if (nthreads < 1)
        nthreads = 1;
    c.per_thread = (obonds*) calloc((size_t) nthreads, sizeof(obonds));
    c.hist = (uint64_t**) malloc(sizeof(uint64_t*) * (size_t) nthreads);
    for (int t = 0; t < nthreads; ++t)
    {
        c.hist[t] = (uint64_t*) calloc(bins, sizeof(uint64_t));
    }
    run_query(&c, nthreads);
    for (int t = 0; t < nthreads; ++t)
    {
        for (uint32_t b = 0; b < bins; ++b)
        {
            counts[b] += c.hist[t][b];
        }
        free(c.hist[t]);
        free(c.per_thread[t].b);
    }
    free(c.hist);
    free(c.per_thread);
    grid_free(&g);
    return 0;
}

/* Histogram of a list of distances (RDF.cc:107-109 over a NeighborList). */
void ofg_hist(const float* distances, uint64_t nb, uint32_t bins, float r_min, float r_max, uint64_t* counts)
{
    const float bw = (r_max - r_min) / (float) bins;
    const float inv = 1.0f / bw;
    for (uint64_t b = 0; b < nb; ++b)
    {
        int64_t k = hist_bin(distances[b], r_min, r_max, inv, bins);
        if (k >= 0)
        {
            counts[k]++;
        }
    }
}

/* Bin index of each distance as Histogram::bin assigns it (Histogram.h:327-351),
 * -1 for distances outside [r_min, r_max); used for the CorrelationFunction
 * oracle (CorrelationFunction.cc:79-96), whose FP64 sums are formed in Python. */
void ofg_bin_index(const float* distances, uint64_t nb, uint32_t bins, float r_min, float r_max, int64_t* out)
{
    const float bw = (r_max - r_min) / (float) bins;
    const float inv = 1.0f / bw;
    for (uint64_t b = 0; b < nb; ++b)
    {
        out[b] = hist_bin(distances[b], r_min, r_max, inv, bins);
    }
}

/* PMFT binning of a list's bonds (PMFTR12.cc:92-110, PMFTXYT.cc:79-100,
 * PMFTXY.cc:71-88, PMFTXYZ.cc:116-145), in the reference's float arithmetic with
 * the C library's cosf / sinf / atan2f / fmodf. kind 0 R12, 1 XYT, 2 XY, 3 XYZ.
 * axes: (min, max, n) per axis (n = 1 for the unused third axis of XY). Adds into
 * row-major uint64 counts. */
static float o_modpos(float a, float b)
{
    return fmodf(fmodf(a, b) + b, b);
}

static void o_qrotate(const float* q, const float* b, float* o)
{
    /* rotate(quat, vec3) (VectorMath.h:810-823) */
    const float vv = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    const float t1 = q[0] * q[0] - vv;
    const float s2 = 2.0f * q[0];
    const float cx = q[2] * b[2] - q[3] * b[1];
    const float cy = q[3] * b[0] - q[1] * b[2];
    const float cz = q[1] * b[1] - q[2] * b[0];
    const float d2 = 2.0f * (q[1] * b[0] + q[2] * b[1] + q[3] * b[2]);
    o[0] = t1 * b[0] + s2 * cx + d2 * q[1];
    o[1] = t1 * b[1] + s2 * cy + d2 * q[2];
    o[2] = t1 * b[2] + s2 * cz + d2 * q[3];
}

void ofg_pmft(int kind, uint64_t nb, const uint32_t* ij, const float* dist, const float* vec, const float* p_angle,
              const float* q_angle, const float* q_quat, const float* equiv, uint32_t n_equiv, const float* axes,
              uint64_t* counts)
{
    const float two_pi = (float) (2.0 * M_PI);
    float inv[3];
    for (int a = 0; a < 3; ++a)
    {
        inv[a] = 1.0f / ((axes[3 * a + 1] - axes[3 * a]) / (float) (uint32_t) axes[3 * a + 2]);
    }
    const uint32_t n1 = (uint32_t) axes[5], n2 = (uint32_t) axes[8];
    for (uint64_t e = 0; e < nb; ++e)
    {
        const uint32_t i = ij[2 * e], j = ij[2 * e + 1];
        const float dx = vec[3 * e], dy = vec[3 * e + 1], dz = vec[3 * e + 2];
        float c[3];
        int ncoord = 1;
        float vals[64][3];
        if (kind == 0)
        {
            const float t1 = o_modpos(p_angle[j] - atan2f(dy, dx), two_pi);
            const float t2 = o_modpos(q_angle[i] - atan2f(-dy, -dx), two_pi);
            vals[0][0] = dist[e];
            vals[0][1] = t1;
            vals[0][2] = t2;
        }
        else if (kind == 1 || kind == 2)
        {
            const float th = -q_angle[i];
            const float cs = cosf(th), sn = sinf(th);
            vals[0][0] = cs * dx + (-sn) * dy;
            vals[0][1] = sn * dx + cs * dy;
            vals[0][2] = kind == 1 ? o_modpos(p_angle[j] - atan2f(-dy, -dx), two_pi) : 0.0f;
        }
        else
        {
            const float cq[4] = {q_quat[4 * i], -q_quat[4 * i + 1], -q_quat[4 * i + 2], -q_quat[4 * i + 3]};
            const float d[3] = {dx, dy, dz};
            float u[3];
            o_qrotate(cq, d, u);
            ncoord = (int) n_equiv;
            for (int k = 0; k < ncoord && k < 64; ++k)
            {
                o_qrotate(equiv + 4 * k, u, vals[k]);
            }
        }
        for (int k = 0; k < ncoord && k < 64; ++k)
        {
            int64_t b[3];
            int ok = 1;
            for (int a = 0; a < 3; ++a)
            {
                c[a] = vals[k][a];
                b[a] = hist_bin(c[a], axes[3 * a], axes[3 * a + 1], inv[a], (uint32_t) axes[3 * a + 2]);
                ok &= b[a] >= 0;
            }
            if (ok)
            {
                counts[((uint64_t) b[0] * n1 + (uint64_t) b[1]) * n2 + (uint64_t) b[2]]++;
            }
        }
    }
}

/* Bin edges / centres (Histogram.h:126-138, :72-80). */
void ofg_bin_edges(uint32_t bins, float r_min, float r_max, float* edges, float* centers)
{
    const float bw = (r_max - r_min) / (float) bins;
    for (uint32_t i = 0; i <= bins; ++i)
    {
        edges[i] = r_min + (float) i * bw;
    }
    for (uint32_t i = 0; i < bins; ++i)
    {
        centers[i] = (edges[i] + edges[i + 1]) / 2.0f;
    }
}

/* RDF normalisation in float32 (RDF.cc:52-63 shell volumes, :73-99 reduce).
 * counts are the uint32 bin counts the reference stores (the caller truncates). */
void ofg_rdf_reduce(const uint32_t* counts, uint32_t bins, float r_min, float r_max, uint32_t n_frames,
                    uint32_t n_points, uint32_t n_query_points, float volume, int is2d, int finite_size,
                    float* rdf, float* n_r)
{
    float* edges = (float*) malloc(sizeof(float) * (bins + 1));
    float* centers = (float*) malloc(sizeof(float) * (bins + 1));
    ofg_bin_edges(bins, r_min, r_max, edges, centers);
    const float volume_prefactor = (float) ((4.0f / 3.0f) * M_PI);
    const float nqp = (float) n_query_points;
    float number_density = nqp / volume;
    if (finite_size)
    {
        number_density *= (float) (n_query_points - 1) / (float) n_query_points;
    }
    const float np = (float) n_points;
    const float nf = (float) n_frames;
    const float prefactor = 1.0f / (np * number_density * nf);
    for (uint32_t i = 0; i < bins; ++i)
    {
        const float r = edges[i];
        const float nr = edges[i + 1];
        float vol;
        if (is2d)
        {
            vol = (float) (M_PI * (double) (nr * nr - r * r));
        }
        else
        {
            vol = volume_prefactor * (nr * nr * nr - r * r * r);
        }
        rdf[i] = (float) counts[i] * prefactor / vol;
    }
    const float pf2 = 1.0f / (nqp * (float) n_frames);
    n_r[0] = (float) counts[0] * pf2;
    for (uint32_t i = 1; i < bins; ++i)
    {
        n_r[i] = n_r[i - 1] + (float) counts[i] * pf2;
    }
    free(edges);
    free(centers);
}

/* ------------------------------------------------------------------------- */
/* Steinhardt (FP64)                                                         */
/* ------------------------------------------------------------------------- */

/* Y_l^m(theta, phi) in double, m order 0..l, -1..-l, equal to
 * scipy.special.sph_harm_y(l, m, theta, phi) (Condon-Shortley phase included),
 * which is the contract Steinhardt.cc:31-52 produces. Associated Legendre values
 * come from the standard three-term recurrence in l. */
void ofg_ylm(int l, double theta, double phi, double* out /* 2*(2l+1) */)
{
    const double x = cos(theta);
    const double s = sqrt(fmax(0.0, 1.0 - x * x));
    for (int m = 0; m <= l; ++m)
    {
        double pmm = 1.0; /* P_m^m without CS phase: (2m-1)!! s^m */
        for (int k = 1; k <= m; ++k)
        {
            pmm *= (2.0 * k - 1.0) * s;
        }
        double plm;
        if (l == m)
        {
            plm = pmm;
        }
        else
        {
            double pm1 = x * (2.0 * m + 1.0) * pmm;
            if (l == m + 1)
            {
                plm = pm1;
            }
            else
            {
                double a = pmm, bb = pm1, cc = 0.0;
                for (int ll = m + 2; ll <= l; ++ll)
                {
                    cc = ((2.0 * ll - 1.0) * x * bb - (ll + m - 1.0) * a) / (ll - m);
                    a = bb;
                    bb = cc;
                }
                plm = cc;
            }
        }
        double ratio = 1.0;
        for (int k = l - m + 1; k <= l + m; ++k)
        {
            ratio /= k;
        }
        const double nrm = sqrt((2.0 * l + 1.0) / (4.0 * M_PI) * ratio) * plm;
        const double cs = (m % 2) ? -1.0 : 1.0;
        /* m >= 0 : CS * N P e^{i m phi} */
        out[2 * m] = cs * nrm * cos(m * phi);
        out[2 * m + 1] = cs * nrm * sin(m * phi);
        if (m > 0)
        {
            /* Y_l^{-m} = (-1)^m conj(Y_l^m) */
            out[2 * (l + m)] = nrm * cos(m * phi);
            out[2 * (l + m) + 1] = -nrm * sin(m * phi);
        }
    }
}

static double lfact(int n)
{
    return lgamma((double) n + 1.0);
}

/* Wigner 3j symbol (l l l; m1 m2 m3) by the Racah formula, in double. */
double ofg_wigner3j(int l, int m1, int m2, int m3)
{
    if (m1 + m2 + m3 != 0 || abs(m1) > l || abs(m2) > l || abs(m3) > l)
    {
        return 0.0;
    }
    const int j1 = l, j2 = l, j3 = l;
    const double tri = 0.5 * (lfact(j1 + j2 - j3) + lfact(j1 - j2 + j3) + lfact(-j1 + j2 + j3) - lfact(j1 + j2 + j3 + 1));
    const double pre = 0.5 * (lfact(j1 + m1) + lfact(j1 - m1) + lfact(j2 + m2) + lfact(j2 - m2) + lfact(j3 + m3)
                              + lfact(j3 - m3));
    int kmin = 0;
    if (j2 - j3 - m1 > kmin)
        kmin = j2 - j3 - m1;
    if (j1 - j3 + m2 > kmin)
        kmin = j1 - j3 + m2;
    int kmax = j1 + j2 - j3;
    if (j1 - m1 < kmax)
        kmax = j1 - m1;
    if (j2 + m2 < kmax)
        kmax = j2 + m2;
    double sum = 0.0;
    for (int k = kmin; k <= kmax; ++k)
    {
        const double lt = lfact(k) + lfact(j1 + j2 - j3 - k) + lfact(j1 - m1 - k) + lfact(j2 + m2 - k)
            + lfact(j3 - j2 + m1 + k) + lfact(j3 - j1 - m2 + k);
        const double term = exp(tri + pre - lt);
        sum += (k % 2) ? -term : term;
    }
    const int ph = j1 - j2 - m3;
    return ((ph % 2) != 0 ? -1.0 : 1.0) * sum;
}

static int lm_index(int l, int m)
{
    return m < 0 ? l - m : m; /* Wigner3j.cc:17-20 */
}

/* Wigner-3j coefficients of one l in the iteration order of reduce_w3j_tab
 * (m1 ascending, then m2 ascending): computed once per l, not per particle. */
static double* w3j_table(int l)
{
    size_t n = 0;
    for (int m1 = -l; m1 <= l; ++m1)
    {
        const int lo = (-l - m1) > -l ? (-l - m1) : -l;
        const int hi = (l - m1) < l ? (l - m1) : l;
        n += (size_t) (hi - lo + 1);
    }
    double* t = (double*) malloc(sizeof(double) * (n ? n : 1));
    size_t k = 0;
    for (int m1 = -l; m1 <= l; ++m1)
    {
        const int lo = (-l - m1) > -l ? (-l - m1) : -l;
        const int hi = (l - m1) < l ? (l - m1) : l;
        for (int m2 = lo; m2 <= hi; ++m2)
            t[k++] = ofg_wigner3j(l, m1, m2, -m1 - m2);
    }
    return t;
}

/* Wigner3j.cc:22-57 in double, with the coefficients from w3j_table(l); *mag
 * (optional) receives the sum of |terms|, the scale against which the
 * cancellation in the sum is judged. */
static double reduce_w3j_tab(const double* q, int l, const double* w3j, double* mag)
{
    double res = 0.0;
    double m_abs = 0.0;
    size_t k = 0;
    for (int m1 = -l; m1 <= l; ++m1)
    {
        const int lo = (-l - m1) > -l ? (-l - m1) : -l;
        const int hi = (l - m1) < l ? (l - m1) : l;
        for (int m2 = lo; m2 <= hi; ++m2)
        {
            const int m3 = -m1 - m2;
            const double w = w3j[k++];
            const double* a = q + 2 * lm_index(l, m1);
            const double* b = q + 2 * lm_index(l, m2);
            const double* c = q + 2 * lm_index(l, m3);
            const double abr = a[0] * b[0] - a[1] * b[1];
            const double abi = a[0] * b[1] + a[1] * b[0];
            const double term = w * (abr * c[0] - abi * c[1]);
            res += term;
            m_abs += fabs(term);
        }
    }
    if (mag)
        *mag = m_abs;
    return res;
}

/* Shared state of the threaded Steinhardt phases; each phase is a loop over
 * particles split into contiguous ranges, one per thread. Every particle's
 * result depends only on its own bonds (and, for the average, on the finished
 * plain qlm), so the output does not depend on the thread count. */
typedef struct
{
    const uint32_t* ls;
    uint32_t nl, maxl;
    int weighted, wl_normalize, average;
    obox box;
    const float* pts;
    uint32_t n;
    const uint32_t* ij;
    const float* bond_dist;
    const float* bond_w;
    const uint64_t* first;
    size_t stride;
    double* ql;
    double* ql_ave;
    double* wl_out;
    double* wl_mag;
    double* qlm;
    double* qave;
    double** w3j; /* per l index */
    int phase;    /* 0 plain qlm, 1 average, 2 wl */
    int nthreads;
} stctx;

typedef struct
{
    stctx* c;
    int tid;
} starg;

/* Steinhardt.cc:120-222 for particle i in FP64 (pair vector wrap(p_j - p_i) in float32) */
static void st_plain(stctx* c, uint32_t i, double* ylm)
{
    double tw = 0.0;
    const float* pi = c->pts + 3 * (size_t) i;
    double* row = c->qlm + 2 * (size_t) i * c->stride;
    for (uint64_t t = c->first[i]; t < c->first[i + 1]; ++t)
    {
        const uint32_t j = c->ij[2 * t + 1];
        const float* pj = c->pts + 3 * (size_t) j;
        float dv[3] = {pj[0] - pi[0], pj[1] - pi[1], pj[2] - pi[2]};
        float dl[3];
        box_wrap(&c->box, dv, dl);
        const double w = c->weighted ? (double) c->bond_w[t] : 1.0;
        const double phi = atan2((double) dl[1], (double) dl[0]);
        const double dist = (double) c->bond_dist[t];
        double ct = (double) dl[2] / dist;
        if (ct < -1.0)
            ct = -1.0;
        if (ct > 1.0)
            ct = 1.0;
        double theta = acos(ct);
        if (c->bond_dist[t] == 0.0f)
            theta = 0.0;
        size_t off = 0;
        for (uint32_t k = 0; k < c->nl; ++k)
        {
            const int l = (int) c->ls[k];
            ofg_ylm(l, theta, phi, ylm);
            for (int m = 0; m < 2 * l + 1; ++m)
            {
                row[2 * (off + m)] += w * ylm[2 * m];
                row[2 * (off + m) + 1] += w * ylm[2 * m + 1];
            }
            off += 2 * l + 1;
        }
        tw += w;
    }
    size_t off = 0;
    for (uint32_t k = 0; k < c->nl; ++k)
    {
        const int l = (int) c->ls[k];
        double s = 0.0;
        for (int m = 0; m < 2 * l + 1; ++m)
        {
            double* v = &row[2 * (off + m)];
            v[0] /= tw;
            v[1] /= tw;
            s += v[0] * v[0] + v[1] * v[1];
        }
        c->ql[(size_t) i * c->nl + k] = sqrt(s * (4.0 * M_PI / (2 * l + 1)));
        off += 2 * l + 1;
    }
}

/* Steinhardt.cc:224-289 for particle i in FP64 */
static void st_average(stctx* c, uint32_t i)
{
    const size_t s2 = 2 * c->stride;
    double* dst = &c->qave[(size_t) i * s2];
    for (size_t m = 0; m < s2; ++m)
        dst[m] = c->qlm[(size_t) i * s2 + m];
    uint64_t cnt = 1;
    for (uint64_t t = c->first[i]; t < c->first[i + 1]; ++t)
    {
        const uint32_t j = c->ij[2 * t + 1];
        for (size_t m = 0; m < s2; ++m)
            dst[m] += c->qlm[(size_t) j * s2 + m];
        cnt++;
    }
    for (size_t m = 0; m < s2; ++m)
        dst[m] /= (double) cnt;
    size_t off = 0;
    for (uint32_t k = 0; k < c->nl; ++k)
    {
        const int l = (int) c->ls[k];
        double s = 0.0;
        for (int m = 0; m < 2 * l + 1; ++m)
        {
            const double* v = &dst[2 * (off + m)];
            s += v[0] * v[0] + v[1] * v[1];
        }
        c->ql_ave[(size_t) i * c->nl + k] = sqrt(s * (4.0 * M_PI / (2 * l + 1)));
        off += 2 * l + 1;
    }
}

/* Steinhardt.cc:329-359 (wl of the plain or averaged qlm) for particle i in FP64 */
static void st_wl(stctx* c, uint32_t i)
{
    const double* src = c->average ? c->qave : c->qlm;
    const double* nsrc = c->average ? c->ql_ave : c->ql;
    size_t off = 0;
    for (uint32_t k = 0; k < c->nl; ++k)
    {
        const int l = (int) c->ls[k];
        double mag = 0.0;
        double v = reduce_w3j_tab(&src[2 * ((size_t) i * c->stride + off)], l, c->w3j[k], &mag);
        if (c->wl_normalize)
        {
            const double nf = sqrt(4.0 * M_PI / (2 * l + 1)) / nsrc[(size_t) i * c->nl + k];
            v *= nf * nf * nf;
            mag *= nf * nf * nf;
        }
        c->wl_out[(size_t) i * c->nl + k] = v;
        if (c->wl_mag)
            c->wl_mag[(size_t) i * c->nl + k] = mag;
        off += 2 * l + 1;
    }
}

static void* st_worker(void* varg)
{
    starg* a = (starg*) varg;
    stctx* c = a->c;
    const uint32_t per = (c->n + (uint32_t) c->nthreads - 1) / (uint32_t) c->nthreads;
    const uint32_t i0 = per * (uint32_t) a->tid;
    const uint32_t i1 = i0 + per < c->n ? i0 + per : c->n;
    double* ylm = (double*) malloc(sizeof(double) * 2 * (2 * c->maxl + 1));
    for (uint32_t i = i0; i < i1; ++i)
    {
        if (c->phase == 0)
            st_plain(c, i, ylm);
        else if (c->phase == 1)
            st_average(c, i);
        else
            st_wl(c, i);
    }
    free(ylm);
    return NULL;
}

static void st_run(stctx* c, int phase)
{
    c->phase = phase;
    pthread_t* th = (pthread_t*) malloc(sizeof(pthread_t) * (size_t) c->nthreads);
    starg* args = (starg*) malloc(sizeof(starg) * (size_t) c->nthreads);
    for (int t = 0; t < c->nthreads; ++t)
    {
        args[t].c = c;
        args[t].tid = t;
        pthread_create(&th[t], NULL, st_worker, &args[t]);
    }
    for (int t = 0; t < c->nthreads; ++t)
        pthread_join(th[t], NULL);
    free(th);
    free(args);
}

/* Steinhardt over a NeighborList sorted by query index (Steinhardt.cc:120-359).
 * Pair vectors are recomputed as wrap(p_j - p_i) in float32 (Steinhardt.cc:155),
 * the rest is FP64. Per-particle phases run on nthreads threads (the results do
 * not depend on the thread count). Outputs (row-major, n rows):
 *   ql      (n, nl)        plain ql
 *   ql_ave  (n, nl)        averaged ql (only when average)
 *   wl      (n, nl)        wl of (averaged if average) qlm (only when wl)
 *   qlm     (n, sum(2l+1)) complex as re/im pairs (plain qlmi)
 *   order   (nl)           system order */
int ofg_steinhardt(const uint32_t* ls, uint32_t nl, int average, int wl, int weighted, int wl_normalize,
                   const float* box7, const float* pts, uint32_t n, uint64_t nbonds, const uint32_t* ij,
                   const float* bond_dist, const float* bond_w, double* ql, double* ql_ave, double* wl_out,
                   double* qlm, double* order, double* wl_mag, int nthreads)
{
    stctx c;
    memset(&c, 0, sizeof(c));
    box_init(&c.box, box7);
    c.ls = ls;
    c.nl = nl;
    c.weighted = weighted;
    c.wl_normalize = wl_normalize;
    c.average = average;
    c.pts = pts;
    c.n = n;
    c.ij = ij;
    c.bond_dist = bond_dist;
    c.bond_w = bond_w;
    c.ql = ql;
    c.ql_ave = ql_ave;
    c.wl_out = wl_out;
    c.wl_mag = wl_mag;
    c.qlm = qlm;
    c.nthreads = nthreads < 1 ? 1 : nthreads;
    for (uint32_t k = 0; k < nl; ++k)
    {
        c.stride += 2 * ls[k] + 1;
        if (ls[k] > c.maxl)
            c.maxl = ls[k];
    }
    const size_t stride = c.stride;
    c.qave = (double*) calloc((size_t) n * stride * 2 + 1, sizeof(double));
    double* sys = (double*) calloc(stride * 2, sizeof(double));
    uint64_t* first = (uint64_t*) malloc(sizeof(uint64_t) * ((size_t) n + 1));
    /* segments (NeighborList.cc:199-232) */
    uint64_t b = 0;
    for (uint32_t i = 0; i <= n; ++i)
    {
        while (b < nbonds && ij[2 * b] < i)
            ++b;
        first[i] = b;
    }
    c.first = first;
    memset(qlm, 0, sizeof(double) * (size_t) n * stride * 2);
    st_run(&c, 0);
    const double* src = qlm;
    if (average)
    {
        st_run(&c, 1);
        src = c.qave;
    }
    /* system qlm: mean over particles of qlmi (or qlmiAve), Steinhardt.cc:203-207,
     * 265-266, summed in particle order */
    for (uint32_t i = 0; i < n; ++i)
    {
        for (size_t m = 0; m < 2 * stride; ++m)
            sys[m] += src[2 * (size_t) i * stride + m] / (double) n;
    }
    if (wl)
    {
        c.w3j = (double**) malloc(sizeof(double*) * (nl ? nl : 1));
        for (uint32_t k = 0; k < nl; ++k)
            c.w3j[k] = w3j_table((int) ls[k]);
        st_run(&c, 2);
    }
    /* Steinhardt.cc:291-327 */
    size_t off = 0;
    for (uint32_t k = 0; k < nl; ++k)
    {
        const int l = (int) ls[k];
        const double nf = 4.0 * M_PI / (2 * l + 1);
        double s = 0.0;
        for (int m = 0; m < 2 * l + 1; ++m)
            s += sys[2 * (off + m)] * sys[2 * (off + m)] + sys[2 * (off + m) + 1] * sys[2 * (off + m) + 1];
        const double qsys = sqrt(s * nf);
        if (wl)
        {
            double v = reduce_w3j_tab(&sys[2 * off], l, c.w3j[k], NULL);
            if (wl_normalize)
            {
                const double w = sqrt(nf) / qsys;
                v *= w * w * w;
            }
            order[k] = v;
        }
        else
        {
            order[k] = qsys;
        }
        off += 2 * l + 1;
    }
    if (c.w3j)
    {
        for (uint32_t k = 0; k < nl; ++k)
            free(c.w3j[k]);
        free(c.w3j);
    }
    free(c.qave);
    free(sys);
    free(first);
    return 0;
}

/* Box helpers exported for the Python tests. */
void ofg_box_wrap(const float* box7, const float* v, uint64_t n, float* out)
{
    obox box;
    box_init(&box, box7);
    for (uint64_t i = 0; i < n; ++i)
        box_wrap(&box, v + 3 * i, out + 3 * i);
}

void ofg_box_fractional(const float* box7, const float* v, uint64_t n, float* out)
{
    obox box;
    box_init(&box, box7);
    for (uint64_t i = 0; i < n; ++i)
        make_fractional(&box, v + 3 * i, out + 3 * i);
}
