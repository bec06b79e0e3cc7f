/*
 * lss_oracle.c -- CPU restatement of the reference's GPU hybrid solve path.
 *
 * TEST INFRASTRUCTURE ONLY (the reference for parity tests, never the
 * product).  Parity status:
 * UNPINNED -- the reference has no golden vectors for this path and cannot be
 * compiled here; see lss_oracle.h.
 *
 * Every function cites the reference file:line it restates.  Paths are
 * relative to the reference project root.  Built with -ffp-contract=off so
 * that x86 and aarch64 builds round identically.
 */
#include "lss_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define BANK 32

static void *xmalloc(size_t n) { void *p = malloc(n ? n : 1); return p; }
static void *xcalloc(size_t n, size_t s) { void *p = calloc(n ? n : 1, s ? s : 1); return p; }

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* ===================================================================== */
/* Selection                                                               */
/* ===================================================================== */

/* GPUHybrid.cu:753-765 -- sequential sum in storage order, per outer slice. */
void lsso_row_l1_norms(int32_t n, const int32_t *outer, const double *values, double *rn)
{
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int32_t k = outer[i]; k < outer[i + 1]; ++k) s += fabs(values[k]);
        rn[i] = s;
    }
}

/* E-step of one row, GPUHybrid.cu:800-818 (same expression tree). */
static void estep_row(double x, double w0, double w1, double m0, double m1, double v0,
                      double v1, double *lg0_out, double *lg1_out, double *g0, double *g1)
{
    double log_w0 = log(w0);
    double log_w1 = log(w1);
    double log_N0 = -0.5 * log(2.0 * M_PI * v0) - 0.5 * (x - m0) * (x - m0) / v0;
    double log_N1 = -0.5 * log(2.0 * M_PI * v1) - 0.5 * (x - m1) * (x - m1) / v1;
    double lg0 = log_w0 + log_N0;
    double lg1 = log_w1 + log_N1;
    double mx = fmax(lg0, lg1);
    double lt = mx + log(exp(lg0 - mx) + exp(lg1 - mx));
    *g0 = exp(lg0 - lt);
    *g1 = exp(lg1 - lt);
    *lg0_out = lg0;
    *lg1_out = lg1;
}

/* GPUHybrid.cu:767-879.  Sums run sequentially in index order (the reference's
 * thrust reductions have an unspecified order; the selected set is insensitive
 * to the last-ulp differences this causes unless a row sits on the decision
 * boundary, which stats->min_log_margin reports). */
int32_t lsso_gmm_select(int32_t n, const double *rn, double jump_threshold, double tol,
                        int32_t max_iterations, int32_t *sel, lsso_gmm_stats *st)
{
    lsso_gmm_stats dummy;
    if (!st) st = &dummy;
    memset(st, 0, sizeof(*st));
    if (n <= 0) return 0;

    double sum = 0.0;
    for (int32_t i = 0; i < n; ++i) sum += rn[i];
    double global_mean = sum / n;
    double vs = 0.0;
    for (int32_t i = 0; i < n; ++i) vs += (rn[i] - global_mean) * (rn[i] - global_mean);
    double global_var = vs / n;
    double mn = rn[0], mx = rn[0];
    for (int32_t i = 1; i < n; ++i) {
        if (rn[i] < mn) mn = rn[i];
        if (rn[i] > mx) mx = rn[i];
    }

    double mean0 = mn, mean1 = mx, var0 = global_var, var1 = global_var;
    double w0 = 0.5, w1 = 0.5;
    const double var_reg = 1e-6;

    /* thrust::device_vector<double>(n) is value-initialised: gammas start at 0,
     * so with zero EM iterations nothing is selected. */
    double *g0 = (double *)xcalloc((size_t)n, sizeof(double));
    double *g1 = (double *)xcalloc((size_t)n, sizeof(double));
    double *lg0 = (double *)xcalloc((size_t)n, sizeof(double));
    double *lg1 = (double *)xcalloc((size_t)n, sizeof(double));
    int32_t it, esteps = 0;
    for (it = 0; it < max_iterations; ++it) {
        for (int32_t i = 0; i < n; ++i)
            estep_row(rn[i], w0, w1, mean0, mean1, var0, var1, &lg0[i], &lg1[i], &g0[i], &g1[i]);
        ++esteps;
        double s0 = 0.0, s1 = 0.0;
        for (int32_t i = 0; i < n; ++i) s0 += g0[i];
        for (int32_t i = 0; i < n; ++i) s1 += g1[i];
        w0 = s0 / n;
        w1 = s1 / n;
        double om0 = mean0, om1 = mean1, ov0 = var0, ov1 = var1;
        double a0 = 0.0, a1 = 0.0;
        for (int32_t i = 0; i < n; ++i) a0 += g0[i] * rn[i];
        for (int32_t i = 0; i < n; ++i) a1 += g1[i] * rn[i];
        mean0 = a0 / s0;
        mean1 = a1 / s1;
        double b0 = 0.0, b1 = 0.0;
        for (int32_t i = 0; i < n; ++i) b0 += g0[i] * (rn[i] - mean0) * (rn[i] - mean0);
        for (int32_t i = 0; i < n; ++i) b1 += g1[i] * (rn[i] - mean1) * (rn[i] - mean1);
        var0 = b0 / s0 + var_reg;
        var1 = b1 / s1 + var_reg;
        /* GPUHybrid.cu:850-856: relative change against the old value, no epsilon */
        if (fabs(mean0 - om0) / fabs(om0) < tol && fabs(mean1 - om1) / fabs(om1) < tol &&
            fabs(var0 - ov0) / fabs(ov0) < tol && fabs(var1 - ov1) / fabs(ov1) < tol)
            break;
    }

    int32_t count = 0;
    int32_t jump = fabs(mean1) / fabs(mean0) > jump_threshold; /* GPUHybrid.cu:860, strict */
    double margin = INFINITY;
    if (esteps > 0)
        for (int32_t i = 0; i < n; ++i) {
            double d = fabs(lg0[i] - lg1[i]);
            if (d < margin) margin = d;
        }
    if (jump)
        for (int32_t i = 0; i < n; ++i)
            if (g0[i] < g1[i]) sel[count++] = i; /* GPUHybrid.cu:863-868, ascending */

    st->global_mean = global_mean;
    st->global_var = global_var;
    st->mean0 = mean0; st->mean1 = mean1; st->var0 = var0; st->var1 = var1;
    st->w0 = w0; st->w1 = w1;
    st->min_log_margin = margin;
    st->gmm_iters = it;
    st->estep_count = esteps;
    st->jump_passed = jump;
    st->num_selected = count;
    free(g0); free(g1); free(lg0); free(lg1);
    return count;
}

/* ---- disjoint set, Hybrid.hpp:223-260 ---------------------------------- */
typedef struct { int32_t *parent, *rank; } dset;
static void ds_init(dset *d, int32_t n)
{
    d->parent = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    d->rank = (int32_t *)xcalloc((size_t)(n > 0 ? n : 1), sizeof(int32_t));
    for (int32_t i = 0; i < n; ++i) d->parent[i] = i;
}
static void ds_free(dset *d) { free(d->parent); free(d->rank); }
static int32_t ds_find(dset *d, int32_t v)
{
    int32_t r = v;
    while (d->parent[r] != r) r = d->parent[r];
    while (d->parent[v] != r) { int32_t nx = d->parent[v]; d->parent[v] = r; v = nx; }
    return r;
}
static void ds_union(dset *d, int32_t x, int32_t y)
{
    if (x == y) return;
    x = ds_find(d, x);
    y = ds_find(d, y);
    if (x == y) return;
    if (d->rank[x] > d->rank[y]) d->parent[y] = x;
    else {
        d->parent[x] = y;
        if (d->rank[x] == d->rank[y]) d->rank[y]++;
    }
}

/* Components of `sel` (ascending) in the pattern: comp[local] = root label
 * renumbered so that components are numbered by their smallest member.
 * (GPUHybrid.cu:695-720 / 895-919) */
static int32_t components(int32_t n, const int32_t *outer, const int32_t *inner,
                          const int32_t *sel, int32_t nsel, int32_t *g2l, int32_t *comp)
{
    for (int32_t i = 0; i < nsel; ++i) g2l[sel[i]] = i;
    dset d;
    ds_init(&d, nsel);
    for (int32_t a = 0; a < nsel; ++a) {
        int32_t k = sel[a];
        for (int32_t e = outer[k]; e < outer[k + 1]; ++e) {
            int32_t row = inner[e];
            if (row >= 0 && row < n && g2l[row] != -1) ds_union(&d, g2l[row], a);
        }
    }
    int32_t *label = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nsel > 0 ? nsel : 1));
    for (int32_t i = 0; i < nsel; ++i) label[i] = -1;
    int32_t nc = 0;
    for (int32_t a = 0; a < nsel; ++a) {
        int32_t r = ds_find(&d, a);
        if (label[r] < 0) label[r] = nc++;
        comp[a] = label[r];
    }
    free(label);
    ds_free(&d);
    return nc;
}

int32_t lsso_filter_subdomains(int32_t n, const int32_t *outer, const int32_t *inner,
                               const double *values, const int32_t *sel, int32_t nsel,
                               int32_t min_size, int32_t max_size, double cond_threshold,
                               int32_t *out, int32_t *counters)
{
    int32_t *g2l = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (int32_t i = 0; i < n; ++i) g2l[i] = -1;
    int32_t *comp = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nsel > 0 ? nsel : 1));
    int32_t nc = components(n, outer, inner, sel, nsel, g2l, comp);

    int32_t *size = (int32_t *)xcalloc((size_t)(nc > 0 ? nc : 1), sizeof(int32_t));
    double *lmin = (double *)xmalloc(sizeof(double) * (size_t)(nc > 0 ? nc : 1));
    double *lmax = (double *)xmalloc(sizeof(double) * (size_t)(nc > 0 ? nc : 1));
    for (int32_t c = 0; c < nc; ++c) { lmin[c] = DBL_MAX; lmax[c] = 0.0; }
    for (int32_t a = 0; a < nsel; ++a) size[comp[a]]++;
    /* Gershgorin bounds, GPUHybrid.cu:936-958 */
    for (int32_t a = 0; a < nsel; ++a) {
        int32_t k = sel[a];
        double diag = 0.0, off = 0.0;
        for (int32_t e = outer[k]; e < outer[k + 1]; ++e) {
            int32_t row = inner[e];
            if (g2l[row] != -1) {
                if (row == k) diag = values[e];
                else off += fabs(values[e]);
            }
        }
        int32_t c = comp[a];
        if (diag - off < lmin[c]) lmin[c] = diag - off;
        if (diag + off > lmax[c]) lmax[c] = diag + off;
    }
    int32_t too_small = 0, too_large = 0, not_poor = 0;
    char *keep = (char *)xcalloc((size_t)(nc > 0 ? nc : 1), 1);
    for (int32_t c = 0; c < nc; ++c) {
        if (size[c] < min_size) { ++too_small; continue; }
        if (size[c] > max_size) { ++too_large; continue; }
        if (lmin[c] * lmax[c] < 0.0 || lmax[c] / lmin[c] > cond_threshold) { keep[c] = 1; continue; }
        ++not_poor;
    }
    int32_t cnt = 0;
    for (int32_t a = 0; a < nsel; ++a)
        if (keep[comp[a]]) out[cnt++] = sel[a];
    if (counters) { counters[0] = too_small; counters[1] = too_large; counters[2] = not_poor; }
    free(g2l); free(comp); free(size); free(lmin); free(lmax); free(keep);
    return cnt;
}

int32_t lsso_expand_subdomains(int32_t n, const int32_t *outer, const int32_t *inner,
                               const int32_t *sel, int32_t nsel, int32_t *out)
{
    char *mark = (char *)xcalloc((size_t)(n > 0 ? n : 1), 1);
    for (int32_t a = 0; a < nsel; ++a) {
        int32_t k = sel[a];
        for (int32_t e = outer[k]; e < outer[k + 1]; ++e) mark[inner[e]] = 1;
    }
    int32_t cnt = 0;
    for (int32_t i = 0; i < n; ++i)
        if (mark[i]) out[cnt++] = i;
    free(mark);
    return cnt;
}

int32_t lsso_decompose_subdomains(int32_t n, const int32_t *outer, const int32_t *inner,
                                  const int32_t *sel, int32_t nsel, int32_t max_size,
                                  int32_t *offsets, int32_t *dofs)
{
    int32_t *g2l = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (int32_t i = 0; i < n; ++i) g2l[i] = -1;
    int32_t *comp = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nsel > 0 ? nsel : 1));
    int32_t nc = components(n, outer, inner, sel, nsel, g2l, comp);
    int32_t *size = (int32_t *)xcalloc((size_t)(nc > 0 ? nc : 1), sizeof(int32_t));
    for (int32_t a = 0; a < nsel; ++a) size[comp[a]]++;
    int32_t *start = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nc > 0 ? nc : 1));
    int32_t nout = 0, pos = 0;
    offsets[0] = 0;
    for (int32_t c = 0; c < nc; ++c) {
        if (size[c] > max_size) { start[c] = -1; continue; } /* GPUHybrid.cu:726-729 */
        start[c] = pos;
        pos += size[c];
        offsets[++nout] = pos;
    }
    for (int32_t a = 0; a < nsel; ++a) {
        int32_t c = comp[a];
        if (start[c] >= 0) dofs[start[c]++] = sel[a];
    }
    free(g2l); free(comp); free(size); free(start);
    return nout;
}

/* ===================================================================== */
/* Dense SPD helpers (packed upper, row major: MASPreconditioner.cu:484-491) */
/* ===================================================================== */

static inline int64_t upk(int64_t dim, int64_t i, int64_t j)
{
    if (i > j) { int64_t t = i; i = j; j = t; }
    return i * dim - (i * (i + 1) / 2) + j;
}

/* In-place inverse of a packed symmetric matrix by the symmetric sweep
 * (the Gauss-Jordan variant of MASPreconditioner.cu:799-900); returns 0 on a
 * zero or non-finite pivot.  Result is A^-1 (sign already restored). */
static int packed_sym_inverse(double *A, int dim)
{
    double *col = (double *)xmalloc(sizeof(double) * (size_t)dim);
    int ok = 1;
    for (int p = 0; p < dim; ++p) {
        double piv = A[upk(dim, p, p)];
        if (!isfinite(piv) || piv == 0.0) ok = 0;
        for (int t = 0; t < dim; ++t) col[t] = (t == p) ? 0.0 : A[upk(dim, t, p)];
        for (int t = 0; t < dim; ++t) {
            if (t == p) continue;
            double scale = col[t] / piv;
            for (int c = t; c < dim; ++c) {
                if (c == p) continue;
                A[upk(dim, t, c)] -= scale * col[c];
            }
        }
        A[upk(dim, p, p)] = -1.0 / piv;
        for (int t = 0; t < dim; ++t)
            if (t != p) A[upk(dim, t, p)] = col[t] / piv;
    }
    int64_t L = (int64_t)dim * (dim + 1) / 2;
    for (int64_t k = 0; k < L; ++k) {
        A[k] = -A[k];
        if (!isfinite(A[k])) ok = 0;
    }
    free(col);
    return ok;
}

/* y = A x for packed symmetric A */
static void packed_symv(const double *A, int dim, const double *x, double *y)
{
    for (int i = 0; i < dim; ++i) y[i] = 0.0;
    int64_t k = 0;
    for (int i = 0; i < dim; ++i) {
        double xi = x[i], acc = 0.0;
        for (int j = i; j < dim; ++j, ++k) {
            double a = A[k];
            acc += a * x[j];
            if (j != i) y[j] += a * xi;
        }
        y[i] += acc;
    }
}

/* ===================================================================== */
/* MAS (MASPreconditioner.cu)                                             */
/* ===================================================================== */

#define MAXLV 8

struct lsso_mas {
    int32_t nb, bd, nparts, levels; /* levels = matrix levels incl. level 0 */
    int32_t *part_offsets;          /* nparts+1 */
    int32_t *cmap[MAXLV];           /* cmap[m][i], m>=1: coarse id of block row i */
    int32_t nitems[MAXLV];          /* level 0: nparts*32; m>=1: CCO count */
    int32_t nbanks[MAXLV];
    int32_t N;                      /* 32*bd */
    int64_t S;                      /* N(N+1)/2 */
    double *inv[MAXLV];
};

/* Bank-local connected components over `items` grouped 32 per bank.
 * Edges given as pairs on item ids.  Components are numbered per bank by their
 * lowest lane (MASPreconditioner.cu:201-212) and globally by bank order
 * (prefix sum, :401-418). */
static int32_t bank_components(int32_t nitems, const int32_t *valid, int64_t nedges,
                               const int32_t *eu, const int32_t *ev, int32_t *out_id)
{
    int32_t nbank = (nitems + BANK - 1) / BANK;
    uint32_t *mask = (uint32_t *)xcalloc((size_t)(nitems > 0 ? nitems : 1), sizeof(uint32_t));
    for (int32_t t = 0; t < nitems; ++t) mask[t] = valid[t] ? (1u << (t % BANK)) : 0u;
    for (int64_t e = 0; e < nedges; ++e) {
        int32_t u = eu[e], v = ev[e];
        if (u / BANK != v / BANK || u == v) continue;
        mask[u] |= 1u << (v % BANK);
        mask[v] |= 1u << (u % BANK);
    }
    int32_t total = 0;
    for (int32_t b = 0; b < nbank; ++b) {
        int32_t lead_of[BANK];
        uint32_t leads = 0;
        for (int l = 0; l < BANK; ++l) {
            int32_t t = b * BANK + l;
            lead_of[l] = -1;
            if (t >= nitems || !valid[t]) continue;
            uint32_t conn = mask[t], visited = 1u << l, to_visit = conn ^ visited;
            while (to_visit) {
                int v = __builtin_ctz(to_visit);
                conn |= mask[b * BANK + v];
                visited |= 1u << v;
                to_visit = conn ^ visited;
            }
            lead_of[l] = __builtin_ctz(conn);
            if (lead_of[l] == l) leads |= 1u << l;
        }
        for (int l = 0; l < BANK; ++l) {
            int32_t t = b * BANK + l;
            if (t >= nitems || !valid[t]) continue;
            uint32_t before = (uint32_t)((1ull << lead_of[l]) - 1ull);
            out_id[t] = total + __builtin_popcount(leads & before);
        }
        total += __builtin_popcount(leads);
    }
    free(mask);
    return total;
}

lsso_mas *lsso_mas_create(int32_t nb, int32_t bd, const int32_t *rows, const int32_t *cols,
                          const double *vals, int32_t nparts, const int32_t *part_offsets,
                          int32_t max_coarse_levels, int32_t *status)
{
    if (status) *status = 0;
    if (bd < 1 || bd > 3 || nparts < 1 || part_offsets[nparts] != nb) {
        if (status) *status = 1;
        return NULL;
    }
    for (int32_t p = 0; p < nparts; ++p)
        if (part_offsets[p + 1] - part_offsets[p] > BANK || part_offsets[p + 1] < part_offsets[p]) {
            if (status) *status = 1;
            return NULL;
        }
    if (max_coarse_levels > MAXLV - 1) max_coarse_levels = MAXLV - 1;
    lsso_mas *m = (lsso_mas *)xcalloc(1, sizeof(lsso_mas));
    m->nb = nb; m->bd = bd; m->nparts = nparts;
    m->part_offsets = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nparts + 1));
    memcpy(m->part_offsets, part_offsets, sizeof(int32_t) * (size_t)(nparts + 1));
    m->N = BANK * bd;
    m->S = (int64_t)m->N * (m->N + 1) / 2;

    int32_t *part_of = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nb > 0 ? nb : 1));
    for (int32_t p = 0; p < nparts; ++p)
        for (int32_t i = part_offsets[p]; i < part_offsets[p + 1]; ++i) part_of[i] = p;

    /* off-diagonal pattern edges (block level) */
    int64_t nnzb = rows[nb];
    int32_t *eu = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nnzb > 0 ? nnzb : 1));
    int32_t *ev = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nnzb > 0 ? nnzb : 1));
    int32_t *tu = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nnzb > 0 ? nnzb : 1));
    int32_t *tv = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nnzb > 0 ? nnzb : 1));
    int64_t ne = 0;
    for (int32_t i = 0; i < nb; ++i)
        for (int32_t k = rows[i]; k < rows[i + 1]; ++k)
            if (cols[k] != i) { eu[ne] = i; ev[ne] = cols[k]; ++ne; }

    /* level 0 CCO: components inside each partition (MASPreconditioner.cu:128-213) */
    int32_t padded = nparts * BANK;
    int32_t *valid = (int32_t *)xcalloc((size_t)padded, sizeof(int32_t));
    int32_t *pid = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)padded);
    int32_t *real_to_padded = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nb > 0 ? nb : 1));
    for (int32_t p = 0; p < nparts; ++p)
        for (int32_t i = part_offsets[p]; i < part_offsets[p + 1]; ++i) {
            real_to_padded[i] = p * BANK + (i - part_offsets[p]);
            valid[real_to_padded[i]] = 1;
        }
    for (int64_t e = 0; e < ne; ++e) { tu[e] = real_to_padded[eu[e]]; tv[e] = real_to_padded[ev[e]]; }
    int32_t cnum = bank_components(padded, valid, ne, tu, tv, pid);
    m->nitems[0] = padded;
    m->nbanks[0] = nparts;
    m->cmap[1] = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nb > 0 ? nb : 1));
    for (int32_t i = 0; i < nb; ++i) m->cmap[1][i] = pid[real_to_padded[i]];
    m->nitems[1] = cnum;
    int32_t level_num = 1;
    free(valid); free(pid);

    /* coarser maps (MASPreconditioner.cu:424-474) */
    for (int32_t lv = 1; lv < max_coarse_levels; ++lv) {
        int32_t *prev = m->cmap[lv];
        int32_t pn = m->nitems[lv];
        int32_t *v2 = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(pn > 0 ? pn : 1));
        for (int32_t t = 0; t < pn; ++t) v2[t] = 1;
        for (int64_t e = 0; e < ne; ++e) { tu[e] = prev[eu[e]]; tv[e] = prev[ev[e]]; }
        int32_t *cid = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(pn > 0 ? pn : 1));
        int32_t next = bank_components(pn, v2, ne, tu, tv, cid);
        free(v2);
        if (next == pn) { free(cid); break; }
        m->cmap[lv + 1] = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nb > 0 ? nb : 1));
        for (int32_t i = 0; i < nb; ++i) m->cmap[lv + 1][i] = cid[prev[i]];
        m->nitems[lv + 1] = next;
        level_num = lv + 1;
        free(cid);
    }
    m->levels = 1 + level_num;
    for (int32_t l = 1; l < m->levels; ++l) m->nbanks[l] = (m->nitems[l] + BANK - 1) / BANK;

    /* Galerkin blocks (MASPreconditioner.cu:494-591), packed upper */
    const int32_t N = m->N;
    const int32_t bs = bd * bd;
    for (int32_t l = 0; l < m->levels; ++l)
        m->inv[l] = (double *)xcalloc((size_t)m->nbanks[l] * (size_t)m->S, sizeof(double));
    for (int32_t i = 0; i < nb; ++i) {
        for (int32_t k = rows[i]; k < rows[i + 1]; ++k) {
            int32_t j = cols[k];
            if (i > j) continue;
            const double *blk = vals + (int64_t)k * bs;
            if (part_of[i] == part_of[j]) {
                double *mat = m->inv[0] + (int64_t)part_of[i] * m->S;
                int32_t ri = (i - part_offsets[part_of[i]]) * bd, rj = (j - part_offsets[part_of[j]]) * bd;
                for (int bi = 0; bi < bd; ++bi)
                    for (int bj = 0; bj < bd; ++bj) {
                        int32_t row = ri + bi, col = rj + bj;
                        if (row > col) continue;
                        if (i == j && bi > bj) continue;
                        mat[upk(N, row, col)] += blk[bi * bd + bj];
                    }
            }
            for (int32_t l = 1; l < m->levels; ++l) {
                int32_t ci = m->cmap[l][i], cj = m->cmap[l][j];
                if (ci / BANK != cj / BANK) continue;
                double *mat = m->inv[l] + (int64_t)(ci / BANK) * m->S;
                int32_t ri = (ci % BANK) * bd, rj = (cj % BANK) * bd;
                for (int bi = 0; bi < bd; ++bi)
                    for (int bj = 0; bj < bd; ++bj) {
                        int32_t row = ri + bi, col = rj + bj;
                        if (row > col) continue;
                        if (i == j && bi > bj) continue;
                        double v = blk[bi * bd + bj];
                        if (i != j && ci == cj) v += blk[bj * bd + bi];
                        mat[upk(N, row, col)] += v;
                    }
            }
        }
    }
    /* pad zero diagonals (MASPreconditioner.cu:779-796) and invert (:799-936) */
    int ok = 1;
    for (int32_t l = 0; l < m->levels; ++l) {
        int32_t nbk = m->nbanks[l];
        int bad = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : bad)
        for (int32_t b = 0; b < nbk; ++b) {
            double *mat = m->inv[l] + (int64_t)b * m->S;
            for (int32_t d = 0; d < N; ++d)
                if (mat[upk(N, d, d)] == 0.0) mat[upk(N, d, d)] = 1.0;
            if (!packed_sym_inverse(mat, N)) bad |= 1;
        }
        if (bad) ok = 0;
    }
    free(part_of); free(eu); free(ev); free(tu); free(tv); free(real_to_padded);
    if (!ok && status) *status = 2;
    return m;
}

int32_t lsso_mas_level_count(const lsso_mas *m) { return m->levels; }
int32_t lsso_mas_level_items(const lsso_mas *m, int32_t l)
{
    if (l < 0 || l >= m->levels) return -1;
    return l == 0 ? m->nb : m->nitems[l];
}
void lsso_mas_coarse_map(const lsso_mas *m, int32_t l, int32_t *out)
{
    if (l < 1 || l >= m->levels) return;
    memcpy(out, m->cmap[l], sizeof(int32_t) * (size_t)m->nb);
}

/* MASPreconditioner::apply (MASPreconditioner.cu:1099-1164) */
void lsso_mas_apply(const lsso_mas *m, const double *r, double *z)
{
    const int32_t bd = m->bd, N = m->N, nb = m->nb;
    /* level 0: per-partition block (padded with zeros) */
#pragma omp parallel
    {
        double *x = (double *)xmalloc(sizeof(double) * (size_t)N);
        double *y = (double *)xmalloc(sizeof(double) * (size_t)N);
#pragma omp for schedule(static)
        for (int32_t p = 0; p < m->nparts; ++p) {
            int32_t b0 = m->part_offsets[p], sz = m->part_offsets[p + 1] - b0;
            for (int32_t t = 0; t < N; ++t) x[t] = 0.0;
            for (int32_t t = 0; t < sz * bd; ++t) x[t] = r[(int64_t)b0 * bd + t];
            packed_symv(m->inv[0] + (int64_t)p * m->S, N, x, y);
            for (int32_t t = 0; t < sz * bd; ++t) z[(int64_t)b0 * bd + t] = y[t];
        }
        free(x); free(y);
    }
    /* coarse levels: restrict (sum), invert, prolong (inject and add) */
    for (int32_t l = 1; l < m->levels; ++l) {
        int32_t items = m->nbanks[l] * BANK;
        double *rc = (double *)xcalloc((size_t)items * bd, sizeof(double));
        double *zc = (double *)xcalloc((size_t)items * bd, sizeof(double));
        const int32_t *map = m->cmap[l];
        for (int32_t i = 0; i < nb; ++i)
            for (int c = 0; c < bd; ++c) rc[(int64_t)map[i] * bd + c] += r[(int64_t)i * bd + c];
#pragma omp parallel for schedule(static)
        for (int32_t b = 0; b < m->nbanks[l]; ++b)
            packed_symv(m->inv[l] + (int64_t)b * m->S, N, rc + (int64_t)b * N, zc + (int64_t)b * N);
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < nb; ++i)
            for (int c = 0; c < bd; ++c) z[(int64_t)i * bd + c] += zc[(int64_t)map[i] * bd + c];
        free(rc); free(zc);
    }
}

void lsso_mas_destroy(lsso_mas *m)
{
    if (!m) return;
    free(m->part_offsets);
    for (int l = 0; l < MAXLV; ++l) { free(m->cmap[l]); free(m->inv[l]); }
    free(m);
}

/* ===================================================================== */
/* The library's partition, restated: recursive breadth-first bisection   */
/* into k = ceil(m / 30) connected, bank-aligned parts of <= 32 block rows */
/* (the product's csrc/partition.cpp; it stands in for KaMinPar,          */
/* GraphPartition.cpp:176-289).  Restated here so that the CPU method runs */
/* with the GPU's partition without loading the product library; the CPU  */
/* tests require the two to agree exactly.                                */
/* ===================================================================== */
typedef struct {
    const int32_t *rows, *cols;
    int32_t *owner, *seen;
    int32_t next_task, next_stamp;
    int32_t **parts;
    int32_t *part_len;
} bp_ctx;

typedef struct { int32_t *v; int32_t n, cap; } ivec;

static void iv_push(ivec *a, int32_t x)
{
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 16;
        a->v = (int32_t *)realloc(a->v, sizeof(int32_t) * (size_t)a->cap);
    }
    a->v[a->n++] = x;
}

/* breadth-first order of `nodes` (owned by task) from `start`, restarting at
 * the next unvisited node of `nodes` for disconnected pieces */
static void bp_bfs(bp_ctx *c, int32_t task, const int32_t *nodes, int32_t m, int32_t start, int32_t *order)
{
    const int32_t stamp = c->next_stamp++;
    int32_t len = 0, head = 0, scan = 0, s = start;
    for (;;) {
        if (c->seen[s] != stamp) {
            c->seen[s] = stamp;
            order[len++] = s;
            while (head < len) {
                const int32_t u = order[head++];
                for (int32_t k = c->rows[u]; k < c->rows[u + 1]; ++k) {
                    const int32_t v = c->cols[k];
                    if (c->owner[v] == task && c->seen[v] != stamp) {
                        c->seen[v] = stamp;
                        order[len++] = v;
                    }
                }
            }
        }
        while (scan < m && c->seen[nodes[scan]] == stamp) ++scan;
        if (scan == m) break;
        s = nodes[scan];
    }
}

/* connected components of `nodes` (owned by task), in order of first node:
 * flat[] holds them one after the other, off[] their offsets; returns the count */
static int32_t bp_components(bp_ctx *c, int32_t task, const int32_t *nodes, int32_t m, int32_t *flat, int32_t *off)
{
    const int32_t stamp = c->next_stamp++;
    int32_t nc = 0, len = 0;
    off[0] = 0;
    for (int32_t i = 0; i < m; ++i) {
        const int32_t s = nodes[i];
        if (c->seen[s] == stamp) continue;
        int32_t h = len;
        flat[len++] = s;
        c->seen[s] = stamp;
        for (; h < len; ++h) {
            const int32_t u = flat[h];
            for (int32_t k = c->rows[u]; k < c->rows[u + 1]; ++k) {
                const int32_t v = c->cols[k];
                if (c->owner[v] == task && c->seen[v] != stamp) {
                    c->seen[v] = stamp;
                    flat[len++] = v;
                }
            }
        }
        off[++nc] = len;
    }
    return nc;
}

/* parts in the left child of a subtree with k leaves: a multiple of the
 * largest power of 32 below k */
static int32_t bp_left_parts(int32_t k)
{
    int64_t B = 1;
    while (B * 32 < k) B *= 32;
    const int64_t g = (k + B - 1) / B;
    int64_t k1 = (g / 2) * B;
    if (k1 <= 0 || k1 >= k) k1 = k / 2;
    return (int32_t)k1;
}

static void bp_split(bp_ctx *c, int32_t task, int32_t *nodes, int32_t m, int32_t part0, int32_t k)
{
    if (k <= 1 || m <= 1) {
        int32_t *o = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)m);
        if (m > 1) {
            bp_bfs(c, task, nodes, m, nodes[0], o);
            const int32_t last = o[m - 1];
            bp_bfs(c, task, nodes, m, last, o);
        } else {
            memcpy(o, nodes, sizeof(int32_t) * (size_t)m);
        }
        c->parts[part0] = o;
        c->part_len[part0] = m;
        free(nodes);
        return;
    }
    const int32_t k1 = bp_left_parts(k), k2 = k - k1;
    int64_t m1 = ((int64_t)m * k1 + k / 2) / k;
    if (m1 < (int64_t)m - 32 * (int64_t)k2) m1 = (int64_t)m - 32 * (int64_t)k2;
    if (m1 > 32 * (int64_t)k1) m1 = 32 * (int64_t)k1;
    if (m1 > m - 1) m1 = m - 1;
    if (m1 < 1) m1 = 1;
    int32_t *order = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)m);
    bp_bfs(c, task, nodes, m, nodes[0], order);
    const int32_t last = order[m - 1];
    bp_bfs(c, task, nodes, m, last, order);
    free(nodes);
    const int32_t tl = c->next_task++, tr = c->next_task++;
    ivec left = {0, 0, 0}, right = {0, 0, 0};
    for (int32_t i = 0; i < m; ++i) iv_push(i < m1 ? &left : &right, order[i]);
    free(order);
    for (int32_t i = 0; i < left.n; ++i) c->owner[left.v[i]] = tl;
    for (int32_t i = 0; i < right.n; ++i) c->owner[right.v[i]] = tr;
    /* reconnect the right side: swap its small pieces with the prefix's tail */
    for (int round = 0; round < 4; ++round) {
        int32_t *flat = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(right.n + 1));
        int32_t *off = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(right.n + 2));
        const int32_t nc = bp_components(c, tr, right.v, right.n, flat, off);
        if (nc <= 1) { free(flat); free(off); break; }
        int32_t big = 0;
        for (int32_t q = 1; q < nc; ++q)
            if (off[q + 1] - off[q] > off[big + 1] - off[big]) big = q;
        const int32_t npieces = right.n - (off[big + 1] - off[big]);
        if (npieces >= left.n) { free(flat); free(off); break; }
        /* the last nodes of the prefix go right, the pieces go left */
        int32_t *moved = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)npieces);
        memcpy(moved, left.v + left.n - npieces, sizeof(int32_t) * (size_t)npieces);
        left.n -= npieces;
        for (int32_t q = 0; q < nc; ++q) {
            if (q == big) continue;
            for (int32_t t = off[q]; t < off[q + 1]; ++t) {
                c->owner[flat[t]] = tl;
                iv_push(&left, flat[t]);
            }
        }
        for (int32_t t = 0; t < npieces; ++t) c->owner[moved[t]] = tr;
        right.n = 0;
        for (int32_t t = off[big]; t < off[big + 1]; ++t) iv_push(&right, flat[t]);
        for (int32_t t = 0; t < npieces; ++t) iv_push(&right, moved[t]);
        free(moved); free(flat); free(off);
    }
    bp_split(c, tl, left.v, left.n, part0, k1);
    bp_split(c, tr, right.v, right.n, part0 + k1, k2);
}

int32_t lsso_bisect_partition(int32_t nb, const int32_t *rows, const int32_t *cols, int32_t *perm,
                              int32_t *part_offsets)
{
    part_offsets[0] = 0;
    if (nb <= 0) return 0;
    bp_ctx c;
    c.rows = rows;
    c.cols = cols;
    c.owner = (int32_t *)xcalloc((size_t)nb, sizeof(int32_t));
    c.seen = (int32_t *)xcalloc((size_t)nb, sizeof(int32_t));
    c.next_task = 1;
    c.next_stamp = 1;
    int32_t *coupled = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)nb);
    int32_t *isolated = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)nb);
    int32_t m = 0, ni = 0;
    for (int32_t i = 0; i < nb; ++i) {
        int any = 0;
        for (int32_t q = rows[i]; q < rows[i + 1] && !any; ++q) any = cols[q] != i;
        if (any) coupled[m++] = i;
        else isolated[ni++] = i;
    }
    for (int32_t t = 0; t < ni; ++t) c.owner[isolated[t]] = -1;
    const int32_t k = m == 0 ? 0 : (m <= 32 ? 1 : (m + 29) / 30);
    c.parts = (int32_t **)xcalloc((size_t)(k > 0 ? k : 1), sizeof(int32_t *));
    c.part_len = (int32_t *)xcalloc((size_t)(k > 0 ? k : 1), sizeof(int32_t));
    if (k > 0) bp_split(&c, 0, coupled, m, 0, k);
    else free(coupled);
    int32_t next = 0, np = 0;
    for (int32_t p = 0; p < k; ++p) {
        const int32_t len = c.part_len[p];
        /* a leaf larger than a bank (possible only after the reconnect swaps) is cut in BFS order */
        for (int32_t s0 = 0; s0 < len; s0 += 32) {
            const int32_t e = s0 + 32 < len ? s0 + 32 : len;
            for (int32_t q = s0; q < e; ++q) perm[c.parts[p][q]] = next++;
            part_offsets[++np] = next;
        }
        free(c.parts[p]);
    }
    for (int32_t s0 = 0; s0 < ni; s0 += 32) {
        const int32_t e = s0 + 32 < ni ? s0 + 32 : ni;
        for (int32_t q = s0; q < e; ++q) perm[isolated[q]] = next++;
        part_offsets[++np] = next;
    }
    free(isolated); free(c.parts); free(c.part_len); free(c.owner); free(c.seen);
    return np;
}

/* ===================================================================== */
/* Oracle partition: greedy BFS region growing into parts of <= max_part   */
/* (a simple, independent stand-in for KaMinPar, GraphPartition.cpp:176)  */
/* ===================================================================== */
int32_t lsso_greedy_partition(int32_t nb, const int32_t *rows, const int32_t *cols,
                              int32_t max_part, int32_t *part_of)
{
    for (int32_t i = 0; i < nb; ++i) part_of[i] = -1;
    int32_t *order = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nb > 0 ? nb : 1));
    char *seen = (char *)xcalloc((size_t)(nb > 0 ? nb : 1), 1);
    /* global BFS order gives the seed sequence (locality of part ids) */
    int32_t head = 0, tail = 0;
    for (int32_t s = 0; s < nb; ++s) {
        if (seen[s]) continue;
        seen[s] = 1; order[tail++] = s;
        while (head < tail) {
            int32_t u = order[head++];
            for (int32_t k = rows[u]; k < rows[u + 1]; ++k) {
                int32_t v = cols[k];
                if (!seen[v]) { seen[v] = 1; order[tail++] = v; }
            }
        }
    }
    int32_t *q = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nb > 0 ? nb : 1));
    int32_t np = 0;
    for (int32_t o = 0; o < nb; ++o) {
        int32_t s = order[o];
        if (part_of[s] >= 0) continue;
        int32_t qh = 0, qt = 0, size = 0;
        part_of[s] = np; q[qt++] = s; ++size;
        while (qh < qt && size < max_part) {
            int32_t u = q[qh++];
            for (int32_t k = rows[u]; k < rows[u + 1] && size < max_part; ++k) {
                int32_t v = cols[k];
                if (part_of[v] < 0) { part_of[v] = np; q[qt++] = v; ++size; }
            }
        }
        ++np;
    }
    free(order); free(seen); free(q);
    return np;
}

/* ===================================================================== */
/* Full CPU method                                                          */
/* ===================================================================== */

size_t lsso_params_size(void) { return sizeof(lsso_params); }

void lsso_default_params(lsso_params *p)
{
    /* linear-solver-spec.json defaults for /GPUHybrid (spec:646-747) */
    p->max_iter = 10000;
    p->rel_tol = 1e-10;
    p->abs_tol = 0.0;
    p->block_size = 1;
    p->do_hybrid = 1;
    p->select_from_l1 = 1;
    p->jump_threshold = 100.0;
    p->gmm_tol = 1e-3;
    p->max_gmm_iterations = 20;
    p->cond_threshold = 100.0;
    p->decompose = 1;
    p->min_sub = 1;
    p->max_sub = 10000000;
    p->expand = 1;
    p->max_coarse_levels = 4;
    p->threads = 0;
    p->additive = 0;
    p->mas_omega = 0.0;
    p->omega_iters = 20;
    p->omega_factor = 1.5;
    p->greedy_partition = 0;
}

void lsso_probe_vector(int32_t n, double *v)
{
    for (int32_t i = 0; i < n; ++i) {
        uint32_t h = (uint32_t)((uint64_t)(uint32_t)i * 2654435761u);
        v[i] = (double)h / 4294967296.0 - 0.5;
    }
}

static int32_t sturm_count(int32_t k, const double *d, const double *e, double x)
{
    int32_t cnt = 0;
    double q = d[0] - x;
    if (q < 0) ++cnt;
    for (int32_t j = 1; j < k; ++j) {
        if (q == 0.0) q = 1e-300;
        q = d[j] - x - e[j - 1] * e[j - 1] / q;
        if (q < 0) ++cnt;
    }
    return cnt;
}

double lsso_tridiag_max_eig(int32_t k, const double *d, const double *e)
{
    if (k <= 0) return 0.0;
    double lo = d[0], hi = d[0];
    for (int32_t j = 0; j < k; ++j) {
        double r = (j > 0 ? fabs(e[j - 1]) : 0.0) + (j + 1 < k ? fabs(e[j]) : 0.0);
        if (d[j] - r < lo) lo = d[j] - r;
        if (d[j] + r > hi) hi = d[j] + r;
    }
    for (int it = 0; it < 200 && hi - lo > 1e-14 * fabs(hi); ++it) {
        double mid = 0.5 * (lo + hi);
        if (sturm_count(k, d, e, mid) >= k) hi = mid; else lo = mid;
    }
    return hi;
}

typedef struct {
    int32_t m;
    int32_t *dofs;   /* original scalar ids, ascending */
    double *chol;    /* m x m lower Cholesky factor, row major */
} stiff_block;

struct lsso_solver {
    double omega, lambda_max;
    int32_t n, bd, nb;
    const int32_t *outer, *inner;
    const double *values;
    lsso_params p;
    int32_t *perm, *iperm; /* block old->new, new->old */
    lsso_mas *mas;
    int32_t nsub, nstiff;
    stiff_block *sub;
    double *t0, *t1, *t2, *t3, *t4; /* work vectors */
};

static double estimate_lambda_max(lsso_solver *s, int32_t k);

static void csr_spmv(int32_t n, const int32_t *outer, const int32_t *inner, const double *v,
                     const double *x, double *y)
{
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int32_t k = outer[i]; k < outer[i + 1]; ++k) s += v[k] * x[inner[k]];
        y[i] = s;
    }
}

static double dotv(int32_t n, const double *a, const double *b)
{
    double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
    for (int32_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* dense Cholesky, lower, row major; 0 on failure */
static int dense_cholesky(double *A, int32_t m)
{
    for (int32_t j = 0; j < m; ++j) {
        double d = A[(int64_t)j * m + j];
        for (int32_t k = 0; k < j; ++k) d -= A[(int64_t)j * m + k] * A[(int64_t)j * m + k];
        if (!(d > 0.0) || !isfinite(d)) return 0;
        d = sqrt(d);
        A[(int64_t)j * m + j] = d;
#pragma omp parallel for schedule(static) if (m > 256)
        for (int32_t i = j + 1; i < m; ++i) {
            double s = A[(int64_t)i * m + j];
            for (int32_t k = 0; k < j; ++k) s -= A[(int64_t)i * m + k] * A[(int64_t)j * m + k];
            A[(int64_t)i * m + j] = s / d;
        }
    }
    return 1;
}

static void chol_solve(const double *L, int32_t m, double *x)
{
    for (int32_t i = 0; i < m; ++i) {
        double s = x[i];
        for (int32_t k = 0; k < i; ++k) s -= L[(int64_t)i * m + k] * x[k];
        x[i] = s / L[(int64_t)i * m + i];
    }
    for (int32_t i = m - 1; i >= 0; --i) {
        double s = x[i];
        for (int32_t k = i + 1; k < m; ++k) s -= L[(int64_t)k * m + i] * x[k];
        x[i] = s / L[(int64_t)i * m + i];
    }
}

static int32_t find_sorted(const int32_t *a, int32_t m, int32_t v)
{
    int32_t lo = 0, hi = m;
    while (lo < hi) {
        int32_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return (lo < m && a[lo] == v) ? lo : -1;
}

lsso_solver *lsso_solver_create(int32_t n, const int32_t *outer, const int32_t *inner,
                                const double *values, const lsso_params *p,
                                const int32_t *perm_in, int32_t nparts_in,
                                const int32_t *part_offsets_in, int32_t *status)
{
    if (status) *status = 0;
    int32_t bd = p->block_size;
    if (bd < 1 || bd > 3 || n <= 0 || n % bd) { if (status) *status = 1; return NULL; }
#ifdef _OPENMP
    if (p->threads > 0) omp_set_num_threads(p->threads);
#endif
    lsso_solver *s = (lsso_solver *)xcalloc(1, sizeof(lsso_solver));
    s->n = n; s->bd = bd; s->nb = n / bd;
    s->outer = outer; s->inner = inner; s->values = values;
    s->p = *p;
    const int32_t nb = s->nb;

    /* ---- stiff DOFs: GPUHybrid::factorize, GPUHybrid.cu:214-264 ---- */
    int32_t *sel = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)n);
    int32_t nsel = 0;
    if (p->do_hybrid && p->select_from_l1) {
        double *rn = (double *)xmalloc(sizeof(double) * (size_t)n);
        lsso_row_l1_norms(n, outer, values, rn);
        nsel = lsso_gmm_select(n, rn, p->jump_threshold, p->gmm_tol, p->max_gmm_iterations, sel, NULL);
        free(rn);
    }
    int32_t *tmp = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)n);
    if (p->do_hybrid && p->decompose) {
        nsel = lsso_filter_subdomains(n, outer, inner, values, sel, nsel, p->min_sub, p->max_sub,
                                      p->cond_threshold, tmp, NULL);
        memcpy(sel, tmp, sizeof(int32_t) * (size_t)nsel);
    }
    if (p->do_hybrid && p->expand && nsel > 0) {
        nsel = lsso_expand_subdomains(n, outer, inner, sel, nsel, tmp);
        memcpy(sel, tmp, sizeof(int32_t) * (size_t)nsel);
    }
    int32_t *offs = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(n + 1));
    int32_t nsub = 0;
    if (p->do_hybrid && nsel > 0) {
        /* With decompose_subdomains=false the reference factors one block holding
         * every selected DOF; its inverse is block diagonal over the connected
         * components, so factoring the components separately is the same operator. */
        nsub = lsso_decompose_subdomains(n, outer, inner, sel, nsel,
                                         p->decompose ? p->max_sub : 0x7fffffff, offs, tmp);
    }
    s->nsub = nsub;
    s->sub = (stiff_block *)xcalloc((size_t)(nsub > 0 ? nsub : 1), sizeof(stiff_block));
    s->nstiff = 0;
    int fail = 0;
    for (int32_t c = 0; c < nsub; ++c) {
        stiff_block *sb = &s->sub[c];
        sb->m = offs[c + 1] - offs[c];
        s->nstiff += sb->m;
        sb->dofs = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)sb->m);
        memcpy(sb->dofs, tmp + offs[c], sizeof(int32_t) * (size_t)sb->m);
        sb->chol = (double *)xcalloc((size_t)sb->m * (size_t)sb->m, sizeof(double));
        /* A_SS extraction, GPUHybrid.cu:1147-1196 (outer slice = row) */
        for (int32_t r = 0; r < sb->m; ++r) {
            int32_t g = sb->dofs[r];
            for (int32_t k = outer[g]; k < outer[g + 1]; ++k) {
                int32_t c2 = find_sorted(sb->dofs, sb->m, inner[k]);
                if (c2 >= 0) sb->chol[(int64_t)r * sb->m + c2] = values[k];
            }
        }
        if (!dense_cholesky(sb->chol, sb->m)) fail = 1;
    }
    free(sel); free(tmp); free(offs);
    if (fail) { if (status) *status = 3; }

    /* ---- partition + permuted BSR + MAS ---- */
    s->perm = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)nb);
    s->iperm = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)nb);
    /* block graph of the scalar pattern */
    int32_t *brow = (int32_t *)xcalloc((size_t)nb + 1, sizeof(int32_t));
    int32_t *bcol = NULL;
    {
        int32_t *mark = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)nb);
        for (int32_t i = 0; i < nb; ++i) mark[i] = -1;
        int64_t cnt = 0;
        for (int32_t bi = 0; bi < nb; ++bi) {
            for (int32_t c = 0; c < bd; ++c)
                for (int32_t k = outer[bi * bd + c]; k < outer[bi * bd + c + 1]; ++k) {
                    int32_t bj = inner[k] / bd;
                    if (mark[bj] != bi) { mark[bj] = bi; ++cnt; }
                }
            brow[bi + 1] = (int32_t)cnt;
        }
        bcol = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(cnt > 0 ? cnt : 1));
        for (int32_t i = 0; i < nb; ++i) mark[i] = -1;
        int64_t pos = 0;
        for (int32_t bi = 0; bi < nb; ++bi) {
            int64_t start = pos;
            for (int32_t c = 0; c < bd; ++c)
                for (int32_t k = outer[bi * bd + c]; k < outer[bi * bd + c + 1]; ++k) {
                    int32_t bj = inner[k] / bd;
                    if (mark[bj] != bi) { mark[bj] = bi; bcol[pos++] = bj; }
                }
            qsort(bcol + start, (size_t)(pos - start), sizeof(int32_t), cmp_i32);
        }
        free(mark);
    }
    int32_t nparts;
    int32_t *poff;
    if (perm_in && part_offsets_in) {
        memcpy(s->perm, perm_in, sizeof(int32_t) * (size_t)nb);
        nparts = nparts_in;
        poff = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nparts + 1));
        memcpy(poff, part_offsets_in, sizeof(int32_t) * (size_t)(nparts + 1));
    } else if (!p->greedy_partition) {
        poff = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nb + 2));
        nparts = lsso_bisect_partition(nb, brow, bcol, s->perm, poff);
    } else {
        int32_t *part_of = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)nb);
        nparts = lsso_greedy_partition(nb, brow, bcol, BANK, part_of);
        /* MASSolver.cu:90-118: offsets then stable placement */
        poff = (int32_t *)xcalloc((size_t)nparts + 1, sizeof(int32_t));
        for (int32_t i = 0; i < nb; ++i) poff[part_of[i] + 1]++;
        for (int32_t q = 0; q < nparts; ++q) poff[q + 1] += poff[q];
        int32_t *next = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nparts + 1));
        memcpy(next, poff, sizeof(int32_t) * (size_t)(nparts + 1));
        for (int32_t i = 0; i < nb; ++i) s->perm[i] = next[part_of[i]]++;
        free(next); free(part_of);
    }
    for (int32_t i = 0; i < nb; ++i) s->iperm[s->perm[i]] = i;
    /* permuted BSR, blocks row major: block (I,J)[bi][bj] = A[(I*bd+bi), (J*bd+bj)] */
    int32_t *prow = (int32_t *)xcalloc((size_t)nb + 1, sizeof(int32_t));
    for (int32_t I = 0; I < nb; ++I) {
        int32_t o = s->iperm[I];
        prow[I + 1] = prow[I] + (brow[o + 1] - brow[o]);
    }
    int64_t nnzb = prow[nb];
    int32_t *pcol = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nnzb > 0 ? nnzb : 1));
    double *pval = (double *)xcalloc((size_t)(nnzb > 0 ? nnzb : 1) * bd * bd, sizeof(double));
    {
        int32_t *slot = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)nb);
        for (int32_t i = 0; i < nb; ++i) slot[i] = -1;
        for (int32_t I = 0; I < nb; ++I) {
            int32_t o = s->iperm[I];
            int32_t cnt = brow[o + 1] - brow[o];
            /* new column ids, sorted */
            for (int32_t t = 0; t < cnt; ++t) pcol[prow[I] + t] = s->perm[bcol[brow[o] + t]];
            qsort(pcol + prow[I], (size_t)cnt, sizeof(int32_t), cmp_i32);
            for (int32_t t = 0; t < cnt; ++t) slot[s->iperm[pcol[prow[I] + t]]] = prow[I] + t;
            for (int32_t c = 0; c < bd; ++c)
                for (int32_t k = outer[o * bd + c]; k < outer[o * bd + c + 1]; ++k) {
                    int32_t col = inner[k];
                    int32_t sl = slot[col / bd];
                    pval[(int64_t)sl * bd * bd + c * bd + (col % bd)] += values[k];
                }
            for (int32_t t = 0; t < cnt; ++t) slot[bcol[brow[o] + t]] = -1;
        }
        free(slot);
    }
    int32_t mst = 0;
    s->mas = lsso_mas_create(nb, bd, prow, pcol, pval, nparts, poff, p->max_coarse_levels, &mst);
    if (mst && status) *status = 4;
    free(prow); free(pcol); free(pval); free(poff); free(brow); free(bcol);
    s->t0 = (double *)xcalloc((size_t)n, sizeof(double));
    s->t1 = (double *)xcalloc((size_t)n, sizeof(double));
    s->t2 = (double *)xcalloc((size_t)n, sizeof(double));
    s->t3 = (double *)xcalloc((size_t)n, sizeof(double));
    s->t4 = (double *)xcalloc((size_t)n, sizeof(double));
    s->omega = 1.0;
    s->lambda_max = 0.0;
    if (p->do_hybrid && s->nstiff > 0 && !p->additive) {
        if (p->mas_omega > 0) s->omega = p->mas_omega;
        else {
            s->lambda_max = estimate_lambda_max(s, p->omega_iters);
            if (s->lambda_max > 0) s->omega = p->omega_factor / s->lambda_max;
        }
    }
    return s;
}

int32_t lsso_solver_num_stiff(const lsso_solver *s) { return s->nstiff; }
double lsso_solver_omega(const lsso_solver *s) { return s->omega; }
void lsso_solver_set_max_iter(lsso_solver *s, int32_t max_iter) { s->p.max_iter = max_iter; }
double lsso_solver_lambda_max(const lsso_solver *s) { return s->lambda_max; }
int32_t lsso_solver_num_subdomains(const lsso_solver *s) { return s->nsub; }

/* MAS in the original ordering */
static void mas_orig(lsso_solver *s, const double *r, double *z)
{
    const int32_t bd = s->bd, nb = s->nb;
    double *rp = s->t3, *zp = s->t4;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < nb; ++i)
        for (int c = 0; c < bd; ++c) rp[(int64_t)s->perm[i] * bd + c] = r[(int64_t)i * bd + c];
    lsso_mas_apply(s->mas, rp, zp);
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < nb; ++i)
        for (int c = 0; c < bd; ++c) z[(int64_t)i * bd + c] = zp[(int64_t)s->perm[i] * bd + c];
}

/* custom_mixed_precond_iter (GPUHybrid.cu:521-542) with dss_precond_iter
 * (:544-675), MAS in place of one BoomerAMG V-cycle:
 *   z1 = w M r;  z2 = z1 + S^T A_SS^-1 S (r - A z1);  z = z2 + w M (r - A z2).
 * The symmetric product is positive definite only when I - w M A is a
 * contraction in the A-norm (a V-cycle is; additive MAS, whose
 * lambda_max(M A) grows with the level count, is not), hence the damping
 * w = omega_factor / lambda_max(M A).  additive: z = M r + S^T A_SS^-1 S r
 * (MASSolver.cu:583-615). */
static void stiff_correct(lsso_solver *s, const double *r, const double *z, double *z2, int residual)
{
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t c = 0; c < s->nsub; ++c) {
        stiff_block *sb = &s->sub[c];
        double *t = (double *)xmalloc(sizeof(double) * (size_t)sb->m);
        for (int32_t a = 0; a < sb->m; ++a) {
            int32_t g = sb->dofs[a];
            double acc = 0.0;
            if (residual)
                for (int32_t k = s->outer[g]; k < s->outer[g + 1]; ++k) acc += s->values[k] * z[s->inner[k]];
            t[a] = r[g] - acc;
        }
        chol_solve(sb->chol, sb->m, t);
        for (int32_t a = 0; a < sb->m; ++a) z2[sb->dofs[a]] = z[sb->dofs[a]] + t[a];
        free(t);
    }
}

void lsso_solver_precond(lsso_solver *s, const double *r, double *z)
{
    const int32_t n = s->n;
    if (!s->p.do_hybrid || s->nstiff == 0) {
        mas_orig(s, r, z);
        return;
    }
    double *z2 = s->t0, *w = s->t1, *az = s->t2;
    if (s->p.additive) {
        mas_orig(s, r, z);
        memcpy(z2, z, sizeof(double) * (size_t)n);
        stiff_correct(s, r, z, z2, 0);  /* z2 = M r + S^T A_SS^-1 S r */
        memcpy(z, z2, sizeof(double) * (size_t)n);
        (void)w;
        return;
    }
    const double om = s->omega;
    mas_orig(s, r, z);
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < n; ++i) z[i] *= om;   /* z = z1 */
    memcpy(z2, z, sizeof(double) * (size_t)n);
    stiff_correct(s, r, z, z2, 1);
    csr_spmv(n, s->outer, s->inner, s->values, z2, az);
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < n; ++i) w[i] = r[i] - az[i];
    mas_orig(s, w, z);
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < n; ++i) z[i] = z2[i] + om * z[i];
}

/* lambda_max(M A) from the Lanczos tridiagonal of omega_iters PCG steps with
 * M = MAS on the probe vector (CG coefficients give T: diagonal
 * 1/a_j + b_{j-1}/a_{j-1}, off-diagonal sqrt(b_j)/a_j). */
static double estimate_lambda_max(lsso_solver *s, int32_t k)
{
    const int32_t n = s->n;
    double *b = (double *)xmalloc(sizeof(double) * (size_t)n);
    double *r = (double *)xmalloc(sizeof(double) * (size_t)n);
    double *z = (double *)xmalloc(sizeof(double) * (size_t)n);
    double *pv = (double *)xmalloc(sizeof(double) * (size_t)n);
    double *ap = (double *)xmalloc(sizeof(double) * (size_t)n);
    double *al = (double *)xcalloc((size_t)k + 1, sizeof(double));
    double *be = (double *)xcalloc((size_t)k + 1, sizeof(double));
    lsso_probe_vector(n, b);
    memcpy(r, b, sizeof(double) * (size_t)n);
    mas_orig(s, r, z);
    memcpy(pv, z, sizeof(double) * (size_t)n);
    double g = dotv(n, r, z);
    int32_t m = 0;
    for (int32_t j = 0; j < k; ++j) {
        csr_spmv(n, s->outer, s->inner, s->values, pv, ap);
        double pap = dotv(n, pv, ap);
        if (!(pap > 0)) break;
        double a = g / pap;
        al[m] = a;
        for (int32_t i = 0; i < n; ++i) r[i] -= a * ap[i];
        mas_orig(s, r, z);
        double gn = dotv(n, r, z);
        be[m] = gn / g;
        ++m;
        if (!(gn > 0)) break;
        for (int32_t i = 0; i < n; ++i) pv[i] = z[i] + be[m - 1] * pv[i];
        g = gn;
    }
    double *d = (double *)xcalloc((size_t)m + 1, sizeof(double));
    double *e = (double *)xcalloc((size_t)m + 1, sizeof(double));
    for (int32_t j = 0; j < m; ++j) {
        d[j] = 1.0 / al[j] + (j > 0 ? be[j - 1] / al[j - 1] : 0.0);
        if (j + 1 < m) e[j] = sqrt(be[j]) / al[j];
    }
    double lam = lsso_tridiag_max_eig(m, d, e);
    free(b); free(r); free(z); free(pv); free(ap); free(al); free(be); free(d); free(e);
    return lam;
}

/* GPUHybrid::pcg_solve (GPUHybrid.cu:1413-1512) + final residual (:383-386) */
int32_t lsso_solver_solve(lsso_solver *s, const double *b, double *x, int32_t *iterations,
                          double *final_res_norm)
{
    const int32_t n = s->n;
    double *r = (double *)xmalloc(sizeof(double) * (size_t)n);
    double *pv = (double *)xmalloc(sizeof(double) * (size_t)n);
    double *z = (double *)xcalloc((size_t)n, sizeof(double));
    double *ap = (double *)xmalloc(sizeof(double) * (size_t)n);
    int32_t iters = 0, code = 0;
    double bb = dotv(n, b, b);
    if (!(bb > 0.0)) {
        memset(x, 0, sizeof(double) * (size_t)n);
        if (iterations) *iterations = 0;
        if (final_res_norm) *final_res_norm = 0.0;
        free(r); free(pv); free(z); free(ap);
        return 0;
    }
    double rel_eps = s->p.rel_tol * s->p.rel_tol, abs_eps = s->p.abs_tol * s->p.abs_tol;
    csr_spmv(n, s->outer, s->inner, s->values, x, ap);
    for (int32_t i = 0; i < n; ++i) r[i] = b[i] - ap[i];
    lsso_solver_precond(s, r, z);
    memcpy(pv, z, sizeof(double) * (size_t)n);
    double gamma = dotv(n, r, z), old_gamma = gamma;
    for (int32_t k = 0; k < s->p.max_iter; ++k) {
        iters = k + 1;
        csr_spmv(n, s->outer, s->inner, s->values, pv, ap);
        double sdotp = dotv(n, pv, ap);
        if (sdotp == 0.0) { code = 1; break; }
        double alpha = gamma / sdotp;
        if (alpha <= 0.0) { code = 2; break; }
        if (alpha < DBL_MIN) { code = 3; break; }
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < n; ++i) { x[i] += alpha * pv[i]; r[i] -= alpha * ap[i]; }
        double rr = dotv(n, r, r);
        if (rel_eps > 0 && rr / bb < rel_eps) { code = 10; break; }
        if (abs_eps > 0 && rr < abs_eps) { code = 11; break; }
        lsso_solver_precond(s, r, z);
        gamma = dotv(n, r, z);
        double beta = gamma / old_gamma;
        old_gamma = gamma;
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < n; ++i) pv[i] = beta * pv[i] + z[i];
    }
    csr_spmv(n, s->outer, s->inner, s->values, x, ap);
    for (int32_t i = 0; i < n; ++i) ap[i] -= b[i];
    if (iterations) *iterations = iters;
    if (final_res_norm) *final_res_norm = sqrt(dotv(n, ap, ap));
    free(r); free(pv); free(z); free(ap);
    return code;
}

void lsso_solver_destroy(lsso_solver *s)
{
    if (!s) return;
    for (int32_t c = 0; c < s->nsub; ++c) { free(s->sub[c].dofs); free(s->sub[c].chol); }
    free(s->sub);
    lsso_mas_destroy(s->mas);
    free(s->perm); free(s->iperm);
    free(s->t0); free(s->t1); free(s->t2); free(s->t3); free(s->t4);
    free(s);
}

/* ===================================================================== */
/* MAS-side bad-DOF selections                                            */
/* ===================================================================== */

/* index sort by value with ties broken by index (qsort: single-threaded use) */
static const double *g_key;
static int g_desc;
static int cmp_by_key(const void *a, const void *b)
{
    const int32_t i = *(const int32_t *)a, j = *(const int32_t *)b;
    const double x = g_key[i], y = g_key[j];
    if (x < y) return g_desc ? 1 : -1;
    if (x > y) return g_desc ? -1 : 1;
    return (i > j) - (i < j);
}
static int32_t *sorted_positions(int32_t n, const double *key, int desc)
{
    int32_t *order = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (int32_t i = 0; i < n; ++i) order[i] = i;
    g_key = key;
    g_desc = desc;
    qsort(order, (size_t)n, sizeof(int32_t), cmp_by_key);
    return order;
}

/* positions of `hit` (visited in `visit` order), each widened by +-w; first-seen order */
static int32_t widen(int32_t n, int32_t m, const int32_t *visit, const unsigned char *hit, int32_t w, int32_t *out)
{
    int32_t k = 0;
    if (w <= 0) {
        for (int32_t t = 0; t < m; ++t)
            if (hit[t]) out[k++] = visit[t];
        return k;
    }
    unsigned char *mask = (unsigned char *)xcalloc((size_t)(n > 0 ? n : 1), 1);
    for (int32_t t = 0; t < m; ++t) {
        if (!hit[t]) continue;
        const int32_t pos = visit[t];
        const int32_t lo = pos - w < 0 ? 0 : pos - w, hi = pos + w > n - 1 ? n - 1 : pos + w;
        for (int32_t j = lo; j <= hi; ++j)
            if (!mask[j]) {
                mask[j] = 1;
                out[k++] = j;
            }
    }
    free(mask);
    return k;
}

/* BadDOFPreconditioner.cu:61-100 */
int32_t lsso_mas_select_elbow(int32_t n, const double *diag_abs, int32_t *out)
{
    if (n <= 0) return 0;
    int32_t *order = sorted_positions(n, diag_abs, 0);
    int32_t cut = 0;
    if (n > 1) {
        const double lo = log(diag_abs[order[0]]), hi = log(diag_abs[order[n - 1]]);
        double best = -1.0;
        for (int32_t i = 0; i < n; ++i) {
            const double chord = (hi - lo) / (n - 1.0) * i + lo;
            const double dev = fabs(chord - log(diag_abs[order[i]]));
            if (dev > best) {
                best = dev;
                cut = i;
            }
        }
    }
    int32_t k = 0;
    for (int32_t i = cut; i < n; ++i) out[k++] = order[i];
    free(order);
    return k;
}

/* BadDofKMeanPreconditioner.cu:63-172 (the assignment writes a value to the
 * cluster of the other centre, and a centre moves only with >= 1 (cluster 0)
 * or >= 2 (cluster 1) members: both as in the reference) */
int32_t lsso_mas_select_kmean(int32_t n, const double *v, double search_fraction, double jump_threshold,
                              int32_t max_iterations, int32_t expand_neighbors, int32_t *out)
{
    if (n < 2) return 0;
    int32_t *order = sorted_positions(n, v, 1);
    int32_t m = (int32_t)(n * search_fraction);
    if (m < 2) m = 2;
    if (m > n) m = n;
    double c0 = v[order[0]], c1 = v[order[m - 1]];
    for (int32_t it = 0; it < max_iterations; ++it) {
        double s0 = 0.0, s1 = 0.0;
        int32_t k0 = 0, k1 = 0;
        for (int32_t t = 0; t < m; ++t) {
            const double x = v[order[t]];
            if (fabs(x - c0) < fabs(x - c1)) {
                ++k1;
                s1 += x;
            } else {
                ++k0;
                s0 += x;
            }
        }
        const double n0 = k0 > 0 ? s0 / k0 : c0;
        const double n1 = k1 > 1 ? s1 / k1 : c1;
        if (n0 == c0 && n1 == c1) break;
        c0 = n0;
        c1 = n1;
    }
    if (c0 < c1) {
        const double t = c0;
        c0 = c1;
        c1 = t;
    }
    const double ratio = c0 / c1;
    int32_t k = 0;
    if (!isnan(ratio) && !(ratio < jump_threshold)) {
        const double sep = 0.5 * (c0 + c1);
        unsigned char *hit = (unsigned char *)xmalloc((size_t)m);
        for (int32_t t = 0; t < m; ++t) hit[t] = v[order[t]] > sep;
        k = widen(n, m, order, hit, expand_neighbors, out);
        free(hit);
    }
    free(order);
    return k;
}

static double rel_change(double now, double before)
{
    const double d = fabs(before) > 1e-300 ? fabs(before) : 1e-300;
    return fabs(now - before) / d;
}
static double log_normal_density(double x, double mean, double var)
{
    const double two_pi = 2.0 * 3.141592653589793238462643383279502884;
    return -0.5 * log(two_pi * var) - 0.5 * (x - mean) * (x - mean) / var;
}

/* BadDofGMMPreconditioner.cu:73-255 */
int32_t lsso_mas_select_gmm(int32_t n, const double *x, double jump_threshold, double tol, int32_t max_iterations,
                            int32_t expand_neighbors, int32_t *out)
{
    if (n < 2) return 0;
    double sum = 0.0;
    for (int32_t i = 0; i < n; ++i) sum += x[i];
    const double gmean = sum / n;
    double vs = 0.0;
    for (int32_t i = 0; i < n; ++i) {
        const double d = x[i] - gmean;
        vs += d * d;
    }
    const double gvar = vs / n;
    double m0 = x[0], m1 = x[0];
    for (int32_t i = 1; i < n; ++i) {
        if (x[i] < m0) m0 = x[i];
        if (x[i] > m1) m1 = x[i];
    }
    const double var_reg = 1e-6;
    double v0 = gvar > var_reg ? gvar : var_reg, v1 = v0, w0 = 0.5, w1 = 0.5;
    if (m0 == m1 || !isfinite(gvar)) return 0;
    double *g0 = (double *)xcalloc((size_t)n, sizeof(double));
    double *g1 = (double *)xcalloc((size_t)n, sizeof(double));
    const int32_t iters = max_iterations > 1 ? max_iterations : 1;
    for (int32_t it = 0; it < iters; ++it) {
        const double lw0 = log(w0 > DBL_MIN ? w0 : DBL_MIN), lw1 = log(w1 > DBL_MIN ? w1 : DBL_MIN);
        for (int32_t i = 0; i < n; ++i) {
            const double a = lw0 + log_normal_density(x[i], m0, v0);
            const double b = lw1 + log_normal_density(x[i], m1, v1);
            const double mx = a > b ? a : b;
            const double lt = mx + log(exp(a - mx) + exp(b - mx));
            g0[i] = exp(a - lt);
            g1[i] = exp(b - lt);
        }
        double s0 = 0.0, s1 = 0.0;
        for (int32_t i = 0; i < n; ++i) {
            s0 += g0[i];
            s1 += g1[i];
        }
        if (s0 <= 0.0 || s1 <= 0.0) break;
        w0 = s0 / n;
        w1 = s1 / n;
        const double pm0 = m0, pm1 = m1, pv0 = v0, pv1 = v1;
        m0 = 0.0;
        m1 = 0.0;
        for (int32_t i = 0; i < n; ++i) {
            m0 += g0[i] * x[i];
            m1 += g1[i] * x[i];
        }
        m0 /= s0;
        m1 /= s1;
        v0 = 0.0;
        v1 = 0.0;
        for (int32_t i = 0; i < n; ++i) {
            const double d0 = x[i] - m0, d1 = x[i] - m1;
            v0 += g0[i] * d0 * d0;
            v1 += g1[i] * d1 * d1;
        }
        v0 = v0 / s0 + var_reg;
        v1 = v1 / s1 + var_reg;
        if (rel_change(m0, pm0) < tol && rel_change(m1, pm1) < tol && rel_change(v0, pv0) < tol &&
            rel_change(v1, pv1) < tol)
            break;
    }
    const int high0 = fabs(m0) > fabs(m1);
    const double ratio = high0 ? fabs(m0) / fabs(m1) : fabs(m1) / fabs(m0);
    int32_t k = 0;
    if (!isnan(ratio) && !(ratio < jump_threshold)) {
        int32_t *visit = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)n);
        unsigned char *hit = (unsigned char *)xmalloc((size_t)n);
        for (int32_t i = 0; i < n; ++i) {
            visit[i] = i;
            hit[i] = high0 ? (g0[i] > g1[i]) : (g1[i] > g0[i]);
        }
        k = widen(n, n, visit, hit, expand_neighbors, out);
        free(visit);
        free(hit);
    }
    free(g0);
    free(g1);
    return k;
}

