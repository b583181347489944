/*
 * Plain-C restatement of the MCUT (v1.2.0) intersection front end.
 *
 * TEST INFRASTRUCTURE ONLY. It is the oracle the CUDA path is compared
 * against and the CPU baseline that bench.py times; the product library never
 * links, loads or calls it.
 *
 * Parity is pinned: tests/test_oracle_pin.py compares every output of this
 * file with the unmodified reference compiled from its own sources
 * (oracle/ref_harness.cpp) on the reference's 64 benchmark mesh pairs, its
 * named meshes and the synthetic workloads, and tests/golden/ keeps those
 * reference outputs as fixtures for hosts without the reference checkout.
 *
 * Every step follows the reference file:line it cites. The robust predicates
 * are written from Shewchuk, "Adaptive Precision Floating-Point Arithmetic
 * and Fast Robust Geometric Predicates" (DCG 18, 1997): orient2d keeps the
 * paper's four adaptive stages because its returned VALUE (not just its sign)
 * ranks vertex triplets (math.cpp:289-389); for orient3d only the sign is
 * ever used (math.cpp:391-427), so the sign comes from the paper's stage-A
 * filter followed by the exact 4x4 expansion determinant.
 *
 * Build flags: -ffp-contract=off (no fused multiply-add anywhere).
 */
#include "mcut_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* small vector helpers with the reference's exact operation order            */
/* ------------------------------------------------------------------------- */

/* dot_product: out = 0; out += a[i]*b[i]  (math.h:635-643) */
static double dot3(const double *a, const double *b)
{
    double o = 0.0;
    o = o + a[0] * b[0];
    o = o + a[1] * b[1];
    o = o + a[2] * b[2];
    return o;
}
/* std::max / std::min / compwise_{min,max} (math.h:580-600) */
static double dmax(double a, double b) { return (a < b) ? b : a; }
static double dmin(double a, double b) { return (b < a) ? b : a; }

typedef struct { double mn[3], mx[3]; } box_t;

/* bounding_box_t() / expand / enlarge / intersect_bounding_boxes (math.h:866-943) */
static void box_init(box_t *b)
{
    for (int j = 0; j < 3; ++j) { b->mn[j] = DBL_MAX; b->mx[j] = -DBL_MAX; }
}
static void box_expand_pt(box_t *b, const double *p)
{
    for (int j = 0; j < 3; ++j) { b->mx[j] = dmax(b->mx[j], p[j]); b->mn[j] = dmin(b->mn[j], p[j]); }
}
static void box_expand_box(box_t *b, const box_t *o)
{
    for (int j = 0; j < 3; ++j) { b->mx[j] = dmax(b->mx[j], o->mx[j]); b->mn[j] = dmin(b->mn[j], o->mn[j]); }
}
static int box_overlap(const box_t *a, const box_t *b)
{
    return (a->mn[0] <= b->mx[0] && a->mx[0] >= b->mn[0]) && (a->mn[1] <= b->mx[1] && a->mx[1] >= b->mn[1])
        && (a->mn[2] <= b->mx[2] && a->mx[2] >= b->mn[2]);
}

/* ------------------------------------------------------------------------- */
/* Shewchuk expansion arithmetic (restated from the paper, section 2)         */
/* ------------------------------------------------------------------------- */

static const double SPLITTER = 134217729.0;            /* 2^27 + 1 */
static const double EPS = 1.1102230246251565e-16;       /* 2^-53 */
#define CCW_A ((3.0 + 16.0 * EPS) * EPS)
#define CCW_B ((2.0 + 12.0 * EPS) * EPS)
#define CCW_C ((9.0 + 64.0 * EPS) * EPS * EPS)
#define RES_BOUND ((3.0 + 8.0 * EPS) * EPS)
#define O3D_A ((7.0 + 56.0 * EPS) * EPS)

static void two_sum(double a, double b, double *x, double *y)
{
    double s = a + b, bv = s - a, av = s - bv;
    *x = s;
    *y = (a - av) + (b - bv);
}
static void fast_two_sum(double a, double b, double *x, double *y)
{
    double s = a + b;
    *x = s;
    *y = b - (s - a);
}
static void two_diff(double a, double b, double *x, double *y)
{
    double s = a - b, bv = a - s, av = s + bv;
    *x = s;
    *y = (a - av) + (bv - b);
}
static double two_diff_tail(double a, double b, double x)
{
    double bv = a - x, av = x + bv;
    return (a - av) + (bv - b);
}
static void split(double a, double *hi, double *lo)
{
    double c = SPLITTER * a, big = c - a;
    *hi = c - big;
    *lo = a - *hi;
}
static void two_product(double a, double b, double *x, double *y)
{
    double p = a * b, ah, al, bh, bl;
    split(a, &ah, &al);
    split(b, &bh, &bl);
    double e1 = p - ah * bh, e2 = e1 - al * bh, e3 = e2 - ah * bl;
    *x = p;
    *y = al * bl - e3;
}
/* (a1 + a0) - (b1 + b0) as a 4-component expansion x[0..3] (least first) */
static void two_two_diff(double a1, double a0, double b1, double b0, double *x)
{
    double i, j, k0, t;
    two_diff(a0, b0, &i, &x[0]);
    two_sum(a1, i, &j, &k0);
    two_diff(k0, b1, &i, &x[1]);
    two_sum(j, i, &x[3], &x[2]);
    (void)t;
}
static double estimate(int n, const double *e)
{
    double q = e[0];
    for (int i = 1; i < n; ++i) q += e[i];
    return q;
}
/* merge two nonoverlapping expansions, eliminating zeros */
static int fast_expansion_sum_zeroelim(int elen, const double *e, int flen, const double *f, double *h)
{
    int ei = 0, fi = 0, hi = 0;
    double q, qn, hh, en = e[0], fn = f[0];
    if ((fn > en) == (fn > -en)) { q = en; ++ei; en = ei < elen ? e[ei] : 0.0; }
    else { q = fn; ++fi; fn = fi < flen ? f[fi] : 0.0; }
    if (ei < elen && fi < flen) {
        if ((fn > en) == (fn > -en)) { fast_two_sum(en, q, &qn, &hh); ++ei; en = ei < elen ? e[ei] : 0.0; }
        else { fast_two_sum(fn, q, &qn, &hh); ++fi; fn = fi < flen ? f[fi] : 0.0; }
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
        while (ei < elen && fi < flen) {
            if ((fn > en) == (fn > -en)) { two_sum(q, en, &qn, &hh); ++ei; en = ei < elen ? e[ei] : 0.0; }
            else { two_sum(q, fn, &qn, &hh); ++fi; fn = fi < flen ? f[fi] : 0.0; }
            q = qn;
            if (hh != 0.0) h[hi++] = hh;
        }
    }
    while (ei < elen) {
        two_sum(q, en, &qn, &hh); ++ei; en = ei < elen ? e[ei] : 0.0;
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
    }
    while (fi < flen) {
        two_sum(q, fn, &qn, &hh); ++fi; fn = fi < flen ? f[fi] : 0.0;
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
    }
    if (q != 0.0 || hi == 0) h[hi++] = q;
    return hi;
}
/* expansion times a double, eliminating zeros */
static int scale_expansion_zeroelim(int elen, const double *e, double b, double *h)
{
    double q, sum, hh, p1, p0, bh, bl, ah, al;
    int hi = 0;
    split(b, &bh, &bl);
    /* two_product(e[0], b) with b pre-split */
    {
        double p = e[0] * b;
        split(e[0], &ah, &al);
        double e1 = p - ah * bh, e2 = e1 - al * bh, e3 = e2 - ah * bl;
        q = p;
        hh = al * bl - e3;
    }
    if (hh != 0.0) h[hi++] = hh;
    for (int i = 1; i < elen; ++i) {
        double p = e[i] * b;
        split(e[i], &ah, &al);
        double e1 = p - ah * bh, e2 = e1 - al * bh, e3 = e2 - ah * bl;
        p1 = p;
        p0 = al * bl - e3;
        two_sum(q, p0, &sum, &hh);
        if (hh != 0.0) h[hi++] = hh;
        fast_two_sum(p1, sum, &q, &hh);
        if (hh != 0.0) h[hi++] = hh;
    }
    if (q != 0.0 || hi == 0) h[hi++] = q;
    return hi;
}

/* Adaptive orient2d: sign-exact, and the returned value follows the paper's
 * four stages (A: plain determinant, B: exact leading terms, C: first-order
 * tail correction, D: exact). Its magnitude ranks triplets, so the stage
 * outputs are reproduced, not just the sign. (shewchuk.c:1695-1721, 1610-1693) */
static double orient2d_adapt(const double *pa, const double *pb, const double *pc, double detsum)
{
    double acx = pa[0] - pc[0], bcx = pb[0] - pc[0], acy = pa[1] - pc[1], bcy = pb[1] - pc[1];
    double dl, dlt, dr, drt, B[4], C1[8], C2[12], D[16], u[4], s1, s0, t1, t0;
    two_product(acx, bcy, &dl, &dlt);
    two_product(acy, bcx, &dr, &drt);
    two_two_diff(dl, dlt, dr, drt, B);
    double det = estimate(4, B), eb = CCW_B * detsum;
    if (det >= eb || -det >= eb) return det;
    double acxt = two_diff_tail(pa[0], pc[0], acx), bcxt = two_diff_tail(pb[0], pc[0], bcx);
    double acyt = two_diff_tail(pa[1], pc[1], acy), bcyt = two_diff_tail(pb[1], pc[1], bcy);
    if (acxt == 0.0 && acyt == 0.0 && bcxt == 0.0 && bcyt == 0.0) return det;
    eb = CCW_C * detsum + RES_BOUND * fabs(det);
    det += (acx * bcyt + bcy * acxt) - (acy * bcxt + bcx * acyt);
    if (det >= eb || -det >= eb) return det;
    two_product(acxt, bcy, &s1, &s0);
    two_product(acyt, bcx, &t1, &t0);
    two_two_diff(s1, s0, t1, t0, u);
    int c1 = fast_expansion_sum_zeroelim(4, B, 4, u, C1);
    two_product(acx, bcyt, &s1, &s0);
    two_product(acy, bcxt, &t1, &t0);
    two_two_diff(s1, s0, t1, t0, u);
    int c2 = fast_expansion_sum_zeroelim(c1, C1, 4, u, C2);
    two_product(acxt, bcyt, &s1, &s0);
    two_product(acyt, bcxt, &t1, &t0);
    two_two_diff(s1, s0, t1, t0, u);
    int dn = fast_expansion_sum_zeroelim(c2, C2, 4, u, D);
    return D[dn - 1];
}
static double orient2d(const double *pa, const double *pb, const double *pc)
{
    double dl = (pa[0] - pc[0]) * (pb[1] - pc[1]);
    double dr = (pa[1] - pc[1]) * (pb[0] - pc[0]);
    double det = dl - dr, ds;
    if (dl > 0.0) {
        if (dr <= 0.0) return det;
        ds = dl + dr;
    } else if (dl < 0.0) {
        if (dr >= 0.0) return det;
        ds = -dl - dr;
    } else {
        return det;
    }
    double eb = CCW_A * ds;
    if (det >= eb || -det >= eb) return det;
    return orient2d_adapt(pa, pb, pc, ds);
}

/* exact orient3d sign from the 4x4 expansion determinant */
static void cross2(const double *p, const double *q, double *out4)
{
    double a1, a0, b1, b0;
    two_product(p[0], q[1], &a1, &a0);
    two_product(q[0], p[1], &b1, &b0);
    two_two_diff(a1, a0, b1, b0, out4);
}
static int orient3d_exact_sign(const double *pa, const double *pb, const double *pc, const double *pd)
{
    double ab[4], bc[4], cd[4], da[4], ac[4], bd[4], t8[8], abc[12], bcd[12], cda[12], dab[12];
    double adet[24], bdet[24], cdet[24], ddet[24], abd[48], cdd[48], det[96];
    cross2(pa, pb, ab); cross2(pb, pc, bc); cross2(pc, pd, cd);
    cross2(pd, pa, da); cross2(pa, pc, ac); cross2(pb, pd, bd);
    int tl = fast_expansion_sum_zeroelim(4, cd, 4, da, t8);
    int cdal = fast_expansion_sum_zeroelim(tl, t8, 4, ac, cda);
    tl = fast_expansion_sum_zeroelim(4, da, 4, ab, t8);
    int dabl = fast_expansion_sum_zeroelim(tl, t8, 4, bd, dab);
    for (int i = 0; i < 4; ++i) { bd[i] = -bd[i]; ac[i] = -ac[i]; }
    tl = fast_expansion_sum_zeroelim(4, ab, 4, bc, t8);
    int abcl = fast_expansion_sum_zeroelim(tl, t8, 4, ac, abc);
    tl = fast_expansion_sum_zeroelim(4, bc, 4, cd, t8);
    int bcdl = fast_expansion_sum_zeroelim(tl, t8, 4, bd, bcd);
    int al = scale_expansion_zeroelim(bcdl, bcd, pa[2], adet);
    int bl = scale_expansion_zeroelim(cdal, cda, -pb[2], bdet);
    int cl = scale_expansion_zeroelim(dabl, dab, pc[2], cdet);
    int dl = scale_expansion_zeroelim(abcl, abc, -pd[2], ddet);
    int abl = fast_expansion_sum_zeroelim(al, adet, bl, bdet, abd);
    int cdl = fast_expansion_sum_zeroelim(cl, cdet, dl, ddet, cdd);
    int n = fast_expansion_sum_zeroelim(abl, abd, cdl, cdd, det);
    double top = det[n - 1];
    return top > 0.0 ? 1 : (top < 0.0 ? -1 : 0);
}
/* sign of orient3d (shewchuk.c:2367-2407): stage-A filter, then exact */
static int orient3d_sign(const double *pa, const double *pb, const double *pc, const double *pd)
{
    double adx = pa[0] - pd[0], bdx = pb[0] - pd[0], cdx = pc[0] - pd[0];
    double ady = pa[1] - pd[1], bdy = pb[1] - pd[1], cdy = pc[1] - pd[1];
    double adz = pa[2] - pd[2], bdz = pb[2] - pd[2], cdz = pc[2] - pd[2];
    double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy;
    double cdxady = cdx * ady, adxcdy = adx * cdy;
    double adxbdy = adx * bdy, bdxady = bdx * ady;
    double det = adz * (bdxcdy - cdxbdy) + bdz * (cdxady - adxcdy) + cdz * (adxbdy - bdxady);
    double perm = (fabs(bdxcdy) + fabs(cdxbdy)) * fabs(adz) + (fabs(cdxady) + fabs(adxcdy)) * fabs(bdz)
        + (fabs(adxbdy) + fabs(bdxady)) * fabs(cdz);
    double eb = O3D_A * perm;
    if (det > eb) return 1;
    if (-det > eb) return -1;
    return orient3d_exact_sign(pa, pb, pc, pd);
}

/* ------------------------------------------------------------------------- */
/* geometry of the narrow phase                                              */
/* ------------------------------------------------------------------------- */

typedef struct {
    double n[3], d;
    int mc;          /* largest |normal| component */
    int degenerate;
    int ti, tj, tk;  /* plane-defining vertex triplet */
    double P[2][3];  /* 3D -> 2D projection (calculate_projection_matrix) */
} plane_t;

/* calculate_projection_matrix (math.cpp:710-793): P = K * R */
static void projection_matrix(const double *nrm, int mc, double P[2][3])
{
    double len = sqrt(dot3(nrm, nrm));
    double a[3] = { nrm[0] / len, nrm[1] / len, nrm[2] / len };
    double b[3] = { 0.0, 0.0, 0.0 };
    int s = (0.0 < nrm[mc]) - (nrm[mc] < 0.0);
    b[mc] = 1.0 * (double)s;
    double I[3][3] = { { 1.0, 0.0, 0.0 }, { 0.0, -1.0, 0.0 }, { 0.0, 0.0, 1.0 } };
    double R[3][3];
    memcpy(R, I, sizeof R);
    if (a[0] != b[0] || a[1] != b[1] || a[2] != b[2]) {
        double apb[3] = { a[0] + b[0], a[1] + b[1], a[2] + b[2] };
        double adb = dot3(a, b);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double outer = apb[i] * apb[j];
                R[i][j] = ((outer / adb) * 2.0) - I[i][j];
            }
    }
    double K[2][3] = { { 0 } };
    if (mc == 0) { K[0][1] = 1.0; K[1][2] = 1.0; }
    else if (mc == 1) { K[0][0] = 1.0; K[1][2] = 1.0; }
    else { K[0][0] = 1.0; K[1][1] = 1.0; }
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc = acc + K[i][k] * R[k][j];
            P[i][j] = acc;
        }
}
/* matrix_t * vec3 (math.h:508-520) */
static void project(const double P[2][3], const double *v, double *out)
{
    double r0 = 0.0, r1 = 0.0;
    for (int c = 0; c < 3; ++c) {
        r0 = r0 + P[0][c] * v[c];
        r1 = r1 + P[1][c] * v[c];
    }
    out[0] = r0;
    out[1] = r1;
}
/* 2-D crossing test, O'Rourke variant (math.cpp:643-703) */
static char pip2d(const double *q, const double (*poly)[2], int n)
{
    int rc = 0, lc = 0;
    for (int i = 0; i < n; ++i) {
        double xi = poly[i][0] - q[0], yi = poly[i][1] - q[1];
        if (xi == 0.0 && yi == 0.0) return 'v';
        int il = (i + n - 1) % n;
        double xl = poly[il][0] - q[0], yl = poly[il][1] - q[1];
        int rs = (yi > 0.0) != (yl > 0.0);
        int ls = (yi < 0.0) != (yl < 0.0);
        if (rs || ls) {
            double x = (xi * yl - xl * yi) / (yl - yi);
            if (rs && x > 0.0) rc++;
            if (ls && x < 0.0) lc++;
        }
    }
    if ((rc % 2) != (lc % 2)) return 'e';
    return (rc % 2) == 1 ? 'i' : 'o';
}
/* compute_point_in_polygon_test(vec3 ...) (math.cpp:851-902) */
static char pip3d(const double *p, const double *const *fv, int n, const plane_t *pl)
{
    double q[2], stackbuf[16][2];
    double (*poly)[2] = n <= 16 ? stackbuf : (double (*)[2])malloc(sizeof(double) * 2 * (size_t)n);
    project(pl->P, p, q);
    for (int i = 0; i < n; ++i) project(pl->P, fv[i], poly[i]);
    char c = pip2d(q, (const double (*)[2])poly, n);
    if (poly != stackbuf) free(poly);
    return c;
}

/* compute_polygon_plane_coefficients (math.cpp:130-239) */
static void face_plane(const double *const *fv, int n, plane_t *pl)
{
    double nx = 0.0, ny = 0.0, nz = 0.0;
    for (int i = 0; i < n; ++i) {
        const double *c = fv[i], *x = fv[(i + 1) % n];
        nx = nx + (c[1] - x[1]) * (c[2] + x[2]);
        ny = ny + (c[2] - x[2]) * (c[0] + x[0]);
        nz = nz + (c[0] - x[0]) * (c[1] + x[1]);
    }
    double nn[3] = { nx, ny, nz };
    memset(pl, 0, sizeof *pl);
    double sq = dot3(nn, nn);
    if (isnan(nx) || isnan(ny) || isnan(nz) || sq < 1e-9 || sq == 0.0) {
        pl->degenerate = 1;
        return;
    }
    double len = sqrt(sq);
    pl->n[0] = nx / len; pl->n[1] = ny / len; pl->n[2] = nz / len;
    pl->d = dot3(fv[0], pl->n);
    double big = 0.0;
    pl->mc = 0;
    for (int i = 0; i < 3; ++i) {
        double t = fabs(pl->n[i]);
        if (t > big) { big = t; pl->mc = i; }
    }
    projection_matrix(pl->n, pl->mc, pl->P);
    pl->ti = 0; pl->tj = 1; pl->tk = 2;
}

/* libstdc++'s std::sort on (|orient2d|, descending); its tie order decides
 * which triplet wins, so the same introsort + insertion-sort schedule is
 * replayed here (bits/stl_algo.h: __introsort_loop, __final_insertion_sort). */
typedef struct { int i, j, k; double v; } trip_t;
static int trip_less(const trip_t *a, const trip_t *b) { return fabs(a->v) > fabs(b->v); }
static void trip_swap(trip_t *a, trip_t *b) { trip_t t = *a; *a = *b; *b = t; }
static void ins_sort(trip_t *f, long n)
{
    for (long i = 1; i < n; ++i) {
        trip_t v = f[i];
        if (trip_less(&v, &f[0])) {
            memmove(f + 1, f, sizeof(trip_t) * (size_t)i);
            f[0] = v;
        } else {
            long j = i;
            while (trip_less(&v, &f[j - 1])) { f[j] = f[j - 1]; --j; }
            f[j] = v;
        }
    }
}
static void unguarded_ins_sort(trip_t *f, long from, long n)
{
    for (long i = from; i < n; ++i) {
        trip_t v = f[i];
        long j = i;
        while (trip_less(&v, &f[j - 1])) { f[j] = f[j - 1]; --j; }
        f[j] = v;
    }
}
static void median_to_first(trip_t *res, trip_t *a, trip_t *b, trip_t *c)
{
    if (trip_less(a, b)) {
        if (trip_less(b, c)) trip_swap(res, b);
        else if (trip_less(a, c)) trip_swap(res, c);
        else trip_swap(res, a);
    } else if (trip_less(a, c)) trip_swap(res, a);
    else if (trip_less(b, c)) trip_swap(res, c);
    else trip_swap(res, b);
}
static void sift_down(trip_t *f, long hole, long len, trip_t v)
{
    long top = hole, child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (trip_less(&f[child], &f[child - 1])) child--;
        f[hole] = f[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        f[hole] = f[child - 1];
        hole = child - 1;
    }
    long parent = (hole - 1) / 2;
    while (hole > top && trip_less(&f[parent], &v)) {
        f[hole] = f[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    f[hole] = v;
}
static void heap_sort_range(trip_t *f, long n)
{
    if (n < 2) return;
    for (long parent = (n - 2) / 2;; --parent) {
        sift_down(f, parent, n, f[parent]);
        if (parent == 0) break;
    }
    for (long last = n - 1; last > 0; --last) {
        trip_t v = f[last];
        f[last] = f[0];
        sift_down(f, 0, last, v);
    }
}
static void introsort_loop(trip_t *f, long n, int depth)
{
    while (n > 16) {
        if (depth == 0) { heap_sort_range(f, n); return; }
        --depth;
        long mid = n / 2;
        median_to_first(&f[0], &f[1], &f[mid], &f[n - 1]);
        long lo = 1, hi = n;
        for (;;) {
            while (trip_less(&f[lo], &f[0])) ++lo;
            --hi;
            while (trip_less(&f[0], &f[hi])) --hi;
            if (!(lo < hi)) break;
            trip_swap(&f[lo], &f[hi]);
            ++lo;
        }
        introsort_loop(f + lo, n - lo, depth);
        n = lo;
    }
}
static void std_sort_trips(trip_t *f, long n)
{
    if (n < 2) return;
    int lg = 63 - __builtin_clzll((unsigned long long)n);
    introsort_loop(f, n, 2 * lg);
    if (n > 16) {
        ins_sort(f, 16);
        unguarded_ins_sort(f, 16, n);
    } else {
        ins_sort(f, n);
    }
}
/* determine_three_noncollinear_vertices (math.cpp:289-389) */
static int noncollinear_triplet(const double *const *fv, int n, plane_t *pl)
{
    double (*x)[2] = (double (*)[2])malloc(sizeof(double) * 2 * (size_t)n);
    for (int i = 0; i < n; ++i) project(pl->P, fv[i], x[i]);
    long cap = (long)n * (n - 1) * (n - 2) / 6, m = 0;
    trip_t *t = (trip_t *)malloc(sizeof(trip_t) * (size_t)(cap > 0 ? cap : 1));
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j)
            for (int k = j + 1; k < n; ++k) {
                double r = orient2d(x[i], x[j], x[k]);
                if (!(r == 0.0)) { t[m].i = i; t[m].j = j; t[m].k = k; t[m].v = r; ++m; }
            }
    int ok = m > 0;
    if (ok) {
        std_sort_trips(t, m);
        pl->ti = t[0].i; pl->tj = t[0].j; pl->tk = t[0].k;
    }
    free(t);
    free(x);
    return ok;
}

/* ------------------------------------------------------------------------- */
/* meshes, recentring, OIBVH                                                 */
/* ------------------------------------------------------------------------- */

typedef struct {
    const void *v;      /* double[3*nv], or float[3*nv] when the input is float */
    const uint32_t *f;
    const uint32_t *fs;
    uint32_t nv, nf;
    uint64_t *off; /* nf+1 CSR offsets into f */
} mesh_t;

static int mesh_offsets(mesh_t *m)
{
    m->off = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)m->nf + 1));
    m->off[0] = 0;
    for (uint32_t i = 0; i < m->nf; ++i) {
        uint32_t n = m->fs ? m->fs[i] : 3;
        if (n < 3) return -1;
        m->off[i + 1] = m->off[i] + n;
    }
    uint64_t tot = m->off[m->nf];
    for (uint64_t i = 0; i < tot; ++i)
        if (m->f[i] >= m->nv) return -1;
    return 0;
}

/* get_bbox lambda of calculate_vertex_parameters (preproc.cpp:2152-2215);
 * float input compares in float (the running bound narrowed to float) */
static float fmaxr(float a, float b) { return (a < b) ? b : a; }
static float fminr(float a, float b) { return (b < a) ? b : a; }
static void vertex_bounds(const void *v, int fin, uint32_t n, double *mn, double *mx, double *com)
{
    for (int j = 0; j < 3; ++j) { mn[j] = DBL_MAX; mx[j] = -DBL_MAX; com[j] = 0.0; }
    for (uint32_t i = 0; i < n; ++i)
        for (int j = 0; j < 3; ++j) {
            if (fin) {
                float p = ((const float *)v)[(size_t)i * 3 + j];
                mx[j] = (double)fmaxr((float)mx[j], p);
                mn[j] = (double)fminr((float)mn[j], p);
                com[j] += (double)p;
            } else {
                double p = ((const double *)v)[(size_t)i * 3 + j];
                mx[j] = dmax(mx[j], p);
                mn[j] = dmin(mn[j], p);
                com[j] += p;
            }
        }
    for (int j = 0; j < 3; ++j) com[j] = com[j] / (double)n;
}
static double input_coord(const mesh_t *m, int fin, size_t k, double c, double t)
{
    if (fin) {
        float x = (((const float *)m->v)[k] - (float)c) + (float)t;
        return (double)x;
    }
    return (((const double *)m->v)[k] - c) + t;
}

/* calculate_vertex_parameters + the conversion in client_input_arrays_to_hmesh
 * (preproc.cpp:2124-2290, 147-181); eps = |cut box diagonal| * the general-
 * position constant, or the constant alone with absolute enforcement
 * (preproc.cpp:2518, 2667-2676) */
static double recentre(const mesh_t *S, const mesh_t *Cm, int fin, double gp_constant, int gp_absolute, double *sx,
    double *cx)
{
    double smn[3], smx[3], scom[3], cmn[3], cmx[3], ccom[3], com[3], gmn[3], tp[3], t[3];
    vertex_bounds(S->v, fin, S->nv, smn, smx, scom);
    vertex_bounds(Cm->v, fin, Cm->nv, cmn, cmx, ccom);
    for (int j = 0; j < 3; ++j) {
        com[j] = (scom[j] + ccom[j]) / 2.0;
        gmn[j] = dmin(smn[j], cmn[j]);
        tp[j] = com[j] - gmn[j];
    }
    double len = sqrt(dot3(tp, tp));
    for (int j = 0; j < 3; ++j) t[j] = tp[j] + tp[j] / len;
    for (uint32_t i = 0; i < S->nv; ++i)
        for (int j = 0; j < 3; ++j) sx[(size_t)i * 3 + j] = input_coord(S, fin, (size_t)i * 3 + j, com[j], t[j]);
    for (uint32_t i = 0; i < Cm->nv; ++i)
        for (int j = 0; j < 3; ++j) cx[(size_t)i * 3 + j] = input_coord(Cm, fin, (size_t)i * 3 + j, com[j], t[j]);
    double d[3];
    for (int j = 0; j < 3; ++j) d[j] = (cmx[j] + t[j]) - (cmn[j] + t[j]);
    return (gp_absolute ? 1.0 : sqrt(dot3(d, d))) * gp_constant;
}

/* face boxes (bvh.cpp:242-314) */
static void face_boxes(const mesh_t *m, const double *x, double eps, box_t *fb)
{
#pragma omp parallel for schedule(static)
    for (long f = 0; f < (long)m->nf; ++f) {
        box_t b;
        box_init(&b);
        for (uint64_t k = m->off[f]; k < m->off[f + 1]; ++k) box_expand_pt(&b, x + (size_t)m->f[k] * 3);
        if (eps > 0.0)
            for (int j = 0; j < 3; ++j) { b.mx[j] = b.mx[j] + eps; b.mn[j] = b.mn[j] - eps; }
        fb[f] = b;
    }
}

/* expandBits / morton3D (bvh.cpp:196-217) */
static unsigned expand_bits(unsigned v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
static unsigned morton3d(float x, float y, float z)
{
    x = fminf(fmaxf(x * 1024.0f, 0.0f), 1023.0f);
    y = fminf(fmaxf(y * 1024.0f, 0.0f), 1023.0f);
    z = fminf(fmaxf(z * 1024.0f, 0.0f), 1023.0f);
    return expand_bits((unsigned)x) * 4 + expand_bits((unsigned)y) * 2 + expand_bits((unsigned)z);
}

typedef struct { uint32_t code, face; } leaf_t;
static int leaf_cmp(const void *a, const void *b)
{
    const leaf_t *x = (const leaf_t *)a, *y = (const leaf_t *)b;
    if (x->code != y->code) return x->code < y->code ? -1 : 1;
    return x->face < y->face ? -1 : (x->face > y->face);
}

/* Implicit complete binary tree over the Morton-sorted leaves (the layout of
 * bvh.cpp:71-193 without the compacted memory map: node boxes are indexed by
 * implicit index directly). "Real" nodes on a level are the ancestors of real
 * leaves: implicit ids [2^l - 1, rightmost_real(l)]. */
typedef struct {
    int leaf_level;
    int64_t rightmost_leaf;  /* implicit id of the last real leaf */
    box_t *node;             /* 2^(leaf_level+1) - 1 entries */
    uint32_t *leaf_face;     /* sorted leaves -> face id */
} oibvh_t;

static int ilog2u(uint64_t x) { return 63 - __builtin_clzll(x); }
static uint64_t np2(uint64_t x) { uint64_t p = 1; while (p < x) p <<= 1; return p; }
static int64_t ancestor(int64_t node, int dist) { return ((node + 1) >> dist) - 1; }

static void build_oibvh(const mesh_t *m, const box_t *fb, oibvh_t *t)
{
    const uint32_t F = m->nf;
    box_t mb;
    box_init(&mb);
    for (uint32_t f = 0; f < F; ++f) box_expand_box(&mb, &fb[f]);
    leaf_t *lv = (leaf_t *)malloc(sizeof(leaf_t) * F);
#pragma omp parallel for schedule(static)
    for (long f = 0; f < (long)F; ++f) {
        double c[3], o[3], dm[3];
        for (int j = 0; j < 3; ++j) {
            c[j] = (fb[f].mn[j] + fb[f].mx[j]) / 2.0;
            o[j] = c[j] - mb.mn[j];
            dm[j] = mb.mx[j] - mb.mn[j];
        }
        lv[f].code = morton3d((float)(o[0] / dm[0]), (float)(o[1] / dm[1]), (float)(o[2] / dm[2]));
        lv[f].face = (uint32_t)f;
    }
    qsort(lv, F, sizeof(leaf_t), leaf_cmp);
    t->leaf_level = ilog2u(np2(F));
    const int L = t->leaf_level;
    const int64_t first_leaf = ((int64_t)1 << L) - 1;
    t->rightmost_leaf = first_leaf + F - 1;
    t->node = (box_t *)malloc(sizeof(box_t) * (size_t)(((int64_t)2 << L) - 1));
    t->leaf_face = (uint32_t *)malloc(sizeof(uint32_t) * F);
    for (uint32_t i = 0; i < F; ++i) {
        t->leaf_face[i] = lv[i].face;
        t->node[first_leaf + i] = fb[lv[i].face];
    }
    for (int l = L - 1; l >= 0; --l) {
        const int64_t lo = ((int64_t)1 << l) - 1, hi = ancestor(t->rightmost_leaf, L - l);
        const int64_t child_hi = ancestor(t->rightmost_leaf, L - l - 1);
#pragma omp parallel for schedule(static)
        for (int64_t nd = lo; nd <= hi; ++nd) {
            box_t b;
            box_init(&b);
            box_expand_box(&b, &t->node[2 * nd + 1]);
            if (2 * nd + 2 <= child_hi) box_expand_box(&b, &t->node[2 * nd + 2]);
            t->node[nd] = b;
        }
    }
    free(lv);
}

typedef struct { uint32_t s, c; } pair_t;
typedef struct { pair_t *p; int64_t n, cap; } pairvec_t;
static void pv_push(pairvec_t *v, uint32_t s, uint32_t c)
{
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 1024;
        v->p = (pair_t *)realloc(v->p, sizeof(pair_t) * (size_t)v->cap);
    }
    v->p[v->n].s = s;
    v->p[v->n].c = c;
    v->n++;
}

/* intersectOIBVHs (bvh.cpp:638-783): breadth-first over node pairs, closed
 * box test, leaf-leaf overlaps emitted. Serial, as in the reference. */
static void traverse(const oibvh_t *a, const oibvh_t *b, pairvec_t *out)
{
    int64_t cap = 1 << 16, head = 0, tail = 0;
    int64_t *qa = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap), *qb = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap);
#define PUSH(x, y)                                                                          \
    do {                                                                                    \
        if (tail - head == cap) {                                                           \
            int64_t nc = cap * 2;                                                           \
            int64_t *na = (int64_t *)malloc(sizeof(int64_t) * (size_t)nc);                  \
            int64_t *nb = (int64_t *)malloc(sizeof(int64_t) * (size_t)nc);                  \
            for (int64_t z = 0; z < tail - head; ++z) {                                     \
                na[z] = qa[(head + z) % cap];                                               \
                nb[z] = qb[(head + z) % cap];                                               \
            }                                                                               \
            free(qa); free(qb); qa = na; qb = nb; tail = tail - head; head = 0; cap = nc;   \
        }                                                                                   \
        qa[tail % cap] = (x); qb[tail % cap] = (y); ++tail;                                 \
    } while (0)
    PUSH(0, 0);
    const int La = a->leaf_level, Lb = b->leaf_level;
    while (head < tail) {
        const int64_t na = qa[head % cap], nb = qb[head % cap];
        ++head;
        const int la = ilog2u((uint64_t)na + 1), lb = ilog2u((uint64_t)nb + 1);
        if (!box_overlap(&a->node[na], &b->node[nb])) continue;
        const int a_leaf = la == La, b_leaf = lb == Lb;
        if (a_leaf && b_leaf) {
            pv_push(out, a->leaf_face[na - (((int64_t)1 << La) - 1)], b->leaf_face[nb - (((int64_t)1 << Lb) - 1)]);
        } else if (a_leaf) {
            const int64_t rhi = ancestor(b->rightmost_leaf, Lb - lb - 1);
            PUSH(na, 2 * nb + 1);
            if (2 * nb + 2 <= rhi) PUSH(na, 2 * nb + 2);
        } else if (b_leaf) {
            const int64_t rhi = ancestor(a->rightmost_leaf, La - la - 1);
            PUSH(2 * na + 1, nb);
            if (2 * na + 2 <= rhi) PUSH(2 * na + 2, nb);
        } else {
            const int64_t rha = ancestor(a->rightmost_leaf, La - la - 1), rhb = ancestor(b->rightmost_leaf, Lb - lb - 1);
            const int ar = 2 * na + 2 <= rha, br = 2 * nb + 2 <= rhb;
            PUSH(2 * na + 1, 2 * nb + 1);
            if (br) PUSH(2 * na + 1, 2 * nb + 2);
            if (ar) {
                PUSH(2 * na + 2, 2 * nb + 1);
                if (br) PUSH(2 * na + 2, 2 * nb + 2);
            }
        }
    }
#undef PUSH
    free(qa);
    free(qb);
}

static int pair_cmp(const void *x, const void *y)
{
    const pair_t *a = (const pair_t *)x, *b = (const pair_t *)y;
    if (a->s != b->s) return a->s < b->s ? -1 : 1;
    return a->c < b->c ? -1 : (a->c > b->c);
}
static int u64_cmp(const void *x, const void *y)
{
    uint64_t a = *(const uint64_t *)x, b = *(const uint64_t *)y;
    return a < b ? -1 : (a > b);
}

/* ------------------------------------------------------------------------- */
/* polygon-soup edges (hmesh add_face / add_edge, hmesh.cpp:405-651)          */
/* ------------------------------------------------------------------------- */

typedef struct { uint32_t q, r, f0, f1; } edge_t;
typedef struct { uint64_t *key; uint32_t *val; uint64_t mask; } hash_t;

static uint64_t mix64(uint64_t x)
{
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
    return x;
}

/* ------------------------------------------------------------------------- */
/* the front end                                                             */
/* ------------------------------------------------------------------------- */

typedef struct { uint32_t q, r, g; int8_t info[4]; double p[3]; int rec; } test_t;
static int test_cmp(const void *x, const void *y)
{
    const test_t *a = (const test_t *)x, *b = (const test_t *)y;
    if (a->q != b->q) return a->q < b->q ? -1 : 1;
    if (a->r != b->r) return a->r < b->r ? -1 : 1;
    return a->g < b->g ? -1 : (a->g > b->g);
}

static int front_end_core(mesh_t *Sp, mesh_t *Cp, double *x, double eps, const double *perturbation,
    fe_result *out);

/* One front-end pass. With a perturbation (general-position enforcement,
 * preproc.cpp:2590-2699) the cut vertices of the narrow phase are the
 * recentred ones plus the perturbation (one rounding, preproc.cpp:131-133,
 * 176-180), while the face boxes and the candidate pairs stay those of the
 * unperturbed meshes: the reference builds the cut BVH only on the first
 * attempt (preproc.cpp:2680) and traverses only after a rebuild
 * (preproc.cpp:2820-2846). A perturbed pass with no record is a general-
 * position violation (kernel.cpp:3211-3225). */
int oracle_front_end2(const void *sv, const uint32_t *sf, const uint32_t *sfs, uint32_t nsv, uint32_t nsf,
    const void *cv, const uint32_t *cf, const uint32_t *cfs, uint32_t ncv, uint32_t ncf, int float_input,
    int threads, double gp_constant, int gp_absolute, const double *perturbation, fe_result *out)
{
    memset(out, 0, sizeof *out);
    out->bad_face = -1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    mesh_t S = { sv, sf, sfs, nsv, nsf, NULL }, Cm = { cv, cf, cfs, ncv, ncf, NULL };
    if (nsv < 3 || ncv < 3 || nsf < 1 || ncf < 1 || mesh_offsets(&S) || mesh_offsets(&Cm)) {
        free(S.off); free(Cm.off);
        out->status = FE_INVALID_INPUT;
        return 0;
    }
    double *x = (double *)malloc(sizeof(double) * 3 * ((size_t)nsv + ncv)); /* ps vertices */
    const double eps = recentre(&S, &Cm, float_input, gp_constant, gp_absolute, x, x + (size_t)nsv * 3);
    return front_end_core(&S, &Cm, x, eps, perturbation, out);
}

/* The same pass over internal (already recentred) coordinates and a given
 * cut-box enlargement: the form the front end has inside dispatch(), where
 * the halfedge meshes hold recentred coordinates (kernel.h:122-170). */
int oracle_front_end_internal(const double *xs, const uint32_t *sf, const uint32_t *sfs, uint32_t nsv, uint32_t nsf,
    const double *xc, const uint32_t *cf, const uint32_t *cfs, uint32_t ncv, uint32_t ncf, double eps, int threads,
    fe_result *out)
{
    memset(out, 0, sizeof *out);
    out->bad_face = -1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    mesh_t S = { xs, sf, sfs, nsv, nsf, NULL }, Cm = { xc, cf, cfs, ncv, ncf, NULL };
    if (nsv < 3 || ncv < 3 || nsf < 1 || ncf < 1 || mesh_offsets(&S) || mesh_offsets(&Cm)) {
        free(S.off); free(Cm.off);
        out->status = FE_INVALID_INPUT;
        return 0;
    }
    double *x = (double *)malloc(sizeof(double) * 3 * ((size_t)nsv + ncv));
    memcpy(x, xs, sizeof(double) * 3 * (size_t)nsv);
    memcpy(x + (size_t)nsv * 3, xc, sizeof(double) * 3 * (size_t)ncv);
    return front_end_core(&S, &Cm, x, eps, NULL, out);
}

/* everything after the recentring: x (ps coordinates, taken over and freed)
 * and the cut-box enlargement eps */
static int front_end_core(mesh_t *Sp, mesh_t *Cp, double *x, double eps, const double *perturbation, fe_result *out)
{
    mesh_t S = *Sp, Cm = *Cp;
    const uint32_t nsv = S.nv, nsf = S.nf, ncv = Cm.nv, ncf = Cm.nf;
    const uint32_t *sf = S.f, *cf = Cm.f;
    const uint32_t NV = nsv + ncv, NF = nsf + ncf;
    out->cut_eps = eps;
    out->src_xyz = (double *)malloc(sizeof(double) * 3 * (size_t)nsv);
    out->cut_xyz = (double *)malloc(sizeof(double) * 3 * (size_t)ncv);
    memcpy(out->src_xyz, x, sizeof(double) * 3 * (size_t)nsv);
    memcpy(out->cut_xyz, x + (size_t)nsv * 3, sizeof(double) * 3 * (size_t)ncv);

    box_t *fb = (box_t *)malloc(sizeof(box_t) * NF);
    face_boxes(&S, x, 0.0, fb);
    face_boxes(&Cm, x + (size_t)nsv * 3, eps, fb + nsf);
    out->face_boxes = (double *)malloc(sizeof(double) * 6 * (size_t)NF);
    for (uint32_t f = 0; f < NF; ++f) {
        memcpy(out->face_boxes + (size_t)f * 6, fb[f].mn, sizeof(double) * 3);
        memcpy(out->face_boxes + (size_t)f * 6 + 3, fb[f].mx, sizeof(double) * 3);
    }

    oibvh_t ts, tc;
    build_oibvh(&S, fb, &ts);
    build_oibvh(&Cm, fb + nsf, &tc);
    pairvec_t pv = { 0 };
    traverse(&ts, &tc, &pv);
    free(ts.node); free(ts.leaf_face); free(tc.node); free(tc.leaf_face);
    if (pv.n) qsort(pv.p, (size_t)pv.n, sizeof(pair_t), pair_cmp);
    out->n_pairs = pv.n;
    out->pairs = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)(pv.n ? pv.n : 1));
    for (int64_t i = 0; i < pv.n; ++i) { out->pairs[2 * i] = pv.p[i].s; out->pairs[2 * i + 1] = pv.p[i].c; }
    if (perturbation) {
        for (uint32_t i = 0; i < ncv; ++i)
            for (int j = 0; j < 3; ++j) x[((size_t)nsv + i) * 3 + j] = x[((size_t)nsv + i) * 3 + j] + perturbation[j];
        memcpy(out->cut_xyz, x + (size_t)nsv * 3, sizeof(double) * 3 * (size_t)ncv);
    }

    /* ps face CSR (sources first, then cut faces with vertex ids offset by Vs) */
    uint64_t *foff = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)NF + 1));
    const uint64_t sidx = S.off[nsf], cidx = Cm.off[ncf];
    uint32_t *fidx = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(sidx + cidx));
    memcpy(fidx, sf, sizeof(uint32_t) * sidx);
    for (uint64_t k = 0; k < cidx; ++k) fidx[sidx + k] = cf[k] + nsv;
    for (uint32_t f = 0; f <= nsf; ++f) foff[f] = S.off[f];
    for (uint32_t f = 1; f <= ncf; ++f) foff[nsf + f] = sidx + Cm.off[f];

    /* partner lists per ps face, both directions (bvh.cpp:705-714) */
    uint32_t *pcnt = (uint32_t *)calloc((size_t)NF + 1, sizeof(uint32_t));
    for (int64_t i = 0; i < pv.n; ++i) { pcnt[pv.p[i].s + 1]++; pcnt[nsf + pv.p[i].c + 1]++; }
    uint64_t *poff = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)NF + 1));
    poff[0] = 0;
    for (uint32_t f = 0; f < NF; ++f) poff[f + 1] = poff[f] + pcnt[f + 1];
    uint32_t *pfill = (uint32_t *)calloc(NF, sizeof(uint32_t));
    uint32_t *plist = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(2 * pv.n + 1));
    for (int64_t i = 0; i < pv.n; ++i) {
        const uint32_t s = pv.p[i].s, c = nsf + pv.p[i].c;
        plist[poff[s] + pfill[s]++] = c;
        plist[poff[c] + pfill[c]++] = s;
    }
    free(pcnt); free(pfill); free(pv.p);

    /* ps edges: first occurrence (lowest face, in-face order) fixes q -> r */
    const uint64_t nhe = sidx + cidx;
    hash_t h;
    uint64_t cap = 16;
    while (cap < 2 * nhe) cap <<= 1;
    h.key = (uint64_t *)malloc(sizeof(uint64_t) * cap);
    h.val = (uint32_t *)malloc(sizeof(uint32_t) * cap);
    h.mask = cap - 1;
    memset(h.key, 0xff, sizeof(uint64_t) * cap);
    edge_t *E = (edge_t *)malloc(sizeof(edge_t) * (size_t)(nhe ? nhe : 1));
    uint32_t *he_edge = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(nhe ? nhe : 1));
    uint32_t ne = 0;
    for (uint32_t f = 0; f < NF; ++f) {
        const uint64_t o = foff[f], n = foff[f + 1] - o;
        for (uint64_t k = 0; k < n; ++k) {
            const uint32_t a = fidx[o + k], b = fidx[o + (k + 1) % n];
            const uint64_t key = ((uint64_t)(a < b ? a : b) << 32) | (a < b ? b : a);
            uint64_t s = mix64(key) & h.mask;
            while (h.key[s] != UINT64_MAX && h.key[s] != key) s = (s + 1) & h.mask;
            if (h.key[s] == UINT64_MAX) {
                h.key[s] = key;
                h.val[s] = ne;
                E[ne].q = a; E[ne].r = b; E[ne].f0 = f; E[ne].f1 = UINT32_MAX;
                ++ne;
            } else {
                E[h.val[s]].f1 = f;
            }
            he_edge[o + k] = h.val[s];
        }
    }
    free(h.key); free(h.val);

    /* face properties of every candidate face; a degenerate one aborts
     * before the narrow phase (kernel.cpp:2184-2356). The face's vertex list
     * is the one the polygon soup's get_vertices_around_face returns: the
     * TARGETS of its halfedges (hmesh.cpp:722-733). The soup copies the
     * source mesh, so a source face lists its input corners rotated by one
     * (v1, v2, ..., v0); it adds each cut face as the cut mesh's own
     * get_vertices_around_face lists it (kernel.cpp:1650-1700), so a cut face
     * lists them rotated by two (v2, ..., v0, v1). Newell's sum,
     * d = <v_first, n>, the plane triplet and the 2-D polygon all use that
     * order. */
    plane_t *pl = (plane_t *)calloc(NF, sizeof(plane_t));
    int bad = -1;
#pragma omp parallel for schedule(dynamic, 256)
    for (long f = 0; f < (long)NF; ++f) {
        if (poff[f + 1] == poff[f]) continue;
        const int n = (int)(foff[f + 1] - foff[f]);
        const double **fv = (const double **)malloc(sizeof(double *) * (size_t)n);
        const int rot = (uint32_t)f < nsf ? 1 : 2;
        for (int k = 0; k < n; ++k) fv[k] = x + (size_t)fidx[foff[f] + (k + rot) % n] * 3;
        face_plane(fv, n, &pl[f]);
        if (pl[f].degenerate) {
#pragma omp critical
            if (bad < 0 || f < bad) bad = (int)f;
        } else if (n > 3) {
            if (!noncollinear_triplet(fv, n, &pl[f])) pl[f].ti = -1;
        }
        free(fv);
    }
    if (bad >= 0) {
        out->bad_face = bad;
        out->status = (uint32_t)bad >= nsf ? FE_DEGENERATE_CUT_FACE : FE_DEGENERATE_SRC_FACE;
    }

    /* (edge, face) candidates: edges of each candidate face x its partners,
     * deduplicated (kernel.cpp:1781-1983), then culled by edge box vs face
     * box (kernel.cpp:1989-2177) */
    uint64_t nef = 0;
    for (uint32_t f = 0; f < NF; ++f) nef += (foff[f + 1] - foff[f]) * (poff[f + 1] - poff[f]);
    uint64_t *ef = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(nef ? nef : 1));
    uint64_t w = 0;
    for (uint32_t f = 0; f < NF; ++f)
        for (uint64_t k = foff[f]; k < foff[f + 1]; ++k)
            for (uint64_t p = poff[f]; p < poff[f + 1]; ++p) ef[w++] = ((uint64_t)he_edge[k] << 32) | plist[p];
    qsort(ef, (size_t)nef, sizeof(uint64_t), u64_cmp);
    uint64_t nu = 0;
    for (uint64_t i = 0; i < nef; ++i)
        if (i == 0 || ef[i] != ef[i - 1]) ef[nu++] = ef[i];

    test_t *T = (test_t *)malloc(sizeof(test_t) * (size_t)(nu ? nu : 1));
    uint64_t nt = 0;
    for (uint64_t i = 0; i < nu; ++i) {
        const edge_t *e = &E[ef[i] >> 32];
        const uint32_t g = (uint32_t)ef[i];
        box_t eb;
        box_init(&eb);
        box_expand_pt(&eb, x + (size_t)e->q * 3);
        box_expand_pt(&eb, x + (size_t)e->r * 3);
        if (!box_overlap(&eb, &fb[g])) continue;
        T[nt].q = e->q; T[nt].r = e->r; T[nt].g = g;
        ++nt;
    }
    free(ef);

    int gp = 0;
    if (out->status == FE_OK) {
        /* narrow phase (kernel.cpp:2456-2658) */
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : gp)
        for (long i = 0; i < (long)nt; ++i) {
            test_t *t = &T[i];
            const plane_t *P = &pl[t->g];
            const int n = (int)(foff[t->g + 1] - foff[t->g]);
            const double *fvb[8];
            const double **fv = n <= 8 ? fvb : (const double **)malloc(sizeof(double *) * (size_t)n);
            const int rot = t->g < nsf ? 1 : 2;
            for (int k = 0; k < n; ++k) fv[k] = x + (size_t)fidx[foff[t->g] + (k + rot) % n] * 3;
            const double *q = x + (size_t)t->q * 3, *r = x + (size_t)t->r * 3;
            memset(t->info, 0, 4);
            t->rec = 0;
            char type = '0', pip = 0;
            if (P->ti >= 0) {
                const int sq = orient3d_sign(fv[P->ti], fv[P->tj], fv[P->tk], q);
                const int sr = orient3d_sign(fv[P->ti], fv[P->tj], fv[P->tk], r);
                t->info[0] = (int8_t)sq;
                t->info[1] = (int8_t)sr;
                /* compute_segment_plane_intersection_type (math.cpp:391-427) */
                if (sq == 0 && sr == 0) type = 'p';
                else if (sq == 0) type = 'q';
                else if (sr == 0) type = 'r';
                else if ((sr < 0 && sq < 0) || (sr > 0 && sq > 0)) type = '0';
                else type = '1';
            }
            if (type == 'q' || type == 'r') {
                pip = pip3d(type == 'q' ? q : r, fv, n, P);
            } else if (type == 'p') {
                pip = pip3d(q, fv, n, P);
                if (!(pip == 'i' || pip == 'v' || pip == 'e')) pip = pip3d(r, fv, n, P);
            } else if (type == '1') {
                /* compute_segment_plane_intersection (math.cpp:249-287) */
                double p[3] = { 0.0, 0.0, 0.0 };
                const double num = P->d - dot3(q, P->n);
                const double rq[3] = { r[0] - q[0], r[1] - q[1], r[2] - q[2] };
                const double den = dot3(rq, P->n);
                if (!(den == 0.0)) {
                    const double tt = num / den;
                    for (int k = 0; k < 3; ++k) p[k] = q[k] + tt * (r[k] - q[k]);
                }
                pip = pip3d(p, fv, n, P);
                if (pip == 'i') {
                    t->rec = 1;
                    memcpy(t->p, p, sizeof p);
                }
            }
            if ((type == 'q' || type == 'r' || type == 'p') && (pip == 'i' || pip == 'v' || pip == 'e')) gp = 1;
            if (type == '1' && (pip == 'v' || pip == 'e')) gp = 1;
            t->info[2] = (int8_t)type;
            t->info[3] = (int8_t)pip;
            if (fv != fvb) free((void *)fv);
        }
        if (gp) out->status = FE_GP_VIOLATION;
    }

    if (nt) qsort(T, (size_t)nt, sizeof(test_t), test_cmp);
    const int run = bad < 0; /* tests carry no predicate output after a degenerate face */
    out->n_tests = run ? (int64_t)nt : 0;
    out->tests = (uint32_t *)malloc(sizeof(uint32_t) * 3 * (size_t)(nt ? nt : 1));
    out->test_info = (int8_t *)malloc(4 * (size_t)(nt ? nt : 1));
    int64_t nr = 0;
    for (uint64_t i = 0; run && i < nt; ++i) {
        out->tests[3 * i] = T[i].q; out->tests[3 * i + 1] = T[i].r; out->tests[3 * i + 2] = T[i].g;
        memcpy(out->test_info + 4 * i, T[i].info, 4);
        nr += T[i].rec;
    }
    out->n_records = nr;
    if (perturbation && out->status == FE_OK && nr == 0) out->status = FE_GP_VIOLATION;
    out->rec_ids = (uint32_t *)malloc(sizeof(uint32_t) * 3 * (size_t)(nr ? nr : 1));
    out->rec_pts = (double *)malloc(sizeof(double) * 3 * (size_t)(nr ? nr : 1));
    int64_t k = 0;
    for (uint64_t i = 0; run && i < nt; ++i)
        if (T[i].rec) {
            out->rec_ids[3 * k] = T[i].q; out->rec_ids[3 * k + 1] = T[i].r; out->rec_ids[3 * k + 2] = T[i].g;
            memcpy(out->rec_pts + 3 * k, T[i].p, sizeof(double) * 3);
            ++k;
        }

    free(T); free(pl); free(E); free(he_edge); free(plist); free(poff); free(foff); free(fidx);
    free(fb); free(x); free(S.off); free(Cm.off);
    return 0;
}

int oracle_front_end(const void *sv, const uint32_t *sf, const uint32_t *sfs, uint32_t nsv, uint32_t nsf,
    const void *cv, const uint32_t *cf, const uint32_t *cfs, uint32_t ncv, uint32_t ncf, int float_input,
    int threads, fe_result *out)
{
    return oracle_front_end2(sv, sf, sfs, nsv, nsf, cv, cf, cfs, ncv, ncf, float_input, threads, 1e-4, 0, NULL, out);
}

/* predicate entry points for the predicate-level pin tests */
int oracle_orient3d_sign(const double *pa, const double *pb, const double *pc, const double *pd)
{
    return orient3d_sign(pa, pb, pc, pd);
}
double oracle_orient2d(const double *pa, const double *pb, const double *pc) { return orient2d(pa, pb, pc); }

void oracle_free(fe_result *r)
{
    free(r->pairs); free(r->tests); free(r->test_info); free(r->rec_ids); free(r->rec_pts);
    free(r->face_boxes); free(r->src_xyz); free(r->cut_xyz);
    memset(r, 0, sizeof *r);
}

/* ------------------------------------------------------------------------- */
/* the record hand-over (kernel.cpp:2599-2655, 2673-2714)                    */
/* ------------------------------------------------------------------------- */

typedef struct { uint64_t key; uint32_t vtx; } kv_t;
static int kv_cmp(const void *x, const void *y)
{
    const kv_t *a = (const kv_t *)x, *b = (const kv_t *)y;
    if (a->key != b->key) return a->key < b->key ? -1 : 1;
    return a->vtx < b->vtx ? -1 : (a->vtx > b->vtx);
}
typedef struct { uint32_t edge, g, k; } rord_t; /* edge creation index, tested face, input position */
static int rord_cmp(const void *x, const void *y)
{
    const rord_t *a = (const rord_t *)x, *b = (const rord_t *)y;
    if (a->edge != b->edge) return a->edge < b->edge ? -1 : 1;
    return a->g < b->g ? -1 : (a->g > b->g);
}

/* runs of equal keys in sorted kv: keys, offsets and the vertex column */
static uint32_t kv_runs(const kv_t *kv, uint64_t n, uint32_t **keys, int pairs, uint32_t **off, uint32_t **vtx)
{
    uint32_t nk = 0;
    for (uint64_t i = 0; i < n; ++i) nk += (i == 0 || kv[i].key != kv[i - 1].key);
    *keys = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(pairs ? 2 : 1) * (nk ? nk : 1));
    *off = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)nk + 1));
    *vtx = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
    uint32_t j = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (i == 0 || kv[i].key != kv[i - 1].key) {
            if (pairs) {
                (*keys)[2 * j] = (uint32_t)(kv[i].key >> 32);
                (*keys)[2 * j + 1] = (uint32_t)kv[i].key;
            } else {
                (*keys)[j] = (uint32_t)kv[i].key;
            }
            (*off)[j++] = (uint32_t)i;
        }
        (*vtx)[i] = kv[i].vtx;
    }
    (*off)[nk] = (uint32_t)n;
    return nk;
}

int oracle_seam(const uint32_t *sf, const uint32_t *sfs, uint32_t nsv, uint32_t nsf, const uint32_t *cf,
    const uint32_t *cfs, uint32_t ncv, uint32_t ncf, const uint32_t *rec3, const double *pts, int64_t nr,
    fe_seam *out)
{
    memset(out, 0, sizeof *out);
    mesh_t S = { NULL, sf, sfs, nsv, nsf, NULL }, Cm = { NULL, cf, cfs, ncv, ncf, NULL };
    if (mesh_offsets(&S) || mesh_offsets(&Cm)) { free(S.off); free(Cm.off); return -1; }
    const uint32_t NV = nsv + ncv, NF = nsf + ncf;
    /* the ps edges in creation order (hmesh_t::add_face over the source faces,
     * then the cut faces, hmesh.cpp:406-651): the first face corner fixes q -> r
     * and f0, the second face is f1 */
    const uint64_t sidx = S.off[nsf], cidx = Cm.off[ncf], nhe = sidx + cidx;
    hash_t h;
    uint64_t cap = 16;
    while (cap < 2 * nhe) cap <<= 1;
    h.key = (uint64_t *)malloc(sizeof(uint64_t) * cap);
    h.val = (uint32_t *)malloc(sizeof(uint32_t) * cap);
    h.mask = cap - 1;
    memset(h.key, 0xff, sizeof(uint64_t) * cap);
    edge_t *E = (edge_t *)malloc(sizeof(edge_t) * (size_t)(nhe ? nhe : 1));
    uint32_t ne = 0;
    for (uint32_t f = 0; f < NF; ++f) {
        const mesh_t *m = f < nsf ? &S : &Cm;
        const uint32_t lf = f < nsf ? f : f - nsf, vo = f < nsf ? 0 : nsv;
        const uint64_t o = m->off[lf], n = m->off[lf + 1] - o;
        for (uint64_t k = 0; k < n; ++k) {
            const uint32_t a = m->f[o + k] + vo, b = m->f[o + (k + 1) % n] + vo;
            const uint64_t key = ((uint64_t)(a < b ? a : b) << 32) | (a < b ? b : a);
            uint64_t s = mix64(key) & h.mask;
            while (h.key[s] != UINT64_MAX && h.key[s] != key) s = (s + 1) & h.mask;
            if (h.key[s] == UINT64_MAX) {
                h.key[s] = key;
                h.val[s] = ne;
                E[ne].q = a; E[ne].r = b; E[ne].f0 = f; E[ne].f1 = UINT32_MAX;
                ++ne;
            } else if (E[h.val[s]].f1 == UINT32_MAX && E[h.val[s]].f0 != f) {
                E[h.val[s]].f1 = f;
            }
        }
    }
    /* records in canonical order */
    rord_t *ord = (rord_t *)malloc(sizeof(rord_t) * (size_t)(nr ? nr : 1));
    int bad = 0;
    for (int64_t i = 0; i < nr; ++i) {
        const uint32_t a = rec3[3 * i], b = rec3[3 * i + 1];
        const uint64_t key = ((uint64_t)(a < b ? a : b) << 32) | (a < b ? b : a);
        uint64_t s = mix64(key) & h.mask;
        while (h.key[s] != UINT64_MAX && h.key[s] != key) s = (s + 1) & h.mask;
        if (h.key[s] == UINT64_MAX) { bad = 1; ord[i].edge = 0; }
        else ord[i].edge = h.val[s];
        ord[i].g = rec3[3 * i + 2];
        ord[i].k = (uint32_t)i;
    }
    free(h.key); free(h.val);
    if (bad) { free(ord); free(E); free(S.off); free(Cm.off); return -1; }
    if (nr) qsort(ord, (size_t)nr, sizeof(rord_t), rord_cmp);

    out->n_records = nr;
    out->rec_ids = (uint32_t *)malloc(sizeof(uint32_t) * 5 * (size_t)(nr ? nr : 1));
    out->rec_pts = (double *)malloc(sizeof(double) * 3 * (size_t)(nr ? nr : 1));
    out->edge_off = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)nr + 1));
    out->border = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(nr ? nr : 1));
    kv_t *cp = (kv_t *)malloc(sizeof(kv_t) * 2 * (size_t)(nr ? nr : 1));
    kv_t *fc = (kv_t *)malloc(sizeof(kv_t) * 3 * (size_t)(nr ? nr : 1));
    uint64_t ncp = 0, nfc = 0;
    for (int64_t i = 0; i < nr; ++i) {
        const edge_t *e = &E[ord[i].edge];
        const uint32_t g = ord[i].g, vtx = NV + (uint32_t)i;
        uint32_t *r5 = out->rec_ids + 5 * i;
        r5[0] = e->q; r5[1] = e->r; r5[2] = g; r5[3] = e->f0; r5[4] = e->f1;
        memcpy(out->rec_pts + 3 * i, pts + 3 * (size_t)ord[i].k, sizeof(double) * 3);
        /* ps_intersecting_edges[tested_edge] (kernel.cpp:2609) */
        if (i == 0 || ord[i].edge != ord[i - 1].edge) out->edge_off[out->n_edges++] = (uint32_t)i;
        /* cutpath_edge_creation_info: {source face, cut face} for the tested face
         * and each face of the tested edge (kernel.cpp:2614-2627; utils.h pair
         * orders its two faces, and source faces come first) */
        const int cut_edge = e->q >= nsv; /* the edge's vertices are cut-mesh vertices */
        const uint32_t ef[2] = { e->f0, e->f1 };
        for (int k = 0; k < 2; ++k) {
            if (ef[k] == UINT32_MAX) continue;
            const uint32_t sface = cut_edge ? g : ef[k], cface = cut_edge ? ef[k] : g;
            cp[ncp].key = ((uint64_t)sface << 32) | cface;
            cp[ncp++].vtx = vtx;
        }
        /* ps_iface_to_ivtx_list (kernel.cpp:2638-2644) */
        fc[nfc].key = g; fc[nfc++].vtx = vtx;
        for (int k = 0; k < 2; ++k)
            if (ef[k] != UINT32_MAX) { fc[nfc].key = ef[k]; fc[nfc++].vtx = vtx; }
        /* cm_border_reentrant_ivtx_list / partial_cut_detected (kernel.cpp:2629-2650) */
        if (cut_edge && e->f1 == UINT32_MAX) out->border[out->n_border++] = vtx;
    }
    out->edge_off[out->n_edges] = (uint32_t)nr;
    qsort(cp, (size_t)ncp, sizeof(kv_t), kv_cmp);
    qsort(fc, (size_t)nfc, sizeof(kv_t), kv_cmp);
    out->n_cutpath = kv_runs(cp, ncp, &out->cp_pairs, 1, &out->cp_off, &out->cp_vtx);
    out->n_faces = kv_runs(fc, nfc, &out->face_keys, 0, &out->face_off, &out->face_vtx);
    free(cp); free(fc); free(ord); free(E); free(S.off); free(Cm.off);
    return 0;
}

void oracle_seam_free(fe_seam *s)
{
    free(s->rec_ids); free(s->rec_pts); free(s->edge_off); free(s->cp_pairs); free(s->cp_off); free(s->cp_vtx);
    free(s->face_keys); free(s->face_off); free(s->face_vtx); free(s->border);
    memset(s, 0, sizeof *s);
}
