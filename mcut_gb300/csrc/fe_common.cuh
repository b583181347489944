// Shared device code of the GB300 intersection front end.
//
// Everything here is compiled with --fmad=false: each a*b+c is two IEEE
// roundings, as in the reference's x86 build. That is what keeps face planes,
// intersection points and the point-in-polygon arithmetic bit-identical to
// math.cpp, and what the error-free transforms of the exact predicates need.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mcut_gb300.h"

namespace mcgpu {

constexpr uint32_t kNone = 0xFFFFFFFFu;

// status word bits (device-side, one uint32 per dispatch)
enum : uint32_t {
    ST_GP = 1u,               // a test violated general position
    ST_OVERFLOW_PAIRS = 2u,   // candidate-pair buffer too small
    ST_OVERFLOW_TESTS = 4u,   // edge-face test buffer too small
    ST_STACK = 8u,            // traversal stack overflow (re-run deep)
    ST_INVALID = 16u,         // invalid input (a vertex index out of range)
};

// ---------------------------------------------------------------------------
// fp64 boxes: bounding_box_t / intersect_bounding_boxes (math.h:866-943)
// ---------------------------------------------------------------------------
struct Box {
    double mn[3], mx[3];
};

// (a < b) for non-NaN doubles on the integer pipe: order-preserving bits,
// except that -0 and +0 compare equal as in IEEE. GB300's fp64 pipe runs at a
// small fraction of its integer / fp32 rate, so box code avoids it.
__device__ __forceinline__ bool dlt_int(double a, double b)
{
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const long long oa = ia < 0 ? (long long)(0x8000000000000000ull - (unsigned long long)ia) : ia;
    const long long ob = ib < 0 ? (long long)(0x8000000000000000ull - (unsigned long long)ib) : ib;
    return oa < ob;
}
// fp64 -> fp32 rounded toward -inf / +inf with integer operations only (the
// fp64 pipe's conversions are slow here, and a predicated conversion still
// occupies it): normal results, subnormal results, overflow to +-FLT_MAX or
// +-inf, and inf / NaN passed through.
__device__ __forceinline__ float f32_round(double x, bool up)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
    const unsigned sign = (unsigned)(b >> 63);
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    const bool away = (sign != 0) != up; // rounding away from zero is toward the requested infinity
    unsigned fb;
    if (e == 0x7FFu) {
        fb = (sign << 31) | 0x7F800000u | (m ? 0x00400000u : 0u);
    } else if (e > 1023u + 127u) {
        fb = (sign << 31) | (away ? 0x7F800000u : 0x7F7FFFFFu);
    } else if (e >= 1023u - 126u) {
        fb = (sign << 31) | ((e - 1023u + 127u) << 23) | (unsigned)(m >> 29);
        if (away && (m & 0x1FFFFFFFull) != 0) fb += 1u;
    } else {
        // below fp32's normal range: a multiple of 2^-149 (or zero)
        const unsigned long long sig = e ? (m | (1ull << 52)) : m;
        const unsigned sh = 926u - (e ? e : 1u);       // >= 30
        const unsigned long long q = sh >= 64u ? 0ull : (sig >> sh);
        const bool inexact = sh >= 64u ? sig != 0 : (sig & ((1ull << sh) - 1ull)) != 0;
        fb = (sign << 31) | (unsigned)q;
        if (away && inexact) fb += 1u;
    }
    return __uint_as_float(fb);
}
__device__ __forceinline__ float f32_rd(double x) { return f32_round(x, false); }
__device__ __forceinline__ float f32_ru(double x) { return f32_round(x, true); }

// the same order as a signed integer key: dlt_int(a, b) == (dkey(a) < dkey(b))
__device__ __forceinline__ long long dkey(double a)
{
    const long long ia = __double_as_longlong(a);
    return ia < 0 ? (long long)(0x8000000000000000ull - (unsigned long long)ia) : ia;
}
__device__ __forceinline__ double dmax_ref(double a, double b) { return dlt_int(a, b) ? b : a; }  // std::max
__device__ __forceinline__ double dmin_ref(double a, double b) { return dlt_int(b, a) ? b : a; }  // std::min

// closed box overlap (intersect_bounding_boxes, math.h:931-943) on dkey()
// integers: the IEEE order of non-NaN doubles (-0 == +0), off the fp64 pipe
__device__ __forceinline__ bool box_overlap(const Box& a, const Box& b)
{
    bool ov = true;
    for (int j = 0; j < 3; ++j) ov &= dkey(a.mn[j]) <= dkey(b.mx[j]) && dkey(a.mx[j]) >= dkey(b.mn[j]);
    return ov;
}

__device__ __forceinline__ Box load_box(const double* __restrict__ boxes, uint32_t f)
{
    const double2* p = reinterpret_cast<const double2*>(boxes + (size_t)f * 6);
    double2 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    Box r;
    r.mn[0] = a.x; r.mn[1] = a.y; r.mn[2] = b.x;
    r.mx[0] = b.y; r.mx[1] = c.x; r.mx[2] = c.y;
    return r;
}

__device__ __forceinline__ void load_xyz(const double* __restrict__ X, uint32_t v, double* p)
{
    const double* s = X + (size_t)v * 3;
    p[0] = __ldg(s);
    p[1] = __ldg(s + 1);
    p[2] = __ldg(s + 2);
}

// dot_product: out = 0; out += a[i]*b[i]  (math.h:635-643)
__device__ __forceinline__ double dot3(const double* a, const double* b)
{
    double o = 0.0;
    o = o + a[0] * b[0];
    o = o + a[1] * b[1];
    o = o + a[2] * b[2];
    return o;
}

// order-preserving map of a double onto uint64 (for atomic min / max)
__device__ __forceinline__ unsigned long long ord_of(double x)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ inline double of_ord(unsigned long long u)
{
    u = (u & 0x8000000000000000ull) ? (u & 0x7FFFFFFFFFFFFFFFull) : ~u;
    union { unsigned long long i; double d; } c;
    c.i = u;
    return c.d;
}

// ---------------------------------------------------------------------------
// Expansion arithmetic (Shewchuk, DCG 18:305-363, 1997, section 2)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(double a, double b, double& x, double& y)
{
    double s = a + b, bv = s - a, av = s - bv;
    x = s;
    y = (a - av) + (b - bv);
}
__device__ __forceinline__ void fast_two_sum(double a, double b, double& x, double& y)
{
    double s = a + b;
    x = s;
    y = b - (s - a);
}
__device__ __forceinline__ void two_diff(double a, double b, double& x, double& y)
{
    double s = a - b, bv = a - s, av = s + bv;
    x = s;
    y = (a - av) + (bv - b);
}
__device__ __forceinline__ double two_diff_tail(double a, double b, double x)
{
    double bv = a - x, av = x + bv;
    return (a - av) + (bv - b);
}
__device__ __forceinline__ void split(double a, double& hi, double& lo)
{
    double c = 134217729.0 * a, big = c - a;
    hi = c - big;
    lo = a - hi;
}
__device__ __forceinline__ void two_product(double a, double b, double& x, double& y)
{
    double p = a * b, ah, al, bh, bl;
    split(a, ah, al);
    split(b, bh, bl);
    double e1 = p - ah * bh, e2 = e1 - al * bh, e3 = e2 - ah * bl;
    x = p;
    y = al * bl - e3;
}
__device__ __forceinline__ void two_two_diff(double a1, double a0, double b1, double b0, double* x)
{
    double i, j, k0;
    two_diff(a0, b0, i, x[0]);
    two_sum(a1, i, j, k0);
    two_diff(k0, b1, i, x[1]);
    two_sum(j, i, x[3], x[2]);
}
__device__ inline int fast_expansion_sum_zeroelim(int elen, const double* e, int flen, const double* f, double* h)
{
    int ei = 0, fi = 0, hi = 0;
    double q, qn, hh, en = e[0], fn = f[0];
    if ((fn > en) == (fn > -en)) { q = en; ++ei; en = ei < elen ? e[ei] : 0.0; }
    else { q = fn; ++fi; fn = fi < flen ? f[fi] : 0.0; }
    if (ei < elen && fi < flen) {
        if ((fn > en) == (fn > -en)) { fast_two_sum(en, q, qn, hh); ++ei; en = ei < elen ? e[ei] : 0.0; }
        else { fast_two_sum(fn, q, qn, hh); ++fi; fn = fi < flen ? f[fi] : 0.0; }
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
        while (ei < elen && fi < flen) {
            if ((fn > en) == (fn > -en)) { two_sum(q, en, qn, hh); ++ei; en = ei < elen ? e[ei] : 0.0; }
            else { two_sum(q, fn, qn, hh); ++fi; fn = fi < flen ? f[fi] : 0.0; }
            q = qn;
            if (hh != 0.0) h[hi++] = hh;
        }
    }
    while (ei < elen) {
        two_sum(q, en, qn, hh); ++ei; en = ei < elen ? e[ei] : 0.0;
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
    }
    while (fi < flen) {
        two_sum(q, fn, qn, hh); ++fi; fn = fi < flen ? f[fi] : 0.0;
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
    }
    if (q != 0.0 || hi == 0) h[hi++] = q;
    return hi;
}
__device__ inline int scale_expansion_zeroelim(int elen, const double* e, double b, double* h)
{
    double q, sum, hh, bh, bl, ah, al;
    int hi = 0;
    split(b, bh, bl);
    {
        double p = e[0] * b;
        split(e[0], ah, al);
        double e1 = p - ah * bh, e2 = e1 - al * bh, e3 = e2 - ah * bl;
        q = p;
        hh = al * bl - e3;
    }
    if (hh != 0.0) h[hi++] = hh;
    for (int i = 1; i < elen; ++i) {
        double p = e[i] * b;
        split(e[i], ah, al);
        double e1 = p - ah * bh, e2 = e1 - al * bh, e3 = e2 - ah * bl;
        double p0 = al * bl - e3;
        two_sum(q, p0, sum, hh);
        if (hh != 0.0) h[hi++] = hh;
        fast_two_sum(p, sum, q, hh);
        if (hh != 0.0) h[hi++] = hh;
    }
    if (q != 0.0 || hi == 0) h[hi++] = q;
    return hi;
}

// ---------------------------------------------------------------------------
// orient3d sign: FP32 filter -> FP64 filter -> exact (the reference returns
// Shewchuk's adaptive value, shewchuk.c:2367-2407, of which only the sign is
// read, math.cpp:391-427)
// ---------------------------------------------------------------------------
static __device__ __noinline__ int orient3d_exact_sign(const double* pa, const double* pb, const double* pc, const double* pd)
{
    double ab[4], bc[4], cd[4], da[4], ac[4], bd[4], t8[8], abc[12], bcd[12], cda[12], dab[12];
    double adet[24], bdet[24], cdet[24], ddet[24], abd[48], cdd[48], det[96];
    auto cross2 = [](const double* p, const double* q, double* o) {
        double a1, a0, b1, b0;
        two_product(p[0], q[1], a1, a0);
        two_product(q[0], p[1], b1, b0);
        two_two_diff(a1, a0, b1, b0, o);
    };
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

// Shewchuk's adaptive stages B and C (orient3dadapt, shewchuk.c:1962-2085),
// between the fp64 filter and the full exact expansion. B: the determinant of
// the rounded differences as an exact expansion (three 2x2 minors, each
// scaled by a z difference, summed); its estimate decides past
// o3derrboundB * permanent, and when all nine differences were exact (zero
// tails) the expansion is the determinant itself, so its top component's
// sign is the exact sign. C: the tails' first-order terms added to the
// estimate, deciding past o3derrboundC * permanent + resulterrbound * |det|
// (shewchuk.c:394-400 for the bounds, epsilon = 2^-53). Returns 2 when
// neither decides. Same comparisons as the reference (>=), whose value's sign
// is what it reads.
static __device__ __noinline__ int orient3d_sign_bc(const double* pa, const double* pb, const double* pc,
    const double* pd, double perm)
{
    const double EPS = 1.1102230246251565e-16;
    const double O3D_B = (3.0 + 28.0 * EPS) * EPS, O3D_C = (26.0 + 288.0 * EPS) * EPS * EPS,
                 RES = (3.0 + 8.0 * EPS) * EPS;
    const double adx = pa[0] - pd[0], bdx = pb[0] - pd[0], cdx = pc[0] - pd[0];
    const double ady = pa[1] - pd[1], bdy = pb[1] - pd[1], cdy = pc[1] - pd[1];
    const double adz = pa[2] - pd[2], bdz = pb[2] - pd[2], cdz = pc[2] - pd[2];
    double bc[4], ca[4], ab[4], adet[8], bdet[8], cdet[8], abdet[16], fin[24];
    auto minor2 = [](double p, double q, double r, double s, double* o) { // p q - r s, exactly
        double a1, a0, b1, b0;
        two_product(p, q, a1, a0);
        two_product(r, s, b1, b0);
        two_two_diff(a1, a0, b1, b0, o);
    };
    minor2(bdx, cdy, cdx, bdy, bc);
    minor2(cdx, ady, adx, cdy, ca);
    minor2(adx, bdy, bdx, ady, ab);
    const int al = scale_expansion_zeroelim(4, bc, adz, adet);
    const int bl = scale_expansion_zeroelim(4, ca, bdz, bdet);
    const int cl = scale_expansion_zeroelim(4, ab, cdz, cdet);
    const int abl = fast_expansion_sum_zeroelim(al, adet, bl, bdet, abdet);
    const int n = fast_expansion_sum_zeroelim(abl, abdet, cl, cdet, fin);
    double det = fin[0];
    for (int i = 1; i < n; ++i) det += fin[i];
    double eb = O3D_B * perm;
    if (det >= eb || -det >= eb) return det > 0.0 ? 1 : (det < 0.0 ? -1 : 0);
    const double adxt = two_diff_tail(pa[0], pd[0], adx), bdxt = two_diff_tail(pb[0], pd[0], bdx),
                 cdxt = two_diff_tail(pc[0], pd[0], cdx);
    const double adyt = two_diff_tail(pa[1], pd[1], ady), bdyt = two_diff_tail(pb[1], pd[1], bdy),
                 cdyt = two_diff_tail(pc[1], pd[1], cdy);
    const double adzt = two_diff_tail(pa[2], pd[2], adz), bdzt = two_diff_tail(pb[2], pd[2], bdz),
                 cdzt = two_diff_tail(pc[2], pd[2], cdz);
    if (adxt == 0.0 && bdxt == 0.0 && cdxt == 0.0 && adyt == 0.0 && bdyt == 0.0 && cdyt == 0.0 && adzt == 0.0
        && bdzt == 0.0 && cdzt == 0.0) {
        const double top = fin[n - 1];
        return top > 0.0 ? 1 : (top < 0.0 ? -1 : 0);
    }
    eb = O3D_C * perm + RES * fabs(det);
    det += (adz * ((bdx * cdyt + cdy * bdxt) - (bdy * cdxt + cdx * bdyt)) + adzt * (bdx * cdy - bdy * cdx))
        + (bdz * ((cdx * adyt + ady * cdxt) - (cdy * adxt + adx * cdyt)) + bdzt * (cdx * ady - cdy * adx))
        + (cdz * ((adx * bdyt + bdy * adxt) - (ady * bdxt + bdx * adyt)) + cdzt * (adx * bdy - ady * bdx));
    if (det >= eb || -det >= eb) return det > 0.0 ? 1 : (det < 0.0 ? -1 : 0);
    return 2;
}

// Which stage decided a sign (escalation counters).
enum { ESC_F32 = 0, ESC_F64 = 1, ESC_EXACT = 2 };

// FP32 filter. The nine differences are formed in fp64 and rounded once to
// fp32 to nearest (relative error <= u(1+2^-28), u = 2^-24), by integer
// operations (fp64 conversions run at the fp64 rate). Shewchuk's stage-A
// analysis with that per-input error and u per fp32 operation gives
// |det - det_exact| <= (7u + 56u^2) * permanent; 8u covers the slightly
// larger input error. The filter only runs when every nonzero difference
// lies in [2^-40, 2^41). Then the permanent, a sum of six products each
// < 2^123, stays below 2^126 (no overflow), and a nonzero permanent is at
// least 2^-120: the bound's slack over 7u, u * permanent >= 2^-144, covers
// the absolute error of the at most five operations whose result can be
// subnormal (<= 2^-150 each; a subnormal difference of products is exact).
// Otherwise, or when the bound is not met, it escalates.
__device__ __forceinline__ bool f32_filter_input(double d, float& f)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    if ((b << 1) == 0ull) {
        f = 0.0f;
        return true;
    }
    const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
    if (e < 1023u - 40u || e > 1023u + 40u) return false;
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    unsigned fb = ((unsigned)(b >> 63) << 31) | ((e - 1023u + 127u) << 23) | (unsigned)(m >> 29);
    const unsigned r = (unsigned)(m & 0x1FFFFFFFull);
    if (r > 0x10000000u || (r == 0x10000000u && (fb & 1u))) fb += 1u; // to nearest, ties to even
    f = __uint_as_float(fb);
    return true;
}
// A coordinate's fp32 copy for the fp32-vertex filter below: zero stays zero,
// a magnitude in [2^-100, 2^40) is rounded to nearest (ties to even) with
// integer operations (normal in fp32 either way), anything else becomes NaN,
// which sends every test touching the vertex to the next stage.
__device__ __forceinline__ float f32_vertex_coord(double x)
{
    // on the two 32-bit halves: sign | exponent (11) | mantissa high (20) and mantissa low (32)
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    if (((hi << 1) | lo) == 0u) return 0.0f;
    const unsigned e = (hi >> 20) & 0x7FFu;
    if (e < 1023u - 100u || e > 1023u + 39u) return __uint_as_float(0x7FC00000u);
    unsigned fb = (hi & 0x80000000u) | ((e - 1023u + 127u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const unsigned r = lo & 0x1FFFFFFFu;
    if (r > 0x10000000u || (r == 0x10000000u && (fb & 1u))) fb += 1u; // a carry moves into the exponent
    return __uint_as_float(fb);
}

// Stage 0: orient3d's sign from the fp32 vertex copies, or 0 to escalate.
// Differences s = fl(P~ - D~) of the rounded coordinates miss the true ones
// by at most E = c (|s| + |P~| + |D~|) (c = 2^-24 (1 + 2^-20) covers the
// coordinate rounding, the difference's rounding and E's own evaluation);
// with M = |s| + E each monomial t_a t_b t_c of the determinant lies within
// E_a M_b M_c + M_a E_b M_c + M_a M_b E_c of s_a s_b s_c (delta, summed over
// the six monomials), and Shewchuk's stage-A bound covers the fp32
// evaluation, 8u times the permanent of the M values. The bound's own
// evaluation (products and sums of non-negative values) is covered by the
// factor 1 + 2^-20, underflow by 2^-140; coordinates below 2^40 keep every
// product below 2^128. tests/test_fp32_vertex_filter.py restates this
// operation for operation and checks it against exact signs.
__device__ __forceinline__ int orient3d_sign_f32v(float4 pa, float4 pb, float4 pc, float4 pd)
{
    const float kC = 0x1.00001p-24f;    // 2^-24 (1 + 2^-20)
    const float kU8 = 0x1p-21f;         // 8 * 2^-24
    const float kGrow = 0x1.00001p0f;   // 1 + 2^-20
    const float kTiny = 0x1p-140f;      // 2^-140 (subnormal)
    const float ax = pa.x - pd.x, ay = pa.y - pd.y, az = pa.z - pd.z;
    const float bx = pb.x - pd.x, by = pb.y - pd.y, bz = pb.z - pd.z;
    const float cx = pc.x - pd.x, cy = pc.y - pd.y, cz = pc.z - pd.z;
    const float det = az * (bx * cy - cx * by) + bz * (cx * ay - ax * cy) + cz * (ax * by - bx * ay);
    const float Eax = kC * ((fabsf(ax) + fabsf(pa.x)) + fabsf(pd.x));
    const float Eay = kC * ((fabsf(ay) + fabsf(pa.y)) + fabsf(pd.y));
    const float Eaz = kC * ((fabsf(az) + fabsf(pa.z)) + fabsf(pd.z));
    const float Ebx = kC * ((fabsf(bx) + fabsf(pb.x)) + fabsf(pd.x));
    const float Eby = kC * ((fabsf(by) + fabsf(pb.y)) + fabsf(pd.y));
    const float Ebz = kC * ((fabsf(bz) + fabsf(pb.z)) + fabsf(pd.z));
    const float Ecx = kC * ((fabsf(cx) + fabsf(pc.x)) + fabsf(pd.x));
    const float Ecy = kC * ((fabsf(cy) + fabsf(pc.y)) + fabsf(pd.y));
    const float Ecz = kC * ((fabsf(cz) + fabsf(pc.z)) + fabsf(pd.z));
    const float Max = fabsf(ax) + Eax, May = fabsf(ay) + Eay, Maz = fabsf(az) + Eaz;
    const float Mbx = fabsf(bx) + Ebx, Mby = fabsf(by) + Eby, Mbz = fabsf(bz) + Ebz;
    const float Mcx = fabsf(cx) + Ecx, Mcy = fabsf(cy) + Ecy, Mcz = fabsf(cz) + Ecz;
    const float P1 = Mbx * Mcy + Mcx * Mby;
    const float Q1 = (Ebx * Mcy + Mbx * Ecy) + (Ecx * Mby + Mcx * Eby);
    const float P2 = Mcx * May + Max * Mcy;
    const float Q2 = (Ecx * May + Mcx * Eay) + (Eax * Mcy + Max * Ecy);
    const float P3 = Max * Mby + Mbx * May;
    const float Q3 = (Eax * Mby + Max * Eby) + (Ebx * May + Mbx * Eay);
    const float permM = Maz * P1 + Mbz * P2 + Mcz * P3;
    const float delta = (Eaz * P1 + Maz * Q1) + (Ebz * P2 + Mbz * Q2) + (Ecz * P3 + Mcz * Q3);
    const float bound = (kU8 * permM + delta) * kGrow + kTiny;
    if (det > bound) return 1;
    if (-det > bound) return -1;
    return 0;
}

__device__ __forceinline__ int orient3d_sign_filtered(const double* pa, const double* pb, const double* pc,
    const double* pd, int& stage)
{
    const double adx = pa[0] - pd[0], bdx = pb[0] - pd[0], cdx = pc[0] - pd[0];
    const double ady = pa[1] - pd[1], bdy = pb[1] - pd[1], cdy = pc[1] - pd[1];
    const double adz = pa[2] - pd[2], bdz = pb[2] - pd[2], cdz = pc[2] - pd[2];
    {
        float ax, bx, cx, ay, by, cy, az, bz, cz;
        const bool ok = f32_filter_input(adx, ax) & f32_filter_input(bdx, bx) & f32_filter_input(cdx, cx)
            & f32_filter_input(ady, ay) & f32_filter_input(bdy, by) & f32_filter_input(cdy, cy)
            & f32_filter_input(adz, az) & f32_filter_input(bdz, bz) & f32_filter_input(cdz, cz);
        if (ok) {
            const float bxcy = bx * cy, cxby = cx * by, cxay = cx * ay, axcy = ax * cy, axby = ax * by, bxay = bx * ay;
            const float det = az * (bxcy - cxby) + bz * (cxay - axcy) + cz * (axby - bxay);
            const float perm = (fabsf(bxcy) + fabsf(cxby)) * fabsf(az) + (fabsf(cxay) + fabsf(axcy)) * fabsf(bz)
                + (fabsf(axby) + fabsf(bxay)) * fabsf(cz);
            const float eb = 4.76837158203125e-07f * perm; // 8 * 2^-24
            if (det > eb) { stage = ESC_F32; return 1; }
            if (-det > eb) { stage = ESC_F32; return -1; }
        }
    }
    const double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy, cdxady = cdx * ady, adxcdy = adx * cdy;
    const double adxbdy = adx * bdy, bdxady = bdx * ady;
    const double det = adz * (bdxcdy - cdxbdy) + bdz * (cdxady - adxcdy) + cdz * (adxbdy - bdxady);
    const double perm = (fabs(bdxcdy) + fabs(cdxbdy)) * fabs(adz) + (fabs(cdxady) + fabs(adxcdy)) * fabs(bdz)
        + (fabs(adxbdy) + fabs(bdxady)) * fabs(cdz);
    const double eb = 7.7715611723761027e-16 * perm; // o3derrboundA
    if (det > eb) { stage = ESC_F64; return 1; }
    if (-det > eb) { stage = ESC_F64; return -1; }
    stage = ESC_EXACT;
    const int s = orient3d_sign_bc(pa, pb, pc, pd, perm);
    if (s != 2) return s;
    return orient3d_exact_sign(pa, pb, pc, pd);
}

// ---------------------------------------------------------------------------
// orient2d with the paper's adaptive stage outputs (value, not just sign):
// its magnitude ranks vertex triplets of polygons (math.cpp:289-389)
// ---------------------------------------------------------------------------
static __device__ __noinline__ double orient2d_adapt(const double* pa, const double* pb, const double* pc, double detsum)
{
    const double EPS = 1.1102230246251565e-16;
    const double CCW_B = (2.0 + 12.0 * EPS) * EPS, CCW_C = (9.0 + 64.0 * EPS) * EPS * EPS,
                 RES = (3.0 + 8.0 * EPS) * EPS;
    double acx = pa[0] - pc[0], bcx = pb[0] - pc[0], acy = pa[1] - pc[1], bcy = pb[1] - pc[1];
    double dl, dlt, dr, drt, B[4], C1[8], C2[12], D[16], u[4], s1, s0, t1, t0;
    two_product(acx, bcy, dl, dlt);
    two_product(acy, bcx, dr, drt);
    two_two_diff(dl, dlt, dr, drt, B);
    double det = B[0];
    for (int i = 1; i < 4; ++i) det += B[i];
    double eb = CCW_B * detsum;
    if (det >= eb || -det >= eb) return det;
    double acxt = two_diff_tail(pa[0], pc[0], acx), bcxt = two_diff_tail(pb[0], pc[0], bcx);
    double acyt = two_diff_tail(pa[1], pc[1], acy), bcyt = two_diff_tail(pb[1], pc[1], bcy);
    if (acxt == 0.0 && acyt == 0.0 && bcxt == 0.0 && bcyt == 0.0) return det;
    eb = CCW_C * detsum + RES * fabs(det);
    det += (acx * bcyt + bcy * acxt) - (acy * bcxt + bcx * acyt);
    if (det >= eb || -det >= eb) return det;
    two_product(acxt, bcy, s1, s0);
    two_product(acyt, bcx, t1, t0);
    two_two_diff(s1, s0, t1, t0, u);
    int c1 = fast_expansion_sum_zeroelim(4, B, 4, u, C1);
    two_product(acx, bcyt, s1, s0);
    two_product(acy, bcxt, t1, t0);
    two_two_diff(s1, s0, t1, t0, u);
    int c2 = fast_expansion_sum_zeroelim(c1, C1, 4, u, C2);
    two_product(acxt, bcyt, s1, s0);
    two_product(acyt, bcxt, t1, t0);
    two_two_diff(s1, s0, t1, t0, u);
    int dn = fast_expansion_sum_zeroelim(c2, C2, 4, u, D);
    return D[dn - 1];
}
__device__ inline double orient2d(const double* pa, const double* pb, const double* pc)
{
    const double CCW_A = 3.3306690738754716e-16;
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

// ---------------------------------------------------------------------------
// Per-face plane record (compute_polygon_plane_coefficients, math.cpp:130-239;
// calculate_projection_matrix, math.cpp:710-793)
// ---------------------------------------------------------------------------
struct FacePlane {
    double n[3];
    double d;
    double P[6];      // 2x3 projection, row major
    int32_t mc;       // largest |n| component
    int32_t tri[3];   // plane-defining vertex positions in the face's vertex list (-1: none)
};

// projection matrix P = K * R (calculate_projection_matrix,
// math.cpp:710-793), with the reference's rounding:
//   a = n / |n|, b = sign(n[mc]) e_mc, R = 2 (a+b)(a+b)^T / (a.b) - diag(1,-1,1)
// (R = diag(1,-1,1) when a == b), K picks rows i != mc of R. Here
//   * a.b == |a[mc]| exactly (b has one nonzero component, +-1) and is at
//     least 3^-1/2, so every entry of R is finite;
//   * (K R)_ij = ((0 + K_i0 R_0j) + K_i1 R_1j) + K_i2 R_2j adds one selected
//     entry to +0 and +-0 terms: it equals R_sj, except that -0 becomes +0;
//   * apb_i apb_j == apb_j apb_i, so the two selected rows need 5 distinct
//     quotients, each rounded exactly as the reference's.
__device__ inline void projection_matrix(const double* nrm, int mc, double* P)
{
    const double len = sqrt(dot3(nrm, nrm));
    const double a[3] = { nrm[0] / len, nrm[1] / len, nrm[2] / len };
    double b[3] = { 0.0, 0.0, 0.0 };
    const int s = (0.0 < nrm[mc]) - (nrm[mc] < 0.0);
    b[mc] = 1.0 * (double)s;
    const int r0 = mc == 0 ? 1 : 0, r1 = mc == 2 ? 1 : 2; // the rows K selects, r0 < r1
    if (a[0] != b[0] || a[1] != b[1] || a[2] != b[2]) {
        const double apb[3] = { a[0] + b[0], a[1] + b[1], a[2] + b[2] };
        const double adb = dot3(a, b);
        double q0[3], q1[3];
        for (int j = 0; j < 3; ++j) q0[j] = (apb[r0] * apb[j]) / adb;
        for (int j = 0; j < 3; ++j) q1[j] = (j == r0) ? q0[r1] : (apb[r1] * apb[j]) / adb;
        for (int j = 0; j < 3; ++j) {
            const double e0 = (q0[j] * 2.0) - ((r0 == j) ? (r0 == 1 ? -1.0 : 1.0) : 0.0);
            const double e1 = (q1[j] * 2.0) - ((r1 == j) ? (r1 == 1 ? -1.0 : 1.0) : 0.0);
            P[j] = e0 == 0.0 ? 0.0 : e0;
            P[3 + j] = e1 == 0.0 ? 0.0 : e1;
        }
    } else {
        for (int j = 0; j < 3; ++j) {
            P[j] = (r0 == j) ? (r0 == 1 ? -1.0 : 1.0) : 0.0;
            P[3 + j] = (r1 == j) ? (r1 == 1 ? -1.0 : 1.0) : 0.0;
        }
    }
}

// matrix_t * vec3 (math.h:508-520)
__device__ __forceinline__ void project2(const double* P, const double* v, double* o)
{
    double r0 = 0.0, r1 = 0.0;
    for (int c = 0; c < 3; ++c) {
        r0 = r0 + P[c] * v[c];
        r1 = r1 + P[3 + c] * v[c];
    }
    o[0] = r0;
    o[1] = r1;
}

} // namespace mcgpu
