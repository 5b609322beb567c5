// eig_sturm.cuh -- eigenvalues of one unreduced symmetric tridiagonal block by
// bisection on Sturm counts, in FP32 and in double-float arithmetic.
//
// GB300 issues FP64 at 1/64 of the FP32 rate, so the counts avoid FP64 altogether:
//   - Determinant form of the Sturm sequence, p_0 = 1, p_1 = d_0 - x,
//     p_i = (d_{i-1} - x) p_{i-1} - e2_{i-2} p_{i-2}; the count of eigenvalues below x
//     is the number of sign changes along p_0 .. p_m.  No division (the ratio form
//     q_i = p_i / p_{i-1} of LAPACK's dstebz needs one per step).  Each computed p_i
//     is exact for d and e2 perturbed by a few units in the last place, so the count
//     is that of a nearby matrix (Wilkinson's backward analysis of the recurrence).
//   - The block is scaled by a power of two so that its Gershgorin norm lies in
//     [1/2, 1); then |p_i| <= 2^i, and the pair (p_i, p_{i-1}) is rescaled by 2^-+64
//     whenever |p_i| leaves [2^-40, 2^40], which keeps both inside the FP32 range.
//   - FP32 counts bracket each eigenvalue to ~1e-6 of the norm; double-float counts
//     (hi + lo pairs of FP32, ~48-bit significands; Dekker's and Knuth's error-free
//     sum and product, the product through FMA) check the bracket and finish it.
//     Once the bracket holds only the wanted eigenvalue, the double-float value of
//     p_m(x) = det(T - x I) drives regula falsi with the Illinois modification
//     (Dowell and Jarratt, BIT 11 (1971) 168), which converges superlinearly; else
//     the bracket is trisected.  Every pass evaluates several points at once (their
//     recurrences interleave in one thread).  Stopping rule: bracket width
//     <= max(1e-12 |W|, 1e-13 |T_b|), then W is the bracket's midpoint.
//
// Host- and device-compilable: the same arithmetic is checked on the CPU against
// LAPACK.  The error-free transformations use explicitly rounded operations so the
// compiler cannot contract them into FMAs.
#pragma once
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define BD_HD __host__ __device__ __forceinline__
#else
#define BD_HD inline
#endif

namespace bd {
namespace sturm {

BD_HD float add_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

BD_HD float mul_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

BD_HD float fma_rn(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

BD_HD unsigned sign_bit(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x) >> 31;
#else
    unsigned u;
    memcpy(&u, &x, sizeof u);
    return u >> 31;
#endif
}

// 2^e for -126 <= e <= 127
BD_HD float pow2f(int e) {
    const unsigned u = (unsigned)(e + 127) << 23;
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
#endif
}

// 2^e for -1022 <= e <= 1023
BD_HD double pow2(int e) {
    const unsigned long long u = (unsigned long long)(e + 1023) << 52;
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double f;
    memcpy(&f, &u, sizeof f);
    return f;
#endif
}

// FP32 rounding of x towards -inf / +inf
BD_HD float f_down(double x) {
#if defined(__CUDA_ARCH__)
    return __double2float_rd(x);
#else
    float f = (float)x;
    if ((double)f > x) f = nextafterf(f, -INFINITY);
    return f;
#endif
}

BD_HD float f_up(double x) {
#if defined(__CUDA_ARCH__)
    return __double2float_ru(x);
#else
    float f = (float)x;
    if ((double)f < x) f = nextafterf(f, INFINITY);
    return f;
#endif
}

// Gershgorin interval [lo, hi] of row i and its absolute row sum rn, from d_i and the
// moduli of its two off-diagonals inside the block (0 at the block's ends)
BD_HD void gershgorin_row(double d, double el, double er, float &lo, float &hi, float &rn) {
    const double r = el + er;
    lo = f_down(d - r);
    hi = f_up(d + r);
    rn = f_up(fabs(d) + r);
}

// Relative split test of the QR and bisection codes: off-diagonal e between d0 and d1
// is negligible when |e| <= eps (|d0| + |d1|), below the rounding of T.
BD_HD bool negligible(double e, double d0, double d1) {
    return fabs(e) <= 2.220446049250313e-16 * (fabs(d0) + fabs(d1));
}

// Exponent s with 2^-s t in [1/2, 1) (0 for t == 0)
BD_HD int scale_exponent(float t) {
    int e = 0;
    if (t > 0.0f) frexpf(t, &e);
    return e;
}

// s + e == a + b exactly (Knuth's two-sum)
BD_HD void two_sum(float a, float b, float &s, float &e) {
    s = add_rn(a, b);
    const float bb = add_rn(s, -a);
    e = add_rn(add_rn(a, -add_rn(s, -bb)), add_rn(b, -bb));
}

// Split of a double into hi + lo floats (hi the FP32 rounding, lo the rounding of the rest).
BD_HD void split(double x, float &h, float &l) {
    h = (float)x;
    l = (float)(x - (double)h);
}

// FP32 count of eigenvalues below x (d, e2 of a scaled block of order m >= 1).
BD_HD int count_f(const float *d, const float *e2, int m, float x) {
    float pp = 1.0f, p = d[0] - x;
    int c = (int)sign_bit(p);
    for (int i = 1; i < m; ++i) {
        const float np = fmaf(d[i] - x, p, -(e2[i - 1] * pp));
        c += (int)(sign_bit(np) ^ sign_bit(p));
        pp = p;
        p = np;
        const float a = fabsf(p);
        if (a > 0x1p40f) { p *= 0x1p-64f; pp *= 0x1p-64f; }
        else if (a < 0x1p-40f) { p *= 0x1p64f; pp *= 0x1p64f; }
    }
    return c;
}

// Double-float count of eigenvalues below x = xh + xl; also p_m(x) as fh * 2^fe
// (fh the hi part).  A zero p_i counts with the sign its bits carry: the change it
// adds or drops at i is returned at i + 1, where p_{i+1} = -e2 p_{i-1}.
BD_HD int count_df(const float *dh, const float *dl, const float *eh, const float *el, int m, float xh, float xl,
                   float *fh, int *fe) {
    float ph, pl;
    {
        float s, r;
        two_sum(dh[0], -xh, s, r);
        r = add_rn(r, add_rn(dl[0], -xl));
        two_sum(s, r, ph, pl);
    }
    float qh = 1.0f, ql = 0.0f;   // p_{i-1}
    int c = (int)sign_bit(ph), E = 0;
    for (int i = 1; i < m; ++i) {
        // t = d_i - x, left unnormalised: where the hi parts cancel, |t| < 2^-23 |d_i|
        // and an FP32-relative error in t * p stays below 2^-47 |d_i| |p|
        float th, tl;
        two_sum(dh[i], -xh, th, tl);
        tl = add_rn(tl, add_rn(dl[i], -xl));
        const float ah = mul_rn(th, ph);
        float al = fma_rn(th, ph, -ah);
        al = fma_rn(th, pl, al);
        al = fma_rn(tl, ph, al);
        const float g = eh[i - 1], gl = el[i - 1];
        const float bh = mul_rn(g, qh);
        float bl = fma_rn(g, qh, -bh);
        bl = fma_rn(g, ql, bl);
        bl = fma_rn(gl, qh, bl);
        float s, r;
        two_sum(ah, -bh, s, r);
        r = add_rn(r, add_rn(al, -bl));
        float nh, nl;
        two_sum(s, r, nh, nl);
        c += (int)(sign_bit(nh) ^ sign_bit(ph));
        qh = ph; ql = pl;
        ph = nh; pl = nl;
        const float a = fabsf(ph);
        if (a > 0x1p40f) {
            ph *= 0x1p-64f; pl *= 0x1p-64f; qh *= 0x1p-64f; ql *= 0x1p-64f; E += 64;
        } else if (a < 0x1p-40f && a != 0.0f) {
            ph *= 0x1p64f; pl *= 0x1p64f; qh *= 0x1p64f; ql *= 0x1p64f; E -= 64;
        }
    }
    *fh = ph;
    *fe = E;
    return c;
}

// Evaluators of four points per pass.  LaneEval4 (device): four lanes of a warp each
// count one point and exchange the results by shuffles within their group.
// SeqEval4 (host and device): one thread counts the four points one after another.
// The bisection below is written against either, so the host check runs the same
// driver as the device.
struct SeqEval4 {
    const float *dh, *dl, *eh, *el;
    int m;
    BD_HD void f(const float *x, int *c) const {
        for (int j = 0; j < 4; ++j) c[j] = count_f(dh, eh, m, x[j]);
    }
    BD_HD void df(const double *x, int *c, float *fh, int *fe) const {
        for (int j = 0; j < 4; ++j) {
            float h, l;
            split(x[j], h, l);
            c[j] = count_df(dh, dl, eh, el, m, h, l, &fh[j], &fe[j]);
        }
    }
};

#if defined(__CUDACC__)
struct LaneEval4 {
    const float *dh, *dl, *eh, *el;
    int m;
    int sub;          // this lane's point, 0..3
    int base;         // lane index of the group's first lane
    unsigned mask;    // the group's four lanes
    __device__ void f(const float *x, int *c) const {
        const int mine = count_f(dh, eh, m, x[sub]);
#pragma unroll
        for (int j = 0; j < 4; ++j) c[j] = __shfl_sync(mask, mine, base + j);
    }
    __device__ void df(const double *x, int *c, float *fh, int *fe) const {
        float h, l, f;
        int e;
        split(x[sub], h, l);
        const int mine = count_df(dh, dl, eh, el, m, h, l, &f, &e);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            c[j] = __shfl_sync(mask, mine, base + j);
            fh[j] = __shfl_sync(mask, f, base + j);
            fe[j] = __shfl_sync(mask, e, base + j);
        }
    }
};
#endif

// Eigenvalue k (0-based, ascending) of a block of order m >= 2 given scaled by
// 2^-sexp (the evaluator holds d = dh + dl and e2 = eh + el), Gershgorin bounds
// [glo, ghi] of the scaled block (outward rounded).  Returns it unscaled; *nev counts
// the double-float passes.
//
// Four points per pass.  FP32 stage: the bracket shrinks fivefold per pass, to 2^-20
// of the scaled norm.  Double-float stage: fivefold sections until the bracket holds
// eigenvalue k alone; then the regula falsi point x of the determinant with x -+ delta
// and the bracket's midpoint, delta the last move of x (at first 1e-3 of the bracket;
// at least tol / 2), so that the points usually straddle the root closely.  A pass
// that moves one end only halves the other end's determinant (the Illinois rule).
// Stopping rule: width <= max(1e-12 |W|, 1e-13 |T_b|); W is the bracket's midpoint.
template <class Ev>
BD_HD double bisect4(const Ev &ev, int k, float glo, float ghi, int sexp, int *nev) {
    const double tn = fmax(fabs((double)glo), fabs((double)ghi));
    const double g0 = (double)glo - 0x1p-45, g1 = (double)ghi + 0x1p-45;
    float af = glo, bf = ghi;
    for (int it = 0; it < 20 && bf - af > 0x1p-20f; ++it) {
        float xs[4];
        int cs[4];
        const float wd = bf - af;
        for (int j = 0; j < 4; ++j) xs[j] = af + wd * (0.2f * (float)(j + 1));
        ev.f(xs, cs);
        float na = af, nb = bf;
        for (int j = 0; j < 4; ++j) if (cs[j] <= k && xs[j] > na && xs[j] < bf) na = xs[j];
        for (int j = 3; j >= 0; --j) if (cs[j] > k && xs[j] < nb && xs[j] > af) nb = xs[j];
        if (!(na < nb) || (na == af && nb == bf)) break;   // FP32 rounding or no progress
        af = na; bf = nb;
    }
    double a = fmax(g0, (double)af - 4e-6), b = fmin(g1, (double)bf + 4e-6);
    float fah = 0.0f, fbh = 0.0f;
    int fae = 0, fbe = 0, ca = 0, cb = 0;
    double xs[4];
    int c[4], fe[4];
    float fh[4];
    // both ends and the two trisection points in the first pass
    auto first = [&](double lo, double hi) {
        xs[0] = lo; xs[1] = lo + (hi - lo) / 3.0; xs[2] = lo + 2.0 * (hi - lo) / 3.0; xs[3] = hi;
        ev.df(xs, c, fh, fe);
        ca = c[0]; fah = fh[0]; fae = fe[0]; cb = c[3]; fbh = fh[3]; fbe = fe[3];
    };
    first(a, b);
    int ne = 1;
    if (!(ca <= k && cb > k)) {   // the FP32 bracket missed: start over from Gershgorin
        a = g0; b = g1;
        first(a, b);
        ++ne;
    }
    // the two interior points of the first pass
    for (int j = 1; j <= 2; ++j) {
        if (c[j] <= k && xs[j] > a) { a = xs[j]; ca = c[j]; fah = fh[j]; fae = fe[j]; }
    }
    for (int j = 2; j >= 1; --j) {
        if (c[j] > k && xs[j] < b) { b = xs[j]; cb = c[j]; fbh = fh[j]; fbe = fe[j]; }
    }
    double xprev = 0.0;
    bool have_prev = false;
    for (int it = 0; it < 200; ++it) {
        const double tol = fmax(1e-12 * fmax(fabs(a), fabs(b)), 1e-13 * tn);
        if (b - a <= tol) break;
        const double mid = 0.5 * (a + b);
        if (mid == a || mid == b) break;
        const bool rf = (ca == k && cb == k + 1);
        if (rf) {
            // regula falsi: x = a + (b - a) f(a) / (f(a) - f(b)), f(b) / f(a) < 0
            int de = fbe - fae;
            de = de < -120 ? -120 : (de > 120 ? 120 : de);
            const float r = (fbh / fah) * pow2f(de);
            const float wgt = 1.0f / (1.0f - r);
            double x = a + (double)wgt * (b - a);
            if (!(x > a && x < b)) x = mid;
            const double lo = a + 0.5 * tol, hi = b - 0.5 * tol;
            x = fmin(fmax(x, lo), hi);
            const double delta = fmax(have_prev ? fabs(x - xprev) : 1e-3 * (b - a), 0.5 * tol);
            xprev = x;
            have_prev = true;
            xs[0] = fmin(fmax(x - delta, lo), hi);
            xs[1] = x;
            xs[2] = fmin(fmax(x + delta, lo), hi);
            xs[3] = mid;
        } else {
            for (int j = 0; j < 4; ++j) xs[j] = a + (b - a) * (0.2 * (double)(j + 1));
            have_prev = false;
        }
        ev.df(xs, c, fh, fe);
        ++ne;
        const double a_old = a, b_old = b;
        for (int j = 0; j < 4; ++j)
            if (c[j] <= k && xs[j] > a && xs[j] < b_old) { a = xs[j]; ca = c[j]; fah = fh[j]; fae = fe[j]; }
        for (int j = 0; j < 4; ++j)
            if (c[j] > k && xs[j] < b && xs[j] > a_old) { b = xs[j]; cb = c[j]; fbh = fh[j]; fbe = fe[j]; }
        if (rf) {   // one end moved only: the stale end's value halves (Illinois)
            if (a == a_old && b != b_old) fah *= 0.5f;
            if (b == b_old && a != a_old) fbh *= 0.5f;
        }
    }
    if (nev) *nev = ne;
    return 0.5 * (a + b) * pow2(sexp);
}

}  // namespace sturm
}  // namespace bd
