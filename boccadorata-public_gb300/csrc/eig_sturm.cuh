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
//     the step is a bisection.  Stopping rule: bracket width <= max(1e-12 |W|,
//     1e-13 |T_b|), then W is the bracket's midpoint.
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

// Eigenvalue k (0-based, ascending) of a block of order m >= 2 given scaled by
// 2^-sexp: d = dh + dl, e2 = eh + el, Gershgorin bounds [glo, ghi] of the scaled
// block (outward rounded).  Returns it unscaled; *nev counts the double-float Sturm
// evaluations.
BD_HD double bisect(const float *dh, const float *dl, const float *eh, const float *el, int m, int k, float glo,
                    float ghi, int sexp, int *nev) {
    const double tn = fmax(fabs((double)glo), fabs((double)ghi));
    const double g0 = (double)glo - 0x1p-45, g1 = (double)ghi + 0x1p-45;
    // FP32 bracket to 2^-20 of the scaled norm; the FP32 rounding of the block moves
    // its eigenvalues by ~1e-7
    float af = glo, bf = ghi;
    for (int it = 0; it < 40 && bf - af > 0x1p-20f; ++it) {
        const float mid = 0.5f * (af + bf);
        if (mid <= af || mid >= bf) break;
        if (count_f(dh, eh, m, mid) > k) bf = mid; else af = mid;
    }
    const double margin = 4e-6;
    double a = fmax(g0, (double)af - margin), b = fmin(g1, (double)bf + margin);
    float fah, fbh, xh, xl;
    int fae, fbe;
    split(a, xh, xl);
    int ca = count_df(dh, dl, eh, el, m, xh, xl, &fah, &fae);
    split(b, xh, xl);
    int cb = count_df(dh, dl, eh, el, m, xh, xl, &fbh, &fbe);
    int ne = 2;
    if (!(ca <= k && cb > k)) {   // the FP32 bracket missed: start over from Gershgorin
        a = g0; b = g1;
        split(a, xh, xl);
        ca = count_df(dh, dl, eh, el, m, xh, xl, &fah, &fae);
        split(b, xh, xl);
        cb = count_df(dh, dl, eh, el, m, xh, xl, &fbh, &fbe);
        ne += 2;
    }
    int side = -1;   // endpoint replaced last: 0 = a, 1 = b
    for (int it = 0; it < 200; ++it) {
        const double tol = fmax(1e-12 * fmax(fabs(a), fabs(b)), 1e-13 * tn);
        if (b - a <= tol) break;
        const double mid = 0.5 * (a + b);
        if (mid == a || mid == b) break;
        double x = mid;
        const bool rf = (ca == k && cb == k + 1);
        if (rf) {
            // regula falsi: x = a + (b - a) f(a) / (f(a) - f(b)), f(b) / f(a) < 0
            int de = fbe - fae;
            de = de < -120 ? -120 : (de > 120 ? 120 : de);
            const float r = (fbh / fah) * pow2f(de);
            const float w = 1.0f / (1.0f - r);
            x = a + (double)w * (b - a);
            if (!(x > a && x < b)) x = mid;
            // a step closer than tol / 2 to an end moves to tol / 2, so the bracket
            // either closes on the root or shrinks by at least that much
            x = fmin(fmax(x, a + 0.5 * tol), b - 0.5 * tol);
        }
        float fxh;
        int fxe;
        split(x, xh, xl);
        const int cx = count_df(dh, dl, eh, el, m, xh, xl, &fxh, &fxe);
        ++ne;
        if (cx > k) {
            b = x; cb = cx; fbh = fxh; fbe = fxe;
            if (rf && side == 1) fah *= 0.5f;   // Illinois: the stale end's value halves
            side = rf ? 1 : -1;
        } else {
            a = x; ca = cx; fah = fxh; fae = fxe;
            if (rf && side == 0) fbh *= 0.5f;
            side = rf ? 0 : -1;
        }
    }
    if (nev) *nev = ne;
    return 0.5 * (a + b) * pow2(sexp);
}

}  // namespace sturm
}  // namespace bd
