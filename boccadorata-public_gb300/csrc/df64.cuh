// df64.cuh -- double-float arithmetic on the FP32 pipe: a value is hi + lo, two FP32
// numbers with |lo| <= ulp(hi) / 2 (about 48 significant bits).  GB300 issues FP64 at
// 1/64 of the FP32 rate, so a double-float multiply-add (about fifteen FP32
// instructions) outruns an FP64 FMA several times over where the FP64 unit is the
// bound.  Built from Knuth's two-sum and the FMA two-product (Dekker); the sums are
// the "sloppy" double-float addition, whose absolute error stays within ~2^-47 of the
// larger operand.  Every operation is explicitly rounded so the compiler cannot fuse
// the error-free transformations.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace bd {
namespace dfm {

struct alignas(8) df {   // 8-byte aligned: one 64-bit load or store per value
    float h, l;
};

// explicitly rounded FP32 operations (plain operators on the host, built without
// contraction for the CPU check)
DF_HD float fadd(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
DF_HD float fmul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
DF_HD float ffma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}
DF_HD float to_float(double x) {
#if defined(__CUDA_ARCH__)
    return __double2float_rn(x);
#else
    return (float)x;
#endif
}

DF_HD void two_sum(float a, float b, float &s, float &e) {
    s = fadd(a, b);
    const float bb = fadd(s, -a);
    e = fadd(fadd(a, -fadd(s, -bb)), fadd(b, -bb));
}

DF_HD df renorm(float s, float e) {   // fast two-sum, |s| >= |e| or s == 0
    df r;
    r.h = fadd(s, e);
    r.l = fadd(e, -fadd(r.h, -s));   // e - (h - s)
    return r;
}

DF_HD df from_double(double x) {
    df r;
    r.h = to_float(x);
    r.l = to_float(x - (double)r.h);
    return r;
}

DF_HD double to_double(df a) { return (double)a.h + (double)a.l; }

DF_HD df neg(df a) { return df{-a.h, -a.l}; }

DF_HD df add(df a, df b) {
    float s, e;
    two_sum(a.h, b.h, s, e);
    e = fadd(e, fadd(a.l, b.l));
    return renorm(s, e);
}

DF_HD df mul(df a, df b) {
    const float p = fmul(a.h, b.h);
    float e = ffma(a.h, b.h, -p);
    e = ffma(a.h, b.l, e);
    e = ffma(a.l, b.h, e);
    return renorm(p, e);
}

// a * b + c
DF_HD df fma(df a, df b, df c) {
    const float p = fmul(a.h, b.h);
    float e = ffma(a.h, b.h, -p);
    e = ffma(a.h, b.l, e);
    e = ffma(a.l, b.h, e);
    float s, f;
    two_sum(p, c.h, s, f);
    f = fadd(f, fadd(e, c.l));
    return renorm(s, f);
}

// 1/sqrt(x), x > 0 in the FP32 range: the FP32 seed and `its` Newton steps
// y <- y + y (1 - x y^2) / 2 in double-float (the relative error squares each step:
// one step from a seed within 2 ulp leaves about 2^-43, two reach double-float rounding)
DF_HD df rsqrt(df x, int its = 2) {
#if defined(__CUDA_ARCH__)
    const float y0 = rsqrtf(x.h);
#else
    const float y0 = 1.0f / sqrtf(x.h);
#endif
    df y{y0, 0.0f};
    const df half{0.5f, 0.0f};
    for (int it = 0; it < its; ++it) {
        const df t = mul(x, mul(y, y));              // x y^2
        const df c = fma(neg(half), t, half);         // (1 - x y^2) / 2
        y = fma(y, c, y);
    }
    return y;
}

// 1/d, d in the FP32 range: the FP32 seed and `its` Newton steps r <- r + r (1 - d r)
DF_HD df rcp(df d, int its = 2) {
    df r{1.0f / d.h, 0.0f};
    const df one{1.0f, 0.0f};
    for (int it = 0; it < its; ++it) r = fma(r, fma(neg(d), r, one), r);
    return r;
}

#if defined(__CUDACC__)

__device__ __forceinline__ df shfl_xor(df a, int o) {
    return df{__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)};
}

__device__ __forceinline__ df warp_sum(df a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a = add(a, shfl_xor(a, o));
    return a;
}
#endif

}  // namespace dfm
}  // namespace bd
