// Host build of the double-float arithmetic in csrc/df64.cuh for the CPU check
// (tests/test_df64_host.py).  Built with -ffp-contract=off.
#include "../boccadorata-public_gb300/csrc/df64.cuh"

using namespace bd::dfm;

// op 0: a + b, 1: a * b, 2: a * b + c, each on the double-float images of the inputs
extern "C" void bd_df64_ops(int op, const double *a, const double *b, const double *c, int n, double *out) {
    for (int i = 0; i < n; ++i) {
        const df x = from_double(a[i]), y = from_double(b[i]), z = from_double(c[i]);
        const df r = op == 0 ? add(x, y) : op == 1 ? mul(x, y) : fma(x, y, z);
        out[i] = to_double(r);
    }
}

// sum of squares by a chain of double-float multiply-adds
extern "C" double bd_df64_sumsq(const double *a, int n) {
    df s{0.0f, 0.0f};
    for (int i = 0; i < n; ++i) { const df x = from_double(a[i]); s = fma(x, x, s); }
    return to_double(s);
}

// op 0: 1/sqrt(a), 1: 1/a, on the double-float images of the inputs; ops 2, 3: the
// same with one Newton step
extern "C" void bd_df64_fun(int op, const double *a, int n, double *out) {
    const int its = op < 2 ? 2 : 1;
    for (int i = 0; i < n; ++i)
        out[i] = to_double(op % 2 == 0 ? rsqrt(from_double(a[i]), its) : rcp(from_double(a[i]), its));
}
