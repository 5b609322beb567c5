// Host build of the tridiagonal eigenvalue arithmetic in csrc/eig_sturm.cuh, for the
// CPU check against LAPACK (tests/test_sturm_host.py).  The glue below follows the
// device kernels k_bisect_prep / k_bisect: split at negligible off-diagonals, scale
// each block by a power of two, split d and e^2 into FP32 pairs, bisect each
// eigenvalue (the device's four-lane evaluator replaced by one that counts its four
// points one after another).  Built with -ffp-contract=off so no FMA is formed that
// the device code does not form.
#include <math.h>
#include <vector>
#include "../boccadorata-public_gb300/csrc/eig_sturm.cuh"

using namespace bd::sturm;

extern "C" int bd_sturm_eigenvalues(const double *d, const double *e_in, int n, double *w, int *blk_start,
                                    int *nev_total) {
    std::vector<double> e(n, 0.0);
    for (int i = 0; i + 1 < n; ++i) e[i] = negligible(e_in[i], d[i], d[i + 1]) ? 0.0 : e_in[i];
    std::vector<float> dh(n), dl(n), eh(n), el(n);
    int ev = 0;
    for (int b0 = 0; b0 < n;) {
        int b1 = b0;
        while (b1 + 1 < n && e[b1] != 0.0) ++b1;
        float lo = 0.0f, hi = 0.0f, rn = 0.0f;
        for (int i = b0; i <= b1; ++i) {
            float l, h, r;
            gershgorin_row(d[i], i > b0 ? fabs(e[i - 1]) : 0.0, i < b1 ? fabs(e[i]) : 0.0, l, h, r);
            if (i == b0 || l < lo) lo = l;
            if (i == b0 || h > hi) hi = h;
        }
        const int sx = scale_exponent(fmaxf(fabsf(lo), fabsf(hi)));
        const double sc = pow2(-sx);
        for (int i = b0; i <= b1; ++i) {
            split(d[i] * sc, dh[i], dl[i]);
            const double e2 = (i < b1) ? e[i] * e[i] * sc * sc : 0.0;
            split(e2, eh[i], el[i]);
        }
        const int m = b1 - b0 + 1;
        for (int k = 0; k < m; ++k) {
            blk_start[b0 + k] = b0;
            if (m == 1) { w[b0] = d[b0]; continue; }
            int ne = 0;
            const SeqEval4 evl{&dh[b0], &dl[b0], &eh[b0], &el[b0], m};
            w[b0 + k] = bisect4(evl, k, lo * (float)sc, hi * (float)sc, sx, &ne);
            ev += ne;
        }
        b0 = b1 + 1;
    }
    if (nev_total) *nev_total = ev;
    return 0;
}
