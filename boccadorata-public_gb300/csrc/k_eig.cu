// k_eig.cu -- K4b..K5: eigen-decomposition of the tridiagonal T = Q^T A Q left by
// k_tridiag, for many matrices at once, returning only what DysonMatrix uses
// (source/BcDor-DysonMatrix.cpp:442-488): every eigenvalue W_k and the first D
// components x_k[0:D] of the corresponding eigenvector of A.
//
//   k_qrows   R = first D rows of Q = H_0 H_1 ... H_{n-3} (reflectors kept in A's rows;
//             matrices of order <= kTsMax get R from k_tridiag_small)
//   k_bisect_prep  splits T into unreduced blocks at negligible off-diagonals
//   k_bisect  W_k by bisection on Sturm counts over its block, four threads per
//             eigenvalue (eig_sturm.cuh): an FP32 bracket, checked and finished in
//             double-float arithmetic (FP64 issues at 1/64 of the FP32 rate) to
//             max(1e-12 |W|, 1e-13 |T_b|)
//   k_invit   y_k by inverse iteration on T_b - W_k I (tridiagonal LU with partial
//             pivoting) over its block, one thread per eigenvalue, each from its own
//             start vector (k_invit_small: the factors in shared memory, orders <= 160)
//   k_cluster_orth  eigenvalues of one block closer than 1e-6 |T_b| form a cluster;
//             its vectors are orthonormalised together (the exactly degenerate
//             groups of tens to hundreds of zero-strength solutions in the Dyson
//             spectra fall into different blocks and need nothing)
//   k_post    x_k[0:D] = R y_k, Z_k = sum_d x_k[d]^2
//   k_place   quasiparticle / quasihole split by E_F with both lists by descending W
//   k_koltun  Koltun partial sums (Calc_En, source/BcDor-DysonMatrix.cpp:542-594)
#include <climits>
#include "bd_common.cuh"
#include "df64.cuh"
#include "bd_kernels.h"
#include "eig_sturm.cuh"

namespace bd {

constexpr int kEigThreads = 256;

// ------------------------------------------------------------------ K4b
__global__ void __launch_bounds__(kEigThreads) k_qrows(const DyJob *jobs, int njobs) {
    const int jid = blockIdx.x;
    if (jid >= njobs) return;
    const DyJob J = jobs[jid];
    const int n = J.nc, D = J.D, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;   // order after deflation
    if (n <= kTsMax) return;   // k_tridiag_small formed R
    __shared__ double red[kEigThreads / 32][8];
    __shared__ double sums[8];
    double *R = J.R;
    for (int q = tid; q < D * n; q += kEigThreads) R[q] = ((q % n) == (q / n)) ? 1.0 : 0.0;
    __syncthreads();
    for (int k = 0; k + 2 < n; ++k) {
        const double tau = J.tau[k];
        if (tau == 0.0) continue;
        const int b0 = k + 1, m = n - b0;
        const double *v = J.A + (size_t)k * n + b0;
        double s[8];
#pragma unroll
        for (int d = 0; d < 8; ++d) s[d] = 0.0;
        for (int t = tid; t < m; t += kEigThreads) {
            const double vt = v[t];
#pragma unroll
            for (int d = 0; d < 8; ++d) if (d < D) s[d] += R[(size_t)d * n + b0 + t] * vt;
        }
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            double x = s[d];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) red[warp][d] = x;
        }
        __syncthreads();
        if (tid < D) {
            double x = 0.0;
            for (int q = 0; q < kEigThreads / 32; ++q) x += red[q][tid];
            sums[tid] = tau * x;
        }
        __syncthreads();
        for (int t = tid; t < m; t += kEigThreads) {
            const double vt = v[t];
            for (int d = 0; d < D; ++d) R[(size_t)d * n + b0 + t] -= sums[d] * vt;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ K4c
// Split T where an off-diagonal is negligible (sturm::negligible, the relative split
// test of the QR / bisection codes; the perturbation is below the rounding of T).
// The Dyson matrices' tridiagonal forms fall apart into many blocks: the exactly
// degenerate poles of the HO spectrum give identical eigenvalues in different blocks,
// whose eigenvectors then have disjoint supports and need no orthogonalisation.
// Every later kernel works on the block of its own position: positions are
// block-major, eigenvalues ascending within a block.
//
// One CTA per matrix.  Outputs:
//   J.e        split off-diagonals (zero between blocks)
//   J.blk      first and last position of each position's block
//   J.tau      the block's 1-norm, max_i |d_i| + |e_{i-1}| + |e_i| (rounded up), at
//              every position (k_qrows has consumed the reflector scalars)
//   work       FP32 tables at the start of the job's work area (free until k_invit),
//              n = J.nc entries each: d 2^-s as hi / lo pair, e_i^2 2^-2s as hi / lo
//              pair (zero at a block's last row), and at each block's first position
//              its scaled Gershgorin bounds and the exponent s (2^-s |T_b| in [1/2, 1))
//   scratch    split flags and row sums behind them
struct BisectTables {
    float *dh, *dl, *eh, *el, *glo, *ghi, *rn;
    int *sx, *flag;
};

__device__ inline BisectTables bisect_tables(double *work, int n) {
    float *f = reinterpret_cast<float *>(work);
    BisectTables t;
    t.dh = f; t.dl = f + n; t.eh = f + 2 * n; t.el = f + 3 * n; t.glo = f + 4 * n; t.ghi = f + 5 * n;
    t.sx = reinterpret_cast<int *>(f + 6 * n);
    t.flag = reinterpret_cast<int *>(f + 7 * n);
    t.rn = f + 8 * n;
    return t;
}

__global__ void k_bisect_prep(const DyJob *jobs, int njobs, double *work, const long long *work_first) {
    const int jid = blockIdx.x;
    if (jid >= njobs) return;
    const DyJob J = jobs[jid];
    const int n = J.nc;
    const BisectTables T = bisect_tables(work + work_first[jid], n);
    int *bs = J.blk, *be = J.blk + n;
    // 1. split flags, row Gershgorin intervals and row sums (each thread repeats the
    //    split test of its left neighbour: identical inputs, identical answer)
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double di = J.d[i];
        double er = 0.0, el = 0.0;
        if (i + 1 < n) { er = J.e[i]; if (sturm::negligible(er, di, J.d[i + 1])) er = 0.0; }
        if (i > 0) { el = J.e[i - 1]; if (sturm::negligible(el, J.d[i - 1], di)) el = 0.0; }
        T.flag[i] = (i + 1 == n || er == 0.0);
        float lo, hi, r;
        sturm::gershgorin_row(di, fabs(el), fabs(er), lo, hi, r);
        T.glo[i] = lo; T.ghi[i] = hi; T.rn[i] = r;
    }
    __syncthreads();
    // 2. block bounds: one integer pass
    if (threadIdx.x == 0) {
        int b0 = 0;
        for (int i = 0; i < n; ++i)
            if (T.flag[i]) {
                for (int k = b0; k <= i; ++k) { bs[k] = b0; be[k] = i; }
                b0 = i + 1;
            }
    }
    __syncthreads();
    // 3. each block's first position reduces its block and picks the scale
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        if (bs[i] != i) continue;
        const int b1 = be[i];
        float lo = T.glo[i], hi = T.ghi[i], r = T.rn[i];
        for (int q = i + 1; q <= b1; ++q) { lo = fminf(lo, T.glo[q]); hi = fmaxf(hi, T.ghi[q]); r = fmaxf(r, T.rn[q]); }
        const int s = sturm::scale_exponent(fmaxf(fabsf(lo), fabsf(hi)));
        const float sc = sturm::pow2f(-s);
        T.glo[i] = lo * sc; T.ghi[i] = hi * sc; T.rn[i] = r; T.sx[i] = s;
    }
    __syncthreads();
    // 4. scaled FP32 pairs; split off-diagonals back into J.e; block norms into J.tau
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int b0 = bs[i], b1 = be[i];
        const double sc = sturm::pow2(-T.sx[b0]);
        sturm::split(J.d[i] * sc, T.dh[i], T.dl[i]);
        double e = (i + 1 < n) ? J.e[i] : 0.0;
        if (i + 1 < n && i == b1) { e = 0.0; J.e[i] = 0.0; }
        sturm::split(e * e * sc * sc, T.eh[i], T.el[i]);
        J.tau[i] = (double)T.rn[b0];
    }
}

// matrix and position of a global eigenvalue index
__device__ inline int job_of(const long long *row_first, int njobs, long long g) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (row_first[mid] <= g) lo = mid; else hi = mid - 1; }
    return lo;
}

// Four threads per position: the eigenvalue of its block with the position's local
// index, by sturm::bisect4 (FP32 bracket, double-float finish, four points per pass,
// one per lane; no FP64 in the counts).  A matrix's eigenvalues are few hundred at
// most, so the per-eigenvalue chain is the latency that matters; four lanes shorten
// it and still leave most of the GPU's sub-partitions idle.
constexpr int kBisectThreads = 128;   // 32 positions per CTA

__global__ void __launch_bounds__(kBisectThreads) k_bisect(const DyJob *jobs, int njobs, const long long *row_first,
                                                           long long total, double *work, const long long *work_first) {
    const long long g4 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long g = g4 >> 2;   // the group's position; its four lanes share every branch
    const int sub = (int)(g4 & 3);
    if (g >= total) return;
    const int lo = job_of(row_first, njobs, g);
    const DyJob J = jobs[lo];
    const int t = (int)(g - row_first[lo]), n = J.nc;
    if (t >= n) return;   // deflated rows need no eigenvalue
    const int b0 = J.blk[t], b1 = J.blk[n + t], m = b1 - b0 + 1, k = t - b0;
    double W;
    if (m == 1) {
        W = J.d[t];
    } else {
        const BisectTables T = bisect_tables(work + work_first[lo], n);
        const int lane = threadIdx.x & 31, base = lane & ~3;
        const sturm::LaneEval4 ev{T.dh + b0, T.dl + b0, T.eh + b0, T.el + b0, m, sub, base, 0xFu << base};
        W = sturm::bisect4(ev, k, T.glo[b0], T.ghi[b0], T.sx[b0], nullptr);
    }
    if (sub == 0) J.sol[(size_t)t * (2 + J.D)] = W;   // eigenvalue parked in the W slot of its position
}

// ------------------------------------------------------------------ K4d
// Inverse iteration, one thread per position, on its block only.  Eigenvalues of
// the block closer than ortol = 1e-6 |T_b| to their predecessor belong to the same
// cluster; inside a cluster the shifts are kept at least pertol apart (the shift
// rule of LAPACK's dstein) and every member starts from its own pseudo-random vector,
// so the members span the cluster's invariant subspace; k_cluster_orth then makes
// them orthonormal.  Y (the n x n region of A, column t at stride n) receives y_t on
// the block's rows; the LU factors live in the job's work buffer, columns at stride n.
__device__ inline unsigned hash32(unsigned x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

constexpr double kEps = 2.220446049250313e-16;

struct EigTol { double onenrm, ortol, pertol; };

__device__ inline EigTol eig_tol(double onenrm) {
    EigTol t;
    t.onenrm = onenrm;
    t.ortol = 1e-6 * onenrm;
    t.pertol = 10.0 * kEps * fmax(onenrm, 1e-300);
    return t;
}

// Storage of one eigenvector's LU factors (first and second superdiagonal, pivots as
// reciprocals, multipliers, interchanges) and of its iterate, element i of each.
struct InvitGlobal {   // the job's work area and matrix region, column k at stride n
    double *U1, *U2, *DD, *LL, *PV, *Y;
    int n, k;
    __device__ double &u1(int i) { return U1[(size_t)i * n + k]; }
    __device__ double &u2(int i) { return U2[(size_t)i * n + k]; }
    __device__ double &dd(int i) { return DD[(size_t)i * n + k]; }
    __device__ double &ll(int i) { return LL[(size_t)i * n + k]; }
    __device__ double &y(int i) { return Y[(size_t)i * n + k]; }
    __device__ bool pv(int i) { return PV[(size_t)i * n + k] != 0.0; }
    __device__ void set_pv(int i, bool b) { PV[(size_t)i * n + k] = b ? 1.0 : 0.0; }
};

constexpr int kIvThreads = 16;   // eigenvectors per CTA of the shared-memory variant

// Eigenvector k of block [b0, b1] (b1 > b0) into a.y(b0 .. b1).
template <class S>
__device__ void invit_vector(const DyJob &J, int k, int b0, int b1, S &a) {
    const int NS = 2 + J.D;
    const double *d = J.d, *e = J.e;
    const EigTol tl = eig_tol(J.tau[k]);
    auto W = [&](int q) { return J.sol[(size_t)q * NS]; };
    // shift: walk to the start of the cluster inside the block, then apply the separation rule forward
    int k0 = k;
    while (k0 > b0 && W(k0) - W(k0 - 1) <= tl.ortol) --k0;
    double x = W(k0);
    for (int q = k0 + 1; q <= k; ++q) x = fmax(W(q), x + tl.pertol);
    // LU with partial pivoting of T_b - x I; rows i and i+1 may swap
    for (int i = b0; i <= b1; ++i) {
        a.dd(i) = d[i] - x;
        a.u1(i) = (i < b1) ? e[i] : 0.0;
        a.ll(i) = (i < b1) ? e[i] : 0.0;
        a.u2(i) = 0.0;
    }
    for (int i = b0; i < b1; ++i) {
        const double di = a.dd(i), li = a.ll(i);
        if (fabs(di) >= fabs(li)) {
            a.set_pv(i, false);
            const double f = (di != 0.0) ? li * rcp_newton(di) : 0.0;
            a.ll(i) = f;
            a.dd(i + 1) -= f * a.u1(i);
        } else {
            a.set_pv(i, true);
            const double f = di * rcp_newton(li);
            a.dd(i) = li;
            a.ll(i) = f;
            const double tt = a.u1(i);
            a.u1(i) = a.dd(i + 1);
            a.dd(i + 1) = tt - f * a.dd(i + 1);
            if (i + 1 < b1) {
                a.u2(i) = a.u1(i + 1);
                a.u1(i + 1) = -f * a.u1(i + 1);
            }
        }
    }
    // pivots no smaller than pertol, kept as reciprocals for the solves
    for (int i = b0; i <= b1; ++i) {
        double p = a.dd(i);
        if (fabs(p) < tl.pertol) p = (p < 0 ? -tl.pertol : tl.pertol);
        a.dd(i) = rcp_newton(p);
    }
    for (int i = b0; i <= b1; ++i)
        a.y(i) = 0.5 + (double)(hash32((unsigned)(i * 2654435761u) ^ (unsigned)(k * 97 + 13)) & 0xffff) / 65536.0;
    // two sweeps: the shift is within 1e-13 |T_b| of W_k and eigenvalues of a block
    // closer than 1e-6 |T_b| are clustered (orthonormalised together), so each sweep
    // scales the other eigenvectors' share by at most 1e-7 against this one's
    for (int it = 0; it < 2; ++it) {
        for (int i = b0; i < b1; ++i) {   // L^-1 with the interchanges
            double bi = a.y(i), bi1 = a.y(i + 1);
            const double f = a.ll(i);
            if (!a.pv(i)) bi1 -= f * bi;
            else { const double tt = bi; bi = bi1; bi1 = tt - f * bi1; }
            a.y(i) = bi; a.y(i + 1) = bi1;
        }
        double y1 = 0.0, y2 = 0.0, nrm = 0.0;
        for (int i = b1; i >= b0; --i) {   // U y = b, two superdiagonals
            double v = a.y(i);
            if (i + 1 <= b1) v -= a.u1(i) * y1;
            if (i + 2 <= b1) v -= a.u2(i) * y2;
            v *= a.dd(i);
            a.y(i) = v;
            y2 = y1; y1 = v;
            nrm = fmax(nrm, fabs(v));
        }
        const double sc = (nrm > 0.0) ? rcp_newton(nrm) : 1.0;
        double s2 = 0.0;
        for (int i = b0; i <= b1; ++i) { const double v = a.y(i) * sc; a.y(i) = v; s2 += v * v; }
        const double inv = (s2 > 0.0) ? 1.0 / sqrt(s2) : 0.0;
        for (int i = b0; i <= b1; ++i) a.y(i) *= inv;
    }
}

// The same in double-float (df64.cuh: FP32 hi + lo pairs, ~48 bits) for the shared-memory
// variant: every step of the factorisation and of the solves is a dependent chain, and
// an FP64 instruction holds an SM sub-partition's FP64 unit for ~64 cycles on this GPU
// (a reciprocal by Newton's iteration is four of them), while the double-float forms
// run on the FP32 pipe at a few cycles per operation.  The shifts, the tolerances and
// the start vectors are those of invit_vector; the pivot choice compares the high parts
// (any choice that keeps the multipliers bounded serves), and the result goes to y in
// FP64.  The tridiagonal is converted to double-float once per CTA, into shared memory.
struct InvitSharedDF {   // shared memory, element i of this thread at i * kIvThreads + lane
    dfm::df *U1, *U2, *DD, *LL, *Y;
    unsigned char *PV;
    int lane;
    __device__ dfm::df &u1(int i) { return U1[i * kIvThreads + lane]; }
    __device__ dfm::df &u2(int i) { return U2[i * kIvThreads + lane]; }
    __device__ dfm::df &dd(int i) { return DD[i * kIvThreads + lane]; }
    __device__ dfm::df &ll(int i) { return LL[i * kIvThreads + lane]; }
    __device__ dfm::df &y(int i) { return Y[i * kIvThreads + lane]; }
    __device__ bool pv(int i) { return PV[i * kIvThreads + lane] != 0; }
    __device__ void set_pv(int i, bool b) { PV[i * kIvThreads + lane] = b ? 1 : 0; }
};

__device__ inline dfm::df df_abs(dfm::df a) { return a.h < 0.0f ? dfm::neg(a) : a; }
__device__ inline dfm::df df_sub(dfm::df a, dfm::df b) { return dfm::add(a, dfm::neg(b)); }

__device__ void invit_vector_df(const DyJob &J, int k, int b0, int b1, const dfm::df *dt, const dfm::df *et,
                                InvitSharedDF &a) {
    using dfm::df;
    const int NS = 2 + J.D;
    const EigTol tl = eig_tol(J.tau[k]);
    auto W = [&](int q) { return J.sol[(size_t)q * NS]; };
    int k0 = k;
    while (k0 > b0 && W(k0) - W(k0 - 1) <= tl.ortol) --k0;
    double xs = W(k0);
    for (int q = k0 + 1; q <= k; ++q) xs = fmax(W(q), xs + tl.pertol);
    const df x = dfm::from_double(xs);
    const df zero{0.0f, 0.0f};
    const float pt = (float)tl.pertol;
    // Reciprocals by one Newton step from the FP32 seed (~2^-44): the factors only need
    // to keep the shifted matrix's direction, far looser than that.
    auto rcp1 = [&](df p) { return dfm::rcp(p, 1); };
    auto clamp_piv = [&](df p) {   // pivots no smaller than pertol
        return (fabsf(p.h) < pt) ? df{p.h < 0.0f ? -pt : pt, 0.0f} : p;
    };
    // LU with partial pivoting of T_b - x I (rows i and i+1 may swap).  The running
    // diagonal and superdiagonal entries of the next row stay in registers, so the
    // dependent chain is the arithmetic alone (one reciprocal per row: the multiplier's
    // and the kept pivot's are the same unless the pivot is below pertol); each row's
    // factors go to shared memory for the solves as soon as they are final.  The
    // tridiagonal comes in double-float from dt, et (shared memory).
    df cur_d = df_sub(dt[b0], x);                 // dd(i) as updated so far
    df cur_u = (b0 < b1) ? et[b0] : zero;         // u1(i) as updated so far
    for (int i = b0; i < b1; ++i) {
        const df di = cur_d, li = et[i], ui = cur_u;
        const df nd = df_sub(dt[i + 1], x);                     // dd(i+1) before this row
        const df nu = (i + 1 < b1) ? et[i + 1] : zero;          // u1(i+1) before this row
        if (fabsf(di.h) >= fabsf(li.h)) {
            a.set_pv(i, false);
            const df cp = clamp_piv(di), r = rcp1(cp);
            const df f = (di.h != 0.0f) ? dfm::mul(li, (cp.h == di.h) ? r : rcp1(di)) : zero;
            a.ll(i) = f;
            a.u1(i) = ui;
            a.u2(i) = zero;
            a.dd(i) = r;
            cur_d = dfm::fma(dfm::neg(f), ui, nd);
            cur_u = nu;
        } else {
            a.set_pv(i, true);
            const df cp = clamp_piv(li), r = rcp1(cp);
            const df f = dfm::mul(di, (cp.h == li.h) ? r : rcp1(li));
            a.ll(i) = f;
            a.u1(i) = nd;
            a.u2(i) = nu;
            a.dd(i) = r;
            cur_d = dfm::fma(dfm::neg(f), nd, ui);
            cur_u = dfm::mul(dfm::neg(f), nu);
        }
    }
    a.u1(b1) = zero;
    a.u2(b1) = zero;
    a.dd(b1) = rcp1(clamp_piv(cur_d));
    for (int i = b0; i <= b1; ++i)
        a.y(i) = df{0.5f + (float)(hash32((unsigned)(i * 2654435761u) ^ (unsigned)(k * 97 + 13)) & 0xffff) / 65536.0f, 0.0f};
    for (int it = 0; it < 2; ++it) {
        df cur = a.y(b0);
        for (int i = b0; i < b1; ++i) {   // L^-1 with the interchanges, y(i) carried in a register
            df bi = cur, bi1 = a.y(i + 1);
            const df f = a.ll(i);
            if (!a.pv(i)) bi1 = dfm::fma(dfm::neg(f), bi, bi1);
            else { const df tt = bi; bi = bi1; bi1 = dfm::fma(dfm::neg(f), bi1, tt); }
            a.y(i) = bi;
            cur = bi1;
        }
        a.y(b1) = cur;
        // U y = b, two superdiagonals: the term of y(i+2) first, off the chain through y(i+1)
        df y1 = zero, y2 = zero;
        float nrm = 0.0f;
        for (int i = b1; i >= b0; --i) {
            df v = a.y(i);
            if (i + 2 <= b1) v = dfm::fma(dfm::neg(a.u2(i)), y2, v);
            if (i + 1 <= b1) v = dfm::fma(dfm::neg(a.u1(i)), y1, v);
            v = dfm::mul(v, a.dd(i));
            a.y(i) = v;
            y2 = y1; y1 = v;
            nrm = fmaxf(nrm, fabsf(v.h));
        }
        const df sc = (nrm > 0.0f) ? rcp1(df{nrm, 0.0f}) : df{1.0f, 0.0f};
        if (it == 0) {   // scaled to a largest entry of about one; the norm matters only at the end
            for (int i = b0; i <= b1; ++i) a.y(i) = dfm::mul(a.y(i), sc);
            continue;
        }
        df s2a = zero, s2b = zero;   // two chains
        int i = b0;
        for (; i + 1 <= b1; i += 2) {
            const df v0 = dfm::mul(a.y(i), sc), v1 = dfm::mul(a.y(i + 1), sc);
            a.y(i) = v0;
            a.y(i + 1) = v1;
            s2a = dfm::fma(v0, v0, s2a);
            s2b = dfm::fma(v1, v1, s2b);
        }
        if (i <= b1) { const df v0 = dfm::mul(a.y(i), sc); a.y(i) = v0; s2a = dfm::fma(v0, v0, s2a); }
        const df s2 = dfm::add(s2a, s2b);
        const df inv = (s2.h > 0.0f) ? dfm::rsqrt(s2, 1) : zero;
        for (int q = b0; q <= b1; ++q) a.y(q) = dfm::mul(a.y(q), inv);
    }
}

// Matrices of order > kTsMax: one thread per position, factors in the job's work area.
__global__ void k_invit(const DyJob *jobs, int njobs, const long long *row_first, long long total, double *work,
                        const long long *work_first) {
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= total) return;
    const int lo = job_of(row_first, njobs, g);
    const DyJob J = jobs[lo];
    const int k = (int)(g - row_first[lo]), n = J.nc;
    if (k >= n || n <= kTsMax) return;
    const int b0 = J.blk[k], b1 = J.blk[n + k];
    double *Y = J.A;
    if (b0 == b1) { Y[(size_t)b0 * n + k] = 1.0; return; }
    double *wk = work + work_first[lo];   // 5 arrays of n*n
    InvitGlobal a{wk, wk + (size_t)n * n, wk + 2 * (size_t)n * n, wk + 3 * (size_t)n * n, wk + 4 * (size_t)n * n, Y,
                  n, k};
    invit_vector(J, k, b0, b1, a);
}

// Orders <= kTsMax: CTA (job, chunk of kIvThreads positions), each thread's factors and
// iterate in shared memory (the LU and the solves read back what they just wrote,
// which from global memory is an L2 round trip per step); the iterate goes to the
// matrix region at the end.
__global__ void __launch_bounds__(kIvThreads) k_invit_small(const DyJob *jobs, int njobs) {
    const int jid = blockIdx.x;
    if (jid >= njobs) return;
    const DyJob J = jobs[jid];
    const int n = J.nc, lane = threadIdx.x, k = blockIdx.y * kIvThreads + lane;
    if (n > kTsMax || blockIdx.y * kIvThreads >= n) return;   // uniform over the CTA
    extern __shared__ double smi[];
    const int cap = kTsMax * kIvThreads;
    dfm::df *sd = reinterpret_cast<dfm::df *>(smi);
    InvitSharedDF a{sd, sd + cap, sd + 2 * cap, sd + 3 * cap, sd + 4 * cap,
                    reinterpret_cast<unsigned char *>(sd + 5 * cap), lane};
    // the tridiagonal in double-float, converted once by the CTA's threads
    dfm::df *dt = sd + 5 * cap + cap / 8, *et = dt + kTsMax;
    for (int i = lane; i < n; i += kIvThreads) {
        dt[i] = dfm::from_double(J.d[i]);
        et[i] = dfm::from_double(J.e[i]);
    }
    __syncthreads();
    if (k >= n) return;
    const int b0 = J.blk[k], b1 = J.blk[n + k];
    double *Y = J.A;
    if (b0 == b1) { Y[(size_t)b0 * n + k] = 1.0; return; }
    invit_vector_df(J, k, b0, b1, dt, et, a);
    for (int i = b0; i <= b1; ++i) Y[(size_t)i * n + k] = dfm::to_double(a.y(i));
}

// kOrthCtas CTAs per matrix.  Each takes 256 positions at a time, a thread per
// position marks the first members of clusters (two or more members, inside one
// block), then the CTA orthonormalises each marked cluster's members with two
// classical Gram-Schmidt sweeps over the block's rows.  Clusters are disjoint sets of
// columns, so the order the CTA takes them in changes nothing.
constexpr int kOrthCtas = 8;

__global__ void __launch_bounds__(kEigThreads) k_cluster_orth(const DyJob *jobs, int njobs) {
    const int jid = blockIdx.x / kOrthCtas;
    if (jid >= njobs) return;
    const DyJob J = jobs[jid];
    const int n = J.nc, NS = 2 + J.D, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ double cbuf[1024];
    __shared__ double red[kEigThreads / 32];
    __shared__ int s_first[kEigThreads], s_last[kEigThreads], s_nc;
    auto W = [&](int q) { return J.sol[(size_t)q * NS]; };
    double *Y = J.A;   // y_p is column p: element (i, p) at i * n + p
    for (int base = (blockIdx.x % kOrthCtas) * kEigThreads; base < n; base += kOrthCtas * kEigThreads) {
        __syncthreads();   // the previous pass's list is read
        if (tid == 0) s_nc = 0;
        __syncthreads();
        if (base + tid < n) {
            const int k0 = base + tid, b0 = J.blk[k0], b1 = J.blk[n + k0];
            if (b0 != b1) {
                const double ortol = eig_tol(J.tau[k0]).ortol;
                if (!(k0 > b0 && W(k0) - W(k0 - 1) <= ortol) && k0 < b1 && W(k0 + 1) - W(k0) <= ortol) {
                    int k1 = k0 + 2;
                    while (k1 <= b1 && W(k1) - W(k1 - 1) <= ortol) ++k1;
                    const int slot = atomicAdd(&s_nc, 1);
                    s_first[slot] = k0;
                    s_last[slot] = k1;
                }
            }
        }
        __syncthreads();
        for (int c = 0; c < s_nc; ++c) {
            const int k0 = s_first[c], k1 = s_last[c], b0 = J.blk[k0], b1 = J.blk[n + k0];
            for (int q = k0; q < k1; ++q) {
                for (int sweep = 0; sweep < 2; ++sweep) {
                    // c_p = <y_p, y_q> for the earlier members, blocks of 1024: a warp per member
                    for (int p0 = k0; p0 < q; p0 += 1024) {
                        const int p1 = min(q, p0 + 1024);
                        for (int p = p0 + warp; p < p1; p += kEigThreads / 32) {
                            double s = 0.0;
                            for (int i = b0 + lane; i <= b1; i += 32) s += Y[(size_t)i * n + p] * Y[(size_t)i * n + q];
                            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                            if (lane == 0) cbuf[p - p0] = s;
                        }
                        __syncthreads();
                        // y_q -= sum_p c_p y_p: a thread per row, running along the row's members
                        for (int i = b0 + tid; i <= b1; i += kEigThreads) {
                            double acc = 0.0;
                            for (int p = p0; p < p1; ++p) acc += cbuf[p - p0] * Y[(size_t)i * n + p];
                            Y[(size_t)i * n + q] -= acc;
                        }
                        __syncthreads();
                    }
                }
                double s = 0.0;
                for (int i = b0 + tid; i <= b1; i += kEigThreads) s += Y[(size_t)i * n + q] * Y[(size_t)i * n + q];
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) red[warp] = s;
                __syncthreads();
                double tot = 0.0;
                for (int w = 0; w < kEigThreads / 32; ++w) tot += red[w];
                const double inv = (tot > 0.0) ? 1.0 / sqrt(tot) : 0.0;
                for (int i = b0 + tid; i <= b1; i += kEigThreads) Y[(size_t)i * n + q] *= inv;
                __syncthreads();
            }
        }
    }
}

// ------------------------------------------------------------------ K5
// Four lanes per position: each sums every fourth row of the block, the quad then
// combines its partials (the FP64 dependent chains a quarter as long).
__global__ void k_post(const DyJob *jobs, int njobs, const long long *row_first, long long total) {
    const long long g4 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long g = g4 >> 2;   // the quad's position; its lanes share every branch
    const int sub = (int)(g4 & 3), lane = threadIdx.x & 31;
    const unsigned qmask = 0xFu << (lane & ~3);
    if (g >= total) return;
    const int lo = job_of(row_first, njobs, g);
    const DyJob J = jobs[lo];
    const int k = (int)(g - row_first[lo]), n = J.nc, D = J.D, NS = 2 + D;
    if (k >= n) return;
    const int b0 = J.blk[k], b1 = J.blk[n + k];
    double x[8];
#pragma unroll
    for (int dd = 0; dd < 8; ++dd) x[dd] = 0.0;
    for (int i = b0 + sub; i <= b1; i += 4) {
        const double y = J.A[(size_t)i * n + k];
#pragma unroll
        for (int dd = 0; dd < 8; ++dd) if (dd < D) x[dd] += J.R[(size_t)dd * n + i] * y;
    }
#pragma unroll
    for (int dd = 0; dd < 8; ++dd) {
        x[dd] += __shfl_xor_sync(qmask, x[dd], 1);
        x[dd] += __shfl_xor_sync(qmask, x[dd], 2);
    }
    if (sub != 0) return;
    // rows [W, Z, x] staged behind R, by position; k_place orders them
    double z = 0.0;
    for (int dd = 0; dd < D; ++dd) z += x[dd] * x[dd];
    double *st = J.R + (size_t)D * J.n + (size_t)k * NS;   // staging behind R sized for the full order
    st[0] = J.sol[(size_t)k * NS];
    st[1] = z;
    for (int dd = 0; dd < D; ++dd) st[2 + dd] = x[dd];
}

// Places the staged rows: quasiparticles (W > E_F) then quasiholes, each by
// descending W (ties by position).  kPlaceCtas CTAs per matrix; each thread takes up
// to kPlacePer rows and finds each one's rank among all staged rows (the staged rows
// are block-major, not sorted).  The energies are compared as order-preserving 64-bit
// integer keys (negative values bit-inverted, others with the sign bit set): FP64
// compares would issue on the FP64 pipe, 1/64 of the integer rate here.  The keys go
// through shared memory kPlaceChunk at a time.
constexpr int kPlaceCtas = 8, kPlacePer = 4, kPlaceChunk = 2048, kPlaceThreads = 256;

constexpr int kKtVirt = 256;   // k_koltun's virtual threads

__global__ void __launch_bounds__(kPlaceThreads) k_place(const DyJob *jobs, int njobs, double *work,
                                                         const long long *work_first) {
    const int jid = blockIdx.x, tid = threadIdx.x;
    if (jid >= njobs) return;
    const DyJob J = jobs[jid];
    const int n = J.n, D = J.D, NS = 2 + D, first = (int)blockIdx.y * kPlaceThreads;
    if (first >= n) {   // the whole CTA; an empty matrix still reports its counts
        if (n == 0 && blockIdx.y == 0 && tid == 0) { J.nq[0] = 0; J.nq[1] = 0; }
        return;
    }
    const double *st = J.R + (size_t)D * n;
    const double ef = J.efp ? *J.efp : J.efermi;
    auto key = [](double x) -> unsigned long long {
        const unsigned long long b = (unsigned long long)__double_as_longlong(x);
        return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
    };
    __shared__ unsigned long long wbuf[kPlaceChunk];
    __shared__ int nbelow;
    if (tid == 0) nbelow = 0;
    constexpr int span = kPlaceCtas * kPlaceThreads;
    for (int g0 = first; g0 < n; g0 += kPlacePer * span) {
        int r[kPlacePer];
        unsigned long long w[kPlacePer];
#pragma unroll
        for (int u = 0; u < kPlacePer; ++u) {
            const int k = g0 + tid + u * span;
            r[u] = 0;
            w[u] = key((k < n) ? st[(size_t)k * NS] : 0.0);
        }
        int c = 0;
        for (int q0 = 0; q0 < n; q0 += kPlaceChunk) {
            const int qn = min(kPlaceChunk, n - q0);
            __syncthreads();
            for (int q = tid; q < qn; q += kPlaceThreads) {
                const double x = st[(size_t)(q0 + q) * NS];
                wbuf[q] = key(x);
                c += !(x > ef);
            }
            __syncthreads();
#pragma unroll
            for (int u = 0; u < kPlacePer; ++u) {
                const int k = g0 + tid + u * span;
                if (k >= n) continue;
                // rows before k in this chunk count when not above it, the rest when below
                const int split = min(max(k - q0, 0), qn);
                int c2 = 0;
                for (int q = 0; q < split; ++q) c2 += (wbuf[q] <= w[u]);
                for (int q = split; q < qn; ++q) c2 += (wbuf[q] < w[u]);
                r[u] += c2;
            }
        }
        if (g0 == first) atomicAdd(&nbelow, c);
        __syncthreads();
        const int nqh = nbelow, nqp = n - nqh;
        if (g0 == first && blockIdx.y == 0 && tid == 0) {
            J.nq[0] = nqp; J.nq[1] = nqh;
            if (nqh > kKtVirt)   // k_koltun's ticket, behind its partials in the work area
                *reinterpret_cast<unsigned *>(work + work_first[jid] + kPlaceCtas * 9) = 0u;
        }
#pragma unroll
        for (int u = 0; u < kPlacePer; ++u) {
            const int k = g0 + tid + u * span;
            if (k >= n) continue;
            // quasiparticles descending, then quasiholes descending
            const int row = (r[u] >= nqh) ? (n - 1 - r[u]) : (nqp + (nqh - 1 - r[u]));
            for (int q = 0; q < NS; ++q) J.sol[(size_t)row * NS + q] = st[(size_t)k * NS + q];
        }
    }
}

// The Koltun partial sums over the placed quasiholes (Calc_En,
// source/BcDor-DysonMatrix.cpp:542-594).  Virtual thread vt = 0..255 takes quasiholes
// ne = vt, vt + 256, ... in that order into its own three buckets by |x|^2 (> 0.01,
// > 1e-5, the rest); the 32 virtual threads of a virtual warp meet in a shuffle tree and
// the eight virtual warps in order, so the sums are deterministic (the reference adds
// the rows one by one, ne from nqh - 1 down).  Up to 256 quasiholes one CTA runs the
// virtual threads as its own threads.  Beyond, CTA y of the matrix's kPlaceCtas is
// virtual warp y: its eight warps form the rows' |x|^2 and x^T S1 x (the FP64 work)
// side by side, its first warp adds them up in each virtual thread's order, and the
// eight partials meet in the matrix's work area, summed by the CTA that finishes last.
static_assert(kPlaceCtas * 32 == kKtVirt && kPlaceThreads == kKtVirt, "one CTA per virtual warp");

__device__ inline void koltun_row(const DyJob &J, const double *x, double &x1, double &x2) {
    const int D = J.D;
    x1 = 0.0;
    x2 = 0.0;
    for (int r = 0; r < D; ++r) {
        x1 += x[r] * x[r];
        for (int cc = 0; cc < D; ++cc) x2 += J.sig1b[r * D + cc] * x[r] * x[cc];
    }
}

__device__ inline void koltun_add(double *acc, double x1, double x2, double w) {
    const int b = (x1 > 0.01) ? 0 : (x1 > 1.e-5) ? 1 : 2;
    acc[b] += x2; acc[3 + b] += x1 * w; acc[6 + b] += x1;
}

__device__ inline void koltun_store(const DyJob &J, const double *t) {
    const double xj = (double)J.j2 + 1.0;
    J.koltun[0] = (t[0] + t[1] + t[2]) * xj;
    J.koltun[1] = (t[3] + t[4] + t[5]) * xj;
    J.koltun[2] = (t[6] + t[7] + t[8]) * xj;
}

__global__ void __launch_bounds__(kPlaceThreads) k_koltun(const DyJob *jobs, int njobs, double *work,
                                                          const long long *work_first) {
    const int jid = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (jid >= njobs) return;
    const DyJob J = jobs[jid];
    const int NS = 2 + J.D, nqp = J.nq[0], nqh = J.nq[1];
    const bool multi = nqh > kKtVirt;
    if (!multi && blockIdx.y != 0) return;
    double acc[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[q] = 0.0;
    if (!multi) {
        for (int ne = tid; ne < nqh; ne += kKtVirt) {
            const double *p1 = J.sol + (size_t)(nqp + ne) * NS;
            double x1, x2;
            koltun_row(J, p1 + 2, x1, x2);
            koltun_add(acc, x1, x2, p1[0]);
        }
        __shared__ double kred[9][32];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            double v = acc[q];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) kred[q][warp] = v;
        }
        __syncthreads();
        if (tid == 0) {
            double t[9];
            for (int q = 0; q < 9; ++q) {
                t[q] = 0.0;
                for (int w = 0; w < kKtVirt / 32; ++w) t[q] += kred[q][w];
            }
            koltun_store(J, t);
        }
        return;
    }
    __shared__ double s_x1[8][32], s_x2[8][32];
    const int vt = (int)blockIdx.y * 32 + lane;         // warp 0's lane: its virtual thread
    const int nj = (nqh + kKtVirt - 1) / kKtVirt;       // rows of a virtual thread, at most
    for (int j0 = 0; j0 < nj; j0 += 8) {
        const int ne = vt + kKtVirt * (j0 + warp);      // warp w: row j0 + w of each virtual thread
        if (ne < nqh) koltun_row(J, J.sol + (size_t)(nqp + ne) * NS + 2, s_x1[warp][lane], s_x2[warp][lane]);
        __syncthreads();
        if (warp == 0)
            for (int h = 0; h < 8; ++h) {
                const int nh = vt + kKtVirt * (j0 + h);
                if (nh < nqh) koltun_add(acc, s_x1[h][lane], s_x2[h][lane], J.sol[(size_t)(nqp + nh) * NS]);
            }
        __syncthreads();
    }
    if (warp != 0) return;
    double *part = work + work_first[jid];              // [kPlaceCtas][9], then the ticket
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        double v = acc[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) part[blockIdx.y * 9 + q] = v;
    }
    if (lane == 0) {
        __threadfence();
        unsigned *ticket = reinterpret_cast<unsigned *>(part + kPlaceCtas * 9);
        if (atomicAdd(ticket, 1u) == kPlaceCtas - 1) {   // every other partial is visible
            __threadfence();
            double t[9];
            for (int q = 0; q < 9; ++q) {
                t[q] = 0.0;
                for (int w = 0; w < kPlaceCtas; ++w) t[q] += __ldcg(part + w * 9 + q);
            }
            koltun_store(J, t);
        }
    }
}

cudaError_t launch_eig(const DyJob *d_jobs, int njobs, const long long *d_row_first, long long total_rows,
                       double *work, const long long *d_work_first, cudaStream_t st) {
    k_qrows<<<njobs, kEigThreads, 0, st>>>(d_jobs, njobs);
    k_bisect_prep<<<njobs, 256, 0, st>>>(d_jobs, njobs, work, d_work_first);
    // four lanes per eigenvalue; a matrix's few hundred eigenvalues spread over many SMs
    k_bisect<<<(unsigned)((total_rows * 4 + kBisectThreads - 1) / kBisectThreads), kBisectThreads, 0, st>>>(
        d_jobs, njobs, d_row_first, total_rows, work, d_work_first);
    k_invit<<<(unsigned)((total_rows + 31) / 32), 32, 0, st>>>(d_jobs, njobs, d_row_first, total_rows, work,
                                                               d_work_first);
    {
        const int smem = (int)(sizeof(double) * 5 * kTsMax * kIvThreads + kTsMax * kIvThreads + sizeof(double) * 2 * kTsMax);
        cudaError_t e = allow_dynamic_smem((const void *)k_invit_small);
        if (e != cudaSuccess) return e;
        k_invit_small<<<dim3(njobs, (kTsMax + kIvThreads - 1) / kIvThreads), kIvThreads, smem, st>>>(d_jobs, njobs);
    }
    k_cluster_orth<<<(unsigned)(njobs * kOrthCtas), kEigThreads, 0, st>>>(d_jobs, njobs);
    k_post<<<(unsigned)((total_rows * 4 + 127) / 128), 128, 0, st>>>(d_jobs, njobs, d_row_first, total_rows);
    k_place<<<dim3(njobs, kPlaceCtas), kPlaceThreads, 0, st>>>(d_jobs, njobs, work, d_work_first);
    k_koltun<<<dim3(njobs, kPlaceCtas), kPlaceThreads, 0, st>>>(d_jobs, njobs, work, d_work_first);
    return cudaGetLastError();
}

void eig_smem_init() { allow_dynamic_smem((const void *)k_invit_small); }

}  // namespace bd
