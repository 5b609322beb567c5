// k_dyson.cu -- K3-K5: Dyson matrix assembly, batched FP64 symmetric
// eigensolve, quasiparticle / quasihole split and Koltun partial sums.
//
// Restates DysonMatrix (source/BcDor-DysonMatrix.cpp:123-532) and Calc_En
// (:542-594).  The reference calls LAPACK dsyevd for all eigenvectors but only
// uses the first D components of each (:448-470).  Here:
//   K3 k_dyson_assemble   fills the dense matrix row by row (:269-390),
//   K4a k_tridiag_small   Householder reduction A = Q T Q^T of a matrix of order
//                         <= 160 in one CTA's shared memory, with the first D rows of Q,
//       k_tridiag         the same for larger orders, one thread-block cluster per
//                         matrix (rows split across the CTAs, Q's rows by k_qrows),
//   K4b..K5 (k_eig.cu)    eigenvalues and the first D eigenvector components of T,
//                         back-transformed, split by E_F, Koltun sums.
#include <algorithm>
#include <atomic>
#include <cooperative_groups.h>
#include "bd_common.cuh"
#include "bd_kernels.h"
#include "df64.cuh"

namespace cg = cooperative_groups;

namespace bd {

// ---------------------------------------------------------------- K3 assembly
// Row order of the full matrix: D one-body rows, nfw forward poles, nbk backward poles.
//
// Deflation: a pole row whose every off-diagonal entry is exactly zero (no coupling to
// the orbitals, no beta to its neighbours, no fishbone entry) is an eigenvector of
// the Dyson matrix by itself: eigenvalue its diagonal, no strength.  The deflated
// tails of exhausted Lanczos chains are such rows, often most of a chain.  They are
// taken out before the eigensolve; the matrix keeps the other rows in their order.

// value of the coupling of pole i of part (0 fw, 1 bk) to orbital d
__device__ inline double dy_mcoup(const DyJob &J, int part, int i, int d) {
    const int NT = J.nden + J.D;
    if (part == 0) return J.fw_rows ? J.fw_rows[(size_t)i * NT + J.nden + d] : J.M_fw[(size_t)d * J.nfw + i];
    return J.bk_rows ? J.bk_rows[(size_t)i * NT + J.nden + d] : J.M_bk[(size_t)d * J.nbk + i];
}

__device__ inline double dy_diag(const DyJob &J, int part, int i) {
    const int NT = J.nden + J.D;
    const double *rows = part == 0 ? J.fw_rows : J.bk_rows;
    return rows ? rows[(size_t)i * NT] : (part == 0 ? J.E_fw[i] : J.E_bk[i]);
}

// whether full-matrix row r has an off-diagonal entry, apart from the fishbone
// entries of a branch's start row s-1 to the later rows (k_dyson_deflate marks
// those from the later rows' side)
__device__ inline bool dy_coupled(const DyJob &J, int r) {
    const int D = J.D;
    if (r < D) return true;
    const int part = (r < D + J.nfw) ? 0 : 1;
    const int i = r - (part == 0 ? D : D + J.nfw);
    const int np = part == 0 ? J.nfw : J.nbk;
    for (int d = 0; d < D; ++d) if (dy_mcoup(J, part, i, d) != 0.0) return true;
    const bool lz = part == 0 ? J.lanczos_fw : J.lanczos_bk;
    if (!lz) return false;
    const int NT = J.nden + D;
    const double *rows = part == 0 ? J.fw_rows : J.bk_rows;
    const int *ipiv = part == 0 ? J.ipiv_fw : J.ipiv_bk;
    if (i >= 1 && rows[(size_t)i * NT + 1] != 0.0) return true;
    if (i + 1 < np && rows[(size_t)(i + 1) * NT + 1] != 0.0) return true;
    for (int nc = 1; nc < ipiv[0]; ++nc) {
        const int s = ipiv[nc + 1];
        if (s < 1 || s >= np) continue;
        if (i >= s && rows[(size_t)i * NT + 1 + nc] != 0.0) return true;
    }
    return false;
}

// Row r >= s of a branch starting at s with a fishbone entry: row s-1 is coupled.
__device__ inline void dy_mark_branch_starts(const DyJob &J, int r, int *flag) {
    const int D = J.D;
    if (r < D) return;
    const int part = (r < D + J.nfw) ? 0 : 1;
    const int off = part == 0 ? D : D + J.nfw;
    const int i = r - off, np = part == 0 ? J.nfw : J.nbk;
    if (!(part == 0 ? J.lanczos_fw : J.lanczos_bk)) return;
    const int NT = J.nden + D;
    const double *rows = part == 0 ? J.fw_rows : J.bk_rows;
    const int *ipiv = part == 0 ? J.ipiv_fw : J.ipiv_bk;
    for (int nc = 1; nc < ipiv[0]; ++nc) {
        const int s = ipiv[nc + 1];
        if (s < 1 || s >= np) continue;
        if (i >= s && rows[(size_t)i * NT + 1 + nc] != 0.0) flag[off + s - 1] = 1;
    }
}

// One CTA per matrix: the compact index of every kept row (work area, ints; -1 for a
// deflated row), the compact order into the job, and the deflated rows' solutions
// [W, 0, 0 ..] staged behind R after the nc rows the eigensolver will stage.
constexpr int kDfThreads = 256;

__global__ void __launch_bounds__(kDfThreads) k_dyson_deflate(DyJob *jobs, int njobs, double *work,
                                                              const long long *work_first) {
    const int jid = blockIdx.x;
    if (jid >= njobs) return;
    const DyJob J = jobs[jid];
    const int n = J.n, D = J.D, NS = 2 + D, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int *map = reinterpret_cast<int *>(work + work_first[jid]);
    __shared__ int wsum[kDfThreads / 32][2];
    __shared__ int s_keep, s_defl;
    if (tid == 0) { s_keep = 0; s_defl = 0; }
    __syncthreads();
    double *st = J.R + (size_t)D * n;
    int nkept_total = 0;
    // first pass: keep flags (a branch's start row from its later rows' side), then
    // the count of kept rows (the deflated rows' staged positions start after them)
    for (int r = tid; r < n; r += kDfThreads) map[r] = dy_coupled(J, r);
    __syncthreads();
    for (int r = tid; r < n; r += kDfThreads) dy_mark_branch_starts(J, r, map);
    __syncthreads();
    for (int b = 0; b < n; b += kDfThreads) {
        const int r = b + tid;
        const int keep = (r < n) ? map[r] : 0;
        int x = __syncthreads_count(keep);
        nkept_total += x;
    }
    // second pass: ranks among kept / deflated rows, in row order
    for (int b = 0; b < n; b += kDfThreads) {
        const int r = b + tid;
        const int keep = (r < n) ? map[r] : 0, defl = (r < n) ? !keep : 0;
        int xk = keep, xd = defl;
        for (int o = 1; o < 32; o <<= 1) {
            const int yk = __shfl_up_sync(0xffffffffu, xk, o), yd = __shfl_up_sync(0xffffffffu, xd, o);
            if (lane >= o) { xk += yk; xd += yd; }
        }
        if (lane == 31) { wsum[warp][0] = xk; wsum[warp][1] = xd; }
        __syncthreads();
        int ok = s_keep, od = s_defl;
        for (int q = 0; q < warp; ++q) { ok += wsum[q][0]; od += wsum[q][1]; }
        if (r < n) {
            if (keep) {
                map[r] = ok + xk - 1;
            } else {
                map[r] = -1;
                const int part = (r < D + J.nfw) ? 0 : 1;
                const int i = r - (part == 0 ? D : D + J.nfw);
                double *row = st + (size_t)(nkept_total + od + xd - 1) * NS;
                row[0] = dy_diag(J, part, i);
                for (int q = 1; q < NS; ++q) row[q] = 0.0;
            }
        }
        __syncthreads();
        if (tid == kDfThreads - 1) { s_keep = ok + xk; s_defl = od + xd; }
        __syncthreads();
    }
    if (tid == 0) jobs[jid].nc = nkept_total;
}

// One thread per full-matrix row; kept rows are written at their compact index, in a
// matrix of order nc (deflated columns hold zeros in every kept row).  Only the lower
// triangle (columns up to the row's own) is written: the reductions read nothing else,
// and every entry right of the diagonal (a model-space row's pole couplings, the beta
// to the next row, a branch start's fishbone entries) is also left of it in its
// partner row.
__global__ void k_dyson_assemble(const DyJob *jobs, int njobs, const long long *row_first, long long total_rows,
                                 const double *work, const long long *work_first) {
    long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= total_rows) return;
    int lo = 0, hi = njobs - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (row_first[mid] <= g) lo = mid; else hi = mid - 1; }
    const DyJob J = jobs[lo];
    const int r = (int)(g - row_first[lo]);
    const int *map = reinterpret_cast<const int *>(work + work_first[lo]);
    const int cr = map[r];
    if (cr < 0) return;
    const int nc = J.nc, D = J.D, nfw = J.nfw, nbk = J.nbk;
    double *Ar = J.A + (size_t)cr * nc;
    for (int c = 0; c <= cr; ++c) Ar[c] = 0.0;
    auto put = [&](int c, double v) { const int cc = map[c]; if (cc >= 0 && cc <= cr) Ar[cc] = v; };
    if (r < D) {   // the model-space rows are never deflated and come first: cr == r
        for (int c = 0; c <= r; ++c) Ar[c] = J.sig1b[r * D + c] + J.sighf[r * D + c];
        return;
    }
    const int part = (r < D + nfw) ? 0 : 1;
    const int off = part == 0 ? D : D + nfw;
    const int np = part == 0 ? nfw : nbk;
    const int i = r - off;
    const bool lz = part == 0 ? J.lanczos_fw : J.lanczos_bk;
    for (int d = 0; d < D; ++d) Ar[d] = dy_mcoup(J, part, i, d);
    Ar[cr] = dy_diag(J, part, i);
    if (!lz) return;
    const int NT = J.nden + D;
    const double *rows = part == 0 ? J.fw_rows : J.bk_rows;
    const int *ipiv = part == 0 ? J.ipiv_fw : J.ipiv_bk;
    const int nbr = ipiv[0];  // branches (pivots used)
    if (i >= 1) put(r - 1, rows[(size_t)i * NT + 1]);
    // fishbone (:303-333): branch nc (1 .. nbr-1) starts at s = ipiv[nc+1];
    // row s-1 couples to every later row nr >= s with row_nr[1 + nc] (held by row nr)
    for (int nc2 = 1; nc2 < nbr; ++nc2) {
        const int s = ipiv[nc2 + 1];
        if (s < 1 || s >= np) continue;
        if (i >= s) put(off + s - 1, rows[(size_t)i * NT + 1 + nc2]);
    }
}

// ---------------------------------------------------------------- K4a Householder
constexpr int kTdThreads = 256;

__device__ inline double block_sum(double v, double *scratch) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += scratch[q];
    return s;
}

// Symmetric Householder reduction on the lower triangle.  Row i belongs to CTA
// (i mod CL) of the cluster, so the shrinking triangle stays balanced; inside a
// CTA the warps take its rows in turn.  One step k (trailing size m = n - k - 1):
//   1. every CTA reads column k below the diagonal and forms the reflector v and
//      tau itself (identical data and order, so identical results and branches);
//   2. one pass over the own rows gives the symmetric product A v: each row's
//      dot product (warp sum) and its transposed contributions A_ij v_i to p_j,
//      gathered in per-warp shared partial vectors (shared atomics only when eight
//      copies do not fit);
//   3. the CTAs' partial vectors are summed through distributed shared memory in
//      rank order; w = tau A v - (tau^2/2)(v^T A v) v;
//   4. the own rows' lower parts get A -= v w^T + w v^T.
// Two FP64 multiply-adds per stored element and step (against three with full
// storage), two cluster barriers per step.  The reflector is kept in row k,
// columns > k (unused by the lower triangle), for the back-transformation.
//
// Shared layout (doubles): v[nmax] | p[nmax] | pc[nmax] | pt[npriv][nmax] |
// pr[nmax / CL + 1] | scratch[32]
// A deflated matrix of order beyond the launch's shared-memory layout (sized for at
// most the largest order that layout can hold): the cluster leaves together before its
// first barrier, the job reports kDyStatCapacity, and a zero tridiagonal with no
// reflectors lets the eigen kernels after it finish on it at once.
__device__ inline void tridiag_beyond_layout(const DyJob &J, int rank) {
    if (rank != 0) return;
    for (int i = threadIdx.x; i < J.nc; i += blockDim.x) { J.d[i] = 0.0; J.e[i] = 0.0; J.tau[i] = 0.0; }
    if (threadIdx.x == 0) *J.stat = kDyStatCapacity;
}

__global__ void __launch_bounds__(kTdThreads) k_tridiag(const DyJob *jobs, int njobs, int nmax, int npriv) {
    cg::cluster_group cluster = cg::this_cluster();
    const int CL = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int jid = blockIdx.x / CL;
    if (jid >= njobs) return;
    const DyJob J = jobs[jid];
    const int n = J.nc;   // order after deflation
    if (n <= kTsMax) return;   // k_tridiag_small's (the whole cluster leaves together)
    if (n > nmax) { tridiag_beyond_layout(J, rank); return; }
    extern __shared__ double sm[];
    double *v = sm;
    double *p = v + nmax;
    double *pc = p + nmax;
    double *pt = pc + nmax;
    double *pr = pt + (size_t)npriv * nmax;
    double *scratch = pr + (nmax / CL + 1);
    double *A = J.A;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int kWarps = kTdThreads / 32;
    const bool priv = (npriv >= kWarps);
    double *ptw = pt + (size_t)(warp % npriv) * nmax;
    for (int k = 0; k + 2 < n; ++k) {
        const int b0 = k + 1, m = n - b0;
        // 1. reflector from column k (rows > k)
        double sig = 0.0;
        for (int t = 1 + tid; t < m; t += kTdThreads) { const double x = __ldcg(A + (size_t)(b0 + t) * n + k); sig += x * x; }
        sig = block_sum(sig, scratch);
        const double alpha = __ldcg(A + (size_t)b0 * n + k);
        double tau = 0.0, beta = alpha;
        if (sig != 0.0) {
            beta = -copysign(sqrt(alpha * alpha + sig), alpha);
            tau = (beta - alpha) / beta;
            const double scal = 1.0 / (alpha - beta);
            for (int t = tid; t < m; t += kTdThreads) v[t] = (t == 0) ? 1.0 : __ldcg(A + (size_t)(b0 + t) * n + k) * scal;
        }
        if (rank == 0 && tid == 0) { J.e[k] = beta; J.tau[k] = tau; J.d[k] = __ldcg(A + (size_t)k * n + k); }
        if (sig != 0.0) {
            for (int t = tid; t < npriv * m; t += kTdThreads) pt[(size_t)(t / m) * nmax + t % m] = 0.0;
            __syncthreads();
            // 2. own rows i = first, first + CL, ...; row part and transposed part of A v
            const int first = b0 + ((rank - b0 % CL) % CL + CL) % CL;
            for (int i = first + warp * CL; i < n; i += CL * kWarps) {
                const double *Ai = A + (size_t)i * n;
                const double vi = v[i - b0];
                double rs = 0.0;
                int j = b0 + lane;
                for (; j + 96 < i; j += 128) {
                    const double a0 = __ldcg(Ai + j), a1 = __ldcg(Ai + j + 32), a2 = __ldcg(Ai + j + 64),
                                 a3 = __ldcg(Ai + j + 96);
                    const int t = j - b0;
                    rs += a0 * v[t] + a1 * v[t + 32] + a2 * v[t + 64] + a3 * v[t + 96];
                    if (priv) {
                        ptw[t] += a0 * vi; ptw[t + 32] += a1 * vi; ptw[t + 64] += a2 * vi; ptw[t + 96] += a3 * vi;
                    } else {
                        atomicAdd(ptw + t, a0 * vi); atomicAdd(ptw + t + 32, a1 * vi);
                        atomicAdd(ptw + t + 64, a2 * vi); atomicAdd(ptw + t + 96, a3 * vi);
                    }
                }
                for (; j <= i; j += 32) {
                    const double a = __ldcg(Ai + j);
                    rs += a * v[j - b0];
                    if (j < i) {
                        if (priv) ptw[j - b0] += a * vi;
                        else atomicAdd(ptw + (j - b0), a * vi);
                    }
                }
                for (int o = 16; o > 0; o >>= 1) rs += __shfl_xor_sync(0xffffffffu, rs, o);
                if (lane == 0) pr[(i - first) / CL] = rs;
            }
            __syncthreads();
            // this CTA's share of A v: transposed partials plus its own rows' sums
            for (int t = tid; t < m; t += kTdThreads) {
                double s = 0.0;
                for (int q = 0; q < npriv; ++q) s += pt[(size_t)q * nmax + t];
                const int i = b0 + t;
                if (i >= first && (i - first) % CL == 0) s += pr[(i - first) / CL];
                pc[t] = s;
            }
            cluster.sync();
            // 3. p = tau A v summed over the cluster in rank order; w = p - (tau/2)(p.v) v
            double kv = 0.0;
            for (int t = tid; t < m; t += kTdThreads) {
                double s = 0.0;
                for (int r = 0; r < CL; ++r) s += cluster.map_shared_rank(pc, r)[t];
                s *= tau;
                p[t] = s;
                kv += s * v[t];
            }
            const double K = block_sum(kv, scratch);
            for (int t = tid; t < m; t += kTdThreads) p[t] -= 0.5 * tau * K * v[t];
            __syncthreads();
            // 4. A_ij -= v_i w_j + w_i v_j on the own rows, j <= i
            for (int i = first + warp * CL; i < n; i += CL * kWarps) {
                double *Ai = A + (size_t)i * n;
                const double vi = v[i - b0], wi = p[i - b0];
                int j = b0 + lane;
                for (; j + 96 <= i; j += 128) {
                    const int t = j - b0;
                    const double a0 = __ldcg(Ai + j), a1 = __ldcg(Ai + j + 32), a2 = __ldcg(Ai + j + 64),
                                 a3 = __ldcg(Ai + j + 96);
                    Ai[j] = a0 - (vi * p[t] + wi * v[t]);
                    Ai[j + 32] = a1 - (vi * p[t + 32] + wi * v[t + 32]);
                    Ai[j + 64] = a2 - (vi * p[t + 64] + wi * v[t + 64]);
                    Ai[j + 96] = a3 - (vi * p[t + 96] + wi * v[t + 96]);
                }
                for (; j <= i; j += 32) Ai[j] = __ldcg(Ai + j) - (vi * p[j - b0] + wi * v[j - b0]);
            }
            if (rank == 0)
                for (int t = tid; t < m; t += kTdThreads) A[(size_t)k * n + b0 + t] = v[t];
        }
        cluster.sync();
    }
    if (rank == 0 && tid == 0) {
        if (n >= 2) {
            J.d[n - 2] = __ldcg(A + (size_t)(n - 2) * n + (n - 2));
            J.e[n - 2] = __ldcg(A + (size_t)(n - 1) * n + (n - 2));
            J.tau[n - 2] = 0.0;
        }
        J.d[n - 1] = __ldcg(A + (size_t)(n - 1) * n + (n - 1));
        J.e[n - 1] = 0.0;
        J.tau[n - 1] = 0.0;
    }
    cluster.sync();
}

// ---------------------------------------------------------------- K4a'' double-float clusters
// The cluster reduction above in double-float (df64.cuh) where every warp keeps its own
// partial vector (npriv = 8): k_tridiag's steps, rows and sums unchanged, the matrix's
// lower triangle turned into (hi, lo) FP32 pairs in place first (each CTA its own rows,
// from the doubles' bits), the reflector's scalars from the column scaled by a power of
// two (as k_tridiag_small forms them), and the reflectors stored for k_qrows in FP64 as
// before.  An FP64 multiply-add holds an SM sub-partition's FP64 unit for ~64 cycles;
// the double-float one is ~14 FP32 instructions.
namespace {

__device__ inline dfm::df ld_df(const double *p) {
    const float2 f = __ldcg(reinterpret_cast<const float2 *>(p));
    return dfm::df{f.x, f.y};
}
__device__ inline void st_df(double *p, dfm::df x) { *reinterpret_cast<float2 *>(p) = make_float2(x.h, x.l); }

// x as hi + lo from its bits: hi the double truncated to FP32, lo the next bits of the
// significand (rounded to FP32), then renormalised; no FP64 instruction (values inside
// the FP32 range; below it, zero)
__device__ inline dfm::df df_from_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((b >> 52) & 0x7FF) - 1023;
    if (E < -126) return dfm::df{0.0f, 0.0f};
    const unsigned s = (unsigned)(b >> 63) << 31;
    const float hi = __uint_as_float(s | ((unsigned)(E + 127) << 23) | (unsigned)((b >> 29) & 0x7FFFFFu));
    // remainder (b & (2^29 - 1)) 2^(E - 52); below 2^-126 the factor goes in two steps
    float lo = __uint2float_rn((unsigned)(b & 0x1FFFFFFFull));
    if (E - 52 >= -126) {
        lo = __fmul_rn(lo, __uint_as_float((unsigned)(E - 52 + 127) << 23));
    } else {
        lo = __fmul_rn(lo, __uint_as_float((unsigned)(E - 52 + 64 + 127) << 23));
        lo = __fmul_rn(lo, 5.42101086242752217e-20f);   // 2^-64
    }
    if (s) lo = -lo;
    return dfm::renorm(hi, lo);
}

__device__ inline dfm::df block_sum_df(dfm::df v, dfm::df *scratch) {
    v = dfm::warp_sum(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    dfm::df s{0.0f, 0.0f};
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s = dfm::add(s, scratch[q]);
    return s;
}

__device__ inline int f32_exponent(float x) { return (int)((__float_as_uint(x) >> 23) & 255u) - 127; }
__device__ inline float pow2_f32(int e) { return __uint_as_float((unsigned)(e + 127) << 23); }

}  // namespace

__global__ void __launch_bounds__(kTdThreads) k_tridiag_df(const DyJob *jobs, int njobs, int nmax, int npriv) {
    using dfm::df;
    cg::cluster_group cluster = cg::this_cluster();
    const int CL = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int jid = blockIdx.x / CL;
    if (jid >= njobs) return;
    const DyJob J = jobs[jid];
    const int n = J.nc;
    if (n <= kTsMax) return;   // k_tridiag_small's (the whole cluster leaves together)
    if (n > nmax) { tridiag_beyond_layout(J, rank); return; }
    extern __shared__ double sm[];
    df *v = reinterpret_cast<df *>(sm);
    df *p = v + nmax;
    df *pc = p + nmax;
    df *pt = pc + nmax;
    df *pr = pt + (size_t)npriv * nmax;
    df *scratch = pr + (nmax / CL + 1);
    double *A = J.A;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int kWarps = kTdThreads / 32;
    df *ptw = pt + (size_t)warp * nmax;   // npriv == kWarps: a partial vector per warp
    const df zero{0.0f, 0.0f};
    // this CTA's rows (i = rank, rank + CL, ...), lower triangle, to double-float in place
    for (int i = rank; i < n; i += CL)
        for (int j = tid; j <= i; j += kTdThreads) {
            double *a = A + (size_t)i * n + j;
            st_df(a, df_from_bits(__ldcg(a)));
        }
    cluster.sync();
    for (int k = 0; k + 2 < n; ++k) {
        const int b0 = k + 1, m = n - b0;
        // 1. reflector from column k (rows > k), every CTA alike: alpha, |x_1:|^2, the
        //    power of two that scales them into [1, 2), then beta, tau and 1/(alpha - beta)
        df s2 = zero;
        for (int t = 1 + tid; t < m; t += kTdThreads) { const df x = ld_df(A + (size_t)(b0 + t) * n + k); s2 = dfm::fma(x, x, s2); }
        s2 = block_sum_df(s2, scratch);
        const df al = ld_df(A + (size_t)b0 * n + k);
        const bool nz = (s2.h != 0.0f || s2.l != 0.0f);
        df tau = zero, scal = zero, beta = al;
        if (nz) {
            const int ea = (al.h != 0.0f) ? f32_exponent(al.h) : -1000;
            int e = max(ea, f32_exponent(s2.h) >> 1);
            e = min(max(e, -126), 126);
            const float sg = pow2_f32(-e);
            const df alt{al.h * sg, al.l * sg}, s2t{(s2.h * sg) * sg, (s2.l * sg) * sg};
            const df x2 = dfm::fma(alt, alt, s2t);   // in [1, 12)
            const df r = dfm::rsqrt(x2, 2), nx = dfm::mul(x2, r);
            const bool ng = signbit(alt.h);
            const df aa = ng ? dfm::neg(alt) : alt;
            tau = dfm::fma(aa, r, df{1.0f, 0.0f});
            df st = dfm::rcp(dfm::add(aa, nx), 2);   // 1 / (alpha~ - beta~)
            if (ng) st = dfm::neg(st);
            scal = df{st.h * sg, st.l * sg};         // 1 / (alpha - beta)
            const df bt = ng ? nx : dfm::neg(nx);
            const float un = pow2_f32(e);
            beta = df{bt.h * un, bt.l * un};
            for (int t = tid; t < m; t += kTdThreads) v[t] = (t == 0) ? df{1.0f, 0.0f} : dfm::mul(ld_df(A + (size_t)(b0 + t) * n + k), scal);
        }
        if (rank == 0 && tid == 0) { J.e[k] = dfm::to_double(beta); J.tau[k] = dfm::to_double(tau); J.d[k] = dfm::to_double(ld_df(A + (size_t)k * n + k)); }
        if (nz) {
            for (int t = tid; t < kWarps * m; t += kTdThreads) pt[(size_t)(t / m) * nmax + t % m] = zero;
            __syncthreads();
            // 2. own rows: row part and transposed part of A v (two chains per lane)
            const int first = b0 + ((rank - b0 % CL) % CL + CL) % CL;
            for (int i = first + warp * CL; i < n; i += CL * kWarps) {
                const double *Ai = A + (size_t)i * n;
                const df vi = v[i - b0];
                df rs0 = zero, rs1 = zero;
                int j = b0 + lane;
                for (; j + 32 < i; j += 64) {
                    const int t = j - b0;
                    const df a0 = ld_df(Ai + j), a1 = ld_df(Ai + j + 32);
                    rs0 = dfm::fma(a0, v[t], rs0);
                    rs1 = dfm::fma(a1, v[t + 32], rs1);
                    ptw[t] = dfm::fma(a0, vi, ptw[t]);
                    ptw[t + 32] = dfm::fma(a1, vi, ptw[t + 32]);
                }
                for (; j <= i; j += 32) {
                    const df a = ld_df(Ai + j);
                    rs0 = dfm::fma(a, v[j - b0], rs0);
                    if (j < i) ptw[j - b0] = dfm::fma(a, vi, ptw[j - b0]);
                }
                const df rs = dfm::warp_sum(dfm::add(rs0, rs1));
                if (lane == 0) pr[(i - first) / CL] = rs;
            }
            __syncthreads();
            for (int t = tid; t < m; t += kTdThreads) {
                df s = zero;
                for (int q = 0; q < kWarps; ++q) s = dfm::add(s, pt[(size_t)q * nmax + t]);
                const int i = b0 + t;
                if (i >= first && (i - first) % CL == 0) s = dfm::add(s, pr[(i - first) / CL]);
                pc[t] = s;
            }
            cluster.sync();
            // 3. p = tau A v over the cluster in rank order; w = p - (tau/2)(p.v) v
            df kv = zero;
            for (int t = tid; t < m; t += kTdThreads) {
                df s = zero;
                for (int r = 0; r < CL; ++r) s = dfm::add(s, cluster.map_shared_rank(pc, r)[t]);
                s = dfm::mul(s, tau);
                p[t] = s;
                kv = dfm::fma(s, v[t], kv);
            }
            const df K = block_sum_df(kv, scratch);
            const df nK = dfm::neg(dfm::mul(df{0.5f * tau.h, 0.5f * tau.l}, K));
            for (int t = tid; t < m; t += kTdThreads) p[t] = dfm::fma(nK, v[t], p[t]);
            __syncthreads();
            // 4. A_ij -= v_i w_j + w_i v_j on the own rows, j <= i
            for (int i = first + warp * CL; i < n; i += CL * kWarps) {
                double *Ai = A + (size_t)i * n;
                const df vi = v[i - b0], wi = p[i - b0];
                for (int j = b0 + lane; j <= i; j += 32) {
                    const int t = j - b0;
                    const df t2 = dfm::fma(vi, p[t], dfm::mul(wi, v[t]));
                    st_df(Ai + j, dfm::add(ld_df(Ai + j), dfm::neg(t2)));
                }
            }
            if (rank == 0)   // the reflector for k_qrows, in FP64, in row k right of the diagonal
                for (int t = tid; t < m; t += kTdThreads) A[(size_t)k * n + b0 + t] = dfm::to_double(v[t]);
        }
        cluster.sync();
    }
    if (rank == 0 && tid == 0) {
        if (n >= 2) {
            J.d[n - 2] = dfm::to_double(ld_df(A + (size_t)(n - 2) * n + (n - 2)));
            J.e[n - 2] = dfm::to_double(ld_df(A + (size_t)(n - 1) * n + (n - 2)));
            J.tau[n - 2] = 0.0;
        }
        J.d[n - 1] = dfm::to_double(ld_df(A + (size_t)(n - 1) * n + (n - 1)));
        J.e[n - 1] = 0.0;
        J.tau[n - 1] = 0.0;
    }
    cluster.sync();
}

// ---------------------------------------------------------------- K4a' small matrices
// Matrices of order nc <= kTsMax (after deflation nearly all: the N_max = 10 channels
// reduce to 11..94) are reduced by one CTA with the matrix resident in shared memory
// (both triangles), and the first D rows of Q = H_0 ... H_{n-3} (what k_qrows forms
// for the cluster path) are updated in the same pass.  The element arithmetic is
// double-float (df64.cuh: hi + lo FP32 pairs, ~48 bits): on this GPU an FP64 FMA
// issues at 1/64 of the FP32 rate.
//
// Step k reduces column k (x = rows k+1 .. n-1, alpha = x_0) with H = I - tau v v^T,
// v = (1, s x_1 ..), s = 1 / (alpha - beta), beta = -sign(alpha) |x|.  The column is
// carried scaled by a power of two, xs = 2^-e x with max(|alpha|, |x_1:|) in [1, 2)
// (exact), so the reflector's scalars need no range checks.  Every sum the step needs
// is formed from xs without the scalars, which lets one thread form them beside the
// product instead of before it:
//   S_i = sum_{t>=1} A_{b0+i, b0+t} xs_t   (eight parts per row, over fifteen warps),
//   Q = sum_{i>=1} xs_i S_i                 (per-warp partials of the same pass),
//   A v = A_{:,0} + s S,  v^T A v = A_00 + 2 s S_0 + s^2 Q,  p = tau A v,
//   w = p - (tau^2 / 2) (v^T A v) v,  A <- A - v w^T - w v^T,  R <- R - tau (R v) v^T.
// One step, three barriers:
//   2. warp 0, lane 0: beta, tau and s from (alpha, |x_1:|^2) in double-float (Newton's
//      reciprocal and square root); warps 1..15: the parts of S and Q; the last D
//      warps also R_d[b0+1:] . xs[1:];
//   3. every thread of a trailing row t: v_t and w_t from the parts (each thread sums
//      the warp partials of Q itself, in one fixed order), and the R update;
//   4. the rank-2 update of the trailing block, each result also at its mirror
//      position; warp 0 takes column k + 1 and scales it for the next step.
constexpr int kTsThreads = 512;
constexpr int kTsParts = 8;                   // threads per row of the symmetric product
constexpr int kTsIt = kTsMax / 32;            // column entries per lane of warp 0
static_assert(kTsMax % 32 == 0, "warp 0 holds a column in kTsIt entries per lane");
static_assert(2 * kTsMax <= kTsThreads, "the R update keeps at least half the threads");

__device__ inline double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Binary exponent of a non-zero float (denormals give -127), and 2^e for -126 <= e <= 127.
__device__ inline int f32_exp(float x) { return (int)((__float_as_uint(x) >> 23) & 255u) - 127; }
__device__ inline float f32_pow2(int e) { return __uint_as_float((unsigned)(e + 127) << 23); }

__global__ void __launch_bounds__(kTsThreads) k_tridiag_small(const DyJob *jobs, int njobs) {
    using dfm::df;
    const int jid = blockIdx.x;
    if (jid >= njobs) return;
    const DyJob J = jobs[jid];
    const int n = J.nc, D = J.D;
    if (n > kTsMax) return;   // the cluster kernel's
    const int ld = n | 1;     // odd stride: column reads hit distinct bank pairs
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    extern __shared__ double sm[];
    df *A = reinterpret_cast<df *>(sm);      // [n][ld], both triangles
    df *v = A + (size_t)n * ld;              // [n]
    df *ph = v + n;                          // [kTsParts][n] parts of S
    df *w = ph + kTsParts * n;               // [n]
    df *xs = w + n;                          // [n] the step's scaled column
    df *R = xs + n;                          // [D][n]
    __shared__ df s_col[2][2];               // alpha and |x_1:|^2 of a column, scaled, by parity
    __shared__ int s_nz[2], s_exp[2];        // the column has a reflector; e, by parity
    __shared__ df s_sc[2];                   // tau, s of the step
    __shared__ df s_q[kTsThreads / 32];      // per-warp partials of Q
    __shared__ df s_rx[8][2];                // R_d[b0+1:] . xs[1:], R_d[b0] before the update
    for (int q = tid; q < n * n; q += kTsThreads) {
        const int i = q / n, j = q - i * n;
        if (j <= i) {   // the assembled lower triangle, mirrored
            const df x = dfm::from_double(__ldcg(J.A + q));
            A[(size_t)i * ld + j] = x;
            A[(size_t)j * ld + i] = x;
        }
    }
    for (int q = tid; q < D * n; q += kTsThreads) R[q] = df{((q % n) == (q / n)) ? 1.0f : 0.0f, 0.0f};
    __syncthreads();
    const df zero{0.0f, 0.0f};
    // Warp 0: column kc's entries below the diagonal (rows kc+1 .. n-1), alpha, the sum of
    // the other entries' squares, the power of two 2^-e that brings the larger of |alpha|
    // and that norm into [1, 2), and xs = 2^-e x, into the column's parity slots.
    auto scale_column = [&](int kc) {
        const int b = kc + 1, mc = n - b, par = kc & 1;
        df x[kTsIt];
        df s2 = zero;
#pragma unroll
        for (int it = 0; it < kTsIt; ++it) {
            const int t = lane + 32 * it;
            x[it] = (t < mc) ? A[(size_t)(b + t) * ld + kc] : zero;
            if (t >= 1) s2 = dfm::fma(x[it], x[it], s2);
        }
        s2 = dfm::warp_sum(s2);
        const df al{__shfl_sync(0xffffffffu, x[0].h, 0), __shfl_sync(0xffffffffu, x[0].l, 0)};
        const int ea = (al.h != 0.0f) ? f32_exp(al.h) : -1000;
        const int es = (s2.h != 0.0f) ? (f32_exp(s2.h) >> 1) : -1000;   // floor(e / 2)
        int e = max(ea, es);
        e = (e == -1000) ? 0 : min(max(e, -126), 126);
        const float sg = f32_pow2(-e);
#pragma unroll
        for (int it = 0; it < kTsIt; ++it) {
            const int t = lane + 32 * it;
            if (t < mc) xs[t] = df{x[it].h * sg, x[it].l * sg};
        }
        if (lane == 0) {
            s_nz[par] = (s2.h != 0.0f || s2.l != 0.0f);
            s_exp[par] = e;
            s_col[par][0] = df{al.h * sg, al.l * sg};
            s_col[par][1] = df{(s2.h * sg) * sg, (s2.l * sg) * sg};
        }
    };
    if (n >= 3 && warp == 0) scale_column(0);
    __syncthreads();
    for (int k = 0; k + 2 < n; ++k) {
        const int b0 = k + 1, m = n - b0, par = k & 1;
        if (!s_nz[par]) {                    // column already reduced: H_k = I
            if (warp == 0) {
                if (lane == 0) A[(size_t)k * ld + k + 2] = zero;   // tau (e is alpha, in place)
                if (k + 3 < n) scale_column(k + 1);
            }
            __syncthreads();
            continue;
        }
        // 2. the reflector's scalars (warp 0, lane 0) beside the parts of S and Q
        if (warp == 0) {
            if (lane == 0) {
                const df al = s_col[par][0], s2 = s_col[par][1];
                const df x2 = dfm::fma(al, al, s2);   // in [1, 12)
                const df r = dfm::rsqrt(x2, 1), nx = dfm::mul(x2, r);
                const bool ng = signbit(al.h);
                const df aa = ng ? dfm::neg(al) : al;
                const df tau = dfm::fma(aa, r, df{1.0f, 0.0f});   // (beta - alpha) / beta = 1 + |alpha| / |x|
                df s = dfm::rcp(dfm::add(aa, nx), 1);               // 1 / (alpha - beta) = sign(alpha) / (|alpha| + |x|)
                if (ng) s = dfm::neg(s);
                s_sc[0] = tau;
                s_sc[1] = s;
                s_q[0] = zero;
                // e and tau of the step into row k, right of the diagonal (never read again),
                // converted to FP64 with d at the end: FP64 instructions stay off this chain
                const float un = f32_pow2(s_exp[par]);        // beta = 2^e beta~
                const df beta = ng ? nx : dfm::neg(nx);
                A[(size_t)k * ld + k + 1] = df{beta.h * un, beta.l * un};
                A[(size_t)k * ld + k + 2] = tau;
            }
        } else {
            if (warp >= kTsThreads / 32 - D) {   // R_d[b0+1:] . xs[1:] and R_d[b0]
                const int d = kTsThreads / 32 - 1 - warp;
                df sx = zero;
                for (int t = 1 + lane; t < m; t += 32) sx = dfm::fma(R[(size_t)d * n + b0 + t], xs[t], sx);
                sx = dfm::warp_sum(sx);
                if (lane == 0) { s_rx[d][0] = sx; s_rx[d][1] = R[(size_t)d * n + b0]; }
            }
            df qa = zero;
            for (int u = tid - 32; u < kTsParts * m; u += kTsThreads - 32) {
                const int i = u / kTsParts, h = u - i * kTsParts;
                const int q0 = (m * h) / kTsParts, q1 = (m * (h + 1)) / kTsParts;
                const df *Ai = A + (size_t)(b0 + i) * ld + b0;   // the full row (the update mirrors)
                df acc0 = zero, acc1 = zero;   // two chains
                int q = q0 > 0 ? q0 : 1;
                for (; q + 1 < q1; q += 2) {
                    acc0 = dfm::fma(Ai[q], xs[q], acc0);
                    acc1 = dfm::fma(Ai[q + 1], xs[q + 1], acc1);
                }
                if (q < q1) acc0 = dfm::fma(Ai[q], xs[q], acc0);
                const df r = dfm::add(acc0, acc1);
                ph[h * n + i] = r;
                if (i >= 1) qa = dfm::fma(xs[i], r, qa);
            }
            qa = dfm::warp_sum(qa);
            if (lane == 0) s_q[warp] = qa;
        }
        __syncthreads();
        // 3. v and w of every trailing row; R <- R - tau (R v) v^T
        const df tau = s_sc[0], s = s_sc[1];
        if (tid < m) {
            const int t = tid;
            df qv[kTsThreads / 32];
#pragma unroll
            for (int q = 0; q < kTsThreads / 32; ++q) qv[q] = s_q[q];
#pragma unroll
            for (int o = kTsThreads / 64; o > 0; o >>= 1)
#pragma unroll
                for (int q = 0; q < o; ++q) qv[q] = dfm::add(qv[q], qv[q + o]);
            df p0[kTsParts], pt[kTsParts];
#pragma unroll
            for (int h = 0; h < kTsParts; ++h) { p0[h] = ph[h * n]; pt[h] = ph[h * n + t]; }
#pragma unroll
            for (int o = kTsParts / 2; o > 0; o >>= 1)
#pragma unroll
                for (int h = 0; h < o; ++h) { p0[h] = dfm::add(p0[h], p0[h + o]); pt[h] = dfm::add(pt[h], pt[h + o]); }
            // v^T A v = A_00 + s (2 S_0 + s Q); K = (tau^2 / 2) v^T A v
            const df vav = dfm::fma(s, dfm::fma(s, qv[0], dfm::add(p0[0], p0[0])), A[(size_t)b0 * ld + b0]);
            const df tk = dfm::mul(tau, tau);
            const df nK = dfm::neg(dfm::mul(df{0.5f * tk.h, 0.5f * tk.l}, vav));
            const df vt = (t == 0) ? df{1.0f, 0.0f} : dfm::mul(s, xs[t]);
            const df p = dfm::mul(tau, dfm::fma(s, pt[0], A[(size_t)(b0 + t) * ld + b0]));
            v[t] = vt;
            w[t] = dfm::fma(nK, vt, p);
        }
        // the R update on the warps that form no v and w
        const int rb = (m + 31) & ~31;
        for (int u = tid - rb; u >= 0 && u < D * m; u += kTsThreads - rb) {
            const int d = u / m, t = u - d * m;
            const df vt = (t == 0) ? df{1.0f, 0.0f} : dfm::mul(s, xs[t]);
            const df nc = dfm::neg(dfm::mul(tau, dfm::fma(s, s_rx[d][0], s_rx[d][1])));
            df &r = R[(size_t)d * n + b0 + t];
            r = dfm::fma(nc, vt, r);
        }
        __syncthreads();
        // 4. A -= v w^T + w v^T on the trailing block: warp 0 takes column k + 1 (local
        //    column 0) and then scales it for the next step; warps 1..15 the rest, rows i
        //    and m-1-i per warp so the triangle's rows balance, each result also at its mirror
        if (warp == 0) {
            for (int r = lane; r < m; r += 32) {
                df *a = A + (size_t)(b0 + r) * ld + b0;
                const df t2 = dfm::fma(w[r], v[0], dfm::mul(v[r], w[0]));
                const df x = dfm::add(*a, dfm::neg(t2));
                *a = x;
                A[(size_t)b0 * ld + b0 + r] = x;
            }
            __syncwarp();
            if (k + 3 < n) scale_column(k + 1);
        } else {
            for (int i1 = warp - 1; i1 < (m + 1) / 2; i1 += kTsThreads / 32 - 1) {
                const int i2 = m - 1 - i1;
                const int len = (i1 == i2) ? (i1 + 1) : (m + 1);
                // two entries per pass, both read before either is written: the entries
                // are distinct lower-triangle ones, so no write meets the other's reads
                for (int u = lane; u < len; u += 64) {
                    int r[2], c[2];
                    df x[2];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int uu = u + 32 * h;
                        r[h] = (uu <= i1) ? i1 : i2;
                        c[h] = (uu <= i1) ? uu : uu - i1 - 1;
                        if (uu < len && c[h] != 0) {   // column k + 1: warp 0's
                            const df t2 = dfm::fma(w[r[h]], v[c[h]], dfm::mul(v[r[h]], w[c[h]]));
                            x[h] = dfm::add(A[(size_t)(b0 + r[h]) * ld + b0 + c[h]], dfm::neg(t2));
                        } else {
                            c[h] = 0;
                        }
                    }
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        if (c[h] != 0) {
                            A[(size_t)(b0 + r[h]) * ld + b0 + c[h]] = x[h];
                            A[(size_t)(b0 + c[h]) * ld + b0 + r[h]] = x[h];   // the mirror, read by the next product
                        }
                }
            }
        }
        __syncthreads();
    }
    for (int k = tid; k < n; k += kTsThreads) {   // d, e, tau in FP64 (row k: d_k, e_k, tau_k)
        const df *Ak = A + (size_t)k * ld + k;
        J.d[k] = dfm::to_double(Ak[0]);
        J.e[k] = (k + 1 < n) ? dfm::to_double(Ak[1]) : 0.0;
        J.tau[k] = (k + 2 < n) ? dfm::to_double(Ak[2]) : 0.0;
    }
    for (int q = tid; q < D * n; q += kTsThreads) J.R[q] = dfm::to_double(R[q]);
}

size_t tridiag_small_smem_bytes(int nmax, int Dmax) {
    const size_t n = (size_t)std::min(nmax, kTsMax);
    return sizeof(double) * (n * (n | 1) + (size_t)(kTsParts + 3) * n + (size_t)Dmax * n);
}

// Per-warp partial vectors that fit next to the other arrays (8 = one per warp).
int tridiag_npriv(int nmax, int cluster) {
    const size_t fixed = (size_t)3 * nmax + (size_t)(nmax / cluster + 1) + 32;
    const size_t cap = (size_t)200 * 1024 / sizeof(double);
    int np = 8;
    while (np > 1 && fixed + (size_t)np * nmax > cap) --np;
    return np;
}

size_t tridiag_smem_bytes(int nmax, int cluster) {
    return sizeof(double) * ((size_t)(3 + tridiag_npriv(nmax, cluster)) * nmax + (size_t)(nmax / cluster + 1) + 32);
}

// The largest order whose layout fits the dynamic shared memory a CTA may opt into.
// Up to the orders that leave room for two partial vectors the layout stays within
// 200 KB; beyond, it grows with the order, so the orders that fit are a prefix.
// Cached per cluster size (bd_create fills the cache, so no attribute query falls inside
// a stream capture); the GPUs a process drives are of one kind.
static std::atomic<int> g_fit_order[17];

int tridiag_fit_order(int cluster) {
    const bool cached = cluster >= 1 && cluster <= 16;
    if (cached) {
        const int v = g_fit_order[cluster].load(std::memory_order_relaxed);
        if (v) return v;
    }
    int dev = 0, optin = 0;
    cudaFuncAttributes a{}, b{};
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&a, k_tridiag) != cudaSuccess || cudaFuncGetAttributes(&b, k_tridiag_df) != cudaSuccess)
        return kTsMax + 1;   // the launch that follows reports the error
    const size_t limit = (size_t)optin - std::max(a.sharedSizeBytes, b.sharedSizeBytes);
    int lo = kTsMax + 1, hi = 1 << 22;
    while (lo < hi) {
        const int mid = lo + (hi - lo + 1) / 2;
        if (tridiag_smem_bytes(mid, cluster) <= limit) lo = mid; else hi = mid - 1;
    }
    if (cached) g_fit_order[cluster].store(lo, std::memory_order_relaxed);
    return lo;
}

void tridiag_fit_warm() {
    for (int c = 1; c <= 16; c <<= 1) tridiag_fit_order(c);
    allow_dynamic_smem((const void *)k_tridiag_small);
    allow_dynamic_smem((const void *)k_tridiag);
    allow_dynamic_smem((const void *)k_tridiag_df);
}

// Kernels launch_dyson starts for matrices of order up to nmax: deflate, assemble, the
// small-matrix reduction (and the cluster one beyond kTsMax), then launch_eig's nine.
int dyson_launch_count(int nmax) { return (nmax <= kTsMax ? 3 : 4) + 9; }

cudaError_t launch_dyson(const DyJob *d_jobs, int njobs, const long long *d_row_first, long long total_rows,
                         int nmax, int Dmax, int cluster, double *work, const long long *d_work_first, cudaStream_t st) {
    if (njobs <= 0) return cudaSuccess;
    k_dyson_deflate<<<njobs, kDfThreads, 0, st>>>(const_cast<DyJob *>(d_jobs), njobs, work, d_work_first);
    k_dyson_assemble<<<(unsigned)((total_rows + 127) / 128), 128, 0, st>>>(d_jobs, njobs, d_row_first, total_rows, work,
                                                                       d_work_first);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t ssmem = tridiag_small_smem_bytes(nmax, Dmax);
    e = allow_dynamic_smem((const void *)k_tridiag_small);
    if (e != cudaSuccess) return e;
    k_tridiag_small<<<njobs, kTsThreads, ssmem, st>>>(d_jobs, njobs);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (nmax <= kTsMax) return launch_eig(d_jobs, njobs, d_row_first, total_rows, work, d_work_first, st);
    // the full orders bound the deflated ones; the layout is sized for at most the
    // largest order shared memory holds, and larger deflated orders report it
    nmax = std::min(nmax, tridiag_fit_order(cluster));
    size_t smem = tridiag_smem_bytes(nmax, cluster);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(njobs * cluster, 1, 1);
    cfg.blockDim = dim3(kTdThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const int npriv = tridiag_npriv(nmax, cluster);
    auto kern = (npriv == kTdThreads / 32) ? k_tridiag_df : k_tridiag;   // double-float with a partial per warp
    e = allow_dynamic_smem((const void *)kern);
    if (e == cudaSuccess && cluster > 8) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    e = cudaLaunchKernelEx(&cfg, kern, d_jobs, njobs, nmax, npriv);
    if (e != cudaSuccess) return e;
    return launch_eig(d_jobs, njobs, d_row_first, total_rows, work, d_work_first, st);
}

}  // namespace bd
