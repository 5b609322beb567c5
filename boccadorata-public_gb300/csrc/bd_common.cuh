// bd_common.cuh -- device-side data structures shared by the kernels of the
// Sigma(2) -> Lanczos -> Dyson chain (sm_103a).
#pragma once
#include <cstdint>
#include <mutex>
#include <unordered_set>
#include <cuda_runtime.h>

namespace bd {

// Lets a kernel take all the dynamic shared memory a CTA may opt into, once per kernel
// in the process.  The limit is a property of the function, not of a launch: set to a
// launch's own size, contexts on other host threads (other problem sizes) could lower
// it between that setting and the launch.  bd_create registers every kernel that needs
// it, so no first setting falls inside a stream capture.
inline cudaError_t allow_dynamic_smem(const void *kernel) {
    static std::mutex mu;
    static std::unordered_set<const void *> done;
    std::lock_guard<std::mutex> lock(mu);
    if (done.count(kernel)) return cudaSuccess;
    int dev = 0, optin = 0;
    cudaFuncAttributes a{};
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, kernel);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)a.sharedSizeBytes);
    if (e == cudaSuccess) done.insert(kernel);
    return e;
}

constexpr double kSqr2 = 1.4142135623730950488016887;
constexpr int kChOff = -2, kJMult = 128, kABMult = 1024, kChMult = 5;
constexpr int kSegTable = kChMult * kJMult * 2;

// Device-resident problem: model space, propagator and interaction
// (ModSpace_t / SpProp_t / VppInt_t).  Plain pointers into device memory.
struct DevProblem {
    int nsubsh, norb, jmax, nspb;
    const int *l, *j2, *ip, *ch, *no, *orb_start, *orb_sh;
    const double *orb_xe;
    const int *np, *nh, *p_start, *h_start;
    const double *ep, *eh, *fqp, *fqh;
    int n_me;
    const int *iabJ, *icdJ;
    const double *V;
    const int *seg_str, *seg_end;
    // Row table of the sorted interaction: first and last element of the run with
    // pair index iabJ = ind_i1i2J(a, b, J), at (a * norb + b) * nJ + J; set only when
    // the list is strictly sorted by (iabJ, icdJ) inside every segment (else null).
    const int2 *rows;
    int nJ;
    // Rank of every pair index (a, b, J) among the elements of the first row of its
    // segment (-1: not there); with a complete canonical list that row holds every
    // pair of the segment, so row iab's element for pair icd sits at
    // rows[iab].x + rank(icd) - rank(iab).  Set with rows.
    const int *prank;
};

// One (Jab, ia, ib, ig) block of the Sigma(2) build of one channel.  Its poles
// occupy [fw_first, fw_first + nfw) of the channel's forward rows (same for bk);
// its V' coefficients occupy vp_first .. vp_first + D*na*nb*ng (dense,
// [d][alpha][beta][gamma], entries the reference skips are left unused).
struct S2Block {
    int ch;              // channel (subshell I)
    int Jab, ia, ib, ig;
    int nJab, nJgd;
    int fw_first, nfw;   // global pole index of the block's first fw pole
    int bk_first, nbk;
    long long vp_first;  // offset into the V' scratch
    int nvp;             // D * no[ia] * no[ib] * no[ig]
    double x3;           // sqrt((2Jab+1)/(2j_I+1)), correctly rounded (formed on the host)
};

// Per-channel layout of the structure-of-arrays Sigma(2) on the device:
// E[k], S2[k] at pole offset + k, M[d][k] at moff + d*N + k.
struct ChanSig {
    int D, nfw, nbk;
    int fw_off, bk_off;          // pole offsets (global)
    long long mfw_off, mbk_off;  // offsets into the M arrays
};

// Leading dimension of a chain's vector store: room for any cluster size up to 16
// with 4-aligned slices (CL * round4(ceil(N / CL)) <= N + 63).
__host__ __device__ inline int lz_ld(int N) { return (N + 64 + 31) / 32 * 32; }

// One Lanczos chain set (channel x direction), processed by one thread-block cluster.
struct LzChain {
    int N, D, L;            // poles, orbitals, Lanczos vectors to compute
    int n_used;             // pivots actually iterated (n_itr > 0)
    int nden_out;           // leading doubles per output row (= n_pvt + 1)
    int ld;                 // leading dimension of the vector store (>= CL * S, multiple of 32)
    int S;                  // pole rows per CTA (multiple of 4)
    const double *E;        // [N]   sorted energies
    const double *M;        // [D][N] sorted couplings
    const float *Mf;        // [D][N] FP32 copy of M (read by the FP32-vector form only)
    const double *piv;      // [n_used][D] normalised pivots in use order
    const int *start;       // [n_used + 1] first Lanczos index of each pivot chain
    const int *last;        // [n_used] last index of each chain (may exceed L-1)
    void *V;                // [L][ld] Lanczos vectors (double or float)
    double *out;            // [L][nden_out + D] rows
    int *stat;              // [2]: number of two-pass steps, error flag
    char *slice;            // per-CTA E / w / touched slices in global memory (large chains), CTA r at
    long long slice_stride; //   slice + r * slice_stride; unused when the slices live in shared memory
    // Energy groups of the sorted poles (runs of equal E), from k_lz_groups: gE[q], and
    // gInfo[0] = number of groups, gInfo[1 + q] = m_q - rank(M_q), the dimension of the
    // group's eigenvectors of E that no coupling reaches.  nullptr: no deflation.
    const double *gE;
    const int *gInfo;
    int *rowslot;           // [L] vector slot of every row, -1 for a deflated row (written at the end)
};

// Energy-group scratch of a chain of N poles, behind gE [2N doubles] and gInfo [N + 1
// ints]: the Gram pieces of the groups of more than kGrpSmall poles (a piece is at most
// kGrpPiece of a group's poles) -- the piece list {group, first pole, end pole}, every
// group's first piece, the pieces' partial Gram matrices (up to 36 entries, the lower
// triangle of 8 x 8) and the number of pieces.
constexpr int kGrpSmall = 64;
constexpr int kGrpPiece = 1024;
constexpr int kGramEntries = 36;
__host__ __device__ inline long long lz_gram_cap(long long N) { return N / (kGrpSmall + 1) + N / kGrpPiece + 2; }
struct GrpScratch {
    int *first;     // [N]   first piece of group q (groups of more than kGrpSmall poles)
    int4 *list;     // [cap] pieces: group, first pole, end pole
    double *part;   // [cap][kGramEntries] partial Gram matrices
    int *count;     // [1]   pieces
};
__host__ __device__ inline long long lz_grp_first_off(long long N) { return (16 * N + 4 * (N + 1) + 15) / 16 * 16; }
__host__ __device__ inline long long lz_grp_list_off(long long N) { return lz_grp_first_off(N) + (4 * N + 15) / 16 * 16; }
__host__ __device__ inline long long lz_grp_part_off(long long N) { return lz_grp_list_off(N) + 16 * lz_gram_cap(N); }
__host__ __device__ inline long long lz_grp_count_off(long long N) {
    return lz_grp_part_off(N) + 8 * (long long)kGramEntries * lz_gram_cap(N);
}
// bytes of the whole group scratch, a multiple of 256
__host__ __device__ inline long long lz_group_bytes(long long N) { return (lz_grp_count_off(N) + 16 + 255) / 256 * 256; }
__host__ __device__ inline GrpScratch lz_grp_scratch(const double *gE, long long N) {
    char *g = reinterpret_cast<char *>(const_cast<double *>(gE));
    return GrpScratch{reinterpret_cast<int *>(g + lz_grp_first_off(N)), reinterpret_cast<int4 *>(g + lz_grp_list_off(N)),
                      reinterpret_cast<double *>(g + lz_grp_part_off(N)), reinterpret_cast<int *>(g + lz_grp_count_off(N))};
}

// Global scratch of one chain's slices: enough for any cluster size up to 16 with FP64
// slices (E, w and E w as doubles and a touched byte: 25 bytes per pole, each CTA's share
// rounded up to 256 bytes); a multiple of 256 bytes, so consecutive chains' slices stay
// aligned.
constexpr int kLzSliceBytesPerPole = 25;
__host__ __device__ inline long long lz_slice_bytes(long long N) {
    return (kLzSliceBytesPerPole * N + 16 * (kLzSliceBytesPerPole * 4 + 256) + 255) / 256 * 256;
}

// Doubles of one pass's partial sums in the Lanczos kernel: a recurrence step's pass
// sums two products per vector (with w and with E w) over the stored vectors, w and
// E w, and one per coupling vector M_d.
__host__ __device__ inline int lz_partials_per_pass(int rmax) { return 2 * ((rmax + 1) & ~1) + 32; }

// One Dyson eigenproblem.
struct DyJob {
    int ch, D, n, j2;
    int nc;                  // order of the matrix after deflation (set by k_dyson_deflate)
    int nfw, nbk;            // pole-block sizes in the matrix
    int nden;                // leading doubles of the self-energy rows
    int lanczos_fw, lanczos_bk;  // whether the fw / bk parts are Lanczos rows
    const double *fw_rows;   // [nfw][nden + D] (Lanczos) or nullptr (plain: SoA below)
    const double *bk_rows;
    const int *ipiv_fw, *ipiv_bk;  // [2 + n_used] start indices of the g branches
    const double *E_fw, *M_fw;     // plain Sigma(2), SoA (M: [D][nfw])
    const double *E_bk, *M_bk;
    const double *sighf;     // [D][D] static self-energy
    const double *sig1b;     // [D][D]
    double efermi;
    const double *efp;       // the Fermi energy in device memory (it follows device-side updates
                             // of the propagator), or nullptr: efermi
    double *A;               // [n][n] scratch (row-major)
    double *d, *e, *tau;     // [n] tridiagonal diagonal, off-diagonal, reflector scalars
    int *blk;                // [2n] first and last position of each position's tridiagonal block
    double *R;               // [D][n] first D rows of Q, then n staged rows of 2 + D
    double *sol;             // [n][2 + D] output rows (qp first, then qh)
    int *nq;                 // [2] n_qp, n_qh
    double *koltun;          // [3]
    int *stat;               // [1] error flag
};

__host__ __device__ inline int tri_fail(int a, int b, int c) { return (a + b < c) || (b + c < a) || (c + a < b); }
__host__ __device__ inline int ind_chipJ(int ch, int ip, int J) { return ((ch - kChOff) * 2 + ip) * kJMult + J; }
__host__ __device__ inline int ind_i1i2J(int i1, int i2, int J) { return (i1 * kABMult + i2) * kJMult + J; }

// VppInt_t::get (source/BcDor-Vpp_potential.cpp:557-607): exchange phase, ordering
// of the two pair keys, binary search inside the (charge, parity, J) segment.
__device__ inline double vget(const DevProblem &P, int ia, int ib, int ic, int id, int J) {
    int isha = P.orb_sh[ia], ishb = P.orb_sh[ib];
    int ip = (P.ip[isha] + P.ip[ishb]) % 2;
    int ch = P.ch[isha] + P.ch[ishb];
    int iph = 0, iab, icd;
    if (ia <= ib) iab = ind_i1i2J(ia, ib, J);
    else { iab = ind_i1i2J(ib, ia, J); iph += (P.j2[isha] + P.j2[ishb]) / 2 - J + 1; }
    if (ic <= id) icd = ind_i1i2J(ic, id, J);
    else {
        int ishc = P.orb_sh[ic], ishd = P.orb_sh[id];
        icd = ind_i1i2J(id, ic, J); iph += (P.j2[ishc] + P.j2[ishd]) / 2 - J + 1;
    }
    // the phase (-1)^iph as a sign flip on the integer pipe: V * (+-1) exactly, without an
    // FP64 multiply (one FP64 instruction holds the sub-partition's FP64 unit ~64 cycles)
    const unsigned long long xph = (abs(iph) % 2) ? 0x8000000000000000ull : 0ull;
    auto phased = [xph](double x) { return __longlong_as_double((long long)((unsigned long long)__double_as_longlong(x) ^ xph)); };
    if (icd < iab) { int t = iab; iab = icd; icd = t; }
    int key = ind_chipJ(ch, ip, J);
    int lo = P.seg_str[key], hi = P.seg_end[key];
    if (lo < 0 || hi < 0) return 0.0;
    if (P.rows) {
        // On a list sorted by (iabJ, icdJ) inside the segment the reference's search
        // below finds the one element with both indices, or nothing; so does a search
        // of icdJ inside iab's run, when the run lies in this segment.
        if (J >= P.nJ) return 0.0;
        const int a = iab / (kJMult * kABMult), b = (iab / kJMult) % kABMult;
        const size_t pa = ((size_t)a * P.norb + b) * P.nJ + J;
        const int2 rw = P.rows[pa];
        if (rw.x < lo || rw.y > hi) return 0.0;
        {   // the position a complete list puts it at; pairs are unique, so a match is it
            const int c = icd / (kJMult * kABMult), d = (icd / kJMult) % kABMult;
            const int r1 = P.prank[((size_t)c * P.norb + d) * P.nJ + J], r0 = P.prank[pa];
            if (r1 >= 0 && r0 >= 0) {
                const int pos = rw.x + (r1 - r0);
                if (pos >= rw.x && pos <= rw.y && P.icdJ[pos] == icd) return phased(P.V[pos]);
            }
        }
        int f = rw.x, l = rw.y;
        while (f <= l) {
            const int mid = (f + l) >> 1;
            const int cm = P.icdJ[mid];
            if (cm == icd) return phased(P.V[mid]);
            if (cm < icd) f = mid + 1; else l = mid - 1;
        }
        return 0.0;
    }
    for (int it = 0; it < 100; ++it) {   // the reference's bounded search
        int mid = (hi + lo) / 2;
        int am = P.iabJ[mid];
        int test = (iab < am);
        if (am == iab) {
            int cm = P.icdJ[mid];
            if (cm == icd) return phased(P.V[mid]);
            test = (icd < cm);
        }
        if (test) hi = mid;
        else { lo = mid; if (lo < hi) lo++; }
    }
    return 0.0;
}

// FP64 division and square root are dependent chains of about ten FP64 instructions,
// each of which holds an SM sub-partition's FP64 unit for ~64 cycles on this GPU; where
// a few ulp suffice they are replaced by an FP32 seed refined by Newton's iteration
// (the relative error squares at every step).
//
// 1/q to ~2^-48 (one step) from the FP32 reciprocal; plain division outside the FP32 range.
__device__ inline double rcp_newton(double q) {
    const double aq = fabs(q);
    if (aq > 1e-36 && aq < 1e36) {
        const double r = (double)__frcp_rn((float)q);
        return fma(r, fma(-q, r, 1.0), r);
    }
    return 1.0 / q;
}

// 1/q to a few ulp (two steps)
__device__ inline double rcp_newton2(double q) {
    const double aq = fabs(q);
    if (aq > 1e-36 && aq < 1e36) {
        double r = (double)__frcp_rn((float)q);
        r = fma(r, fma(-q, r, 1.0), r);
        return fma(r, fma(-q, r, 1.0), r);
    }
    return 1.0 / q;
}

// 1/sqrt(x), x > 0, to a few ulp: the FP32 seed and two steps of y <- y (3/2 - x y^2 / 2)
__device__ inline double rsqrt_newton(double x) {
    if (x > 1e-36 && x < 1e36) {
        const double hx = 0.5 * x;
        double y = (double)__frsqrt_rn((float)x);
        y = y * fma(-hx * y, y, 1.5);
        return y * fma(-hx * y, y, 1.5);
    }
    return 1.0 / sqrt(x);
}

// Largest Dyson order (after deflation) reduced in one CTA's shared memory; larger
// matrices go to the cluster kernel.
constexpr int kTsMax = 160;

}  // namespace bd
