// k_sigma2.cu -- K0/K1: V' gather and 2p1h / 2h1p coupling build of the
// second-order self-energy, plus the static (extended Hartree-Fock) term.
//
// Restates Wide_self_energy_t::Build_Dynamic_SlfEn_2ndOrder
// (source/BcDor-Self_energy_ext_Op_c.cpp:323-561) and
// SpProp_t::ExtendedHartreeFock_Pot (source/BcDor-Sp_Propagator_a.cpp:39-130).
// Every floating-point operation uses an explicit round-to-nearest intrinsic in
// the reference's order, so no multiply-add is contracted and the rows are
// bit-identical to the reference's x86-64 build.
#include "bd_common.cuh"
#include "bd_kernels.h"
#include <algorithm>
#include <climits>

namespace bd {

// x == +0 or -0, by the bits (no FP64 instruction)
__device__ inline bool is_zero(double x) { return (__double_as_longlong(x) << 1) == 0; }

// x / d for 0 <= x < 2^21 and d >= 1 from one FP32 product: with rd = 1/d correctly
// rounded, (x + 1/2) rd is within 2^-2 / d of (x + 1/2) / d, whose fraction lies in
// [1/(2d), 1 - 1/(2d)], so truncation gives the quotient exactly (a few instructions
// instead of an integer division's twenty; checked exhaustively for d <= 64)
__device__ __forceinline__ int small_div(int x, float rd) { return __float2int_rz(__fmul_rn((float)x + 0.5f, rd)); }

__device__ inline int find_block(const long long *first, int nblk, long long g) {
    int lo = 0, hi = nblk - 1;
    while (lo < hi) {  // largest b with first[b] <= g
        int mid = (lo + hi + 1) >> 1;
        if (first[mid] <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// K0: V'[d][alpha][beta][gamma] = sqrt((2Jab+1)/(2j_I+1)) * V^Jab_{ab,dg} (* sqrt2 if g == d),
// source/BcDor-Self_energy_ext_Op_c.cpp:396-421.  One warp per 32 consecutive
// coefficients of a (Jab, ia, ib, ig) block (chunk w of the warp range; chunk_blk maps
// it to its block, chunk_first[b] is the block's first chunk), a lane per coefficient:
// every lookup of the launch is in flight at once.  The prefactor comes with the
// block: FP64 division and square root take tens of FP64 instructions, each a full
// warp slot on a pipe that issues at 1/64 of the FP32 rate.
__global__ void k_vgather(DevProblem P, const S2Block *blk, const int *chunk_blk, const int *chunk_first, int w0,
                          int nw, double *vp) {
    const int wl = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (wl >= nw) return;
    const int w = w0 + wl, b = chunk_blk[w];
    const S2Block B = blk[b];
    const int t = (w - chunk_first[b]) * 32 + lane;
    if (t >= B.nvp) return;
    const int I = B.ch;
    const int na = P.no[B.ia], nb = P.no[B.ib], ng = P.no[B.ig];
    int r = small_div(t, __frcp_rn((float)ng));
    const int ngs = t - r * ng;
    const int r2 = small_div(r, __frcp_rn((float)nb));
    const int nbs = r - r2 * nb;
    const int d = small_div(r2, __frcp_rn((float)na));
    const int nas = r2 - d * na;
    if (B.ia == B.ib && nbs < nas + B.nJab) return;
    int iid = P.orb_start[I] + d, iig = P.orb_start[B.ig] + ngs;
    if (iig == iid && B.nJgd) return;
    int iia = P.orb_start[B.ia] + nas, iib = P.orb_start[B.ib] + nbs;
    double v = __dmul_rn(B.x3, vget(P, iia, iib, iid, iig, B.Jab));   // IEEE division and sqrt: the host's bits
    if (iig == iid) v = __dmul_rn(v, kSqr2);
    vp[B.vp_first + t] = v;
}

// K1: one thread per pole.  dir 0 = 2p1h (forward), 1 = 2h1p (backward);
// source/BcDor-Self_energy_ext_Op_c.cpp:425-481 and :484-539.
__global__ void k_poles(DevProblem P, const S2Block *blk, const long long *pole_first, int nblk, long long g0,
                        long long total, const ChanSig *cs, int dir, const double *vp, double *E, double *S2,
                        double *M) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const long long g = g0 + idx;
    int b = find_block(pole_first, nblk, g);
    const S2Block B = blk[b];
    int t = (int)(g - pole_first[b]);
    const int I = B.ch, NS = P.nspb;
    const ChanSig C = cs[I];
    const int *nA = dir == 0 ? P.np : P.nh, *nGv = dir == 0 ? P.nh : P.np;
    const int *sA = dir == 0 ? P.p_start : P.h_start, *sG = dir == 0 ? P.h_start : P.p_start;
    const double *eA = dir == 0 ? P.ep : P.eh, *eG = dir == 0 ? P.eh : P.ep;
    const double *fA = dir == 0 ? P.fqp : P.fqh, *fG = dir == 0 ? P.fqh : P.fqp;
    const int nG = nGv[B.ig];
    const bool fdiv = t < (1 << 21);   // a block's poles: beyond 2^21, integer division
    int q = fdiv ? small_div(t, __frcp_rn((float)nG)) : t / nG;
    int na, nbf, ngf = t - q * nG;
    if (B.ia == B.ib) {
        const int nAa = nA[B.ia];
        na = 0;
        while (na < nAa && q >= nAa - na - B.nJab) { q -= nAa - na - B.nJab; ++na; }
        if (na >= nAa) return;  // index outside the block: leave the row untouched
        nbf = na + B.nJab + q;
    } else {
        const int nB = nA[B.ib];
        na = fdiv ? small_div(q, __frcp_rn((float)nB)) : q / nB;
        nbf = q - na * nB;
    }
    const double *fa = fA + (size_t)(sA[B.ia] + na) * NS;
    const double *fb = fA + (size_t)(sA[B.ib] + nbf) * NS;
    const double *fg = fG + (size_t)(sG[B.ig] + ngf) * NS;
    const double e = __dsub_rn(__dadd_rn(eA[sA[B.ia] + na], eA[sA[B.ib] + nbf]), eG[sG[B.ig] + ngf]);
    // (1 - 2 nJab) x as a sign flip and 1 / sqrt2 as the constant the IEEE division gives
    // (0x3FE6A09E667F3BCC): the same bits without their FP64 instructions
    const unsigned long long jflip = B.nJab ? 0x8000000000000000ull : 0ull;
    auto xj = [jflip](double x) { return __longlong_as_double((long long)((unsigned long long)__double_as_longlong(x) ^ jflip)); };
    const double x4 = (B.ia == B.ib && na == nbf) ? __longlong_as_double(0x3FE6A09E667F3BCCll) : 1.0;
    const int noa = P.no[B.ia], nob = P.no[B.ib], nog = P.no[B.ig], D = C.D;
    const int iid0 = P.orb_start[I], iig0 = P.orb_start[B.ig];
    const double *V = vp + B.vp_first;
    double s2 = 0.0;
    const int N = dir == 0 ? C.nfw : C.nbk;
    const long long k = g - (dir == 0 ? C.fw_off : C.bk_off);
    double *Mout = M + (dir == 0 ? C.mfw_off : C.mbk_off) + k;
    // The amplitude products x2(alpha, beta) do not depend on the orbital d: form the
    // non-zero ones once, in the reference's (alpha, beta) order, and reuse them for
    // every d.  A product with an exactly zero factor is an exact zero (skipped by the
    // reference's test below), so integer tests on the factors' bits spare its FP64
    // operations.  Each kept term is computed by the same operations as before.
    constexpr int kMaxTerms = 48;
    double x2v[kMaxTerms];
    int ab[kMaxTerms];
    int nterm = 0;
    bool listed = true;
    for (int nas = 0; nas < noa && listed; ++nas) {
        const int nst2 = (B.ia == B.ib) ? nas + B.nJab : 0;
        for (int nbs = nst2; nbs < nob; ++nbs) {
            const bool z1 = is_zero(fa[nas]) || is_zero(fb[nbs]);
            const bool z2 = (B.ia != B.ib) || is_zero(fa[nbs]) || is_zero(fb[nas]);
            if (z1 && z2) continue;
            double x2 = __dmul_rn(fa[nas], fb[nbs]);
            if (B.ia == B.ib) {
                x2 = __dadd_rn(x2, __dmul_rn(xj(fa[nbs]), fb[nas]));
                if (nas == nbs) x2 = __ddiv_rn(x2, kSqr2);
            }
            if (x2 == 0.0) continue;
            if (nterm == kMaxTerms) { listed = false; break; }
            x2v[nterm] = x2;
            ab[nterm] = nas * nob + nbs;
            ++nterm;
        }
    }
    if (listed) {
        for (int nd = 0; nd < D; ++nd) {
            double x1 = 0.0;
            const int iid = iid0 + nd;
            for (int q = 0; q < nterm; ++q) {
                const double x2 = x2v[q];
                const double *Vr = V + ((size_t)nd * noa * nob + ab[q]) * nog;
                for (int ngs = 0; ngs < nog; ++ngs) {
                    if (iig0 + ngs == iid && B.nJgd) continue;
                    if (is_zero(fg[ngs])) continue;
                    x1 = __dadd_rn(x1, __dmul_rn(__dmul_rn(Vr[ngs], x2), fg[ngs]));
                }
            }
            x1 = __dmul_rn(x1, x4);
            Mout[(size_t)nd * N] = x1;
            s2 = __dadd_rn(s2, __dmul_rn(x1, x1));
        }
        E[g] = e;
        S2[g] = s2;
        return;
    }
    for (int nd = 0; nd < D; ++nd) {
        double x1 = 0.0;
        const int iid = iid0 + nd;
        for (int nas = 0; nas < noa; ++nas) {
            const int nst2 = (B.ia == B.ib) ? nas + B.nJab : 0;
            for (int nbs = nst2; nbs < nob; ++nbs) {
                double x2 = __dmul_rn(fa[nas], fb[nbs]);
                if (B.ia == B.ib) {
                    x2 = __dadd_rn(x2, __dmul_rn(xj(fa[nbs]), fb[nas]));
                    if (nas == nbs) x2 = __ddiv_rn(x2, kSqr2);
                }
                // Terms with a zero amplitude factor add an exact zero to x1, which starts
                // at +0 and so is never -0: skipping them changes no bit of the sum (with the
                // one-hot amplitudes of an unperturbed propagator, all but one term go).
                if (x2 == 0.0) continue;
                const double *Vr = V + (((size_t)nd * noa + nas) * nob + nbs) * nog;
                for (int ngs = 0; ngs < nog; ++ngs) {
                    if (iig0 + ngs == iid && B.nJgd) continue;
                    if (is_zero(fg[ngs])) continue;
                    x1 = __dadd_rn(x1, __dmul_rn(__dmul_rn(Vr[ngs], x2), fg[ngs]));
                }
            }
        }
        x1 = __dmul_rn(x1, x4);
        Mout[(size_t)nd * N] = x1;
        s2 = __dadd_rn(s2, __dmul_rn(x1, x1));
    }
    E[g] = e;
    S2[g] = s2;
}

// Static self-energy, per (channel I, nr >= nc) entry:
//   U = sum_c x1(c) x7(c),   x7(c) = sum_{nm, nv} (x2 x3) x6(nm, nv) V(...)
// over the (iv, J2) combinations c of channel I (their list and the offset of each
// one's no[iv]^2 terms inside an entry come from the host, ctab_*).  The terms are
// independent of one another: k_ehf_terms forms every term of every entry, a thread
// each, so all interaction lookups are in flight together; k_ehf_sum, a CTA per entry,
// adds each c's terms in the reference's (nm, nv) order and thread 0 adds the c
// partials in the reference's (iv, J2) order: every sum keeps the reference's
// sequence of roundings.
__device__ inline bool ehf_skip(int iv, int I, int nm, int nv, int nr, int nc, int nJ) {
    return iv == I && nJ != 1 && (nm == nr || nv == nc);
}

__global__ void k_ehf_terms(DevProblem P, const int3 *entries, const long long *term_first, int e0, int e1,
                            const int *ctab_cmb, const int *ctab_toff, const int *ctab_off, const int *ncomb,
                            double *terms) {
    const long long g = term_first[e0] + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= term_first[e1]) return;
    int lo = e0, hi = e1 - 1;   // the entry of term g
    while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (term_first[mid] <= g) lo = mid; else hi = mid - 1; }
    const int I = entries[lo].x, nr = entries[lo].y, nc = entries[lo].z;
    const int u = (int)(g - term_first[lo]);
    const int *toff = ctab_toff + ctab_off[I];
    int cl = 0, ch = ncomb[I] - 1;   // the combination of term u
    while (cl < ch) { const int mid = (cl + ch + 1) >> 1; if (toff[mid] <= u) cl = mid; else ch = mid - 1; }
    const int cm = ctab_cmb[ctab_off[I] + cl], iv = cm & 0xffff, J2 = cm >> 16, no = P.no[iv];
    const int r = u - toff[cl], nm = r / no, nv = r - nm * no;
    const int j2I = P.j2[I], NS = P.nspb;
    const int nJ = ((j2I + P.j2[iv] + J2) / 2) % 2;
    if (ehf_skip(iv, I, nm, nv, nr, nc, nJ)) return;
    const double x2 = (iv == I && nm == nr) ? kSqr2 : 1.0;
    const double x3 = (iv == I && nv == nc) ? kSqr2 : 1.0;
    const int ia = P.orb_start[I] + nr, im = P.orb_start[iv] + nm;
    const int ib = P.orb_start[I] + nc, iu = P.orb_start[iv] + nv;
    double x6 = 0.0;
    const double *q = P.fqh + (size_t)P.h_start[iv] * NS;
    for (int kg = 0; kg < P.nh[iv]; ++kg) { x6 = __dadd_rn(x6, __dmul_rn(q[nv], q[nm])); q += NS; }
    terms[g] = __dmul_rn(__dmul_rn(__dmul_rn(x2, x3), x6), vget(P, ia, im, ib, iu, J2 / 2));
}

constexpr int kEhfThreads = 256, kEhfComb = 2048;

__global__ void __launch_bounds__(kEhfThreads) k_ehf_sum(DevProblem P, const int3 *entries, const long long *term_first,
                                                         int e0, const int *ctab_cmb, const int *ctab_toff,
                                                         const int *ctab_off, const int *ncomb, const double *terms,
                                                         const long long *out_off, double *out) {
    __shared__ double part[kEhfComb];
    const int e = e0 + blockIdx.x;
    const int I = entries[e].x, nr = entries[e].y, nc = entries[e].z;
    const int D = P.no[I], j2I = P.j2[I], nco = ncomb[I];
    if (nco > kEhfComb) return;
    const int *cmb = ctab_cmb + ctab_off[I], *toff = ctab_toff + ctab_off[I];
    const double *t0 = terms + term_first[e];
    for (int c = threadIdx.x; c < nco; c += kEhfThreads) {
        const int iv = cmb[c] & 0xffff, J2 = cmb[c] >> 16, no = P.no[iv];
        const int nJ = ((j2I + P.j2[iv] + J2) / 2) % 2;
        const double x1 = __ddiv_rn((double)(J2 + 1), (double)(j2I + 1));
        double x7 = 0.0;
        const double *t = t0 + toff[c];
        for (int nm = 0; nm < no; ++nm)
            for (int nv = 0; nv < no; ++nv)
                if (!ehf_skip(iv, I, nm, nv, nr, nc, nJ)) x7 = __dadd_rn(x7, t[nm * no + nv]);
        part[c] = __dmul_rn(x1, x7);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double u = 0.0;
        for (int c = 0; c < nco; ++c) u = __dadd_rn(u, part[c]);
        double *U = out + out_off[I];
        U[nr * D + nc] = u;
        U[nc * D + nr] = u;
    }
}

// Segment table of the sorted interaction (prepare_for_reading,
// source/BcDor-Vpp_potential.cpp:478-496): element i opens the segment of its
// (charge sum, parity, J) key when the previous element's key differs and closes it
// when the next one's differs.  A key opened twice means the list is not sorted by
// key; an element with an orbit out of range or a key off the table is reported by
// the smallest such index (bad[0]) and its reason (bad[1]: 1 orbit, 2 key).
__device__ inline int interaction_key(int k, int norb, const int *orb_sh, const int *ch, const int *ip, int *why) {
    const int J = k % kJMult, ab = k / kJMult, a = ab / kABMult, b = ab % kABMult;
    if (k < 0 || a < 0 || b < 0 || a >= norb || b >= norb) { *why = 1; return -1; }
    const int key = ind_chipJ(ch[orb_sh[a]] + ch[orb_sh[b]], (ip[orb_sh[a]] + ip[orb_sh[b]]) % 2, J);
    if (key < 0 || key >= kSegTable) { *why = 2; return -1; }
    return key;
}

//
// The same pass fills the row table (DevProblem::rows) when rows is non-null: each run
// of equal iabJ records its first and last element.  bad[2] is set when the table
// cannot stand in for the reference's search: a pair out of order or repeated inside
// a segment, a run that appears twice, or a J beyond the table.
__global__ void k_segments(const int *iabJ, const int *icdJ, int n, int norb, const int *orb_sh, const int *ch,
                           const int *ip, int *seg_str, int *seg_end, int *seg_cnt, int *bad, int2 *rows, int nJ) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int why = 0, w2 = 0;
    const int iab = iabJ[i];
    const int key = interaction_key(iab, norb, orb_sh, ch, ip, &why);
    if (key < 0) {
        if (atomicMin(&bad[0], i) > i) atomicExch(&bad[1], why);
        return;
    }
    const int prev = i > 0 ? interaction_key(iabJ[i - 1], norb, orb_sh, ch, ip, &w2) : -1;
    const int next = i + 1 < n ? interaction_key(iabJ[i + 1], norb, orb_sh, ch, ip, &w2) : -1;
    if (key != prev) { seg_str[key] = i; atomicAdd(&seg_cnt[key], 1); }
    if (key != next) seg_end[key] = i;
    if (!rows) return;
    if (key == prev) {
        const int pa = iabJ[i - 1], pc = icdJ[i - 1], c = icdJ[i];
        if (!(pa < iab || (pa == iab && pc < c))) bad[2] = 1;
    }
    const int J = iab % kJMult, a = iab / (kJMult * kABMult), b = (iab / kJMult) % kABMult;
    if (J >= nJ) { bad[2] = 1; return; }
    int2 *rw = rows + ((size_t)a * norb + b) * nJ + J;
    if (i == 0 || iabJ[i - 1] != iab)
        if (atomicCAS(&rw->x, -1, i) != -1) bad[2] = 1;
    if (i + 1 == n || iabJ[i + 1] != iab) rw->y = i;
}

// Pair ranks (DevProblem::prank): each element of the first row of its segment
// records its position in the segment under its pair index icdJ.
__global__ void k_pair_rank(const int *iabJ, const int *icdJ, int n, int norb, const int *orb_sh, const int *ch,
                            const int *ip, const int *seg_str, int nJ, int *prank) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int why = 0;
    const int key = interaction_key(iabJ[i], norb, orb_sh, ch, ip, &why);
    if (key < 0) return;
    const int s0 = seg_str[key];
    if (s0 < 0 || iabJ[i] != iabJ[s0]) return;   // not in the segment's first row
    const int icd = icdJ[i];
    const int J = icd % kJMult, c = icd / (kJMult * kABMult), d = (icd / kJMult) % kABMult;
    if (J >= nJ || c >= norb || d >= norb || c < 0 || d < 0) return;
    prank[((size_t)c * norb + d) * nJ + J] = i - s0;
}

// Stable sort of each channel's poles by energy (ascending, or descending with desc),
// for channels of at most kSortMax poles, in two kernels over chunks of kSortChunk
// consecutive poles of one channel (the chunk table lists, per chunk, its first pole
// and length and its channel's first pole and length, relative to the range):
//   k_chunk_sort   one CTA per chunk sorts (key, index) pairs with a bitonic network
//                  in shared memory, the key the order-preserving integer image of the
//                  double (sign bit set: all bits flipped, else the sign bit set; the
//                  radix sort's mapping, -0 before +0), complemented for descending
//                  order, the index (the pole's global index) breaking ties;
//   k_chunk_place  one thread per pole: its rank in the channel is the number of
//                  pairs below its own in every chunk of the channel (binary searches
//                  in the sorted chunks), so perm[rank] = its global index.
// (key, index) pairs are distinct, so the order is the stable sort's.
__device__ inline unsigned long long sort_key(double e, bool desc) {
    unsigned long long u = (unsigned long long)__double_as_longlong(e);
    u = (u >> 63) ? ~u : (u | (1ull << 63));
    return desc ? ~u : u;
}

__global__ void __launch_bounds__(kSortThreads) k_chunk_sort(const double *E, const int4 *chunks, bool desc,
                                                             long long base, unsigned long long *tk, int *ti) {
    const int4 ch = chunks[blockIdx.x];   // first pole, length, channel's first pole, channel's length
    __shared__ unsigned long long skey[kSortChunk];
    __shared__ int sidx[kSortChunk];
    const int n = ch.y;
    int P = 32;
    while (P < n) P <<= 1;
    for (int t = threadIdx.x; t < P; t += kSortThreads) {
        unsigned long long k = ~0ull;
        int ix = INT_MAX;
        if (t < n) { k = sort_key(E[ch.x + t], desc); ix = (int)(base + ch.x + t); }
        skey[t] = k;
        sidx[t] = ix;
    }
    __syncthreads();
    for (int kk = 2; kk <= P; kk <<= 1)
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int t = threadIdx.x; t < P; t += kSortThreads) {
                const int u = t ^ j;
                if (u <= t) continue;
                const unsigned long long ka = skey[t], kb = skey[u];
                const int ia = sidx[t], ib = sidx[u];
                const bool gt = (ka > kb) || (ka == kb && ia > ib);
                if (((t & kk) == 0) ? gt : !gt) { skey[t] = kb; skey[u] = ka; sidx[t] = ib; sidx[u] = ia; }
            }
            __syncthreads();
        }
    for (int t = threadIdx.x; t < n; t += kSortThreads) { tk[ch.x + t] = skey[t]; ti[ch.x + t] = sidx[t]; }
}

__global__ void k_chunk_place(const unsigned long long *tk, const int *ti, const int4 *chunks, int nchunks,
                              long long n, long long base, int *perm) {
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= n) return;
    int lo = 0, hi = nchunks - 1;   // the chunk holding g
    while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (chunks[mid].x <= g) lo = mid; else hi = mid - 1; }
    const int4 me = chunks[lo];
    const unsigned long long key = tk[g];
    const int idx = ti[g];
    int rank = (int)(g - me.x);   // pairs below it in its own chunk
    // the channel's other chunks (a channel's chunks are consecutive in the table)
    int c0 = lo, c1 = lo;
    while (c0 > 0 && chunks[c0 - 1].z == me.z) --c0;
    while (c1 + 1 < nchunks && chunks[c1 + 1].z == me.z) ++c1;
    for (int c = c0; c <= c1; ++c) {
        if (c == lo) continue;
        const int4 o = chunks[c];
        int a = 0, b = o.y;   // first pair of chunk c not below (key, idx)
        while (a < b) {
            const int mid = (a + b) >> 1;
            const unsigned long long km = tk[o.x + mid];
            const bool below = km < key || (km == key && ti[o.x + mid] < idx);
            if (below) a = mid + 1; else b = mid;
        }
        rank += a;
    }
    perm[me.z + rank] = idx;
}

// Channel of every pole (offsets off[0..ns], off[ns] = n) and the identity order.
__global__ void k_pole_index(const int *off, int ns, long long n, int *seg, int *idx) {
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= n) return;
    int lo = 0, hi = ns - 1;   // last channel whose offset is <= g
    while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (off[mid] <= g) lo = mid; else hi = mid - 1; }
    seg[g] = lo;
    idx[g] = (int)g;
}

// Gather rows in a given order into separate SoA arrays (used after the sort), plus an
// FP32 copy of the couplings for the FP32-vector Lanczos form.
__global__ void k_permute_soa(const int *perm, long long n0, long long n, const int *seg_of, const ChanSig *cs, int dir,
                              const double *Ein, const double *Min, double *Eout, double *Mout, float *Mfout) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= n) return;
    const long long g = n0 + idx;
    const int ch = seg_of[g];
    const ChanSig C = cs[ch];
    const long long off = dir == 0 ? C.fw_off : C.bk_off;
    const long long moff = dir == 0 ? C.mfw_off : C.mbk_off;
    const int N = dir == 0 ? C.nfw : C.nbk;
    const long long k = g - off;
    const long long src = perm[g];  // global source index (same segment)
    Eout[g] = Ein[src];
    for (int d = 0; d < C.D; ++d) {
        const double m = Min[moff + (long long)d * N + (src - off)];
        Mout[moff + (long long)d * N + k] = m;
        Mfout[moff + (long long)d * N + k] = (float)m;
    }
}

// AoS rows [E, S2, M_0..] of one channel, for host copies in the reference layout.
__global__ void k_rows_aos(const double *E, const double *S2, const double *M, int N, int D, double *rows) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    double *r = rows + (size_t)k * (2 + D);
    r[0] = E[k]; r[1] = S2[k];
    for (int d = 0; d < D; ++d) r[2 + d] = M[(size_t)d * N + k];
}

// The same rows in the order of a sort: row k is pole perm[off + k] (a global index of
// the channel, whose first pole is off; E, S2 and M are the channel's unsorted arrays).
__global__ void k_rows_aos_perm(const int *perm, long long off, const double *E, const double *S2, const double *M,
                                int N, int D, double *rows) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    long long src = (long long)perm[off + k] - off;
    if (src < 0 || src >= N) src = k;   // a permutation of the channel by construction
    double *r = rows + (size_t)k * (2 + D);
    r[0] = E[src]; r[1] = S2[src];
    for (int d = 0; d < D; ++d) r[2 + d] = M[(size_t)d * N + src];
}

// The reference's order of equal energies.  Sort_u_double2dim / Sort_d_double2dim
// (source/BcDor-Utilities.cpp:25-94) are heap sorts, so rows of equal energy end in
// the order the heap's moves leave them, not in their input order.  k_heap_order
// runs that heap sort again on every channel's poles, one CTA per channel, starting
// from the stable order a previous sort left in perm (perm[off + r] = global index of
// the pole of rank r; off[b] .. off[b + 1] is channel b's range relative to n0):
//   * each pole gets the dense rank of its energy, from the runs of equal energies in
//     the stable order.  The heap sort compares nothing but energies, so ranks give it
//     the same moves (-0 and +0 compare equal, as doubles do).  Rank and position in
//     the channel are packed into one 32-bit word, rank << 16 | position, in shared
//     memory (position p at word p + 1, so a node's two children are one 8-byte load);
//   * the heap is built level by level: the reference sifts nodes n/2 - 1 .. 0 in turn,
//     and the nodes of one depth own disjoint subtrees, so they sift at once, the
//     deepest level first;
//   * the n - 1 extractions are one serial chain, each sift done by a warp five heap
//     levels at a time (heap_sift_root_warp);
//   * perm receives the result.  Sort_d's descending heap sort is Sort_u's on the
//     ranks of the descending stable order, so one routine serves both.
// A channel without equal energies keeps the stable order, which is then the heap
// sort's; channels of more than kHeapMax poles keep the stable order.
__device__ __forceinline__ void heap_sift(unsigned *a, int i, unsigned tmp, int ir) {
    const unsigned kt = tmp >> 16;
    int j = 2 * i + 1;
    while (j <= ir) {
        unsigned cj = a[j];
        if (j < ir) {
            const unsigned cj1 = a[j + 1];
            if ((cj >> 16) < (cj1 >> 16)) { ++j; cj = cj1; }
        }
        if (kt < (cj >> 16)) { a[i] = cj; i = j; j = 2 * j + 1; }
        else break;
    }
    a[i] = tmp;
}

// One extraction's sift from the root, by a whole warp, five levels per round: lane l
// holds node r = l + 1 of the five-level subtree below the hole v (r's global index
// g(r) = (v + 1) 2^t + r - 2^t - 1 at relative depth t) and loads its two children in
// one 8-byte load; ballots give, for every such node, whether it has children and
// whether the right one is the larger (the reference's tie rule: right only if
// strictly larger).  Every lane then follows the path of larger children through the
// ballot bits (no memory), the lanes on the path test tmp against their chosen child,
// and the first that does not exceed tmp is where the sift stops: the parents above it
// take their chosen child, the stop (or the node without children the path reached)
// takes tmp.  Otherwise the hole moves five levels down and the next round starts.
__device__ __forceinline__ void heap_sift_root_warp(unsigned *hs, unsigned tmp, int ir, int lane) {
    unsigned *a = hs + 1;
    const unsigned kt = tmp >> 16;
    const int r = lane + 1;
    const int t = 31 - __clz(r);
    int v = 0;
    for (;;) {
        const int gr = ((v + 1) << t) + (r - (1 << t)) - 1;
        const int c0 = 2 * gr + 1;
        const bool ok = lane < 31 && c0 <= ir;
        uint2 w = make_uint2(0u, 0u);
        if (ok) w = *reinterpret_cast<const uint2 *>(hs + c0 + 1);
        const bool right = ok && c0 + 1 <= ir && (w.x >> 16) < (w.y >> 16);
        const unsigned big = right ? w.y : w.x;
        const unsigned mh = __ballot_sync(0xffffffffu, ok), mr = __ballot_sync(0xffffffffu, right);
        unsigned pm = 0u;
        int rr = 1, depth = 0;
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            if (!((mh >> (rr - 1)) & 1u)) break;
            pm |= 1u << (rr - 1);
            rr = 2 * rr + (int)((mr >> (rr - 1)) & 1u);
            ++depth;
        }
        const unsigned ms = __ballot_sync(0xffffffffu, ((pm >> lane) & 1u) && !(kt < (big >> 16)));
        const unsigned mv = ms ? (pm & ((ms & (0u - ms)) - 1u)) : pm;
        if ((mv >> lane) & 1u) a[gr] = big;
        __syncwarp();
        if (ms || depth < 5) {
            const int hr = ms ? __ffs(ms) : rr;
            const int th = 31 - __clz(hr);
            if (lane == 0) a[((v + 1) << th) + (hr - (1 << th)) - 1] = tmp;
            __syncwarp();
            return;
        }
        v = ((v + 1) << 5) + (rr - 32) - 1;
    }
}

constexpr int kHeapThreads = 1024;
static_assert(kHeapMax < 65536, "positions are packed into 16 bits");
__global__ void __launch_bounds__(kHeapThreads) k_heap_order(const double *E, const int *off, long long n0, int *perm) {
    const int s0 = off[blockIdx.x], n = off[blockIdx.x + 1] - s0;
    if (n < 2 || n > kHeapMax) return;
    extern __shared__ __align__(16) unsigned hs[];   // position p at hs[p + 1]
    unsigned *a = hs + 1;
    __shared__ int wsum[kHeapThreads / 32];
    int *pm = perm + n0 + s0;
    const long long gbase = n0 + s0;   // global index of the channel's first pole
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    // 1. dense ranks along the stable order; thread t takes positions [p0, p1)
    const int c = (n + kHeapThreads - 1) / kHeapThreads;
    const int p0 = min(n, tid * c), p1 = min(n, p0 + c);
    int cnt = 0;
    {
        double pv = (p0 > 0 && p0 < n) ? E[pm[p0 - 1]] : 0.0;
        for (int p = p0; p < p1; ++p) {
            const double e = E[pm[p]];
            cnt += (p == 0 || e != pv);
            pv = e;
        }
    }
    int x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int v = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        wsum[lane] = v;
    }
    __syncthreads();
    const int ndist = wsum[kHeapThreads / 32 - 1];
    if (ndist == n) return;   // no equal energies: the stable order is the heap sort's
    {
        int run = x - cnt + (wid > 0 ? wsum[wid - 1] : 0);   // rank runs before p0
        double pv = (p0 > 0 && p0 < n) ? E[pm[p0 - 1]] : 0.0;
        for (int p = p0; p < p1; ++p) {
            const int g = pm[p];
            const double e = E[g];
            run += (p == 0 || e != pv);
            pv = e;
            const long long loc = (long long)g - gbase;
            if (loc >= 0 && loc < n) a[loc] = ((unsigned)(run - 1) << 16) | (unsigned)loc;
        }
    }
    __syncthreads();
    // 2. the heap: nodes n/2 - 1 .. 0 sifted over [0, n - 1], one depth at a time
    const int lastl = n / 2 - 1;
    for (int d = 31 - __clz(lastl + 1); d >= 0; --d) {
        const int lo = (1 << d) - 1, hi = min((2 << d) - 2, lastl);
        for (int l = lo + tid; l <= hi; l += kHeapThreads) heap_sift(a, l, a[l], n - 1);
        __syncthreads();
    }
    // 3. extractions by warp 0: the largest to the end of the shrinking heap, the last
    //    node sifted from the root
    if (wid == 0) {
        for (int ir = n - 1; ir > 0;) {
            const unsigned tmp = a[ir];
            __syncwarp();
            if (lane == 0) a[ir] = a[0];
            --ir;
            __syncwarp();
            if (ir == 0) {
                if (lane == 0) a[0] = tmp;
                break;
            }
            heap_sift_root_warp(hs, tmp, ir, lane);
        }
    }
    __syncthreads();
    for (int p = tid; p < n; p += kHeapThreads) {
        int loc = (int)(a[p] & 0xffffu);
        if (loc >= n) loc = p;   // a permutation of the channel by construction
        pm[p] = (int)(gbase + loc);
    }
}

// Channels longer than kSortMax poles: a stable radix sort of the range by the energies'
// integer images (k_sort.cu), then a stable one by channel, so each channel's poles end
// in energy order and equal energies keep their build order.
__global__ void k_pole_keys(const double *E, long long n0, long long n, bool desc, unsigned long long *key,
                            unsigned *val) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    key[i] = sort_key(E[n0 + i], desc);
    val[i] = (unsigned)(n0 + i);
}
__global__ void k_pole_chan(const unsigned *val, const int *seg_of, int ch_lo, long long n, unsigned long long *key) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    key[i] = (unsigned long long)(seg_of[val[i]] - ch_lo);
}
__global__ void k_perm_out(const unsigned *val, long long n0, long long n, int *perm) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    perm[n0 + i] = (int)val[i];
}

cudaError_t launch_pole_radix(const double *E, const int *seg_of, int ch_lo, int nseg, long long n0, long long n,
                              bool desc, unsigned long long *k0, unsigned *v0, unsigned long long *k1, unsigned *v1,
                              void *scratch, int *perm, int *launches, cudaStream_t st) {
    const unsigned nb = (unsigned)((n + 255) / 256);
    k_pole_keys<<<nb, 256, 0, st>>>(E, n0, n, desc, k0, v0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int p1 = 0, p2 = 0;
    if ((e = radix_sort_pairs(k0, v0, k1, v1, n, 0, 64, false, scratch, &p1, st)) != cudaSuccess) return e;
    k_pole_chan<<<nb, 256, 0, st>>>(v0, seg_of, ch_lo, n, k0);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int cbits = nseg <= 256 ? 8 : 16;
    if ((e = radix_sort_pairs(k0, v0, k1, v1, n, 0, cbits, false, scratch, &p2, st)) != cudaSuccess) return e;
    k_perm_out<<<nb, 256, 0, st>>>(v0, n0, n, perm);
    if (launches) *launches += 3 + radix_launches(p1, false) + radix_launches(p2, false);
    return cudaGetLastError();
}

// The next iteration's propagator on the device (bd_dressed_propagator): one warp per
// (subshell, side) picks, of that channel's Dyson solutions (rows [W, Z, x..]: the
// quasiparticles, then the quasiholes, each by descending W), those with Z >= z_cut, at
// most max_frag of them (max_frag <= 0: all) by largest Z, ties to the earlier row, and
// lists them in row order: cnt[2 I + side], sel[(2 I + side) * cap + r].
__global__ void k_dressed_select(const double *sol, const long long *sol_off, const int *nq, const int *D_of, int ns,
                                 double z_cut, int max_frag, int cap, int *cnt, int *sel) {
    const int wg = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (wg >= 2 * ns) return;
    const int I = wg >> 1, side = wg & 1, NS = 2 + D_of[I];
    const int n = nq[2 * I + side];
    const double *rows = sol + sol_off[I] + (side ? (size_t)nq[2 * I] * NS : 0);
    int *out = sel + (size_t)wg * cap;
    int m = 0;   // candidates
    for (int b = 0; b < n; b += 32) {
        const int k = b + lane;
        const bool c = k < n && rows[(size_t)k * NS + 1] >= z_cut;
        const unsigned bal = __ballot_sync(0xffffffffu, c);
        if (max_frag <= 0 && c) {
            const int r = m + __popc(bal & ((1u << lane) - 1u));
            if (r < cap) out[r] = k;
        }
        m += __popc(bal);
    }
    if (max_frag <= 0 || m <= max_frag) {
        if (max_frag > 0)   // every candidate, in row order
            for (int b = 0, r = 0; b < n; b += 32) {
                const int k = b + lane;
                const bool c = k < n && rows[(size_t)k * NS + 1] >= z_cut;
                const unsigned bal = __ballot_sync(0xffffffffu, c);
                if (c && r + __popc(bal & ((1u << lane) - 1u)) < cap) out[r + __popc(bal & ((1u << lane) - 1u))] = k;
                r += __popc(bal);
            }
        if (lane == 0) cnt[wg] = m;
        return;
    }
    // the max_frag largest Z (ties: the earlier row), one warp argmax at a time
    int taken[32];
    for (int t = 0; t < max_frag && t < 32; ++t) {
        double bz = -1.0;
        int bk = INT_MAX;
        for (int k = lane; k < n; k += 32) {
            const double z = rows[(size_t)k * NS + 1];
            bool used = false;
            for (int u = 0; u < t; ++u) used |= (taken[u] == k);
            if (!used && z >= z_cut && (z > bz || (z == bz && k < bk))) { bz = z; bk = k; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double oz = __shfl_xor_sync(0xffffffffu, bz, o);
            const int ok = __shfl_xor_sync(0xffffffffu, bk, o);
            if (oz > bz || (oz == bz && ok < bk)) { bz = oz; bk = ok; }
        }
        taken[t] = bk;
    }
    if (lane == 0) {
        const int k = max_frag < 32 ? max_frag : 32;
        for (int a = 1; a < k; ++a)   // back to row order (descending W, as add_qp / add_qh store them)
            for (int b = a; b > 0 && taken[b - 1] > taken[b]; --b) { const int t = taken[b]; taken[b] = taken[b - 1]; taken[b - 1] = t; }
        for (int r = 0; r < k && r < cap; ++r) out[r] = taken[r];
        cnt[wg] = k;
    }
}

// The selected solutions written over the propagator in place (the fragment counts are
// the current ones): energies, amplitudes x_0..x_{D-1}, zeros up to nspb.
__global__ void k_dressed_write(const double *sol, const long long *sol_off, const int *nq, const int *D_of,
                                const int *p_start, const int *h_start, int ns, int nspb, int cap, const int *cnt,
                                const int *sel, double *ep, double *eh, double *fqp, double *fqh) {
    const int wg = blockIdx.x;   // (subshell, side)
    if (wg >= 2 * ns) return;
    const int I = wg >> 1, side = wg & 1, D = D_of[I], NS = 2 + D;
    const double *rows = sol + sol_off[I] + (side ? (size_t)nq[2 * I] * NS : 0);
    const int m = cnt[wg];
    const int base = side ? h_start[I] : p_start[I];
    double *E = side ? eh : ep;
    double *F = side ? fqh : fqp;
    for (int t = threadIdx.x; t < m * nspb; t += blockDim.x) {
        const int r = t / nspb, q = t - r * nspb;
        const double *row = rows + (size_t)sel[(size_t)wg * cap + r] * NS;
        F[(size_t)(base + r) * nspb + q] = q < D ? row[2 + q] : 0.0;
        if (q == 0) E[base + r] = row[0];
    }
}

// Finiteness of n doubles: bad receives 1 + the index of a non-finite one (any, when
// there are several), and stays as it was when all are finite.
__global__ void k_nonfinite(const double *x, long long n, int *bad) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long u = (unsigned long long)__double_as_longlong(x[i]);
        if (((u >> 52) & 0x7ff) == 0x7ff) atomicMax(bad, (int)min(i + 1, (long long)INT_MAX));
    }
}

cudaError_t launch_nonfinite(const double *x, long long n, int *bad, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const long long blocks = std::min<long long>((n + 255) / 256, 152 * 8);
    k_nonfinite<<<(unsigned)blocks, 256, 0, st>>>(x, n, bad);
    return cudaGetLastError();
}

cudaError_t launch_heap_order(const double *E, const int *d_off, int nseg, int max_len, long long n0, int *perm,
                              cudaStream_t st) {
    if (nseg <= 0 || max_len < 2) return cudaSuccess;
    const size_t smem = sizeof(unsigned) * (size_t)(std::min(max_len, kHeapMax) + 4);
    cudaError_t e = allow_dynamic_smem((const void *)k_heap_order);
    if (e != cudaSuccess) return e;
    k_heap_order<<<nseg, kHeapThreads, smem, st>>>(E, d_off, n0, perm);
    return cudaGetLastError();
}

void sigma2_smem_init() { allow_dynamic_smem((const void *)k_heap_order); }

}  // namespace bd
