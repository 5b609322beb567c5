// k_coupling_tc.cu -- the 2p1h / 2h1p couplings M of the second-order self-energy on
// the tensor cores, for the mixed-precision form on a dressed propagator.
//
// Restates the contraction of Build_Dynamic_SlfEn_2ndOrder
// (source/BcDor-Self_energy_ext_Op_c.cpp:425-481 forward, :484-539 backward), which
// k_poles (k_sigma2.cu) keeps in the reference's FP64 order for the plain form.  For a
// block (I, Jab, ia, ib, ig) and a pole t = (na, nb, ng) of fragments,
//   M[d][t] = x4(t) sum_{p = (alpha, beta), gamma} V'[d][p][gamma] x2(p; na, nb) f_ng[gamma],
// a GEMM of the block's V' (rows d, columns (p, gamma)) with the matrix
// B[(p, gamma)][t] = x4(t) x2(p; t) f_ng[gamma].  B depends on (ia, ib, ig, nJab) and the
// propagator only, so the blocks of every channel that share those are stacked into one
// operand of 128 rows (their D rows each): one tile is one 128 x N x K product, N the
// block's poles padded to 16, K = pairs x orbitals of ig.
//
// Each tile: a CTA of four warps stages A (V') and B in shared memory in the canonical
// no-swizzle K-major layout (8-row x 16-byte core matrices), 64 K columns at a time; every
// value is split into two TF32 parts, hi + lo, and thread 0 issues three tcgen05.mma
// (kind::tf32, M = 128) per 8 columns, hi*hi + hi*lo + lo*hi, accumulating in FP32 in
// tensor memory (about 2^-21 relative per product, against the FP32 Lanczos vectors'
// 2^-24 rounding); their completion comes back through an mbarrier (tcgen05.commit).
// Then each warp reads its 32 rows from tensor memory (tcgen05.ld) and writes M, and the
// CTA forms the poles' energies (FP64, the reference's operations: the same bits as
// k_poles) and S2 = sum_d M^2.  Every FP64 -> FP32 conversion of the staging is done on
// the integer pipe (the double's bits truncated): the FP64 unit issues at 1/64 of FP32.
#include "bd_common.cuh"
#include "bd_kernels.h"

namespace bd {

namespace {

constexpr int kTcRows = 128;     // MMA M: rows of a tile
constexpr int kTcKc = 64;        // K columns staged per round
constexpr int kTcThreads = 128;  // four warps: one per 32 lanes of tensor memory
constexpr int kTcPairs = 64;     // (alpha, beta) pairs of a block at most (orbitals <= 8)

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of tcgen05: start address, leading (K direction) and
// stride (8-row groups) byte offsets, all in 16-byte units; version 1, no swizzle.
__device__ __forceinline__ uint64_t mma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Element (r, k) of a K-major tile of kTcKc columns: [r / 8][k / 4][r % 8][k % 4] (floats).
__device__ __forceinline__ int tc_off(int r, int k) { return (((r >> 3) * (kTcKc / 4) + (k >> 2)) * 8 + (r & 7)) * 4 + (k & 3); }

// x truncated to FP32 from its bits (|x| inside the FP32 normal range, else 0 or the
// largest float): no FP64 instruction
__device__ __forceinline__ float f64_to_f32(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
    const unsigned s = (unsigned)(b >> 63) << 31;
    if (e <= 0) return __uint_as_float(s);
    if (e >= 255) return __uint_as_float(s | 0x7F7FFFFFu);
    return __uint_as_float(s | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7FFFFFu));
}

// FP32 to FP64 from the bits (exact; zero and normal values)
__device__ __forceinline__ double f32_to_f64(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned e = (u >> 23) & 0xFF;
    if (e == 0) return __longlong_as_double((long long)((unsigned long long)(u >> 31) << 63));
    return __longlong_as_double((long long)(((unsigned long long)(u >> 31) << 63) |
                                            ((unsigned long long)(e - 127 + 1023) << 52) |
                                            ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}

__device__ __forceinline__ float tf32_rna(float x) {
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// x = hi + lo, both TF32 (the rest is below 2^-21 |x|)
__device__ __forceinline__ void tf32_split(float x, float &hi, float &lo) {
    hi = tf32_rna(x);
    lo = tf32_rna(__fsub_rn(x, hi));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
}

// wait for the completion of the given phase, at most `limit` polls (false: gave up)
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, int phase, int limit) {
    uint32_t done = 0;
    for (int it = 0; it < limit && !done; ++it)
        asm volatile("{\n .reg .pred q;\n mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n selp.u32 %0, 1, 0, q;\n}"
                     : "=r"(done) : "r"(smem_addr(bar)), "r"(phase));
    return done != 0;
}

// D (tensor memory) [+]= A B^T, both operands K-major in shared memory (descriptors)
__device__ __forceinline__ void tc_mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
                 :: "r"(d), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

// the MMAs issued so far by this thread arrive on the mbarrier when they complete
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(smem_addr(bar)));
}

// sixteen 32-bit columns of this warp's 32 lanes of tensor memory
__device__ __forceinline__ void tc_ld16(uint32_t a, uint32_t (&v)[16]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                   "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                 : "r"(a));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
}

// fragments (na, nb, ng) of pole t of a block, as k_poles enumerates them
__device__ __forceinline__ void pole_frags(const S2Block &B, int t, int nAa, int nAb, int nG, int &na, int &nb, int &ng) {
    ng = t % nG;
    int q = t / nG;
    if (B.ia == B.ib) {
        na = 0;
        while (na < nAa && q >= nAa - na - B.nJab) { q -= nAa - na - B.nJab; ++na; }
        nb = na + B.nJab + q;
    } else {
        na = q / nAb;
        nb = q % nAb;
    }
}

}  // namespace

__global__ void __launch_bounds__(kTcThreads) k_poles_tc(DevProblem P, const S2Block *blk, const int *tile_blk,
                                                         const int4 *tiles, int ntiles, const ChanSig *cs, int dir,
                                                         const double *vp, double *E, double *S2, double *M,
                                                         int *err) {
    const int tile = blockIdx.x;
    if (tile >= ntiles) return;
    const int4 T4 = tiles[tile];   // first entry in tile_blk, blocks, rows
    const int b_first = T4.x, nblk = T4.y, rows = T4.z;
    const S2Block B0 = blk[tile_blk[b_first]];
    const int T = dir == 0 ? B0.nfw : B0.nbk;   // poles of each block of the tile
    if (T <= 0) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int NS = P.nspb;
    const int *nA = dir == 0 ? P.np : P.nh, *nGv = dir == 0 ? P.nh : P.np;
    const int *sA = dir == 0 ? P.p_start : P.h_start, *sG = dir == 0 ? P.h_start : P.p_start;
    const double *eA = dir == 0 ? P.ep : P.eh, *eG = dir == 0 ? P.eh : P.ep;
    const double *fA = dir == 0 ? P.fqp : P.fqh, *fG = dir == 0 ? P.fqh : P.fqp;
    const int ia = B0.ia, ib = B0.ib, ig = B0.ig;
    const int noa = P.no[ia], nob = P.no[ib], nog = P.no[ig];
    const int nAa = nA[ia], nAb = nA[ib], nG = nGv[ig];
    const int Np = (T + 15) & ~15;

    extern __shared__ __align__(1024) unsigned char smc[];
    float *Ahi = reinterpret_cast<float *>(smc);           // [kTcRows][kTcKc] K-major core matrices
    float *Alo = Ahi + kTcRows * kTcKc;
    float *Bhi = Alo + kTcRows * kTcKc;                    // [Np][kTcKc]
    float *Blo = Bhi + Np * kTcKc;
    __shared__ int s_pa[kTcPairs], s_pb[kTcPairs];          // (alpha, beta) of pair p
    __shared__ int s_np;
    __shared__ short s_rblk[kTcRows], s_rd[kTcRows];        // block (in the tile) and d of every row
    __shared__ uint32_t s_taddr;
    __shared__ __align__(8) uint64_t s_bar;

    if (tid == 0) {
        int n = 0;
        for (int a = 0; a < noa; ++a)
            for (int b = (ia == ib) ? a + B0.nJab : 0; b < nob; ++b)
                if (n < kTcPairs) { s_pa[n] = a; s_pb[n] = b; ++n; }
        s_np = n;
        int r = 0;
        for (int q = 0; q < nblk && r < kTcRows; ++q) {
            const int D = P.no[blk[tile_blk[b_first + q]].ch];
            for (int d = 0; d < D && r < kTcRows; ++d, ++r) { s_rblk[r] = (short)q; s_rd[r] = (short)d; }
        }
        mbar_init(&s_bar);
    }
    const int ncols = Np <= 32 ? 32 : Np <= 64 ? 64 : Np <= 128 ? 128 : 256;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(&s_taddr)), "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t taddr = s_taddr;
    const int npair = s_np, K = npair * nog;
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(Np >> 3) << 17) |
                           ((uint32_t)(kTcRows >> 4) << 24);   // F32 += TF32 x TF32, K-major, M = 128, N = Np
    bool ok = true;
    int phase = 0;
    for (int kc0 = 0; kc0 < K; kc0 += kTcKc) {
        // A: V' of every row's block at columns k = p * nog + gamma (the reference's
        // excluded gamma == d terms as zeros), split into TF32 hi + lo
        for (int u = tid; u < kTcRows * kTcKc; u += kTcThreads) {
            const int r = u / kTcKc, kk = u - r * kTcKc, k = kc0 + kk;
            float x = 0.0f;
            if (r < rows && k < K) {
                const S2Block &Bb = blk[tile_blk[b_first + s_rblk[r]]];
                const int d = s_rd[r], p = k / nog, gam = k - p * nog;
                const bool excl = (P.orb_start[ig] + gam == P.orb_start[Bb.ch] + d) && Bb.nJgd;
                if (!excl) x = f64_to_f32(__ldg(vp + Bb.vp_first + (((size_t)d * noa + s_pa[p]) * nob + s_pb[p]) * nog + gam));
            }
            float hi, lo;
            tf32_split(x, hi, lo);
            Ahi[tc_off(r, kk)] = hi;
            Alo[tc_off(r, kk)] = lo;
        }
        // B: column t = pole (na, nb, ng), row k = (p, gamma): x4 x2(p) f_ng[gamma]
        for (int u = tid; u < Np * kTcKc; u += kTcThreads) {
            const int t = u / kTcKc, kk = u - t * kTcKc, k = kc0 + kk;
            float x = 0.0f;
            if (t < T && k < K) {
                int na, nb, ng;
                pole_frags(B0, t, nAa, nAb, nG, na, nb, ng);
                const int p = k / nog, gam = k - p * nog, a = s_pa[p], b = s_pb[p];
                const double *fa = fA + (size_t)(sA[ia] + na) * NS, *fb = fA + (size_t)(sA[ib] + nb) * NS;
                float x2 = f64_to_f32(__ldg(fa + a)) * f64_to_f32(__ldg(fb + b));
                if (ia == ib) {
                    x2 += (B0.nJab ? -1.0f : 1.0f) * f64_to_f32(__ldg(fa + b)) * f64_to_f32(__ldg(fb + a));
                    if (a == b) x2 *= 0.70710678118654752f;
                    if (na == nb) x2 *= 0.70710678118654752f;
                }
                x = x2 * f64_to_f32(__ldg(fG + (size_t)(sG[ig] + ng) * NS + gam));
            }
            float hi, lo;
            tf32_split(x, hi, lo);
            Bhi[tc_off(t, kk)] = hi;
            Blo[tc_off(t, kk)] = lo;
        }
        asm volatile("fence.proxy.async.shared::cta;");   // the staged tiles, to the tensor cores
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (tid == 0) {
            const int nstep = (min(kTcKc, K - kc0) + 7) / 8;
            const uint32_t sbo = (kTcKc / 4) * 128;   // next 8-row group
            for (int s = 0; s < nstep; ++s) {
                const uint32_t off = (uint32_t)s * 256;   // two 128-byte core matrices of K per step
                const uint64_t ah = mma_desc(smem_addr(Ahi) + off, 128, sbo), al = mma_desc(smem_addr(Alo) + off, 128, sbo);
                const uint64_t bh = mma_desc(smem_addr(Bhi) + off, 128, sbo), bl = mma_desc(smem_addr(Blo) + off, 128, sbo);
                const uint32_t acc0 = (kc0 > 0 || s > 0) ? 1u : 0u;
                tc_mma_tf32(taddr, ah, bh, idesc, acc0);
                tc_mma_tf32(taddr, ah, bl, idesc, 1u);
                tc_mma_tf32(taddr, al, bh, idesc, 1u);
            }
            tc_commit(&s_bar);
        }
        // the products are done before the tiles are staged again (bounded wait; the CTA
        // agrees on the outcome, so it leaves the loop together)
        const bool done = mbar_wait(&s_bar, phase, 1 << 22);
        phase ^= 1;
        ok = __syncthreads_and(done) != 0 && ok;
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (!ok) break;
    }
    if (!ok && lane == 0) atomicExch(err, 1);
    // every row's accumulators: warp w reads lanes 32w .. 32w + 31, sixteen columns at a time
    const int r = 32 * warp + lane;
    const bool has_row = r < rows;
    const S2Block Br = blk[tile_blk[b_first + (has_row ? s_rblk[r] : 0)]];
    const ChanSig Cr = cs[Br.ch];
    const int Nr = dir == 0 ? Cr.nfw : Cr.nbk;
    double *Mrow = M + (dir == 0 ? Cr.mfw_off : Cr.mbk_off) + (size_t)(has_row ? s_rd[r] : 0) * Nr +
                   ((dir == 0 ? Br.fw_first : Br.bk_first) - (dir == 0 ? Cr.fw_off : Cr.bk_off));
    for (int c0 = 0; c0 < Np; c0 += 16) {
        uint32_t v[16];
        if (ok && K > 0) {
            tc_ld16(taddr + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
        } else {
#pragma unroll
            for (int q = 0; q < 16; ++q) v[q] = 0u;
        }
        if (has_row)
#pragma unroll
            for (int q = 0; q < 16; ++q)
                if (c0 + q < T) Mrow[c0 + q] = f32_to_f64(__uint_as_float(v[q]));
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols));
    // energies (the reference's FP64 operations) and S2 = sum_d M^2 of every pole of the tile
    __threadfence_block();
    for (int u = tid; u < nblk * T; u += kTcThreads) {
        const int q = u / T, t = u - q * T;
        const S2Block Bq = blk[tile_blk[b_first + q]];
        const ChanSig Cq = cs[Bq.ch];
        int na, nb, ng;
        pole_frags(Bq, t, nAa, nAb, nG, na, nb, ng);
        const long long g = (dir == 0 ? Bq.fw_first : Bq.bk_first) + t;
        E[g] = __dsub_rn(__dadd_rn(eA[sA[ia] + na], eA[sA[ib] + nb]), eG[sG[ig] + ng]);
        const int Nq = dir == 0 ? Cq.nfw : Cq.nbk;
        const double *Mq = M + (dir == 0 ? Cq.mfw_off : Cq.mbk_off) + (g - (dir == 0 ? Cq.fw_off : Cq.bk_off));
        float s2 = 0.0f;
        for (int d = 0; d < P.no[Bq.ch]; ++d) { const float m = f64_to_f32(Mq[(size_t)d * Nq]); s2 = fmaf(m, m, s2); }
        S2[g] = f32_to_f64(s2);
    }
}

}  // namespace bd

namespace bd {

size_t tc_smem_bytes(int np) {
    return sizeof(float) * ((size_t)2 * kTcRows * kTcKc + (size_t)2 * np * kTcKc);
}

cudaError_t launch_poles_tc(const DevProblem &P, const S2Block *blk, const int *tile_blk, const int4 *tiles,
                            int ntiles, const ChanSig *cs, int dir, const double *vp, double *E, double *S2, double *M,
                            int *err, size_t smem, cudaStream_t st) {
    if (ntiles <= 0) return cudaSuccess;
    cudaError_t e = allow_dynamic_smem((const void *)k_poles_tc);
    if (e != cudaSuccess) return e;
    k_poles_tc<<<ntiles, kTcThreads, smem, st>>>(P, blk, tile_blk, tiles, ntiles, cs, dir, vp, E, S2, M, err);
    return cudaGetLastError();
}

void tc_smem_init() { allow_dynamic_smem((const void *)k_poles_tc); }

}  // namespace bd
