// k_sort.cu -- stable least-significant-digit radix sort of (64-bit key, 32-bit value)
// pairs, eight bits per pass, used where a sort is longer than a CTA's shared memory:
// channels of more than kSortMax poles (dressed propagators) and the interaction's
// canonical keys (VppInt_t::prepare_for_reading, source/BcDor-Vpp_potential.cpp:440-501).
//
// One pass over digit [shift, shift + 8):
//   k_rs_hist     one CTA per tile of kRsTile pairs: the tile's 256 digit counts,
//                 stored digit-major (count[d * ntiles + tile]);
//   k_rs_scan     exclusive scan of the counts in that order (three kernels: chunk
//                 sums, one CTA scanning the chunk sums, chunk scans), so
//                 count[d * ntiles + tile] becomes the first output position of digit
//                 d's pairs of the tile;
//   k_rs_scatter  the tile again: each warp takes 32 consecutive pairs at a time; lanes
//                 of equal digit find one another with __match_any_sync, so a pair's
//                 rank among the tile's pairs of its digit is (pairs of that digit in
//                 earlier warps) + (in the warp's earlier rounds) + (lower lanes of this
//                 round) -- the input order is kept, so every pass is stable.
// With skip_constant, passes whose digit is the same for every key (known from the OR
// and AND of all keys, read back with one synchronisation) are skipped: they would
// move nothing.
#include <algorithm>
#include <climits>
#include <cstdint>
#include <utility>
#include "bd_kernels.h"

namespace bd {

constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsPerLane = 16;                          // rounds of 32 pairs per warp
constexpr int kRsTile = kRsThreads * kRsPerLane;        // 4096 pairs per CTA
constexpr int kRsScanChunk = 4096;                      // counts per chunk of the scan

__global__ void __launch_bounds__(kRsThreads) k_rs_bits(const unsigned long long *k, long long n,
                                                        unsigned long long *orand) {
    unsigned long long o = 0ull, a = ~0ull;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long x = k[i];
        o |= x;
        a &= x;
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        o |= __shfl_xor_sync(0xffffffffu, o, s);
        a &= __shfl_xor_sync(0xffffffffu, a, s);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicOr(&orand[0], o);
        atomicAnd(&orand[1], a);
    }
}

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const unsigned long long *k, long long n, int shift,
                                                        int ntiles, unsigned *count) {
    __shared__ unsigned h[256];
    h[threadIdx.x] = 0u;
    __syncthreads();
    const long long t0 = (long long)blockIdx.x * kRsTile;
    const long long t1 = t0 + kRsTile < n ? t0 + kRsTile : n;
    for (long long i = t0 + threadIdx.x; i < t1; i += kRsThreads) atomicAdd(&h[(unsigned)(k[i] >> shift) & 255u], 1u);
    __syncthreads();
    count[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Block-wide exclusive scan of one value per thread; returns the prefix, total in *tot.
__device__ inline unsigned rs_block_scan(unsigned x, unsigned *tot, unsigned *ws) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) ws[warp] = v;
    __syncthreads();
    unsigned off = 0, t = 0;
    for (int w = 0; w < kRsWarps; ++w) {
        const unsigned s = ws[w];
        if (w < warp) off += s;
        t += s;
    }
    __syncthreads();
    *tot = t;
    return off + v - x;
}

__global__ void __launch_bounds__(kRsThreads) k_rs_chunk_sums(const unsigned *count, long long m, unsigned *sums) {
    __shared__ unsigned ws[kRsWarps];
    const long long c0 = (long long)blockIdx.x * kRsScanChunk;
    unsigned s = 0;
    for (long long i = c0 + threadIdx.x; i < c0 + kRsScanChunk && i < m; i += kRsThreads) s += count[i];
    unsigned tot;
    rs_block_scan(s, &tot, ws);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scan_sums(unsigned *sums, int nchunks) {
    __shared__ unsigned ws[kRsWarps];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    for (int b = 0; b < nchunks; b += kRsThreads) {
        const int i = b + threadIdx.x;
        const unsigned x = i < nchunks ? sums[i] : 0u;
        unsigned tot;
        const unsigned p = rs_block_scan(x, &tot, ws);
        if (i < nchunks) sums[i] = carry + p;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kRsThreads) k_rs_chunk_scan(unsigned *count, long long m, const unsigned *sums) {
    __shared__ unsigned ws[kRsWarps];
    const long long c0 = (long long)blockIdx.x * kRsScanChunk;
    constexpr int per = kRsScanChunk / kRsThreads;   // 16 consecutive counts per thread
    unsigned v[per];
    unsigned s = 0;
    const long long b = c0 + (long long)threadIdx.x * per;
#pragma unroll
    for (int q = 0; q < per; ++q) {
        v[q] = (b + q < m) ? count[b + q] : 0u;
        s += v[q];
    }
    unsigned tot;
    unsigned p = sums[blockIdx.x] + rs_block_scan(s, &tot, ws);
#pragma unroll
    for (int q = 0; q < per; ++q) {
        if (b + q < m) count[b + q] = p;
        p += v[q];
    }
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const unsigned long long *kin, const unsigned *vin, long long n,
                                                           int shift, int ntiles, const unsigned *offs,
                                                           unsigned long long *kout, unsigned *vout) {
    __shared__ unsigned wc[kRsWarps][256];   // per warp: pairs of each digit so far
    __shared__ unsigned base[kRsWarps][256];  // per warp: pairs of each digit in earlier warps
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < 256 * kRsWarps; d += kRsThreads) (&wc[0][0])[d] = 0u;
    __syncthreads();
    const long long w0 = (long long)blockIdx.x * kRsTile + (long long)warp * (kRsTile / kRsWarps);
    unsigned long long key[kRsPerLane];
    unsigned val[kRsPerLane], rk[kRsPerLane];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kRsPerLane; ++r) {
        const long long i = w0 + r * 32 + lane;
        const bool ok = i < n;
        key[r] = ok ? kin[i] : 0ull;
        val[r] = ok ? vin[i] : 0u;
        const unsigned d = ok ? ((unsigned)(key[r] >> shift) & 255u) : 256u + (unsigned)lane;   // past the end: alone
        const unsigned m = __match_any_sync(0xffffffffu, d);
        unsigned pre = 0u;
        if (ok) pre = wc[warp][d];
        __syncwarp();
        if (ok && (m & lt) == 0u) wc[warp][d] = pre + __popc(m);
        __syncwarp();
        rk[r] = pre + __popc(m & lt);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += kRsThreads) {
        unsigned s = 0u;
        for (int w = 0; w < kRsWarps; ++w) {
            base[w][d] = s;
            s += wc[w][d];
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRsPerLane; ++r) {
        const long long i = w0 + r * 32 + lane;
        if (i >= n) continue;
        const unsigned d = (unsigned)(key[r] >> shift) & 255u;
        const unsigned pos = offs[(size_t)d * ntiles + blockIdx.x] + base[warp][d] + rk[r];
        kout[pos] = key[r];
        vout[pos] = val[r];
    }
}

// In-place exclusive scan of m counts (the radix sort's scan kernels); scratch holds
// one unsigned per kRsScanChunk counts.
size_t scan_scratch_bytes(long long m) { return (size_t)(4 * ((m + kRsScanChunk - 1) / kRsScanChunk) + 16); }

cudaError_t exclusive_scan_u32(unsigned *data, long long m, void *scratch, cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    const long long nchunks = (m + kRsScanChunk - 1) / kRsScanChunk;
    unsigned *sums = static_cast<unsigned *>(scratch);
    k_rs_chunk_sums<<<(unsigned)nchunks, kRsThreads, 0, st>>>(data, m, sums);
    k_rs_scan_sums<<<1, kRsThreads, 0, st>>>(sums, (int)nchunks);
    k_rs_chunk_scan<<<(unsigned)nchunks, kRsThreads, 0, st>>>(data, m, sums);
    return cudaGetLastError();
}

size_t radix_scratch_bytes(long long n) {
    const long long ntiles = (n + kRsTile - 1) / kRsTile;
    const long long m = 256 * ntiles;
    const long long nchunks = (m + kRsScanChunk - 1) / kRsScanChunk;
    return (size_t)(16 + 4 * m + 4 * nchunks + 256);
}

int radix_launches(int passes, bool skip_constant) { return (skip_constant ? 1 : 0) + 5 * passes; }

cudaError_t radix_sort_pairs(unsigned long long *&keys, unsigned *&vals, unsigned long long *&ktmp, unsigned *&vtmp,
                             long long n, int bit0, int bit1, bool skip_constant, void *scratch, int *passes_out,
                             cudaStream_t st) {
    if (passes_out) *passes_out = 0;
    if (n <= 1) return cudaSuccess;
    if (n > (long long)UINT_MAX / 2) return cudaErrorInvalidValue;
    const long long ntiles = (n + kRsTile - 1) / kRsTile;
    const long long m = 256 * ntiles;
    const long long nchunks = (m + kRsScanChunk - 1) / kRsScanChunk;
    char *p = static_cast<char *>(scratch);
    unsigned long long *orand = reinterpret_cast<unsigned long long *>(p);
    unsigned *count = reinterpret_cast<unsigned *>(p + 16);
    unsigned *sums = count + m;
    cudaError_t e = cudaSuccess;
    unsigned long long vary = ~0ull;
    if (skip_constant) {   // which digits vary: OR and AND of all keys, read back
        if ((e = cudaMemsetAsync(orand, 0, 8, st)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(orand + 1, 0xff, 8, st)) != cudaSuccess) return e;
        const unsigned gb = (unsigned)std::min<long long>((n + kRsThreads - 1) / kRsThreads, 152 * 8);
        k_rs_bits<<<gb, kRsThreads, 0, st>>>(keys, n, orand);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        unsigned long long h[2];
        if ((e = cudaMemcpyAsync(h, orand, sizeof h, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
        vary = h[0] ^ h[1];
    }
    int passes = 0;
    for (int shift = bit0; shift < bit1; shift += 8) {
        const unsigned long long mask = (shift + 8 >= 64) ? (~0ull << shift) : (((1ull << 8) - 1ull) << shift);
        if ((vary & mask) == 0ull) continue;
        k_rs_hist<<<(unsigned)ntiles, kRsThreads, 0, st>>>(keys, n, shift, (int)ntiles, count);
        k_rs_chunk_sums<<<(unsigned)nchunks, kRsThreads, 0, st>>>(count, m, sums);
        k_rs_scan_sums<<<1, kRsThreads, 0, st>>>(sums, (int)nchunks);
        k_rs_chunk_scan<<<(unsigned)nchunks, kRsThreads, 0, st>>>(count, m, sums);
        k_rs_scatter<<<(unsigned)ntiles, kRsThreads, 0, st>>>(keys, vals, n, shift, (int)ntiles, count, ktmp, vtmp);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        std::swap(keys, ktmp);
        std::swap(vals, vtmp);
        ++passes;
    }
    if (passes_out) *passes_out = passes;
    return cudaSuccess;
}

}  // namespace bd
