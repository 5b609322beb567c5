// k_lanczos.cu -- K2: multi-pivot Lanczos reduction of a diag(E) + M pole space.
//
// Restates Reduce_Mtx_Lncz (source/BcDor-Lanczos.cpp:44-286): for every Lanczos
// index j, a new pivot chain starts from v = M.p (p normalised) or the chain
// continues from v = diag(E) v_{j-1}; v is orthogonalised against every earlier
// vector; then alpha = <v|E|v>/<v|v>, beta = |v|, m = M^T v / beta and, for every
// earlier pivot q, g_q = <v_last(q)|E|v> / beta are written to the output row.
//
// Orthogonalisation: the reference sweeps once, backward, with modified
// Gram-Schmidt (source/BcDor-Lanczos.cpp:160-173).  Here each sweep is a
// classical Gram-Schmidt projection (two streaming passes over the stored
// vectors: dot products, then the update), repeated while a sweep removes more
// than 1 - 1/sqrt(2) of the remaining norm (the Daniel-Gragg-Kaufman-Stewart
// criterion), at most four sweeps.  A continuing chain first projects out only
// v_{j-1}, v_{j-2} and the last vector of each earlier chain, the only vectors on
// which E v_{j-1} has more than rounding-size components; the full sweep that
// follows then removes little, so one full sweep per step is the common case
// instead of two.  With FP32 vectors such a continuing step takes one cluster
// reduction: the sweep's dot products are summed together with the sums over w that
// the step's scalars need, the scalars of the swept vector follow from those and the
// stored rows to first order in the sweep's rounding-sized coefficients (dots_fused,
// fused_scalars), and the update is applied in the pass that writes the vector; the
// exact scalar pass remains for every step where that does not hold.  On the
// degenerate unperturbed spectra the
// chains break down every few steps and, with few distinct pole energies, the
// reachable subspace (E is diagonal, so the support of M.p never grows) can be
// spanned completely; a single sweep then leaves the new vectors far from
// orthogonal and the reduced self-energy depends on rounding (measured: E_Koltun
// moves by MeV), two sweeps still fail once the reachable subspace is exhausted,
// and the iterated sweeps keep |V^T V - I| at 1e-15 and reproduce the un-reduced
// Dyson solution.
//
// Exhausted subspace: when even the iterated sweeps leave nothing (the squared norm
// falls below tau times its value before the first sweep, tau = 1e-48 in FP64 and
// 1e-22 with FP32 vectors, or is exactly zero), the subspace the chain can reach is
// spanned.  The reference then divides by beta ~ 0 and its rows become NaN.  Here the
// chain continues with the unit vector of the first pole that no stored vector
// touches (exact zeros: diag(E) and the projections never grow a vector's support),
// an exact eigenvector of diag(E) orthogonal to the basis (alpha = E_k, beta = 0,
// g = 0, m = M[k, :]); if every pole is touched, with a pseudo-random vector swept
// orthogonal to the basis (beta = 0, alpha / g / m computed as usual).  Either way the
// kept rows remain the exact projection: with full reorthogonalisation E v_t lies in
// the span of v_0 .. v_{t+1}, so a vector orthogonal to the basis couples by E only
// to the last vector of each earlier pivot chain, which is what g records.
//
// Work split: one thread-block cluster per chain; CTA r of the cluster owns the
// pole rows [r*S, (r+1)*S) of every vector.  Partial sums are combined through
// distributed shared memory; every CTA adds the peers' partials in the same fixed
// order, so all CTAs hold bit-identical totals and take identical branches.
#include <algorithm>
#include <climits>
#include <cooperative_groups.h>
#include "df64.cuh"
#include "bd_common.cuh"
#include "bd_kernels.h"

namespace cg = cooperative_groups;

namespace bd {

template <typename VT> struct LzTraits;
template <> struct LzTraits<double> { using CT = double; };
template <> struct LzTraits<float> { using CT = float; };

template <typename T>
__device__ inline T warp_sum_ct(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Warp sums of NV values at once (NV a power of two <= 32): each level of the xor
// butterfly (offsets 16, 8, ..., 1, the order of warp_sum_ct) sends the half of the
// values a lane does not keep and adds the partner's half to the kept one, so NV - 1
// shuffles (plus one per level left once a single value remains) replace 5 NV; every
// total is associated exactly as warp_sum_ct associates it.  Lane L ends with the total
// of value L >> (5 - log2 NV).
__device__ __forceinline__ float shfl_xor_t(float x, int o) { return __shfl_xor_sync(0xffffffffu, x, o); }
__device__ __forceinline__ double shfl_xor_t(double x, int o) { return __shfl_xor_sync(0xffffffffu, x, o); }
__device__ __forceinline__ dfm::df shfl_xor_t(dfm::df x, int o) { return dfm::shfl_xor(x, o); }
__device__ __forceinline__ float add_t(float a, float b) { return a + b; }
__device__ __forceinline__ double add_t(double a, double b) { return a + b; }
__device__ __forceinline__ dfm::df add_t(dfm::df a, dfm::df b) { return dfm::add(a, b); }
template <int NV, typename T>
__device__ __forceinline__ T warp_sums(T *v, int lane) {
#pragma unroll
    for (int lev = 0; lev < 5; ++lev) {
        const int o = 16 >> lev;
        const int n = NV >> (lev + 1);   // values a lane keeps after this level
        if (n >= 1) {
            const bool up = (lane & o) != 0;
#pragma unroll
            for (int i = 0; i < (NV >> 1); ++i)
                if (i < n) {
                    const T send = up ? v[i] : v[i + n];
                    const T keep = up ? v[i + n] : v[i];
                    v[i] = add_t(keep, shfl_xor_t(send, o));
                }
        } else {
            v[0] = add_t(v[0], shfl_xor_t(v[0], o));
        }
    }
    return v[0];
}

// Sums across warps and CTAs.  FP64 vectors: FP64 adds.  FP32 vectors: the partials
// are FP32 values, summed in double-float (df64.cuh) on the FP32 pipe -- an FP64 add
// holds the SM sub-partition's FP64 unit for about 64 cycles, and the trees below are
// on every step's critical path -- and kept as (hi, lo) pairs in the 8 bytes of a
// double slot.  Both are exact for the first level and far inside FP32 vectors'
// rounding after it.
template <typename CT> struct LzSum {
    using T = double;
    static __device__ __forceinline__ T zero() { return 0.0; }
    static __device__ __forceinline__ T from_ct(CT x) { return (double)x; }
    static __device__ __forceinline__ void put(double *slot, T x) { *slot = x; }
    static __device__ __forceinline__ T get(const double *slot) { return *slot; }
    static __device__ __forceinline__ T add(T a, T b) { return a + b; }
    static __device__ __forceinline__ double value(T x) { return x; }
};
template <> struct LzSum<float> {
    using T = dfm::df;
    static __device__ __forceinline__ T zero() { return T{0.0f, 0.0f}; }
    static __device__ __forceinline__ T from_ct(float x) { return T{x, 0.0f}; }
    static __device__ __forceinline__ void put(double *slot, T x) {
        *reinterpret_cast<float2 *>(slot) = make_float2(x.h, x.l);
    }
    static __device__ __forceinline__ T get(const double *slot) {
        const float2 f = *reinterpret_cast<const float2 *>(slot);
        return T{f.x, f.y};
    }
    static __device__ __forceinline__ T add(T a, T b) { return dfm::add(a, b); }
    static __device__ __forceinline__ double value(T x) { return dfm::to_double(x); }
};

// A thread's partial sum of many terms.  Plain: in the arithmetic type.  Compensated
// (FP32 vectors on long chains, whose slices hold tens of thousands of poles): in
// double-float, each term (or chunk of four FP32 products) added exactly, so a partial
// over hundreds of terms keeps FP64-class accuracy; then the warp combines the pairs.
// Long chains stream their bases from HBM, so the FP32 pipe has the room.
template <typename CT, bool kComp> struct PSum {
    using A = CT;
    static __device__ __forceinline__ A zero() { return (CT)0; }
    static __device__ __forceinline__ void add(A &a, CT x) { a += x; }
    static __device__ __forceinline__ typename LzSum<CT>::T finish(A a) { return LzSum<CT>::from_ct(warp_sum_ct(a)); }
};
template <> struct PSum<float, true> {
    using A = dfm::df;
    static __device__ __forceinline__ A zero() { return A{0.0f, 0.0f}; }
    static __device__ __forceinline__ void add(A &a, float x) { a = dfm::add(a, A{x, 0.0f}); }
    static __device__ __forceinline__ A finish(A a) { return dfm::warp_sum(a); }
};

// Fixed pairwise sums: three (four) dependent adds instead of seven (fifteen).
template <class Sum>
__device__ inline typename Sum::T tree_sum8(const typename Sum::T *x) {
    return Sum::add(Sum::add(Sum::add(x[0], x[1]), Sum::add(x[2], x[3])),
                    Sum::add(Sum::add(x[4], x[5]), Sum::add(x[6], x[7])));
}

// Deterministic pseudo-random restart value of pole i at Lanczos index j, in [0.5, 1.5).
__host__ __device__ inline double restart_value(int i, int j) {
    unsigned x = (unsigned)i * 2654435761u ^ ((unsigned)j * 40503u + 0x9e3779b9u);
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return 0.5 + (double)(x & 0xffffffu) / 16777216.0;
}

constexpr int kLzThreads = 256;
constexpr int kLzWarps = kLzThreads / 32;
static_assert(kLzWarps == 8, "the warp partials are summed by tree_sum8");
constexpr int kMaxScal = 32;   // 3 + D + n_used <= 19 (D <= 8, at most 8 earlier pivots)
// Dynamic shared memory of a launch at least this large (two CTAs per SM), the room
// behind the slices holding the basis cache.
constexpr size_t kLzSmemCache = 108 * 1024;

// 16-byte vector of the storage type: 4 floats or 2 doubles
template <typename VT> struct Vec16;
template <> struct Vec16<float> { using T = float4; static constexpr int n = 4; };
template <> struct Vec16<double> { using T = double2; static constexpr int n = 2; };

template <typename VT>
__device__ inline void load16(const VT *p, VT *out);
template <> __device__ inline void load16<float>(const float *p, float *o) {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
template <> __device__ inline void load16<double>(const double *p, double *o) {
    const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    o[0] = v.x; o[1] = v.y;
}
// the same through a generic address (shared or global memory)
template <typename VT>
__device__ inline void load16g(const VT *p, VT *out);
template <typename VT>
__device__ inline void store16g(VT *p, const VT *v);
template <> __device__ inline void store16g<float>(float *p, const float *v) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
template <> __device__ inline void store16g<double>(double *p, const double *v) {
    *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
}
template <> __device__ inline void load16g<float>(const float *p, float *o) {
    const float4 v = *reinterpret_cast<const float4 *>(p);
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
template <> __device__ inline void load16g<double>(const double *p, double *o) {
    const double2 v = *reinterpret_cast<const double2 *>(p);
    o[0] = v.x; o[1] = v.y;
}

// Slice of a CTA: S pole rows starting at rank*S, S a multiple of 4; rows past N are
// zero in every vector (E, w, V), so the vector loads need no tail handling.
//
// Shared-memory layout: doubles A[2][rmax] (dot partials of alternate passes) |
// c[rmax] (totals) | Bs[kMaxScal] (scalar partials) | red[kLzWarps * kMaxScal] (per warp),
// then CT (the vectors' arithmetic type) cf[rmax rounded up to 4] (totals in CT) |
// Es[S] | w[S], then touched[S] bytes, then the basis cache up to smem_bytes.
//
// Basis cache: a CTA reads and writes only its own slice of every stored vector (the
// dot products, the updates and the step scalars are slice-local; CTAs meet only in
// the cluster sums), so the first ccap vectors' slices are kept in the CTA's shared
// memory as well as in V: ccap = the room left behind the slices divided by S values.
// The reads of those vectors then cost shared-memory latency instead of L2's.  V keeps
// every vector (the host reads the basis back from it).
//
// Arithmetic: with FP64 vectors everything is FP64.  With FP32 vectors every
// per-pole operation (products, the update, the per-thread partial sums of the dot
// products, norms and scalars) is FP32, and only the sums across warps and CTAs are
// wider, in double-float (LzSum): on this GPU FP64 issues at 1/64 of the FP32 rate, and
// a per-pole FP64 operation would cost more than the whole FP32 sweep.
template <typename VT, bool kGlobalSlices>
__global__ void __launch_bounds__(kLzThreads, 2) k_lanczos(const LzChain *chains, int nchains, int rmax, double eta2,
                                                          int smem_bytes) {
    using CT = typename LzTraits<VT>::CT;
    using Sum = LzSum<CT>;
    using ST = typename Sum::T;
    constexpr bool kComp = kGlobalSlices && sizeof(VT) == 4;   // compensated partial sums
    constexpr bool kFused = sizeof(VT) == 4;                     // one-reduction recurrence steps
    using PS = PSum<CT, kComp>;
    using PA = typename PS::A;
    constexpr int VW = Vec16<VT>::n;
    cg::cluster_group cluster = cg::this_cluster();
    const int CL = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int cid = blockIdx.x / CL;
    if (cid >= nchains) return;  // whole clusters only: every CTA of a cluster has the same cid
    const LzChain C = chains[cid];
    const int N = C.N, D = C.D, L = C.L, NT = C.nden_out + C.D;
    const int S = C.S;                       // multiple of 4
    const int i0 = rank * S;
    const int ns = max(0, min(N, i0 + S) - i0);
    const int nv = S / VW;                   // 16-byte vectors per slice
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    extern __shared__ double sm[];
    const int rmax2 = (rmax + 1) & ~1;   // even: keeps the arrays behind 16-byte aligned
    const int rq = (rmax + 3) / 4 * 4;
    const int apn = lz_partials_per_pass(rmax);
    double *A = sm;                      // [2][apn] dot partials, alternating by pass
    double *c = A + 2 * apn;             // [rmax2] totals
    double *dt = c + rmax2;              // [rmax2] <v_t|E w> of a recurrence step's pass
    double *Bs = dt + rmax2;
    double *red = Bs + kMaxScal;
    int *rowslot = reinterpret_cast<int *>(red + kLzWarps * kMaxScal);   // vector slot of every row, -1: deflated
    int *slotrow = rowslot + rq;                                        // row of every vector slot
    CT *cf = reinterpret_cast<CT *>(slotrow + rq);                      // 16-byte aligned
    CT *Es, *w, *ew;
    unsigned char *touched;
    if constexpr (kGlobalSlices) {   // chains too long for shared memory: this CTA's slices in global scratch
        Es = reinterpret_cast<CT *>(C.slice + (size_t)rank * C.slice_stride);
        w = Es + S;
        ew = w + S;
        touched = reinterpret_cast<unsigned char *>(ew + S);
    } else {
        Es = cf + rq;
        w = Es + S;
        ew = w + S;
        touched = reinterpret_cast<unsigned char *>(ew + S);
    }
    // this CTA's slice of the couplings M (CT, [d][S]) behind the slices, then the basis cache
    CT *Msl = nullptr;
    if constexpr (!kGlobalSlices) {
        const uintptr_t mb = (reinterpret_cast<uintptr_t>(touched + S) + 15) & ~static_cast<uintptr_t>(15);
        const uintptr_t me = mb + sizeof(CT) * (size_t)D * S;
        if (me <= reinterpret_cast<uintptr_t>(sm) + static_cast<uintptr_t>(smem_bytes)) Msl = reinterpret_cast<CT *>(mb);
    }
    VT *cache;
    int ccap;
    {
        const char *end = kGlobalSlices ? reinterpret_cast<const char *>(cf + rq)
                                        : (Msl ? reinterpret_cast<const char *>(Msl + (size_t)D * S)
                                               : reinterpret_cast<const char *>(touched + S));
        const uintptr_t e = (reinterpret_cast<uintptr_t>(end) + 15) & ~static_cast<uintptr_t>(15);
        const uintptr_t lim = reinterpret_cast<uintptr_t>(sm) + static_cast<uintptr_t>(smem_bytes);
        cache = reinterpret_cast<VT *>(e);
        ccap = (e < lim && S > 0) ? (int)((lim - e) / ((uintptr_t)S * sizeof(VT))) : 0;
    }
    // FP64 vectors: the two most recent vectors (read by every recurrence step) keep their
    // slices in two ring slots behind the cache once they are beyond it.  (With FP32
    // vectors the cache holds four times as many, and the ring's extra select in every
    // vector access cost more than it saved.)
    const bool hasring = sizeof(VT) == 8 && ccap >= 3;
    if (hasring) ccap -= 2;
    VT *ring = cache + (size_t)ccap * S;
    __shared__ double tot[kMaxScal];
    __shared__ double prow[kMaxScal];   // the last built row, [alpha, beta, g..., m...] (every CTA)
    __shared__ double s_e2v;            // |E v|^2 of the last built vector
    __shared__ double s_xb, s_ixb;
    __shared__ int s_kmin;
    __shared__ int lt[16];       // vectors of a local pass
    __shared__ int s_nl;
    __shared__ int lslot[8];     // slots of the earlier chains' last vectors (-1: deflated)
    __shared__ int s_start[10], s_last[10];   // the chain schedule (read every step: kept on chip)
    __shared__ int s_flag;       // thread 0's decision after a full sweep (0 keep, 1 sweep again, 2 exhausted, 3 restart)
    __shared__ CT s_ixbf;        // 1/|w| in the arithmetic type
    __shared__ CT lcf[16];       // coefficients of a recurrence step's local vectors
    __shared__ double fsc[12];   // a recurrence step's sums of w: |w|^2, <w|E|w>, |E w|^2, <M_d|w>
    // FP32 vectors: the step's scalars in double-float as well, for its serial part (thread
    // 0's decision, warp 0's row), where each FP64 instruction would hold an SM
    // sub-partition's FP64 unit for ~64 cycles
    __shared__ dfm::df fscd[12], totd[kMaxScal];
    __shared__ dfm::df s_rd, s_xbd, s_e2vd;   // 1/|w|, |w| of the step; |E v|^2 of the last built vector
    __shared__ float prowf[kMaxScal];         // the last built row in FP32 (the next step's coefficients)

    VT *V = reinterpret_cast<VT *>(C.V);
    // this CTA's slice of stored vector t: in the cache, or in V
    int nvec = 0;                // vectors stored so far
    auto vslice = [&](int t) -> VT * {
        return t < ccap ? cache + (size_t)t * S
                        : (hasring && t >= nvec - 2 ? ring + (size_t)(t & 1) * S : V + (size_t)t * C.ld + i0);
    };
    const CT *Mc = reinterpret_cast<const CT *>(sizeof(CT) == 4 ? static_cast<const void *>(C.Mf)
                                                                  : static_cast<const void *>(C.M));
    for (int i = tid; i < S; i += kLzThreads) { Es[i] = (i < ns) ? (CT)C.E[i0 + i] : (CT)0; touched[i] = 0; }
    if (Msl)
        for (int q = tid; q < D * S; q += kLzThreads) {
            const int d = q / S, i = q - d * S;
            Msl[q] = (i < ns) ? Mc[(size_t)d * N + i0 + i] : (CT)0;
        }
    if (tid <= C.n_used && tid < 10) s_start[tid] = C.start[tid];
    if (tid < C.n_used && tid < 10) s_last[tid] = C.last[tid];
    __syncthreads();   // the schedule is read at the top of the first step, before its barrier
    const double tau = (sizeof(VT) == 4) ? 1e-22 : 1e-48;
    // Exhausted Krylov space: the squared residual after the sweeps at rounding level
    // relative to its value before them.  The chain's remaining rows then continue with
    // eigenvectors of E that no coupling reaches (energy groups from k_lz_groups): each
    // such row is (E_q, 0, ..., 0), needs no vector, and deflates out of the Dyson matrix.
    const double thr_exh = (sizeof(VT) == 4) ? 1e-9 : 1e-20;
    // the decision's factors in double-float (FP32 vectors)
    const dfm::df c099d = dfm::from_double(0.99), eta2d = dfm::from_double(eta2), thr_exhd = dfm::from_double(thr_exh),
                  taud = dfm::from_double(tau);
    auto df_lt = [](dfm::df a, dfm::df b) { return a.h < b.h || (a.h == b.h && a.l < b.l); };
    auto df_le = [](dfm::df a, dfm::df b) { return a.h < b.h || (a.h == b.h && a.l <= b.l); };
    const int Qg = C.gE ? C.gInfo[0] : 0;
    const int dtot = Qg > 0 ? C.gInfo[Qg] : 0;   // unreached directions of all groups
    int dcur = 0;                // directions used so far (identical in every CTA)
    auto group_of = [&](int d) {   // group holding direction d < dtot: first q with cum[q] > d
        int lo = 0, hi = Qg - 1;
        while (lo < hi) { const int mid = (lo + hi) >> 1; if (C.gInfo[1 + mid] > d) hi = mid; else lo = mid + 1; }
        return lo;
    };
    bool tail = false;           // rest of the current pivot chain deflated
    bool contaminated = false;   // a restart vector was stored: no deflation from here on
    int ndefl = 0;
    auto next_slot = [&]() -> bool { return dcur < dtot; };   // an unused direction is left
    auto deflated_row = [&](int jr) {  // consume a direction and write its row
        const double a = (dcur < dtot) ? C.gE[group_of(dcur)] : C.gE[Qg - 1];
        if (dcur < dtot) ++dcur;
        if (rank == 0 && tid == 0) {
            double *row = C.out + (size_t)jr * NT;
            for (int q = 0; q < NT; ++q) row[q] = 0.0;
            row[0] = a;
        }
        if (tid == 0) rowslot[jr] = -1;
        ++ndefl;
    };

    // Sum over the cluster of one value per CTA held at buf[t], a fixed pairwise tree
    // over the ranks (the loads first, then four levels of adds: one DSMEM round trip
    // and a short chain instead of CL of each).
    auto cluster_sum_st = [&](const double *buf, int t) -> ST {
        ST x[16];
#pragma unroll
        for (int r = 0; r < 16; ++r)
            x[r] = (r < CL) ? Sum::get(cluster.map_shared_rank(const_cast<double *>(buf), r) + t) : Sum::zero();
        return Sum::add(tree_sum8<Sum>(x), tree_sum8<Sum>(x + 8));
    };
    // (b1) dots pass: <v_t, w> for the pass's vectors t < nl and |w|^2, summed over
    // the cluster into cf[0..nl) and c[nl] = |w|^2.  One warp forms each dot product,
    // w itself counting as the pass's vector nl (its square norm), eight vectors per
    // warp at a time: eight independent 16-byte loads in flight per lane (one vector's
    // slice is only a few loads per lane, so a warp that took its vectors one after
    // another would wait out the L2 latency per vector), and no CTA barrier before the
    // cluster's.  The per-CTA partials alternate between two buffers: a peer may still
    // gather the previous pass's while this CTA writes the next (no cluster barrier
    // between a local update and the full sweep's dot products).
    int dpar = 0;
    auto dots_pass = [&](bool loc, int nl) {
        double *Ap = A + (size_t)dpar * apn;
        dpar ^= 1;
        const VT *wv = reinterpret_cast<const VT *>(w);
        // FP32 vectors: eight per warp at a time; FP64: four, two groups per lane in flight
        // (the FP64 products bound that pass, not the loads)
        constexpr int NU = sizeof(CT) == 4 ? 8 : 4;
        constexpr int LS = sizeof(CT) == 4 ? 2 : 3;   // lane L holds the total of vector L >> LS
        constexpr int UNR = sizeof(CT) == 4 ? 1 : 2;
        for (int t0 = warp; t0 <= nl; t0 += NU * kLzWarps) {
            const VT *vp[NU];
#pragma unroll
            for (int u = 0; u < NU; ++u) {
                const int t = t0 + u * kLzWarps;
                vp[u] = (t < nl) ? vslice(loc ? lt[t] : t) : wv;
            }
            const int nu = min(NU, (nl - t0) / kLzWarps + 1);   // vectors of this warp in this round (warp-uniform)
            if constexpr (kComp) {   // each 16-byte group's four products, then exactly into the pair
                PA acc[NU];
#pragma unroll
                for (int u = 0; u < NU; ++u) acc[u] = PS::zero();
#pragma unroll UNR
                for (int q = lane; q < nv; q += 32) {
                    VT wq[VW];
                    load16g<VT>(wv + q * VW, wq);
                    VT x[NU][VW];   // all loads first (vectors beyond the pass read w: valid, unused)
#pragma unroll
                    for (int u = 0; u < NU; ++u) load16g<VT>(vp[u] + q * VW, x[u]);
#pragma unroll
                    for (int u = 0; u < NU; ++u)
                        if (u < nu) {
                            CT g = (CT)0;
#pragma unroll
                            for (int e = 0; e < VW; ++e) g += x[u][e] * wq[e];
                            PS::add(acc[u], g);
                        }
                }
                const PA r = warp_sums<NU>(acc, lane);
                const int u = lane >> LS;
                if ((lane & ((1 << LS) - 1)) == 0 && u < nu) Sum::put(Ap + t0 + u * kLzWarps, r);
            } else {
                CT acc[NU];
#pragma unroll
                for (int u = 0; u < NU; ++u) acc[u] = (CT)0;
#pragma unroll UNR
                for (int q = lane; q < nv; q += 32) {
                    VT wq[VW];
                    load16g<VT>(wv + q * VW, wq);
                    VT x[NU][VW];   // all loads first (vectors beyond the pass read w: valid, unused)
#pragma unroll
                    for (int u = 0; u < NU; ++u) load16g<VT>(vp[u] + q * VW, x[u]);
#pragma unroll
                    for (int u = 0; u < NU; ++u)
                        if (u < nu)
#pragma unroll
                            for (int e = 0; e < VW; ++e) acc[u] += x[u][e] * wq[e];
                }
                const CT r = warp_sums<NU>(acc, lane);   // lane partials combined in CT
                const int u = lane >> LS;
                if ((lane & ((1 << LS) - 1)) == 0 && u < nu) Sum::put(Ap + t0 + u * kLzWarps, Sum::from_ct(r));
            }
        }
        cluster.sync();   // the partials of every CTA (also a barrier of this CTA's threads)
        for (int t = tid; t <= nl; t += kLzThreads) {   // (b2) totals over the cluster
            const ST s = cluster_sum_st(Ap, t);
            if constexpr (sizeof(CT) == 4) {
                cf[t] = s.h + s.l;   // the pair rounded once, as through FP64; no FP64 instruction
                if (t == nl) c[t] = Sum::value(s);
            } else {
                c[t] = s;
                cf[t] = (CT)s;
            }
        }
        __syncthreads();
    };

    // (b1') The pass of a recurrence step: w = E v_{j-1} minus its known components, so
    // the full sweep's coefficients c_t = <v_t|w> are rounding-sized and the scalars of
    // the swept vector w' = w - sum_t c_t v_t follow from sums over w to first order in c
    // (the neglected terms are O(|c|^2)):
    //   |w'|^2 = |w|^2 - sum c_t^2,   <w'|E|w'> = <w|E|w> - 2 sum c_t d_t   (d_t = <v_t|E w>),
    //   <M_d|w'> = <M_d|w> - sum c_t <M_d|v_t>,   <v_s|E|w'> = d_s - sum c_t <v_s|E|v_t>,
    // with <M_d|v_t> and <v_s|E|v_t> the stored rows' m and (alpha, beta, g).  One cluster
    // reduction then serves the step: this pass sums, per CTA, <v_t|w> and <v_t|E w> for
    // every stored vector, the same for w and E w (|w|^2, <w|E|w>, |E w|^2) and <M_d|w>,
    // eight vectors per warp at a time as in dots_pass.
    auto dots_fused = [&](int nl) {
        double *Ap = A + (size_t)dpar * apn;
        dpar ^= 1;
        const VT *wv = reinterpret_cast<const VT *>(w);
        const VT *ev = reinterpret_cast<const VT *>(ew);
        constexpr int NU = sizeof(CT) == 4 ? 8 : 4;
        constexpr int LS2 = sizeof(CT) == 4 ? 1 : 2;   // lane L holds the total of value L >> LS2 of 2 NU
        constexpr int UNR = sizeof(CT) == 4 ? 1 : 2;
        const int nit = nl + 2;   // stored vectors, w, E w
        for (int t0 = warp; t0 < nit; t0 += NU * kLzWarps) {
            const VT *vp[NU];
#pragma unroll
            for (int u = 0; u < NU; ++u) {
                const int t = t0 + u * kLzWarps;
                vp[u] = (t < nl) ? vslice(t) : (t == nl ? wv : ev);
            }
            const int nu = min(NU, (nit - 1 - t0) / kLzWarps + 1);
            PA acc[2 * NU];
#pragma unroll
            for (int u = 0; u < 2 * NU; ++u) acc[u] = PS::zero();
#pragma unroll UNR
            for (int q = lane; q < nv; q += 32) {
                VT wq[VW], eq[VW];
                load16g<VT>(wv + q * VW, wq);
                load16g<VT>(ev + q * VW, eq);
                VT x[NU][VW];   // all loads first (items beyond the pass read E w: valid, unused)
#pragma unroll
                for (int u = 0; u < NU; ++u) load16g<VT>(vp[u] + q * VW, x[u]);
#pragma unroll
                for (int u = 0; u < NU; ++u)
                    if (u < nu) {
                        if constexpr (kComp) {
                            CT g = (CT)0, h = (CT)0;
#pragma unroll
                            for (int e = 0; e < VW; ++e) { g += x[u][e] * wq[e]; h += x[u][e] * eq[e]; }
                            PS::add(acc[u], g);
                            PS::add(acc[NU + u], h);
                        } else {
#pragma unroll
                            for (int e = 0; e < VW; ++e) {
                                acc[u] += x[u][e] * wq[e];
                                acc[NU + u] += x[u][e] * eq[e];
                            }
                        }
                    }
            }
            const PA r = warp_sums<2 * NU>(acc, lane);
            const int vi = lane >> LS2, u = vi % NU, kind = vi / NU;
            if ((lane & ((1 << LS2) - 1)) == 0 && u < nu) {
                if constexpr (kComp) Sum::put(Ap + 2 * (t0 + u * kLzWarps) + kind, r);
                else Sum::put(Ap + 2 * (t0 + u * kLzWarps) + kind, Sum::from_ct(r));
            }
        }
        if (warp < D) {   // <M_d|w>, a warp per coupling vector (this CTA's slice: in Msl, or read from M)
            const int d = warp;
            PA a = PS::zero();
            for (int q = lane; q < nv; q += 32) {
                VT wq[VW], m[VW];
                load16g<VT>(wv + q * VW, wq);
                if (Msl) {
                    load16g<VT>(reinterpret_cast<const VT *>(Msl + (size_t)d * S) + q * VW, m);
                } else {
#pragma unroll
                    for (int e = 0; e < VW; ++e) {
                        const int i = q * VW + e;
                        m[e] = (i < ns) ? (VT)Mc[(size_t)d * N + i0 + i] : (VT)0;
                    }
                }
                if constexpr (kComp) {
                    CT g = (CT)0;
#pragma unroll
                    for (int e = 0; e < VW; ++e) g += m[e] * wq[e];
                    PS::add(a, g);
                } else {
#pragma unroll
                    for (int e = 0; e < VW; ++e) a += m[e] * wq[e];
                }
            }
            const ST r = PS::finish(a);
            if (lane == 0) Sum::put(Ap + 2 * nit + d, r);
        }
        cluster.sync();   // the partials of every CTA (also a barrier of this CTA's threads)
        const int nval = 2 * nit + D;
        for (int t = tid; t < nval; t += kLzThreads) {
            const ST x = cluster_sum_st(Ap, t);
            if (t < 2 * nl) {
                if ((t & 1) == 0) {
                    if constexpr (sizeof(CT) == 4) cf[t >> 1] = x.h + x.l;
                    else cf[t >> 1] = (CT)x;
                } else {
                    Sum::put(dt + (t >> 1), x);   // kept as the sum's pair: no FP64 instruction here
                }
            } else if (t == 2 * nl) {
                if constexpr (kFused) fscd[0] = x; else fsc[0] = Sum::value(x);   // |w|^2
            } else if (t == 2 * nl + 1) {
                if constexpr (kFused) fscd[1] = x; else fsc[1] = Sum::value(x);   // <w|E|w>
            } else if (t == 2 * nl + 3) {
                if constexpr (kFused) fscd[2] = x; else fsc[2] = Sum::value(x);   // |E w|^2
            } else if (t >= 2 * nit) {
                if constexpr (kFused) fscd[3 + (t - 2 * nit)] = x; else fsc[3 + (t - 2 * nit)] = Sum::value(x);   // <M_d|w>
            }
        }
        __syncthreads();
    };

    // <v_s|E|v_t> for s the last vector of earlier chain q, from the stored rows: alpha of
    // row(s) at t = s, its beta for the chain's previous vector, its g for the earlier
    // chains' last vectors, and each later row's g_q (read through L2: rank 0 wrote the
    // rows, the cluster barriers since make them visible).
    auto t_entry = [&](int sl, int q, int t) -> double {
        const int srow = s_last[q];
        const double *rs = C.out + (size_t)srow * NT;
        if (t == sl) return __ldcg(rs);
        if (t < sl) {
            if (slotrow[t] == srow - 1 && srow - 1 >= s_start[q]) return __ldcg(rs + 1);
            for (int p = 0; p < q; ++p)
                if (t == lslot[p]) return __ldcg(rs + 2 + p);
            return 0.0;
        }
        return __ldcg(C.out + (size_t)slotrow[t] * NT + 2 + q);
    };
    // The scalars of w' into tot[] by the corrections above: quantity 0 sum c_t^2, 1
    // sum c_t d_t, 2 + d sum c_t <M_d|v_t>, 2 + D + q sum c_t <v_s(q)|E|v_t>, a warp each
    // (warp 0 takes quantity 0, so thread 0 holds |w'|^2 when it decides).
    auto fused_scalars = [&](int nl, int nq) {
        const int nqty = 2 + D + nq;
        for (int qi = warp; qi < nqty; qi += kLzWarps) {
            CT a = (CT)0;
            for (int t = lane; t < nl; t += 32) {
                const CT ct = cf[t];
                CT term = (CT)0;
                if (qi == 0) term = ct * ct;
                else if (qi == 1) {
                    const ST x = Sum::get(dt + t);
                    if constexpr (sizeof(CT) == 4) term = ct * (x.h + x.l);
                    else term = ct * (CT)x;
                }
                else if (qi < 2 + D) term = ct * (CT)__ldcg(C.out + (size_t)slotrow[t] * NT + C.nden_out + (qi - 2));
                else {
                    const int q = qi - 2 - D, sl = lslot[q];
                    if (sl >= 0) term = ct * (CT)t_entry(sl, q, t);
                }
                a += term;
            }
            a = warp_sum_ct(a);
            if constexpr (kFused) {   // into totd, in double-float
                if (lane == 0) {
                    const dfm::df xa{-(float)a, 0.0f};
                    if (qi == 0) totd[0] = dfm::add(fscd[0], xa);
                    else if (qi == 1) totd[1] = dfm::add(fscd[1], dfm::df{-2.0f * (float)a, 0.0f});
                    else if (qi < 2 + D) totd[qi] = dfm::add(fscd[3 + (qi - 2)], xa);
                    else {
                        const int q = qi - 2 - D, sl = lslot[q];
                        totd[2 + D + q] = (sl >= 0) ? dfm::add(Sum::get(dt + sl), xa) : dfm::df{0.0f, 0.0f};
                    }
                }
            } else if (lane == 0) {
                const double x = (double)a;
                if (qi == 0) tot[0] = fsc[0] - x;
                else if (qi == 1) tot[1] = fsc[1] - 2.0 * x;
                else if (qi < 2 + D) tot[qi] = fsc[3 + (qi - 2)] - x;
                else {
                    const int q = qi - 2 - D, sl = lslot[q];
                    tot[2 + D + q] = (sl >= 0) ? Sum::value(Sum::get(dt + sl)) - x : 0.0;
                }
            }
        }
        if (tid == 0) {   // |E w'|^2 ~ |E w|^2: only a threshold's scale
            if constexpr (kFused) totd[2 + D + nq] = fscd[2]; else tot[2 + D + nq] = fsc[2];
        }
    };

    // (b3) w -= sum_t cf_t v_t over the pass's vectors: 16-byte vectors, eight rows in
    // flight.  Each thread updates the 16-byte groups q = tid, tid + kLzThreads, ...
    // sum_t cf_t v_t over the pass's vectors for the 16-byte group at qo
    auto group_sum = [&](bool loc, int nl, int qo, CT *acc) {
#pragma unroll
        for (int u = 0; u < VW; ++u) acc[u] = 0;
        int t = 0;
        for (; t + 7 < nl; t += 8) {
            VT x[8][VW];
#pragma unroll
            for (int r = 0; r < 8; ++r) load16g<VT>(vslice(loc ? lt[t + r] : t + r) + qo, x[r]);
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const CT cr = cf[t + r];
#pragma unroll
                for (int u = 0; u < VW; ++u) acc[u] += cr * x[r][u];
            }
        }
        for (; t + 3 < nl; t += 4) {
            VT x0[VW], x1[VW], x2[VW], x3[VW];
            load16g<VT>(vslice(loc ? lt[t] : t) + qo, x0);
            load16g<VT>(vslice(loc ? lt[t + 1] : t + 1) + qo, x1);
            load16g<VT>(vslice(loc ? lt[t + 2] : t + 2) + qo, x2);
            load16g<VT>(vslice(loc ? lt[t + 3] : t + 3) + qo, x3);
            const CT c0 = cf[t], c1 = cf[t + 1], c2 = cf[t + 2], c3 = cf[t + 3];
#pragma unroll
            for (int u = 0; u < VW; ++u) acc[u] += c0 * x0[u] + c1 * x1[u] + c2 * x2[u] + c3 * x3[u];
        }
        for (; t < nl; ++t) {
            VT x0[VW];
            load16g<VT>(vslice(loc ? lt[t] : t) + qo, x0);
            const CT c0 = cf[t];
#pragma unroll
            for (int u = 0; u < VW; ++u) acc[u] += c0 * x0[u];
        }
    };
    auto update_pass = [&](bool loc, int nl) {
        for (int q = tid; q < nv; q += kLzThreads) {
            CT acc[VW];
            group_sum(loc, nl, q * VW, acc);
#pragma unroll
            for (int u = 0; u < VW; ++u) w[q * VW + u] -= acc[u];
        }
    };

    // After a full sweep's update: the scalars of step (c) of the updated w
    // (source/BcDor-Lanczos.cpp:180-214): |w|^2, alpha = <w|E|w>, m_d = <M_d|w> and, for
    // each earlier pivot q, g_q = <v_last(q)|E|w>, and |E w|^2, as partials in
    // red[warp][slot], slots [|w|^2, alpha, m_0.., g_0.., |E w|^2].  Each thread reads back
    // only the groups it updated, so no barrier separates this from the update.
    auto scalar_partials = [&](int nq) {
        PA pn = PS::zero(), sa = PS::zero(), se = PS::zero(), sm_[8], sg[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            sm_[q] = PS::zero();
            sg[q] = PS::zero();
        }
        for (int q = tid; q < nv; q += kLzThreads) {
            const int qo = q * VW;
            {
                // the groups of the first four earlier chains' last vectors, loaded together
                // (more earlier chains read theirs element by element)
                VT lv[4][VW];
                bool lok[8];
#pragma unroll
                for (int g = 0; g < 8; ++g) {
                    lok[g] = g < nq && lslot[g] >= 0;
                    if (g < 4 && lok[g]) load16g<VT>(vslice(lslot[g]) + qo, lv[g]);
                }
#pragma unroll
                for (int u = 0; u < VW; ++u) {
                    const int i = qo + u;
                    const CT wi = w[i];
                    PS::add(pn, wi * wi);
                    if (i < ns) {
                        const CT e = Es[i];
                        PS::add(sa, e * wi * wi);
                        PS::add(se, e * e * wi * wi);
#pragma unroll
                        for (int d = 0; d < 8; ++d)
                            if (d < D) PS::add(sm_[d], (Msl ? Msl[d * S + i] : Mc[(size_t)d * N + i0 + i]) * wi);
#pragma unroll
                        for (int g = 0; g < 8; ++g)
                            if (lok[g]) PS::add(sg[g], e * (CT)(g < 4 ? lv[g & 3][u] : vslice(lslot[g])[i]) * wi);
                    }
                }
            }
        }
        // the 19 sums of the warp at once (values 0 |w|^2, 1 alpha, 2 |E w|^2, 3 + d m_d,
        // 11 + q g_q, the rest zero); lane L stores value L into its slot when in use
        PA v[32];
        v[0] = pn; v[1] = sa; v[2] = se;
#pragma unroll
        for (int d = 0; d < 8; ++d) { v[3 + d] = sm_[d]; v[11 + d] = sg[d]; }
#pragma unroll
        for (int q = 19; q < 32; ++q) v[q] = PS::zero();
        const PA x = warp_sums<32>(v, lane);
        int slot = -1;
        if (lane == 0) slot = 0;
        else if (lane == 1) slot = 1;
        else if (lane == 2) slot = 2 + D + nq;
        else if (lane < 11) slot = (lane - 3 < D) ? 2 + (lane - 3) : -1;
        else if (lane < 19) slot = (lane - 11 < nq) ? 2 + D + (lane - 11) : -1;
        if (slot >= 0) {
            if constexpr (kComp) Sum::put(red + warp * kMaxScal + slot, x);
            else Sum::put(red + warp * kMaxScal + slot, Sum::from_ct(x));
        }
    };
    // The cluster totals of the scalars into tot[0 .. 3 + D + nq): the warps' partials
    // summed per CTA into Bs, then over the cluster (no barrier after: the caller's
    // decision follows).
    auto scalar_reduce = [&](int nq) {
        const int nsc = 3 + D + nq;   // |w|^2, <w|E|w>, m_d, g_q, |E w|^2
        __syncthreads();
        if (tid < nsc) {
            ST x[kLzWarps];
#pragma unroll
            for (int q = 0; q < kLzWarps; ++q) x[q] = Sum::get(red + q * kMaxScal + tid);
            Sum::put(Bs + tid, tree_sum8<Sum>(x));
        }
        cluster.sync();
        if (tid < nsc) {
            const ST x = cluster_sum_st(Bs, tid);
            tot[tid] = Sum::value(x);
            if constexpr (kFused) totd[tid] = x;
        }
    };

    int k = -1;           // current pivot chain
    int extra = 0;        // sweeps beyond the first
    bool prow_ok = false; // prow holds row j - 1, a vector this chain built (identical in every CTA)
    for (int j = 0; j < L; ++j) {
        const bool newv = (k + 1 < C.n_used) && (j == s_start[k + 1]);
        if (newv) { ++k; tail = false; }
        __syncthreads();
        if (tail) {
            // The rest of this pivot chain is deflated: rows j .. jend-1 take directions
            // dcur, dcur + 1, ... (the last group's energy once none is left), as
            // deflated_row would one at a time; each thread places rows by binary search
            // in the cumulative counts.
            const int jend = (k + 1 < C.n_used) ? min(L, s_start[k + 1]) : L;
            const int R = jend - j;
            for (int r = tid; r < R; r += kLzThreads) {
                const int d = dcur + r;
                const double a = (d < dtot) ? C.gE[group_of(d)] : C.gE[Qg - 1];
                if (rank == 0) {
                    double *row = C.out + (size_t)(j + r) * NT;
                    for (int e = 0; e < NT; ++e) row[e] = 0.0;
                    row[0] = a;
                }
                rowslot[j + r] = -1;
            }
            dcur = min(dcur + R, dtot);
            ndefl += R;
            j = jend - 1;
            continue;
        }
        const int nq = k;   // earlier pivot chains
        if (tid < nq) lslot[tid] = rowslot[s_last[tid]];
        // A continuing step's E v_{j-1} has large components only on v_{j-1}, v_{j-2} and
        // the last vector of every earlier chain, with the coefficients row j - 1 already
        // holds: <v_{j-1}|E|v_{j-1}> = alpha_{j-1}, <v_{j-2}|E|v_{j-1}> = beta_{j-1} (the
        // previous chain's g on a chain's first row), <v_last(q)|E|v_{j-1}> = g_q.  After a
        // built row the step removes those with the row's values (the three-term
        // recurrence and its fishbone terms), so no reduction is needed before the full
        // sweep; after anything else it measures them (the local pass below).
        const bool rec = !newv && j > 0 && prow_ok;
        // (a) w = M.p  or  w = v_{j-1} * E   (source/BcDor-Lanczos.cpp:137-150)
        if (newv) {
            const double *p = C.piv + (size_t)k * D;
            for (int i = tid; i < S; i += kLzThreads) {
                double s = 0.0;
                if (i < ns)
                    for (int d = 0; d < D; ++d) s = __dadd_rn(s, __dmul_rn(C.M[(size_t)d * N + i0 + i], p[d]));
                w[i] = (CT)s;
            }
        } else if (rec) {
            // v_{j-1}, v_{j-2} and the earlier chains' last vectors with their coefficients
            // (lt, lcf, s_nl), listed by warp 0 when it wrote row j - 1
            const int nl0 = s_nl;
            const VT *vp0 = vslice(lt[0]);
            for (int q = tid; q < nv; q += kLzThreads) {
                const int qo = q * VW;
                VT x0[VW];
                load16g<VT>(vp0 + qo, x0);
                CT x[VW];
#pragma unroll
                for (int u = 0; u < VW; ++u) x[u] = (CT)x0[u] * Es[qo + u];
#pragma unroll 4
                for (int t = 0; t < nl0; ++t) {
                    VT y[VW];
                    load16g<VT>(vslice(lt[t]) + qo, y);
                    const CT ct = lcf[t];
#pragma unroll
                    for (int u = 0; u < VW; ++u) x[u] -= ct * (CT)y[u];
                }
#pragma unroll
                for (int u = 0; u < VW; ++u) {
                    w[qo + u] = x[u];
                    if constexpr (kFused) ew[qo + u] = Es[qo + u] * x[u];
                }
            }
        } else {
            const VT *vp = vslice(rowslot[j - 1]);
            for (int q = tid; q < nv; q += kLzThreads) {
                const int qo = q * VW;
                VT x0[VW];
                load16g<VT>(vp + qo, x0);
#pragma unroll
                for (int u = 0; u < VW; ++u) w[qo + u] = (CT)x0[u] * Es[qo + u];
            }
        }
        bool injected = false;     // w replaced by a pseudo-random restart vector
        bool upd = false;          // the kept sweep's update is still to be applied (with the normalisation)
        bool done = false;         // step finished by an untouched-pole unit vector
        for (int attempt = 0; attempt < 2 && !done; ++attempt) {
            int nfull = 0;
            int fl = 0;            // thread 0's decision after the last sweep (s_flag)
            upd = false;
            // A continuing chain's w = E v_{j-1} has large components only on v_{j-1}, v_{j-2}
            // and the last vector of every earlier chain (the fishbone couplings); everything
            // else is rounding.  The first pass projects out just those few vectors, then
            // full sweeps follow (at least one), each repeated under the DGKS criterion.
            bool local = !newv && attempt == 0 && j > 0 && !rec;
            if (local && tid == 0) {   // slots of v_{j-1}, v_{j-2} and the earlier chains' last vectors
                int n = 0;
                lt[n++] = rowslot[j - 1];
                if (j >= 2 && rowslot[j - 2] >= 0) lt[n++] = rowslot[j - 2];
                for (int q = 0; q < k; ++q)
                    if (s_last[q] < j - 2 && rowslot[s_last[q]] >= 0) lt[n++] = rowslot[s_last[q]];
                s_nl = n;
            }
            __syncthreads();
            int nl = local ? s_nl : nvec;
            // With FP32 vectors a recurrence step's first sweep takes the one-reduction pass
            // (dots_fused); its scalars fall back to the exact pass when the sweep removed
            // more than 1 % of |w|^2 or the step is not kept (the corrections are first order
            // in the sweep).  With FP64 vectors the pass's second product per element would
            // cost more FP64-pipe time than the reduction it saves.
            bool fused = kFused && rec && attempt == 0;
            if (fused) dots_fused(nl);
            else dots_pass(local, nl);
            // |w|^2 before any projection: E v_{j-1}'s, from row j - 1's sums, after the recurrence
            // (FP32 vectors: a recurrence step's two are read in double-float by the fused
            // decision, and converted where the exact pass follows it)
            const bool wf_df = kFused && rec && attempt == 0;
            const double wn2_first0 = (rec && attempt == 0) ? (kFused ? 0.0 : s_e2v) : c[nl];
            double wn2_before = fused ? (kFused ? 0.0 : fsc[0]) : c[nl];
            for (;;) {
                if (fused) {   // the scalars from the pass, before the sweep's update
                    fused = false;
                    fused_scalars(nl, nq);
                    if (tid == 0) {   // in double-float: comparisons, 1/|w| by Newton's iteration
                        const dfm::df x2 = totd[0], wb = fscd[0], wf = s_e2vd;
                        int f = 4;   // the exact scalars of w'
                        if (x2.h > 1e-36f && x2.h < 1e36f && !df_lt(x2, dfm::mul(c099d, wb)) &&
                            !df_lt(x2, dfm::mul(eta2d, wb)) && !df_le(x2, dfm::mul(thr_exhd, wf)) &&
                            !df_le(x2, dfm::mul(taud, wf))) {
                            f = 0;   // keep: normalise
                            const dfm::df r = dfm::rsqrt(x2, 2);
                            s_rd = r;
                            s_xbd = dfm::mul(x2, r);
                            s_ixbf = __fadd_rn(r.h, r.l);
                        }
                        s_flag = f;
                    }
                    __syncthreads();
                    if (s_flag == 0) {   // kept: the sweep's update is applied with the normalisation
                        fl = 0;
                        ++nfull;
                        upd = true;
                        break;
                    }
                    if constexpr (kFused) wn2_before = dfm::to_double(fscd[0]);
                    update_pass(false, nl);   // the exact scalars of the swept vector follow
                }
                else {
                    update_pass(local, nl);
                    if (local) {   // the full sweep's dot products follow the local update directly
                        local = false;
                        nl = nvec;
                        __syncthreads();
                        dots_pass(false, nl);
                        wn2_before = c[nl];
                        continue;
                    }
                }
                scalar_partials(nq);
                scalar_reduce(nq);
                // Thread 0 holds |w|^2 (tot[0]) and takes the step's decision alone (FP64
                // comparisons in one thread instead of every warp), with 1/|w| when the
                // vector is kept; the barrier below publishes it with the totals.
                if (tid == 0) {
                    const double x2 = tot[0];
                    const double wn2_first = wf_df ? dfm::to_double(s_e2vd) : wn2_first0;
                    int f;
                    if (nvec > 0 && nfull + 1 < 4 && x2 < eta2 * wn2_before) f = 1;   // another full sweep
                    else if (attempt == 0 && !contaminated && (x2 <= thr_exh * wn2_first || x2 == 0.0) && next_slot())
                        f = 2;   // this chain's Krylov space is exhausted
                    else if (attempt > 0 || !(x2 <= tau * wn2_first || x2 == 0.0)) {
                        f = 0;   // keep: normalise
                        const double r = rsqrt_newton(x2);   // 1/sqrt(n2) to a few ulp
                        s_xb = x2 * r;
                        s_ixb = r;
                        s_ixbf = (CT)r;
                        if constexpr (kFused) { s_rd = dfm::from_double(r); s_xbd = dfm::from_double(x2 * r); }
                    } else {
                        f = 3;   // the reachable subspace is exhausted: restart
                    }
                    s_flag = f;
                }
                __syncthreads();
                fl = s_flag;
                // another full sweep while this one removed more than half of the squared norm
                if (nfull++ > 0) ++extra;
                if (fl == 1) {
                    dots_pass(false, nl);
                    wn2_before = c[nl];
                    continue;
                }
                break;
            }
            if (fl == 2) {
                deflated_row(j);   // this chain's Krylov space is exhausted
                tail = true;
                done = true;
                prow_ok = false;
                break;
            }
            if (fl == 0) break;
            contaminated = true;
            // (c0) exhausted reachable subspace: an untouched pole's unit vector if one is left,
            // else a pseudo-random vector swept orthogonal to the basis in the second attempt
            int kl = INT_MAX;
            for (int i = tid; i < ns; i += kLzThreads) if (!touched[i]) { kl = i0 + i; break; }
            for (int o = 16; o > 0; o >>= 1) kl = min(kl, __shfl_xor_sync(0xffffffffu, kl, o));
            __shared__ int wmin[kLzWarps];
            if (lane == 0) wmin[warp] = kl;
            __syncthreads();
            if (tid == 0) {
                int m = INT_MAX;
                for (int q = 0; q < kLzWarps; ++q) m = min(m, wmin[q]);
                s_kmin = m;
            }
            cluster.sync();
            int kmin = INT_MAX;
            for (int r = 0; r < CL; ++r) kmin = min(kmin, *cluster.map_shared_rank(&s_kmin, r));
            if (rank == 0 && tid == 0) atomicAdd(&C.stat[1], 1);
            if (kmin != INT_MAX) {
                VT *vj = V + (size_t)nvec * C.ld + i0;
                VT *vc = nvec < ccap ? cache + (size_t)nvec * S : (hasring ? ring + (size_t)(nvec & 1) * S : nullptr);
                for (int i = tid; i < S; i += kLzThreads) {
                    const bool hit = (i0 + i == kmin);
                    vj[i] = hit ? (VT)1 : (VT)0;
                    if (vc) vc[i] = hit ? (VT)1 : (VT)0;
                    if (hit) touched[i] = 1;
                }
                if (rank == 0 && tid == 0) {
                    double *row = C.out + (size_t)j * NT;
                    for (int q = 0; q < NT; ++q) row[q] = 0.0;
                    row[0] = C.E[kmin];
                    for (int d = 0; d < D; ++d) row[C.nden_out + d] = C.M[(size_t)d * N + kmin];
                }
                if (tid == 0) { rowslot[j] = nvec; slotrow[nvec] = j; }
                ++nvec;
                done = true;
                prow_ok = false;
            } else {
                for (int i = tid; i < S; i += kLzThreads) w[i] = (i < ns) ? (CT)restart_value(i0 + i, j) : (CT)0;
                injected = true;
            }
            cluster.sync();   // peers have read s_kmin before it can change again
        }
        if (done) continue;
        // (d) normalise, store, write the output row (source/BcDor-Lanczos.cpp:198-216);
        // the scalars were formed once, with the decision, by Newton's iteration instead
        // of FP64 division and square root (long FP64 chains)
        const double xb = s_xb, ixb = s_ixb;
        VT *vj = V + (size_t)nvec * C.ld + i0;
        {
            VT *vc = nvec < ccap ? cache + (size_t)nvec * S : (hasring ? ring + (size_t)(nvec & 1) * S : nullptr);
            const CT inv = s_ixbf;
            for (int q = tid; q < nv; q += kLzThreads) {
                const int qo = q * VW;
                CT acc[VW] = {};
                if (upd) group_sum(false, nvec, qo, acc);
                VT v[VW];
#pragma unroll
                for (int u = 0; u < VW; ++u) {
                    v[u] = (VT)((w[qo + u] - acc[u]) * inv);
                    touched[qo + u] |= (v[u] != (VT)0);
                }
                store16g<VT>(vj + qo, v);
                if (vc) store16g<VT>(vc + qo, v);
            }
        }
        if constexpr (kFused) {   // the row in double-float, FP64 only for the stored copy
            if (tid < NT) {
                const dfm::df r = s_rd, z{0.0f, 0.0f};
                dfm::df x = z;
                if (tid == 0) x = dfm::mul(dfm::mul(totd[1], r), r);   // <w|E|w> / |w|^2
                else if (tid == 1) x = injected ? z : s_xbd;          // a restart vector has no coupling to v_{j-1}
                else if (tid < 2 + k) x = dfm::mul(totd[2 + D + (tid - 2)], r);
                else if (tid >= C.nden_out && tid < C.nden_out + D) x = dfm::mul(totd[2 + (tid - C.nden_out)], r);
                if (newv && tid == 1) x = (k >= 1) ? dfm::mul(totd[2 + D + (k - 1)], r) : x;
                if (!(tid < 2 + k || tid >= C.nden_out)) x = z;
                prowf[tid] = __fadd_rn(x.h, x.l);
                if (rank == 0) C.out[(size_t)j * NT + tid] = dfm::to_double(x);
            }
            if (tid == 0) {
                rowslot[j] = nvec;
                slotrow[nvec] = j;
                s_e2vd = dfm::mul(dfm::mul(totd[2 + D + k], s_rd), s_rd);   // |E v_j|^2
            }
        } else {
            if (tid < NT) {   // one output element per thread; every CTA keeps the row for the next step
                double x = 0.0;
                if (tid == 0) x = tot[1] * ixb * ixb;   // <w|E|w> / |w|^2
                else if (tid == 1) x = injected ? 0.0 : xb;   // a restart vector has no coupling to v_{j-1}
                else if (tid < 2 + k) x = tot[2 + D + (tid - 2)] * ixb;
                else if (tid >= C.nden_out && tid < C.nden_out + D) x = tot[2 + (tid - C.nden_out)] * ixb;
                if (newv && tid == 1) x = (k >= 1) ? tot[2 + D + (k - 1)] * ixb : x;
                if (!(tid < 2 + k || tid >= C.nden_out)) x = 0.0;
                prow[tid] = x;
                if (rank == 0) C.out[(size_t)j * NT + tid] = x;
            }
            if (tid == 0) {
                rowslot[j] = nvec;
                slotrow[nvec] = j;
                s_e2v = tot[2 + D + k] * ixb * ixb;   // |E v_j|^2
            }
        }
        // The next step's recurrence, when it continues this chain from this row: its
        // vectors v_j, v_{j-1} and the earlier chains' last vectors with the row's alpha,
        // beta and g as coefficients, listed here by warp 0 (which wrote the row), so the
        // next step needs no barrier of its own before it forms w.
        if (warp == 0) {
            __syncwarp();
            const bool next_newv = (k + 1 < C.n_used) && (j + 1 == s_start[k + 1]);
            if (tid == 0 && !injected && !next_newv) {
                auto pr = [&](int q) -> CT { if constexpr (kFused) return prowf[q]; else return (CT)prow[q]; };
                int n = 0;
                lt[n] = nvec; lcf[n++] = pr(0);
                if (j >= 1 && rowslot[j - 1] >= 0) { lt[n] = rowslot[j - 1]; lcf[n++] = pr(1); }
                for (int q = 0; q < k; ++q)
                    if (s_last[q] < j - 1 && rowslot[s_last[q]] >= 0) {
                        lt[n] = rowslot[s_last[q]];
                        lcf[n++] = pr(2 + q);
                    }
                s_nl = n;
            }
        }
        prow_ok = !injected;
        ++nvec;
        // (the barrier at the top of the next step orders these writes before their reads)
    }
    if (rank == 0 && tid == 0) { atomicAdd(&C.stat[0], extra); atomicAdd(&C.stat[2], ndefl); }
    __syncthreads();
    if (rank == 0 && C.rowslot)
        for (int q = tid; q < L; q += kLzThreads) C.rowslot[q] = rowslot[q];
    cluster.sync();  // no CTA leaves while peers may still read its shared memory
}

size_t lanczos_smem_bytes(int S, int rmax, bool global_slices) {
    // sized for FP64 vectors (E, w and E w as doubles); FP32 vectors use less
    const size_t rmax2 = ((size_t)rmax + 1) & ~(size_t)1;
    const size_t rq = (size_t)(rmax + 3) / 4 * 4;
    const size_t fixed = sizeof(double) * (2 * (size_t)lz_partials_per_pass(rmax) + 2 * rmax2 + rq + kMaxScal +
                                           (size_t)kLzWarps * kMaxScal) +
                         sizeof(int) * 2 * rq + 16;
    return global_slices ? fixed : fixed + sizeof(double) * 3 * (size_t)S + (size_t)S;
}

template <typename VT, bool G>
static cudaError_t launch_lz(const cudaLaunchConfig_t &cfg, int cluster, const LzChain *d_chains, int nchains, int rmax,
                             double eta2) {
    const int smem_bytes = (int)cfg.dynamicSmemBytes;
    cudaError_t e = allow_dynamic_smem((const void *)k_lanczos<VT, G>);
    if (e == cudaSuccess && cluster > 8)
        e = cudaFuncSetAttribute(k_lanczos<VT, G>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, k_lanczos<VT, G>, d_chains, nchains, rmax, eta2, smem_bytes);
}

cudaError_t launch_lanczos(const LzChain *d_chains, int nchains, int S_max, int rmax, bool fp32, int cluster,
                           double eta, bool global_slices, cudaStream_t st) {
    if (nchains <= 0) return cudaSuccess;
    // what the slices and scalars need, raised to kLzSmemCache so the rest holds the basis cache
    const size_t smem = std::max(lanczos_smem_bytes(S_max, rmax, global_slices), kLzSmemCache);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nchains * cluster, 1, 1);
    cfg.blockDim = dim3(kLzThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const double eta2 = eta * eta;
    if (fp32)
        return global_slices ? launch_lz<float, true>(cfg, cluster, d_chains, nchains, rmax, eta2)
                             : launch_lz<float, false>(cfg, cluster, d_chains, nchains, rmax, eta2);
    return global_slices ? launch_lz<double, true>(cfg, cluster, d_chains, nchains, rmax, eta2)
                         : launch_lz<double, false>(cfg, cluster, d_chains, nchains, rmax, eta2);
}

}  // namespace bd

namespace bd {
__global__ void k_to_float(const double *in, float *out, long long n) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}

cudaError_t launch_to_float(const double *in, float *out, long long n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_to_float<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}
}  // namespace bd

namespace bd {
// Energy groups of one chain's sorted poles: runs of bit-equal E, and for each the
// dimension of its eigenvectors of E orthogonal to every coupling, m_q - rank(M_q), M_q
// the D x m_q couplings of the group's poles.  The rank comes from the Gram matrix
// G_q = M_q M_q^T by pivoted elimination (pivots above 1e-12 of the largest diagonal
// entry).  Three launches:
//   k_lz_gstart  a CTA per chain: the group starts, and the groups of more than
//                kGrpSmall poles cut into Gram pieces of at most kGrpPiece poles;
//   k_lz_gram    the pieces' partial Gram matrices, spread over the whole GPU (degenerate
//                shells give a chain a few groups of thousands of poles, and their FP64
//                sums on one SM would take tens of microseconds);
//   k_lz_groups  a CTA per chain: one-pole groups, the small groups (a warp each), the
//                sums of the pieces, the eliminations and the cumulative counts.
constexpr int kGrpThreads = 256;
constexpr int kGstartThreads = 512;
constexpr int kGramThreads = 128;
constexpr int kGramCtas = 608;   // four per SM

// Block-wide exclusive scan of one int per thread (T threads, a multiple of 32): returns
// the thread's exclusive prefix and sets total.  ws holds T / 32 ints.
template <int T>
__device__ __forceinline__ int block_excl_scan(int x, int &total, int *ws) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) ws[warp] = v;
    __syncthreads();
    int off = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < T / 32; ++w) {
        const int s = ws[w];
        if (w < warp) off += s;
        tot += s;
    }
    __syncthreads();   // ws is free for the next scan
    total = tot;
    return off + v - x;
}

// Group starts (gInfo[1 + q], with gE[q] = the group's energy, gInfo[0] = the number of
// groups) and the Gram pieces of the groups of more than kGrpSmall poles.  Each thread
// flags eight consecutive poles per pass.
__global__ void __launch_bounds__(kGstartThreads) k_lz_gstart(const LzChain *chains, int nchains) {
    const int cid = blockIdx.x;
    if (cid >= nchains) return;
    const LzChain C = chains[cid];
    if (!C.gE) return;
    double *gE = const_cast<double *>(C.gE);
    int *gInfo = const_cast<int *>(C.gInfo);
    const GrpScratch S = lz_grp_scratch(C.gE, C.N);
    const int N = C.N, tid = threadIdx.x;
    __shared__ int ws[kGstartThreads / 32];
    int base = 0;
    for (int b = 0; b < N; b += 8 * kGstartThreads) {
        const int i0 = b + 8 * tid;
        double e[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const int i = i0 - 1 + k;
            e[k] = (i >= 0 && i < N) ? C.E[i] : 0.0;
        }
        unsigned fl = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int i = i0 + k;
            if (i < N && (i == 0 || e[k + 1] != e[k])) fl |= 1u << k;
        }
        int tot;
        int q = base + block_excl_scan<kGstartThreads>(__popc(fl), tot, ws);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (fl >> k & 1u) {
                gInfo[1 + q] = i0 + k;
                gE[q] = e[k + 1];
                ++q;
            }
        base += tot;
    }
    const int Q = base;
    __syncthreads();   // the starts are read back below
    int pbase = 0;
    for (int b = 0; b < Q; b += kGstartThreads) {
        const int q = b + tid;
        int g0 = 0, m = 0, np = 0;
        if (q < Q) {
            g0 = gInfo[1 + q];
            m = ((q + 1 < Q) ? gInfo[2 + q] : N) - g0;
            np = m > kGrpSmall ? (m + kGrpPiece - 1) / kGrpPiece : 0;
        }
        int tot;
        const int p0 = pbase + block_excl_scan<kGstartThreads>(np, tot, ws);
        if (q < Q) S.first[q] = p0;
        for (int k = 0; k < np; ++k)
            S.list[p0 + k] = make_int4(q, g0 + k * kGrpPiece, min(g0 + m, g0 + (k + 1) * kGrpPiece), 0);
        pbase += tot;
    }
    if (tid == 0) {
        gInfo[0] = Q;
        *S.count = pbase;
    }
}

// One piece's partial Gram matrix (the lower triangle, D(D+1)/2 entries): each thread
// sums its poles' products, each warp's 32 partial sums of an entry are added by one
// lane, and the warps' sums in warp order; the order is fixed, so the sums repeat.
template <int D>
__device__ void gram_piece(const LzChain &C, int4 pc, double *out, double (*red)[kGramEntries][33],
                           double (*wtot)[kGramEntries]) {
    constexpr int P = D * (D + 1) / 2;
    const int N = C.N, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double G[P];
#pragma unroll
    for (int u = 0; u < P; ++u) G[u] = 0.0;
    for (int i = pc.y + tid; i < pc.z; i += kGramThreads) {
        double mv[D];
#pragma unroll
        for (int a = 0; a < D; ++a) mv[a] = C.M[(size_t)a * N + i];
        int u = 0;
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
            for (int b = 0; b <= a; ++b) { G[u] = fma(mv[a], mv[b], G[u]); ++u; }
    }
#pragma unroll
    for (int u = 0; u < P; ++u) red[warp][u][lane] = G[u];
    __syncwarp();
#pragma unroll
    for (int h = 0; h < (P + 31) / 32; ++h) {
        const int u = lane + 32 * h;
        if (u < P) {
            double s = 0.0;
#pragma unroll 8
            for (int k = 0; k < 32; ++k) s += red[warp][u][k];
            wtot[warp][u] = s;
        }
    }
    __syncthreads();
    if (tid < P) {
        double s = wtot[0][tid];
#pragma unroll
        for (int w = 1; w < kGramThreads / 32; ++w) s += wtot[w][tid];
        out[tid] = s;
    }
    __syncthreads();   // red and wtot are reused by the next piece
}

// The pieces of all chains, numbered chain by chain, CTA k taking pieces k, k + grid, ...
__global__ void __launch_bounds__(kGramThreads) k_lz_gram(const LzChain *chains, int nchains) {
    __shared__ double red[kGramThreads / 32][kGramEntries][33];
    __shared__ double wtot[kGramThreads / 32][kGramEntries];
    __shared__ int pre[kGramThreads + 1];
    __shared__ int ws[kGramThreads / 32];
    const int G = gridDim.x;
    int base = 0;
    for (int c0 = 0; c0 < nchains; c0 += kGramThreads) {
        const int c = c0 + threadIdx.x, nc = min(kGramThreads, nchains - c0);
        int cnt = 0;
        if (c < nchains && chains[c].gE) cnt = *lz_grp_scratch(chains[c].gE, chains[c].N).count;
        int tot;
        pre[threadIdx.x] = base + block_excl_scan<kGramThreads>(cnt, tot, ws);
        __syncthreads();
        // the first piece w >= base with w = blockIdx.x (mod G)
        int w = base + (((int)blockIdx.x - base) % G + G) % G;
        for (; w < base + tot; w += G) {
            int lo = 0, hi = nc - 1;   // the last chain whose first piece is <= w
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (pre[mid] <= w) lo = mid; else hi = mid - 1;
            }
            const LzChain &C = chains[c0 + lo];
            const GrpScratch S = lz_grp_scratch(C.gE, C.N);
            const int k = w - pre[lo];
            const int4 pc = S.list[k];
            double *out = S.part + (size_t)k * kGramEntries;
            switch (C.D) {
                case 1: gram_piece<1>(C, pc, out, red, wtot); break;
                case 2: gram_piece<2>(C, pc, out, red, wtot); break;
                case 3: gram_piece<3>(C, pc, out, red, wtot); break;
                case 4: gram_piece<4>(C, pc, out, red, wtot); break;
                case 5: gram_piece<5>(C, pc, out, red, wtot); break;
                case 6: gram_piece<6>(C, pc, out, red, wtot); break;
                case 7: gram_piece<7>(C, pc, out, red, wtot); break;
                default: gram_piece<8>(C, pc, out, red, wtot); break;
            }
        }
        base += tot;
        __syncthreads();   // pre is rewritten for the next chains
    }
}

// Rank of a D x D Gram matrix (lower triangle in tri) by pivoted elimination, pivots
// above 1e-12 of the largest diagonal entry, a warp over the D^2 entries (two a lane, in
// H, D^2 doubles of shared memory).  The matrix is first scaled by a power of two (exact)
// that brings the largest diagonal entry into [1, 2), so the pivots' reciprocals come
// from an FP32 seed and one FP64 Newton step; diagonal entries (never negative before
// the elimination, and compared only against a positive threshold) are compared as
// integers, which the FP64-starved SM does on its integer pipe.
template <int D>
__device__ int warp_rank(const double *tri, double *H, int lane) {
    constexpr int DD = D * D;
    auto tidx = [](int a, int b) { return a >= b ? a * (a + 1) / 2 + b : b * (b + 1) / 2 + a; };
    const int e1 = lane + 32;
    const int a0 = lane / D, b0 = lane % D, a1 = e1 / D, b1 = e1 % D;
    const bool has0 = lane < DD, has1 = e1 < DD;
    long long gbits = 0;
#pragma unroll
    for (int a = 0; a < D; ++a) gbits = max(gbits, __double_as_longlong(tri[tidx(a, a)]));
    if (gbits <= 0 || gbits >= 0x7ff0000000000000LL) return 0;   // zero couplings (or not finite)
    const int ex = (int)(gbits >> 52);                               // biased exponent of the largest entry
    const double scale = __longlong_as_double((long long)max(1, 2046 - ex) << 52);
    double h0 = has0 ? tri[tidx(a0, b0)] * scale : 0.0;
    double h1 = has1 ? tri[tidx(a1, b1)] * scale : 0.0;
    if (has0) H[lane] = h0;
    if (has1) H[e1] = h1;
    const long long thr = __double_as_longlong(1e-12 * (__longlong_as_double(gbits) * scale));
    __syncwarp();
    unsigned used = 0;
    int rank = 0;
    for (int st = 0; st < D; ++st) {
        long long best = thr;
        int pv = -1;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            const long long v = __double_as_longlong(H[a * D + a]);
            if (!(used >> a & 1u) && v > best && v < 0x7ff0000000000000LL) { best = v; pv = a; }
        }
        if (pv < 0) break;
        used |= 1u << pv;
        ++rank;
        const double p = __longlong_as_double(best);
        double inv = (double)__frcp_rn((float)p);
        inv = fma(inv, fma(-p, inv, 1.0), inv);
        __syncwarp();   // the diagonal is read before any entry changes
        // Schur complement on the remaining rows and columns; the pivot row and column
        // are only read
        if (has0 && !(used >> a0 & 1u) && !(used >> b0 & 1u)) {
            h0 = fma(-H[a0 * D + pv] * inv, H[pv * D + b0], h0);
            H[lane] = h0;
        }
        if (has1 && !(used >> a1 & 1u) && !(used >> b1 & 1u)) {
            h1 = fma(-H[a1 * D + pv] * inv, H[pv * D + b1], h1);
            H[e1] = h1;
        }
        __syncwarp();
    }
    return rank;
}

// Directions of group q that no coupling reaches, m - rank(M_q), written to gE[N + q].
// One-pole groups: rank 1 exactly when a coupling is non-zero (the elimination's second
// pivot is rounding), one thread each over the whole CTA.  Larger groups a warp each,
// round robin: up to kGrpSmall poles the Gram entries are summed here (lanes over the
// entries, one FP64 instruction per pole for all of them, when they fit in a warp),
// beyond that from the pieces' partial sums in piece order; then warp_rank.
template <int D>
__device__ void group_counts(const LzChain &C, int Q, double *gE, const int *gInfo, const GrpScratch &S, int warp,
                             int lane, double *tri, double *H) {
    constexpr int P = D * (D + 1) / 2;
    const int N = C.N;
    for (int q = warp * 32 + lane; q < Q; q += kGrpThreads) {
        const int h0 = gInfo[1 + q];
        const int mm = ((q + 1 < Q) ? gInfo[2 + q] : N) - h0;
        if (mm == 1) {
            bool any = false;
#pragma unroll
            for (int a = 0; a < D; ++a) any |= (C.M[(size_t)a * N + h0] != 0.0);
            gE[N + q] = any ? 0.0 : 1.0;
        }
    }
    for (int q = warp; q < Q; q += kGrpThreads / 32) {
        const int g0 = gInfo[1 + q];
        const int g1 = (q + 1 < Q) ? gInfo[2 + q] : N;
        const int m = g1 - g0;
        if (m <= 1) continue;
        if (m > kGrpSmall) {
            const double *pp = S.part + (size_t)S.first[q] * kGramEntries;
            const int np = (m + kGrpPiece - 1) / kGrpPiece;
            double a0 = 0.0, a1 = 0.0;
            for (int k = 0; k < np; ++k, pp += kGramEntries) {
                if (lane < P) a0 += pp[lane];
                if (lane + 32 < P) a1 += pp[lane + 32];
            }
            if (lane < P) tri[lane] = a0;
            if (lane + 32 < P) tri[lane + 32] = a1;
        } else if (P <= 32) {
            if (lane < P) {
                int a = 0, b = lane;
                while (b > a) { b -= a + 1; ++a; }   // entry (a, b) of the lower triangle
                const double *ma = C.M + (size_t)a * N, *mb = C.M + (size_t)b * N;
                double acc = 0.0;
                for (int i = g0; i < g1; ++i) acc += ma[i] * mb[i];
                tri[lane] = acc;
            }
        } else {
            double G[P];
#pragma unroll
            for (int u = 0; u < P; ++u) G[u] = 0.0;
            for (int i = g0 + lane; i < g1; i += 32) {
                double mv[D];
#pragma unroll
                for (int a = 0; a < D; ++a) mv[a] = C.M[(size_t)a * N + i];
                int u = 0;
#pragma unroll
                for (int a = 0; a < D; ++a)
#pragma unroll
                    for (int b = 0; b <= a; ++b) G[u++] += mv[a] * mv[b];
            }
#pragma unroll
            for (int u = 0; u < P; ++u)
                for (int o = 16; o > 0; o >>= 1) G[u] += __shfl_xor_sync(0xffffffffu, G[u], o);
            if (lane == 0)
#pragma unroll
                for (int u = 0; u < P; ++u) tri[u] = G[u];
        }
        __syncwarp();
        const int rank = warp_rank<D>(tri, H, lane);
        if (lane == 0) gE[N + q] = (double)max(0, m - rank);
    }
}

__global__ void __launch_bounds__(kGrpThreads) k_lz_groups(const LzChain *chains, int nchains) {
    const int cid = blockIdx.x;
    if (cid >= nchains) return;
    const LzChain C = chains[cid];
    if (!C.gE) return;
    double *gE = const_cast<double *>(C.gE);
    int *gInfo = const_cast<int *>(C.gInfo);
    const GrpScratch S = lz_grp_scratch(C.gE, C.N);
    const int N = C.N, D = C.D, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __shared__ int ws[kGrpThreads / 32];
    __shared__ double s_tri[kGrpThreads / 32][kGramEntries];
    __shared__ double s_h[kGrpThreads / 32][64];
    const int Q = gInfo[0];
    switch (D) {
        case 1: group_counts<1>(C, Q, gE, gInfo, S, warp, lane, s_tri[warp], s_h[warp]); break;
        case 2: group_counts<2>(C, Q, gE, gInfo, S, warp, lane, s_tri[warp], s_h[warp]); break;
        case 3: group_counts<3>(C, Q, gE, gInfo, S, warp, lane, s_tri[warp], s_h[warp]); break;
        case 4: group_counts<4>(C, Q, gE, gInfo, S, warp, lane, s_tri[warp], s_h[warp]); break;
        case 5: group_counts<5>(C, Q, gE, gInfo, S, warp, lane, s_tri[warp], s_h[warp]); break;
        case 6: group_counts<6>(C, Q, gE, gInfo, S, warp, lane, s_tri[warp], s_h[warp]); break;
        case 7: group_counts<7>(C, Q, gE, gInfo, S, warp, lane, s_tri[warp], s_h[warp]); break;
        default: group_counts<8>(C, Q, gE, gInfo, S, warp, lane, s_tri[warp], s_h[warp]); break;
    }
    __syncthreads();
    // inclusive cumulative counts: gInfo[1 + q] = directions of groups 0..q, so a
    // direction index finds its group by binary search
    int base = 0;
    for (int b = 0; b < Q; b += kGrpThreads) {
        const int q = b + tid;
        const int x = (q < Q) ? (int)gE[N + q] : 0;
        int tot;
        const int ex = block_excl_scan<kGrpThreads>(x, tot, ws);
        if (q < Q) gInfo[1 + q] = base + ex + x;
        base += tot;
    }
}

cudaError_t launch_lz_groups(const LzChain *d_chains, int nchains, long long gram_cap, cudaStream_t st) {
    if (nchains <= 0) return cudaSuccess;
    k_lz_gstart<<<nchains, kGstartThreads, 0, st>>>(d_chains, nchains);
    const int grid = (int)(gram_cap < 1 ? 1 : (gram_cap < kGramCtas ? gram_cap : kGramCtas));
    k_lz_gram<<<grid, kGramThreads, 0, st>>>(d_chains, nchains);
    k_lz_groups<<<nchains, kGrpThreads, 0, st>>>(d_chains, nchains);
    return cudaGetLastError();
}

void lanczos_smem_init() {
    allow_dynamic_smem((const void *)k_lanczos<float, false>);
    allow_dynamic_smem((const void *)k_lanczos<float, true>);
    allow_dynamic_smem((const void *)k_lanczos<double, false>);
    allow_dynamic_smem((const void *)k_lanczos<double, true>);
}

}  // namespace bd
