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
// criterion), at most four sweeps.  On the degenerate unperturbed spectra the
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
// distributed shared memory; every CTA adds the peers' partials in rank order,
// so all CTAs hold bit-identical totals and take identical branches.
#include <climits>
#include <cooperative_groups.h>
#include "bd_common.cuh"
#include "bd_kernels.h"

namespace cg = cooperative_groups;

namespace bd {

template <typename VT> struct LzTraits;
template <> struct LzTraits<double> { using CT = double; };
template <> struct LzTraits<float> { using CT = float; };

__device__ inline double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic pseudo-random restart value of pole i at Lanczos index j, in [0.5, 1.5).
__host__ __device__ inline double restart_value(int i, int j) {
    unsigned x = (unsigned)i * 2654435761u ^ ((unsigned)j * 40503u + 0x9e3779b9u);
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return 0.5 + (double)(x & 0xffffffu) / 16777216.0;
}

constexpr int kLzThreads = 256;
constexpr int kLzWarps = kLzThreads / 32;
constexpr int kMaxScal = 32;   // 2 + D + n_used <= 32

// Shared-memory layout (doubles): Es[S] | w[S] | wc[S] (compute-type copy) |
// A[rmax] (dot partials) | B[kMaxScal] (scalar partials) | c[rmax] (totals) |
// red[kLzWarps * kMaxScal] (block reduction scratch)
template <typename VT>
__global__ void __launch_bounds__(kLzThreads) k_lanczos(const LzChain *chains, int nchains, int rmax, double eta2) {
    using CT = typename LzTraits<VT>::CT;
    cg::cluster_group cluster = cg::this_cluster();
    const int CL = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int cid = blockIdx.x / CL;
    if (cid >= nchains) return;  // whole clusters only: every CTA of a cluster has the same cid
    const LzChain C = chains[cid];
    const int N = C.N, D = C.D, L = C.L, NT = C.nden_out + C.D;
    const int S = (N + CL - 1) / CL;
    const int i0 = rank * S;
    const int ns = max(0, min(N, i0 + S) - i0);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    extern __shared__ double sm[];
    double *Es = sm;
    double *w = Es + S;
    CT *wc = reinterpret_cast<CT *>(w + S);
    double *A = w + 2 * S;
    double *B = A + rmax;
    double *c = B + kMaxScal;
    double *red = c + rmax;
    unsigned char *touched = reinterpret_cast<unsigned char *>(red + kLzWarps * kMaxScal);
    __shared__ double tot[kMaxScal];
    __shared__ int s_kmin;

    VT *V = reinterpret_cast<VT *>(C.V);
    for (int i = tid; i < ns; i += kLzThreads) { Es[i] = C.E[i0 + i]; touched[i] = 0; }
    const double tau = (sizeof(VT) == 4) ? 1e-22 : 1e-48;

    int k = -1;           // current pivot chain
    int two_pass = 0;
    for (int j = 0; j < L; ++j) {
        const bool newv = (k + 1 < C.n_used) && (j == C.start[k + 1]);
        if (newv) ++k;
        __syncthreads();
        // (a) w = M.p  or  w = v_{j-1} * E   (source/BcDor-Lanczos.cpp:137-150)
        if (newv) {
            const double *p = C.piv + (size_t)k * D;
            for (int i = tid; i < ns; i += kLzThreads) {
                double s = 0.0;
                for (int d = 0; d < D; ++d) s = __dadd_rn(s, __dmul_rn(C.M[(size_t)d * N + i0 + i], p[d]));
                w[i] = s;
            }
        } else {
            const VT *vp = V + (size_t)(j - 1) * C.ld + i0;
            for (int i = tid; i < ns; i += kLzThreads) w[i] = (double)vp[i] * Es[i];
        }
        bool injected = false;     // w replaced by a pseudo-random restart vector
        bool done = false;         // step finished by an untouched-pole unit vector
        for (int attempt = 0; attempt < 2 && !done; ++attempt) {
        int pass = 0;
        double wn2_first = 0.0;
        for (;;) {
            __syncthreads();
            for (int i = tid; i < ns; i += kLzThreads) wc[i] = (CT)w[i];
            __syncthreads();
            // (b1) partial dot products <v_t, w> over the own slice, one warp per t
            for (int t = warp; t < j; t += kLzWarps) {
                const VT *vt = V + (size_t)t * C.ld + i0;
                CT acc = 0;
                for (int i = lane; i < ns; i += 32) acc += (CT)vt[i] * wc[i];
                double s = warp_sum((double)acc);
                if (lane == 0) A[t] = s;
            }
            {   // partial |w|^2 before this sweep
                double acc = 0.0;
                for (int i = tid; i < ns; i += kLzThreads) acc += w[i] * w[i];
                acc = warp_sum(acc);
                if (lane == 0) red[warp] = acc;
                __syncthreads();
                if (tid == 0) {
                    double s = 0.0;
                    for (int q = 0; q < kLzWarps; ++q) s += red[q];
                    A[j] = s;
                }
            }
            cluster.sync();
            // (b2) totals over the cluster, in rank order
            for (int t = tid; t <= j; t += kLzThreads) {
                double s = 0.0;
                for (int r = 0; r < CL; ++r) s += cluster.map_shared_rank(A, r)[t];
                c[t] = s;
            }
            __syncthreads();
            const double wn2_before = c[j];
            if (pass == 0) wn2_first = wn2_before;
            // (b3) w -= sum_t c_t v_t, then partial alpha / beta / m / g sums of the new w
            const int nq = k;  // earlier pivots
            const int nsc = 2 + D + nq;
            double acc_s[kMaxScal];
#pragma unroll
            for (int q = 0; q < kMaxScal; ++q) acc_s[q] = 0.0;
            for (int i = tid; i < ns; i += kLzThreads) {
                CT a0 = 0, a1 = 0;
                int t = 0;
                for (; t + 1 < j; t += 2) {
                    a0 += (CT)c[t] * (CT)V[(size_t)t * C.ld + i0 + i];
                    a1 += (CT)c[t + 1] * (CT)V[(size_t)(t + 1) * C.ld + i0 + i];
                }
                if (t < j) a0 += (CT)c[t] * (CT)V[(size_t)t * C.ld + i0 + i];
                const double wi = w[i] - ((double)a0 + (double)a1);
                w[i] = wi;
                const double e = Es[i];
                acc_s[0] += e * wi * wi;
                acc_s[1] += wi * wi;
                for (int d = 0; d < D; ++d) acc_s[2 + d] += C.M[(size_t)d * N + i0 + i] * wi;
                for (int q = 0; q < nq; ++q) acc_s[2 + D + q] += e * (double)V[(size_t)C.last[q] * C.ld + i0 + i] * wi;
            }
            for (int q = 0; q < nsc; ++q) {
                double s = warp_sum(acc_s[q]);
                if (lane == 0) red[warp * kMaxScal + q] = s;
            }
            __syncthreads();
            if (tid < nsc) {
                double s = 0.0;
                for (int q = 0; q < kLzWarps; ++q) s += red[q * kMaxScal + tid];
                B[tid] = s;
            }
            cluster.sync();
            if (tid < nsc) {
                double s = 0.0;
                for (int r = 0; r < CL; ++r) s += cluster.map_shared_rank(B, r)[tid];
                tot[tid] = s;
            }
            __syncthreads();
            // another sweep while this one removed more than half of the squared norm
            if (j > 0 && pass < 3 && tot[1] < eta2 * wn2_before) { ++pass; ++two_pass; continue; }
            break;
        }
        if (attempt > 0 || !(tot[1] <= tau * wn2_first || tot[1] == 0.0)) break;
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
            VT *vj = V + (size_t)j * C.ld + i0;
            for (int i = tid; i < ns; i += kLzThreads) {
                const bool hit = (i0 + i == kmin);
                vj[i] = hit ? (VT)1 : (VT)0;
                if (hit) touched[i] = 1;
            }
            if (rank == 0 && tid == 0) {
                double *row = C.out + (size_t)j * NT;
                for (int q = 0; q < NT; ++q) row[q] = 0.0;
                row[0] = C.E[kmin];
                for (int d = 0; d < D; ++d) row[C.nden_out + d] = C.M[(size_t)d * N + kmin];
            }
            done = true;
        } else {
            for (int i = tid; i < ns; i += kLzThreads) w[i] = restart_value(i0 + i, j);
            injected = true;
        }
        cluster.sync();   // peers have read s_kmin before it can change again
        }
        if (done) continue;
        // (c) normalise, store, write the output row (source/BcDor-Lanczos.cpp:198-216)
        const double xb2 = tot[1];
        const double xa = tot[0] / xb2;
        const double xb = sqrt(xb2);
        VT *vj = V + (size_t)j * C.ld + i0;
        for (int i = tid; i < ns; i += kLzThreads) {
            const VT v = (VT)(w[i] / xb);
            vj[i] = v;
            touched[i] |= (v != (VT)0);
        }
        if (rank == 0 && tid == 0) {
            double *row = C.out + (size_t)j * NT;
            row[0] = xa;
            row[1] = injected ? 0.0 : xb;   // a restart vector has no coupling to v_{j-1}
            for (int q = 0; q < k; ++q) row[2 + q] = tot[2 + D + q] / xb;
            for (int d = 0; d < D; ++d) row[C.nden_out + d] = tot[2 + d] / xb;
            if (newv) row[1] = row[1 + k];
        }
        __syncthreads();
    }
    if (rank == 0 && tid == 0) atomicAdd(&C.stat[0], two_pass);
    cluster.sync();  // no CTA leaves while peers may still read its shared memory
}

size_t lanczos_smem_bytes(int S, int rmax) {
    return sizeof(double) * ((size_t)3 * S + 2 * (size_t)rmax + kMaxScal + (size_t)kLzWarps * kMaxScal) + (size_t)S + 16;
}

cudaError_t launch_lanczos(const LzChain *d_chains, int nchains, int S_max, int rmax, bool fp32, int cluster,
                           double eta, cudaStream_t st) {
    if (nchains <= 0) return cudaSuccess;
    size_t smem = lanczos_smem_bytes(S_max, rmax);
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
    cudaError_t e;
    if (fp32) {
        e = cudaFuncSetAttribute(k_lanczos<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess && cluster > 8)
            e = cudaFuncSetAttribute(k_lanczos<float>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
        return cudaLaunchKernelEx(&cfg, k_lanczos<float>, d_chains, nchains, rmax, eta * eta);
    }
    e = cudaFuncSetAttribute(k_lanczos<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess && cluster > 8)
        e = cudaFuncSetAttribute(k_lanczos<double>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, k_lanczos<double>, d_chains, nchains, rmax, eta * eta);
}

}  // namespace bd
