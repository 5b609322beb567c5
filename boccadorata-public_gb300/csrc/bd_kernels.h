// bd_kernels.h -- kernels and launch helpers of the chain, shared by the host
// orchestration in bd_api.cu.
#pragma once
#include <cstddef>
#include "bd_common.cuh"

namespace bd {

__global__ void k_vgather(DevProblem P, const S2Block *blk, const int *chunk_blk, const int *chunk_first, int w0,
                          int nw, double *vp);
__global__ void k_poles(DevProblem P, const S2Block *blk, const long long *pole_first, int nblk, long long g0,
                        long long total, const ChanSig *cs, int dir, const double *vp, double *E, double *S2,
                        double *M);
__global__ void k_ehf_terms(DevProblem P, const int3 *entries, const long long *term_first, int e0, int e1,
                            const int *ctab_cmb, const int *ctab_toff, const int *ctab_off, const int *ncomb,
                            double *terms);
__global__ void k_ehf_sum(DevProblem P, const int3 *entries, const long long *term_first, int e0, const int *ctab_cmb,
                          const int *ctab_toff, const int *ctab_off, const int *ncomb, const double *terms,
                          const long long *out_off, double *out);
__global__ void k_permute_soa(const int *perm, long long n0, long long n, const int *seg_of, const ChanSig *cs, int dir,
                              const double *Ein, const double *Min, double *Eout, double *Mout, float *Mfout);
__global__ void k_rows_aos(const double *E, const double *S2, const double *M, int N, int D, double *rows);
constexpr int kSortThreads = 512;
constexpr int kSortChunk = 2048;  // poles per chunk of the shared-memory sort
constexpr int kSortMax = 16384;   // longest channel sorted by chunks (longer: radix sort)
__global__ void k_chunk_sort(const double *E, const int4 *chunks, bool desc, long long base, unsigned long long *tk,
                             int *ti);
__global__ void k_chunk_place(const unsigned long long *tk, const int *ti, const int4 *chunks, int nchunks,
                              long long n, long long base, int *perm);
__global__ void k_pair_rank(const int *iabJ, const int *icdJ, int n, int norb, const int *orb_sh, const int *ch,
                            const int *ip, const int *seg_str, int nJ, int *prank);
__global__ void k_pole_index(const int *off, int ns, long long n, int *seg, int *idx);
__global__ void k_segments(const int *iabJ, const int *icdJ, int n, int norb, const int *orb_sh, const int *ch,
                           const int *ip, int *seg_str, int *seg_end, int *seg_cnt, int *bad, int2 *rows, int nJ);

cudaError_t launch_lanczos(const LzChain *d_chains, int nchains, int S_max, int rmax, bool fp32, int cluster,
                           double eta, bool global_slices, cudaStream_t st);
size_t lanczos_smem_bytes(int S, int rmax, bool global_slices = false);
constexpr size_t kLanczosSmemSliceCap = 100 * 1024;   // above this the slices go to global memory
cudaError_t launch_to_float(const double *in, float *out, long long n, cudaStream_t st);
cudaError_t launch_lz_groups(const LzChain *d_chains, int nchains, long long gram_cap, cudaStream_t st);

int dyson_launch_count(int nmax);
cudaError_t launch_dyson(const DyJob *d_jobs, int njobs, const long long *d_row_first, long long total_rows,
                         int nmax, int Dmax, int cluster, double *work, const long long *d_work_first, cudaStream_t st);
cudaError_t launch_eig(const DyJob *d_jobs, int njobs, const long long *d_row_first, long long total_rows,
                       double *work, const long long *d_work_first, cudaStream_t st);
size_t tridiag_smem_bytes(int nmax, int cluster);

}  // namespace bd
