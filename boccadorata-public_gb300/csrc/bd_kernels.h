// bd_kernels.h -- kernels and launch helpers of the chain, shared by the host
// orchestration in bd_api.cu.
#pragma once
#include <cstddef>
#include "bd_common.cuh"

struct bd_files;

namespace bd {

// the interaction lines of a files object (orbits, J, V in file order); false if none
bool files_interaction(const bd_files *f, const int4 **abcd, const int **J, const double **V, long long *n);

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
__global__ void k_rows_aos_perm(const int *perm, long long off, const double *E, const double *S2, const double *M,
                                int N, int D, double *rows);
// Tensor-core coupling build of the mixed form (k_coupling_tc.cu): M, E and S2 of every
// pole of direction dir from the tiles of blocks sharing (ia, ib, ig, nJab).
size_t tc_smem_bytes(int np);
cudaError_t launch_poles_tc(const DevProblem &P, const S2Block *blk, const int *tile_blk, const int4 *tiles,
                            int ntiles, const ChanSig *cs, int dir, const double *vp, double *E, double *S2, double *M,
                            int *err, size_t smem, cudaStream_t st);
constexpr int kSortThreads = 512;
constexpr int kSortChunk = 2048;  // poles per chunk of the shared-memory sort
constexpr int kSortMax = 16384;   // longest channel sorted by chunks (longer: radix sort)
__global__ void k_chunk_sort(const double *E, const int4 *chunks, bool desc, long long base, unsigned long long *tk,
                             int *ti);
// Stable LSD radix sort of (key, value) pairs over key bits [bit0, bit1), eight per pass
// (k_sort.cu).  keys / vals and ktmp / vtmp are ping-pong buffers of n entries: on
// return keys / vals point at the sorted pairs.  scratch: radix_scratch_bytes(n).
size_t radix_scratch_bytes(long long n);
int radix_launches(int passes, bool skip_constant);
cudaError_t radix_sort_pairs(unsigned long long *&keys, unsigned *&vals, unsigned long long *&ktmp, unsigned *&vtmp,
                             long long n, int bit0, int bit1, bool skip_constant, void *scratch, int *passes_out,
                             cudaStream_t st);
size_t scan_scratch_bytes(long long m);
cudaError_t exclusive_scan_u32(unsigned *data, long long m, void *scratch, cudaStream_t st);
__global__ void k_vpp_canon(const int4 *abcd, const int *Jv, long long n, const int *orb_sh, const int *j2,
                            const int *ip, const int *ch, unsigned long long *key, unsigned *val, signed char *sign,
                            int *bad);
__global__ void k_vpp_first(const unsigned long long *key, long long n, unsigned *keep);
__global__ void k_vpp_place(const unsigned long long *key, const unsigned *val, const unsigned *pos, const unsigned *keep,
                            long long n, const double *Vin, const signed char *sign, int *iabJ, int *icdJ, double *V);
cudaError_t launch_pole_radix(const double *E, const int *seg_of, int ch_lo, int nseg, long long n0, long long n,
                              bool desc, unsigned long long *k0, unsigned *v0, unsigned long long *k1, unsigned *v1,
                              void *scratch, int *perm, int *launches, cudaStream_t st);
__global__ void k_dressed_select(const double *sol, const long long *sol_off, const int *nq, const int *D_of, int ns,
                                 double z_cut, int max_frag, int cap, int *cnt, int *sel);
__global__ void k_dressed_write(const double *sol, const long long *sol_off, const int *nq, const int *D_of,
                                const int *p_start, const int *h_start, int ns, int nspb, int cap, const int *cnt,
                                const int *sel, double *ep, double *eh, double *fqp, double *fqh);
cudaError_t launch_nonfinite(const double *x, long long n, int *bad, cudaStream_t st);
constexpr int kHeapMax = 49152;  // longest channel put in the reference's heap-sort order
cudaError_t launch_heap_order(const double *E, const int *d_off, int nseg, int max_len, long long n0, int *perm,
                              cudaStream_t st);
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
int tridiag_fit_order(int cluster);   // the largest order the cluster reduction's layout holds
void tridiag_fit_warm();              // fills tridiag_fit_order's cache (cluster sizes 1..16) and
                                      // registers the Dyson kernels' shared-memory limits
// each translation unit's kernels with large dynamic shared memory (allow_dynamic_smem)
void tc_smem_init();
void eig_smem_init();
void sigma2_smem_init();
void lanczos_smem_init();
// DyJob::stat values: the eigensolver did not converge; the deflated matrix is larger
// than the cluster reduction's shared-memory layout holds (nothing solved)
constexpr int kDyStatNumeric = 1, kDyStatCapacity = 2;

}  // namespace bd
