/*
 * bd_gb300.h -- C ABI of the GB300 (sm_103a) implementation of BoccaDorata's
 *               second-order self-energy -> Lanczos -> Dyson chain.
 *
 * All functions return BD_OK (0) or a negative status; none of them exits the
 * process.  Buffers are caller-owned host memory; sizes are element counts.
 * A context (bd_ctx) owns one CUDA device, one stream and the device-resident
 * copies of the inputs.  Calls on one context are not thread-safe; use one
 * context per host thread.
 *
 * Reference interfaces replaced (paths inside craolus/BoccaDorata-public):
 *   bd_count_poles     Wide_self_energy_t::Count_2p1h_2h1p_poles
 *                      source/BcDor-SlfEn_classes.hh:83, source/BcDor-Self_energy_ext_Op_c.cpp:35
 *   bd_sigma2_build    Wide_self_energy_t::Build_Dynamic_SlfEn_2ndOrder
 *                      source/BcDor-SlfEn_classes.hh:84, source/BcDor-Self_energy_ext_Op_c.cpp:323
 *   bd_sigma2_sorted   the in-place sort of Reduce_SelfEn_Lncz (Sort_u/d_double2dim)
 *                      source/BcDor-Self_energy_ext_Op_e.cpp:116-130, source/BcDor-Utilities.cpp:25-94
 *   bd_ehf             Wide_self_energy_t::Build_ExtendedHartreeFock -> SpProp_t::ExtendedHartreeFock_Pot
 *                      source/BcDor-Self_energy_ext_Op_b.cpp:71, source/BcDor-Sp_Propagator_a.cpp:39
 *   bd_lanczos_reduce  Wide_self_energy_t::Reduce_SelfEn_Lncz + Reduce_Mtx_Lncz
 *                      source/BcDor-SlfEn_classes.hh:88, source/BcDor-Self_energy_ext_Op_e.cpp:55,
 *                      source/BcDor-Run_vars.hh:193-195, source/BcDor-Lanczos.cpp:44
 *   bd_dyson_solve     DysonMatrix (+ Calc_En, Seek_EFermi)
 *   bd_dyson_rows      source/BcDor-Main.cpp:42, source/BcDor-DysonMatrix.cpp:123,542,619
 *   bd_run_all         the per-channel loop of Run_itrs, source/BcDor-Main.cpp:241-391
 *   bd_upload_propagator  Wide_self_energy_t::reset with a new input propagator,
 *                      source/BcDor-Main.cpp:225
 *   bd_dressed_propagator  the next iteration's propagator: DysonMatrix -> SpProp_t::add_qp /
 *                      add_qh (source/BcDor-DysonMatrix.cpp:487-488, source/BcDor-Sp_Propagator.cpp:683-809),
 *                      g_ptr1 = g_ptr2 (source/BcDor-Main.cpp:438-441), SpProp_t::quick_n_dirty_diff
 *                      (source/BcDor-Sp_Propagator.cpp:1189-1219)
 */
#ifndef BD_GB300_H
#define BD_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define BD_OK            0
#define BD_ERR_ARG      -1   /* bad argument, size or index                      */
#define BD_ERR_CUDA     -2   /* a CUDA runtime call failed (see bd_last_error)   */
#define BD_ERR_CAPACITY -3   /* an output buffer is too small                    */
#define BD_ERR_STATE    -4   /* call order: e.g. Dyson before any self-energy    */
#define BD_ERR_NUMERIC  -5   /* eigensolver did not converge / non-finite input  */
#define BD_ERR_TIMEOUT  -6   /* a bounded device wait gave up                    */

/* run flags for bd_run_all */
#define BD_RUN_LANCZOS   1   /* Lanczos-reduce Sigma(2) before Dyson (else full Dyson)  */
#define BD_RUN_MIXED     2   /* FP32 Lanczos vectors / reorthogonalisation              */
#define BD_RUN_PER_CHANNEL 4 /* launch channel by channel (the drop-in call pattern)   */
#define BD_RUN_REF_ORDER   8 /* FP64: the reduction visits equal pole energies in the
                                reference's heap-sort order (k_heap_order, a serial chain
                                per channel: slower) instead of their build order */
#define BD_RUN_GRAPH     16  /* batched: capture the step in a CUDA graph on first use (per
                                flag combination) and replay it; any change of the problem,
                                the pivots or the tuning captures it again */
#define BD_RUN_FP64_COUPLINGS 32 /* batched BD_RUN_MIXED on a dressed propagator: build the
                                couplings with the FP64 kernel instead of the tensor cores */

typedef struct bd_ctx bd_ctx;

/* Model space, ModSpace_t (source/BcDor-Sp_classes.hh:32-79).  Orbits are
 * grouped by subshell in subshell order (MSp_n[ish] - Mor_n = first orbit). */
typedef struct {
    int nsubsh;            /* number of (l, j, parity, charge) subshells = channels */
    int norb;              /* total number of orbits                                */
    const int *l, *j2, *ip, *ch, *no;   /* per subshell: l, 2j, parity, charge, #orbits */
    const int *orb_sh;     /* per orbit: subshell                                   */
    const double *orb_xe;  /* per orbit: model-space xe column                      */
} bd_modspace;

/* Propagator, SpProp_t (source/BcDor-Sp_classes.hh:87-160): fragments listed
 * subshell by subshell; amplitudes fragment-major with row stride nspb. */
typedef struct {
    int nspb;              /* N_SPB_MX = max orbits per subshell */
    const int *np, *nh;    /* per subshell: quasiparticles, quasiholes */
    const double *ep, *eh; /* energies */
    const double *fqp, *fqh; /* amplitudes, rows of nspb */
} bd_propagator;

/* Interaction, VppInt_t after prepare_for_reading (source/BcDor-Int_classes.hh:20-85,
 * source/BcDor-Vpp_potential.cpp:440-501): canonical keys (a<=b, c<=d, ab<=cd),
 * key = (a*1024+b)*128+J, sorted by (charge, parity, J), iabJ, icdJ. */
typedef struct {
    int n_me;
    const int *iabJ, *icdJ;
    const double *V;
} bd_interaction;

/* Lanczos pivots as Make_LancPivots returns them (source/BcDor-Miscellanea.cpp:334-390):
 * for subshell s, npvt[s] rows; iterations n_itr_fw/bk and D-vectors concatenated
 * subshell by subshell. */
typedef struct {
    const int *npvt;
    const int *n_itr_fw, *n_itr_bk;
    const double *vec;
} bd_pivots;

int         bd_create(bd_ctx **ctx, int device);
void        bd_destroy(bd_ctx *ctx);
const char *bd_last_error(const bd_ctx *ctx);
int         bd_version(void);

/* Device-resident copies of the inputs (replaces the ModSpace_t / VppInt_t /
 * SpProp_t objects the reference's calls read).  Must precede any other call. */
int bd_upload_problem(bd_ctx *ctx, const bd_modspace *ms, const bd_interaction *vpp,
                      const bd_propagator *prop);
int bd_upload_pivots(bd_ctx *ctx, const bd_pivots *piv);

/* Pole counts of channel ish (all-poles branch, icut == 0). */
int bd_count_poles(bd_ctx *ctx, int ish, int *n_fw, int *n_bk);

/* Static self-energy of channel ish: D x D, row-major. */
int bd_ehf(bd_ctx *ctx, int ish, double *sig_hf);

/* Sigma(2) of channel ish, built on the device.  Rows of 2 + D doubles
 * [E, sum_d M_d^2, M_0 .. M_{D-1}] in the reference's enumeration order are
 * copied to sig_fw / sig_bk when those are non-NULL (capacities in rows).
 * The device copy stays resident for bd_lanczos_reduce / bd_dyson_solve. */
int bd_sigma2_build(bd_ctx *ctx, int ish, double *sig_fw, int cap_fw, int *n_fw,
                    double *sig_bk, int cap_bk, int *n_bk);

/* Lanczos reduction of the resident Sigma(2) of channel ish.
 * pivots: n_pvt rows of D doubles, normalised in place (as the reference does);
 * n_itr_fw / n_itr_bk: iterations per pivot, rescaled in place when they exceed
 * the pole count (as the reference does).  Output rows have (n_pvt + 1) + D
 * doubles [alpha, beta, g_0 .., m_0 .. m_{D-1}]; ipiv_* receive
 * [n_used_pivots, 1, start_1, ...] and must hold n_pvt + 1 + D ints.
 * flags: 0 = FP64, BD_RUN_MIXED = FP32 vectors, BD_RUN_REF_ORDER = FP64 visiting
 * equal energies in the reference's heap-sort order (the order of equal energies
 * changes only rounding: the Krylov space does not depend on it). */
int bd_lanczos_reduce(bd_ctx *ctx, int ish, int n_pvt, double *pivots, int *n_itr_fw, int *n_itr_bk,
                      double *lz_fw, int cap_fw, int *L_fw, int *ipiv_fw,
                      double *lz_bk, int cap_bk, int *L_bk, int *ipiv_bk, int flags);

/* Rows [E, sum_d M_d^2, M_0 .. M_{D-1}] of channel ish's resident Sigma(2) as the
 * reference leaves them sorted in place before reducing them (Reduce_SelfEn_Lncz,
 * source/BcDor-Self_energy_ext_Op_e.cpp:116-130; forward ascending, backward descending,
 * by the heap sorts of source/BcDor-Utilities.cpp:25-94), equal energies in the heap
 * sort's order, for channels of up to 49 152 poles (longer ones: in their build order).
 * The order is formed on the device on demand (unless the last reduction of the channel
 * already visited it, BD_RUN_REF_ORDER).  Capacities in rows; either buffer may be
 * NULL.  BD_ERR_STATE before any reduction of the channel. */
int bd_sigma2_sorted(bd_ctx *ctx, int ish, double *sig_fw, int cap_fw, double *sig_bk, int cap_bk);

/* Dyson eigensolve of channel ish with the most recent resident self-energy
 * (Lanczos-reduced if bd_lanczos_reduce was called after bd_sigma2_build).
 * sig1b: one-body term (D x D); sig_hf: static self-energy (D x D, NULL = build
 * it with bd_ehf); e_fermi: Fermi energy (NaN = Seek_EFermi on the input propagator).
 * Solutions are rows of 2 + D doubles [W, Z, x_0 .. x_{D-1}], quasiparticles
 * (W > E_F) and quasiholes each sorted by descending W, Z = sum x_d^2 as stored by
 * SpProp_t::add_qp / add_qh.  koltun = {sum_qh x.S1b.x, sum_qh |x|^2 W, sum_qh |x|^2}
 * times (2j+1), as Calc_En. */
int bd_dyson_solve(bd_ctx *ctx, int ish, const double *sig1b, const double *sig_hf, double e_fermi,
                   double *sol_qp, int cap_qp, int *n_qp, double *sol_qh, int cap_qh, int *n_qh,
                   double *koltun);

/* DysonMatrix on a self-energy supplied by the caller (e.g. one loaded with
 * Wide_self_energy_t::load_SelfEn_bin, the ExtSE path of source/BcDor-Main.cpp:350-356).
 * Rows have nden + D doubles: nden = 2 for a plain Sigma(2) [E, *, M_0 ..], or
 * n_pvt + 1 for Lanczos rows [alpha, beta, g_0 .., m_0 ..] with their i_piv array
 * (ipiv_* = NULL marks plain rows).  Outputs as bd_dyson_solve.  Rows with no coupling
 * leave the matrix first; a remaining (deflated) order above what the cluster
 * reduction's shared memory holds (about 7 000 on GB300) gives BD_ERR_CAPACITY, as it
 * does in bd_dyson_solve and bd_sync. */
int bd_dyson_rows(bd_ctx *ctx, int ish, int nden, int n_fw, const double *fw_rows, const int *ipiv_fw,
                  int n_bk, const double *bk_rows, const int *ipiv_bk, const double *sig1b, const double *sig_hf,
                  double e_fermi, double *sol_qp, int cap_qp, int *n_qp, double *sol_qh, int cap_qh, int *n_qh,
                  double *koltun);

/* Copy of the Lanczos basis of the last reduction of channel ish (dir 0 forward,
 * 1 backward) as L rows of N doubles; fp32 = 1 if it ran with BD_RUN_MIXED.  Used to
 * check the basis' orthonormality. */
int bd_lanczos_vectors(bd_ctx *ctx, int ish, int dir, int fp32, double *out, long long cap);

/* Whole chain for every channel (flags BD_RUN_*), asynchronous on the context's
 * stream; one-body term diag(orb_xe) (Trel=7 ExtU1=1).  bd_sync waits for it. */
int bd_run_all(bd_ctx *ctx, int flags);
int bd_sync(bd_ctx *ctx);

/* Results of the last bd_run_all. */
int bd_result_counts(bd_ctx *ctx, int ish, int *n_qp, int *n_qh);
int bd_result_fetch(bd_ctx *ctx, int ish, double *sol_qp, int cap_qp, double *sol_qh, int cap_qh,
                    double *koltun);
/* koltun[3 * nsubsh] for every channel with one copy. */
int bd_result_koltun_all(bd_ctx *ctx, double *koltun);
/* Every channel's solutions with one copy: sol receives, channel after channel, the
 * rows bd_result_fetch gives (n_qp quasiparticles, then n_qh quasiholes, 2 + D doubles
 * each); counts[2 * ish] = n_qp, counts[2 * ish + 1] = n_qh; koltun[3 * nsubsh].  cap is
 * the number of doubles sol holds (any pointer may be NULL). */
int bd_result_fetch_all(bd_ctx *ctx, double *sol, long long cap, int *counts, double *koltun);

/* Replace the input propagator, keeping the model space and the interaction resident
 * (a new iteration of Run_itrs).  Pole counts, the block plan and the Lanczos chain
 * schedules (from the pivots already uploaded) follow the new propagator. */
int bd_upload_propagator(bd_ctx *ctx, const bd_propagator *prop);

/* The next iteration's propagator from the Dyson solutions of the last bd_run_all.
 * The reference appends every solution (add_qp / add_qh), so the pole count of the
 * next Sigma(2) grows with the cube of the fragment count; this build truncates:
 * per subshell, the quasiparticles and the quasiholes with Z >= z_cut, at most
 * max_frag of each (max_frag <= 0: no limit), the largest Z first, kept in the order
 * add_qp / add_qh store them (descending W; amplitudes x_0..x_{D-1}, zero up to nspb).
 * z_cut <= 0 and max_frag <= 0 reproduce the reference's update.
 * Unless keep_current, the new propagator replaces the context's (bd_upload_propagator).
 * np_out / nh_out [nsubsh], ep_out [cap_p], eh_out [cap_h], fqp_out [cap_p * nspb],
 * fqh_out [cap_h * nspb] receive it when non-NULL; *diff receives quick_n_dirty_diff
 * between the propagator the run used and the new one. */
int bd_dressed_propagator(bd_ctx *ctx, double z_cut, int max_frag, int keep_current, int *np_out, int *nh_out,
                          double *ep_out, int cap_p, double *eh_out, int cap_h, double *fqp_out, double *fqh_out,
                          double *diff);
/* 1 when the last bd_dressed_propagator updated the resident propagator on the device:
 * with 0 < max_frag <= 32 and the truncated propagator keeping the current fragment counts
 * of every subshell, the fragments are selected and written in place and the block
 * plan, pole counts and chain schedules stay (no host planning); otherwise 0. */
int bd_dressed_on_device(bd_ctx *ctx);
/* 1 when the last batched bd_run_all built the couplings M on the tensor cores: the
 * BD_RUN_MIXED form (with BD_RUN_LANCZOS) on a propagator with some fragment of more than
 * one non-zero amplitude, unless BD_RUN_FP64_COUPLINGS (tcgen05, TF32 in three products
 * hi*hi + hi*lo + lo*hi with FP32 accumulation, about 2^-21 relative; the FP64 form and
 * the per-channel calls always use the FP64 build, bit for bit the reference's). */
int bd_tensor_couplings(bd_ctx *ctx);
/* Device time of the phases of the last bd_run_all in ms: sigma2, sort, lanczos, dyson, total. */
int bd_last_timings(bd_ctx *ctx, double *ms5);
/* Diagnostics: extra reorthogonalisation sweeps of the last bd_run_all; device time of
 * its Lanczos kernel launch (ms, CUDA events on the context's stream) when the run was
 * batched; kernels of this library launched on the context so far; tuning knobs
 * (cluster sizes 1..16, DGKS threshold eta). */
int       bd_diag_two_pass(bd_ctx *ctx);
double    bd_lanczos_kernel_ms(bd_ctx *ctx);
long long bd_launch_count(bd_ctx *ctx);
int       bd_set_tuning(bd_ctx *ctx, int lz_cluster, int dy_cluster, double eta);
/* Autotuner: runs the batched step (flags as bd_run_all) for each candidate cluster size
 * of the Lanczos kernel (4, 8, 16) and, when a Dyson matrix exceeds order 160, of the
 * cluster Householder reduction (4, 8, 16), reps timed runs each after a warm-up, and
 * keeps the fastest by device time; the chosen sizes are returned. */
int       bd_autotune(bd_ctx *ctx, int flags, int reps, int *lz_cluster, int *dy_cluster);
/* stored[2 * ish + dir]: Lanczos vectors the last reduction of each chain actually
 * built (the other rows are the deflated tail of an exhausted Krylov space). */
int       bd_lanczos_stored(bd_ctx *ctx, int *stored);
/* Where the Lanczos kernel keeps each CTA's slice of the pole energies and of the
 * working vector: 0 = shared memory unless it would exceed 100 KB (default),
 * 1 = shared memory, 2 = global memory (for chains of any length). */
int       bd_set_lanczos_slices(bd_ctx *ctx, int mode);

/* ------------------------------------------------------------------------------
 * The reference's files.  A bd_files object holds, on the host, a problem read from
 * the reference's own input files; bd_upload_files puts it on a context.  Readers keep
 * what the reference's keep and report what it would warn about; a malformed file is
 * a status code (bd_files_error gives the message), never an exit.  The functions
 * below that take no context touch no GPU. */
typedef struct bd_files bd_files;

/* Model space file: ModSpace_t::ModSpace_t(char*), source/BcDor-Mod_Space.cpp:415-505.
 * *f is set (and must be closed) even when the file is refused. */
int  bd_files_open(bd_files **f, const char *modspace_path);
void bd_files_close(bd_files *f);
const char *bd_files_error(const bd_files *f);
/* Propagator file: SpProp_t::SpProp_t(char*, ModSpace_t*), source/BcDor-Sp_Propagator.cpp:
 * 387-610 (optional n1 / n2 / d1 columns read and dropped; amplitude rows of the model
 * space's largest subshell size, missing amplitudes zero; Z = the file's percentage / 100). */
int  bd_files_read_propagator(bd_files *f, const char *path);
/* Lanczos pivots file for every subshell: Make_LancPivots, source/BcDor-Miscellanea.cpp:334-390. */
int  bd_files_read_pivots(bd_files *f, const char *path);
/* Interaction: VppInt_t::read, source/BcDor-Vpp_potential.cpp:205-215 -- read_bin (:406-438)
 * for a name containing ".bin", else read_ascii (:281-375) on `threads` host threads
 * (0 = all): lines with an orbit outside the model space are skipped, Pauli-forbidden
 * ones (a == b or c == d at odd J) discarded; the kept lines stay in file order until
 * bd_upload_files puts them in canonical form on the device. */
int  bd_files_read_interaction(bd_files *f, const char *path, int threads);
/* Views of what was read (pointers into the object, valid until it is closed). */
int  bd_files_modspace(const bd_files *f, bd_modspace *ms, const int **orb_n, const char *const **names);
int  bd_files_propagator(const bd_files *f, bd_propagator *prop, const double **zp, const double **zh);
int  bd_files_pivots(const bd_files *f, bd_pivots *piv);
int  bd_files_interaction_lines(const bd_files *f, long long *kept, long long *outside, long long *pauli);

/* bd_upload_problem (and bd_upload_pivots, when pivots were read) from a files object.
 * The interaction becomes the list VppInt_t holds after Load_interaction
 * (source/BcDor-Initialize.cpp:110-117): read_ascii's canonical pairs and phases
 * (source/BcDor-Vpp_potential.cpp:330-356), prepare_for_reading's order (:440-501) and,
 * of repeated pairs, the first (check_for_double_entries, :663-702) -- built on the
 * device: one kernel per line forms the keys, a radix sort orders them, a scan places
 * the kept ones.  Among repeated pairs the reference keeps the one its heap sort puts
 * first; this build keeps the first in the file. */
int  bd_upload_files(bd_ctx *ctx, const bd_files *f);
/* The context's resident interaction list (cap elements per array; NULL arrays: counts
 * only); *n_repeated = repeated pairs left out of the last bd_upload_files. */
int  bd_interaction_fetch(bd_ctx *ctx, int *iabJ, int *icdJ, double *V, long long cap, long long *n_me,
                          long long *n_repeated);

/* Writers, in the reference's formats (subshell names from the model space file).
 * Propagator: SpProp_t::write with wcode 0, source/BcDor-Sp_Propagator.cpp:613-680;
 * zp / zh NULL: Z = sum of the squared amplitudes (what add_qp / add_qh store). */
int  bd_files_write_propagator(const bd_files *f, const char *path, const bd_propagator *prop, const double *zp,
                               const double *zh);
/* Pivots: SpProp_t::DysPivots(fname, n_bk, n_fw, z_cut), source/BcDor-Sp_Propagator.cpp:1225-1290. */
int  bd_files_write_pivots(const bd_files *f, const char *path, const bd_propagator *prop, const double *zp,
                           const double *zh, int n_fw, int n_bk, double z_cut);
/* Interaction: VppInt_t::write_bin, source/BcDor-Vpp_potential.cpp:377-404 (one interaction;
 * n_alloc = the allocation recorded in the header, <= 0: n_me). */
int  bd_write_interaction_bin(const char *path, const bd_interaction *vpp, long long n_alloc);
/* Self-energy of channel ish in binary form: Wide_self_energy_t::save_SelfEn_bin (fwbk > 0
 * forward only, < 0 backward only) and load_SelfEn_bin for one file,
 * source/BcDor-Self_energy_ext_Op_d.cpp:55-133,136-255.  Rows of nden + D doubles (nden = 2
 * for a plain Sigma(2), n_pvt + 1 for Lanczos rows with their i_piv arrays; NULL ipiv =
 * plain rows), as bd_dyson_rows takes them; the loader checks the header against the
 * model space and fills NULL-free buffers (ipiv: nden + D ints), sizes always. */
int  bd_files_save_selfenergy(const bd_files *f, const char *path, int ish, int nden, int n_fw, const double *fw_rows,
                              const int *ipiv_fw, int n_bk, const double *bk_rows, const int *ipiv_bk, int fwbk);
int  bd_files_load_selfenergy(const bd_files *f, const char *path, int ish, int *nden, int *n_fw, double *fw_rows,
                              int cap_fw, int *ipiv_fw, int *n_bk, double *bk_rows, int cap_bk, int *ipiv_bk);
/* The reference's name of that file: dir/label_Dyn_J2pi=<2j><+|->_dt=<charge>.bin
 * (Wide_self_energy_t::get_filename, source/BcDor-Self_energy_ext_Op_d.cpp:43-52). */
int  bd_files_selfenergy_name(const bd_files *f, const char *dir, const char *label, int ish, char *buf, int len);

/* Allocation-free Lanczos reduction of one pole set.  This entry point has no
 * counterpart in the reference.  It is for host programs that cannot let a
 * library call cudaMalloc: one whose own pool allocator has already reserved the
 * device's memory, or a latency-bound caller that cannot accept the device-wide
 * synchronisation cudaMalloc and cudaFree may imply.  It needs no context.
 *
 * The caller passes device buffers: d_E [N] pole energies and d_M [D][N]
 * couplings (column d of M at d_M + d * N), both in the order the chain should
 * visit them (the reference sorts them first), and d_rows, which receives L rows
 * of n_pvt + 1 + D doubles laid out as for bd_lanczos_reduce (cleared first).
 * pivots, n_itr, L_out and ipiv are host memory with bd_lanczos_reduce's meaning
 * and side effects.  flags: 0 = FP64, BD_RUN_MIXED = FP32 vectors.  stream is a
 * cudaStream_t (NULL = the legacy default stream) of the current device; the call
 * returns once the rows are written.  err (err_len bytes, may be NULL) receives a
 * message for any non-zero status.
 *
 * Scratch: a file-scope device array of BD_NOALLOC_SCRATCH_BYTES, held on every
 * device that loads the library until the process exits.  The Lanczos vectors
 * must fit in it with their companions: L * ld * 8 bytes (L * ld * 4 with
 * BD_RUN_MIXED, plus an FP32 copy of M, D * N * 4 bytes), ld = N + 64 rounded up to a
 * multiple of 32; the energy-group tables of the deflated tails, at most
 * 29 N + 1024 bytes; and the row slots, 4 L bytes; each part rounded up to 256
 * bytes, at most BD_NOALLOC_SCRATCH_BYTES - 4096 in all.  Larger chains are rejected
 * with BD_ERR_CAPACITY before anything is launched.  D <= 8 and n_pvt <= 9.
 * Every call looks up the array's device address on the current device (no set-up
 * call is needed).  All calls share the array, so calls that overlap on the GPU
 * (two streams, two host threads) race.  The call is synchronous and itself
 * allocates no device or pinned memory. */
#define BD_NOALLOC_SCRATCH_BYTES (16u << 20)
int bd_lanczos_chain_noalloc(const double *d_E, const double *d_M, int N, int D, int n_pvt,
                             double *pivots, int *n_itr, double *d_rows, int cap_rows, int *L_out,
                             int *ipiv, int flags, void *stream, char *err, int err_len);

#ifdef __cplusplus
}
#endif
#endif /* BD_GB300_H */
