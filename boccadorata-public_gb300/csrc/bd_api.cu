// bd_api.cu -- host orchestration and the extern "C" entry points of include/bd_gb300.h.
//
// The context keeps every input resident on the device and pre-computes, once
// per upload, the integer plan of the chain: the (Jab, ia, ib, ig) blocks of
// every channel in the reference's loop order (source/BcDor-Self_energy_ext_Op_c.cpp:
// 380-394), the pole offsets, and the buffer layout.  Both call patterns share the
// kernels:
//   * per channel (bd_sigma2_build / bd_lanczos_reduce / bd_dyson_solve), the
//     drop-in for the reference's three calls, one channel per launch;
//   * all channels at once (bd_run_all), one launch per phase over every channel.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <thread>
#include <unistd.h>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bd_gb300.h"
#include "bd_common.cuh"
#include "bd_kernels.h"

using namespace bd;

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

enum ChanState { ST_NONE = 0, ST_SIGMA = 1, ST_LANCZOS = 2 };

struct ChainPlan {     // one Lanczos direction of one channel
    int N = 0, L = 0, n_used = 0, nden_out = 0, n_pvt = 0;
    std::vector<int> nitr;         // rescaled, per pivot (all pivots)
    std::vector<int> start, last;  // per used pivot (+ sentinel in start)
    std::vector<double> piv;       // used pivots, normalised
    std::vector<int> used;         // indices of the pivots that start a chain
    std::vector<int> ipiv;         // [n_used, 1, last+1 ...] padded to nden_out + D with -100
};

struct Chan {
    int D = 0, j2 = 0, ch = 0;
    int nfw = 0, nbk = 0;
    long long fw_off = 0, bk_off = 0, mfw_off = 0, mbk_off = 0;
    int blk_first = 0, nblk = 0;
    long long vp_first = 0, nvp = 0;
    double efermi = 0.0;
    ChainPlan lz[2];
    // resident results of the per-channel API
    int state = ST_NONE;
    bool ref_sorted = false;   // the sort permutation holds the reference's order of equal energies
};

// Host array in page-locked memory (grown by reallocation, contents not kept), so a
// cudaMemcpyAsync from it neither blocks the host nor waits for the stream.  It is
// only regrown while no copy from it is pending.
template <typename T>
struct PinnedArray {
    T *p = nullptr;
    size_t n = 0, cap = 0;
    PinnedArray() = default;
    PinnedArray(const PinnedArray &) = delete;
    PinnedArray &operator=(const PinnedArray &) = delete;
    ~PinnedArray() {
        if (p) cudaFreeHost(p);
    }
    bool resize(size_t m) {
        if (m > cap) {
            if (p) cudaFreeHost(p);
            p = nullptr;
            const size_t c = std::max(m, cap + cap / 2);
            cap = 0;
            n = 0;
            void *q = nullptr;
            if (cudaMallocHost(&q, sizeof(T) * c) != cudaSuccess) return false;
            p = static_cast<T *>(q);
            cap = c;
        }
        n = m;
        return true;
    }
    size_t size() const { return n; }
    T &operator[](size_t i) { return p[i]; }
    const T &operator[](size_t i) const { return p[i]; }
};

// Page-locked staging of the small uploads: dupload copies a vector here and sends it
// with cudaMemcpyAsync, so the host runs on while the interaction is in flight (a copy
// from pageable memory waits for the stream).  Space is handed out between stream
// synchronisations and reclaimed after one; a full buffer is set aside (freed at the
// next reclaim) for a larger one.
struct HostStage {
    char *p = nullptr;
    size_t cap = 0, used = 0;
    std::vector<char *> retired;
    HostStage() = default;
    HostStage(const HostStage &) = delete;
    HostStage &operator=(const HostStage &) = delete;
    ~HostStage() {
        reclaim();
        if (p) cudaFreeHost(p);
    }
    void *take(size_t bytes, cudaStream_t st) {
        const size_t b = (bytes + 255) / 256 * 256;
        if (st && used + b > cap && cap >= ((size_t)64 << 20)) {   // a long run without a synchronisation
            cudaStreamSynchronize(st);
            reclaim();
        }
        if (used + b > cap) {
            if (p) retired.push_back(p);
            p = nullptr;
            const size_t c = std::max<size_t>(std::max(b, (size_t)1 << 20), 2 * cap);
            cap = 0;
            used = 0;
            void *q = nullptr;
            if (cudaMallocHost(&q, c) != cudaSuccess) return nullptr;
            p = static_cast<char *>(q);
            cap = c;
        }
        void *r = p + used;
        used += b;
        return r;
    }
    void reclaim() {   // every copy from the stage has completed
        used = 0;
        for (char *q : retired) cudaFreeHost(q);
        retired.clear();
    }
};

// A few host threads kept for the plan's per-channel passes (started on first use,
// joined with the context): run(n, fn) calls fn(i) for every i < n on the workers and
// the calling thread, and returns when all calls are done.  A forked child has none of
// the workers and runs the calls itself.
class HostPool {
public:
    ~HostPool() {
        if (getpid() != pid_) {
            for (auto &t : th_) t.detach();
            return;
        }
        {
            std::lock_guard<std::mutex> lk(m_);
            quit_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }
    void run(int n, const std::function<void(int)> &fn) {
        if (n <= 0) return;
        if (started_ && getpid() != pid_) {
            for (int i = 0; i < n; ++i) fn(i);
            return;
        }
        if (!started_) {
            started_ = true;
            pid_ = getpid();
            const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
            const int nw = (int)std::min(hw, 8u) - 1;
            for (int t = 0; t < nw; ++t) th_.emplace_back([this] { worker(); });
        }
        if (th_.empty() || n == 1) {
            for (int i = 0; i < n; ++i) fn(i);
            return;
        }
        {
            std::lock_guard<std::mutex> lk(m_);
            job_ = &fn;
            n_ = n;
            next_.store(0);
            active_ = (int)th_.size();
            ++gen_;
        }
        cv_.notify_all();
        for (int i; (i = next_.fetch_add(1)) < n;) fn(i);
        std::unique_lock<std::mutex> lk(m_);
        done_.wait(lk, [this] { return active_ == 0; });
        job_ = nullptr;
    }

private:
    void worker() {
        unsigned seen = 0;
        for (;;) {
            const std::function<void(int)> *job;
            int n;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return quit_ || gen_ != seen; });
                if (quit_) return;
                seen = gen_;
                job = job_;
                n = n_;
            }
            for (int i; (i = next_.fetch_add(1)) < n;) (*job)(i);
            std::lock_guard<std::mutex> lk(m_);
            if (--active_ == 0) done_.notify_one();
        }
    }
    std::vector<std::thread> th_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    const std::function<void(int)> *job_ = nullptr;
    int n_ = 0, active_ = 0;
    std::atomic<int> next_{0};
    unsigned gen_ = 0;
    bool quit_ = false, started_ = false;
    pid_t pid_ = 0;
};

}  // namespace

struct bd_ctx {
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[6] = {};
    cudaEvent_t ev_lz[2] = {};
    // the interaction's matrix elements go over on a second stream, after the index
    // lists, so the segment scan and the plan's uploads overlap their transfer
    cudaStream_t st_aux = nullptr;
    cudaEvent_t ev_up[2] = {};
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;   // the step's auxiliary branch (EHF)
    cudaEvent_t ev_fork2 = nullptr, ev_join2 = nullptr; // and its backward poles
    bool v_pending = false;
    bool v_checked = false;   // h_vcheck holds the check of the last interaction upload
    long long vpp_repeated = 0;   // repeated pairs left out of the last interaction read from a file
    bool lz_timed = false;
    double lz_kernel_ms = 0.0;
    long long launches = 0;   // kernels of this library launched since creation
    std::string err;
    bool uploaded = false, have_pivots = false;
    int lz_cluster = 8, dy_cluster = 8;
    int lz_slices = 0;   // Lanczos slices: 0 by size, 1 shared memory, 2 global memory
    double eta = 0.70710678118654752;
    // host copies of the inputs
    int nsubsh = 0, norb = 0, jmax = 0, nspb = 0;
    std::vector<int> l, j2, ip, ch, no, orb_start, orb_sh, np, nh, p_start, h_start;
    std::vector<double> orb_xe, ep, eh;
    std::vector<int> piv_npvt, piv_nfw, piv_nbk, piv_first;
    std::vector<double> piv_vec;
    // plan
    std::vector<Chan> chans;
    PinnedArray<S2Block> blocks;
    std::vector<std::vector<S2Block>> chan_blocks;   // per channel, before placement (kept for their capacity)
    std::vector<int> tc_blk;                         // block indices grouped for the tensor-core tiles
    std::vector<int4> tc_tiles;                      // (first in tc_blk, blocks, rows, -)
    std::vector<int> chan_chunks;
    HostPool pool_threads;
    PinnedArray<long long> blk_fw_first, blk_bk_first;
    PinnedArray<int> vchunk_first, vchunk_blk;   // V' gather: 32-coefficient chunks of each block
    HostStage stage;
    long long tot_fw = 0, tot_bk = 0, tot_mfw = 0, tot_mbk = 0, tot_vp = 0;
    // device: bufs follow the propagator, sbufs hold the model space and interaction
    std::vector<DevBuf> bufs, sbufs;
    std::vector<DevBuf> *cur = nullptr;   // where dalloc records (nullptr: bufs)
    bool static_ok = false;
    // interaction checks in flight: the segment scan's counters come back into a pinned
    // buffer while the host plans the propagator (finish_static reads them)
    bool static_pending = false;
    int *h_segcheck = nullptr;
    int *h_vcheck = nullptr;   // non-finite matrix elements found where they landed (index + 1, 0: none)
    int2 *pending_rows = nullptr;
    int *pending_prank = nullptr;
    int pending_nJ = 0;
    // freed buffers kept for reuse by size: a repeated upload of a problem of the same
    // shape allocates nothing (cudaMalloc / cudaFree synchronise the device)
    std::multimap<size_t, void *> pool;
    size_t pool_bytes = 0;
    DevProblem dp{};
    S2Block *d_blocks = nullptr;
    // tensor-core coupling build (k_coupling_tc.cu): blocks grouped by (ia, ib, ig, nJab)
    // into tiles of up to 128 rows; usable when every block's pair count fits
    int *d_tc_blk = nullptr;
    int4 *d_tc_tiles = nullptr;
    int ntc_tiles = 0, tc_np_fw = 0, tc_np_bk = 0;
    bool tc_ok = false;
    bool prop_dressed = false;   // some fragment has more than one non-zero amplitude
    bool last_tc = false;        // the last batched step built the couplings on the tensor cores
    bool tc_built = false;       // tensor-core tiles of the current plan uploaded
    int *d_vchunk_first = nullptr, *d_vchunk_blk = nullptr;
    long long *d_blk_fw_first = nullptr, *d_blk_bk_first = nullptr;
    ChanSig *d_cs = nullptr;
    double *d_vp = nullptr;
    double *d_Efw = nullptr, *d_S2fw = nullptr, *d_Mfw = nullptr, *d_Ebk = nullptr, *d_S2bk = nullptr, *d_Mbk = nullptr;
    double *d_Efw_s = nullptr, *d_Mfw_s = nullptr, *d_Ebk_s = nullptr, *d_Mbk_s = nullptr;  // sorted copies
    float *d_Mfw_f = nullptr, *d_Mbk_f = nullptr;                                           // FP32 sorted M
    int *d_seg_fw = nullptr, *d_seg_bk = nullptr, *d_idx_fw = nullptr, *d_idx_bk = nullptr, *d_perm_fw = nullptr,
        *d_perm_bk = nullptr;
    double *d_keys_tmp = nullptr;
    int *d_segoff_fw = nullptr, *d_segoff_bk = nullptr;
    int4 *d_chunks_fw = nullptr, *d_chunks_bk = nullptr;   // chunk tables of the shared-memory sort
    long long chunk_cap_fw = 0, chunk_cap_bk = 0;
    int *d_sorti_fw = nullptr, *d_sorti_bk = nullptr;       // its sorted indices
    unsigned long long *d_rkey[2] = {nullptr, nullptr};   // radix sort ping-pong buffers (long channels)
    unsigned *d_rval[2] = {nullptr, nullptr};
    void *d_rscratch = nullptr;
    double *d_sighf = nullptr, *d_sig1b = nullptr;  // per channel D*D at chan_dd_off
    double *d_efermi = nullptr;   // per channel: the Fermi energy of the input propagator (Seek_EFermi)
    bool ef_override = false;     // a per-channel Dyson call with the caller's Fermi energy
    bool last_update_on_device = false;
    std::vector<long long> chan_dd_off;
    long long *d_dd_off = nullptr;
    int3 *d_ehf_entries = nullptr;
    int n_ehf_entries = 0;
    // static self-energy: per entry its first term, per channel its (iv, J2) list
    std::vector<long long> ehf_term_first;
    long long *d_ehf_term_first = nullptr;
    int *d_ehf_cmb = nullptr, *d_ehf_toff = nullptr, *d_ehf_coff = nullptr, *d_ehf_ncomb = nullptr;
    double *d_ehf_terms = nullptr;
    // Lanczos
    std::vector<long long> lz_v_off[2], lz_out_off[2];
    char *d_lzV = nullptr;
    double *d_lzout = nullptr;
    int *d_lzint = nullptr;      // start / last / ipiv blocks
    double *d_lzpiv = nullptr;
    int *d_lzstat = nullptr;
    size_t lzV_bytes = 0;
    long long lzout_total = 0;
    std::vector<long long> lz_int_off[2], lz_piv_off[2], lz_slice_off[2], lz_grp_off[2], lz_slot_off[2];
    char *d_lzslice = nullptr;
    char *d_lzgrp = nullptr;     // per chain: energy groups and their Gram pieces (lz_group_bytes)
    int *d_lzslot = nullptr;     // per chain: vector slot of every row
    LzChain *d_chains = nullptr;
    int lz_two_pass = 0;
    // Dyson
    std::vector<long long> dy_A_off, dy_vec_off, dy_sol_off, dy_R_off, dy_work_off;
    double *d_dyA = nullptr, *d_dyvec = nullptr, *d_dysol = nullptr, *d_dykol = nullptr, *d_dyR = nullptr,
           *d_dywork = nullptr;
    long long *d_work_first = nullptr;
    size_t dyR_cap = 0, dywork_cap = 0;
    int *d_dynq = nullptr, *d_dystat = nullptr;
    DyJob *d_jobs = nullptr;
    long long *d_row_first = nullptr;
    size_t dyA_cap = 0, dyvec_cap = 0, dysol_cap = 0;
    int last_lanczos_flags = 0;
    bool results_valid = false;
    std::vector<int> res_nq;  // after run_all: 2 per channel
    double timings[5] = {0, 0, 0, 0, 0};
    // CUDA graphs of the batched step, one per run-flag combination: captured on first use,
    // replayed after; every change of the plan, the buffers or the tuning drops them.  While
    // a step is captured, the host tables it copies come from gstage (page-locked, kept as
    // long as the graphs: a replay reads them again).
    bool capturing = false;
    HostStage gstage;
    cudaGraphExec_t gexec[32] = {};
    long long glaunches[32] = {};
};

namespace {

int fail(bd_ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

// A failed runtime call is reported and the thread's last-error state cleared, so a
// non-sticky failure does not resurface in a later, unrelated call.
#define CU(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            cudaGetLastError();                                                                    \
            return fail(ctx, BD_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                 \
        }                                                                                          \
    } while (0)

constexpr size_t kPoolCap = (size_t)16 << 30;   // idle bytes the pool may hold

void drain_pool(bd_ctx *ctx) {
    for (auto &e : ctx->pool) cudaFree(e.second);
    ctx->pool.clear();
    ctx->pool_bytes = 0;
}

// Device bytes from the pool (same size) or from cudaMalloc, recorded in the current list.
int dmalloc(bd_ctx *ctx, void **q, size_t bytes) {
    *q = nullptr;
    auto it = ctx->pool.find(bytes);
    if (it != ctx->pool.end()) {
        *q = it->second;
        ctx->pool.erase(it);
        ctx->pool_bytes -= bytes;
    } else {
        cudaError_t e = cudaMalloc(q, bytes);
        if (e == cudaErrorMemoryAllocation && !ctx->pool.empty()) {
            cudaGetLastError();
            drain_pool(ctx);
            e = cudaMalloc(q, bytes);
        }
        if (e != cudaSuccess) return fail(ctx, BD_ERR_CUDA, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    }
    (ctx->cur ? *ctx->cur : ctx->bufs).push_back({*q, bytes});
    return BD_OK;
}

template <typename T>
int dalloc(bd_ctx *ctx, T **p, size_t count) {
    void *q = nullptr;
    const int rc = dmalloc(ctx, &q, sizeof(T) * (count > 0 ? count : 1));
    *p = reinterpret_cast<T *>(q);
    return rc;
}

template <typename T>
int dupload(bd_ctx *ctx, T **p, const std::vector<T> &h) {
    int rc = dalloc(ctx, p, h.size());
    if (rc) return rc;
    if (h.empty()) return BD_OK;
    const size_t bytes = sizeof(T) * h.size();
    void *st = ctx->stage.take(bytes, ctx->st);
    if (!st) return fail(ctx, BD_ERR_CUDA, "page-locked staging of %zu bytes", bytes);
    std::memcpy(st, h.data(), bytes);
    CU(cudaMemcpyAsync(*p, st, bytes, cudaMemcpyHostToDevice, ctx->st));
    return BD_OK;
}

template <typename T>
int dupload(bd_ctx *ctx, T **p, const PinnedArray<T> &h) {
    int rc = dalloc(ctx, p, h.size());
    if (rc) return rc;
    if (h.size()) CU(cudaMemcpyAsync(*p, h.p, sizeof(T) * h.size(), cudaMemcpyHostToDevice, ctx->st));
    return BD_OK;
}

// The main stream waits for the matrix elements' transfer.
int join_interaction(bd_ctx *ctx) {
    if (!ctx->v_pending) return BD_OK;
    ctx->v_pending = false;
    CU(cudaStreamWaitEvent(ctx->st, ctx->ev_up[1], 0));
    return BD_OK;
}

// Waits for the stream; the staging space is free again.
int sync_stream(bd_ctx *ctx) {
    CU(cudaStreamSynchronize(ctx->st));
    ctx->stage.reclaim();
    return BD_OK;
}

// A host table to the device on the context's stream.  While a step is being captured the
// source is first copied into the graphs' page-locked stage, which outlives the capture.
int h2d_table(bd_ctx *ctx, void *dst, const void *src, size_t bytes) {
    if (bytes == 0) return BD_OK;
    if (ctx->capturing) {
        void *p = ctx->gstage.take(bytes, nullptr);
        if (!p) return fail(ctx, BD_ERR_CUDA, "page-locked staging of %zu bytes", bytes);
        std::memcpy(p, src, bytes);
        src = p;
    }
    CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->st));
    return BD_OK;
}

// A timing event on the context's stream; during a capture it becomes an event-record
// node of the graph (recorded again at every replay), not a capture-internal marker.
cudaError_t record(bd_ctx *ctx, cudaEvent_t ev) {
    return cudaEventRecordWithFlags(ev, ctx->st, ctx->capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
}

// Drops the captured steps (their nodes hold buffer addresses and table contents).
void graph_invalidate(bd_ctx *ctx) {
    bool any = false;
    for (auto &g : ctx->gexec)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; any = true; }
    if (any && ctx->st) cudaStreamSynchronize(ctx->st);
    ctx->gstage.reclaim();
}

// Buffers of a list go back to the pool (beyond kPoolCap idle bytes: to the driver).
void release(bd_ctx *ctx, std::vector<DevBuf> &list) {
    graph_invalidate(ctx);
    if (ctx->st_aux) cudaStreamSynchronize(ctx->st_aux);
    ctx->v_pending = false;
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    ctx->stage.reclaim();
    for (auto &b : list) {
        if (ctx->pool_bytes + b.bytes <= kPoolCap) {
            ctx->pool.emplace(b.bytes, b.p);
            ctx->pool_bytes += b.bytes;
        } else {
            cudaFree(b.p);
        }
    }
    list.clear();
}

void free_all(bd_ctx *ctx) { release(ctx, ctx->bufs); }
void free_static(bd_ctx *ctx) { release(ctx, ctx->sbufs); }

// Allocations made while one of these is alive go to the given list.
struct BufScope {
    bd_ctx *c;
    std::vector<DevBuf> *saved;
    BufScope(bd_ctx *c_, std::vector<DevBuf> *to) : c(c_), saved(c_->cur) { c->cur = to; }
    ~BufScope() { c->cur = saved; }
};

// Seek_EFermi on the input propagator (source/BcDor-DysonMatrix.cpp:619-635).
double seek_efermi(const bd_ctx *c, int I) {
    const int chI = c->ch[I];
    double x1 = (c->ep.empty() ? 0.0 : c->ep[0]) + 100., x2 = (c->eh.empty() ? 0.0 : c->eh[0]) - 100.;
    for (int s = 0; s < c->nsubsh; ++s) {
        if (c->ch[s] != chI) continue;
        for (int k = 0; k < c->np[s]; ++k) if (c->ep[c->p_start[s] + k] < x1) x1 = c->ep[c->p_start[s] + k];
        for (int k = 0; k < c->nh[s]; ++k) if (c->eh[c->h_start[s] + k] > x2) x2 = c->eh[c->h_start[s] + k];
    }
    return (x1 + x2) / 2.0;
}

// Block enumeration in the loop order of Build_Dynamic_SlfEn_2ndOrder and the
// all-poles counts of Count_2p1h_2h1p_poles (source/BcDor-Self_energy_ext_Op_c.cpp:47-111,380-394).
int build_plan(bd_ctx *c) {
    const int ns = c->nsubsh;
    c->chans.assign(ns, Chan());
    // (ia <= ib) pairs satisfying the Jab triangle, in the reference's (ia, ib) order, kept
    // only when they can carry 2p1h (particles in both) or 2h1p (holes in both) poles
    struct Pair { int ia, ib, chs, ips, nJab; bool pfw, pbk; };
    std::vector<std::vector<Pair>> pairs(c->jmax + 1);
    for (int Jab = 0; Jab <= c->jmax; ++Jab)
        for (int ia = 0; ia < ns; ++ia)
            for (int ib = ia; ib < ns; ++ib) {
                if (tri_fail(c->j2[ia], c->j2[ib], 2 * Jab)) continue;
                const bool pfw = c->np[ia] > 0 && c->np[ib] > 0, pbk = c->nh[ia] > 0 && c->nh[ib] > 0;
                if (!pfw && !pbk) continue;
                pairs[Jab].push_back(Pair{ia, ib, c->ch[ia] + c->ch[ib], c->ip[ia] + c->ip[ib],
                                          std::abs((c->j2[ia] + c->j2[ib]) / 2 - Jab + 1) % 2, pfw, pbk});
            }
    // partner-shell buckets by (charge, parity); a charge outside the shells' range has none
    int chmin = INT_MAX, chmax = INT_MIN;
    for (int s = 0; s < ns; ++s) { chmin = std::min(chmin, c->ch[s]); chmax = std::max(chmax, c->ch[s]); }
    const int nkey = 2 * (chmax - chmin + 1);
    auto gkey = [&](int ch, int ip) { return (ch < chmin || ch > chmax) ? -1 : 2 * (ch - chmin) + ((ip % 2) + 2) % 2; };

    // Blocks of one channel, in the reference's (Jab, ia, ib, ig) order, with offsets
    // relative to the channel (fw_first, bk_first, vp_first); the channels are
    // independent and are enumerated on a few host threads.
    c->chan_blocks.resize(ns);
    c->chan_chunks.assign(ns, 0);
    auto channel = [&](int I) {
        std::vector<S2Block> &out = c->chan_blocks[I];
        out.clear();
        int chunks = 0;
        std::vector<std::vector<int>> gl(nkey), gh(nkey), gp(nkey);
        const int D = c->no[I];
        int nfw = 0, nbk = 0;
        long long vp = 0;
        for (int Jab = 0; Jab <= c->jmax; ++Jab) {
            // triangle-valid ig for (I, Jab), in ascending order, bucketed by (charge,
            // parity), since a pair (ia, ib) fixes both of its partner g: all of them,
            // those with holes (2p1h needs a hole in g) and those with particles (2h1p
            // needs a particle in g)
            for (auto &v : gl) v.clear();
            for (auto &v : gh) v.clear();
            for (auto &v : gp) v.clear();
            bool any = false;
            for (int ig = 0; ig < ns; ++ig) {
                if (tri_fail(c->j2[ig], c->j2[I], 2 * Jab)) continue;
                const int key = gkey(c->ch[ig], c->ip[ig]);
                any = true;
                gl[key].push_back(ig);
                if (c->nh[ig] > 0) gh[key].push_back(ig);
                if (c->np[ig] > 0) gp[key].push_back(ig);
            }
            if (!any) continue;
            const double x3 = std::sqrt((double)(Jab + Jab + 1) / (double)(1 + c->j2[I]));
            for (const Pair &pr : pairs[Jab]) {
                const int ia = pr.ia, ib = pr.ib, nJab = pr.nJab;
                // charge and parity of g: ch_a + ch_b - ch_g = ch_I, pi_a + pi_b + pi_g + pi_I even
                const int key = gkey(pr.chs - c->ch[I], pr.ips + c->ip[I]);
                if (key < 0) continue;
                const std::vector<int> &cand = (pr.pfw && pr.pbk) ? gl[key] : (pr.pfw ? gh[key] : gp[key]);
                for (int ig : cand) {
                    S2Block B{};
                    B.ch = I; B.Jab = Jab; B.ia = ia; B.ib = ib; B.ig = ig;
                    B.nJab = nJab;
                    B.nJgd = std::abs((c->j2[ig] + c->j2[I]) / 2 - Jab + 1) % 2;
                    int na = c->np[ia], nb = c->np[ib], ng = c->nh[ig], sz = na * nb * ng;
                    if (ia == ib) { nb = na + 1; if (nJab == 1) nb -= 2; sz = (na * nb / 2) * ng; }
                    B.nfw = sz;
                    na = c->nh[ia]; nb = c->nh[ib]; ng = c->np[ig]; sz = na * nb * ng;
                    if (ia == ib) { nb = na + 1; if (nJab == 1) nb -= 2; sz = (na * nb / 2) * ng; }
                    B.nbk = sz;
                    // blocks without poles add nothing to either list
                    if (B.nfw <= 0 && B.nbk <= 0) continue;
                    B.fw_first = nfw; B.bk_first = nbk;
                    B.vp_first = vp;
                    B.nvp = D * c->no[ia] * c->no[ib] * c->no[ig];
                    B.x3 = x3;
                    nfw += B.nfw; nbk += B.nbk; vp += B.nvp;
                    chunks += (B.nvp + 31) / 32;
                    out.push_back(B);
                }
            }
        }
        Chan &C = c->chans[I];
        C.D = D; C.j2 = c->j2[I]; C.ch = c->ch[I];
        C.nfw = nfw; C.nbk = nbk; C.nvp = vp;
        C.nblk = (int)out.size();
        C.efermi = seek_efermi(c, I);
        c->chan_chunks[I] = chunks;
    };
    c->pool_threads.run(ns, channel);
    // channel offsets (blocks, poles, couplings, coefficients and the V' gather's warps,
    // one per 32 coefficients of a block)
    long long fw = 0, bk = 0, mfw = 0, mbk = 0, vp = 0;
    size_t nb = 0;
    int nchunk = 0;
    std::vector<int> chunk_first(ns);
    for (int I = 0; I < ns; ++I) {
        Chan &C = c->chans[I];
        C.fw_off = fw; C.bk_off = bk; C.mfw_off = mfw; C.mbk_off = mbk;
        C.blk_first = (int)nb; C.vp_first = vp;
        chunk_first[I] = nchunk;
        fw += C.nfw; bk += C.nbk; mfw += (long long)C.nfw * C.D; mbk += (long long)C.nbk * C.D; vp += C.nvp;
        nb += c->chan_blocks[I].size();
        nchunk += c->chan_chunks[I];
    }
    if (!c->blocks.resize(nb) || !c->blk_fw_first.resize(nb) || !c->blk_bk_first.resize(nb) ||
        !c->vchunk_first.resize(nb + 1) || !c->vchunk_blk.resize((size_t)nchunk))
        return fail(c, BD_ERR_CUDA, "page-locked plan arrays of %zu blocks", nb);
    // the blocks at their global offsets, a channel per task
    c->pool_threads.run(ns, [&](int I) {
        const Chan &C = c->chans[I];
        const std::vector<S2Block> &cb = c->chan_blocks[I];
        int acc = chunk_first[I];
        for (size_t q = 0; q < cb.size(); ++q) {
            S2Block B = cb[q];
            B.fw_first += (int)C.fw_off;
            B.bk_first += (int)C.bk_off;
            B.vp_first += C.vp_first;
            const size_t b = (size_t)C.blk_first + q;
            c->blocks[b] = B;
            c->blk_fw_first[b] = B.fw_first;
            c->blk_bk_first[b] = B.bk_first;
            c->vchunk_first[b] = acc;
            const int k = (B.nvp + 31) / 32;
            std::fill(c->vchunk_blk.p + acc, c->vchunk_blk.p + acc + k, (int)b);
            acc += k;
        }
    });
    c->vchunk_first[nb] = nchunk;
    c->tot_fw = fw; c->tot_bk = bk; c->tot_mfw = mfw; c->tot_mbk = mbk; c->tot_vp = vp;
    c->tc_built = false;   // the tensor-core tiles follow on demand (build_tc_tiles)
    c->ntc_tiles = 0;
    return BD_OK;
}

// Lanczos sizes and pivot schedule of one direction (Reduce_SelfEn_Lncz
// source/BcDor-Self_energy_ext_Op_e.cpp:161-226 and Reduce_Mtx_Lncz source/BcDor-Lanczos.cpp:59-135,236-241).
// The pivots of the used chains are normalised in place in `piv` (the caller's
// working copy), as Reduce_Mtx_Lncz does (source/BcDor-Lanczos.cpp:129-132); the
// backward pass sees the vectors the forward pass already normalised.
void plan_chain(ChainPlan &P, int N, int D, int npvt, const int *nitr_in, double *piv) {
    P = ChainPlan();
    P.N = N; P.n_pvt = npvt; P.nden_out = npvt + 1;
    P.nitr.assign(nitr_in, nitr_in + npvt);
    P.ipiv.assign(P.nden_out + D, -100);
    long long tot = 0;
    for (int v : P.nitr) if (v > 0) tot += v;
    if (N < 1 || tot < 1) { P.L = 0; P.start.push_back(0); return; }
    if (tot > N) {
        const double x1 = (double)N / (double)tot;
        for (auto &v : P.nitr) v = (int)(x1 * v + 1.0);
    }
    long long nL = 0;
    for (int v : P.nitr) if (v > 0) nL += v;
    P.L = (int)std::min<long long>(nL, N);
    int jn = 0;
    for (int p = 0; p < npvt && jn < P.L; ++p) {
        if (P.nitr[p] < 1) continue;
        double x1 = 0.0;
        for (int i = 0; i < D; ++i) x1 += piv[(size_t)p * D + i] * piv[(size_t)p * D + i];
        x1 = std::sqrt(x1);
        for (int i = 0; i < D; ++i) piv[(size_t)p * D + i] /= x1;
        P.used.push_back(p);
        P.start.push_back(jn);
        jn += P.nitr[p];
        P.last.push_back(jn - 1);
        for (int i = 0; i < D; ++i) P.piv.push_back(piv[(size_t)p * D + i]);
    }
    P.n_used = (int)P.used.size();
    P.start.push_back(P.L);
    P.ipiv[0] = P.n_used;
    P.ipiv[1] = 1;
    for (int i = 0; i < P.n_used && 2 + i < (int)P.ipiv.size(); ++i) P.ipiv[2 + i] = P.last[i] + 1;
}

int check_chan(bd_ctx *ctx, int ish) {
    if (!ctx) return BD_ERR_ARG;
    if (!ctx->uploaded) return fail(ctx, BD_ERR_STATE, "no problem uploaded");
    if (ish < 0 || ish >= ctx->nsubsh) return fail(ctx, BD_ERR_ARG, "channel %d out of range", ish);
    return BD_OK;
}

// ---------------------------------------------------------------- Sigma(2)
// aux != nullptr: the backward poles go to that stream once the V' gather is done (their
// rows are independent of the forward ones); the caller joins it before the sort.
// Tensor-core tiles of the current plan (host grouping, then upload), built when a dressed
// propagator first asks for them: the blocks of every channel that share (ia, ib, ig,
// nJab) share the contraction's right-hand operand; their D rows are stacked, 128 to a tile.
int build_tc_tiles(bd_ctx *c) {
    const size_t nb = c->blocks.size();
    const long long ns = c->nsubsh;
    auto key = [&](int b) {
        const S2Block &B = c->blocks[b];
        return (size_t)((((long long)B.ia * ns + B.ib) * ns + B.ig) * 2 + (B.nJab ? 1 : 0));
    };
    // counting sort by key, stable (the plan's block order inside a group)
    std::vector<int> first((size_t)(ns * ns * ns * 2) + 1, 0);
    for (size_t b = 0; b < nb; ++b) ++first[key((int)b) + 1];
    for (size_t q = 1; q < first.size(); ++q) first[q] += first[q - 1];
    c->tc_blk.resize(nb);
    for (size_t b = 0; b < nb; ++b) c->tc_blk[first[key((int)b)]++] = (int)b;
    c->tc_tiles.clear();
    c->tc_np_fw = c->tc_np_bk = 0;
    c->tc_ok = true;
    for (size_t q = 0; q < nb;) {
        const int b0 = c->tc_blk[q];
        const S2Block &B = c->blocks[b0];
        if ((long long)c->no[B.ia] * c->no[B.ib] > 64 || B.nfw > 256 || B.nbk > 256) c->tc_ok = false;
        c->tc_np_fw = std::max(c->tc_np_fw, (B.nfw + 15) & ~15);
        c->tc_np_bk = std::max(c->tc_np_bk, (B.nbk + 15) & ~15);
        int rows = 0, n = 0;
        size_t e = q;
        while (e < nb && key(c->tc_blk[e]) == key(b0) && rows + c->no[c->blocks[c->tc_blk[e]].ch] <= 128) {
            rows += c->no[c->blocks[c->tc_blk[e]].ch];
            ++n;
            ++e;
        }
        if (n == 0) { c->tc_ok = false; break; }   // a block of more than 128 rows
        c->tc_tiles.push_back(int4{(int)q, n, rows, 0});
        q = e;
    }
    c->ntc_tiles = (int)c->tc_tiles.size();
    if (c->ntc_tiles > 0) {
        int rc;
        if ((rc = dupload(c, &c->d_tc_blk, c->tc_blk))) return rc;
        if ((rc = dupload(c, &c->d_tc_tiles, c->tc_tiles))) return rc;
    }
    c->tc_built = true;
    return BD_OK;
}

// tc: the couplings on the tensor cores (k_poles_tc, every channel at once); the energies
// are formed there too, with k_poles's operations.
int launch_sigma2(bd_ctx *ctx, int ch_lo, int ch_hi, cudaStream_t aux = nullptr, bool tc = false) {
    const Chan &A = ctx->chans[ch_lo], &Z = ctx->chans[ch_hi - 1];
    const int b0 = A.blk_first, nb = Z.blk_first + Z.nblk - b0;
    if (nb <= 0) {
        if (aux) {   // the join the caller waits for
            CU(cudaEventRecord(ctx->ev_fork2, ctx->st));
            CU(cudaStreamWaitEvent(aux, ctx->ev_fork2, 0));
            CU(cudaEventRecord(ctx->ev_join2, aux));
        }
        return BD_OK;
    }
    const long long vp0 = A.vp_first, nvp = Z.vp_first + Z.nvp - vp0;
    if (nvp > 0) {
        const int w0 = ctx->vchunk_first[b0], nw = ctx->vchunk_first[b0 + nb] - w0;
        k_vgather<<<(unsigned)((nw + 7) / 8), 256, 0, ctx->st>>>(ctx->dp, ctx->d_blocks, ctx->d_vchunk_blk,
                                                                  ctx->d_vchunk_first, w0, nw, ctx->d_vp);
        CU(cudaGetLastError());
        ctx->launches += 1;
    }
    const long long k0 = A.bk_off, nk = Z.bk_off + Z.nbk - k0;
    if (aux) {   // (launched before the forward poles so the two run side by side)
        CU(cudaEventRecord(ctx->ev_fork2, ctx->st));
        CU(cudaStreamWaitEvent(aux, ctx->ev_fork2, 0));
    }
    if (tc) {   // (all channels: the tiles mix them)
        for (int dir = 1; dir >= 0; --dir) {
            const int np = dir == 0 ? ctx->tc_np_fw : ctx->tc_np_bk;
            if (np == 0) continue;
            const size_t smem = tc_smem_bytes(np);
            cudaStream_t st = (dir == 1 && aux) ? aux : ctx->st;
            CU(launch_poles_tc(ctx->dp, ctx->d_blocks, ctx->d_tc_blk, ctx->d_tc_tiles, ctx->ntc_tiles, ctx->d_cs, dir,
                               ctx->d_vp, dir == 0 ? ctx->d_Efw : ctx->d_Ebk, dir == 0 ? ctx->d_S2fw : ctx->d_S2bk,
                               dir == 0 ? ctx->d_Mfw : ctx->d_Mbk, ctx->d_lzstat + 3, smem, st));
            ctx->launches += 1;
            if (dir == 1 && aux) CU(cudaEventRecord(ctx->ev_join2, aux));
        }
        if (aux && ctx->tc_np_bk == 0) CU(cudaEventRecord(ctx->ev_join2, aux));
        return BD_OK;
    }
    if (nk > 0) {
        k_poles<<<(unsigned)((nk + 127) / 128), 128, 0, aux ? aux : ctx->st>>>(ctx->dp, ctx->d_blocks + b0,
                                                                     ctx->d_blk_bk_first + b0, nb, k0, nk, ctx->d_cs,
                                                                     1, ctx->d_vp, ctx->d_Ebk, ctx->d_S2bk, ctx->d_Mbk);
        CU(cudaGetLastError());
        ctx->launches += 1;
    }
    if (aux) CU(cudaEventRecord(ctx->ev_join2, aux));
    const long long f0 = A.fw_off, nf = Z.fw_off + Z.nfw - f0;
    if (nf > 0) {
        k_poles<<<(unsigned)((nf + 127) / 128), 128, 0, ctx->st>>>(ctx->dp, ctx->d_blocks + b0,
                                                                     ctx->d_blk_fw_first + b0, nb, f0, nf, ctx->d_cs,
                                                                     0, ctx->d_vp, ctx->d_Efw, ctx->d_S2fw, ctx->d_Mfw);
        CU(cudaGetLastError());
        ctx->launches += 1;
    }
    return BD_OK;
}

int launch_ehf(bd_ctx *ctx, int ch_lo, int ch_hi, cudaStream_t st = nullptr) {
    if (!st) st = ctx->st;
    // entries of channels [ch_lo, ch_hi) are contiguous in d_ehf_entries
    int e0 = 0, e1 = 0, acc = 0;
    for (int I = 0; I < ctx->nsubsh; ++I) {
        const int cnt = ctx->no[I] * (ctx->no[I] + 1) / 2;
        if (I == ch_lo) e0 = acc;
        acc += cnt;
        if (I == ch_hi - 1) e1 = acc;
    }
    if (e1 > e0) {
        const long long nt = ctx->ehf_term_first[e1] - ctx->ehf_term_first[e0];
        if (nt > 0)
            k_ehf_terms<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(
                ctx->dp, ctx->d_ehf_entries, ctx->d_ehf_term_first, e0, e1, ctx->d_ehf_cmb, ctx->d_ehf_toff,
                ctx->d_ehf_coff, ctx->d_ehf_ncomb, ctx->d_ehf_terms);
        k_ehf_sum<<<e1 - e0, 256, 0, st>>>(ctx->dp, ctx->d_ehf_entries, ctx->d_ehf_term_first, e0, ctx->d_ehf_cmb,
                                                ctx->d_ehf_toff, ctx->d_ehf_coff, ctx->d_ehf_ncomb, ctx->d_ehf_terms,
                                                ctx->d_dd_off, ctx->d_sighf);
        CU(cudaGetLastError());
        ctx->launches += 2;
    }
    return BD_OK;
}

// Sort of each channel's poles by energy: forward ascending, backward descending (the
// orders Reduce_SelfEn_Lncz establishes, source/BcDor-Self_energy_ext_Op_e.cpp:119-130),
// then gather E and M into the sorted copies.  A stable sort runs first; with ref_order
// (the FP64 path) k_heap_order then puts equal energies in the order the reference's
// heap sorts leave them (source/BcDor-Utilities.cpp:25-94).
int launch_sort(bd_ctx *ctx, int ch_lo, int ch_hi, bool ref_order) {
    for (int dir = 0; dir < 2; ++dir) {
        const Chan &A = ctx->chans[ch_lo], &Z = ctx->chans[ch_hi - 1];
        const long long n0 = dir == 0 ? A.fw_off : A.bk_off;
        const long long n = (dir == 0 ? Z.fw_off + Z.nfw : Z.bk_off + Z.nbk) - n0;
        if (n <= 0) continue;
        std::vector<int> rel(ch_hi - ch_lo + 1);
        for (int I = ch_lo; I < ch_hi; ++I)
            rel[I - ch_lo] = (int)((dir == 0 ? ctx->chans[I].fw_off : ctx->chans[I].bk_off) - n0);
        rel[ch_hi - ch_lo] = (int)n;
        int *d_off = dir == 0 ? ctx->d_segoff_fw : ctx->d_segoff_bk;
        if (int rc = h2d_table(ctx, d_off, rel.data(), sizeof(int) * rel.size())) return rc;
        double *E = dir == 0 ? ctx->d_Efw : ctx->d_Ebk;
        int *perm = dir == 0 ? ctx->d_perm_fw : ctx->d_perm_bk;
        const int nseg = ch_hi - ch_lo;
        int seg_max = 0;
        for (int I = ch_lo; I < ch_hi; ++I) seg_max = std::max(seg_max, rel[I - ch_lo + 1] - rel[I - ch_lo]);
        cudaError_t e;
        if (seg_max <= kSortMax) {   // chunks sorted in shared memory, then ranked
            std::vector<int4> chunks;
            for (int I = ch_lo; I < ch_hi; ++I) {
                const int s0 = rel[I - ch_lo], sl = rel[I - ch_lo + 1] - s0;
                for (int c0 = 0; c0 < sl; c0 += kSortChunk) chunks.push_back(make_int4(s0 + c0, std::min(kSortChunk, sl - c0), s0, sl));
            }
            int4 *dch = dir == 0 ? ctx->d_chunks_fw : ctx->d_chunks_bk;
            if ((long long)chunks.size() > (dir == 0 ? ctx->chunk_cap_fw : ctx->chunk_cap_bk))
                return fail(ctx, BD_ERR_STATE, "sort chunk table overflow");
            if (int rc = h2d_table(ctx, dch, chunks.data(), sizeof(int4) * chunks.size())) return rc;
            unsigned long long *tk = reinterpret_cast<unsigned long long *>(ctx->d_keys_tmp);
            int *ti = dir == 0 ? ctx->d_sorti_fw : ctx->d_sorti_bk;
            k_chunk_sort<<<(unsigned)chunks.size(), kSortThreads, 0, ctx->st>>>(E + n0, dch, dir == 1, n0, tk, ti);
            k_chunk_place<<<(unsigned)((n + 255) / 256), 256, 0, ctx->st>>>(tk, ti, dch, (int)chunks.size(), n, n0,
                                                                          perm + n0);
            e = cudaGetLastError();
            ctx->launches += 2;
        } else {   // a channel beyond shared memory: radix sorts over the range
            int nl = 0;
            e = launch_pole_radix(E, dir == 0 ? ctx->d_seg_fw : ctx->d_seg_bk, ch_lo, nseg, n0, n, dir == 1,
                                  ctx->d_rkey[0], ctx->d_rval[0], ctx->d_rkey[1], ctx->d_rval[1], ctx->d_rscratch,
                                  perm, &nl, ctx->st);
            ctx->launches += nl;
        }
        CU(e);
        if (ref_order) {
            CU(launch_heap_order(E, d_off, nseg, seg_max, n0, perm, ctx->st));
            ctx->launches += 1;
        }
        k_permute_soa<<<(unsigned)((n + 255) / 256), 256, 0, ctx->st>>>(
            perm, n0, n, dir == 0 ? ctx->d_seg_fw : ctx->d_seg_bk, ctx->d_cs, dir, E, dir == 0 ? ctx->d_Mfw : ctx->d_Mbk,
            dir == 0 ? ctx->d_Efw_s : ctx->d_Ebk_s, dir == 0 ? ctx->d_Mfw_s : ctx->d_Mbk_s,
            dir == 0 ? ctx->d_Mfw_f : ctx->d_Mbk_f);
        CU(cudaGetLastError());
        ctx->launches += 1;
    }
    return BD_OK;
}

// Cluster size of a launch: the tuned size when many channels share the GPU; a
// channel launched alone (the per-channel call pattern) spreads each chain and each
// Dyson matrix over 16 CTAs, since its few clusters would otherwise leave most SMs idle.
int lz_cluster_for(const bd_ctx *ctx, int nch) { return nch == 1 ? std::max(ctx->lz_cluster, 16) : ctx->lz_cluster; }
int dy_cluster_for(const bd_ctx *ctx, int nch) { return nch == 1 ? std::max(ctx->dy_cluster, 16) : ctx->dy_cluster; }

// Lanczos chains of channels [ch_lo, ch_hi), both directions.
int launch_lanczos_range(bd_ctx *ctx, int ch_lo, int ch_hi, bool fp32) {
    const int CL = lz_cluster_for(ctx, ch_hi - ch_lo);
    std::vector<LzChain> ch;
    int Smax = 1, rmax = 1;
    for (int I = ch_lo; I < ch_hi; ++I) {
        Chan &C = ctx->chans[I];
        for (int dir = 0; dir < 2; ++dir) {
            ChainPlan &P = C.lz[dir];
            if (P.L <= 0) continue;
            LzChain z{};
            z.N = P.N; z.D = C.D; z.L = P.L; z.n_used = P.n_used; z.nden_out = P.nden_out;
            z.ld = lz_ld(P.N);
            z.S = ((P.N + CL - 1) / CL + 3) / 4 * 4;
            z.E = (dir == 0 ? ctx->d_Efw_s : ctx->d_Ebk_s) + (dir == 0 ? C.fw_off : C.bk_off);
            z.M = (dir == 0 ? ctx->d_Mfw_s : ctx->d_Mbk_s) + (dir == 0 ? C.mfw_off : C.mbk_off);
            z.Mf = (dir == 0 ? ctx->d_Mfw_f : ctx->d_Mbk_f) + (dir == 0 ? C.mfw_off : C.mbk_off);
            z.piv = ctx->d_lzpiv + ctx->lz_piv_off[dir][I];
            z.start = ctx->d_lzint + ctx->lz_int_off[dir][I];
            z.last = z.start + (P.n_used + 1);
            z.V = ctx->d_lzV + ctx->lz_v_off[dir][I];
            z.out = ctx->d_lzout + ctx->lz_out_off[dir][I];
            z.stat = ctx->d_lzstat;
            {
                char *g = ctx->d_lzgrp + ctx->lz_grp_off[dir][I];
                z.gE = reinterpret_cast<const double *>(g);
                z.gInfo = reinterpret_cast<const int *>(g + (size_t)16 * P.N);
                z.rowslot = ctx->d_lzslot + ctx->lz_slot_off[dir][I];
            }
            z.slice = ctx->d_lzslice + ctx->lz_slice_off[dir][I];
            z.slice_stride = ((long long)z.S * kLzSliceBytesPerPole + 255) / 256 * 256;
            if (reinterpret_cast<uintptr_t>(z.slice) % 256 != 0 ||
                z.slice_stride * CL > lz_slice_bytes(P.N))
                return fail(ctx, BD_ERR_STATE, "channel %d: Lanczos slice scratch misplaced", I);
            ch.push_back(z);
            Smax = std::max(Smax, z.S);
            rmax = std::max(rmax, P.L + 1);
        }
    }
    if (ch.empty()) return BD_OK;
    if (2 + 7 + 7 > 32) return fail(ctx, BD_ERR_ARG, "too many scalars");
    // Longest chains first so they start in the first wave: a chain's steps follow its
    // row count L (the built vectors and the deflated tail), its step cost depends
    // little on N (measured 1.81 -> 1.55 ms against ordering by N L^2)
    std::sort(ch.begin(), ch.end(), [](const LzChain &a, const LzChain &b) {
        if (a.L != b.L) return a.L > b.L;
        return a.N > b.N;
    });
    // The reference clears the output rows first (source/BcDor-Lanczos.cpp:88); the
    // kernel writes every element of every row itself (zeros where the reference's
    // stay), so no clearing pass is needed.
    // chain descriptors live in a small device array (one slot per chain of the range)
    LzChain *d_ch = ctx->d_chains + 2 * ch_lo;   // this range's own slots
    if (int rc = h2d_table(ctx, d_ch, ch.data(), sizeof(LzChain) * ch.size())) return rc;
    long long gram_cap = 0;
    for (const LzChain &z : ch) gram_cap += lz_gram_cap(z.N);
    CU(launch_lz_groups(d_ch, (int)ch.size(), gram_cap, ctx->st));   // energy groups for the deflated tails
    ctx->launches += 3;
    CU(record(ctx, ctx->ev_lz[0]));
    // chains whose slices do not fit next to the scalars keep them in global memory
    const bool gslices = ctx->lz_slices == 2 || (ctx->lz_slices == 0 && lanczos_smem_bytes(Smax, rmax) > kLanczosSmemSliceCap);
    if (!gslices && lanczos_smem_bytes(Smax, rmax) > (size_t)227 * 1024)
        return fail(ctx, BD_ERR_CAPACITY, "Lanczos slices of %d poles do not fit in shared memory", Smax);
    CU(launch_lanczos(d_ch, (int)ch.size(), Smax, rmax, fp32, CL, ctx->eta, gslices, ctx->st));
    CU(record(ctx, ctx->ev_lz[1]));
    ctx->lz_timed = true;
    ctx->launches += 1;
    return BD_OK;
}

int dyson_order(const bd_ctx *ctx, int I, bool lanczos) {
    const Chan &C = ctx->chans[I];
    return lanczos ? C.D + C.lz[0].L + C.lz[1].L : C.D + C.nfw + C.nbk;
}

// Scratch of every channel's Dyson problem at fixed offsets (no overlap between channels).
int ensure_dyson(bd_ctx *ctx, bool lanczos) {
    const int ns = ctx->nsubsh;
    ctx->dy_A_off.assign(ns, 0); ctx->dy_vec_off.assign(ns, 0); ctx->dy_sol_off.assign(ns, 0);
    ctx->dy_R_off.assign(ns, 0); ctx->dy_work_off.assign(ns, 0);
    size_t a = 0, v = 0, s = 0, r = 0, w = 0;
    for (int I = 0; I < ns; ++I) {
        const size_t n = (size_t)dyson_order(ctx, I, lanczos), D = ctx->chans[I].D;
        ctx->dy_A_off[I] = (long long)a; a += n * n;
        ctx->dy_vec_off[I] = (long long)v; v += 4 * n;   // d, e, tau, block bounds (2n ints)
        ctx->dy_sol_off[I] = (long long)s; s += n * (2 + D);
        ctx->dy_R_off[I] = (long long)r; r += D * n + n * (2 + D);
        ctx->dy_work_off[I] = (long long)w; w += 5 * n * n;
    }
    if (a > (size_t)2 << 30) return fail(ctx, BD_ERR_CAPACITY, "Dyson matrices need %.1f GB", a * 8.0 / 1e9);
    if (a > ctx->dyA_cap || v > ctx->dyvec_cap || s > ctx->dysol_cap || r > ctx->dyR_cap || w > ctx->dywork_cap) {
        graph_invalidate(ctx);
        CU(cudaStreamSynchronize(ctx->st));
        if (r > ctx->dyR_cap) {
            if (ctx->d_dyR) cudaFree(ctx->d_dyR);
            ctx->d_dyR = nullptr; ctx->dyR_cap = 0;
            CU(cudaMalloc(&ctx->d_dyR, sizeof(double) * r));
            ctx->dyR_cap = r;
        }
        if (w > ctx->dywork_cap) {
            if (ctx->d_dywork) cudaFree(ctx->d_dywork);
            ctx->d_dywork = nullptr; ctx->dywork_cap = 0;
            CU(cudaMalloc(&ctx->d_dywork, sizeof(double) * w));
            ctx->dywork_cap = w;
        }
        if (a > ctx->dyA_cap) {
            if (ctx->d_dyA) cudaFree(ctx->d_dyA);
            ctx->d_dyA = nullptr; ctx->dyA_cap = 0;
            CU(cudaMalloc(&ctx->d_dyA, sizeof(double) * a));
            ctx->dyA_cap = a;
        }
        if (v > ctx->dyvec_cap) {
            if (ctx->d_dyvec) cudaFree(ctx->d_dyvec);
            ctx->d_dyvec = nullptr; ctx->dyvec_cap = 0;
            CU(cudaMalloc(&ctx->d_dyvec, sizeof(double) * v));
            ctx->dyvec_cap = v;
        }
        if (s > ctx->dysol_cap) {
            if (ctx->d_dysol) cudaFree(ctx->d_dysol);
            ctx->d_dysol = nullptr; ctx->dysol_cap = 0;
            CU(cudaMalloc(&ctx->d_dysol, sizeof(double) * s));
            ctx->dysol_cap = s;
        }
    }
    return BD_OK;
}

// Dyson jobs of channels [ch_lo, ch_hi); ensure_dyson must have run for this mode.
int launch_dyson_range(bd_ctx *ctx, int ch_lo, int ch_hi, bool lanczos) {
    std::vector<DyJob> jobs;
    std::vector<long long> row_first;
    long long rows = 0;
    int nmax = 1, Dmax = 1;
    for (int I = ch_lo; I < ch_hi; ++I) {
        Chan &C = ctx->chans[I];
        DyJob J{};
        J.ch = I; J.D = C.D; J.j2 = C.j2;
        if (lanczos) {
            const ChainPlan &F = C.lz[0], &B = C.lz[1];
            J.nfw = F.L; J.nbk = B.L; J.nden = F.nden_out;
            J.lanczos_fw = F.L > 0; J.lanczos_bk = B.L > 0;
            J.fw_rows = ctx->d_lzout + ctx->lz_out_off[0][I];
            J.bk_rows = ctx->d_lzout + ctx->lz_out_off[1][I];
            J.ipiv_fw = ctx->d_lzint + ctx->lz_int_off[0][I] + 2 * (F.n_used + 1);
            J.ipiv_bk = ctx->d_lzint + ctx->lz_int_off[1][I] + 2 * (B.n_used + 1);
        } else {
            J.nfw = C.nfw; J.nbk = C.nbk; J.nden = 2;
            J.E_fw = ctx->d_Efw + C.fw_off; J.M_fw = ctx->d_Mfw + C.mfw_off;
            J.E_bk = ctx->d_Ebk + C.bk_off; J.M_bk = ctx->d_Mbk + C.mbk_off;
        }
        J.n = C.D + J.nfw + J.nbk;
        J.nc = J.n;   // k_dyson_deflate sets the order after deflation
        if (J.n != dyson_order(ctx, I, lanczos)) return fail(ctx, BD_ERR_STATE, "Dyson layout mismatch");
        J.sighf = ctx->d_sighf + ctx->chan_dd_off[I];
        J.sig1b = ctx->d_sig1b + ctx->chan_dd_off[I];
        J.efermi = C.efermi;
        J.efp = ctx->ef_override ? nullptr : ctx->d_efermi + I;
        J.A = ctx->d_dyA + ctx->dy_A_off[I];
        J.d = ctx->d_dyvec + ctx->dy_vec_off[I]; J.e = J.d + J.n; J.tau = J.e + J.n;
        J.blk = reinterpret_cast<int *>(J.tau + J.n);
        J.R = ctx->d_dyR + ctx->dy_R_off[I];
        J.sol = ctx->d_dysol + ctx->dy_sol_off[I];
        J.nq = ctx->d_dynq + 2 * I;
        J.koltun = ctx->d_dykol + 3 * I;
        J.stat = ctx->d_dystat + I;
        jobs.push_back(J);
        row_first.push_back(rows);
        rows += J.n;
        nmax = std::max(nmax, J.n);
        Dmax = std::max(Dmax, J.D);
    }
    if (Dmax > 8) return fail(ctx, BD_ERR_CAPACITY, "more than 8 orbitals in a channel");
    // descriptors at the channel's slot so per-channel launches never overwrite queued ones
    int rct;
    if ((rct = h2d_table(ctx, ctx->d_jobs + ch_lo, jobs.data(), sizeof(DyJob) * jobs.size()))) return rct;
    if ((rct = h2d_table(ctx, ctx->d_row_first + ch_lo, row_first.data(), sizeof(long long) * row_first.size()))) return rct;
    if ((rct = h2d_table(ctx, ctx->d_work_first + ch_lo, ctx->dy_work_off.data() + ch_lo, sizeof(long long) * jobs.size())))
        return rct;
    CU(launch_dyson(ctx->d_jobs + ch_lo, (int)jobs.size(), ctx->d_row_first + ch_lo, rows, nmax, Dmax,
                    dy_cluster_for(ctx, ch_hi - ch_lo), ctx->d_dywork, ctx->d_work_first + ch_lo, ctx->st));
    ctx->launches += dyson_launch_count(nmax);
    return BD_OK;
}

int alloc_lanczos(bd_ctx *ctx) {
    // descriptors, vectors, rows for every channel x direction
    size_t vbytes = 0;
    long long out = 0, ints = 0, pv = 0;
    for (int dir = 0; dir < 2; ++dir) {
        ctx->lz_v_off[dir].assign(ctx->nsubsh, 0);
        ctx->lz_out_off[dir].assign(ctx->nsubsh, 0);
        ctx->lz_int_off[dir].assign(ctx->nsubsh, 0);
        ctx->lz_piv_off[dir].assign(ctx->nsubsh, 0);
        ctx->lz_slice_off[dir].assign(ctx->nsubsh, 0);
        ctx->lz_grp_off[dir].assign(ctx->nsubsh, 0);
        ctx->lz_slot_off[dir].assign(ctx->nsubsh, 0);
    }
    long long slices = 0, groups = 0, slots = 0;
    std::vector<int> hints;
    std::vector<double> hpiv;
    for (int I = 0; I < ctx->nsubsh; ++I)
        for (int dir = 0; dir < 2; ++dir) {
            ChainPlan &P = ctx->chans[I].lz[dir];
            const int D = ctx->chans[I].D;
            ctx->lz_v_off[dir][I] = (long long)vbytes;
            vbytes += sizeof(double) * (size_t)std::max(P.L, 0) * lz_ld(P.N);
            vbytes = (vbytes + 255) / 256 * 256;
            ctx->lz_out_off[dir][I] = out;
            out += (long long)std::max(P.L, 0) * (P.nden_out + D);
            ctx->lz_slice_off[dir][I] = slices;
            if (P.L > 0) slices += lz_slice_bytes(P.N);
            ctx->lz_grp_off[dir][I] = groups;
            if (P.L > 0) groups += lz_group_bytes(P.N);
            ctx->lz_slot_off[dir][I] = slots;
            slots += std::max(P.L, 0);
            ctx->lz_int_off[dir][I] = ints;
            // start[n_used+1] | last[n_used+1] | ipiv[nden_out + D]
            std::vector<int> st = P.start, la = P.last;
            la.push_back(0);
            hints.insert(hints.end(), st.begin(), st.end());
            hints.insert(hints.end(), la.begin(), la.end());
            hints.insert(hints.end(), P.ipiv.begin(), P.ipiv.end());
            ints = (long long)hints.size();
            ctx->lz_piv_off[dir][I] = pv;
            hpiv.insert(hpiv.end(), P.piv.begin(), P.piv.end());
            pv = (long long)hpiv.size();
        }
    if (vbytes) {
        void *p = nullptr;
        int rc0 = dmalloc(ctx, &p, vbytes);
        if (rc0) return rc0;
        ctx->d_lzV = reinterpret_cast<char *>(p);
    }
    ctx->lzV_bytes = vbytes;
    ctx->lzout_total = out;
    int rc;
    if ((rc = dalloc(ctx, &ctx->d_lzout, (size_t)out))) return rc;
    if ((rc = dupload(ctx, &ctx->d_lzint, hints))) return rc;
    if ((rc = dupload(ctx, &ctx->d_lzpiv, hpiv))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_lzstat, 4))) return rc;
    CU(cudaMemsetAsync(ctx->d_lzstat, 0, sizeof(int) * 4, ctx->st));
    if ((rc = dalloc(ctx, &ctx->d_chains, (size_t)2 * ctx->nsubsh))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_lzslice, (size_t)slices))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_lzgrp, (size_t)groups))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_lzslot, (size_t)slots))) return rc;
    return BD_OK;
}

// Chain schedules of every channel from the stored pivots (pole counts may have
// changed with the propagator), then the Lanczos buffers.
int plan_pivots(bd_ctx *ctx) {
    graph_invalidate(ctx);
    size_t vo = 0;
    for (int I = 0; I < ctx->nsubsh; ++I) {
        const int D = ctx->no[I], npv = ctx->piv_npvt[I], p0 = ctx->piv_first[I];
        Chan &C = ctx->chans[I];
        std::vector<double> work(ctx->piv_vec.begin() + vo, ctx->piv_vec.begin() + vo + (size_t)npv * D);
        std::vector<int> nf(ctx->piv_nfw.begin() + p0, ctx->piv_nfw.begin() + p0 + npv);
        std::vector<int> nb(ctx->piv_nbk.begin() + p0, ctx->piv_nbk.begin() + p0 + npv);
        plan_chain(C.lz[0], C.nfw, D, npv, nf.data(), work.data());
        plan_chain(C.lz[1], C.nbk, D, npv, nb.data(), work.data());
        vo += (size_t)npv * D;
    }
    int rc = alloc_lanczos(ctx);
    if (rc) return rc;
    if ((rc = sync_stream(ctx))) return rc;
    ctx->have_pivots = true;
    return BD_OK;
}

// Model space and interaction: resident until the next bd_upload_problem (the
// Wide_self_energy_t's MdSp and Vpp, which Run_itrs keeps across iterations).
// Index of the first non-finite value of x[0 .. n), or -1.
long long first_nonfinite(const double *x, long long n) {
    if (!x) return -1;
    for (long long i = 0; i < n; ++i)
        if (!std::isfinite(x[i])) return i;
    return -1;
}

// Interaction lines read from a file (orbits, J, V in file order) on the host.
struct FileLines {
    const int4 *abcd = nullptr;
    const int *J = nullptr;
    const double *V = nullptr;
    long long n = 0;
};

// The canonical, sorted list of VppInt_t after Load_interaction (read_ascii's canonical
// pairs, prepare_for_reading's order, check_for_double_entries' first of each repeated
// pair; source/BcDor-Initialize.cpp:110-117) built on the device from file lines: a
// kernel forms each line's canonical keys and phase, the radix sort orders them (stable,
// so among repeated pairs the first in the file is kept), a scan places the kept ones.
// The model space must already be on the device (ctx->dp).  *pa / *pb / *pv are new
// resident arrays of *pn elements; *n_rep counts the repeated pairs left out.
int build_canonical(bd_ctx *ctx, const FileLines &fl, int **pa, int **pb, double **pv, long long *pn, long long *n_rep) {
    const long long n = fl.n;
    const DevProblem &P = ctx->dp;
    *pa = nullptr; *pb = nullptr; *pv = nullptr; *pn = 0; *n_rep = 0;
    if (n > (long long)INT_MAX / 2) return fail(ctx, BD_ERR_CAPACITY, "%lld interaction lines (at most %d)", n, INT_MAX / 2);
    if (ctx->norb > 1024) return fail(ctx, BD_ERR_CAPACITY, "%d orbits (the canonical keys hold 1024)", ctx->norb);
    std::vector<DevBuf> tmp;
    long long kept = 0;
    int rc;
    unsigned long long *k0 = nullptr;
    unsigned *v0 = nullptr, *pos = nullptr, *keep = nullptr;
    signed char *sg = nullptr;
    double *dV = nullptr;
    {
        BufScope scope(ctx, &tmp);
        int4 *dabcd;
        int *dJ, *bad;
        unsigned long long *k1;
        unsigned *v1;
        char *scratch;
        if ((rc = dalloc(ctx, &dabcd, (size_t)n)) || (rc = dalloc(ctx, &dJ, (size_t)n)) || (rc = dalloc(ctx, &dV, (size_t)n)) ||
            (rc = dalloc(ctx, &k0, (size_t)n)) || (rc = dalloc(ctx, &k1, (size_t)n)) || (rc = dalloc(ctx, &v0, (size_t)n)) ||
            (rc = dalloc(ctx, &v1, (size_t)n)) || (rc = dalloc(ctx, &sg, (size_t)n)) || (rc = dalloc(ctx, &keep, (size_t)n)) ||
            (rc = dalloc(ctx, &pos, (size_t)n)) || (rc = dalloc(ctx, &bad, 1)) ||
            (rc = dalloc(ctx, &scratch, std::max(radix_scratch_bytes(n), scan_scratch_bytes(n))))) {
            release(ctx, tmp);
            return rc;
        }
        if (n > 0) {
            CU(cudaMemcpyAsync(dabcd, fl.abcd, sizeof(int4) * n, cudaMemcpyHostToDevice, ctx->st));
            CU(cudaMemcpyAsync(dJ, fl.J, sizeof(int) * n, cudaMemcpyHostToDevice, ctx->st));
            CU(cudaMemcpyAsync(dV, fl.V, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->st));
        }
        CU(cudaMemsetAsync(bad, 0, sizeof(int), ctx->st));
        const unsigned nb = (unsigned)std::max<long long>(1, (n + 255) / 256);
        if (n > 0) {
            k_vpp_canon<<<nb, 256, 0, ctx->st>>>(dabcd, dJ, n, P.orb_sh, P.j2, P.ip, P.ch, k0, v0, sg, bad);
            CU(cudaGetLastError());
            ctx->launches += 1;
        }
        int passes = 0;
        CU(radix_sort_pairs(k0, v0, k1, v1, n, 0, 51, true, scratch, &passes, ctx->st));
        ctx->launches += radix_launches(passes, true);
        if (n > 0) {
            k_vpp_first<<<nb, 256, 0, ctx->st>>>(k0, n, keep);
            CU(cudaGetLastError());
            CU(cudaMemcpyAsync(pos, keep, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, ctx->st));
            CU(exclusive_scan_u32(pos, n, scratch, ctx->st));
            ctx->launches += 4;
        }
        int hbad = 0;
        unsigned last[2] = {0u, 0u};
        CU(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        if (n > 0) {
            CU(cudaMemcpyAsync(&last[0], pos + n - 1, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->st));
            CU(cudaMemcpyAsync(&last[1], keep + n - 1, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->st));
        }
        CU(cudaStreamSynchronize(ctx->st));
        if (hbad) {
            release(ctx, tmp);
            return fail(ctx, BD_ERR_ARG, "interaction line %d: charge, parity or J differ between its two pairs", hbad - 1);
        }
        kept = n > 0 ? (long long)last[0] + last[1] : 0;
        // the sorted pairs: k0 / v0 point at them after the sort (ping-pong buffers)
    }
    int *a, *b;
    double *v;
    if ((rc = dalloc(ctx, &a, (size_t)kept)) || (rc = dalloc(ctx, &b, (size_t)kept)) || (rc = dalloc(ctx, &v, (size_t)kept))) {
        release(ctx, tmp);
        return rc;
    }
    if (n > 0) {
        k_vpp_place<<<(unsigned)((n + 255) / 256), 256, 0, ctx->st>>>(k0, v0, pos, keep, n, dV, sg, a, b, v);
        CU(cudaGetLastError());
        ctx->launches += 1;
    }
    release(ctx, tmp);   // waits for the stream
    *pa = a; *pb = b; *pv = v; *pn = kept; *n_rep = n - kept;
    return BD_OK;
}

int upload_static(bd_ctx *ctx, const bd_modspace *ms, const bd_interaction *vpp, const FileLines *fl = nullptr) {
    const int ns = ms->nsubsh;
    ctx->v_checked = false;
    if (long long k = first_nonfinite(ms->orb_xe, ms->norb); k >= 0)
        return fail(ctx, BD_ERR_NUMERIC, "model space: xe of orbit %lld is not finite", k);
    ctx->nsubsh = ns; ctx->norb = ms->norb;
    ctx->l.assign(ms->l, ms->l + ns); ctx->j2.assign(ms->j2, ms->j2 + ns); ctx->ip.assign(ms->ip, ms->ip + ns);
    ctx->ch.assign(ms->ch, ms->ch + ns); ctx->no.assign(ms->no, ms->no + ns);
    ctx->orb_sh.assign(ms->orb_sh, ms->orb_sh + ms->norb);
    ctx->orb_xe.assign(ms->orb_xe, ms->orb_xe + ms->norb);
    ctx->jmax = 0;
    for (int s = 0; s < ns; ++s) {
        ctx->jmax = std::max(ctx->jmax, ctx->j2[s]);  // Calculate_Jch_bounds: Jmax = max 2j
        if (ctx->no[s] < 1 || ctx->no[s] > 8)
            return fail(ctx, BD_ERR_ARG, "subshell %d: %d orbits (1..8 supported)", s, ctx->no[s]);
        if (ctx->j2[s] < 1 || ctx->j2[s] % 2 != 1) return fail(ctx, BD_ERR_ARG, "subshell %d: 2j = %d", s, ctx->j2[s]);
    }
    if (ctx->jmax >= kJMult) return fail(ctx, BD_ERR_ARG, "2j too large");
    ctx->orb_start.assign(ns, 0);
    {
        int acc = 0;
        for (int s = 0; s < ns; ++s) { ctx->orb_start[s] = acc; acc += ctx->no[s]; }
        if (acc != ms->norb) return fail(ctx, BD_ERR_ARG, "sum of orbits %d != norb %d", acc, ms->norb);
        for (int o = 0; o < ms->norb; ++o)
            if (ctx->orb_sh[o] < 0 || ctx->orb_sh[o] >= ns) return fail(ctx, BD_ERR_ARG, "orbit %d: bad subshell", o);
    }
    int rc;
    DevProblem &P = ctx->dp;
    BufScope scope(ctx, &ctx->sbufs);   // resident buffers
    P.nsubsh = ns; P.norb = ctx->norb; P.jmax = ctx->jmax; P.n_me = fl ? 0 : vpp->n_me;
    int *t;
    double *td;
    if ((rc = dupload(ctx, &t, ctx->l))) return rc; P.l = t;
    if ((rc = dupload(ctx, &t, ctx->j2))) return rc; P.j2 = t;
    if ((rc = dupload(ctx, &t, ctx->ip))) return rc; P.ip = t;
    if ((rc = dupload(ctx, &t, ctx->ch))) return rc; P.ch = t;
    if ((rc = dupload(ctx, &t, ctx->no))) return rc; P.no = t;
    if ((rc = dupload(ctx, &t, ctx->orb_start))) return rc; P.orb_start = t;
    if ((rc = dupload(ctx, &t, ctx->orb_sh))) return rc; P.orb_sh = t;
    if ((rc = dupload(ctx, &td, ctx->orb_xe))) return rc; P.orb_xe = td;
    ctx->vpp_repeated = 0;
    if (fl) {   // from file lines: the canonical list is built on the device
        int *a, *b;
        double *v;
        long long nk = 0, nrep = 0;
        if ((rc = build_canonical(ctx, *fl, &a, &b, &v, &nk, &nrep))) return rc;
        P.iabJ = a; P.icdJ = b; P.V = v; P.n_me = (int)nk;
        ctx->vpp_repeated = nrep;
        if (nk > 0) {
            int *vbad = nullptr;
            if ((rc = dalloc(ctx, &vbad, 1))) return rc;
            if (!ctx->h_vcheck) CU(cudaMallocHost(&ctx->h_vcheck, sizeof(int)));
            CU(cudaMemsetAsync(vbad, 0, sizeof(int), ctx->st));
            CU(launch_nonfinite(v, nk, vbad, ctx->st));
            ctx->launches += 1;
            CU(cudaMemcpyAsync(ctx->h_vcheck, vbad, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
            ctx->v_checked = true;
        }
    } else {
        int *a, *b;
        double *v;
        if ((rc = dalloc(ctx, &a, vpp->n_me))) return rc;
        if ((rc = dalloc(ctx, &b, vpp->n_me))) return rc;
        if ((rc = dalloc(ctx, &v, vpp->n_me))) return rc;
        if (vpp->n_me > 0) {
            CU(cudaMemcpyAsync(a, vpp->iabJ, sizeof(int) * vpp->n_me, cudaMemcpyHostToDevice, ctx->st));
            CU(cudaMemcpyAsync(b, vpp->icdJ, sizeof(int) * vpp->n_me, cudaMemcpyHostToDevice, ctx->st));
            CU(cudaEventRecord(ctx->ev_up[0], ctx->st));
            CU(cudaStreamWaitEvent(ctx->st_aux, ctx->ev_up[0], 0));
            CU(cudaMemcpyAsync(v, vpp->V, sizeof(double) * vpp->n_me, cudaMemcpyHostToDevice, ctx->st_aux));
            // finiteness of the matrix elements, checked on the device where they land (a
            // host pass over them would cost more than their transfer)
            int *vbad = nullptr;
            if ((rc = dalloc(ctx, &vbad, 1))) return rc;
            if (!ctx->h_vcheck) CU(cudaMallocHost(&ctx->h_vcheck, sizeof(int)));
            CU(cudaMemsetAsync(vbad, 0, sizeof(int), ctx->st_aux));
            CU(launch_nonfinite(v, vpp->n_me, vbad, ctx->st_aux));
            ctx->launches += 1;
            CU(cudaMemcpyAsync(ctx->h_vcheck, vbad, sizeof(int), cudaMemcpyDeviceToHost, ctx->st_aux));
            CU(cudaEventRecord(ctx->ev_up[1], ctx->st_aux));
            ctx->v_checked = true;
            ctx->v_pending = true;
        }
        P.iabJ = a; P.icdJ = b; P.V = v;
    }
    const int n_me = P.n_me;
    // segment table of the sorted interaction, on the device (k_segments)
    {
        const std::vector<int> init(kSegTable, -10), zero(kSegTable + 3, 0);
        int *cnt, *sstr, *send;
        if ((rc = dupload(ctx, &sstr, init))) return rc; P.seg_str = sstr;
        if ((rc = dupload(ctx, &send, init))) return rc; P.seg_end = send;
        if ((rc = dupload(ctx, &cnt, zero))) return rc;
        int *bad = cnt + kSegTable;
        const int big[2] = {INT_MAX, 0};
        CU(cudaMemcpyAsync(bad, big, sizeof(big), cudaMemcpyHostToDevice, ctx->st));
        // row table: norb^2 (2jmax + 1) pairs of ints, skipped beyond 256 MiB
        int2 *rows = nullptr;
        const int nJ = ctx->jmax + 1;
        const size_t nrow = (size_t)ms->norb * ms->norb * nJ;
        int *prank = nullptr;
        if (n_me > 0 && nrow * sizeof(int2) <= ((size_t)256 << 20)) {
            if ((rc = dalloc(ctx, &rows, nrow))) return rc;
            if ((rc = dalloc(ctx, &prank, nrow))) return rc;
            CU(cudaMemsetAsync(rows, 0xff, sizeof(int2) * nrow, ctx->st));
            CU(cudaMemsetAsync(prank, 0xff, sizeof(int) * nrow, ctx->st));
        }
        if (n_me > 0) {
            k_segments<<<(unsigned)((n_me + 255) / 256), 256, 0, ctx->st>>>(
                P.iabJ, P.icdJ, n_me, ms->norb, P.orb_sh, P.ch, P.ip, sstr, send, cnt, bad, rows, nJ);
            CU(cudaGetLastError());
            ctx->launches += 1;
            if (prank) {
                k_pair_rank<<<(unsigned)((n_me + 255) / 256), 256, 0, ctx->st>>>(
                    P.iabJ, P.icdJ, n_me, ms->norb, P.orb_sh, P.ch, P.ip, sstr, nJ, prank);
                CU(cudaGetLastError());
                ctx->launches += 1;
            }
        }
        ctx->pending_prank = prank;
        if (!ctx->h_segcheck) CU(cudaMallocHost(&ctx->h_segcheck, sizeof(int) * (kSegTable + 3)));
        CU(cudaMemcpyAsync(ctx->h_segcheck, cnt, sizeof(int) * (kSegTable + 3), cudaMemcpyDeviceToHost, ctx->st));
        P.rows = nullptr;
        ctx->pending_rows = rows;
        ctx->pending_nJ = nJ;
        ctx->static_pending = true;
    }
    return BD_OK;
}

// Waits for the interaction's transfer and segment scan, then checks the list.
int finish_static(bd_ctx *ctx) {
    if (!ctx->static_pending) return BD_OK;
    ctx->static_pending = false;
    if (int rc = join_interaction(ctx)) return rc;
    CU(cudaStreamSynchronize(ctx->st));
    const int *h = ctx->h_segcheck;
    if (h[kSegTable] != INT_MAX)
        return fail(ctx, BD_ERR_ARG, "element %d: %s", h[kSegTable],
                    h[kSegTable + 1] == 1 ? "orbit out of range" : "bad channel key");
    for (int k = 0; k < kSegTable; ++k)
        if (h[k] > 1) return fail(ctx, BD_ERR_ARG, "interaction list not sorted by (ch, ip, J)");
    if (ctx->v_checked && *ctx->h_vcheck != 0)
        return fail(ctx, BD_ERR_NUMERIC, "interaction: matrix element %d is not finite", *ctx->h_vcheck - 1);
    ctx->dp.rows = (ctx->pending_rows && h[kSegTable + 2] == 0) ? ctx->pending_rows : nullptr;
    ctx->dp.prank = ctx->dp.rows ? ctx->pending_prank : nullptr;
    ctx->dp.nJ = ctx->pending_nJ;
    ctx->static_ok = true;
    return BD_OK;
}

// Propagator and everything that depends on it: fragments, the block plan, the
// pole buffers and the chain schedules (Wide_self_energy_t::reset with a new gin,
// source/BcDor-Main.cpp:225).
int upload_propagator(bd_ctx *ctx, const bd_propagator *prop) {
    const int ns = ctx->nsubsh;
    if (prop->nspb < 1) return fail(ctx, BD_ERR_ARG, "nspb = %d", prop->nspb);
    for (int s = 0; s < ns; ++s)
        if (ctx->no[s] > prop->nspb) return fail(ctx, BD_ERR_ARG, "subshell %d: %d orbits > nspb %d", s, ctx->no[s], prop->nspb);
    ctx->nspb = prop->nspb;
    ctx->np.assign(prop->np, prop->np + ns); ctx->nh.assign(prop->nh, prop->nh + ns);
    ctx->p_start.assign(ns, 0); ctx->h_start.assign(ns, 0);
    int nqp = 0, nqh = 0;
    for (int s = 0; s < ns; ++s) {
        if (ctx->np[s] < 0 || ctx->nh[s] < 0) return fail(ctx, BD_ERR_ARG, "negative fragment count");
        ctx->p_start[s] = nqp; ctx->h_start[s] = nqh; nqp += ctx->np[s]; nqh += ctx->nh[s];
    }
    if (long long k = first_nonfinite(prop->ep, nqp); k >= 0)
        return fail(ctx, BD_ERR_NUMERIC, "propagator: quasiparticle energy %lld is not finite", k);
    if (long long k = first_nonfinite(prop->eh, nqh); k >= 0)
        return fail(ctx, BD_ERR_NUMERIC, "propagator: quasihole energy %lld is not finite", k);
    if (long long k = first_nonfinite(prop->fqp, (long long)nqp * prop->nspb); k >= 0)
        return fail(ctx, BD_ERR_NUMERIC, "propagator: quasiparticle amplitude %lld is not finite", k);
    if (long long k = first_nonfinite(prop->fqh, (long long)nqh * prop->nspb); k >= 0)
        return fail(ctx, BD_ERR_NUMERIC, "propagator: quasihole amplitude %lld is not finite", k);
    ctx->ep.assign(prop->ep, prop->ep + nqp); ctx->eh.assign(prop->eh, prop->eh + nqh);
    ctx->prop_dressed = false;
    for (int side = 0; side < 2 && !ctx->prop_dressed; ++side) {
        const double *f = side == 0 ? prop->fqp : prop->fqh;
        const int nq = side == 0 ? nqp : nqh;
        for (int q = 0; q < nq && !ctx->prop_dressed; ++q) {
            int nz = 0;
            for (int o = 0; o < prop->nspb; ++o) nz += f[(size_t)q * prop->nspb + o] != 0.0;
            ctx->prop_dressed = nz > 1;
        }
    }
    std::vector<double> fqp(prop->fqp, prop->fqp + (size_t)nqp * prop->nspb);
    std::vector<double> fqh(prop->fqh, prop->fqh + (size_t)nqh * prop->nspb);
    int rc;
    if ((rc = build_plan(ctx))) return rc;
    DevProblem &P = ctx->dp;
    P.nspb = ctx->nspb;
    int *t;
    double *td;
    if ((rc = dupload(ctx, &t, ctx->np))) return rc; P.np = t;
    if ((rc = dupload(ctx, &t, ctx->nh))) return rc; P.nh = t;
    if ((rc = dupload(ctx, &t, ctx->p_start))) return rc; P.p_start = t;
    if ((rc = dupload(ctx, &t, ctx->h_start))) return rc; P.h_start = t;
    if ((rc = dupload(ctx, &td, ctx->ep))) return rc; P.ep = td;
    if ((rc = dupload(ctx, &td, ctx->eh))) return rc; P.eh = td;
    if ((rc = dupload(ctx, &td, fqp))) return rc; P.fqp = td;
    if ((rc = dupload(ctx, &td, fqh))) return rc; P.fqh = td;
    // plan arrays
    if ((rc = dupload(ctx, &ctx->d_blocks, ctx->blocks))) return rc;
    if ((rc = dupload(ctx, &ctx->d_vchunk_first, ctx->vchunk_first))) return rc;
    if ((rc = dupload(ctx, &ctx->d_vchunk_blk, ctx->vchunk_blk))) return rc;
    if ((rc = dupload(ctx, &ctx->d_blk_fw_first, ctx->blk_fw_first))) return rc;
    if ((rc = dupload(ctx, &ctx->d_blk_bk_first, ctx->blk_bk_first))) return rc;
    std::vector<ChanSig> cs(ns);
    std::vector<int> segoff_fw(ns + 1), segoff_bk(ns + 1);
    for (int I = 0; I < ns; ++I) {
        const Chan &C = ctx->chans[I];
        cs[I] = ChanSig{C.D, C.nfw, C.nbk, (int)C.fw_off, (int)C.bk_off, C.mfw_off, C.mbk_off};
        segoff_fw[I] = (int)C.fw_off; segoff_bk[I] = (int)C.bk_off;
    }
    segoff_fw[ns] = (int)ctx->tot_fw; segoff_bk[ns] = (int)ctx->tot_bk;
    if ((rc = dupload(ctx, &ctx->d_cs, cs))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_seg_fw, ctx->tot_fw))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_seg_bk, ctx->tot_bk))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_idx_fw, ctx->tot_fw))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_idx_bk, ctx->tot_bk))) return rc;
    // the channel of every pole and the identity order, on the device from the offsets
    // (the sort's per-range offsets overwrite these arrays later)
    if ((rc = dupload(ctx, &ctx->d_segoff_fw, segoff_fw))) return rc;
    if ((rc = dupload(ctx, &ctx->d_segoff_bk, segoff_bk))) return rc;
    if (ctx->tot_fw > 0) {
        k_pole_index<<<(unsigned)((ctx->tot_fw + 255) / 256), 256, 0, ctx->st>>>(ctx->d_segoff_fw, ns, ctx->tot_fw,
                                                                              ctx->d_seg_fw, ctx->d_idx_fw);
        CU(cudaGetLastError());
        ctx->launches += 1;
    }
    if (ctx->tot_bk > 0) {
        k_pole_index<<<(unsigned)((ctx->tot_bk + 255) / 256), 256, 0, ctx->st>>>(ctx->d_segoff_bk, ns, ctx->tot_bk,
                                                                              ctx->d_seg_bk, ctx->d_idx_bk);
        CU(cudaGetLastError());
        ctx->launches += 1;
    }
    ctx->chunk_cap_fw = ctx->tot_fw / kSortChunk + ns + 1;
    ctx->chunk_cap_bk = ctx->tot_bk / kSortChunk + ns + 1;
    if ((rc = dalloc(ctx, &ctx->d_chunks_fw, (size_t)ctx->chunk_cap_fw))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_chunks_bk, (size_t)ctx->chunk_cap_bk))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_sorti_fw, ctx->tot_fw))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_sorti_bk, ctx->tot_bk))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_perm_fw, ctx->tot_fw))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_perm_bk, ctx->tot_bk))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_keys_tmp, std::max(ctx->tot_fw, ctx->tot_bk)))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_vp, ctx->tot_vp))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_Efw, ctx->tot_fw))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_S2fw, ctx->tot_fw))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_Mfw, ctx->tot_mfw))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_Ebk, ctx->tot_bk))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_S2bk, ctx->tot_bk))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_Mbk, ctx->tot_mbk))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_Efw_s, ctx->tot_fw))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_Mfw_s, ctx->tot_mfw))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_Ebk_s, ctx->tot_bk))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_Mbk_s, ctx->tot_mbk))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_Mfw_f, ctx->tot_mfw))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_Mbk_f, ctx->tot_mbk))) return rc;
    {   // radix sort buffers, used when a channel exceeds the shared-memory chunk sort
        long long seg_max = 0;
        for (int I = 0; I < ns; ++I) seg_max = std::max<long long>(seg_max, std::max(ctx->chans[I].nfw, ctx->chans[I].nbk));
        const long long nr = seg_max > kSortMax ? std::max<long long>(1, std::max(ctx->tot_fw, ctx->tot_bk)) : 1;
        for (int b = 0; b < 2; ++b) {
            if ((rc = dalloc(ctx, &ctx->d_rkey[b], (size_t)nr))) return rc;
            if ((rc = dalloc(ctx, &ctx->d_rval[b], (size_t)nr))) return rc;
        }
        if ((rc = dalloc(ctx, reinterpret_cast<char **>(&ctx->d_rscratch), radix_scratch_bytes(nr)))) return rc;
    }
    // one-body (diag xe, Trel=7 ExtU1=1) and static self-energy, per channel D x D
    ctx->chan_dd_off.assign(ns, 0);
    std::vector<double> s1b;
    std::vector<int3> ent;
    for (int I = 0; I < ns; ++I) {
        const int D = ctx->no[I];
        ctx->chan_dd_off[I] = (long long)s1b.size();
        for (int r = 0; r < D; ++r)
            for (int c = 0; c < D; ++c) s1b.push_back(r == c ? ctx->orb_xe[ctx->orb_start[I] + r] : 0.0);
        for (int nc = 0; nc < D; ++nc)
            for (int nr = nc; nr < D; ++nr) ent.push_back(make_int3(I, nr, nc));
    }
    if ((rc = dupload(ctx, &ctx->d_sig1b, s1b))) return rc;
    {
        std::vector<double> ef(ns);
        for (int I = 0; I < ns; ++I) ef[I] = ctx->chans[I].efermi;
        if ((rc = dupload(ctx, &ctx->d_efermi, ef))) return rc;
    }
    if ((rc = dalloc(ctx, &ctx->d_sighf, s1b.size()))) return rc;
    if ((rc = dupload(ctx, &ctx->d_dd_off, ctx->chan_dd_off))) return rc;
    if ((rc = dupload(ctx, &ctx->d_ehf_entries, ent))) return rc;
    ctx->n_ehf_entries = (int)ent.size();
    {   // each channel's (iv, J2) combinations and the offsets of their no[iv]^2 terms
        std::vector<int> cmb, toff, coff(ns), ncomb(ns);
        std::vector<long long> terms_of(ns);
        for (int I = 0; I < ns; ++I) {
            coff[I] = (int)cmb.size();
            int acc = 0, c = 0;
            for (int iv = 0; iv < ns; ++iv) {
                const int lo = std::abs(ctx->j2[I] - ctx->j2[iv]);
                const int nJ2 = (ctx->j2[I] + ctx->j2[iv] - lo) / 2 + 1;
                for (int cc = 0; cc < nJ2; ++cc, ++c) {
                    cmb.push_back(iv | ((lo + 2 * cc) << 16));
                    toff.push_back(acc);
                    acc += ctx->no[iv] * ctx->no[iv];
                }
            }
            cmb.push_back(0);
            toff.push_back(acc);   // one past the last combination
            ncomb[I] = c;
            terms_of[I] = acc;
        }
        ctx->ehf_term_first.assign(ent.size() + 1, 0);
        for (size_t e = 0; e < ent.size(); ++e) ctx->ehf_term_first[e + 1] = ctx->ehf_term_first[e] + terms_of[ent[e].x];
        if ((rc = dupload(ctx, &ctx->d_ehf_term_first, ctx->ehf_term_first))) return rc;
        if ((rc = dupload(ctx, &ctx->d_ehf_cmb, cmb))) return rc;
        if ((rc = dupload(ctx, &ctx->d_ehf_toff, toff))) return rc;
        if ((rc = dupload(ctx, &ctx->d_ehf_coff, coff))) return rc;
        if ((rc = dupload(ctx, &ctx->d_ehf_ncomb, ncomb))) return rc;
        if ((rc = dalloc(ctx, &ctx->d_ehf_terms, (size_t)std::max(1LL, ctx->ehf_term_first.back())))) return rc;
    }
    // Dyson per-channel small outputs
    if ((rc = dalloc(ctx, &ctx->d_dynq, (size_t)2 * ns))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_dykol, (size_t)3 * ns))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_dystat, (size_t)ns))) return rc;
    CU(cudaMemsetAsync(ctx->d_dystat, 0, sizeof(int) * ns, ctx->st));
    if ((rc = dalloc(ctx, &ctx->d_jobs, (size_t)ns))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_row_first, (size_t)ns))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_work_first, (size_t)ns))) return rc;
    ctx->dy_sol_off.assign(ns, 0);
    ctx->res_nq.assign(2 * ns, 0);
    // everything above was queued behind the interaction's transfer; its checks now
    if (int rc0 = finish_static(ctx)) { ctx->static_ok = false; return rc0; }
    if ((rc = sync_stream(ctx))) return rc;
    ctx->uploaded = true;
    if (ctx->have_pivots) {
        ctx->have_pivots = false;
        if ((rc = plan_pivots(ctx))) return rc;
    }
    return BD_OK;
}

}  // namespace

// ============================================================================ C ABI
extern "C" {

int bd_version(void) { return 1; }

int bd_create(bd_ctx **out, int device) {
    if (!out) return BD_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return BD_ERR_CUDA;
    bd_ctx *ctx = new bd_ctx();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return BD_ERR_CUDA;
    }
    for (auto &e : ctx->ev) cudaEventCreate(&e);
    for (auto &e : ctx->ev_lz) cudaEventCreate(&e);
    for (auto &e : ctx->ev_up) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ctx->ev_fork2, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ctx->ev_join2, cudaEventDisableTiming);
    if (cudaStreamCreateWithFlags(&ctx->st_aux, cudaStreamNonBlocking) != cudaSuccess) {
        bd_destroy(ctx);
        return BD_ERR_CUDA;
    }
    // attribute queries and settings now, not inside a later stream capture
    tridiag_fit_warm();
    tc_smem_init();
    eig_smem_init();
    sigma2_smem_init();
    lanczos_smem_init();
    *out = ctx;
    return BD_OK;
}

void bd_destroy(bd_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    graph_invalidate(ctx);
    free_all(ctx);
    free_static(ctx);
    drain_pool(ctx);
    if (ctx->d_dyA) cudaFree(ctx->d_dyA);
    if (ctx->d_dyvec) cudaFree(ctx->d_dyvec);
    if (ctx->d_dysol) cudaFree(ctx->d_dysol);
    if (ctx->d_dyR) cudaFree(ctx->d_dyR);
    if (ctx->d_dywork) cudaFree(ctx->d_dywork);
    for (auto &e : ctx->ev) if (e) cudaEventDestroy(e);
    for (auto &e : ctx->ev_lz) if (e) cudaEventDestroy(e);
    for (auto &e : ctx->ev_up) if (e) cudaEventDestroy(e);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->ev_fork2) cudaEventDestroy(ctx->ev_fork2);
    if (ctx->ev_join2) cudaEventDestroy(ctx->ev_join2);
    if (ctx->h_segcheck) cudaFreeHost(ctx->h_segcheck);
    if (ctx->h_vcheck) cudaFreeHost(ctx->h_vcheck);
    if (ctx->st_aux) cudaStreamDestroy(ctx->st_aux);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
}

const char *bd_last_error(const bd_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }



int bd_upload_problem(bd_ctx *ctx, const bd_modspace *ms, const bd_interaction *vpp, const bd_propagator *prop) {
    if (!ctx || !ms || !vpp || !prop) return BD_ERR_ARG;
    if (ms->nsubsh < 1 || ms->norb < 1 || prop->nspb < 1 || vpp->n_me < 0) return fail(ctx, BD_ERR_ARG, "empty problem");
    CU(cudaSetDevice(ctx->device));
    free_all(ctx);
    free_static(ctx);
    ctx->uploaded = false; ctx->have_pivots = false; ctx->results_valid = false; ctx->static_ok = false;
    int rc = upload_static(ctx, ms, vpp);
    if (rc) {
        ctx->static_pending = false;
        join_interaction(ctx);
        cudaStreamSynchronize(ctx->st);
        return rc;
    }
    ctx->static_ok = true;   // for upload_propagator; finish_static confirms it or fails
    // the propagator's host plan runs while the interaction is in flight
    rc = upload_propagator(ctx, prop);
    const int rc2 = finish_static(ctx);   // no-op when upload_propagator already finished it
    if (rc) return rc;
    if (rc2) { ctx->static_ok = false; ctx->uploaded = false; return rc2; }
    return BD_OK;
}

// bd_upload_problem from a files object: the interaction's canonical list is built on
// the device from the file's lines (build_canonical), then as bd_upload_problem; the
// pivots too when the object holds them.
int bd_upload_files(bd_ctx *ctx, const bd_files *f) {
    if (!ctx || !f) return BD_ERR_ARG;
    bd_modspace ms;
    bd_propagator prop;
    if (bd_files_modspace(f, &ms, nullptr, nullptr) != BD_OK) return fail(ctx, BD_ERR_STATE, "files: no model space");
    if (bd_files_propagator(f, &prop, nullptr, nullptr) != BD_OK) return fail(ctx, BD_ERR_STATE, "files: no propagator read");
    FileLines fl;
    if (!files_interaction(f, &fl.abcd, &fl.J, &fl.V, &fl.n)) return fail(ctx, BD_ERR_STATE, "files: no interaction read");
    CU(cudaSetDevice(ctx->device));
    free_all(ctx);
    free_static(ctx);
    ctx->uploaded = false; ctx->have_pivots = false; ctx->results_valid = false; ctx->static_ok = false;
    const bd_interaction none{0, nullptr, nullptr, nullptr};
    int rc = upload_static(ctx, &ms, &none, &fl);
    if (rc) {
        ctx->static_pending = false;
        join_interaction(ctx);
        cudaStreamSynchronize(ctx->st);
        return rc;
    }
    ctx->static_ok = true;
    rc = upload_propagator(ctx, &prop);
    const int rc2 = finish_static(ctx);
    if (rc) return rc;
    if (rc2) { ctx->static_ok = false; ctx->uploaded = false; return rc2; }
    bd_pivots piv;
    if (bd_files_pivots(f, &piv) == BD_OK) return bd_upload_pivots(ctx, &piv);
    return BD_OK;
}

int bd_interaction_fetch(bd_ctx *ctx, int *iabJ, int *icdJ, double *V, long long cap, long long *n_me,
                         long long *n_repeated) {
    if (!ctx) return BD_ERR_ARG;
    if (!ctx->static_ok) return fail(ctx, BD_ERR_STATE, "no interaction uploaded");
    CU(cudaSetDevice(ctx->device));
    const long long n = ctx->dp.n_me;
    if (n_me) *n_me = n;
    if (n_repeated) *n_repeated = ctx->vpp_repeated;
    if ((iabJ || icdJ || V) && cap < n) return fail(ctx, BD_ERR_CAPACITY, "%lld elements, room for %lld", n, cap);
    CU(cudaStreamSynchronize(ctx->st));
    if (n > 0) {
        if (iabJ) CU(cudaMemcpy(iabJ, ctx->dp.iabJ, sizeof(int) * n, cudaMemcpyDeviceToHost));
        if (icdJ) CU(cudaMemcpy(icdJ, ctx->dp.icdJ, sizeof(int) * n, cudaMemcpyDeviceToHost));
        if (V) CU(cudaMemcpy(V, ctx->dp.V, sizeof(double) * n, cudaMemcpyDeviceToHost));
    }
    return BD_OK;
}

int bd_upload_propagator(bd_ctx *ctx, const bd_propagator *prop) {
    if (!ctx || !prop) return BD_ERR_ARG;
    if (!ctx->static_ok) return fail(ctx, BD_ERR_STATE, "no model space / interaction uploaded");
    CU(cudaSetDevice(ctx->device));
    free_all(ctx);
    ctx->uploaded = false; ctx->results_valid = false;
    return upload_propagator(ctx, prop);
}


int bd_upload_pivots(bd_ctx *ctx, const bd_pivots *piv) {
    if (!ctx || !piv) return BD_ERR_ARG;
    if (!ctx->uploaded) return fail(ctx, BD_ERR_STATE, "no problem uploaded");
    CU(cudaSetDevice(ctx->device));
    ctx->piv_npvt.assign(piv->npvt, piv->npvt + ctx->nsubsh);
    ctx->piv_first.assign(ctx->nsubsh + 1, 0);
    int tot = 0;
    size_t vtot = 0;
    for (int s = 0; s < ctx->nsubsh; ++s) {
        if (ctx->piv_npvt[s] < 0 || ctx->piv_npvt[s] > 9)
            return fail(ctx, BD_ERR_ARG, "subshell %d: %d pivots", s, ctx->piv_npvt[s]);
        ctx->piv_first[s] = tot; tot += ctx->piv_npvt[s]; vtot += (size_t)ctx->piv_npvt[s] * ctx->no[s];
    }
    ctx->piv_first[ctx->nsubsh] = tot;
    if (long long k = first_nonfinite(piv->vec, (long long)vtot); k >= 0)
        return fail(ctx, BD_ERR_NUMERIC, "pivots: element %lld is not finite", k);
    ctx->piv_nfw.assign(piv->n_itr_fw, piv->n_itr_fw + tot);
    ctx->piv_nbk.assign(piv->n_itr_bk, piv->n_itr_bk + tot);
    ctx->piv_vec.assign(piv->vec, piv->vec + vtot);
    ctx->have_pivots = false;
    return plan_pivots(ctx);
}

int bd_count_poles(bd_ctx *ctx, int ish, int *n_fw, int *n_bk) {
    int rc = check_chan(ctx, ish);
    if (rc) return rc;
    if (n_fw) *n_fw = ctx->chans[ish].nfw;
    if (n_bk) *n_bk = ctx->chans[ish].nbk;
    return BD_OK;
}

int bd_ehf(bd_ctx *ctx, int ish, double *sig_hf) {
    int rc = check_chan(ctx, ish);
    if (rc) return rc;
    CU(cudaSetDevice(ctx->device));
    if ((rc = launch_ehf(ctx, ish, ish + 1))) return rc;
    const int D = ctx->chans[ish].D;
    if (sig_hf)
        CU(cudaMemcpyAsync(sig_hf, ctx->d_sighf + ctx->chan_dd_off[ish], sizeof(double) * D * D,
                           cudaMemcpyDeviceToHost, ctx->st));
    CU(cudaStreamSynchronize(ctx->st));
    return BD_OK;
}

int bd_sigma2_build(bd_ctx *ctx, int ish, double *sig_fw, int cap_fw, int *n_fw, double *sig_bk, int cap_bk,
                    int *n_bk) {
    int rc = check_chan(ctx, ish);
    if (rc) return rc;
    CU(cudaSetDevice(ctx->device));
    Chan &C = ctx->chans[ish];
    if (n_fw) *n_fw = C.nfw;
    if (n_bk) *n_bk = C.nbk;
    if (sig_fw && cap_fw < C.nfw) return fail(ctx, BD_ERR_CAPACITY, "sig_fw holds %d rows, %d needed", cap_fw, C.nfw);
    if (sig_bk && cap_bk < C.nbk) return fail(ctx, BD_ERR_CAPACITY, "sig_bk holds %d rows, %d needed", cap_bk, C.nbk);
    if ((rc = launch_sigma2(ctx, ish, ish + 1))) return rc;
    for (int dir = 0; dir < 2; ++dir) {
        double *host = dir == 0 ? sig_fw : sig_bk;
        const int N = dir == 0 ? C.nfw : C.nbk;
        if (!host || N == 0) continue;
        double *tmp = nullptr;  // AoS staging in the reference's row layout
        CU(cudaMallocAsync(&tmp, sizeof(double) * (size_t)N * (2 + C.D), ctx->st));
        k_rows_aos<<<(N + 255) / 256, 256, 0, ctx->st>>>(
            (dir == 0 ? ctx->d_Efw + C.fw_off : ctx->d_Ebk + C.bk_off),
            (dir == 0 ? ctx->d_S2fw + C.fw_off : ctx->d_S2bk + C.bk_off),
            (dir == 0 ? ctx->d_Mfw + C.mfw_off : ctx->d_Mbk + C.mbk_off), N, C.D, tmp);
        CU(cudaGetLastError());
        CU(cudaMemcpyAsync(host, tmp, sizeof(double) * (size_t)N * (2 + C.D), cudaMemcpyDeviceToHost, ctx->st));
        CU(cudaFreeAsync(tmp, ctx->st));
    }
    CU(cudaStreamSynchronize(ctx->st));
    C.state = ST_SIGMA;
    return BD_OK;
}

int bd_sigma2_sorted(bd_ctx *ctx, int ish, double *sig_fw, int cap_fw, double *sig_bk, int cap_bk) {
    int rc = check_chan(ctx, ish);
    if (rc) return rc;
    CU(cudaSetDevice(ctx->device));
    Chan &C = ctx->chans[ish];
    if (C.state < ST_LANCZOS) return fail(ctx, BD_ERR_STATE, "channel %d: no Lanczos reduction (no sorted poles)", ish);
    if (!C.ref_sorted) {   // the reference's order of this channel's equal energies, on demand
        if ((rc = launch_sort(ctx, ish, ish + 1, true))) return rc;
        C.ref_sorted = true;
    }
    if (sig_fw && cap_fw < C.nfw) return fail(ctx, BD_ERR_CAPACITY, "sig_fw holds %d rows, %d needed", cap_fw, C.nfw);
    if (sig_bk && cap_bk < C.nbk) return fail(ctx, BD_ERR_CAPACITY, "sig_bk holds %d rows, %d needed", cap_bk, C.nbk);
    for (int dir = 0; dir < 2; ++dir) {
        double *host = dir == 0 ? sig_fw : sig_bk;
        const int N = dir == 0 ? C.nfw : C.nbk;
        if (!host || N == 0) continue;
        const long long off = dir == 0 ? C.fw_off : C.bk_off;
        double *tmp = nullptr;
        CU(cudaMallocAsync(&tmp, sizeof(double) * (size_t)N * (2 + C.D), ctx->st));
        k_rows_aos_perm<<<(N + 255) / 256, 256, 0, ctx->st>>>(
            dir == 0 ? ctx->d_perm_fw : ctx->d_perm_bk, off, (dir == 0 ? ctx->d_Efw : ctx->d_Ebk) + off,
            (dir == 0 ? ctx->d_S2fw : ctx->d_S2bk) + off, (dir == 0 ? ctx->d_Mfw + C.mfw_off : ctx->d_Mbk + C.mbk_off),
            N, C.D, tmp);
        CU(cudaGetLastError());
        ctx->launches += 1;
        CU(cudaMemcpyAsync(host, tmp, sizeof(double) * (size_t)N * (2 + C.D), cudaMemcpyDeviceToHost, ctx->st));
        CU(cudaFreeAsync(tmp, ctx->st));
    }
    CU(cudaStreamSynchronize(ctx->st));
    return BD_OK;
}

int bd_lanczos_reduce(bd_ctx *ctx, int ish, int n_pvt, double *pivots, int *n_itr_fw, int *n_itr_bk,
                      double *lz_fw, int cap_fw, int *L_fw, int *ipiv_fw,
                      double *lz_bk, int cap_bk, int *L_bk, int *ipiv_bk, int flags) {
    int rc = check_chan(ctx, ish);
    if (rc) return rc;
    CU(cudaSetDevice(ctx->device));
    Chan &C = ctx->chans[ish];
    if (C.state < ST_SIGMA) return fail(ctx, BD_ERR_STATE, "channel %d: no Sigma(2) built", ish);
    if (n_pvt < 0 || (n_pvt > 0 && (!pivots || !n_itr_fw || !n_itr_bk))) return fail(ctx, BD_ERR_ARG, "pivots");
    if (n_pvt > 9) return fail(ctx, BD_ERR_ARG, "too many pivots (%d, at most 9)", n_pvt);
    if (flags & ~(BD_RUN_MIXED | BD_RUN_REF_ORDER)) return fail(ctx, BD_ERR_ARG, "flags 0x%x", flags);
    if (n_pvt > 0 && first_nonfinite(pivots, (long long)n_pvt * C.D) >= 0)
        return fail(ctx, BD_ERR_NUMERIC, "channel %d: a pivot element is not finite", ish);
    // (re)plan this channel with the caller's pivots; same side effects as the reference:
    // started pivots normalised in place, iteration counts rescaled in place
    ChainPlan F, B;
    plan_chain(F, C.nfw, C.D, n_pvt, n_itr_fw, pivots);
    plan_chain(B, C.nbk, C.D, n_pvt, n_itr_bk, pivots);
    if (F.L > 0) for (int p = 0; p < n_pvt; ++p) n_itr_fw[p] = F.nitr[p];
    if (B.L > 0) for (int p = 0; p < n_pvt; ++p) n_itr_bk[p] = B.nitr[p];
    if (L_fw) *L_fw = F.L;
    if (L_bk) *L_bk = B.L;
    if (lz_fw && cap_fw < F.L) return fail(ctx, BD_ERR_CAPACITY, "lz_fw holds %d rows, %d needed", cap_fw, F.L);
    if (lz_bk && cap_bk < B.L) return fail(ctx, BD_ERR_CAPACITY, "lz_bk holds %d rows, %d needed", cap_bk, B.L);
    // the resident layout was sized from the uploaded pivots; a different layout needs a fresh plan
    if (!ctx->have_pivots || C.lz[0].L != F.L || C.lz[1].L != B.L || C.lz[0].nden_out != F.nden_out ||
        C.lz[0].n_used != F.n_used || C.lz[1].n_used != B.n_used)
        return fail(ctx, BD_ERR_STATE, "channel %d: pivots differ in shape from the uploaded ones", ish);
    C.lz[0] = F; C.lz[1] = B;
    graph_invalidate(ctx);
    // refresh this channel's schedule / pivots on the device
    for (int dir = 0; dir < 2; ++dir) {
        const ChainPlan &P = C.lz[dir];
        std::vector<int> ints = P.start, la = P.last;
        la.push_back(0);
        ints.insert(ints.end(), la.begin(), la.end());
        ints.insert(ints.end(), P.ipiv.begin(), P.ipiv.end());
        CU(cudaMemcpyAsync(ctx->d_lzint + ctx->lz_int_off[dir][ish], ints.data(), sizeof(int) * ints.size(),
                           cudaMemcpyHostToDevice, ctx->st));
        if (!P.piv.empty())
            CU(cudaMemcpyAsync(ctx->d_lzpiv + ctx->lz_piv_off[dir][ish], P.piv.data(), sizeof(double) * P.piv.size(),
                               cudaMemcpyHostToDevice, ctx->st));
    }
    const bool fp32 = (flags & BD_RUN_MIXED) != 0;
    const bool ref_order = !fp32 && (flags & BD_RUN_REF_ORDER);
    if ((rc = launch_sort(ctx, ish, ish + 1, ref_order))) return rc;
    C.ref_sorted = ref_order;
    if ((rc = launch_lanczos_range(ctx, ish, ish + 1, fp32))) return rc;
    for (int dir = 0; dir < 2; ++dir) {
        const ChainPlan &P = C.lz[dir];
        double *host = dir == 0 ? lz_fw : lz_bk;
        int *ip = dir == 0 ? ipiv_fw : ipiv_bk;
        if (host && P.L > 0)
            CU(cudaMemcpyAsync(host, ctx->d_lzout + ctx->lz_out_off[dir][ish],
                               sizeof(double) * (size_t)P.L * (P.nden_out + C.D), cudaMemcpyDeviceToHost, ctx->st));
        if (ip) std::memcpy(ip, P.ipiv.data(), sizeof(int) * P.ipiv.size());
    }
    CU(cudaStreamSynchronize(ctx->st));
    C.state = ST_LANCZOS;
    return BD_OK;
}

// A Dyson job's device status as the call's error.
static int dyson_status_error(bd_ctx *ctx, int ish, int st) {
    if (st == kDyStatCapacity)
        return fail(ctx, BD_ERR_CAPACITY,
                    "channel %d: the deflated Dyson matrix is larger than the cluster reduction's shared memory holds", ish);
    return fail(ctx, BD_ERR_NUMERIC, "channel %d: the eigensolver did not converge", ish);
}

int bd_dyson_solve(bd_ctx *ctx, int ish, const double *sig1b, const double *sig_hf, double e_fermi, double *sol_qp,
                   int cap_qp, int *n_qp, double *sol_qh, int cap_qh, int *n_qh, double *koltun) {
    int rc = check_chan(ctx, ish);
    if (rc) return rc;
    CU(cudaSetDevice(ctx->device));
    Chan &C = ctx->chans[ish];
    if (C.state < ST_SIGMA) return fail(ctx, BD_ERR_STATE, "channel %d: no self-energy", ish);
    const int D = C.D;
    if (first_nonfinite(sig1b, (long long)D * D) >= 0 || first_nonfinite(sig_hf, (long long)D * D) >= 0)
        return fail(ctx, BD_ERR_NUMERIC, "channel %d: a one-body or static self-energy entry is not finite", ish);
    if (sig1b)
        CU(cudaMemcpyAsync(ctx->d_sig1b + ctx->chan_dd_off[ish], sig1b, sizeof(double) * D * D, cudaMemcpyHostToDevice,
                           ctx->st));
    if (sig_hf)
        CU(cudaMemcpyAsync(ctx->d_sighf + ctx->chan_dd_off[ish], sig_hf, sizeof(double) * D * D, cudaMemcpyHostToDevice,
                           ctx->st));
    else if ((rc = launch_ehf(ctx, ish, ish + 1)))
        return rc;
    const double saved_ef = C.efermi;
    if (!std::isnan(e_fermi)) { C.efermi = e_fermi; ctx->ef_override = true; }
    rc = ensure_dyson(ctx, C.state == ST_LANCZOS);
    if (!rc) rc = launch_dyson_range(ctx, ish, ish + 1, C.state == ST_LANCZOS);
    C.efermi = saved_ef;
    ctx->ef_override = false;
    if (rc) return rc;
    int nq[2] = {0, 0}, st = 0;
    CU(cudaMemcpyAsync(nq, ctx->d_dynq + 2 * ish, sizeof(int) * 2, cudaMemcpyDeviceToHost, ctx->st));
    CU(cudaMemcpyAsync(&st, ctx->d_dystat + ish, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    double kol[3];
    CU(cudaMemcpyAsync(kol, ctx->d_dykol + 3 * ish, sizeof(double) * 3, cudaMemcpyDeviceToHost, ctx->st));
    CU(cudaStreamSynchronize(ctx->st));
    if (st) {
        CU(cudaMemsetAsync(ctx->d_dystat + ish, 0, sizeof(int), ctx->st));
        return dyson_status_error(ctx, ish, st);
    }
    if (n_qp) *n_qp = nq[0];
    if (n_qh) *n_qh = nq[1];
    if (koltun) std::memcpy(koltun, kol, sizeof kol);
    if ((sol_qp && cap_qp < nq[0]) || (sol_qh && cap_qh < nq[1]))
        return fail(ctx, BD_ERR_CAPACITY, "solution buffers too small (%d, %d needed)", nq[0], nq[1]);
    const double *dsol = ctx->d_dysol + ctx->dy_sol_off[ish];
    if (sol_qp && nq[0])
        CU(cudaMemcpyAsync(sol_qp, dsol, sizeof(double) * (size_t)nq[0] * (2 + D), cudaMemcpyDeviceToHost, ctx->st));
    if (sol_qh && nq[1])
        CU(cudaMemcpyAsync(sol_qh, dsol + (size_t)nq[0] * (2 + D), sizeof(double) * (size_t)nq[1] * (2 + D),
                           cudaMemcpyDeviceToHost, ctx->st));
    CU(cudaStreamSynchronize(ctx->st));
    return BD_OK;
}

int bd_dyson_rows(bd_ctx *ctx, int ish, int nden, int n_fw, const double *fw_rows, const int *ipiv_fw, int n_bk,
                  const double *bk_rows, const int *ipiv_bk, const double *sig1b, const double *sig_hf, double e_fermi,
                  double *sol_qp, int cap_qp, int *n_qp, double *sol_qh, int cap_qh, int *n_qh, double *koltun) {
    int rc = check_chan(ctx, ish);
    if (rc) return rc;
    CU(cudaSetDevice(ctx->device));
    Chan &C = ctx->chans[ish];
    const int D = C.D, NT = nden + D;
    if (nden < 2 || n_fw < 0 || n_bk < 0 || (n_fw > 0 && !fw_rows) || (n_bk > 0 && !bk_rows))
        return fail(ctx, BD_ERR_ARG, "self-energy rows");
    if (first_nonfinite(fw_rows, (long long)n_fw * NT) >= 0 || first_nonfinite(bk_rows, (long long)n_bk * NT) >= 0)
        return fail(ctx, BD_ERR_NUMERIC, "channel %d: a self-energy row element is not finite", ish);
    if (first_nonfinite(sig1b, (long long)D * D) >= 0 || first_nonfinite(sig_hf, (long long)D * D) >= 0)
        return fail(ctx, BD_ERR_NUMERIC, "channel %d: a one-body or static self-energy entry is not finite", ish);
    const int n = D + n_fw + n_bk;
    const size_t nip = (size_t)nden + D;
    double *dfw = nullptr, *dbk = nullptr, *dA = nullptr, *dv = nullptr, *dR = nullptr, *dsol = nullptr, *dwork = nullptr;
    int *dipf = nullptr, *dipb = nullptr;
    long long *dwf = nullptr, *drf = nullptr;
    DyJob *dj = nullptr;
    CU(cudaMallocAsync(&dfw, sizeof(double) * ((size_t)n_fw * NT + 1), ctx->st));
    CU(cudaMallocAsync(&dbk, sizeof(double) * ((size_t)n_bk * NT + 1), ctx->st));
    CU(cudaMallocAsync(&dipf, sizeof(int) * nip, ctx->st));
    CU(cudaMallocAsync(&dipb, sizeof(int) * nip, ctx->st));
    CU(cudaMallocAsync(&dA, sizeof(double) * (size_t)n * n, ctx->st));
    CU(cudaMallocAsync(&dv, sizeof(double) * 4 * (size_t)n, ctx->st));
    CU(cudaMallocAsync(&dR, sizeof(double) * ((size_t)D * n + (size_t)n * (2 + D)), ctx->st));
    CU(cudaMallocAsync(&dsol, sizeof(double) * (size_t)n * (2 + D), ctx->st));
    CU(cudaMallocAsync(&dwork, sizeof(double) * 5 * (size_t)n * n, ctx->st));
    CU(cudaMallocAsync(&dwf, sizeof(long long) * 2, ctx->st));
    CU(cudaMallocAsync(&drf, sizeof(long long) * 2, ctx->st));
    CU(cudaMallocAsync(&dj, sizeof(DyJob), ctx->st));
    if (n_fw) CU(cudaMemcpyAsync(dfw, fw_rows, sizeof(double) * (size_t)n_fw * NT, cudaMemcpyHostToDevice, ctx->st));
    if (n_bk) CU(cudaMemcpyAsync(dbk, bk_rows, sizeof(double) * (size_t)n_bk * NT, cudaMemcpyHostToDevice, ctx->st));
    if (ipiv_fw) CU(cudaMemcpyAsync(dipf, ipiv_fw, sizeof(int) * nip, cudaMemcpyHostToDevice, ctx->st));
    if (ipiv_bk) CU(cudaMemcpyAsync(dipb, ipiv_bk, sizeof(int) * nip, cudaMemcpyHostToDevice, ctx->st));
    if (sig1b) CU(cudaMemcpyAsync(ctx->d_sig1b + ctx->chan_dd_off[ish], sig1b, sizeof(double) * D * D, cudaMemcpyHostToDevice, ctx->st));
    if (sig_hf) CU(cudaMemcpyAsync(ctx->d_sighf + ctx->chan_dd_off[ish], sig_hf, sizeof(double) * D * D, cudaMemcpyHostToDevice, ctx->st));
    else if ((rc = launch_ehf(ctx, ish, ish + 1))) return rc;
    DyJob J{};
    J.ch = ish; J.D = D; J.j2 = C.j2; J.n = n; J.nc = n; J.nfw = n_fw; J.nbk = n_bk; J.nden = nden;
    J.lanczos_fw = (ipiv_fw != nullptr) && n_fw > 0 && ipiv_fw[0] > 0;
    J.lanczos_bk = (ipiv_bk != nullptr) && n_bk > 0 && ipiv_bk[0] > 0;
    J.fw_rows = dfw; J.bk_rows = dbk; J.ipiv_fw = dipf; J.ipiv_bk = dipb;
    J.sighf = ctx->d_sighf + ctx->chan_dd_off[ish];
    J.sig1b = ctx->d_sig1b + ctx->chan_dd_off[ish];
    J.efermi = std::isnan(e_fermi) ? C.efermi : e_fermi;
    J.A = dA; J.d = dv; J.e = dv + n; J.tau = dv + 2 * n; J.blk = reinterpret_cast<int *>(dv + 3 * n);
    J.R = dR; J.sol = dsol;
    J.nq = ctx->d_dynq + 2 * ish; J.koltun = ctx->d_dykol + 3 * ish; J.stat = ctx->d_dystat + ish;
    long long zero[2] = {0, 0};
    CU(cudaMemcpyAsync(dj, &J, sizeof(DyJob), cudaMemcpyHostToDevice, ctx->st));
    CU(cudaMemcpyAsync(dwf, zero, sizeof zero, cudaMemcpyHostToDevice, ctx->st));
    CU(cudaMemcpyAsync(drf, zero, sizeof zero, cudaMemcpyHostToDevice, ctx->st));
    CU(launch_dyson(dj, 1, drf, n, n, D, dy_cluster_for(ctx, 1), dwork, dwf, ctx->st));
    ctx->launches += dyson_launch_count(n);
    int nq[2] = {0, 0}, dst = 0;
    double kol[3];
    CU(cudaMemcpyAsync(nq, ctx->d_dynq + 2 * ish, sizeof nq, cudaMemcpyDeviceToHost, ctx->st));
    CU(cudaMemcpyAsync(kol, ctx->d_dykol + 3 * ish, sizeof kol, cudaMemcpyDeviceToHost, ctx->st));
    CU(cudaMemcpyAsync(&dst, ctx->d_dystat + ish, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CU(cudaStreamSynchronize(ctx->st));
    rc = BD_OK;
    if (dst) {
        CU(cudaMemsetAsync(ctx->d_dystat + ish, 0, sizeof(int), ctx->st));
        rc = dyson_status_error(ctx, ish, dst);
    } else {
        if (n_qp) *n_qp = nq[0];
        if (n_qh) *n_qh = nq[1];
        if (koltun) std::memcpy(koltun, kol, sizeof kol);
    }
    if (!rc && ((sol_qp && cap_qp < nq[0]) || (sol_qh && cap_qh < nq[1])))
        rc = fail(ctx, BD_ERR_CAPACITY, "solution buffers too small (%d, %d needed)", nq[0], nq[1]);
    else if (!rc) {
        if (sol_qp && nq[0]) CU(cudaMemcpyAsync(sol_qp, dsol, sizeof(double) * (size_t)nq[0] * (2 + D), cudaMemcpyDeviceToHost, ctx->st));
        if (sol_qh && nq[1])
            CU(cudaMemcpyAsync(sol_qh, dsol + (size_t)nq[0] * (2 + D), sizeof(double) * (size_t)nq[1] * (2 + D),
                               cudaMemcpyDeviceToHost, ctx->st));
    }
    for (void *q : {(void *)dfw, (void *)dbk, (void *)dipf, (void *)dipb, (void *)dA, (void *)dv, (void *)dR,
                    (void *)dsol, (void *)dwork, (void *)dwf, (void *)drf, (void *)dj})
        CU(cudaFreeAsync(q, ctx->st));
    CU(cudaStreamSynchronize(ctx->st));
    return rc;
}

int bd_lanczos_vectors(bd_ctx *ctx, int ish, int dir, int fp32, double *out, long long cap) {
    int rc = check_chan(ctx, ish);
    if (rc) return rc;
    if (dir != 0 && dir != 1) return fail(ctx, BD_ERR_ARG, "direction");
    CU(cudaSetDevice(ctx->device));
    const ChainPlan &P = ctx->chans[ish].lz[dir];
    const long long need = (long long)P.L * P.N;
    if (!out || cap < need) return fail(ctx, BD_ERR_CAPACITY, "need %lld doubles", need);
    const int ld = lz_ld(P.N);
    const char *base = ctx->d_lzV + ctx->lz_v_off[dir][ish];
    CU(cudaStreamSynchronize(ctx->st));
    // rows of a deflated tail have no stored vector: zero rows
    std::vector<int> slot(std::max(P.L, 0));
    if (P.L > 0)
        CU(cudaMemcpy(slot.data(), ctx->d_lzslot + ctx->lz_slot_off[dir][ish], sizeof(int) * P.L, cudaMemcpyDeviceToHost));
    if (fp32) {
        std::vector<float> tmp((size_t)P.L * ld);
        CU(cudaMemcpy(tmp.data(), base, sizeof(float) * tmp.size(), cudaMemcpyDeviceToHost));
        for (int j = 0; j < P.L; ++j)
            for (int i = 0; i < P.N; ++i) out[(size_t)j * P.N + i] = slot[j] < 0 ? 0.0 : tmp[(size_t)slot[j] * ld + i];
    } else {
        std::vector<double> tmp((size_t)P.L * ld);
        CU(cudaMemcpy(tmp.data(), base, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost));
        for (int j = 0; j < P.L; ++j)
            for (int i = 0; i < P.N; ++i) out[(size_t)j * P.N + i] = slot[j] < 0 ? 0.0 : tmp[(size_t)slot[j] * ld + i];
    }
    return BD_OK;
}

}  // extern "C"

namespace {

// The whole chain for every channel, queued on the context's stream (between the
// events ev[0] .. ev[4] that time its phases).
int enqueue_step(bd_ctx *ctx, int flags) {
    const bool lanczos = (flags & BD_RUN_LANCZOS) != 0, fp32 = (flags & BD_RUN_MIXED) != 0;
    const bool ref_order = !fp32 && (flags & BD_RUN_REF_ORDER);
    const int ns = ctx->nsubsh;
    int rc;
    if (ctx->d_lzstat) CU(cudaMemsetAsync(ctx->d_lzstat, 0, sizeof(int) * 4, ctx->st));
    CU(record(ctx, ctx->ev[0]));
    if (flags & BD_RUN_PER_CHANNEL) {
        // the drop-in call pattern: every phase launched channel by channel
        for (int I = 0; I < ns; ++I) {
            if ((rc = launch_ehf(ctx, I, I + 1))) return rc;
            if ((rc = launch_sigma2(ctx, I, I + 1))) return rc;
        }
        CU(record(ctx, ctx->ev[1]));
        if (lanczos) for (int I = 0; I < ns; ++I) if ((rc = launch_sort(ctx, I, I + 1, ref_order))) return rc;
        CU(record(ctx, ctx->ev[2]));
        if (lanczos) for (int I = 0; I < ns; ++I) if ((rc = launch_lanczos_range(ctx, I, I + 1, fp32))) return rc;
        CU(record(ctx, ctx->ev[3]));
        for (int I = 0; I < ns; ++I) if ((rc = launch_dyson_range(ctx, I, I + 1, lanczos))) return rc;
    } else {
        // The static self-energy (EHF) depends only on the propagator and is read only by
        // the Dyson solve: it runs on the auxiliary stream beside Sigma(2), the sort and
        // the Lanczos reduction, joined before the Dyson solve (a branch of the graph when
        // the step is captured).
        CU(cudaEventRecord(ctx->ev_fork, ctx->st));
        CU(cudaStreamWaitEvent(ctx->st_aux, ctx->ev_fork, 0));
        if ((rc = launch_ehf(ctx, 0, ns, ctx->st_aux))) return rc;
        CU(cudaEventRecord(ctx->ev_join, ctx->st_aux));
        const bool tc = fp32 && lanczos && ctx->prop_dressed && ctx->tc_built && ctx->tc_ok && ctx->ntc_tiles > 0 && ctx->d_lzstat &&
                        !(flags & BD_RUN_FP64_COUPLINGS);
        ctx->last_tc = tc;
        if ((rc = launch_sigma2(ctx, 0, ns, ctx->st_aux, tc))) return rc;
        CU(cudaStreamWaitEvent(ctx->st, ctx->ev_join2, 0));
        CU(record(ctx, ctx->ev[1]));
        if (lanczos && (rc = launch_sort(ctx, 0, ns, ref_order))) return rc;
        CU(record(ctx, ctx->ev[2]));
        if (lanczos && (rc = launch_lanczos_range(ctx, 0, ns, fp32))) return rc;
        CU(record(ctx, ctx->ev[3]));
        CU(cudaStreamWaitEvent(ctx->st, ctx->ev_join, 0));
        if ((rc = launch_dyson_range(ctx, 0, ns, lanczos))) return rc;
    }
    CU(record(ctx, ctx->ev[4]));
    return BD_OK;
}

// The step captured once per flag combination into a CUDA graph, then replayed: one
// launch of the whole chain instead of one per kernel from the host.
int graph_step(bd_ctx *ctx, int flags) {
    const int key = flags & 15;
    if (!ctx->gexec[key]) {
        CU(cudaStreamSynchronize(ctx->st));
        ctx->capturing = true;
        const long long l0 = ctx->launches;
        cudaError_t e = cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) {
            ctx->capturing = false;
            return fail(ctx, BD_ERR_CUDA, "cudaStreamBeginCapture: %s", cudaGetErrorString(e));
        }
        const int rc = enqueue_step(ctx, flags);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(ctx->st, &g);
        ctx->capturing = false;
        if (rc || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            if (rc) return rc;
            return fail(ctx, BD_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
        }
        e = cudaGraphInstantiate(&ctx->gexec[key], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            ctx->gexec[key] = nullptr;
            return fail(ctx, BD_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
        }
        ctx->glaunches[key] = ctx->launches - l0;
        ctx->launches = l0;
    }
    CU(cudaGraphLaunch(ctx->gexec[key], ctx->st));
    ctx->launches += ctx->glaunches[key];
    return BD_OK;
}

}  // namespace

extern "C" {

int bd_run_all(bd_ctx *ctx, int flags) {
    if (!ctx) return BD_ERR_ARG;
    if (!ctx->uploaded) return fail(ctx, BD_ERR_STATE, "no problem uploaded");
    if (flags & ~(BD_RUN_LANCZOS | BD_RUN_MIXED | BD_RUN_PER_CHANNEL | BD_RUN_REF_ORDER | BD_RUN_GRAPH | BD_RUN_FP64_COUPLINGS))
        return fail(ctx, BD_ERR_ARG, "flags 0x%x", flags);
    const bool lanczos = (flags & BD_RUN_LANCZOS) != 0;
    if (lanczos && !ctx->have_pivots) return fail(ctx, BD_ERR_STATE, "no pivots uploaded");
    CU(cudaSetDevice(ctx->device));
    const int ns = ctx->nsubsh;
    int rc;
    ctx->results_valid = false;
    ctx->lz_timed = false;
    if ((rc = ensure_dyson(ctx, lanczos))) return rc;
    const bool graph = (flags & BD_RUN_GRAPH) && !(flags & BD_RUN_PER_CHANNEL);
    // the tensor-core tiles, when this step will use them (built here, before any capture)
    if (lanczos && (flags & BD_RUN_MIXED) && !(flags & (BD_RUN_FP64_COUPLINGS | BD_RUN_PER_CHANNEL)) &&
        ctx->prop_dressed && !ctx->tc_built && (rc = build_tc_tiles(ctx)))
        return rc;
    rc = graph ? graph_step(ctx, flags & ~BD_RUN_GRAPH) : enqueue_step(ctx, flags & ~BD_RUN_GRAPH);
    if (rc) return rc;
    if (graph && lanczos) ctx->lz_timed = true;
    for (int I = 0; I < ns; ++I) {
        ctx->chans[I].state = lanczos ? ST_LANCZOS : ST_SIGMA;
        ctx->chans[I].ref_sorted = lanczos && (flags & BD_RUN_REF_ORDER) && !(flags & BD_RUN_MIXED);
    }
    ctx->last_lanczos_flags = flags;
    ctx->results_valid = true;
    return BD_OK;
}

// Cluster sizes of the Lanczos kernel (and of the Dyson reduction beyond order 160) for
// this problem: each candidate runs the batched step (after one warm-up) `reps` times
// and the fastest by device time is kept.  Returns the chosen sizes.
int bd_autotune(bd_ctx *ctx, int flags, int reps, int *lz_cluster, int *dy_cluster) {
    if (!ctx) return BD_ERR_ARG;
    if (!ctx->uploaded) return fail(ctx, BD_ERR_STATE, "no problem uploaded");
    flags &= ~(BD_RUN_PER_CHANNEL | BD_RUN_GRAPH);
    reps = std::max(1, std::min(reps, 20));
    int nmax = 0;
    for (int I = 0; I < ctx->nsubsh; ++I) nmax = std::max(nmax, dyson_order(ctx, I, (flags & BD_RUN_LANCZOS) != 0));
    const int lz_c[3] = {4, 8, 16};
    const int dy_c[3] = {4, 8, 16};
    const int ndy = nmax > kTsMax ? 3 : 1;   // the cluster reduction runs only beyond kTsMax
    double best = 1e300;
    int bl = ctx->lz_cluster, bdc = ctx->dy_cluster;
    for (int a = 0; a < ((flags & BD_RUN_LANCZOS) ? 3 : 1); ++a)
        for (int b = 0; b < ndy; ++b) {
            ctx->lz_cluster = lz_c[a];
            ctx->dy_cluster = ndy > 1 ? dy_c[b] : ctx->dy_cluster;
            double tot = 0.0;
            for (int r = 0; r <= reps; ++r) {
                int rc = bd_run_all(ctx, flags);
                if (!rc) rc = bd_sync(ctx);
                if (rc) return rc;
                if (r > 0) tot += ctx->timings[4];
            }
            if (tot < best) { best = tot; bl = ctx->lz_cluster; bdc = ctx->dy_cluster; }
        }
    ctx->lz_cluster = bl;
    ctx->dy_cluster = bdc;
    graph_invalidate(ctx);
    if (lz_cluster) *lz_cluster = bl;
    if (dy_cluster) *dy_cluster = bdc;
    return BD_OK;
}

int bd_sync(bd_ctx *ctx) {
    if (!ctx) return BD_ERR_ARG;
    CU(cudaSetDevice(ctx->device));
    if (int rc = sync_stream(ctx)) return rc;
    if (ctx->results_valid) {
        std::vector<int> st(ctx->nsubsh, 0);
        CU(cudaMemcpy(ctx->res_nq.data(), ctx->d_dynq, sizeof(int) * 2 * ctx->nsubsh, cudaMemcpyDeviceToHost));
        CU(cudaMemcpy(st.data(), ctx->d_dystat, sizeof(int) * ctx->nsubsh, cudaMemcpyDeviceToHost));
        float ms[4];
        for (int q = 0; q < 4; ++q) CU(cudaEventElapsedTime(&ms[q], ctx->ev[q], ctx->ev[q + 1]));
        for (int q = 0; q < 4; ++q) ctx->timings[q] = ms[q];
        ctx->timings[4] = ms[0] + ms[1] + ms[2] + ms[3];
        ctx->lz_two_pass = 0;
        int lzs[4] = {0, 0, 0, 0};
        if (ctx->d_lzstat) CU(cudaMemcpy(lzs, ctx->d_lzstat, sizeof(lzs), cudaMemcpyDeviceToHost));
        ctx->lz_two_pass = lzs[0];
        if (lzs[3]) {
            ctx->results_valid = false;
            CU(cudaMemset(ctx->d_lzstat, 0, sizeof(lzs)));
            return fail(ctx, BD_ERR_TIMEOUT, "tensor-core coupling build: a bounded wait for the MMAs gave up");
        }
        ctx->lz_kernel_ms = 0.0;
        if (ctx->lz_timed) {
            float m = 0.f;
            CU(cudaEventElapsedTime(&m, ctx->ev_lz[0], ctx->ev_lz[1]));
            ctx->lz_kernel_ms = m;
        }
        for (int I = 0; I < ctx->nsubsh; ++I)
            if (st[I]) {
                ctx->results_valid = false;
                CU(cudaMemset(ctx->d_dystat, 0, sizeof(int) * ctx->nsubsh));
                return dyson_status_error(ctx, I, st[I]);
            }
    }
    return BD_OK;
}

int bd_result_counts(bd_ctx *ctx, int ish, int *n_qp, int *n_qh) {
    int rc = check_chan(ctx, ish);
    if (rc) return rc;
    if (!ctx->results_valid) return fail(ctx, BD_ERR_STATE, "no results (run bd_run_all and bd_sync)");
    if (n_qp) *n_qp = ctx->res_nq[2 * ish];
    if (n_qh) *n_qh = ctx->res_nq[2 * ish + 1];
    return BD_OK;
}

int bd_result_fetch(bd_ctx *ctx, int ish, double *sol_qp, int cap_qp, double *sol_qh, int cap_qh, double *koltun) {
    int rc = check_chan(ctx, ish);
    if (rc) return rc;
    if (!ctx->results_valid) return fail(ctx, BD_ERR_STATE, "no results (run bd_run_all and bd_sync)");
    CU(cudaSetDevice(ctx->device));
    const int nqp = ctx->res_nq[2 * ish], nqh = ctx->res_nq[2 * ish + 1], D = ctx->chans[ish].D;
    if ((sol_qp && cap_qp < nqp) || (sol_qh && cap_qh < nqh)) return fail(ctx, BD_ERR_CAPACITY, "solution buffers");
    const double *dsol = ctx->d_dysol + ctx->dy_sol_off[ish];
    if (sol_qp && nqp) CU(cudaMemcpy(sol_qp, dsol, sizeof(double) * (size_t)nqp * (2 + D), cudaMemcpyDeviceToHost));
    if (sol_qh && nqh)
        CU(cudaMemcpy(sol_qh, dsol + (size_t)nqp * (2 + D), sizeof(double) * (size_t)nqh * (2 + D),
                      cudaMemcpyDeviceToHost));
    if (koltun) CU(cudaMemcpy(koltun, ctx->d_dykol + 3 * ish, sizeof(double) * 3, cudaMemcpyDeviceToHost));
    return BD_OK;
}

int bd_result_fetch_all(bd_ctx *ctx, double *sol, long long cap, int *counts, double *koltun) {
    if (!ctx) return BD_ERR_ARG;
    if (!ctx->results_valid) return fail(ctx, BD_ERR_STATE, "no results (run bd_run_all and bd_sync)");
    CU(cudaSetDevice(ctx->device));
    long long need = 0;
    for (int I = 0; I < ctx->nsubsh; ++I)
        need += (long long)(ctx->res_nq[2 * I] + ctx->res_nq[2 * I + 1]) * (2 + ctx->chans[I].D);
    if (sol && cap < need) return fail(ctx, BD_ERR_CAPACITY, "sol holds %lld doubles, %lld needed", cap, need);
    // the channels' rows are contiguous on the device (every Dyson solution is kept)
    if (sol && need) CU(cudaMemcpy(sol, ctx->d_dysol, sizeof(double) * need, cudaMemcpyDeviceToHost));
    if (counts) std::memcpy(counts, ctx->res_nq.data(), sizeof(int) * 2 * ctx->nsubsh);
    if (koltun) CU(cudaMemcpy(koltun, ctx->d_dykol, sizeof(double) * 3 * ctx->nsubsh, cudaMemcpyDeviceToHost));
    return BD_OK;
}

int bd_result_koltun_all(bd_ctx *ctx, double *koltun) {
    if (!ctx || !koltun) return BD_ERR_ARG;
    if (!ctx->results_valid) return fail(ctx, BD_ERR_STATE, "no results (run bd_run_all and bd_sync)");
    CU(cudaSetDevice(ctx->device));
    CU(cudaMemcpy(koltun, ctx->d_dykol, sizeof(double) * 3 * ctx->nsubsh, cudaMemcpyDeviceToHost));
    return BD_OK;
}

int bd_dressed_propagator(bd_ctx *ctx, double z_cut, int max_frag, int keep_current, int *np_out, int *nh_out,
                          double *ep_out, int cap_p, double *eh_out, int cap_h, double *fqp_out, double *fqh_out,
                          double *diff) {
    if (!ctx) return BD_ERR_ARG;
    if (!ctx->results_valid) return fail(ctx, BD_ERR_STATE, "no results (run bd_run_all and bd_sync)");
    CU(cudaSetDevice(ctx->device));
    const int ns = ctx->nsubsh, NSP = ctx->nspb;
    ctx->last_update_on_device = false;
    if (!keep_current && max_frag > 0 && max_frag <= 32) {
        // On the device when the truncated propagator keeps the current fragment counts
        // (from the second iteration on, as a rule): the fragments are selected and
        // written over the resident propagator in place, and the block plan, the pole
        // counts and the chain schedules stay as they are -- nothing is planned again.
        const int cap = max_frag;
        int *dcnt = nullptr, *dsel = nullptr, *ddof = nullptr;
        long long *doff = nullptr;
        std::vector<int> dof(ns);
        for (int I = 0; I < ns; ++I) dof[I] = ctx->chans[I].D;
        CU(cudaMallocAsync(&dcnt, sizeof(int) * 2 * ns, ctx->st));
        CU(cudaMallocAsync(&dsel, sizeof(int) * 2 * ns * cap, ctx->st));
        CU(cudaMallocAsync(&ddof, sizeof(int) * ns, ctx->st));
        CU(cudaMallocAsync(&doff, sizeof(long long) * ns, ctx->st));
        CU(cudaMemcpyAsync(ddof, dof.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, ctx->st));
        CU(cudaMemcpyAsync(doff, ctx->dy_sol_off.data(), sizeof(long long) * ns, cudaMemcpyHostToDevice, ctx->st));
        k_dressed_select<<<(unsigned)((2 * ns * 32 + 255) / 256), 256, 0, ctx->st>>>(
            ctx->d_dysol, doff, ctx->d_dynq, ddof, ns, z_cut, max_frag, cap, dcnt, dsel);
        CU(cudaGetLastError());
        ctx->launches += 1;
        std::vector<int> cnt(2 * ns);
        CU(cudaMemcpyAsync(cnt.data(), dcnt, sizeof(int) * 2 * ns, cudaMemcpyDeviceToHost, ctx->st));
        CU(cudaStreamSynchronize(ctx->st));
        bool same = true;
        for (int I = 0; I < ns; ++I) same = same && cnt[2 * I] == ctx->np[I] && cnt[2 * I + 1] == ctx->nh[I];
        if (same) {
            DevProblem &P = ctx->dp;
            k_dressed_write<<<2 * ns, 128, 0, ctx->st>>>(ctx->d_dysol, doff, ctx->d_dynq, ddof, P.p_start, P.h_start, ns,
                                                       NSP, cap, dcnt, dsel, const_cast<double *>(P.ep),
                                                       const_cast<double *>(P.eh), const_cast<double *>(P.fqp),
                                                       const_cast<double *>(P.fqh));
            CU(cudaGetLastError());
            ctx->launches += 1;
            // the new energies back to the host copies: the Fermi energies and the difference
            // between the two propagators follow from them as on the host path
            std::vector<double> ep(ctx->ep.size()), eh(ctx->eh.size());
            if (!ep.empty()) CU(cudaMemcpyAsync(ep.data(), P.ep, sizeof(double) * ep.size(), cudaMemcpyDeviceToHost, ctx->st));
            if (!eh.empty()) CU(cudaMemcpyAsync(eh.data(), P.eh, sizeof(double) * eh.size(), cudaMemcpyDeviceToHost, ctx->st));
            CU(cudaStreamSynchronize(ctx->st));
            if (diff) {
                double d = 0.0;
                for (size_t i = 0; i < ep.size(); ++i) d += std::fabs(ep[i] - ctx->ep[i]);
                for (size_t i = 0; i < eh.size(); ++i) d += std::fabs(eh[i] - ctx->eh[i]);
                *diff = d;
            }
            ctx->ep.swap(ep);
            ctx->eh.swap(eh);
            std::vector<double> ef(ns);
            for (int I = 0; I < ns; ++I) ef[I] = ctx->chans[I].efermi = seek_efermi(ctx, I);
            CU(cudaMemcpyAsync(ctx->d_efermi, ef.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, ctx->st));
            if (np_out) std::memcpy(np_out, ctx->np.data(), sizeof(int) * ns);
            if (nh_out) std::memcpy(nh_out, ctx->nh.data(), sizeof(int) * ns);
            int rc = BD_OK;
            if ((ep_out && cap_p < (int)ctx->ep.size()) || (eh_out && cap_h < (int)ctx->eh.size()))
                rc = fail(ctx, BD_ERR_CAPACITY, "propagator buffers hold %d / %d fragments, %zu / %zu needed", cap_p,
                          cap_h, ctx->ep.size(), ctx->eh.size());
            else {
                if (ep_out && !ctx->ep.empty()) std::memcpy(ep_out, ctx->ep.data(), sizeof(double) * ctx->ep.size());
                if (eh_out && !ctx->eh.empty()) std::memcpy(eh_out, ctx->eh.data(), sizeof(double) * ctx->eh.size());
                if (fqp_out && !ctx->ep.empty())
                    CU(cudaMemcpyAsync(fqp_out, P.fqp, sizeof(double) * ctx->ep.size() * NSP, cudaMemcpyDeviceToHost, ctx->st));
                if (fqh_out && !ctx->eh.empty())
                    CU(cudaMemcpyAsync(fqh_out, P.fqh, sizeof(double) * ctx->eh.size() * NSP, cudaMemcpyDeviceToHost, ctx->st));
            }
            for (void *q : {(void *)dcnt, (void *)dsel, (void *)ddof, (void *)doff}) CU(cudaFreeAsync(q, ctx->st));
            CU(cudaStreamSynchronize(ctx->st));
            ctx->results_valid = false;
            for (int I = 0; I < ns; ++I) ctx->chans[I].state = ST_NONE;
            ctx->last_update_on_device = true;
            if (!ctx->prop_dressed) {   // the solutions' amplitudes are general: the mixed form's
                ctx->prop_dressed = true;   // captured steps switch to the tensor-core couplings
                graph_invalidate(ctx);
            }
            return rc;
        }
        for (void *q : {(void *)dcnt, (void *)dsel, (void *)ddof, (void *)doff}) CU(cudaFreeAsync(q, ctx->st));
    }
    std::vector<int> np(ns, 0), nh(ns, 0);
    std::vector<double> ep, eh, fqp, fqh;
    std::vector<double> rows;
    for (int I = 0; I < ns; ++I) {
        const int D = ctx->chans[I].D, NS = 2 + D;
        const int nqp = ctx->res_nq[2 * I], nqh = ctx->res_nq[2 * I + 1];
        rows.resize((size_t)(nqp + nqh) * NS);
        if (nqp + nqh > 0)
            CU(cudaMemcpy(rows.data(), ctx->d_dysol + ctx->dy_sol_off[I], sizeof(double) * rows.size(),
                          cudaMemcpyDeviceToHost));
        for (int side = 0; side < 2; ++side) {
            const int n0 = side == 0 ? 0 : nqp, n = side == 0 ? nqp : nqh;
            // candidates: Z >= z_cut; at most max_frag of them, largest Z first (earlier row on ties)
            std::vector<int> keep;
            for (int k = 0; k < n; ++k)
                if (rows[(size_t)(n0 + k) * NS + 1] >= z_cut) keep.push_back(k);
            if (max_frag > 0 && (int)keep.size() > max_frag) {
                std::stable_sort(keep.begin(), keep.end(), [&](int a, int b) {
                    return rows[(size_t)(n0 + a) * NS + 1] > rows[(size_t)(n0 + b) * NS + 1];
                });
                keep.resize(max_frag);
                std::sort(keep.begin(), keep.end());   // back to descending W, as add_qp / add_qh store them
            }
            std::vector<double> &E = side == 0 ? ep : eh, &F = side == 0 ? fqp : fqh;
            for (int k : keep) {
                const double *r = rows.data() + (size_t)(n0 + k) * NS;
                E.push_back(r[0]);
                for (int q = 0; q < NSP; ++q) F.push_back(q < D ? r[2 + q] : 0.0);
            }
            (side == 0 ? np : nh)[I] = (int)keep.size();
        }
    }
    // quick_n_dirty_diff between the propagator this iteration read and the new one
    if (diff) {
        double d = 0.0;
        const size_t ip = std::max(ep.size(), ctx->ep.size()), ih = std::max(eh.size(), ctx->eh.size());
        for (size_t i = 0; i < ip; ++i) d += std::fabs((i < ep.size() ? ep[i] : 0.0) - (i < ctx->ep.size() ? ctx->ep[i] : 0.0));
        for (size_t i = 0; i < ih; ++i) d += std::fabs((i < eh.size() ? eh[i] : 0.0) - (i < ctx->eh.size() ? ctx->eh[i] : 0.0));
        *diff = d;
    }
    if ((ep_out && cap_p < (int)ep.size()) || (eh_out && cap_h < (int)eh.size()))
        return fail(ctx, BD_ERR_CAPACITY, "propagator buffers hold %d / %d fragments, %zu / %zu needed", cap_p, cap_h,
                    ep.size(), eh.size());
    if (np_out) std::memcpy(np_out, np.data(), sizeof(int) * ns);
    if (nh_out) std::memcpy(nh_out, nh.data(), sizeof(int) * ns);
    if (ep_out && !ep.empty()) std::memcpy(ep_out, ep.data(), sizeof(double) * ep.size());
    if (eh_out && !eh.empty()) std::memcpy(eh_out, eh.data(), sizeof(double) * eh.size());
    if (fqp_out && !fqp.empty()) std::memcpy(fqp_out, fqp.data(), sizeof(double) * fqp.size());
    if (fqh_out && !fqh.empty()) std::memcpy(fqh_out, fqh.data(), sizeof(double) * fqh.size());
    if (keep_current) return BD_OK;
    bd_propagator P{NSP, np.data(), nh.data(), ep.data(), eh.data(), fqp.data(), fqh.data()};
    free_all(ctx);
    ctx->uploaded = false; ctx->results_valid = false;
    return upload_propagator(ctx, &P);
}

int bd_last_timings(bd_ctx *ctx, double *ms5) {
    if (!ctx || !ms5) return BD_ERR_ARG;
    for (int q = 0; q < 5; ++q) ms5[q] = ctx->timings[q];
    return BD_OK;
}

/* Not part of the public header: number of Lanczos steps that took a second
 * reorthogonalisation sweep in the last bd_run_all, and tuning knobs. */
int bd_diag_two_pass(bd_ctx *ctx) { return ctx ? ctx->lz_two_pass : -1; }
int bd_dressed_on_device(bd_ctx *ctx) { return ctx ? (ctx->last_update_on_device ? 1 : 0) : -1; }
int bd_tensor_couplings(bd_ctx *ctx) { return ctx ? (ctx->last_tc ? 1 : 0) : -1; }
double bd_lanczos_kernel_ms(bd_ctx *ctx) { return ctx ? ctx->lz_kernel_ms : -1.0; }
long long bd_launch_count(bd_ctx *ctx) { return ctx ? ctx->launches : -1; }
int bd_lanczos_stored(bd_ctx *ctx, int *stored) {
    if (!ctx || !stored) return BD_ERR_ARG;
    if (!ctx->have_pivots || !ctx->d_lzslot) return fail(ctx, BD_ERR_STATE, "no Lanczos reduction yet");
    CU(cudaSetDevice(ctx->device));
    CU(cudaStreamSynchronize(ctx->st));
    for (int I = 0; I < ctx->nsubsh; ++I)
        for (int dir = 0; dir < 2; ++dir) {
            const int L = std::max(ctx->chans[I].lz[dir].L, 0);
            std::vector<int> slot(L);
            if (L) CU(cudaMemcpy(slot.data(), ctx->d_lzslot + ctx->lz_slot_off[dir][I], sizeof(int) * L,
                                 cudaMemcpyDeviceToHost));
            int c = 0;
            for (int v : slot) c += (v >= 0);
            stored[2 * I + dir] = c;
        }
    return BD_OK;
}

int bd_set_lanczos_slices(bd_ctx *ctx, int mode) {
    if (!ctx) return BD_ERR_ARG;
    if (mode < 0 || mode > 2) return fail(ctx, BD_ERR_ARG, "slice mode %d", mode);
    ctx->lz_slices = mode;
    graph_invalidate(ctx);
    return BD_OK;
}

int bd_set_tuning(bd_ctx *ctx, int lz_cluster, int dy_cluster, double eta) {
    if (!ctx) return BD_ERR_ARG;
    if (lz_cluster != 1 && lz_cluster != 2 && lz_cluster != 4 && lz_cluster != 8 && lz_cluster != 16)
        return fail(ctx, BD_ERR_ARG, "cluster size");
    if (dy_cluster != 1 && dy_cluster != 2 && dy_cluster != 4 && dy_cluster != 8 && dy_cluster != 16)
        return fail(ctx, BD_ERR_ARG, "cluster size");
    if (!(eta > 0.0 && eta < 1.0)) return fail(ctx, BD_ERR_ARG, "eta");
    ctx->lz_cluster = lz_cluster; ctx->dy_cluster = dy_cluster; ctx->eta = eta;
    graph_invalidate(ctx);
    return BD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free Lanczos reduction of one pole set (bd_lanczos_chain_noalloc).
//
// Some host programs cannot let a library call cudaMalloc.  One case is an
// application whose own pool allocator has already reserved nearly all of the
// device's memory, so a second allocator would fail or fragment it.  Another is a
// latency-bound caller that cannot accept the device-wide synchronisation that
// cudaMalloc and cudaFree may imply.  Such callers pass their own device buffers
// for the inputs and outputs.  The Lanczos vector store, the chain descriptor
// and the counters then live in the file-scope array below.
//
// Every device on which this library's module is loaded holds the array
// (BD_NOALLOC_SCRATCH_BYTES) until the process exits.  All calls share it and it
// keeps the last call's contents.  Each call rewrites the descriptor, the
// schedule and the counters (the counters start at zero), and the kernel writes
// every vector before it reads it.  Calls that overlap on the GPU, from two
// streams or two host threads, race on the array.

static __device__ __align__(256) unsigned char g_lz_scratch[BD_NOALLOC_SCRATCH_BYTES];

namespace {

// scratch layout: [0, 256) descriptor | [256, 272) counters | [512, 1024) chain starts
// and ends | [1024, 2048) pivots | [4096, end) Lanczos vectors
constexpr size_t kNoallocCounters = 256, kNoallocInts = 512, kNoallocPiv = 1024, kNoallocStage = 2048;
constexpr size_t kNoallocVectors = 4096;
constexpr int kNoallocCluster = 16;                      // as for a channel launched alone
constexpr double kNoallocEta = 0.70710678118654752;      // the context's DGKS threshold
static_assert(sizeof(LzChain) <= kNoallocCounters, "descriptor slot");

int noalloc_fail(char *err, int err_len, int code, const char *fmt, ...) {
    if (err && err_len > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, (size_t)err_len, fmt, ap);
        va_end(ap);
    }
    return code;
}

// Device address of the scratch array on the current device.  It is looked up on every
// call (a host-side lookup, no synchronisation): an address kept from an earlier call
// would go stale if the host program reset the device or its primary context was torn
// down and created again, since the module and its array are then loaded anew.
int noalloc_scratch(char **base, char *err, int err_len) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(err, err_len, BD_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_lz_scratch);
    if (e != cudaSuccess || !p)
        return noalloc_fail(err, err_len, BD_ERR_CUDA, "cudaGetSymbolAddress(scratch) on device %d: %s", dev,
                            cudaGetErrorString(e));
    *base = static_cast<char *>(p);
    return BD_OK;
}

}  // namespace

extern "C" int bd_lanczos_chain_noalloc(const double *d_E, const double *d_M, int N, int D, int n_pvt,
                                        double *pivots, int *n_itr, double *d_rows, int cap_rows, int *L_out,
                                        int *ipiv, int flags, void *stream, char *err, int err_len) {
    if (err && err_len > 0) err[0] = 0;
    if (N < 0) return noalloc_fail(err, err_len, BD_ERR_ARG, "N = %d", N);
    if (D < 1 || D > 8) return noalloc_fail(err, err_len, BD_ERR_ARG, "D = %d (1..8 orbitals supported)", D);
    if (n_pvt < 1 || n_pvt > 9 || !pivots || !n_itr)
        return noalloc_fail(err, err_len, BD_ERR_ARG, "pivots: n_pvt = %d (1..9), pivots and n_itr required", n_pvt);
    if ((flags & ~BD_RUN_MIXED) != 0) return noalloc_fail(err, err_len, BD_ERR_ARG, "flags 0x%x", flags);
    for (long long i = 0; i < (long long)n_pvt * D; ++i)
        if (!std::isfinite(pivots[i])) return noalloc_fail(err, err_len, BD_ERR_NUMERIC, "pivot element %lld is not finite", i);
    ChainPlan P;
    plan_chain(P, N, D, n_pvt, n_itr, pivots);
    if (P.L > 0)
        for (int p = 0; p < n_pvt; ++p) n_itr[p] = P.nitr[p];
    if (L_out) *L_out = P.L;
    if (ipiv) std::memcpy(ipiv, P.ipiv.data(), sizeof(int) * P.ipiv.size());
    if (P.L == 0) return BD_OK;
    if (!d_E || !d_M) return noalloc_fail(err, err_len, BD_ERR_ARG, "device pole arrays required");
    if (!d_rows || cap_rows < P.L)
        return noalloc_fail(err, err_len, BD_ERR_CAPACITY, "d_rows holds %d rows, %d needed", cap_rows, P.L);
    const bool fp32 = (flags & BD_RUN_MIXED) != 0;
    const int ld = lz_ld(N);
    const size_t vbytes = (size_t)P.L * (size_t)ld * (fp32 ? sizeof(float) : sizeof(double));
    // behind the vectors: an FP32 copy of M (FP32 form), the energy groups of the
    // deflated tails (lz_group_bytes(N)) and the row slots (4 L bytes)
    const size_t mf_off = kNoallocVectors + (vbytes + 255) / 256 * 256;
    const size_t grp_off = mf_off + (fp32 ? (sizeof(float) * (size_t)D * (size_t)N + 255) / 256 * 256 : 0);
    const size_t slot_off = grp_off + (size_t)lz_group_bytes(N);
    const size_t need = slot_off + sizeof(int) * (size_t)P.L - kNoallocVectors;
    if (need > BD_NOALLOC_SCRATCH_BYTES - kNoallocVectors)
        return noalloc_fail(err, err_len, BD_ERR_CAPACITY,
                            "%d Lanczos vectors of %d poles need %zu bytes of scratch; this entry point has %zu "
                            "(use bd_lanczos_reduce for larger chains)",
                            P.L, N, need, (size_t)(BD_NOALLOC_SCRATCH_BYTES - kNoallocVectors));
    const int S = ((N + kNoallocCluster - 1) / kNoallocCluster + 3) / 4 * 4;
    if (lanczos_smem_bytes(S, P.L + 1) > (size_t)227 * 1024)
        return noalloc_fail(err, err_len, BD_ERR_CAPACITY, "%d poles per CTA exceed shared memory", S);
    char *base = nullptr;
    int rc = noalloc_scratch(&base, err, err_len);
    if (rc) return rc;

    // descriptor, zeroed counters, schedule and pivots, staged on the host and sent in one copy
    unsigned char stage[kNoallocStage];
    std::memset(stage, 0, sizeof(stage));
    int *h_ints = reinterpret_cast<int *>(stage + kNoallocInts);
    int ni = 0;
    for (int v : P.start) h_ints[ni++] = v;
    for (int v : P.last) h_ints[ni++] = v;
    std::memcpy(stage + kNoallocPiv, P.piv.data(), sizeof(double) * P.piv.size());
    LzChain z{};
    z.N = N; z.D = D; z.L = P.L; z.n_used = P.n_used; z.nden_out = P.nden_out;
    z.ld = ld; z.S = S;
    z.E = d_E; z.M = d_M;
    z.Mf = fp32 ? reinterpret_cast<const float *>(base + mf_off) : nullptr;
    z.gE = reinterpret_cast<const double *>(base + grp_off);
    z.gInfo = reinterpret_cast<const int *>(base + grp_off + (size_t)16 * N);
    z.rowslot = reinterpret_cast<int *>(base + slot_off);
    z.piv = reinterpret_cast<const double *>(base + kNoallocPiv);
    z.start = reinterpret_cast<const int *>(base + kNoallocInts);
    z.last = z.start + (P.n_used + 1);
    z.V = base + kNoallocVectors;
    z.out = d_rows;
    z.stat = reinterpret_cast<int *>(base + kNoallocCounters);
    std::memcpy(stage, &z, sizeof(z));

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t row_bytes = sizeof(double) * (size_t)P.L * (size_t)(P.nden_out + D);
    cudaError_t e = cudaMemcpyAsync(base, stage, sizeof(stage), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_rows, 0, row_bytes, st);   // the reference clears the rows
    if (e == cudaSuccess && fp32)
        e = launch_to_float(d_M, reinterpret_cast<float *>(base + mf_off), (long long)D * N, st);
    if (e == cudaSuccess) e = launch_lz_groups(reinterpret_cast<const LzChain *>(base), 1, lz_gram_cap(N), st);
    if (e == cudaSuccess)
        e = launch_lanczos(reinterpret_cast<const LzChain *>(base), 1, S, P.L + 1, fp32, kNoallocCluster, kNoallocEta,
                           false, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return noalloc_fail(err, err_len, BD_ERR_CUDA, "Lanczos launch: %s", cudaGetErrorString(e));
    return BD_OK;
}
