#!/usr/bin/env python3
"""Benchmark of the GB300 Sigma(2) -> Lanczos -> Dyson chain.

Default arm: ``python bench.py [--gpus N] [--steps K] [--warmup W]``
  A step is the whole chain for every (l, j, parity, charge) channel of the N_max=10
  workload (hw = 16 MeV, seed 2, 100 Lanczos iterations per pivot; 42 channels) in the
  mixed-precision batched form (FP32 Lanczos vectors, FP64 elsewhere), with all inputs
  resident in HBM.  ``value`` is channels solved per second over all ranks.  The same
  run also times the plain FP64 forms, checks the mixed form against FP64, measures the
  end-to-end rate through the C ABI with host buffers, and times the CPU oracle on a
  bounded sample.  Multi-GPU (torchrun): every rank solves its own copy of the workload
  (replicas; the channels share no data), rank 0 prints one JSON line.

Reference arm: ``python bench.py --impl reference ...``
  The reference's algorithm on the host cores: the C restatement in oracle/ (the
  reference program itself is built only where its sources are mounted), channels
  spread over all cores, single-pass Gram-Schmidt Lanczos and OpenBLAS dsyevd, as the
  reference does.
"""
from __future__ import annotations

import argparse
import importlib
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "channels solved/s at N_max=10: mixed vs FP64 GPU at <=1 keV qp-energy error"
WORKLOAD = "nmax10_lanczos100"
CPU_SAMPLE = [20, 16, 13, 9, 4, 0]          # neutron channels with D = 1, 2, 2, 3, 5, 6
# Per-launch traffic of the FP32 Lanczos kernel on this workload, from one ncu capture
# of that kernel at the current source (dram__bytes_read.sum 22.402816 MB +
# dram__bytes_write.sum 8.712448 MB; lts__t_bytes.sum 1.810563 GB; issue active 32.3 %
# of active cycles, barrier stalls 3.89 per issue).
LANCZOS_TRAFFIC_BYTES = 31_193_600
LANCZOS_L2_BYTES = 1_811_236_000
LANCZOS_ISSUE_ACTIVE = 0.323
# GB300's nominal FP64 rate (no measured FP64 peak exists for this machine): the
# denominator of the Dyson phase's FP64-class fraction.
FP64_NOMINAL_TFLOPS = 1.25
# Accuracy the metric is quoted at: mixed against FP64 on every solution with Z > 1e-4.
MAX_QP_ERROR_KEV = 1.0
MAX_Z_ERROR = 1e-5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the N_max=12 precision run and the dressed second iteration")
    ap.add_argument("--profile", choices=["mixed", "fp64", "fp64-per-channel", "mixed-dressed", "mixed-dressed-fp64c"],
                    default=None,
                    help="run only this form's warm-up and timed steps (for ncu); prints its timings, not a bench line; "
                         "*-dressed: on the second iteration's propagator (z_cut 1e-3, two fragments), the couplings "
                         "on the tensor cores (-fp64c: with the FP64 build)")
    ap.add_argument("--many", action="store_true",
                    help="the batched many-instance run (independent problems, iterated); prints its own line")
    ap.add_argument("--problems", type=int, default=256)
    ap.add_argument("--iterations", type=int, default=10)
    ap.add_argument("--concurrent", type=int, default=3,
                    help="--many: problems run side by side, each on its own context and host thread")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def rank_reduce_max(x, dist, device):
    """Maximum of a per-rank number over all ranks (the slowest rank's step time);
    x itself without a process group."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, channels, step_s):
    """Channels per second of the whole job: every rank solves its own replica of the
    workload (the channels share no data), timed by the slowest rank."""
    return world * channels / step_s


# ------------------------------------------------------------------------------------------
# shared helpers
# ------------------------------------------------------------------------------------------
def lanczos_sizes(ctx, prob, with_index=False):
    """(N, L, n_pvt, D) of every Lanczos chain, with the sizing rules of Reduce_SelfEn_Lncz
    (with_index: also (ish, dir) of each)."""
    out = []
    for ish in range(prob.ms.nsubsh):
        nfw, nbk = ctx.count_poles(ish)
        D = int(prob.ms.no[ish])
        for d, (N, nit) in enumerate(((nfw, prob.piv.n_fw[ish]), (nbk, prob.piv.n_bk[ish]))):
            tot = int(np.sum(nit[nit > 0]))
            if N < 1 or tot < 1:
                continue
            if tot > N:
                nit = np.array([int(N / tot * v + 1.0) for v in nit])
            L = min(int(np.sum(nit[nit > 0])), N)
            out.append(((N, L, len(nit), D), (ish, d)) if with_index else (N, L, len(nit), D))
    return out


def lanczos_algorithmic_bytes(chains, w, stored=None):
    """Per-launch algorithmic HBM bytes of the Lanczos kernel.  A built step reads all
    earlier built vectors once for the dot products and once for the update (w*N*R^2
    over a chain of R built vectors), plus E, v and the g vectors (w*N*(4+n_pvt)*R) and
    the M, E streams (8*N*(2+D)*R); deflated rows of an exhausted Krylov space read
    nothing.  stored: R per chain (default: every row built, R = L)."""
    tot = 0.0
    for q, (N, L, npv, D) in enumerate(chains):
        R = L if stored is None else stored[q]
        tot += w * N * (R * R + (4 + npv) * R) + 8 * N * (2 + D) * R
    return float(tot)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1])); mx = max(mx, float(r[2]))
                for k, v in zip(names, r[5:9]):
                    if v.strip() == "Active":
                        reasons.add(k)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------
# CPU work (oracle) -- used for cpu_baseline and the reference arm only
# ------------------------------------------------------------------------------------------
_W = {}


def _worker_init(workload):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    synth = importlib.import_module("boccadorata-public_gb300.synth")
    import oracle
    prob = synth.make_workload(workload)
    _W["prob"] = prob
    _W["orc"] = oracle.Oracle().bind(prob)


def _chain_channel(ish):
    """The reference's three boundary calls for one channel; returns their wall time."""
    orc, prob = _W["orc"], _W["prob"]
    s1, sh = orc.sig1b(ish), orc.ehf(ish)
    t0 = time.perf_counter()
    fw, bk = orc.sigma2(ish)
    pv = prob.piv
    lz = orc.reduce_lanczos(ish, fw, bk, pv.vec[ish], pv.n_fw[ish], pv.n_bk[ish], 1)
    orc.dyson(ish, s1, sh, lz["NDEN"], lz["lz_fw"], lz["lz_bk"], lz["n_piv_fw"], lz["ipiv_fw"], lz["n_piv_bk"],
              lz["ipiv_bk"])
    return time.perf_counter() - t0


def cpu_baseline(workload, sample):
    env_before = os.environ.get("OPENBLAS_NUM_THREADS")
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    _worker_init(workload)
    t = sum(_chain_channel(i) for i in sample)
    if env_before is None:
        os.environ.pop("OPENBLAS_NUM_THREADS", None)
    return {"value": len(sample) / t, "unit": "channels/s", "cores": 1, "kind": "port",
            "sample": f"channels {sample} of {workload} (D=1..6), Sigma(2) + single-pass Lanczos + dsyevd Dyson, "
                      f"{t:.1f} s on 1 host core"}


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    synth = importlib.import_module("boccadorata-public_gb300.synth")
    nch = synth.make_modspace(synth.WORKLOADS[args.workload]["nmax"], 1.0).nsubsh
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    chans = list(range(nch))
    # roughly most expensive first (low l within each charge) so the pool drains evenly
    order = sorted(chans, key=lambda i: (i % (nch // 2), i))
    with ctx.Pool(cores, initializer=_worker_init, initargs=(args.workload,)) as pool:
        pool.map(_chain_channel, [20] * cores)            # make sure every worker is initialised
        times = []
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            pool.map(_chain_channel, order, chunksize=1)
            dt = time.perf_counter() - t0
            if step >= args.warmup:
                times.append(dt)
    ms = 1e3 * statistics.mean(times)
    value = nch / (ms / 1e3)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "channels/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "channels": nch, "host_cores": cores},
            "cpu_baseline": {"value": value, "unit": "channels/s", "cores": cores, "kind": "port",
                             "sample": f"all {nch} channels of {args.workload} per step over {cores} processes; "
                                       "oracle/ restatement of the reference chain (single-pass Lanczos, "
                                       "OpenBLAS dsyevd), bit-identical to the reference on its fixtures"},
            "e2e": {"value": value, "unit": "channels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------
def strong_errors(ref, got, zmin=1e-4):
    """max |dW| (MeV) and max |dZ| over solutions with Z > zmin, nearest-energy match."""
    dW = dZ = 0.0
    for tag in ("qp", "qh"):
        a, b = ref[tag], got[tag]
        for r in a[a[:, 1] > zmin]:
            k = np.argmin(np.abs(b[:, 0] - r[0]))
            dW = max(dW, abs(b[k, 0] - r[0]))
            win = 1e-5 * max(1.0, abs(r[0]))
            dZ = max(dZ, abs(a[np.abs(a[:, 0] - r[0]) < win, 1].sum() - b[np.abs(b[:, 0] - r[0]) < win, 1].sum()))
    return dW, dZ


def solution_errors(ref, got, zmin=1e-4):
    """|dW| (MeV) and |dZ| of every solution of ref with Z > zmin against got, matched by
    nearest energy; Z compared per degenerate group (summed within 1e-5 relative)."""
    dW, dZ = [], []
    for tag in ("qp", "qh"):
        a, b = ref[tag], got[tag]
        for r in a[a[:, 1] > zmin]:
            k = np.argmin(np.abs(b[:, 0] - r[0]))
            dW.append(abs(b[k, 0] - r[0]))
            win = 1e-5 * max(1.0, abs(r[0]))
            dZ.append(abs(a[np.abs(a[:, 0] - r[0]) < win, 1].sum() - b[np.abs(b[:, 0] - r[0]) < win, 1].sum()))
    return dW, dZ


def error_summary(refs, gots, k64, k32, zmin=1e-4):
    dW, dZ = [], []
    for a, b in zip(refs, gots):
        w, z = solution_errors(a, b, zmin)
        dW += w
        dZ += z
    e64 = float(((k64[:, 0] + k64[:, 1]) / 2).sum())
    e32 = float(((k32[:, 0] + k32[:, 1]) / 2).sum())
    w = np.array(dW) * 1e3 if dW else np.zeros(1)
    z = np.array(dZ) if dZ else np.zeros(1)
    return {"solutions_compared": len(dW), "z_min": zmin,
            "qp_energy_error_keV": {"max": float(w.max()), "p99": float(np.percentile(w, 99)),
                                    "median": float(np.median(w))},
            "spectroscopic_factor_error": {"max": float(z.max()), "p99": float(np.percentile(z, 99)),
                                           "median": float(np.median(z))},
            "koltun_energy_fp64": e64, "koltun_energy_mixed": e32, "koltun_rel_error": abs(e32 - e64) / abs(e64)}


def precision_run(bd, synth, device, workload="nmax12_lanczos100"):
    """The precision configuration (N_max=12, hw = 16 MeV, seed 3, 100 iterations per
    pivot, 50 channels): the all-FP64 path and the mixed form once each (after a warm-up
    run), every solution's error of the mixed form against FP64."""
    t0 = time.perf_counter()
    prob = synth.make_workload(workload)
    gen_s = time.perf_counter() - t0
    ctx = bd.Context(device).upload(prob)
    out = {"workload": workload, "channels": prob.ms.nsubsh, "tbmes": int(prob.vpp.n), "generate_s": gen_s}
    res = {}
    for form, mixed in (("fp64", False), ("mixed", True)):
        ctx.run_all(lanczos=True, mixed=mixed)
        ctx.run_all(lanczos=True, mixed=mixed)
        res[form] = (ctx.timings(), ctx.results_all(), ctx.koltun_all(), ctx.lanczos_kernel_ms())
    nfw = sum(ctx.count_poles(i)[0] for i in range(prob.ms.nsubsh))
    ctx.close()
    (t64, r64, k64, l64), (t32, r32, k32, l32) = res["fp64"], res["mixed"]
    out.update({"forward_poles": int(nfw), "fp64_ms": t64["total"], "mixed_ms": t32["total"],
                "fp64_phases_ms": t64, "mixed_phases_ms": t32, "fp64_lanczos_kernel_ms": l64,
                "mixed_lanczos_kernel_ms": l32, "speedup_mixed_vs_fp64": t64["total"] / t32["total"],
                "errors_vs_fp64": error_summary(r64, r32, k64, k32)})
    return out


def dressed_run(bd, prob, device, z_cut=1e-3, max_frag=2):
    """A second iteration on the bench workload: the FP64 first iteration's solutions
    become the propagator (per subshell and side the solutions with Z >= z_cut, at most
    max_frag, largest Z first), Sigma(2) is rebuilt from it, and both forms run the whole
    chain once more (after a warm-up run).  Its pole spectra are dense, so the Lanczos
    chains build every vector (nothing deflates) and stream their bases from HBM.

    Accuracy: a few solutions of these dense spectra are ill-conditioned -- FP64 itself
    moves them when only the order of its sums changes -- so the FP64 chain is run twice
    (Lanczos clusters of 8 and of 16 CTAs) and that run-to-run spread is reported beside
    the mixed form's error, over all solutions and over those FP64 reproduces to 1 keV."""
    ctx = bd.Context(device).upload(prob)
    ctx.run_all(lanczos=True, mixed=False)
    ctx.dressed_propagator(z_cut, max_frag)
    ns = prob.ms.nsubsh
    cnt = [ctx.count_poles(i) for i in range(ns)]
    res = {}
    tc = {}
    # Dyson clusters of 16 CTAs: the orders near 1000 reduce in 96 ms against 118 with 8 and
    # 189 with 4 (the cluster sizes bd_autotune sweeps; its pick)
    for form, mixed, cl in (("fp64", False, 8), ("fp64_cl16", False, 16), ("mixed", True, 8)):
        ctx.set_tuning(lz_cluster=cl, dy_cluster=16)
        ctx.run_all(lanczos=True, mixed=mixed)
        ctx.run_all(lanczos=True, mixed=mixed)
        res[form] = (ctx.timings(), ctx.results_all(), ctx.koltun_all(), ctx.lanczos_kernel_ms())
        if mixed:   # the couplings on the tensor cores; the FP64 build beside it for its Sigma(2) time
            tc["tensor_couplings"] = ctx.tensor_couplings()
            tc["sigma2_ms_tensor"] = ctx.timings()["sigma2"]
            ctx.run_all(lanczos=True, mixed=True, fp64_couplings=True)
            tc["sigma2_ms_fp64_couplings"] = ctx.timings()["sigma2"]
    ctx.set_tuning(lz_cluster=8)
    st = ctx.lanczos_stored()
    chi = lanczos_sizes(ctx, ctx.prob, with_index=True)
    chains = [c for c, _ in chi]
    stored = [int(st[i, d]) for _, (i, d) in chi]
    ctx.close()
    (t64, r64, k64, l64), (_, r64b, k64b, _), (t32, r32, k32, l32) = res["fp64"], res["fp64_cl16"], res["mixed"]
    peak, src = measured_peaks()
    alg32 = lanczos_algorithmic_bytes(chains, 4, stored)
    alg64 = lanczos_algorithmic_bytes(chains, 8, stored)
    acc = {}
    for zmin in (1e-2, 1e-4):
        w0, z0, w1, z1 = [], [], [], []
        for a, b, c in zip(r64, r64b, r32):
            x, y = solution_errors(a, b, zmin)
            u, v = solution_errors(a, c, zmin)
            w0 += x; z0 += y; w1 += u; z1 += v
        w0, z0, w1, z1 = (np.array(q) for q in (w0, z0, w1, z1))
        ok = (w0 * 1e3 <= 1.0) & (z0 <= 1e-4)
        st_ = lambda q: {"max": float(q.max()) if len(q) else 0.0, "p99": float(np.percentile(q, 99)) if len(q) else 0.0,
                         "median": float(np.median(q)) if len(q) else 0.0}
        acc[f"z_above_{zmin:g}"] = {
            "solutions": int(len(w0)), "fp64_reproducible": int(ok.sum()),
            "fp64_run_to_run_keV": st_(w0 * 1e3), "fp64_run_to_run_dZ": st_(z0),
            "mixed_vs_fp64_keV": st_(w1 * 1e3), "mixed_vs_fp64_dZ": st_(z1),
            "mixed_vs_fp64_on_fp64_reproducible_keV": st_(w1[ok] * 1e3),
            "mixed_vs_fp64_on_fp64_reproducible_dZ": st_(z1[ok])}
    e64 = float(((k64[:, 0] + k64[:, 1]) / 2).sum())
    acc["koltun_energy"] = {"fp64": e64, "fp64_cl16": float(((k64b[:, 0] + k64b[:, 1]) / 2).sum()),
                            "mixed": float(((k32[:, 0] + k32[:, 1]) / 2).sum())}
    return {"z_cut": z_cut, "max_fragments": max_frag, "forward_poles": int(sum(c[0] for c in cnt)),
            "backward_poles": int(sum(c[1] for c in cnt)), "lanczos_vectors_built": int(sum(stored)),
            "lanczos_rows": int(sum(c[1] for c in chains)),
            "fp64_ms": t64["total"], "mixed_ms": t32["total"], "fp64_phases_ms": t64, "mixed_phases_ms": t32,
            "speedup_mixed_vs_fp64": t64["total"] / t32["total"], "mixed_couplings": tc, "dyson_cluster": 16,
            "mixed_lanczos": {"kernel": "k_lanczos<float> (global slices)", "kernel_ms": l32, "algorithmic_bytes": alg32,
                              "achieved_gbs": alg32 / (l32 / 1e3) / 1e9, "peak_gbs": peak,
                              "frac": alg32 / (l32 / 1e3) / 1e9 / peak, "peak_source": src},
            "fp64_lanczos": {"kernel": "k_lanczos<double> (global slices)", "kernel_ms": l64, "algorithmic_bytes": alg64,
                             "achieved_gbs": alg64 / (l64 / 1e3) / 1e9, "frac": alg64 / (l64 / 1e3) / 1e9 / peak},
            "accuracy": acc}


def pinned_problem(prob, torch):
    """Copies of the problem's input arrays in page-locked host memory."""
    import copy
    q = copy.deepcopy(prob)

    def pin(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        return t.numpy()
    q.vpp.iabJ, q.vpp.icdJ, q.vpp.V = pin(q.vpp.iabJ), pin(q.vpp.icdJ), pin(q.vpp.V)
    q.prop.fqp, q.prop.fqh, q.prop.ep, q.prop.eh = pin(q.prop.fqp), pin(q.prop.fqh), pin(q.prop.ep), pin(q.prop.eh)
    return q


def gpu_arm(args):
    rank, world, local = dist_env()
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    bd = importlib.import_module("boccadorata-public_gb300.bd")
    synth = importlib.import_module("boccadorata-public_gb300.synth")

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        return rank_reduce_max(x, dist, f"cuda:{local}")

    prob = synth.make_workload(args.workload)
    nch = prob.ms.nsubsh
    ctx = bd.Context(local).upload(prob)

    if args.profile:
        kw = {"mixed": dict(mixed=True), "fp64": dict(mixed=False),
              "fp64-per-channel": dict(mixed=False, per_channel=True), "mixed-dressed": dict(mixed=True),
              "mixed-dressed-fp64c": dict(mixed=True, fp64_couplings=True)}[args.profile]
        if args.profile.startswith("mixed-dressed"):
            ctx.run_all(lanczos=True, mixed=False)
            ctx.dressed_propagator(1e-3, 2)
        for _ in range(args.warmup):
            ctx.run_all(lanczos=True, **kw)
        ms = []
        for _ in range(args.steps):
            ctx.run_all(lanczos=True, **kw)
            ms.append(ctx.timings())
        if rank == 0:
            print(json.dumps({"profile": args.profile, "workload": args.workload, "steps": args.steps,
                              "timings_ms": ms, "lanczos_kernel_ms": ctx.lanczos_kernel_ms(),
                              "tensor_couplings": ctx.tensor_couplings(),
                              "extra_sweeps": ctx.two_pass_steps(),
                              "lanczos_steps": sum(L for _, L, _, _ in lanczos_sizes(ctx, prob)),
                              "lanczos_vectors_built": int(ctx.lanczos_stored().sum())}), flush=True)
        ctx.close()
        return 0

    # ---- accuracy of the mixed form against FP64 (outside the timed region)
    ctx.run_all(lanczos=True, mixed=False)
    ref = [ctx.result(i) for i in range(nch)]
    k64 = ctx.koltun_all()
    ctx.run_all(lanczos=True, mixed=True)
    got = [ctx.result(i) for i in range(nch)]
    k32 = ctx.koltun_all()
    dW = dZ = 0.0
    for i in range(nch):
        a, b = strong_errors(ref[i], got[i])
        dW, dZ = max(dW, a), max(dZ, b)
    e64 = float(((k64[:, 0] + k64[:, 1]) / 2).sum())
    e32 = float(((k32[:, 0] + k32[:, 1]) / 2).sum())

    def timed(flags_kw, steps, warmup):
        for _ in range(warmup):
            ctx.run_all(lanczos=True, **flags_kw)
        barrier()
        dev, lz = [], []
        l0 = ctx.launch_count()
        t0 = time.perf_counter()
        for _ in range(steps):
            ctx.run_all(lanczos=True, **flags_kw)
            dev.append(ctx.timings()["total"])
            lz.append(ctx.lanczos_kernel_ms())
        barrier()
        wall = time.perf_counter() - t0
        return statistics.mean(dev), wall / steps * 1e3, lz, ctx.launch_count() - l0

    # ---- the headline: mixed-precision batched form, the step replayed as one captured CUDA
    # graph (BD_RUN_GRAPH: the same 27 kernels, captured once, replayed every step)
    clocks = Clocks(local) if rank == 0 else None
    dev_ms, wall_ms, lz_ms, launches = timed(dict(mixed=True, graph=True), args.steps, args.warmup)
    dev_phases = ctx.timings()
    clk = clocks.stop() if clocks else None
    # the same form launched kernel by kernel on the stream
    stream_ms, stream_wall_ms, _, _ = timed(dict(mixed=True), max(3, min(args.steps, 5)), 1)
    step_s = max_over_ranks(dev_ms / 1e3)
    value = whole_job_rate(world, nch, step_s)

    # ---- the plain FP64 forms (the stable pole order the mixed form uses), and the FP64 form
    # whose reduction visits equal energies in the reference's heap-sort order
    f64_ms, _, f64_lz, _ = timed(dict(mixed=False, graph=True), max(2, min(args.steps, 3)), 1)
    f64_phases = ctx.timings()
    f64s_ms, _, _, _ = timed(dict(mixed=False), max(2, min(args.steps, 3)), 1)
    f64r_ms, _, _, _ = timed(dict(mixed=False, ref_order=True), max(2, min(args.steps, 3)), 1)
    f64r_phases = ctx.timings()
    pc_ms, _, _, _ = timed(dict(mixed=False, per_channel=True), 1, 1)

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        pq = pinned_problem(prob, torch)
        h2d = int(pq.vpp.iabJ.nbytes + pq.vpp.icdJ.nbytes + pq.vpp.V.nbytes + pq.prop.fqp.nbytes + pq.prop.fqh.nbytes
                  + pq.prop.ep.nbytes + pq.prop.eh.nbytes + sum(np.asarray(v).nbytes for v in pq.piv.vec))
        ctx2 = bd.Context(local)
        times = []
        d2h = 0
        for step in range(1 + max(2, min(args.steps, 3))):
            barrier()
            t0 = time.perf_counter()
            ctx2.upload(pq)
            ctx2.run_all(lanczos=True, mixed=True)
            res = ctx2.results_all()
            barrier()
            dt = time.perf_counter() - t0
            d2h = int(sum(r["qp"].nbytes + r["qh"].nbytes + r["koltun"].nbytes for r in res))
            if step > 0:
                times.append(dt)
        ctx2.close()
        seq_s = max_over_ranks(statistics.mean(times))
        # Pipelined: three contexts, each driven by its own host thread on its own stream.
        # The uploads (the 293 MB interaction over the host link, which one copy already
        # fills) are taken one at a time, so each runs at the link's rate while the other
        # contexts' chains and read-backs run; the chains overlap one another as well.
        # Every step still uploads its inputs from pinned host memory and reads its
        # results back.
        import threading
        nctx = 3
        nstep = nctx * max(3, min(args.steps, 5))
        ring = [bd.Context(local) for _ in range(nctx)]
        for c in ring:   # one untimed step each (first-use costs)
            c.upload(pq)
            c.run_all(lanczos=True, mixed=True)
            c.results_all()
        errs = []
        link = threading.Lock()   # one upload on the host link at a time

        def worker(c, n):
            try:
                for _ in range(n):
                    with link:
                        c.upload(pq)
                    c.run_all(lanczos=True, mixed=True)
                    c.results_all()
            except Exception as ex:   # reported below; the other threads finish their steps
                errs.append(repr(ex))
        barrier()
        t0 = time.perf_counter()
        ths = [threading.Thread(target=worker, args=(c, nstep // nctx)) for c in ring]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        barrier()
        wall = time.perf_counter() - t0
        for c in ring:
            c.close()
        if errs:
            raise RuntimeError("pipelined end-to-end steps failed: " + "; ".join(errs))
        e2e_s = max_over_ranks(wall / nstep)
        e2e = {"value": whole_job_rate(world, nch, e2e_s), "unit": "channels/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": 1e3 * e2e_s, "steps": nstep,
               "mode": "three contexts on three host threads and streams (upload, chain, read-back), uploads one at a time",
               "sequential": {"value": whole_job_rate(world, nch, seq_s), "ms_per_step": 1e3 * seq_s}}

    if rank != 0:
        ctx.close()
        if dist is not None:
            dist.destroy_process_group()
        return 0

    ctx.run_all(lanczos=True, mixed=True)           # the timed form's chains, for their built vectors
    st = ctx.lanczos_stored()
    chi = lanczos_sizes(ctx, prob, with_index=True)
    chains = [c for c, _ in chi]
    stored = [int(st[i, d]) for _, (i, d) in chi]
    alg = lanczos_algorithmic_bytes(chains, 4, stored)
    lz_mean = statistics.mean(lz_ms)
    peak, src = measured_peaks()
    achieved = alg / (lz_mean / 1e3) / 1e9
    roof = {"kernel": "k_lanczos<float> (FP32 vectors, all 84 chains in one launch)", "bound": "hbm",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)" if src == "measured" else "fallback 6.8 TB/s",
            "traffic": LANCZOS_TRAFFIC_BYTES, "algorithmic_bytes": alg, "kernel_ms": lz_mean,
            "lanczos_rows": int(sum(c[1] for c in chains)), "lanczos_vectors_built": int(sum(stored)),
            "l2_bytes": LANCZOS_L2_BYTES, "issue_active": LANCZOS_ISSUE_ACTIVE,
            "note": "the built basis stays in L2 (traffic is 1.1 % of the algorithmic bytes): the launch is "
                    "bound by the longest chain's step latency, so the HBM fraction is nominal"}
    # The Dyson phase against FP64: Householder (4/3 n^3) and the first D rows of Q
    # (2 n^2 D) over the deflated orders n = D + the chain's built rows (the deflated
    # tails leave the matrix), divided by the phase's CUDA-event time.
    dflops = 0.0
    for ish in range(nch):
        D = int(prob.ms.no[ish])
        n = D + int(st[ish, 0]) + int(st[ish, 1])
        dflops += 4.0 / 3.0 * n ** 3 + 2.0 * n * n * D
    dy_ms = dev_phases["dyson"]
    dyson = {"kernels": "k_dyson_deflate .. k_place (Householder, bisection, inverse iteration, placement)",
             "algorithmic_flops": dflops, "phase_ms": dy_ms, "achieved_tflops": dflops / (dy_ms / 1e3) / 1e12,
             "fp64_nominal_tflops": FP64_NOMINAL_TFLOPS,
             "frac_of_fp64_nominal": dflops / (dy_ms / 1e3) / 1e12 / FP64_NOMINAL_TFLOPS,
             "note": "latency-bound: the largest matrix's serial Householder columns (one CTA per matrix)"}
    extra = {}
    if world == 1 and not args.no_extra:
        extra["precision_nmax12"] = precision_run(bd, synth, local)
        extra["dressed_iteration2"] = dressed_run(bd, prob, local)
    cpu = None
    if world == 1 and not args.no_cpu:
        cpu = cpu_baseline(args.workload, CPU_SAMPLE)
    line = {
        "metric": METRIC, "value": value, "unit": "channels/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded generator in the reference's formats)",
        "config": {"workload": args.workload, "nmax": 10, "hw": 16.0, "seed": 2, "lanczos_iterations_per_pivot": 100,
                   "channels": nch, "form": "mixed precision (FP32 Lanczos vectors), all channels batched, the step replayed as a captured CUDA graph",
                   "l2": "inputs larger than L2 (293 MB interaction, ~0.9 GB Lanczos basis); no flush",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "roofline": roof,
        "dyson_fp64": dyson,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clk,
        "gpu_launches": launches,
        "forms": {"mixed_batched_ms": dev_ms, "mixed_batched_wall_ms": wall_ms,
                  "mixed_batched_stream_launches_ms": stream_ms, "mixed_batched_stream_launches_wall_ms": stream_wall_ms,
                  "mixed_batched_phases_ms": dev_phases,
                  "fp64_batched_ms": f64_ms, "fp64_batched_channels_per_s": nch / (f64_ms / 1e3),
                  "fp64_batched_stream_launches_ms": f64s_ms,
                  "fp64_batched_phases_ms": f64_phases,
                  "fp64_batched_reference_order_ms": f64r_ms, "fp64_batched_reference_order_phases_ms": f64r_phases,
                  "fp64_per_channel_ms": pc_ms, "fp64_per_channel_channels_per_s": nch / (pc_ms / 1e3),
                  "fp64_lanczos_kernel_ms": statistics.mean(f64_lz),
                  "speedup_mixed_vs_fp64_per_channel": pc_ms / dev_ms, "speedup_mixed_vs_fp64_batched": f64_ms / dev_ms},
        "accuracy": {"max_qp_energy_error_keV": dW * 1e3, "max_spectroscopic_factor_error": dZ,
                     "koltun_energy_fp64": e64, "koltun_energy_mixed": e32,
                     "koltun_rel_error": abs(e32 - e64) / abs(e64)},
    }
    line.update(extra)
    ok = dW * 1e3 <= MAX_QP_ERROR_KEV and dZ <= MAX_Z_ERROR
    line["accuracy"]["within_targets"] = bool(ok)
    print(json.dumps(line), flush=True)
    ctx.close()
    if not ok:
        sys.stderr.write(f"mixed form outside its accuracy targets: {dW * 1e3:.4f} keV, dZ {dZ:.2e}\n")
        return 1
    return 0


def many_problems(args):
    """The batched many-instance run: independent synthetic problems from seeds 100 on,
    each with N_max drawn from {4, 6, 8, 10}, hw uniform in [10, 30] MeV and interaction
    scale sigma uniform in [1, 3] MeV (8p+8n closed shells, 50 Lanczos iterations per
    pivot), each iterated `iterations` times: run the whole chain, then the next
    propagator from the Dyson solutions (z_cut 1e-3, at most one fragment per subshell
    and side: the truncation that keeps the dressed pole spaces of N_max = 10 inside
    minutes), Sigma(2) rebuilt from it.  Every step replays the context's captured graph;
    from the second update on the propagator is updated on the device when the fragment
    counts stay.  Problems go in batches of `concurrent` (default 3), side by side, each
    on its own context and host thread (one chain leaves most of the GPU idle); each form
    times its batches.  Problem generation (host numpy) is outside the timed region; the
    upload of each problem is inside it.

    Accuracy against FP64: the first iteration (both forms on the same input) measures
    the mixed form's precision; the last iteration compares two trajectories, and the
    truncated update (the strongest solution of each subshell and side) is a discontinuous
    choice between nearly equal strengths, so small differences can send the trajectories
    apart.  A second FP64 run with another reduction order (Lanczos clusters of 16 CTAs)
    measures that sensitivity of the iteration itself."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    bd = importlib.import_module("boccadorata-public_gb300.bd")
    synth = importlib.import_module("boccadorata-public_gb300.synth")
    z_cut, max_frag, n_itr = 1e-3, 1, 50
    times = {"mixed": [], "fp64": []}
    acc = {k: ([], [], []) for k in ("first_mixed_vs_fp64", "last_mixed_vs_fp64", "last_fp64_vs_fp64_cl16")}
    device_updates, sizes = 0, []
    import threading
    nconc = max(1, args.concurrent)

    def solve(prob, mixed, cl, out, j):
        """One problem in one form on its own context: upload, every iteration."""
        ctx = bd.Context(local).upload(prob)
        if cl != 8:
            ctx.set_tuning(lz_cluster=cl)
        dev_ms, first, upd = 0.0, None, 0
        for it in range(args.iterations):
            ctx.run_all(lanczos=True, mixed=mixed, graph=True)
            dev_ms += ctx.timings()["total"]
            if it == 0:
                first = (ctx.results_all(), ctx.koltun_all())
            if it + 1 < args.iterations:
                ctx.dressed_propagator(z_cut, max_frag)
                upd += int(mixed and ctx.dressed_on_device())
        out[j] = (first, (ctx.results_all(), ctx.koltun_all()), dev_ms, upd)
        ctx.close()

    for b0 in range(0, args.problems, nconc):
        batch = []
        for i in range(b0, min(b0 + nconc, args.problems)):
            seed = 100 + i
            r = np.random.default_rng(seed)
            nmax = int(r.choice([4, 6, 8, 10]))
            hw = float(r.uniform(10.0, 30.0))
            sigma = float(r.uniform(1.0, 3.0))
            batch.append((i, seed, nmax, synth.make_problem(nmax, hw, seed, n_itr, sigma)))
        res = [dict() for _ in batch]
        for form, mixed, cl in (("fp64", False, 8), ("mixed", True, 8), ("fp64_cl16", False, 16)):
            # the batch's problems side by side, each on its own context and host thread
            out, errs = [None] * len(batch), []

            def run(j):
                try:
                    solve(batch[j][3], mixed, cl, out, j)
                except Exception as ex:
                    errs.append(repr(ex))
            t0 = time.perf_counter()
            ths = [threading.Thread(target=run, args=(j,)) for j in range(len(batch))]
            for t in ths:
                t.start()
            for t in ths:
                t.join()
            wall = time.perf_counter() - t0
            if errs:
                raise RuntimeError(f"problems {b0}..: " + "; ".join(errs))
            if form in times:
                times[form].append((wall, sum(o[2] for o in out)))
            device_updates += sum(o[3] for o in out)
            for j, o in enumerate(out):
                res[j][form] = (o[0], o[1])
        for (i, seed, nmax, _), rj in zip(batch, res):
            for key, (a, b) in (("first_mixed_vs_fp64", (rj["fp64"][0], rj["mixed"][0])),
                                ("last_mixed_vs_fp64", (rj["fp64"][1], rj["mixed"][1])),
                                ("last_fp64_vs_fp64_cl16", (rj["fp64"][1], rj["fp64_cl16"][1]))):
                (ra, ka), (rb, kb) = a, b
                for x, y in zip(ra, rb):
                    w, z = solution_errors(x, y, 1e-2)
                    acc[key][0].extend(w)
                    acc[key][1].extend(z)
                ea = float(((ka[:, 0] + ka[:, 1]) / 2).sum())
                eb = float(((kb[:, 0] + kb[:, 1]) / 2).sum())
                acc[key][2].append(abs(eb - ea) / max(abs(ea), 1e-30))
            sizes.append(nmax)
        sys.stderr.write(f"problems {b0}..{b0 + len(batch) - 1} (N_max {[x[2] for x in batch]}): "
                         f"fp64 {times['fp64'][-1][0]:.2f} s, mixed {times['mixed'][-1][0]:.2f} s\n")
    st = lambda q: {"max": float(np.max(q)) if len(q) else 0.0, "p99": float(np.percentile(q, 99)) if len(q) else 0.0,
                    "median": float(np.median(q)) if len(q) else 0.0}
    errors = {k: {"solutions_z_above_0.01": len(w), "qp_energy_keV": st(np.array(w) * 1e3),
                  "spectroscopic_factor": st(np.array(z)), "koltun_rel": st(np.array(kr))}
              for k, (w, z, kr) in acc.items()}
    wall32 = sum(t for t, _ in times["mixed"])
    wall64 = sum(t for t, _ in times["fp64"])
    dev32 = sum(d for _, d in times["mixed"]) / 1e3
    dev64 = sum(d for _, d in times["fp64"]) / 1e3
    line = {"metric": "problems/s, batched many-instance run (iterated, mixed precision)", "impl": "gpu",
            "value": args.problems / wall32, "unit": "problems/s", "n_gpus": 1, "higher_is_better": True,
            "config": {"workload": "many_problems", "problems": args.problems, "seeds": [100, 100 + args.problems - 1],
                       "nmax_choices": [4, 6, 8, 10], "nmax_counts": {str(k): sizes.count(k) for k in (4, 6, 8, 10)},
                       "hw_MeV": [10, 30], "sigma_MeV": [1, 3], "lanczos_iterations_per_pivot": n_itr,
                       "iterations": args.iterations, "z_cut": z_cut, "max_fragments_per_subshell_side": max_frag,
                       "concurrent_problems": nconc,
                       "timed": "per batch of concurrent problems, per form: upload + every iteration (chain, next "
                                "propagator) of each, on its own context and host thread; generation excluded"},
            "mixed": {"problems_per_s": args.problems / wall32, "wall_s": wall32, "device_s": dev32},
            "fp64": {"problems_per_s": args.problems / wall64, "wall_s": wall64, "device_s": dev64},
            "speedup_mixed_vs_fp64_wall": wall64 / wall32, "speedup_mixed_vs_fp64_device": dev64 / dev32,
            "device_propagator_updates": device_updates, "errors": errors}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.many:
        return many_problems(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
