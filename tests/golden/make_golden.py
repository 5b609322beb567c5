"""Generates the golden fixtures of tests/golden/ by running the reference program
itself (oracle/_ref/bd_ref_harness, built from the reference's own sources by
oracle/Makefile) on seeded synthetic inputs, and storing its in-memory FP64
results.  Run in a container where the reference tree is mounted:

    python tests/golden/make_golden.py

Each fixture is a compressed .npz with, per workload:
  * Sigma(2) rows of a few channels (every double, for bit-exact checks) and
    per-channel checksums of all the others;
  * the static self-energy of every channel;
  * Lanczos rows / i_piv of a few channels and the sorted Sigma(2) of one;
  * every solution with Z > 1e-6 and the Koltun partial sums of every channel.

The *_iter2 fixtures are a second iteration: the reference's own first-iteration
solutions become a dressed propagator (oracle.dressed_propagator: per subshell and
side, Z >= z_cut, at most max_frag, the largest Z), written in the reference's
propagator format, and the reference program runs again on it.  The fixture holds
that propagator (p_np, p_nh, p_ep, p_eh, p_fqp, p_fqh) and the second run's results.
"""
from __future__ import annotations

import dataclasses
import importlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

synth = importlib.import_module("boccadorata-public_gb300.synth")
import oracle as O  # noqa: E402

FIXTURES = {
    # name: (nmax, hw, seed, iterations per pivot (0 = full Dyson), channels stored in full)
    "nmax2_full": (2, 20.0, 0, 0, None),
    "nmax4_full": (4, 20.0, 0, 0, [0, 5, 17]),
    "nmax4_lanczos20": (4, 20.0, 0, 20, [0, 5]),
}


ITER2 = {
    # name: (first-iteration fixture, z_cut, max_frag)
    "nmax2_full_iter2": ("nmax2_full", 1e-3, 4),
    "nmax4_lanczos20_iter2": ("nmax4_lanczos20", 1e-3, 4),
}


def make(name):
    if name in ITER2:
        return make_iter2(name)
    nmax, hw, seed, nit, keep = FIXTURES[name]
    prob = synth.make_problem(nmax, hw, seed, max(nit, 1))
    ns = prob.ms.nsubsh
    keep = list(range(ns)) if keep is None else keep
    with tempfile.TemporaryDirectory() as td:
        paths = synth.write_problem(prob, td)
        dump = O.run_reference(paths, hw, os.path.join(td, "ref.bin"), nit > 0)
    out = dict(meta=np.array([nmax, hw, seed, nit], np.float64), keep=np.array(keep, np.int32))
    store(out, dump, prob, nit, keep)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return os.path.getsize(os.path.join(HERE, f"{name}.npz"))


def make_iter2(name):
    base, z_cut, max_frag = ITER2[name]
    nmax, hw, seed, nit, keep = FIXTURES[base]
    prob = synth.make_problem(nmax, hw, seed, max(nit, 1))
    ns = prob.ms.nsubsh
    keep = list(range(ns)) if keep is None else keep
    with tempfile.TemporaryDirectory() as td:
        paths = synth.write_problem(prob, td)
        dump1 = O.run_reference(paths, hw, os.path.join(td, "ref1.bin"), nit > 0)
        res1 = [O.reference_channel(dump1, ish, int(prob.ms.no[ish])) for ish in range(ns)]
        dp = O.dressed_propagator(prob.ms, res1, prob.prop.nspb, z_cut, max_frag)
        nspb = prob.prop.nspb
        prop2 = synth.propagator_from_arrays(nspb, dp["np"], dp["nh"], dp["ep"], dp["eh"],
                                             np.reshape(dp["fqp"], (-1, nspb)), np.reshape(dp["fqh"], (-1, nspb)))
        prob2 = dataclasses.replace(prob, prop=prop2)
        td2 = os.path.join(td, "iter2")
        os.makedirs(td2)
        paths2 = synth.write_problem(prob2, td2)
        dump = O.run_reference(paths2, hw, os.path.join(td, "ref2.bin"), nit > 0)
    out = dict(meta=np.array([nmax, hw, seed, nit], np.float64), keep=np.array(keep, np.int32),
               trunc=np.array([z_cut, max_frag], np.float64),
               p_np=np.asarray(prop2.np_, np.int32), p_nh=np.asarray(prop2.nh, np.int32),
               p_ep=prop2.ep, p_eh=prop2.eh, p_fqp=prop2.fqp, p_fqh=prop2.fqh,
               diff1=np.array([O.quick_n_dirty_diff(prob.prop.ep, prob.prop.eh, prop2.ep, prop2.eh)]))
    store(out, dump, prob2, nit, keep, full_rows=False)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return os.path.getsize(os.path.join(HERE, f"{name}.npz"))


def store(out, dump, prob, nit, keep, full_rows=True):
    """Per-channel results of one reference run; full_rows=False keeps the Sigma(2) rows
    only as checksums (the dressed self-energies are large)."""
    ns = prob.ms.nsubsh
    for ish in range(ns):
        D = int(prob.ms.no[ish])
        r = O.reference_channel(dump, ish, D)
        out[f"c{ish}_sig_hf"] = r["sig_hf"]
        out[f"c{ish}_koltun"] = r["koltun"]
        for tag in ("sig_fw", "sig_bk"):
            a = r[tag]
            out[f"c{ish}_{tag}_sum"] = np.array([len(a), a.sum(), (a * a).sum(), np.abs(a).max() if len(a) else 0.0])
        for tag in ("qp", "qh"):
            a = r[tag]
            out[f"c{ish}_{tag}_n"] = np.array([len(a)], np.int32)
            out[f"c{ish}_{tag}_strong"] = a[a[:, 1] > 1e-6]
        if ish in keep:
            if full_rows:
                out[f"c{ish}_sig_fw"] = r["sig_fw"]
                out[f"c{ish}_sig_bk"] = r["sig_bk"]
            if nit > 0:
                for tag in ("lz_fw", "lz_bk", "ipiv_fw", "ipiv_bk"):
                    out[f"c{ish}_{tag}"] = r[tag]
                out[f"c{ish}_nden"] = np.array([r["NDEN"]], np.int32)
                if full_rows:
                    out[f"c{ish}_sorted_fw"] = r["sorted_fw"]
                    out[f"c{ish}_sorted_bk"] = r["sorted_bk"]


if __name__ == "__main__":
    if not O.build_ref():
        raise SystemExit("the reference sources are not mounted here; fixtures are generated where they are")
    for n in (sys.argv[1:] or list(FIXTURES) + list(ITER2)):
        print(n, make(n), "bytes")
