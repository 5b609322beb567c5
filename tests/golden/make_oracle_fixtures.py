"""Generates the oracle fixtures of the bench-size workloads (tests/golden/*_oracle.npz)
with the C restatement in oracle/ (no GPU involved):

    python tests/golden/make_oracle_fixtures.py

The reference program itself runs these sizes too, but its single Gram-Schmidt sweep
loses orthogonality after the first breakdown of a chain, so its reduced self-energy
(and every solution past the breakdown) depends on rounding.  The oracle's two-sweep
variant keeps the basis orthonormal, as the device does; that variant is pinned to the
reference program on the smaller fixtures (tests/test_oracle_golden.py) up to the
first breakdown.  Per workload and channel the fixture holds:
  * the pole counts and the sums of the pole energies of both directions;
  * every solution with Z > 1e-6 as (W, Z) pairs, quasiparticles and quasiholes;
  * the Koltun partial sums of Calc_En.
"""
from __future__ import annotations

import importlib
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

FIXTURES = {
    # name: synthetic workload (N_max, hw, seed, iterations per pivot)
    "nmax8_lanczos100_oracle": "nmax8_lanczos100",
    "nmax10_lanczos100_oracle": "nmax10_lanczos100",
}
ZMIN = 1e-6

_W = {}


def _init(workload):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    synth = importlib.import_module("boccadorata-public_gb300.synth")
    import oracle
    _W["prob"] = synth.make_workload(workload)
    _W["orc"] = oracle.Oracle().bind(_W["prob"])


def _channel(ish):
    r = _W["orc"].run_channel(ish, True, passes=2)
    out = {"nfw": len(r["sig_fw"]), "nbk": len(r["sig_bk"]),
           "efw_sum": float(r["sig_fw"][:, 0].sum()) if len(r["sig_fw"]) else 0.0,
           "ebk_sum": float(r["sig_bk"][:, 0].sum()) if len(r["sig_bk"]) else 0.0,
           "koltun": r["koltun"]}
    for tag in ("qp", "qh"):
        s = r[tag]
        out[tag] = np.ascontiguousarray(s[s[:, 1] > ZMIN, :2])
    return ish, out


def make(name, workload):
    sys.path.insert(0, ROOT)
    synth = importlib.import_module("boccadorata-public_gb300.synth")
    w = synth.WORKLOADS[workload]
    ns = synth.make_modspace(w["nmax"], w["hw"]).nsubsh
    with mp.get_context("spawn").Pool(os.cpu_count() or 1, initializer=_init, initargs=(workload,)) as pool:
        res = dict(pool.map(_channel, range(ns), chunksize=1))
    arrs = {"meta": np.array([w["nmax"], w["hw"], w["seed"], w["n_itr"], ns], np.float64)}
    for ish in range(ns):
        r = res[ish]
        arrs[f"c{ish}_counts"] = np.array([r["nfw"], r["nbk"]], np.int64)
        arrs[f"c{ish}_esum"] = np.array([r["efw_sum"], r["ebk_sum"]])
        arrs[f"c{ish}_koltun"] = r["koltun"]
        arrs[f"c{ish}_qp_strong"] = r["qp"]
        arrs[f"c{ish}_qh_strong"] = r["qh"]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
    print(name, ns, "channels")


if __name__ == "__main__":
    for n, wl in FIXTURES.items():
        make(n, wl)
