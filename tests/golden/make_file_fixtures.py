"""Generates the file fixtures of tests/golden/files_nmax2/ by running the reference
program's own readers and writers (oracle/_ref/bd_ref_files, built from the reference's
sources by oracle/Makefile) on a seeded synthetic problem.  Run where the reference tree
is mounted:

    python tests/golden/make_file_fixtures.py

Inputs (regenerated by the tests from the same seeds, not stored): N_max = 2, hw = 20 MeV,
seed 0, 10 Lanczos iterations per pivot, in the reference's formats, the interaction as a
scrambled .bcd (synth.write_interaction_bcd_scrambled, seed 7: pairs in random order with
their exchange phases, shuffled, 3 % repeated, Pauli-forbidden and out-of-space lines).
Stored: the reference's written propagator and DysPivots files, its .bin interaction, its
loaded interaction list, and the binary self-energies (plain and Lanczos-reduced) of
channels 0 and 3 with their rows.
"""
from __future__ import annotations

import importlib
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

synth = importlib.import_module("boccadorata-public_gb300.synth")
import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "files_nmax2")
PROBLEM = (2, 20.0, 0, 10)
SCRAMBLE_SEED = 7
CHANNELS = (0, 3)


def inputs(folder):
    """Writes the fixture's input files into folder; returns their paths and the problem."""
    prob = synth.make_problem(*PROBLEM)
    paths = synth.write_problem(prob, folder)
    paths["vpp"] = os.path.join(folder, "vint_scrambled.bcd")
    counts = synth.write_interaction_bcd_scrambled(prob.ms, prob.vpp, paths["vpp"], seed=SCRAMBLE_SEED)
    return paths, prob, counts


def main():
    if not O.build_ref():
        raise SystemExit("the reference sources are not mounted here; fixtures are generated where they are")
    ref = os.path.join(os.path.dirname(O.REF_BIN), "bd_ref_files")
    os.makedirs(OUT, exist_ok=True)
    with tempfile.TemporaryDirectory() as td:
        paths, prob, counts = inputs(td)
        outd = os.path.join(td, "out")
        for sub in ("", "plain", "lanczos"):
            os.makedirs(os.path.join(outd, sub), exist_ok=True)
        subprocess.run([ref, paths["msp"], paths["prop"], paths["vpp"], paths["piv"], outd] + [str(c) for c in CHANNELS],
                       check=True, stdout=subprocess.DEVNULL)
        for name in ("prop_written.dat", "pivots_written.dat", "vpp_written.bin"):
            shutil.copy(os.path.join(outd, name), os.path.join(OUT, name))
        for sub in ("plain", "lanczos"):
            os.makedirs(os.path.join(OUT, sub), exist_ok=True)
            for fn in sorted(os.listdir(os.path.join(outd, sub))):
                shutil.copy(os.path.join(outd, sub, fn), os.path.join(OUT, sub, fn))
        lst = O.read_dump(os.path.join(outd, "vpp_list.bin"))
        sig = O.read_dump(os.path.join(outd, "sig.bin"))
        arrs = {"vpp_iabJ": lst["iabJ"], "vpp_icdJ": lst["icdJ"], "vpp_V": lst["V"],
                "counts": np.array([counts["lines"], counts["repeated"], counts["pauli"], counts["outside"]], np.int64)}
        for k, v in sig.items():
            arrs["sig_" + k.replace("/", "_")] = v
        np.savez_compressed(os.path.join(OUT, "reference_lists.npz"), **arrs)
    print("written", sorted(os.listdir(OUT)))


if __name__ == "__main__":
    main()
