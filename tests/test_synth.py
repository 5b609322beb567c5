"""Synthetic workload generator: sizes against the counts the reference's own rules give."""
import numpy as np


def test_tbme_counts(synth):
    # canonical matrix elements per N_max (one line per pair of pairs, Pauli filter applied)
    for nmax, n in ((4, 34320), (6, 467032)):
        ms = synth.make_modspace(nmax, 20.0)
        assert synth.make_interaction(ms, 0).n == n


def test_interaction_sorted_like_prepare_for_reading(synth):
    ms = synth.make_modspace(4, 20.0)
    v = synth.make_interaction(ms, 0)
    sh = ms.orb_sh
    a = (v.iabJ // 128) // 1024
    b = (v.iabJ // 128) % 1024
    J = v.iabJ % 128
    key = ((ms.ch[sh[a]] + ms.ch[sh[b]] + 2) * 2 + (ms.ip[sh[a]] + ms.ip[sh[b]]) % 2) * 128 + J
    order = np.lexsort((v.icdJ, v.iabJ, key))
    assert np.array_equal(order, np.arange(v.n))
    assert np.all(v.iabJ <= v.icdJ)
    # Pauli filter: no a == b pair with odd J
    assert not np.any((a == b) & (J % 2 == 1))


def test_modspace_and_propagator(synth):
    ms = synth.make_modspace(10, 16.0)
    assert ms.nsubsh == 42 and ms.norb == 132 and ms.nspb_mx == 6
    pr = synth.make_unperturbed_propagator(ms)
    assert len(pr.eh) == 6 and len(pr.ep) == 126          # 8p + 8n in 0s, 0p
    assert np.allclose(pr.zp, 1.0) and np.allclose(pr.fqp.sum(1), 1.0)
    piv = synth.make_pivots(ms, pr, 100)
    assert [len(v) for v in piv.vec] == list(ms.no)


def test_writers(tmp_path, synth):
    p = synth.make_problem(2, 20.0, 0, 10)
    paths = synth.write_problem(p, str(tmp_path))
    lines = open(paths["vpp"]).read().splitlines()
    assert int(lines[0].split()[0]) == p.vpp.n and len(lines) == p.vpp.n + 1
    assert open(paths["msp"]).read().count("# subshell:") == p.ms.nsubsh
    assert open(paths["piv"]).read().count("shell,npvts:") == p.ms.nsubsh
