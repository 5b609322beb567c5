"""Seeded synthetic inputs for the Sigma(2) -> Lanczos -> Dyson chain.

The generator builds, in memory, the four inputs the reference program reads
and can write each of them in the reference's own text format:

* the model space      (format of ``ModSpace_t(char*)``, source/BcDor-Mod_Space.cpp:415-505)
* the sp propagator    (format of ``SpProp_t(char*, ModSpace_t*)``, source/BcDor-Sp_Propagator.cpp:387-611)
* the interaction      (``.bcd`` lines read by ``VppInt_t::read_ascii``, source/BcDor-Vpp_potential.cpp:256-374)
* the Lanczos pivots   (``shell,npvts:`` file read by ``Make_LancPivots``, source/BcDor-Miscellanea.cpp:334-390,
                        written like ``SpProp_t::DysPivots``, source/BcDor-Sp_Propagator.cpp:1225-1290)

Workload definition (spherical HO basis, 8 protons + 8 neutrons, closed 0s/0p):

* subshells (l, j) for every l <= N_max, j = l - 1/2 then l + 1/2, neutrons (ch=0) first and then
  protons (ch=1); orbits n = 0 .. (N_max - l)/2 inside each subshell;
* shell flag F = 1 (hole) for 0s1/2, 0p1/2, 0p3/2;
* single-particle energy xe = (2n + l + 3/2) * hw - 40 MeV, written in the model-space xe column;
  with ``Trel=7 ExtU1=1`` the reference uses it as a diagonal one-body potential
  (source/BcDor-Main.cpp:266,279-285);
* unperturbed propagator: one fragment per orbit, energy xe, Z = 100 %, one-hot amplitude;
* interaction: one matrix element per canonical pair of pairs (a <= b, c <= d, (ab) <= (cd) in orbit
  order) inside each (Tz, parity, J) channel, a == b with odd J excluded (the Pauli filter of
  source/BcDor-Vpp_potential.cpp:321-328); V ~ N(0, (sigma * exp(-(N_a+N_b+N_c+N_d)/8))^2) with
  N = 2n + l, drawn from ``numpy.random.default_rng(seed)`` channel by channel in that order.
  The exchange phase (-1)^(j_a+j_b-J+1) and the hermiticity V_abcd = V_cdab come from the reader's
  canonicalisation (source/BcDor-Vpp_potential.cpp:331-356, 557-607).
* pivots: one per fragment with Z >= 60 % (every orbit here), holes first by ascending energy and
  then particles by ascending energy, ``n_itr`` forward and backward iterations each.

Because the canonical enumeration order is also the reference's sort order of the matrix elements
(key ((ch+2)*2+ip)*128+J, then (a*1024+b)*128+J, then (c*1024+d)*128+J; source/BcDor-Vpp_potential.cpp:
74-81,440-501), the in-memory arrays are already in the order ``VppInt_t::prepare_for_reading``
produces.
"""
from __future__ import annotations

import dataclasses
import math
import os

import numpy as np

CHOFF, JMULT, ABMULT = -2, 128, 1024


@dataclasses.dataclass
class ModelSpace:
    nmax: int
    hw: float
    l: np.ndarray       # per subshell
    j2: np.ndarray
    ip: np.ndarray
    ch: np.ndarray
    no: np.ndarray      # orbits in the subshell (D)
    nqp: np.ndarray
    nqh: np.ndarray
    name: list
    orb_start: np.ndarray   # first orbit index of each subshell
    # per orbit
    orb_sh: np.ndarray
    orb_n: np.ndarray
    orb_F: np.ndarray
    orb_xe: np.ndarray

    @property
    def nsubsh(self) -> int:
        return len(self.l)

    @property
    def norb(self) -> int:
        return len(self.orb_sh)

    @property
    def jmax(self) -> int:
        """``ModSpace_t::Calculate_Jch_bounds``: Jmax = max 2j (source/BcDor-Mod_Space.cpp:593-594)."""
        return int(self.j2.max())

    @property
    def nspb_mx(self) -> int:
        return int(self.no.max())


@dataclasses.dataclass
class Propagator:
    """Lehmann representation per subshell; amplitudes fragment-major with stride ``nspb``."""
    nspb: int
    np_: np.ndarray        # particle fragments per subshell
    nh: np.ndarray
    p_start: np.ndarray    # offsets into ep / fqp rows
    h_start: np.ndarray
    ep: np.ndarray
    eh: np.ndarray
    zp: np.ndarray
    zh: np.ndarray
    fqp: np.ndarray        # (n_qp, nspb)
    fqh: np.ndarray        # (n_qh, nspb)


@dataclasses.dataclass
class Interaction:
    """Canonical, sorted matrix-element list (the arrays of ``VppInt_t`` after ``prepare_for_reading``)."""
    iabJ: np.ndarray   # int32
    icdJ: np.ndarray   # int32
    V: np.ndarray      # float64

    @property
    def n(self) -> int:
        return len(self.V)


@dataclasses.dataclass
class Pivots:
    """Per subshell: (n_fw, n_bk, vector) triples, as ``Make_LancPivots`` returns them."""
    n_fw: list   # list of int arrays
    n_bk: list
    vec: list    # list of (npvt, D) float arrays


@dataclasses.dataclass
class Problem:
    ms: ModelSpace
    prop: Propagator
    vpp: Interaction
    piv: Pivots
    seed: int
    sigma: float


def _subshell_name(ch: int, l: int, j2: int) -> str:
    letters = "spdfghijklmnoqrtuv"
    return ("v" if ch == 0 else "p") + "_" + letters[l] + f"{j2}/2"


def make_modspace(nmax: int, hw: float, fermi_holes=((0, 1), (1, 1), (1, 3))) -> ModelSpace:
    l_, j2_, ip_, ch_, no_, name = [], [], [], [], [], []
    for ch in (0, 1):
        for l in range(nmax + 1):
            for j2 in ((2 * l + 1,) if l == 0 else (2 * l - 1, 2 * l + 1)):
                l_.append(l); j2_.append(j2); ip_.append(l % 2); ch_.append(ch)
                no_.append(1 + (nmax - l) // 2); name.append(_subshell_name(ch, l, j2))
    no = np.array(no_, np.int32)
    orb_start = np.concatenate([[0], np.cumsum(no)[:-1]]).astype(np.int32)
    orb_sh, orb_n, orb_F, orb_xe = [], [], [], []
    for s in range(len(l_)):
        for n in range(no[s]):
            orb_sh.append(s); orb_n.append(n)
            orb_F.append(1 if (n == 0 and (l_[s], j2_[s]) in fermi_holes) else 0)
            orb_xe.append((2 * n + l_[s] + 1.5) * hw - 40.0)
    nqh = no // 2
    return ModelSpace(nmax, float(hw), np.array(l_, np.int32), np.array(j2_, np.int32),
                      np.array(ip_, np.int32), np.array(ch_, np.int32), no, no - nqh, nqh, name,
                      orb_start, np.array(orb_sh, np.int32), np.array(orb_n, np.int32),
                      np.array(orb_F, np.int32), np.array(orb_xe, np.float64))


def make_unperturbed_propagator(ms: ModelSpace) -> Propagator:
    nspb = ms.nspb_mx
    np_, nh_, ep, eh, fqp, fqh = [], [], [], [], [], []
    for s in range(ms.nsubsh):
        cp = ch = 0
        for k in range(ms.no[s]):
            o = ms.orb_start[s] + k
            amp = np.zeros(nspb); amp[k] = 1.0
            if ms.orb_F[o] == 1:
                eh.append(ms.orb_xe[o]); fqh.append(amp); ch += 1
            else:
                ep.append(ms.orb_xe[o]); fqp.append(amp); cp += 1
        np_.append(cp); nh_.append(ch)
    np_ = np.array(np_, np.int32); nh_ = np.array(nh_, np.int32)
    p_start = np.concatenate([[0], np.cumsum(np_)[:-1]]).astype(np.int32)
    h_start = np.concatenate([[0], np.cumsum(nh_)[:-1]]).astype(np.int32)
    fqp = np.array(fqp, np.float64).reshape(-1, nspb)
    fqh = np.array(fqh, np.float64).reshape(-1, nspb)
    return Propagator(nspb, np_, nh_, p_start, h_start, np.array(ep), np.array(eh),
                      np.ones(len(ep)), np.ones(len(eh)), fqp, fqh)


def propagator_from_arrays(nspb, np_, nh, ep, eh, fqp, fqh) -> Propagator:
    """A Propagator from per-subshell fragment counts and flat arrays (fragments listed
    subshell by subshell, amplitudes rows of nspb); Z = sum of squared amplitudes, as
    SpProp_t::add_qp / add_qh store it."""
    np_ = np.asarray(np_, np.int32); nh = np.asarray(nh, np.int32)
    fqp = np.asarray(fqp, np.float64).reshape(-1, nspb); fqh = np.asarray(fqh, np.float64).reshape(-1, nspb)
    p_start = np.concatenate([[0], np.cumsum(np_)[:-1]]).astype(np.int32)
    h_start = np.concatenate([[0], np.cumsum(nh)[:-1]]).astype(np.int32)
    return Propagator(int(nspb), np_, nh, p_start, h_start, np.asarray(ep, np.float64), np.asarray(eh, np.float64),
                      (fqp ** 2).sum(1), (fqh ** 2).sum(1), fqp, fqh)


def _triangle_ok(j2a: int, j2b: int, J: int) -> bool:
    return abs(j2a - j2b) <= 2 * J <= j2a + j2b


def two_body_channels(ms: ModelSpace):
    """Yield (chsum, parity, J, pairs) in the reference's sort order; pairs = list of (a, b), a <= b."""
    norb = ms.norb
    osh = ms.orb_sh
    och = ms.ch[osh]; oip = ms.ip[osh]; oj2 = ms.j2[osh]
    for chs in (0, 1, 2):
        for par in (0, 1):
            for J in range(ms.jmax + 1):
                pairs = []
                for a in range(norb):
                    for b in range(a, norb):
                        if och[a] + och[b] != chs or (oip[a] + oip[b]) % 2 != par:
                            continue
                        if not _triangle_ok(oj2[a], oj2[b], J):
                            continue
                        if a == b and J % 2 == 1:
                            continue
                        pairs.append((a, b))
                if pairs:
                    yield chs, par, J, pairs


def make_interaction(ms: ModelSpace, seed: int, sigma: float = 2.0) -> Interaction:
    rng = np.random.default_rng(seed)
    Nosc = (2 * ms.orb_n + ms.l[ms.orb_sh]).astype(np.float64)
    iab_l, icd_l, v_l = [], [], []
    for chs, par, J, pairs in two_body_channels(ms):
        P = np.array(pairs, np.int64)
        key = (P[:, 0] * ABMULT + P[:, 1]) * JMULT + J
        nsum = Nosc[P[:, 0]] + Nosc[P[:, 1]]
        i1, i2 = np.triu_indices(len(pairs))
        z = rng.standard_normal(len(i1))
        v = sigma * np.exp(-(nsum[i1] + nsum[i2]) / 8.0) * z
        iab_l.append(key[i1].astype(np.int32)); icd_l.append(key[i2].astype(np.int32)); v_l.append(v)
    return Interaction(np.concatenate(iab_l), np.concatenate(icd_l), np.concatenate(v_l))


def make_pivots(ms: ModelSpace, prop: Propagator, n_itr: int, z_cut: float = 60.0) -> Pivots:
    n_fw, n_bk, vec = [], [], []
    for s in range(ms.nsubsh):
        rows = []
        for (n, start, e, z, f) in ((prop.nh[s], prop.h_start[s], prop.eh, prop.zh, prop.fqh),
                                    (prop.np_[s], prop.p_start[s], prop.ep, prop.zp, prop.fqp)):
            # ascending energies, strictly increasing, Z >= z_cut (DysPivots' selection loop)
            last = -1.0e10
            while True:
                best, bi = 1.0e10, -1
                for k in range(n):
                    ek = e[start + k]
                    if ek < best and ek > last and 100.0 * z[start + k] >= z_cut:
                        best, bi = ek, k
                if bi < 0:
                    break
                last = best
                rows.append(f[start + bi, :ms.no[s]].copy())
        vec.append(np.array(rows, np.float64).reshape(-1, ms.no[s]))
        n_fw.append(np.full(len(rows), n_itr, np.int32))
        n_bk.append(np.full(len(rows), n_itr, np.int32))
    return Pivots(n_fw, n_bk, vec)


def make_problem(nmax: int, hw: float, seed: int, n_itr: int = 100, sigma: float = 2.0) -> Problem:
    ms = make_modspace(nmax, hw)
    prop = make_unperturbed_propagator(ms)
    vpp = make_interaction(ms, seed, sigma)
    piv = make_pivots(ms, prop, n_itr)
    return Problem(ms, prop, vpp, piv, seed, sigma)


# Named workloads (N_max, hw, seed, Lanczos iterations per pivot or 0 for full Dyson).
WORKLOADS = {
    "nmax4_full": dict(nmax=4, hw=20.0, seed=0, n_itr=0),
    "nmax6_lanczos50": dict(nmax=6, hw=20.0, seed=1, n_itr=50),
    "nmax8_lanczos100": dict(nmax=8, hw=20.0, seed=1, n_itr=100),
    "nmax10_lanczos100": dict(nmax=10, hw=16.0, seed=2, n_itr=100),
    "nmax12_lanczos100": dict(nmax=12, hw=16.0, seed=3, n_itr=100),
}


def make_workload(name: str) -> Problem:
    w = WORKLOADS[name]
    return make_problem(w["nmax"], w["hw"], w["seed"], max(w["n_itr"], 1))


# ---------------------------------------------------------------------------------------------
# writers in the reference's text formats
# ---------------------------------------------------------------------------------------------

def write_modspace(ms: ModelSpace, path: str) -> None:
    with open(path, "w") as f:
        f.write("# Definition of the model space by listing its s.p. orbitals\n")
        f.write("#------------------------------------------------------------\n\n")
        f.write("# number of (ilj\\pi) subshells and total number of orbitals:\n")
        f.write(f" {ms.nsubsh:7d} {ms.norb:7d}\n")
        for s in range(ms.nsubsh):
            f.write(f"\n# subshell:  {ms.name[s]} \n")
            f.write(f" {ms.l[s]:7d} {ms.j2[s]:7d} {ms.ip[s]:7d} {ms.ch[s]:7d}\n")
            f.write(f" {ms.no[s]:7d} {ms.nqp[s]:7d} {ms.nqh[s]:7d}\n")
            f.write("# principal q.#,  p/h character and sp energies:\n")
            for k in range(ms.no[s]):
                o = ms.orb_start[s] + k
                f.write(f" {ms.orb_n[o]:7d} {ms.orb_F[o]:7d} {ms.orb_xe[o]:.10f}     # {ms.orb_n[o]}{ms.name[s]}\n")


def write_propagator(ms: ModelSpace, prop: Propagator, path: str) -> None:
    with open(path, "w") as f:
        f.write("#  Quasi- particle and hole fragments of the sp propagator\n")
        f.write("#----------------------------------------------------------\n")
        f.write("\n# number of (ilj\\pi) subshells, max n. of radial orbitals:\n")
        f.write(f"# {ms.nsubsh:7d} {prop.nspb:7d} {0:7d}\n")
        f.write("\n# Total numbers of qp and qh stored here:\n")
        f.write(f"# {len(prop.ep):7d} {len(prop.eh):7d}\n")
        for s in range(ms.nsubsh):
            f.write("\n# Subshell:\n")
            f.write(f"# {ms.name[s]} \n")
            for n, st, e, z, amp, tag in ((prop.np_[s], prop.p_start[s], prop.ep, prop.zp, prop.fqp, "quasiparticles"),
                                          (prop.nh[s], prop.h_start[s], prop.eh, prop.zh, prop.fqh, "quasiholes")):
                f.write(f"# {n:7d}  # -> tot n. of {tag}\n")
                for k in range(n):
                    row = " ".join(f"{x:.17e}" for x in amp[st + k, :ms.no[s]])
                    f.write(f" {e[st + k]:.17e} {100.0 * z[st + k]:.17e} {row}\n")


def write_interaction_bcd(ms: ModelSpace, vpp: Interaction, path: str) -> None:
    """One ``.bcd`` line per stored element: ``n 2j ip ch`` for a, b, c, d, then J and V (%.17e)."""
    iab = vpp.iabJ.astype(np.int64); icd = vpp.icdJ.astype(np.int64)
    J = iab % JMULT
    a = (iab // JMULT) // ABMULT; b = (iab // JMULT) % ABMULT
    c = (icd // JMULT) // ABMULT; d = (icd // JMULT) % ABMULT
    sh = ms.orb_sh
    q = lambda o: np.stack([ms.orb_n[o], ms.j2[sh[o]], ms.ip[sh[o]], ms.ch[sh[o]]], 1)
    cols = np.concatenate([q(a), q(b), q(c), q(d), J[:, None]], 1)
    with open(path, "w") as f:
        f.write(f" {vpp.n}  {vpp.n}  # tot number of mtx el.\n")
        chunk = 1 << 20
        for s in range(0, vpp.n, chunk):
            cc = cols[s:s + chunk]; vv = vpp.V[s:s + chunk]
            lines = [" ".join(map(str, r)) + f" {x:.17e}\n" for r, x in zip(cc.tolist(), vv.tolist())]
            f.write("".join(lines))


def write_interaction_bcd_scrambled(ms: ModelSpace, vpp: Interaction, path: str, seed: int = 0,
                                    repeat: float = 0.03, pauli: int = 5, outside: int = 5) -> dict:
    """The same interaction as a ``.bcd`` a reader must put in canonical form: each line's
    pairs in random order (a <-> b and c <-> d with the exchange phase (-1)^(j_a + j_b - J + 1)
    folded into V, bra <-> ket), the lines shuffled, a fraction repeated (same value), and
    a few lines a reader must drop -- Pauli-forbidden pairs (a == b at odd J) and orbits
    outside the model space.  Returns the counts written."""
    rng = np.random.default_rng(seed)
    iab = vpp.iabJ.astype(np.int64); icd = vpp.icdJ.astype(np.int64)
    J = iab % JMULT
    a = (iab // JMULT) // ABMULT; b = (iab // JMULT) % ABMULT
    c = (icd // JMULT) // ABMULT; d = (icd // JMULT) % ABMULT
    V = vpp.V.copy()
    sh = ms.orb_sh
    j2 = ms.j2[sh]
    n = len(V)
    rep = rng.random(n) < repeat
    idx = np.concatenate([np.arange(n), np.nonzero(rep)[0]])
    a, b, c, d, J, V = a[idx], b[idx], c[idx], d[idx], J[idx], V[idx]
    m = len(V)
    s1 = rng.random(m) < 0.5
    ph1 = np.where((((j2[a] + j2[b]) // 2 - J + 1) % 2) != 0, -1.0, 1.0)
    a, b = np.where(s1, b, a), np.where(s1, a, b)
    V = np.where(s1, V * ph1, V)
    s2 = rng.random(m) < 0.5
    ph2 = np.where((((j2[c] + j2[d]) // 2 - J + 1) % 2) != 0, -1.0, 1.0)
    c, d = np.where(s2, d, c), np.where(s2, c, d)
    V = np.where(s2, V * ph2, V)
    s3 = rng.random(m) < 0.5
    a, c = np.where(s3, c, a), np.where(s3, a, c)
    b, d = np.where(s3, d, b), np.where(s3, b, d)
    q = lambda o: np.stack([ms.orb_n[o], ms.j2[sh[o]], ms.ip[sh[o]], ms.ch[sh[o]]], 1)
    cols = np.concatenate([q(a), q(b), q(c), q(d), J[:, None]], 1)
    extra, vals = [], []
    for k in range(pauli):                       # a == b at odd J
        o = int(rng.integers(ms.norb)); Jo = 2 * int(rng.integers(0, (ms.j2[sh[o]] + 1) // 2)) + 1
        if Jo > ms.j2[sh[o]]:
            Jo -= 2
        extra.append(np.concatenate([q(np.array([o]))[0], q(np.array([o]))[0], q(np.array([o]))[0],
                                     q(np.array([o]))[0], [Jo]]))
        vals.append(float(rng.normal()))
    for k in range(outside):                      # a principal number beyond the model space
        o = int(rng.integers(ms.norb))
        row = np.concatenate([q(np.array([o]))[0]] * 4 + [[0]])
        row[0] = ms.nmax + 7
        extra.append(row); vals.append(float(rng.normal()))
    if extra:
        cols = np.concatenate([cols, np.array(extra, np.int64)], 0)
        V = np.concatenate([V, np.array(vals)])
    order = rng.permutation(len(V))
    cols, V = cols[order], V[order]
    with open(path, "w") as f:
        f.write(f" {len(V)}  {len(V)}  # tot number of mtx el.\n")
        f.write("".join(" ".join(map(str, r)) + f" {x:.17e}\n" for r, x in zip(cols.tolist(), V.tolist())))
    return dict(lines=len(V), repeated=int(rep.sum()), pauli=pauli, outside=outside)


def write_pivots(ms: ModelSpace, piv: Pivots, path: str) -> None:
    with open(path, "w") as f:
        f.write("#   Template pivots file\n#\n")
        f.write("# number of (ilj\\pi) subshells, max n. of radial orbitals:\n")
        f.write(f"# {ms.nsubsh:7d} {ms.nspb_mx:7d}\n\n")
        for s in range(ms.nsubsh):
            f.write(f"\n\nshell,npvts:   {s}   {len(piv.vec[s])}  # {ms.name[s]} \n")
            for k in range(len(piv.vec[s])):
                row = " ".join(f"{x:.17e}" for x in piv.vec[s][k])
                f.write(f" {piv.n_fw[s][k]:3d}  {piv.n_bk[s][k]:3d}  {row}\n")


def write_problem(p: Problem, folder: str) -> dict:
    os.makedirs(folder, exist_ok=True)
    paths = dict(msp=os.path.join(folder, "modspace.dat"), prop=os.path.join(folder, "gprop.dat"),
                 vpp=os.path.join(folder, "vint.bcd"), piv=os.path.join(folder, "pvts.dat"))
    write_modspace(p.ms, paths["msp"])
    write_propagator(p.ms, p.prop, paths["prop"])
    write_interaction_bcd(p.ms, p.vpp, paths["vpp"])
    write_pivots(p.ms, p.piv, paths["piv"])
    return paths
