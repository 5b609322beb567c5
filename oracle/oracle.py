"""Python driver of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference arm may import
this module.  It drives the C restatement in ``oracle/bd_oracle.c`` (built by ``oracle/Makefile``)
through the reference chain of ``Run_itrs`` (source/BcDor-Main.cpp:241-391, Trel=7 ExtU1=1, one
iteration), and reads the tagged FP64 dumps written by the reference program itself
(``oracle/_ref/bd_ref_harness``) so both can be compared with the device results.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libbd_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "bd_ref_harness")

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


class _Problem(C.Structure):
    _fields_ = [("nsubsh", C.c_int), ("norb", C.c_int), ("jmax", C.c_int), ("nspb", C.c_int),
                ("l", C.c_void_p), ("j2", C.c_void_p), ("ip", C.c_void_p), ("ch", C.c_void_p),
                ("no", C.c_void_p), ("orb_start", C.c_void_p), ("orb_sh", C.c_void_p),
                ("np", C.c_void_p), ("nh", C.c_void_p), ("p_start", C.c_void_p), ("h_start", C.c_void_p),
                ("ep", C.c_void_p), ("eh", C.c_void_p), ("fqp", C.c_void_p), ("fqh", C.c_void_p),
                ("n_qp", C.c_int), ("n_qh", C.c_int),
                ("n_me", C.c_int), ("iabJ", C.c_void_p), ("icdJ", C.c_void_p), ("V", C.c_void_p),
                ("seg_str", C.c_void_p), ("seg_end", C.c_void_p)]


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


# The reference's source folder (BD_REFERENCE_SOURCE overrides the mount point).
REF_SOURCE = os.environ.get("BD_REFERENCE_SOURCE", "/root/reference/source")


def build_ref() -> bool:
    """Builds oracle/_ref from the reference sources when they are mounted."""
    if not os.path.isdir(REF_SOURCE):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", "-j8"], check=True, stdout=subprocess.DEVNULL)
    return os.path.exists(REF_BIN)


def find_openblas():
    """(path, symbol) of a dsyevd in SciPy's or NumPy's bundled OpenBLAS, or None."""
    try:
        import scipy
        cands = sorted(glob.glob(os.path.dirname(scipy.__file__) + ".libs/libscipy_openblas*.so*"))
        for c in cands:
            return c, "scipy_dsyevd_"
    except ImportError:
        pass
    return None


class Oracle:
    def __init__(self, use_lapack: bool = True):
        if not os.path.exists(PORT_SO):
            build()
        lib = C.CDLL(PORT_SO)
        self.lib = lib
        pp = C.POINTER(_Problem)
        lib.bdo_count_poles.argtypes = [pp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.bdo_sigma2.argtypes = [pp, C.c_int, _f64p, C.c_int, _f64p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.bdo_sigma2.restype = C.c_int
        lib.bdo_sort_u.argtypes = [C.c_int, C.c_int, C.c_int, _f64p]
        lib.bdo_sort_d.argtypes = [C.c_int, C.c_int, C.c_int, _f64p]
        lib.bdo_sort_perm.argtypes = [C.c_int, _f64p, C.c_int, _i32p]
        lib.bdo_reduce_mtx_lncz.argtypes = [C.c_int, C.c_int, C.c_int, _f64p, _i32p, C.c_int, C.c_int, C.c_int,
                                            _f64p, C.c_int, _f64p, _i32p]
        lib.bdo_reduce_mtx_lncz.restype = C.c_int
        lib.bdo_reduce_mtx_lncz_passes.argtypes = lib.bdo_reduce_mtx_lncz.argtypes + [C.c_int]
        lib.bdo_reduce_mtx_lncz_passes.restype = C.c_int
        lib.bdo_lanczos_sizes.argtypes = [C.c_int, _i32p, C.c_int]
        lib.bdo_lanczos_sizes.restype = C.c_int
        lib.bdo_ehf.argtypes = [pp, C.c_int, _f64p]
        lib.bdo_seek_efermi.argtypes = [pp, C.c_int]
        lib.bdo_seek_efermi.restype = C.c_double
        lib.bdo_vget.argtypes = [pp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        lib.bdo_vget.restype = C.c_double
        lib.bdo_segments.argtypes = [C.c_int, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p]
        lib.bdo_set_lapack.argtypes = [C.c_char_p, C.c_char_p]
        lib.bdo_set_lapack.restype = C.c_int
        lib.bdo_has_lapack.restype = C.c_int
        lib.bdo_dyson.argtypes = [C.c_int, C.c_int, _f64p, _f64p, C.c_double, C.c_int,
                                  C.c_int, _f64p, C.c_int, _i32p, C.c_int, _f64p, C.c_int, _i32p,
                                  _f64p, C.POINTER(C.c_int), C.POINTER(C.c_int), _f64p]
        lib.bdo_dyson.restype = C.c_int
        self.lapack = None
        if use_lapack and not lib.bdo_has_lapack():
            ob = find_openblas()
            if ob and lib.bdo_set_lapack(ob[0].encode(), ob[1].encode()) == 0:
                self.lapack = ob
        elif lib.bdo_has_lapack():
            self.lapack = ("preloaded", "")

    # ------------------------------------------------------------------ problem binding
    def bind(self, prob):
        ms, pr, vp = prob.ms, prob.prop, prob.vpp
        keep = dict(
            l=np.ascontiguousarray(ms.l, np.int32), j2=np.ascontiguousarray(ms.j2, np.int32),
            ip=np.ascontiguousarray(ms.ip, np.int32), ch=np.ascontiguousarray(ms.ch, np.int32),
            no=np.ascontiguousarray(ms.no, np.int32), orb_start=np.ascontiguousarray(ms.orb_start, np.int32),
            orb_sh=np.ascontiguousarray(ms.orb_sh, np.int32),
            np=np.ascontiguousarray(pr.np_, np.int32), nh=np.ascontiguousarray(pr.nh, np.int32),
            p_start=np.ascontiguousarray(pr.p_start, np.int32), h_start=np.ascontiguousarray(pr.h_start, np.int32),
            ep=np.ascontiguousarray(pr.ep, np.float64) if len(pr.ep) else np.zeros(1),
            eh=np.ascontiguousarray(pr.eh, np.float64) if len(pr.eh) else np.zeros(1),
            fqp=np.ascontiguousarray(pr.fqp, np.float64).reshape(-1) if len(pr.ep) else np.zeros(pr.nspb),
            fqh=np.ascontiguousarray(pr.fqh, np.float64).reshape(-1) if len(pr.eh) else np.zeros(pr.nspb),
            iabJ=np.ascontiguousarray(vp.iabJ, np.int32), icdJ=np.ascontiguousarray(vp.icdJ, np.int32),
            V=np.ascontiguousarray(vp.V, np.float64),
            seg_str=np.zeros(5 * 128 * 2, np.int32), seg_end=np.zeros(5 * 128 * 2, np.int32))
        self.lib.bdo_segments(vp.n, keep["iabJ"], keep["orb_sh"], keep["ch"], keep["ip"],
                              keep["seg_str"], keep["seg_end"])
        P = _Problem()
        P.nsubsh, P.norb, P.jmax, P.nspb = ms.nsubsh, ms.norb, ms.jmax, pr.nspb
        for k in ("l", "j2", "ip", "ch", "no", "orb_start", "orb_sh", "np", "nh", "p_start", "h_start",
                  "ep", "eh", "fqp", "fqh", "iabJ", "icdJ", "V", "seg_str", "seg_end"):
            setattr(P, k, keep[k].ctypes.data)
        P.n_qp, P.n_qh, P.n_me = len(pr.ep), len(pr.eh), vp.n
        self._keep, self._P, self.prob = keep, P, prob
        return self

    # ------------------------------------------------------------------ boundary calls
    def count_poles(self, ish):
        a, b = C.c_int(), C.c_int()
        self.lib.bdo_count_poles(C.byref(self._P), ish, C.byref(a), C.byref(b))
        return a.value, b.value

    def sigma2(self, ish):
        nfw, nbk = self.count_poles(ish)
        D = int(self.prob.ms.no[ish])
        fw = np.zeros(max(nfw, 1) * (2 + D)); bk = np.zeros(max(nbk, 1) * (2 + D))
        a, b = C.c_int(), C.c_int()
        rc = self.lib.bdo_sigma2(C.byref(self._P), ish, fw, max(nfw, 1), bk, max(nbk, 1), C.byref(a), C.byref(b))
        assert rc == 0 and a.value == nfw and b.value == nbk
        return fw[: nfw * (2 + D)].reshape(nfw, 2 + D), bk[: nbk * (2 + D)].reshape(nbk, 2 + D)

    def ehf(self, ish):
        D = int(self.prob.ms.no[ish]); U = np.zeros(D * D)
        self.lib.bdo_ehf(C.byref(self._P), ish, U)
        return U.reshape(D, D)

    def sig1b(self, ish):
        ms = self.prob.ms
        s = ms.orb_start[ish]
        return np.diag(ms.orb_xe[s:s + ms.no[ish]]).astype(np.float64)

    def efermi(self, ish):
        return self.lib.bdo_seek_efermi(C.byref(self._P), ish)

    def sort_perm(self, key, desc: bool):
        """Row permutation of Sort_u_double2dim (ascending) / Sort_d_double2dim (descending),
        source/BcDor-Utilities.cpp:25-94: sorted row r is input row perm[r]."""
        key = np.ascontiguousarray(key, np.float64)
        perm = np.zeros(len(key), np.int32)
        if len(key):
            self.lib.bdo_sort_perm(len(key), key, 1 if desc else 0, perm)
        return perm

    def reduce_lanczos(self, ish, fw, bk, pivots, nitr_fw, nitr_bk, passes: int = 1):
        """Reduce_SelfEn_Lncz (source/BcDor-Self_energy_ext_Op_e.cpp:55-232): sorts fw ascending and
        bk descending in place, then Reduce_Mtx_Lncz for each direction.  ``passes`` = 1 is the
        reference's single backward Gram-Schmidt sweep (bit-identical); 2 repeats the sweep, which keeps
        the Lanczos basis orthonormal after breakdowns.  Returns dict."""
        D = int(self.prob.ms.no[ish]); npv = len(pivots)
        NDEN_out = npv + 1; NT_out = NDEN_out + D
        out = {"NDEN": NDEN_out}
        fw = np.ascontiguousarray(fw).copy(); bk = np.ascontiguousarray(bk).copy()
        if len(fw): self.lib.bdo_sort_u(len(fw), 2 + D, 0, fw.reshape(-1))
        if len(bk): self.lib.bdo_sort_d(len(bk), 2 + D, 0, bk.reshape(-1))
        out["sorted_fw"], out["sorted_bk"] = fw, bk
        for tag, rows, nitr in (("fw", fw, nitr_fw), ("bk", bk, nitr_bk)):
            N = len(rows)
            nit = np.ascontiguousarray(nitr, np.int32).copy()
            tot = int(nit[nit > 0].sum())
            nL = min(tot, N)
            piv = np.ascontiguousarray(pivots, np.float64).copy()
            if N < 1 or nL < 1:
                out["lz_" + tag] = np.zeros((0, NT_out)); out["ipiv_" + tag] = np.full(NT_out, -100, np.int32)
                out["n_piv_" + tag] = 0; continue
            if tot > N:
                x1 = float(N) / float(tot)
                nit = np.array([int(x1 * v + 1.0) for v in nit], np.int32)
            Mout = np.zeros(nL * NT_out); ipiv = np.full(NT_out, -100, np.int32)
            L = self.lib.bdo_reduce_mtx_lncz_passes(NDEN_out, D, nL, Mout, ipiv, 2, D, N,
                                                    np.ascontiguousarray(rows).reshape(-1), npv, piv.reshape(-1),
                                                    nit, passes)
            assert L >= 0, L
            out["lz_" + tag] = Mout[: L * NT_out].reshape(L, NT_out)
            out["ipiv_" + tag] = ipiv
            out["n_piv_" + tag] = int(ipiv[0])
            out["nitr_" + tag] = nit
        return out

    def dyson(self, ish, sig1b, sighf, NDEN, fw, bk, n_piv_fw=0, ipiv_fw=None, n_piv_bk=0, ipiv_bk=None):
        D = int(self.prob.ms.no[ish]); j2 = int(self.prob.ms.j2[ish])
        fw = np.ascontiguousarray(fw, np.float64).copy(); bk = np.ascontiguousarray(bk, np.float64).copy()
        n = D + len(fw) + len(bk)
        sol = np.zeros(n * (2 + D)); kol = np.zeros(3); nf, nb = C.c_int(), C.c_int()
        dummy = np.zeros(1, np.int32)
        rc = self.lib.bdo_dyson(D, j2, np.ascontiguousarray(sig1b).reshape(-1), np.ascontiguousarray(sighf).reshape(-1),
                                self.efermi(ish), NDEN, len(fw), fw.reshape(-1) if len(fw) else np.zeros(1),
                                n_piv_fw, ipiv_fw if ipiv_fw is not None else dummy,
                                len(bk), bk.reshape(-1) if len(bk) else np.zeros(1),
                                n_piv_bk, ipiv_bk if ipiv_bk is not None else dummy,
                                sol, C.byref(nf), C.byref(nb), kol)
        assert rc == 0, rc
        sol = sol.reshape(n, 2 + D)
        return dict(qp=sol[: nf.value], qh=sol[nf.value:], koltun=kol)

    def run_channel(self, ish, lanczos: bool, passes: int = 1):
        sighf = self.ehf(ish); sig1b = self.sig1b(ish)
        fw, bk = self.sigma2(ish)
        res = dict(sig_hf=sighf, sig_1b=sig1b, sig_fw=fw, sig_bk=bk)
        if lanczos:
            pv = self.prob.piv
            lz = self.reduce_lanczos(ish, fw, bk, pv.vec[ish], pv.n_fw[ish], pv.n_bk[ish], passes)
            res.update(lz)
            dy = self.dyson(ish, sig1b, sighf, lz["NDEN"], lz["lz_fw"], lz["lz_bk"],
                            lz["n_piv_fw"], lz["ipiv_fw"], lz["n_piv_bk"], lz["ipiv_bk"])
        else:
            dy = self.dyson(ish, sig1b, sighf, 2, fw, bk)
        res.update(dy)
        return res


# ---------------------------------------------------------------------------------------------
# the next iteration's propagator
# ---------------------------------------------------------------------------------------------

def dressed_propagator(ms, results, nspb, z_cut, max_frag):
    """Propagator of the next iteration from every channel's Dyson solutions.

    DysonMatrix hands its solutions, quasiparticles and quasiholes each sorted by
    descending W, to SpProp_t::add_qp / add_qh (source/BcDor-DysonMatrix.cpp:481-488),
    which append them subshell by subshell with amplitudes x_0..x_{D-1} padded with
    zeros to N_SPB_MX and Z recomputed as sum x^2 (source/BcDor-Sp_Propagator.cpp:683-809);
    Run_itrs then uses that propagator as the next input (source/BcDor-Main.cpp:438-441).
    The truncation is this build's (the reference keeps everything): per subshell and
    side, the solutions with Z >= z_cut, at most max_frag of them (max_frag <= 0: all)
    with the largest Z, earlier rows first on ties, kept in their stored order.
    results[ish] = dict(qp=rows, qh=rows), rows [W, Z, x...] as DysonMatrix returns them."""
    out = {"np": [], "nh": [], "ep": [], "eh": [], "fqp": [], "fqh": []}
    for ish in range(ms.nsubsh):
        D = int(ms.no[ish])
        for side, (kn, ke, kf) in (("qp", ("np", "ep", "fqp")), ("qh", ("nh", "eh", "fqh"))):
            rows = np.asarray(results[ish][side]).reshape(-1, 2 + D)
            z = (rows[:, 2:2 + D] ** 2).sum(1)
            keep = [k for k in range(len(rows)) if z[k] >= z_cut]
            if max_frag > 0 and len(keep) > max_frag:
                keep = sorted(sorted(keep, key=lambda k: -z[k])[:max_frag])
            for k in keep:
                out[ke].append(rows[k, 0])
                amp = np.zeros(nspb); amp[:D] = rows[k, 2:2 + D]
                out[kf].append(amp)
            out[kn].append(len(keep))
    return out


def quick_n_dirty_diff(ep_a, eh_a, ep_b, eh_b):
    """SpProp_t::quick_n_dirty_diff (source/BcDor-Sp_Propagator.cpp:1189-1219): sum of
    |E_a - E_b| over the flat quasiparticle and quasihole lists, the shorter padded
    with zeros."""
    d = 0.0
    for a, b in ((np.asarray(ep_a), np.asarray(ep_b)), (np.asarray(eh_a), np.asarray(eh_b))):
        n = max(len(a), len(b))
        aa = np.zeros(n); aa[:len(a)] = a
        bb = np.zeros(n); bb[:len(b)] = b
        d += float(np.abs(aa - bb).sum())
    return d


# ---------------------------------------------------------------------------------------------
# reference dumps
# ---------------------------------------------------------------------------------------------

def read_dump(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    off = 0
    while off < len(data):
        (ln,) = struct.unpack_from("<i", data, off); off += 4
        tag = data[off:off + ln].decode(); off += ln
        kind, cnt = struct.unpack_from("<iq", data, off); off += 12
        dt = np.float64 if kind == 0 else np.int32
        nb = cnt * (8 if kind == 0 else 4)
        out[tag] = np.frombuffer(data[off:off + nb], dtype=dt).copy(); off += nb
    return out


def run_reference(paths: dict, hw: float, out_path: str, lanczos: bool, channels=None, threads: int = 1):
    """Runs oracle/_ref/bd_ref_harness on reference-format files; returns the parsed dump."""
    env = dict(os.environ, OPENBLAS_NUM_THREADS=str(threads))
    args = [REF_BIN, paths["msp"], paths["prop"], paths["vpp"], paths["piv"] if lanczos else "-", repr(float(hw)), out_path]
    args += [str(c) for c in (channels or [])]
    subprocess.run(args, check=True, env=env, stdout=subprocess.DEVNULL)
    return read_dump(out_path)


def reference_channel(dump: dict, ish: int, D: int):
    """Splits one channel of a reference dump into the same keys as Oracle.run_channel."""
    g = lambda k: dump.get(f"c{ish}/{k}")
    r = dict(sig_hf=g("sig_hf").reshape(D, D), sig_1b=g("sig_1b").reshape(D, D),
             sig_fw=g("sig_fw").reshape(-1, 2 + D), sig_bk=g("sig_bk").reshape(-1, 2 + D),
             qp=g("qp").reshape(-1, 2 + D), qh=g("qh").reshape(-1, 2 + D), koltun=g("koltun"), time=g("time"))
    if g("lz_hdr") is not None:
        nden, npf, npb = (int(x) for x in g("lz_hdr"))
        r.update(NDEN=nden, n_piv_fw=npf, n_piv_bk=npb,
                 lz_fw=g("lz_fw").reshape(-1, nden + D), lz_bk=g("lz_bk").reshape(-1, nden + D),
                 ipiv_fw=g("ipiv_fw"), ipiv_bk=g("ipiv_bk"),
                 sorted_fw=g("sorted_fw").reshape(-1, 2 + D), sorted_bk=g("sorted_bk").reshape(-1, 2 + D))
    return r
