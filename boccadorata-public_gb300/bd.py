"""ctypes binding of the C ABI (include/bd_gb300.h) and a host-side mirror of the
reference's call boundaries.

``Context`` wraps one ``bd_ctx``.  ``WideSelfEnergy`` and ``dyson_matrix`` mirror,
name for name, the three calls of the reference's per-channel loop
(source/BcDor-Main.cpp:241-391):

* ``WideSelfEnergy.Build_Dynamic_SlfEn_2ndOrder``  (source/BcDor-Self_energy_ext_Op_c.cpp:323)
* ``WideSelfEnergy.Reduce_SelfEn_Lncz``            (source/BcDor-Self_energy_ext_Op_e.cpp:55)
* ``dyson_matrix``                                 (source/BcDor-DysonMatrix.cpp:123)

There is no CPU fallback: importing this module raises when the CUDA library has
not been built, and every call goes through the device.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import importlib
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbd_gb300.so")

BD_OK, BD_ERR_ARG, BD_ERR_CUDA, BD_ERR_CAPACITY, BD_ERR_STATE, BD_ERR_NUMERIC, BD_ERR_TIMEOUT = 0, -1, -2, -3, -4, -5, -6
BD_RUN_LANCZOS, BD_RUN_MIXED, BD_RUN_PER_CHANNEL, BD_RUN_REF_ORDER, BD_RUN_GRAPH = 1, 2, 4, 8, 16
BD_RUN_FP64_COUPLINGS = 32

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)


class _ModSpace(C.Structure):
    _fields_ = [("nsubsh", C.c_int), ("norb", C.c_int), ("l", _ip), ("j2", _ip), ("ip", _ip), ("ch", _ip),
                ("no", _ip), ("orb_sh", _ip), ("orb_xe", _dp)]


class _Propagator(C.Structure):
    _fields_ = [("nspb", C.c_int), ("np", _ip), ("nh", _ip), ("ep", _dp), ("eh", _dp), ("fqp", _dp), ("fqh", _dp)]


class _Interaction(C.Structure):
    _fields_ = [("n_me", C.c_int), ("iabJ", _ip), ("icdJ", _ip), ("V", _dp)]


class _Pivots(C.Structure):
    _fields_ = [("npvt", _ip), ("n_itr_fw", _ip), ("n_itr_bk", _ip), ("vec", _dp)]


class BDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"bd error {code}: {msg}")
        self.code = code


EXPORTED = ["bd_create", "bd_destroy", "bd_last_error", "bd_version", "bd_upload_problem", "bd_upload_pivots",
            "bd_count_poles", "bd_ehf", "bd_sigma2_build", "bd_lanczos_reduce", "bd_dyson_solve", "bd_run_all",
            "bd_sync", "bd_result_counts", "bd_result_fetch", "bd_result_koltun_all", "bd_last_timings",
            "bd_dyson_rows", "bd_lanczos_vectors", "bd_upload_propagator", "bd_dressed_propagator",
            "bd_result_fetch_all", "bd_sigma2_sorted", "bd_files_open", "bd_files_close", "bd_files_error",
            "bd_files_read_propagator", "bd_files_read_pivots", "bd_files_read_interaction", "bd_files_modspace",
            "bd_files_propagator", "bd_files_pivots", "bd_files_interaction_lines", "bd_upload_files",
            "bd_interaction_fetch", "bd_files_write_propagator", "bd_files_write_pivots", "bd_write_interaction_bin",
            "bd_files_save_selfenergy", "bd_files_load_selfenergy", "bd_files_selfenergy_name", "bd_autotune",
            "bd_dressed_on_device", "bd_tensor_couplings"]


def load_library(path: str = LIB_PATH):
    if not os.path.exists(path):
        raise ImportError(f"CUDA library not built: {path} (run __graft_entry__.build())")
    lib = C.CDLL(path)
    vp = C.c_void_p
    lib.bd_create.argtypes = [C.POINTER(vp), C.c_int]
    lib.bd_destroy.argtypes = [vp]; lib.bd_destroy.restype = None
    lib.bd_last_error.argtypes = [vp]; lib.bd_last_error.restype = C.c_char_p
    lib.bd_upload_problem.argtypes = [vp, C.POINTER(_ModSpace), C.POINTER(_Interaction), C.POINTER(_Propagator)]
    lib.bd_upload_pivots.argtypes = [vp, C.POINTER(_Pivots)]
    lib.bd_count_poles.argtypes = [vp, C.c_int, _ip, _ip]
    lib.bd_ehf.argtypes = [vp, C.c_int, _dp]
    lib.bd_sigma2_build.argtypes = [vp, C.c_int, _dp, C.c_int, _ip, _dp, C.c_int, _ip]
    lib.bd_sigma2_sorted.argtypes = [vp, C.c_int, _dp, C.c_int, _dp, C.c_int]
    lib.bd_lanczos_reduce.argtypes = [vp, C.c_int, C.c_int, _dp, _ip, _ip, _dp, C.c_int, _ip, _ip,
                                      _dp, C.c_int, _ip, _ip, C.c_int]
    lib.bd_dyson_solve.argtypes = [vp, C.c_int, _dp, _dp, C.c_double, _dp, C.c_int, _ip, _dp, C.c_int, _ip, _dp]
    lib.bd_dyson_rows.argtypes = [vp, C.c_int, C.c_int, C.c_int, _dp, _ip, C.c_int, _dp, _ip, _dp, _dp, C.c_double,
                                  _dp, C.c_int, _ip, _dp, C.c_int, _ip, _dp]
    lib.bd_lanczos_vectors.argtypes = [vp, C.c_int, C.c_int, C.c_int, _dp, C.c_longlong]
    lib.bd_upload_propagator.argtypes = [vp, C.POINTER(_Propagator)]
    lib.bd_dressed_propagator.argtypes = [vp, C.c_double, C.c_int, C.c_int, _ip, _ip, _dp, C.c_int, _dp, C.c_int,
                                          _dp, _dp, _dp]
    lib.bd_run_all.argtypes = [vp, C.c_int]
    lib.bd_sync.argtypes = [vp]
    lib.bd_result_counts.argtypes = [vp, C.c_int, _ip, _ip]
    lib.bd_result_fetch.argtypes = [vp, C.c_int, _dp, C.c_int, _dp, C.c_int, _dp]
    lib.bd_result_koltun_all.argtypes = [vp, _dp]
    lib.bd_result_fetch_all.argtypes = [vp, _dp, C.c_longlong, _ip, _dp]
    lib.bd_last_timings.argtypes = [vp, _dp]
    lib.bd_diag_two_pass.argtypes = [vp]
    lib.bd_dressed_on_device.argtypes = [vp]
    lib.bd_tensor_couplings.argtypes = [vp]
    lib.bd_set_tuning.argtypes = [vp, C.c_int, C.c_int, C.c_double]
    lib.bd_autotune.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.bd_set_lanczos_slices.argtypes = [vp, C.c_int]
    lib.bd_lanczos_stored.argtypes = [vp, _ip]
    lib.bd_lanczos_kernel_ms.argtypes = [vp]; lib.bd_lanczos_kernel_ms.restype = C.c_double
    lib.bd_launch_count.argtypes = [vp]; lib.bd_launch_count.restype = C.c_longlong
    cp = C.c_char_p
    lp = C.POINTER(C.c_longlong)
    lib.bd_files_open.argtypes = [C.POINTER(vp), cp]
    lib.bd_files_close.argtypes = [vp]; lib.bd_files_close.restype = None
    lib.bd_files_error.argtypes = [vp]; lib.bd_files_error.restype = cp
    lib.bd_files_read_propagator.argtypes = [vp, cp]
    lib.bd_files_read_pivots.argtypes = [vp, cp]
    lib.bd_files_read_interaction.argtypes = [vp, cp, C.c_int]
    lib.bd_files_modspace.argtypes = [vp, C.POINTER(_ModSpace), C.POINTER(_ip), C.POINTER(C.POINTER(cp))]
    lib.bd_files_propagator.argtypes = [vp, C.POINTER(_Propagator), C.POINTER(_dp), C.POINTER(_dp)]
    lib.bd_files_pivots.argtypes = [vp, C.POINTER(_Pivots)]
    lib.bd_files_interaction_lines.argtypes = [vp, lp, lp, lp]
    lib.bd_upload_files.argtypes = [vp, vp]
    lib.bd_interaction_fetch.argtypes = [vp, _ip, _ip, _dp, C.c_longlong, lp, lp]
    lib.bd_files_write_propagator.argtypes = [vp, cp, C.POINTER(_Propagator), _dp, _dp]
    lib.bd_files_write_pivots.argtypes = [vp, cp, C.POINTER(_Propagator), _dp, _dp, C.c_int, C.c_int, C.c_double]
    lib.bd_write_interaction_bin.argtypes = [cp, C.POINTER(_Interaction), C.c_longlong]
    lib.bd_files_save_selfenergy.argtypes = [vp, cp, C.c_int, C.c_int, C.c_int, _dp, _ip, C.c_int, _dp, _ip, C.c_int]
    lib.bd_files_load_selfenergy.argtypes = [vp, cp, C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp, C.c_int, _ip]
    lib.bd_files_selfenergy_name.argtypes = [vp, cp, cp, C.c_int, C.c_char_p, C.c_int]
    return lib


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = load_library()
    return _LIB


def _i(a):
    return np.ascontiguousarray(a, np.int32)


def _d(a):
    return np.ascontiguousarray(a, np.float64)


def _pi(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def _pd(a):
    return a.ctypes.data_as(_dp) if a is not None else None


class Context:
    """One device context with the problem resident in HBM."""

    def __init__(self, device: int = 0):
        self.lib = lib()
        h = C.c_void_p()
        rc = self.lib.bd_create(C.byref(h), device)
        if rc != BD_OK:
            raise BDError(rc, "bd_create failed (no usable CUDA device?)")
        self.h = h
        self._keep = []
        self.prob = None

    def close(self):
        if self.h:
            self.lib.bd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        if rc != BD_OK:
            raise BDError(rc, self.lib.bd_last_error(self.h).decode())
        return rc

    # ---------------------------------------------------------------- inputs
    def upload(self, prob, with_pivots: bool = True):
        ms, pr, vp = prob.ms, prob.prop, prob.vpp
        arrs = dict(l=_i(ms.l), j2=_i(ms.j2), ip=_i(ms.ip), ch=_i(ms.ch), no=_i(ms.no), orb_sh=_i(ms.orb_sh),
                    orb_xe=_d(ms.orb_xe), np=_i(pr.np_), nh=_i(pr.nh),
                    ep=_d(pr.ep if len(pr.ep) else np.zeros(1)), eh=_d(pr.eh if len(pr.eh) else np.zeros(1)),
                    fqp=_d(pr.fqp.reshape(-1) if len(pr.ep) else np.zeros(pr.nspb)),
                    fqh=_d(pr.fqh.reshape(-1) if len(pr.eh) else np.zeros(pr.nspb)),
                    iabJ=_i(vp.iabJ), icdJ=_i(vp.icdJ), V=_d(vp.V))
        m = _ModSpace(ms.nsubsh, ms.norb, _pi(arrs["l"]), _pi(arrs["j2"]), _pi(arrs["ip"]), _pi(arrs["ch"]),
                      _pi(arrs["no"]), _pi(arrs["orb_sh"]), _pd(arrs["orb_xe"]))
        p = _Propagator(pr.nspb, _pi(arrs["np"]), _pi(arrs["nh"]), _pd(arrs["ep"]), _pd(arrs["eh"]),
                        _pd(arrs["fqp"]), _pd(arrs["fqh"]))
        v = _Interaction(vp.n, _pi(arrs["iabJ"]), _pi(arrs["icdJ"]), _pd(arrs["V"]))
        self._chk(self.lib.bd_upload_problem(self.h, C.byref(m), C.byref(v), C.byref(p)))
        self.prob = prob
        if with_pivots and prob.piv is not None:
            self.upload_pivots(prob.piv)
        return self

    def upload_files(self, files: "Files", prob=None):
        """The problem of a Files object (bd_upload_files); prob (optional) is kept for the
        helpers that read model-space sizes."""
        self._chk(self.lib.bd_upload_files(self.h, files.h))
        self.prob = prob
        return self

    def interaction(self):
        """The resident interaction list (iabJ, icdJ, V) and the repeated pairs left out."""
        n, r = C.c_longlong(), C.c_longlong()
        self._chk(self.lib.bd_interaction_fetch(self.h, None, None, None, 0, C.byref(n), C.byref(r)))
        a, b, v = np.zeros(max(n.value, 1), np.int32), np.zeros(max(n.value, 1), np.int32), np.zeros(max(n.value, 1))
        self._chk(self.lib.bd_interaction_fetch(self.h, _pi(a), _pi(b), _pd(v), len(v), C.byref(n), C.byref(r)))
        return a[:n.value], b[:n.value], v[:n.value], r.value

    def upload_propagator(self, prop):
        """Replace the input propagator; model space, interaction and pivots stay."""
        arrs = dict(np=_i(prop.np_), nh=_i(prop.nh), ep=_d(prop.ep if len(prop.ep) else np.zeros(1)),
                    eh=_d(prop.eh if len(prop.eh) else np.zeros(1)),
                    fqp=_d(prop.fqp.reshape(-1) if len(prop.ep) else np.zeros(prop.nspb)),
                    fqh=_d(prop.fqh.reshape(-1) if len(prop.eh) else np.zeros(prop.nspb)))
        p = _Propagator(prop.nspb, _pi(arrs["np"]), _pi(arrs["nh"]), _pd(arrs["ep"]), _pd(arrs["eh"]),
                        _pd(arrs["fqp"]), _pd(arrs["fqh"]))
        self._chk(self.lib.bd_upload_propagator(self.h, C.byref(p)))
        self.prob = dataclasses.replace(self.prob, prop=prop)
        return self

    def dressed_propagator(self, z_cut: float, max_frag: int, keep_current: bool = False):
        """The next iteration's (truncated) propagator from the last run_all; returns it and
        the reference's quick_n_dirty_diff against the propagator the run used.  Unless
        keep_current, it becomes the context's input propagator."""
        ns, nspb = self.prob.ms.nsubsh, self.prob.prop.nspb
        cnt = [self.result_counts(i) for i in range(ns)]
        cap_p = max(1, sum(c[0] for c in cnt)); cap_h = max(1, sum(c[1] for c in cnt))
        npo, nho = np.zeros(ns, np.int32), np.zeros(ns, np.int32)
        ep, eh = np.zeros(cap_p), np.zeros(cap_h)
        fqp, fqh = np.zeros(cap_p * nspb), np.zeros(cap_h * nspb)
        diff = C.c_double()
        self._chk(self.lib.bd_dressed_propagator(self.h, z_cut, max_frag, 1 if keep_current else 0, _pi(npo), _pi(nho),
                                                 _pd(ep), cap_p, _pd(eh), cap_h, _pd(fqp), _pd(fqh), C.byref(diff)))
        a, b = int(npo.sum()), int(nho.sum())
        synth = importlib.import_module("boccadorata-public_gb300.synth")
        prop = synth.propagator_from_arrays(nspb, npo, nho, ep[:a], eh[:b], fqp[:a * nspb], fqh[:b * nspb])
        if not keep_current:
            self.prob = dataclasses.replace(self.prob, prop=prop)
        return prop, diff.value

    def upload_pivots(self, piv):
        npvt = _i([len(v) for v in piv.vec])
        nfw = _i(np.concatenate([np.asarray(x, np.int32) for x in piv.n_fw]) if len(piv.n_fw) else [])
        nbk = _i(np.concatenate([np.asarray(x, np.int32) for x in piv.n_bk]) if len(piv.n_bk) else [])
        vec = _d(np.concatenate([np.asarray(x, np.float64).reshape(-1) for x in piv.vec]))
        pv = _Pivots(_pi(npvt), _pi(nfw), _pi(nbk), _pd(vec))
        self._chk(self.lib.bd_upload_pivots(self.h, C.byref(pv)))

    def set_tuning(self, lz_cluster=8, dy_cluster=8, eta=0.70710678118654752):
        self._chk(self.lib.bd_set_tuning(self.h, lz_cluster, dy_cluster, eta))

    def lanczos_stored(self):
        """(nsubsh, 2) vectors built per chain in the last reduction (fw, bk)."""
        out = np.zeros(2 * self.prob.ms.nsubsh, np.int32)
        self._chk(self.lib.bd_lanczos_stored(self.h, _pi(out)))
        return out.reshape(-1, 2)

    def set_lanczos_slices(self, mode: int):
        """0: by size (default), 1: shared memory, 2: global memory."""
        self._chk(self.lib.bd_set_lanczos_slices(self.h, mode))

    # ---------------------------------------------------------------- per channel
    def D(self, ish):
        return int(self.prob.ms.no[ish])

    def count_poles(self, ish):
        a, b = C.c_int(), C.c_int()
        self._chk(self.lib.bd_count_poles(self.h, ish, C.byref(a), C.byref(b)))
        return a.value, b.value

    def ehf(self, ish):
        D = self.D(ish)
        U = np.zeros(D * D)
        self._chk(self.lib.bd_ehf(self.h, ish, _pd(U)))
        return U.reshape(D, D)

    def sigma2_build(self, ish, copy: bool = True):
        nfw, nbk = self.count_poles(ish)
        D = self.D(ish)
        fw = np.zeros((max(nfw, 1), 2 + D)) if copy else None
        bk = np.zeros((max(nbk, 1), 2 + D)) if copy else None
        a, b = C.c_int(), C.c_int()
        self._chk(self.lib.bd_sigma2_build(self.h, ish, _pd(fw), max(nfw, 1), C.byref(a), _pd(bk), max(nbk, 1),
                                           C.byref(b)))
        if not copy:
            return None, None
        return fw[:a.value], bk[:b.value]

    def sigma2_sorted(self, ish):
        """Rows of the resident Sigma(2) as the reference's in-place sort of
        Reduce_SelfEn_Lncz leaves them (heap-sort order of equal energies)."""
        nfw, nbk = self.count_poles(ish)
        D = self.D(ish)
        fw, bk = np.zeros((max(nfw, 1), 2 + D)), np.zeros((max(nbk, 1), 2 + D))
        self._chk(self.lib.bd_sigma2_sorted(self.h, ish, _pd(fw), max(nfw, 1), _pd(bk), max(nbk, 1)))
        return fw[:nfw], bk[:nbk]

    def lanczos_reduce(self, ish, pivots, nitr_fw, nitr_bk, mixed: bool = False, ref_order: bool = False):
        D = self.D(ish)
        piv = _d(np.array(pivots, np.float64).reshape(-1, D)).copy()
        nf, nb = _i(nitr_fw).copy(), _i(nitr_bk).copy()
        npv = len(piv)
        nfw, nbk = self.count_poles(ish)
        capf, capb = max(1, min(int(nf[nf > 0].sum()), nfw)), max(1, min(int(nb[nb > 0].sum()), nbk))
        nt = npv + 1 + D
        lf, lb = np.zeros((capf, nt)), np.zeros((capb, nt))
        ipf, ipb = np.zeros(nt, np.int32), np.zeros(nt, np.int32)
        Lf, Lb = C.c_int(), C.c_int()
        self._chk(self.lib.bd_lanczos_reduce(self.h, ish, npv, _pd(piv), _pi(nf), _pi(nb), _pd(lf), capf, C.byref(Lf),
                                             _pi(ipf), _pd(lb), capb, C.byref(Lb), _pi(ipb),
                                             (BD_RUN_MIXED if mixed else 0) | (BD_RUN_REF_ORDER if ref_order else 0)))
        return dict(lz_fw=lf[:Lf.value], lz_bk=lb[:Lb.value], ipiv_fw=ipf, ipiv_bk=ipb, NDEN=npv + 1,
                    n_piv_fw=int(ipf[0]) if Lf.value else 0, n_piv_bk=int(ipb[0]) if Lb.value else 0,
                    pivots=piv, nitr_fw=nf, nitr_bk=nb)

    def dyson_solve(self, ish, sig1b=None, sighf=None, efermi=float("nan")):
        D = self.D(ish)
        nfw, nbk = self.count_poles(ish)
        cap = D + nfw + nbk + 8
        qp, qh = np.zeros((cap, 2 + D)), np.zeros((cap, 2 + D))
        a, b = C.c_int(), C.c_int()
        kol = np.zeros(3)
        s1 = _d(sig1b) if sig1b is not None else None
        sh = _d(sighf) if sighf is not None else None
        self._chk(self.lib.bd_dyson_solve(self.h, ish, _pd(s1), _pd(sh), efermi, _pd(qp), cap, C.byref(a), _pd(qh), cap,
                                          C.byref(b), _pd(kol)))
        return dict(qp=qp[:a.value], qh=qh[:b.value], koltun=kol)

    def lanczos_vectors(self, ish, dir, L, N, fp32=False):
        out = np.zeros((max(L, 1), max(N, 1)))
        self._chk(self.lib.bd_lanczos_vectors(self.h, ish, dir, 1 if fp32 else 0, _pd(out), out.size))
        return out[:L, :N]

    def dyson_rows(self, ish, nden, fw, bk, ipiv_fw=None, ipiv_bk=None, sig1b=None, sighf=None, efermi=float("nan")):
        """DysonMatrix on caller-supplied self-energy rows (plain if ipiv_* is None)."""
        D = self.D(ish)
        fw = _d(np.asarray(fw).reshape(-1, nden + D)); bk = _d(np.asarray(bk).reshape(-1, nden + D))
        n = D + len(fw) + len(bk)
        qp, qh = np.zeros((n, 2 + D)), np.zeros((n, 2 + D))
        a, b = C.c_int(), C.c_int()
        kol = np.zeros(3)
        ipf = _i(ipiv_fw) if ipiv_fw is not None else None
        ipb = _i(ipiv_bk) if ipiv_bk is not None else None
        s1 = _d(sig1b) if sig1b is not None else None
        sh = _d(sighf) if sighf is not None else None
        self._chk(self.lib.bd_dyson_rows(self.h, ish, nden, len(fw), _pd(fw) if len(fw) else None, _pi(ipf), len(bk),
                                         _pd(bk) if len(bk) else None, _pi(ipb), _pd(s1), _pd(sh), efermi,
                                         _pd(qp), n, C.byref(a), _pd(qh), n, C.byref(b), _pd(kol)))
        return dict(qp=qp[:a.value], qh=qh[:b.value], koltun=kol)

    # ---------------------------------------------------------------- all channels
    @staticmethod
    def _flags(lanczos=True, mixed=False, per_channel=False, ref_order=False, graph=False, fp64_couplings=False):
        flags = (BD_RUN_LANCZOS if lanczos else 0) | (BD_RUN_MIXED if mixed else 0) | (BD_RUN_PER_CHANNEL if per_channel else 0)
        flags |= BD_RUN_FP64_COUPLINGS if fp64_couplings else 0
        return flags | (BD_RUN_REF_ORDER if ref_order else 0) | (BD_RUN_GRAPH if graph else 0)

    def autotune(self, reps=3, **kw):
        """bd_autotune: the fastest Lanczos / Dyson cluster sizes for the batched step."""
        a, b = C.c_int(), C.c_int()
        self._chk(self.lib.bd_autotune(self.h, self._flags(**kw), reps, C.byref(a), C.byref(b)))
        return a.value, b.value

    def run_all(self, lanczos=True, mixed=False, per_channel=False, sync=True, ref_order=False, graph=False,
                fp64_couplings=False):
        """bd_run_all.  fp64_couplings: the mixed form on a dressed propagator builds its
        couplings with the FP64 kernel instead of the tensor cores."""
        flags = self._flags(lanczos, mixed, per_channel, ref_order, graph, fp64_couplings)
        self._chk(self.lib.bd_run_all(self.h, flags))
        if sync:
            self.sync()

    def sync(self):
        self._chk(self.lib.bd_sync(self.h))

    def timings(self):
        t = np.zeros(5)
        self._chk(self.lib.bd_last_timings(self.h, _pd(t)))
        return dict(sigma2=t[0], sort=t[1], lanczos=t[2], dyson=t[3], total=t[4])

    def dressed_on_device(self):
        """Whether the last dressed_propagator stayed on the device (no re-planning)."""
        return bool(self.lib.bd_dressed_on_device(self.h))

    def tensor_couplings(self):
        """Whether the last batched run_all built the couplings on the tensor cores."""
        return bool(self.lib.bd_tensor_couplings(self.h))

    def two_pass_steps(self):
        return int(self.lib.bd_diag_two_pass(self.h))

    def lanczos_kernel_ms(self):
        return float(self.lib.bd_lanczos_kernel_ms(self.h))

    def launch_count(self):
        return int(self.lib.bd_launch_count(self.h))

    def koltun_all(self):
        k = np.zeros(3 * self.prob.ms.nsubsh)
        self._chk(self.lib.bd_result_koltun_all(self.h, _pd(k)))
        return k.reshape(-1, 3)

    def results_all(self):
        """Every channel's result (as result()) from one device copy."""
        ms = self.prob.ms
        n = [sum(self.result_counts(i)) for i in range(ms.nsubsh)]
        tot = sum(n[i] * (2 + int(ms.no[i])) for i in range(ms.nsubsh))
        sol = np.zeros(max(tot, 1)); cnt = np.zeros(2 * ms.nsubsh, np.int32); kol = np.zeros(3 * ms.nsubsh)
        self._chk(self.lib.bd_result_fetch_all(self.h, _pd(sol), len(sol), _pi(cnt), _pd(kol)))
        out, o = [], 0
        for i in range(ms.nsubsh):
            NS = 2 + int(ms.no[i]); a, b = int(cnt[2 * i]), int(cnt[2 * i + 1])
            rows = sol[o:o + (a + b) * NS].reshape(-1, NS); o += (a + b) * NS
            out.append(dict(qp=rows[:a], qh=rows[a:a + b], koltun=kol[3 * i:3 * i + 3]))
        return out

    def result_counts(self, ish):
        a, b = C.c_int(), C.c_int()
        self._chk(self.lib.bd_result_counts(self.h, ish, C.byref(a), C.byref(b)))
        return a.value, b.value

    def result(self, ish):
        a, b = C.c_int(), C.c_int()
        self._chk(self.lib.bd_result_counts(self.h, ish, C.byref(a), C.byref(b)))
        D = self.D(ish)
        qp, qh, kol = np.zeros((max(a.value, 1), 2 + D)), np.zeros((max(b.value, 1), 2 + D)), np.zeros(3)
        self._chk(self.lib.bd_result_fetch(self.h, ish, _pd(qp), max(a.value, 1), _pd(qh), max(b.value, 1), _pd(kol)))
        return dict(qp=qp[:a.value], qh=qh[:b.value], koltun=kol)


class Files:
    """A problem read from the reference's own files, on the host (bd_files_*): model space,
    propagator, Lanczos pivots and interaction, and the reference's writers.  No GPU is
    needed until it is uploaded with Context.upload_files."""

    def __init__(self, modspace_path: str):
        self.lib = lib()
        h = C.c_void_p()
        rc = self.lib.bd_files_open(C.byref(h), os.fsencode(modspace_path))
        self.h = h
        self._chk(rc)

    def _chk(self, rc):
        if rc != BD_OK:
            raise BDError(rc, self.lib.bd_files_error(self.h).decode() if self.h else "bd_files_open")
        return rc

    def close(self):
        if self.h:
            self.lib.bd_files_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def read_propagator(self, path):
        self._chk(self.lib.bd_files_read_propagator(self.h, os.fsencode(path)))
        return self

    def read_pivots(self, path):
        self._chk(self.lib.bd_files_read_pivots(self.h, os.fsencode(path)))
        return self

    def read_interaction(self, path, threads: int = 0):
        self._chk(self.lib.bd_files_read_interaction(self.h, os.fsencode(path), threads))
        return self

    def modspace(self):
        m = _ModSpace()
        on = _ip()
        names = C.POINTER(C.c_char_p)()
        self._chk(self.lib.bd_files_modspace(self.h, C.byref(m), C.byref(on), C.byref(names)))
        ns, no_ = m.nsubsh, m.norb
        arr = lambda p, n: np.ctypeslib.as_array(p, shape=(n,)).copy()
        return dict(nsubsh=ns, norb=no_, l=arr(m.l, ns), j2=arr(m.j2, ns), ip=arr(m.ip, ns), ch=arr(m.ch, ns),
                    no=arr(m.no, ns), orb_sh=arr(m.orb_sh, no_), orb_xe=arr(m.orb_xe, no_), orb_n=arr(on, no_),
                    names=[names[i].decode() for i in range(ns)])

    def propagator(self):
        p = _Propagator()
        zp, zh = _dp(), _dp()
        self._chk(self.lib.bd_files_propagator(self.h, C.byref(p), C.byref(zp), C.byref(zh)))
        ns = self.modspace()["nsubsh"]
        npa = np.ctypeslib.as_array(p.np, shape=(ns,)).copy(); nha = np.ctypeslib.as_array(p.nh, shape=(ns,)).copy()
        a, b = int(npa.sum()), int(nha.sum())
        g = lambda q, n: np.ctypeslib.as_array(q, shape=(n,)).copy() if n else np.zeros(0)
        return dict(nspb=p.nspb, np=npa, nh=nha, ep=g(p.ep, a), eh=g(p.eh, b), zp=g(zp, a), zh=g(zh, b),
                    fqp=g(p.fqp, a * p.nspb).reshape(a, p.nspb), fqh=g(p.fqh, b * p.nspb).reshape(b, p.nspb))

    def pivots(self):
        pv = _Pivots()
        self._chk(self.lib.bd_files_pivots(self.h, C.byref(pv)))
        ms = self.modspace()
        npvt = np.ctypeslib.as_array(pv.npvt, shape=(ms["nsubsh"],)).copy()
        tot = int(npvt.sum()); vt = int((npvt * ms["no"]).sum())
        g = lambda q, n, t: np.ctypeslib.as_array(q, shape=(n,)).copy() if n else np.zeros(0, t)
        return dict(npvt=npvt, n_fw=g(pv.n_itr_fw, tot, np.int32), n_bk=g(pv.n_itr_bk, tot, np.int32),
                    vec=g(pv.vec, vt, np.float64))

    def lines(self):
        a, b, c = C.c_longlong(), C.c_longlong(), C.c_longlong()
        self._chk(self.lib.bd_files_interaction_lines(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return dict(kept=a.value, outside=b.value, pauli=c.value)

    @staticmethod
    def _prop_struct(prop):
        arrs = dict(np=_i(prop["np"]), nh=_i(prop["nh"]), ep=_d(prop["ep"] if len(prop["ep"]) else np.zeros(1)),
                    eh=_d(prop["eh"] if len(prop["eh"]) else np.zeros(1)),
                    fqp=_d(np.asarray(prop["fqp"]).reshape(-1) if len(prop["ep"]) else np.zeros(prop["nspb"])),
                    fqh=_d(np.asarray(prop["fqh"]).reshape(-1) if len(prop["eh"]) else np.zeros(prop["nspb"])))
        st = _Propagator(prop["nspb"], _pi(arrs["np"]), _pi(arrs["nh"]), _pd(arrs["ep"]), _pd(arrs["eh"]),
                         _pd(arrs["fqp"]), _pd(arrs["fqh"]))
        return st, arrs

    def write_propagator(self, path, prop, zp=None, zh=None):
        st, keep = self._prop_struct(prop)
        zpa = _d(zp) if zp is not None else None
        zha = _d(zh) if zh is not None else None
        self._chk(self.lib.bd_files_write_propagator(self.h, os.fsencode(path), C.byref(st), _pd(zpa), _pd(zha)))

    def write_pivots(self, path, prop, n_fw, n_bk, z_cut=60.0, zp=None, zh=None):
        st, keep = self._prop_struct(prop)
        zpa = _d(zp) if zp is not None else None
        zha = _d(zh) if zh is not None else None
        self._chk(self.lib.bd_files_write_pivots(self.h, os.fsencode(path), C.byref(st), _pd(zpa), _pd(zha), n_fw,
                                                 n_bk, z_cut))

    def selfenergy_name(self, folder, ish, label="SelfEn"):
        buf = C.create_string_buffer(1024)
        self._chk(self.lib.bd_files_selfenergy_name(self.h, os.fsencode(folder), label.encode(), ish, buf, len(buf)))
        return buf.value.decode()

    def save_selfenergy(self, path, ish, nden, fw, bk, ipiv_fw=None, ipiv_bk=None, fwbk=0):
        fw = _d(np.asarray(fw).reshape(-1)); bk = _d(np.asarray(bk).reshape(-1))
        D = int(self.modspace()["no"][ish]); nt = nden + D
        ipf = _i(ipiv_fw) if ipiv_fw is not None else None
        ipb = _i(ipiv_bk) if ipiv_bk is not None else None
        self._chk(self.lib.bd_files_save_selfenergy(self.h, os.fsencode(path), ish, nden, len(fw) // nt, _pd(fw),
                                                    _pi(ipf), len(bk) // nt, _pd(bk), _pi(ipb), fwbk))

    def load_selfenergy(self, path, ish):
        nden, nf, nb = C.c_int(), C.c_int(), C.c_int()
        self._chk(self.lib.bd_files_load_selfenergy(self.h, os.fsencode(path), ish, C.byref(nden), C.byref(nf), None, 0,
                                                    None, C.byref(nb), None, 0, None))
        D = int(self.modspace()["no"][ish]); nt = nden.value + D
        fw, bk = np.zeros((max(nf.value, 1), nt)), np.zeros((max(nb.value, 1), nt))
        ipf, ipb = np.zeros(nt, np.int32), np.zeros(nt, np.int32)
        self._chk(self.lib.bd_files_load_selfenergy(self.h, os.fsencode(path), ish, C.byref(nden), C.byref(nf), _pd(fw),
                                                    len(fw), _pi(ipf), C.byref(nb), _pd(bk), len(bk), _pi(ipb)))
        return dict(nden=nden.value, fw=fw[:nf.value], bk=bk[:nb.value], ipiv_fw=ipf, ipiv_bk=ipb)


def write_interaction_bin(path, iabJ, icdJ, V, n_alloc: int = 0):
    """VppInt_t::write_bin of one interaction list."""
    a, b, v = _i(iabJ), _i(icdJ), _d(V)
    st = _Interaction(len(v), _pi(a), _pi(b), _pd(v))
    rc = lib().bd_write_interaction_bin(os.fsencode(path), C.byref(st), n_alloc)
    if rc != BD_OK:
        raise BDError(rc, f"writing {path}")


def koltun_totals(kol_per_channel, ch):
    """Koltun totals as Run_itrs forms them (source/BcDor-Main.cpp:387-417): per charge
    U1 = sum x1, E = sum (x1 + x2)/2, A = sum x3."""
    out = {}
    k = np.asarray(kol_per_channel)
    for c in (0, 1):
        m = np.asarray(ch) == c
        out[c] = dict(U1=float(k[m, 0].sum()), E=float(((k[m, 0] + k[m, 1]) / 2.0).sum()), A=float(k[m, 2].sum()))
    out["E_tot"] = out[0]["E"] + out[1]["E"]
    out["A_tot"] = out[0]["A"] + out[1]["A"]
    return out


# ------------------------------------------------------------------------------------------
# mirror of the reference's per-channel interface
# ------------------------------------------------------------------------------------------
class WideSelfEnergy:
    """Per-channel self-energy with the reference's method names (Wide_self_energy_t,
    source/BcDor-SlfEn_classes.hh:16-111).  State lives on the device."""

    def __init__(self, ctx: Context, ish: int):
        self.ctx, self.I_SH = ctx, ish
        self.NTOT_ORB = ctx.D(ish)
        self.Sig_dyn_fw = self.Sig_dyn_bk = None
        self.N_PLS_fw = self.N_PLS_bk = 0
        self.lanczos = None

    def Count_2p1h_2h1p_poles(self):
        return self.ctx.count_poles(self.I_SH)

    def Build_ExtendedHartreeFock(self):
        self.Sig_HF = self.ctx.ehf(self.I_SH)
        return self.Sig_HF

    def Build_Dynamic_SlfEn_2ndOrder(self):
        self.Sig_dyn_fw, self.Sig_dyn_bk = self.ctx.sigma2_build(self.I_SH)
        self.N_PLS_fw, self.N_PLS_bk = len(self.Sig_dyn_fw), len(self.Sig_dyn_bk)
        return self.N_PLS_fw, self.N_PLS_bk

    def Reduce_SelfEn_Lncz(self, pivots, n_itr_fw, n_itr_bk, mixed=False):
        self.lanczos = self.ctx.lanczos_reduce(self.I_SH, pivots, n_itr_fw, n_itr_bk, mixed=mixed)
        return self.lanczos


def dyson_matrix(sfv: WideSelfEnergy, sig1b, sighf=None, efermi=float("nan")):
    """DysonMatrix: returns dict(qp=rows, qh=rows, koltun=[x1, x2, x3])."""
    return sfv.ctx.dyson_solve(sfv.I_SH, sig1b, sighf, efermi)


def lanczos_chain_noalloc(d_E: int, d_M: int, N: int, D: int, pivots, n_itr, d_rows: int, cap_rows: int,
                          mixed: bool = False, stream: int = 0):
    """bd_lanczos_chain_noalloc: Lanczos rows of one pole set into caller-owned device
    memory, with no device allocation by the library.  d_E [N], d_M [D][N] and
    d_rows [cap_rows][n_pvt + 1 + D] are device addresses of float64 buffers on the
    current device; pivots and n_itr are updated in place as bd_lanczos_reduce does.
    Returns (L, ipiv, pivots, n_itr)."""
    L_ = lib()
    f = L_.bd_lanczos_chain_noalloc
    vp = C.c_void_p
    f.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, _dp, _ip, vp, C.c_int, _ip, _ip, C.c_int, vp, C.c_char_p,
                  C.c_int]
    piv = _d(np.array(pivots, np.float64).reshape(-1, D)).copy()
    nit = _i(n_itr).copy()
    ipiv = np.zeros(len(piv) + 1 + D, np.int32)
    Lout = C.c_int()
    err = C.create_string_buffer(512)
    rc = f(d_E, d_M, N, D, len(piv), _pd(piv), _pi(nit), d_rows, cap_rows, C.byref(Lout), _pi(ipiv),
           BD_RUN_MIXED if mixed else 0, stream, err, len(err))
    if rc != BD_OK:
        raise BDError(rc, err.value.decode(errors="replace"))
    return Lout.value, ipiv, piv, nit
