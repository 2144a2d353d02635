"""Python view of one engine context: the calls NECI's Fortran shim makes.

``Engine`` owns a ``neci_gpu_ctx``; its methods map one-to-one onto the C ABI
(include/neci_gpu.h).  ``Engine.perform_fcimc_cyc_par`` is the drop-in for
``PerformFCIMCycPar(iter_data, err)`` (FciMCPar.F90:1177): it raises on a
non-zero status exactly where NECI would call stop_all.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import check, ptr
from .systems import SystemSpec, encode_det, make_rows


class Engine:
    def __init__(self, spec: SystemSpec, max_walkers: int, max_spawned: int, device: int = 0,
                 hash_frac: float = 0.7, pchb: bool = True):
        self.lib = capi.load()
        self.spec = spec
        self.W = spec.W
        self.L = spec.lenof_sign
        self.R = self.W + self.L + 1
        self.csys = spec.c_system(max_walkers, max_spawned, hash_frac)
        h = C.c_void_p()
        check(self.lib.neci_gpu_init(C.byref(h), C.byref(self.csys), device))
        self.ctx = h
        check(self.lib.neci_gpu_set_random_hash(self.ctx, ptr(np.ascontiguousarray(spec.random_hash2, dtype=np.int32))))
        check(self.lib.neci_gpu_set_tmat(self.ctx, ptr(np.ascontiguousarray(spec.tmat, dtype=np.float64))))
        if spec.umat is not None:
            u = np.ascontiguousarray(spec.umat, dtype=np.float64)
            check(self.lib.neci_gpu_set_umat(self.ctx, ptr(u), u.size))
        if spec.neighbours is not None:
            nb = np.ascontiguousarray(spec.neighbours, dtype=np.int32)
            check(self.lib.neci_gpu_set_lattice(self.ctx, ptr(nb), nb.shape[0]))
        self.ilut_ref = encode_det(spec.reference, spec.nifd)
        # Hii = <D0|H|D0> from the device Slater-Condon / Hubbard kernels
        check(self.lib.neci_gpu_set_reference(self.ctx, ptr(self.ilut_ref), 0.0))
        self.hii = float(self.helement(self.ilut_ref[None], self.ilut_ref[None])[0])
        check(self.lib.neci_gpu_set_reference(self.ctx, ptr(self.ilut_ref), self.hii))
        if spec.kind == capi.SYS_MOLECULAR and spec.generator == capi.EXGEN_PCHB and pchb:
            check(self.lib.neci_gpu_init_pchb(self.ctx))

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.neci_gpu_free(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- walkers
    def upload(self, rows: np.ndarray, diag_h=None, offdiag_h=None):
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        check(self.lib.neci_gpu_upload_walkers(self.ctx, ptr(rows), rows.shape[0],
                                               ptr(None if diag_h is None else np.ascontiguousarray(diag_h, float)),
                                               ptr(None if offdiag_h is None else np.ascontiguousarray(offdiag_h, float))))

    def start_from_reference(self, initial_part: float = 1.0, initiator: bool = True):
        """InitFCIMCCalcPar's single-determinant start (InitialPart walkers on D0,
        initiator flag set, fcimc_initialisation.fpp:2753)."""
        flags = 0
        if initiator:
            for k in range(self.L):
                flags |= 1 << capi.FLAG_INITIATOR[k]
        rows = make_rows(self.ilut_ref[None], np.full((1, self.L), float(initial_part)), np.array([flags]))
        self.upload(rows)

    def download(self, max_rows: int | None = None):
        max_rows = max_rows or int(self.csys.max_walkers)
        rows = np.zeros((max_rows, self.R), dtype=np.int64)
        dh = np.zeros(max_rows)
        odh = np.zeros(max_rows)
        n = C.c_int64()
        check(self.lib.neci_gpu_download_walkers(self.ctx, ptr(rows), ptr(dh), ptr(odh), max_rows, C.byref(n)))
        return rows[: n.value], dh[: n.value], odh[: n.value]

    # ----------------------------------------------------------------- steps
    def perform_fcimc_cyc_par(self, params: capi.IterParams) -> capi.IterStats:
        st = capi.IterStats()
        check(self.lib.neci_gpu_iterate(self.ctx, C.byref(params), C.byref(st)))
        return st

    def iterate_n(self, params: capi.IterParams, n: int):
        arr = (capi.IterStats * n)()
        check(self.lib.neci_gpu_iterate_n(self.ctx, C.byref(params), n, C.cast(arr, C.c_void_p)))
        return list(arr)

    def iterate_timed(self, params: capi.IterParams, n: int):
        """n steps back to back; returns (stats, device milliseconds by CUDA events)."""
        arr = (capi.IterStats * n)()
        ms = C.c_double()
        check(self.lib.neci_gpu_iterate_timed(self.ctx, C.byref(params), n, C.cast(arr, C.c_void_p), C.byref(ms)))
        return list(arr), ms.value

    def annihilate(self, params: capi.IterParams, spawned: np.ndarray) -> capi.IterStats:
        sp = np.ascontiguousarray(spawned, dtype=np.int64)
        st = capi.IterStats()
        check(self.lib.neci_gpu_annihilate(self.ctx, C.byref(params), ptr(sp), sp.shape[0], C.byref(st)))
        return st

    def compress_spawns(self, spawned: np.ndarray):
        sp = np.ascontiguousarray(spawned, dtype=np.int64)
        out = np.zeros((max(sp.shape[0], 1), self.R), dtype=np.int64)
        n = C.c_int64()
        nann = np.zeros(2)
        check(self.lib.neci_gpu_compress_spawns(self.ctx, ptr(sp), sp.shape[0], ptr(out), C.byref(n), ptr(nann)))
        return out[: n.value], nann[: self.L]

    def set_core_space(self, core_dets: np.ndarray, precision: int = capi.PREC_FP64):
        cd = np.ascontiguousarray(core_dets, dtype=np.int64)
        check(self.lib.neci_gpu_set_core_space(self.ctx, ptr(cd), cd.shape[0], precision))

    def select_core(self, n_core: int, precision: int = capi.PREC_FP64) -> np.ndarray:
        """Selects the n_core most populated determinants on the device
        (neci_gpu_select_core) and makes them the core space; returns them."""
        out = np.zeros((n_core, self.W), dtype=np.int64)
        n = C.c_int64()
        check(self.lib.neci_gpu_select_core(self.ctx, n_core, precision, ptr(out), C.byref(n)))
        return out[: n.value]

    def set_option(self, option: int, value: int):
        check(self.lib.neci_gpu_set_option(self.ctx, option, value))

    def autotune(self, params: capi.IterParams, steps_per_setting: int = 3):
        """neci_gpu_autotune: times the candidate settings on live steps and
        keeps the fastest.  Returns (stats of the steps run, the tuning kept);
        the caller advances params.iter by len(stats)."""
        cap = 16 * (steps_per_setting + 1)
        arr = (capi.IterStats * cap)()
        n = C.c_int32()
        t = capi.Tuning()
        check(self.lib.neci_gpu_autotune(self.ctx, C.byref(params), steps_per_setting, C.cast(arr, C.c_void_p),
                                         cap, C.byref(n), C.byref(t)))
        return list(arr[: n.value]), t

    def tuning(self) -> capi.Tuning:
        t = capi.Tuning()
        check(self.lib.neci_gpu_get_tuning(self.ctx, C.byref(t)))
        return t

    def set_tuning(self, t: capi.Tuning):
        check(self.lib.neci_gpu_set_tuning(self.ctx, C.byref(t)))

    def core_nnz(self) -> int:
        n = C.c_int64()
        check(self.lib.neci_gpu_core_nnz(self.ctx, C.byref(n)))
        return n.value

    # ------------------------------------------------------ batch primitives
    def find_walker_hash(self, dets: np.ndarray, table_len: int) -> np.ndarray:
        d = np.ascontiguousarray(dets, dtype=np.int64)
        out = np.zeros(d.shape[0], dtype=np.int64)
        check(self.lib.neci_gpu_find_walker_hash(self.ctx, ptr(d), d.shape[0], table_len, ptr(out)))
        return out

    def excit_level(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=np.int64)
        b = np.ascontiguousarray(b, dtype=np.int64)
        out = np.zeros(a.shape[0], dtype=np.int32)
        check(self.lib.neci_gpu_excit_level(self.ctx, ptr(a), ptr(b), a.shape[0], ptr(out)))
        return out

    def helement(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=np.int64)
        b = np.ascontiguousarray(b, dtype=np.int64)
        out = np.zeros(a.shape[0])
        check(self.lib.neci_gpu_helement(self.ctx, ptr(a), ptr(b), a.shape[0], ptr(out)))
        return out

    def gen_excit(self, det: np.ndarray, n: int, seed: int, it: int):
        d = np.ascontiguousarray(det, dtype=np.int64)
        child = np.zeros((n, self.W), dtype=np.int64)
        pgen = np.zeros(n)
        hel = np.zeros(n)
        check(self.lib.neci_gpu_gen_excit(self.ctx, ptr(d), n, seed, it, ptr(child), ptr(pgen), ptr(hel)))
        return child, pgen, hel

    # ------------------------------------------------------------ tau search
    def set_tau_search(self, on: bool):
        check(self.lib.neci_gpu_set_tau_search(self.ctx, 1 if on else 0))

    def tau_stats(self, reset: bool = False) -> capi.TauStats:
        t = capi.TauStats()
        check(self.lib.neci_gpu_get_tau_stats(self.ctx, C.byref(t), 1 if reset else 0))
        return t

    def set_excit_biases(self, p_singles: float, p_parallel: float):
        check(self.lib.neci_gpu_set_excit_biases(self.ctx, p_singles, p_parallel))

    # ---------------------------------------------------------------- 2-RDM
    def set_rdm_sampling(self, on: bool):
        check(self.lib.neci_gpu_set_rdm_sampling(self.ctx, 1 if on else 0))

    def rdm2(self, reset: bool = False) -> np.ndarray:
        """The accumulated spin-orbital 2-RDM, npair x npair (unnormalised)."""
        nb = self.spec.nbasis
        npair = nb * (nb - 1) // 2
        out = np.zeros((npair, npair))
        check(self.lib.neci_gpu_get_rdm(self.ctx, ptr(out), out.size, 1 if reset else 0))
        return out

    # ---------------------------------------------------------------- timing
    def set_profiling(self, on: bool):
        check(self.lib.neci_gpu_set_profiling(self.ctx, 1 if on else 0))

    def kernel_times(self) -> dict:
        n = self.lib.neci_gpu_num_kernels()
        ms = np.zeros(n)
        cnt = np.zeros(n, dtype=np.int64)
        check(self.lib.neci_gpu_kernel_times(self.ctx, ptr(ms), ptr(cnt), n))
        return {self.lib.neci_gpu_kernel_name(k).decode(): (float(ms[k]), int(cnt[k])) for k in range(n)}


def iterate_batch(engines, params, n_iter: int):
    """n_iter steps of several engines side by side on one device
    (neci_gpu_iterate_batch).  Returns (stats[engine][step], device ms)."""
    lib = capi.load()
    n = len(engines)
    ctxs = (C.c_void_p * n)(*[e.ctx for e in engines])
    par = (capi.IterParams * n)(*params)
    st = (capi.IterStats * (n * n_iter))()
    ms = C.c_double()
    check(lib.neci_gpu_iterate_batch(C.cast(ctxs, C.c_void_p), n, C.cast(par, C.c_void_p), n_iter,
                                     C.cast(st, C.c_void_p), C.byref(ms)))
    return [list(st[i * n_iter:(i + 1) * n_iter]) for i in range(n)], ms.value
