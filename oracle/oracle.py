"""ctypes wrapper of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker.  It mirrors the engine's C ABI with an
``orc_`` prefix so the same inputs can be pushed through both.  It also holds
the exact-diagonalisation helper (scipy eigsh on the oracle's sparse
Hamiltonian), which plays the role of NECI's Davidson (davidson_neci.F90:65).
"""
from __future__ import annotations

import ctypes as C
import itertools
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_P = C.c_void_p


def build() -> Path:
    subprocess.run(["sh", str(HERE / "build_oracle.sh")], check=True)
    return LIB


def _load():
    if not LIB.exists() or LIB.stat().st_mtime < (HERE / "neci_oracle.cpp").stat().st_mtime:
        build()
    lib = C.CDLL(str(LIB))
    import neci_stable_gb300.capi as capi  # struct layouts of include/neci_gpu.h
    sig = {
        "orc_init": [C.POINTER(_P), C.POINTER(capi.System)],
        "orc_free": [_P],
        "orc_set_random_hash": [_P, _P],
        "orc_set_tmat": [_P, _P],
        "orc_set_umat": [_P, _P, C.c_int64],
        "orc_set_lattice": [_P, _P, C.c_int32],
        "orc_set_reference": [_P, _P, C.c_double],
        "orc_init_pchb": [_P],
        "orc_set_excit_biases": [_P, C.c_double, C.c_double],
        "orc_set_tau_search": [_P, C.c_int32],
        "orc_set_core_segment": [_P, C.c_int32],
        "orc_set_rdm_sampling": [_P, C.c_int32],
        "orc_get_rdm": [_P, _P, C.c_int64, C.c_int32],
        "orc_get_tau_stats": [_P, C.POINTER(capi.TauStats), C.c_int32],
        "orc_upload_walkers": [_P, _P, C.c_int64, _P, _P],
        "orc_download_walkers": [_P, _P, _P, _P, C.c_int64, _P],
        "orc_iterate": [_P, C.POINTER(capi.IterParams), C.POINTER(capi.IterStats)],
        "orc_annihilate": [_P, C.POINTER(capi.IterParams), _P, C.c_int64, C.POINTER(capi.IterStats)],
        "orc_find_walker_hash": [_P, _P, C.c_int64, C.c_int64, _P],
        "orc_compress_spawns": [_P, C.POINTER(capi.IterParams), _P, C.c_int64, _P, _P, _P],
        "orc_excit_level": [_P, _P, _P, C.c_int64, _P],
        "orc_helement": [_P, _P, _P, C.c_int64, _P],
        "orc_gen_excit": [_P, _P, C.c_int64, C.c_uint64, C.c_int64, _P, _P, _P],
        "orc_calc_pgen": [_P, _P, _P, _P],
        "orc_cum_list_rs_hubbard": [_P, _P, C.c_int32, _P, C.c_int32, _P, _P],
        "orc_calc_pgen_rs_hubbard": [_P, _P, C.c_int32, C.c_int32, C.c_int32, _P],
        "orc_init_alias": [_P, C.c_int64, _P, _P],
        "orc_set_core_space": [_P, _P, C.c_int64],
        "orc_core_nnz": [_P, _P],
        "orc_hamiltonian": [_P, _P, C.c_int64, _P, _P, _P],
        "orc_stream": [C.c_uint64, C.c_int64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int64, _P],
        "orc_philox_block": [_P, _P, _P],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = C.c_int32
    lib.orc_hamiltonian_nnz.argtypes = [_P, _P, C.c_int64]
    lib.orc_hamiltonian_nnz.restype = C.c_int64
    lib.orc_det_key.argtypes = [_P, C.c_int32, C.c_uint64]
    lib.orc_det_key.restype = C.c_uint64
    lib.orc_last_error.restype = C.c_char_p
    return lib


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = _load()
    return _lib


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(C.c_void_p)


def _ok(rc):
    if rc != 0:
        raise RuntimeError(f"oracle error {rc}: {lib().orc_last_error().decode()}")


class Oracle:
    """CPU restatement of the engine for one system (same inputs as Engine)."""

    def __init__(self, spec, max_walkers: int, max_spawned: int, hii: float | None = None, pchb: bool = True):
        from neci_stable_gb300 import capi
        from neci_stable_gb300.systems import encode_det
        self.spec = spec
        self.W = spec.W
        self.L = spec.lenof_sign
        self.R = self.W + self.L + 1
        self.csys = spec.c_system(max_walkers, max_spawned)
        h = C.c_void_p()
        _ok(lib().orc_init(C.byref(h), C.byref(self.csys)))
        self.h = h
        _ok(lib().orc_set_random_hash(h, _ptr(np.ascontiguousarray(spec.random_hash2, dtype=np.int32))))
        _ok(lib().orc_set_tmat(h, _ptr(np.ascontiguousarray(spec.tmat, dtype=np.float64))))
        if spec.umat is not None:
            u = np.ascontiguousarray(spec.umat, dtype=np.float64)
            _ok(lib().orc_set_umat(h, _ptr(u), u.size))
        if spec.neighbours is not None:
            nb = np.ascontiguousarray(spec.neighbours, dtype=np.int32)
            _ok(lib().orc_set_lattice(h, _ptr(nb), nb.shape[0]))
        self.ilut_ref = encode_det(spec.reference, spec.nifd)
        _ok(lib().orc_set_reference(h, _ptr(self.ilut_ref), 0.0))
        self.hii = float(self.helement(self.ilut_ref[None], self.ilut_ref[None])[0]) if hii is None else hii
        _ok(lib().orc_set_reference(h, _ptr(self.ilut_ref), self.hii))
        if spec.umat is not None and pchb and spec.generator == capi.EXGEN_PCHB:
            _ok(lib().orc_init_pchb(h))

    def __del__(self):
        try:
            lib().orc_free(self.h)
        except Exception:
            pass

    def upload(self, rows, diag_h=None, offdiag_h=None):
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        _ok(lib().orc_upload_walkers(self.h, _ptr(rows), rows.shape[0],
                                     _ptr(None if diag_h is None else np.ascontiguousarray(diag_h, float)),
                                     _ptr(None if offdiag_h is None else np.ascontiguousarray(offdiag_h, float))))

    def download(self, max_rows: int | None = None):
        max_rows = max_rows or int(self.csys.max_walkers)
        rows = np.zeros((max_rows, self.R), dtype=np.int64)
        dh = np.zeros(max_rows)
        odh = np.zeros(max_rows)
        n = C.c_int64()
        _ok(lib().orc_download_walkers(self.h, _ptr(rows), _ptr(dh), _ptr(odh), max_rows, C.byref(n)))
        return rows[: n.value], dh[: n.value], odh[: n.value]

    def set_tau_search(self, on: bool):
        _ok(lib().orc_set_tau_search(self.h, 1 if on else 0))

    def tau_stats(self, reset: bool = False):
        import neci_stable_gb300.capi as capi
        t = capi.TauStats()
        _ok(lib().orc_get_tau_stats(self.h, C.byref(t), 1 if reset else 0))
        return t

    def set_excit_biases(self, p_singles: float, p_parallel: float):
        _ok(lib().orc_set_excit_biases(self.h, p_singles, p_parallel))

    def set_rdm_sampling(self, on: bool):
        _ok(lib().orc_set_rdm_sampling(self.h, 1 if on else 0))

    def rdm2(self, reset: bool = False):
        nb = self.spec.nbasis
        npair = nb * (nb - 1) // 2
        out = np.zeros((npair, npair))
        _ok(lib().orc_get_rdm(self.h, _ptr(out), out.size, 1 if reset else 0))
        return out

    def iterate(self, params):
        import neci_stable_gb300.capi as capi
        st = capi.IterStats()
        rc = lib().orc_iterate(self.h, C.byref(params), C.byref(st))
        return st, rc

    def annihilate(self, params, spawned):
        import neci_stable_gb300.capi as capi
        sp = np.ascontiguousarray(spawned, dtype=np.int64)
        st = capi.IterStats()
        rc = lib().orc_annihilate(self.h, C.byref(params), _ptr(sp), sp.shape[0], C.byref(st))
        return st, rc

    def compress_spawns(self, params, spawned):
        sp = np.ascontiguousarray(spawned, dtype=np.int64)
        out = np.zeros((max(sp.shape[0], 1), self.R), dtype=np.int64)
        n = C.c_int64()
        nann = np.zeros(2)
        _ok(lib().orc_compress_spawns(self.h, C.byref(params), _ptr(sp), sp.shape[0], _ptr(out), C.byref(n), _ptr(nann)))
        return out[: n.value], nann[: self.L]

    def find_walker_hash(self, dets, table_len):
        d = np.ascontiguousarray(dets, dtype=np.int64)
        out = np.zeros(d.shape[0], dtype=np.int64)
        _ok(lib().orc_find_walker_hash(self.h, _ptr(d), d.shape[0], table_len, _ptr(out)))
        return out

    def excit_level(self, a, b):
        a = np.ascontiguousarray(a, dtype=np.int64)
        b = np.ascontiguousarray(b, dtype=np.int64)
        out = np.zeros(a.shape[0], dtype=np.int32)
        _ok(lib().orc_excit_level(self.h, _ptr(a), _ptr(b), a.shape[0], _ptr(out)))
        return out

    def helement(self, a, b):
        a = np.ascontiguousarray(a, dtype=np.int64)
        b = np.ascontiguousarray(b, dtype=np.int64)
        out = np.zeros(a.shape[0])
        _ok(lib().orc_helement(self.h, _ptr(a), _ptr(b), a.shape[0], _ptr(out)))
        return out

    def gen_excit(self, det, n, seed, it):
        d = np.ascontiguousarray(det, dtype=np.int64)
        child = np.zeros((n, self.W), dtype=np.int64)
        pgen = np.zeros(n)
        hel = np.zeros(n)
        _ok(lib().orc_gen_excit(self.h, _ptr(d), n, seed, it, _ptr(child), _ptr(pgen), _ptr(hel)))
        return child, pgen, hel

    def calc_pgen(self, det, child):
        out = C.c_double()
        _ok(lib().orc_calc_pgen(self.h, _ptr(np.ascontiguousarray(det, dtype=np.int64)),
                                _ptr(np.ascontiguousarray(child, dtype=np.int64)), C.byref(out)))
        return out.value

    def set_core_segment(self, per_lane: int):
        """Elements per partial sum of a core-row segment (the engine's
        NECI_OPT_CORE_SEGMENT); applies to the next set_core_space."""
        _ok(lib().orc_set_core_segment(self.h, per_lane))

    def set_core_space(self, core):
        c = np.ascontiguousarray(core, dtype=np.int64)
        _ok(lib().orc_set_core_space(self.h, _ptr(c), c.shape[0]))

    def core_nnz(self):
        n = C.c_int64()
        _ok(lib().orc_core_nnz(self.h, C.byref(n)))
        return n.value

    def hamiltonian(self, dets):
        import scipy.sparse as sp
        d = np.ascontiguousarray(dets, dtype=np.int64)
        n = d.shape[0]
        nnz = lib().orc_hamiltonian_nnz(self.h, _ptr(d), n)
        rp = np.zeros(n + 1, dtype=np.int64)
        cols = np.zeros(nnz, dtype=np.int64)
        vals = np.zeros(nnz)
        _ok(lib().orc_hamiltonian(self.h, _ptr(d), n, _ptr(rp), _ptr(cols), _ptr(vals)))
        return sp.csr_matrix((vals, cols, rp), shape=(n, n))


def all_determinants(nbasis: int, nalpha: int, nbeta: int, nifd: int) -> np.ndarray:
    """Every determinant with the given alpha/beta counts (Sz sector)."""
    from neci_stable_gb300.systems import encode_det
    n = nbasis // 2
    out = []
    for a in itertools.combinations(range(1, n + 1), nalpha):
        for b in itertools.combinations(range(1, n + 1), nbeta):
            out.append(encode_det(sorted([2 * p for p in a] + [2 * p - 1 for p in b]), nifd))
    return np.array(out, dtype=np.int64)


def exact_ground_state(oracle: Oracle, nalpha: int, nbeta: int, reference_sector: bool = True, k: int = 6):
    """(E, dets, vector) by sparse Lanczos (scipy eigsh).

    With reference_sector (the default) E is the lowest eigenvalue whose
    eigenvector overlaps the reference determinant: the state a projection
    from the reference converges to (FCIQMC's E_proj and NECI's Davidson
    started from the reference).  The Sz sector may hold lower states of
    other total spin that the reference cannot reach."""
    from scipy.sparse.linalg import eigsh
    dets = all_determinants(oracle.spec.nbasis, nalpha, nbeta, oracle.spec.nifd)
    H = oracle.hamiltonian(dets)
    H = 0.5 * (H + H.T)
    k = min(k, dets.shape[0] - 2)
    vals, vecs = eigsh(H, k=max(k, 1), which="SA", tol=1e-12)
    order = np.argsort(vals)
    vals, vecs = vals[order], vecs[:, order]
    if not reference_sector:
        return float(vals[0]), dets, vecs[:, 0]
    ref = np.all(dets == oracle.ilut_ref[None, :], axis=1)
    i0 = int(np.argmax(ref))
    for j in range(vals.size):
        if abs(vecs[i0, j]) > 1e-6:
            return float(vals[j]), dets, vecs[:, j]
    raise RuntimeError("no low-lying state overlaps the reference")


def stream(dkey: int, it: int, purpose: int, run: int, attempt: int, n: int) -> np.ndarray:
    out = np.zeros(n)
    _ok(lib().orc_stream(dkey, it, purpose, run, attempt, n, _ptr(out)))
    return out


def det_key(det, seed):
    d = np.ascontiguousarray(det, dtype=np.int64)
    return lib().orc_det_key(_ptr(d), d.size, seed)


def init_alias(w):
    w = np.ascontiguousarray(w, dtype=np.float64)
    bias = np.zeros(w.size)
    alias = np.zeros(w.size, dtype=np.int32)
    _ok(lib().orc_init_alias(_ptr(w), w.size, _ptr(bias), _ptr(alias)))
    return bias, alias


def cum_list_rs_hubbard(oracle, ilut, src, neigh):
    neigh = np.ascontiguousarray(neigh, dtype=np.int32)
    cum = np.zeros(neigh.size)
    s = C.c_double()
    _ok(lib().orc_cum_list_rs_hubbard(oracle.h, _ptr(np.ascontiguousarray(ilut, dtype=np.int64)), src, _ptr(neigh),
                                      neigh.size, _ptr(cum), C.byref(s)))
    return cum, s.value


def calc_pgen_rs_hubbard(oracle, ilut, src, tgt, ic):
    out = C.c_double()
    _ok(lib().orc_calc_pgen_rs_hubbard(oracle.h, _ptr(np.ascontiguousarray(ilut, dtype=np.int64)), src, tgt, ic,
                                       C.byref(out)))
    return out.value
