"""ctypes binding of the C ABI in include/neci_gpu.h.

This is the same binding a Fortran host makes with ``iso_c_binding``: POD
structs and plain pointers.  Loading fails loudly when the library has not
been built; there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "libneci_gpu.so"

OK = 0
ERR_SPAWN_FULL = 1
ERR_LIST_FULL = 2
ERR_HASH_FULL = 3
ERR_TIMEOUT = 4
ERR_UNSUPPORTED = 5
ERR_INVALID = 6
ERR_CUDA = 7
ERR_UNSTABLE = 8
ERR_OVERFLOW = 9

SYS_HUBBARD_REAL_SPACE = 0
SYS_MOLECULAR = 1
EXGEN_RS_HUBBARD = 0
EXGEN_UNIFORM = 1
EXGEN_PCHB = 2
PREC_FP64 = 0
PREC_MIXED = 1
OPT_FUSE_PROBE = 0
OPT_ANNIHILATION = 1
ANN_HASH = 0
ANN_SORT = 1
OPT_CORE_SEGMENT = 2
FLAG_INITIATOR = (13, 14)
FLAG_DETERMINISTIC = (19, 20)
SPAWN_FIXED_BITS = 32


class System(C.Structure):
    _fields_ = [
        ("nel", C.c_int32), ("nbasis", C.c_int32), ("nifd", C.c_int32), ("lenof_sign", C.c_int32),
        ("system", C.c_int32), ("excitgen", C.c_int32), ("max_neighbours", C.c_int32), ("reserved", C.c_int32),
        ("uhub", C.c_double), ("bhub", C.c_double), ("ecore", C.c_double), ("p_singles", C.c_double),
        ("p_parallel", C.c_double), ("max_walkers", C.c_int64), ("max_spawned", C.c_int64),
        ("n_walker_hashes", C.c_int64),
    ]


class IterParams(C.Structure):
    _fields_ = [
        ("tau", C.c_double), ("diag_sft", C.c_double * 2), ("initiator_walk_no", C.c_double),
        ("occupied_thresh", C.c_double), ("real_spawn_cutoff", C.c_double), ("av_mc_excits", C.c_double),
        ("t_trunc_initiator", C.c_int32), ("t_init_coherent_rule", C.c_int32), ("t_all_real_coeff", C.c_int32),
        ("t_real_spawn_cutoff", C.c_int32), ("t_core_inits", C.c_int32), ("precision", C.c_int32),
        ("seed", C.c_uint64), ("iter", C.c_int64),
    ]


class IterStats(C.Structure):
    _fields_ = [
        ("nborn", C.c_double * 2), ("ndied", C.c_double * 2), ("nannihil", C.c_double * 2),
        ("naborted", C.c_double * 2), ("nremoved", C.c_double * 2), ("tot_parts", C.c_double * 2),
        ("tot_parts_old", C.c_double * 2), ("noat_hf", C.c_double * 2), ("hf_cyc", C.c_double * 2),
        ("enum_cyc", C.c_double * 2), ("norm_psi_sq", C.c_double * 2),
        ("tot_walkers", C.c_int64), ("n_occupied", C.c_int64), ("holes_in_list", C.c_int64),
        ("n_attempts", C.c_int64), ("n_spawned", C.c_int64), ("n_unique", C.c_int64), ("n_new", C.c_int64),
        ("n_core", C.c_int64), ("err", C.c_int32), ("reserved", C.c_int32),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, typ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if isinstance(v, C.Array) else v
        return out


class TauStats(C.Structure):
    """neci_gpu_tau_stats: the conventional tau search's class maxima."""
    _fields_ = [
        ("gamma_sing", C.c_double), ("gamma_doub", C.c_double), ("gamma_par", C.c_double),
        ("gamma_opp", C.c_double), ("max_death_cpt", C.c_double),
        ("cnt_sing", C.c_int64), ("cnt_doub", C.c_int64), ("cnt_par", C.c_int64), ("cnt_opp", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class Tuning(C.Structure):
    """neci_gpu_tuning: launch shapes and the annihilation form of a context."""
    _fields_ = [
        ("annihilation", C.c_int32), ("spawn_blocks_per_sm", C.c_int32), ("table_shift", C.c_int32),
        ("sort_blocks_per_sm", C.c_int32), ("ns_per_update", C.c_double), ("reserved", C.c_int32 * 2),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


def default_params(**kw) -> IterParams:
    """NECI's defaults for an initiator run with real coefficients."""
    p = IterParams()
    p.tau = 0.01
    p.diag_sft[0] = p.diag_sft[1] = 0.0
    p.initiator_walk_no = 3.0
    p.occupied_thresh = 1.0
    p.real_spawn_cutoff = 0.95
    p.av_mc_excits = 1.0
    p.t_trunc_initiator = 1
    p.t_init_coherent_rule = 1
    p.t_all_real_coeff = 1
    p.t_real_spawn_cutoff = 1
    p.t_core_inits = 1
    p.precision = PREC_FP64
    p.seed = 12345
    p.iter = 1
    for k, v in kw.items():
        if k == "diag_sft":
            p.diag_sft[0] = v[0]
            p.diag_sft[1] = v[1] if len(v) > 1 else v[0]
        else:
            setattr(p, k, v)
    return p


_P = C.c_void_p
_i32, _i64, _u64, _dbl = C.c_int32, C.c_int64, C.c_uint64, C.c_double
_SIGS = {
    "neci_gpu_init": (_i32, [C.POINTER(_P), C.POINTER(System), _i32]),
    "neci_gpu_free": (_i32, [_P]),
    "neci_gpu_last_error": (C.c_char_p, []),
    "neci_gpu_set_random_hash": (_i32, [_P, _P]),
    "neci_gpu_set_tmat": (_i32, [_P, _P]),
    "neci_gpu_set_umat": (_i32, [_P, _P, _i64]),
    "neci_gpu_set_lattice": (_i32, [_P, _P, _i32]),
    "neci_gpu_set_reference": (_i32, [_P, _P, _dbl]),
    "neci_gpu_init_pchb": (_i32, [_P]),
    "neci_gpu_set_excit_biases": (_i32, [_P, _dbl, _dbl]),
    "neci_gpu_set_tau_search": (_i32, [_P, _i32]),
    "neci_gpu_get_tau_stats": (_i32, [_P, C.POINTER(TauStats), _i32]),
    "neci_gpu_set_rdm_sampling": (_i32, [_P, _i32]),
    "neci_gpu_get_rdm": (_i32, [_P, _P, _i64, _i32]),
    "neci_gpu_upload_walkers": (_i32, [_P, _P, _i64, _P, _P]),
    "neci_gpu_download_walkers": (_i32, [_P, _P, _P, _P, _i64, _P]),
    "neci_gpu_check_rows": (_i64, [_P, _i64, _i32, _i32, _i32, _i32]),
    "neci_gpu_iterate": (_i32, [_P, C.POINTER(IterParams), C.POINTER(IterStats)]),
    "neci_gpu_iterate_n": (_i32, [_P, C.POINTER(IterParams), _i32, _P]),
    "neci_gpu_iterate_timed": (_i32, [_P, C.POINTER(IterParams), _i32, _P, _P]),
    "neci_gpu_iterate_batch": (_i32, [_P, _i32, _P, _i32, _P, _P]),
    "neci_gpu_annihilate": (_i32, [_P, C.POINTER(IterParams), _P, _i64, C.POINTER(IterStats)]),
    "neci_gpu_compress_spawns": (_i32, [_P, _P, _i64, _P, _P, _P]),
    "neci_gpu_compress_spawns_noalloc": (_i32, [_P, _i64, _i32, _i32, _i32, _i32, _P, _P, _P, _P, C.c_char_p, _i32]),
    "neci_gpu_find_walker_hash": (_i32, [_P, _P, _i64, _i64, _P]),
    "neci_gpu_excit_level": (_i32, [_P, _P, _P, _i64, _P]),
    "neci_gpu_helement": (_i32, [_P, _P, _P, _i64, _P]),
    "neci_gpu_gen_excit": (_i32, [_P, _P, _i64, _u64, _i64, _P, _P, _P]),
    "neci_gpu_set_core_space": (_i32, [_P, _P, _i64, _i32]),
    "neci_gpu_select_core": (_i32, [_P, _i64, _i32, _P, _P]),
    "neci_gpu_core_nnz": (_i32, [_P, _P]),
    "neci_gpu_set_option": (_i32, [_P, _i32, _i32]),
    "neci_gpu_set_tuning": (_i32, [_P, C.POINTER(Tuning)]),
    "neci_gpu_get_tuning": (_i32, [_P, C.POINTER(Tuning)]),
    "neci_gpu_autotune": (_i32, [_P, C.POINTER(IterParams), _i32, _P, _i32, _P, C.POINTER(Tuning)]),
    "neci_gpu_set_profiling": (_i32, [_P, _i32]),
    "neci_gpu_kernel_times": (_i32, [_P, _P, _P, _i32]),
    "neci_gpu_kernel_name": (C.c_char_p, [_i32]),
    "neci_gpu_num_kernels": (_i32, []),
    "neci_gpu_sync": (_i32, [_P]),
}
EXPORTS = tuple(_SIGS)

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load libneci_gpu.so (raises if it is missing: no fallback exists)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else _LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with neci_stable_gb300.build.build()")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


class NeciGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"neci_gpu error {code}: {msg}")
        self.code = code


def check(code: int) -> None:
    if code != OK:
        raise NeciGpuError(code, load().neci_gpu_last_error().decode())


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the C ABI must be contiguous"
    return a.ctypes.data_as(C.c_void_p)
