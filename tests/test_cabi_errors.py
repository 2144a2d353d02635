"""CPU checks of the C ABI's error convention: every entry point validates its
arguments before it touches the device, returns a status code and leaves the
reason in ``neci_gpu_last_error``.  NECI's host maps a non-zero status to
``err`` (``FciMCPar.F90:507-508``), and an unsupported system or generator
sends the host back to its Fortran path (``fcimc_initialisation.fpp:2029-2270``
binds the generator the device must match).  None of these calls reaches CUDA,
so they run without a GPU."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

from neci_stable_gb300 import capi, systems

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "neci_gpu.h"


@pytest.fixture(scope="module")
def lib():
    if not capi._LIB_PATH.exists():
        pytest.skip("library not built (run __graft_entry__.build())")
    return capi.load()


def _system(**kw) -> capi.System:
    s = capi.System()
    s.nel, s.nbasis, s.nifd, s.lenof_sign = 10, 48, 0, 1
    s.system, s.excitgen, s.max_neighbours = capi.SYS_MOLECULAR, capi.EXGEN_PCHB, 0
    s.p_singles, s.p_parallel = 0.1, 0.3
    s.max_walkers, s.max_spawned, s.n_walker_hashes = 1000, 1000, 700
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def _init(lib, sys_) -> tuple[int, C.c_void_p]:
    ctx = C.c_void_p(12345)  # overwritten with NULL on failure
    rc = lib.neci_gpu_init(C.byref(ctx), C.byref(sys_), 0)
    return rc, ctx


@pytest.mark.parametrize("kw,code,why", [
    (dict(nbasis=256, nifd=3), capi.ERR_UNSUPPORTED, "nBasis"),
    (dict(nbasis=200, nifd=2), capi.ERR_UNSUPPORTED, "nBasis"),  # 3 words hold 192 orbitals
    (dict(nifd=-1), capi.ERR_UNSUPPORTED, "nBasis"),
    (dict(nel=1), capi.ERR_UNSUPPORTED, "nel"),
    (dict(nel=66, nbasis=200, nifd=3), capi.ERR_UNSUPPORTED, "nel"),
    (dict(lenof_sign=3), capi.ERR_UNSUPPORTED, "lenof_sign"),
    (dict(excitgen=capi.EXGEN_RS_HUBBARD), capi.ERR_UNSUPPORTED, "generator"),
    (dict(system=capi.SYS_HUBBARD_REAL_SPACE, excitgen=capi.EXGEN_PCHB, max_neighbours=4),
     capi.ERR_UNSUPPORTED, "rs-hubbard"),
    (dict(system=capi.SYS_HUBBARD_REAL_SPACE, excitgen=capi.EXGEN_RS_HUBBARD, max_neighbours=0),
     capi.ERR_UNSUPPORTED, "max_neighbours"),
    (dict(system=7), capi.ERR_UNSUPPORTED, "unknown system"),
    (dict(max_walkers=1), capi.ERR_INVALID, "max_walkers"),
    (dict(max_spawned=0), capi.ERR_INVALID, "max_spawned"),
    (dict(max_walkers=1 << 31), capi.ERR_INVALID, "max_walkers"),
])
def test_init_refuses_systems_off_the_device_path(lib, kw, code, why):
    rc, ctx = _init(lib, _system(**kw))
    assert rc == code
    assert ctx.value is None
    assert why in lib.neci_gpu_last_error().decode()


def test_init_null_arguments(lib):
    assert lib.neci_gpu_init(None, C.byref(_system()), 0) == capi.ERR_INVALID
    ctx = C.c_void_p()
    assert lib.neci_gpu_init(C.byref(ctx), None, 0) == capi.ERR_INVALID
    assert "null" in lib.neci_gpu_last_error().decode()


def _context_entry_points():
    """Entry points of the header whose first parameter is the context."""
    text = HEADER.read_text()
    names = re.findall(r"^\s*int32_t\s+(neci_gpu_\w+)\s*\(\s*neci_gpu_ctx\s*\*\s*\w+", text, re.M)
    return sorted(set(names) - {"neci_gpu_free"})


def test_every_context_entry_point_is_bound():
    names = _context_entry_points()
    assert len(names) >= 25
    assert set(names) <= set(capi.EXPORTS)


@pytest.mark.parametrize("name", _context_entry_points())
def test_null_context_is_an_error_not_a_fault(lib, name):
    f = getattr(lib, name)
    args = []
    for t in f.argtypes:
        if t in (C.c_int32, C.c_int64, C.c_uint64):
            args.append(1)
        elif t is C.c_double:
            args.append(0.5)
        else:
            args.append(None)
    assert f(*args) == capi.ERR_INVALID
    assert lib.neci_gpu_last_error().decode() == "null context"


def test_free_of_null_is_a_no_op(lib):
    assert lib.neci_gpu_free(None) == capi.OK


@pytest.mark.parametrize("n_ctx,n_iter", [(0, 1), (1, 0), (-1, 1)])
def test_batch_argument_checks(lib, n_ctx, n_iter):
    ctxs = (C.c_void_p * 1)(None)
    params = (capi.IterParams * 1)(capi.default_params())
    stats = (capi.IterStats * 1)()
    rc = lib.neci_gpu_iterate_batch(ctxs, n_ctx, params, n_iter, stats, None)
    assert rc == capi.ERR_INVALID


def test_batch_with_a_null_context(lib):
    ctxs = (C.c_void_p * 2)(None, None)
    params = (capi.IterParams * 2)(capi.default_params(), capi.default_params())
    stats = (capi.IterStats * 2)()
    assert lib.neci_gpu_iterate_batch(ctxs, 2, params, 1, stats, None) == capi.ERR_INVALID
    assert "null context" in lib.neci_gpu_last_error().decode()


def _noalloc(lib, n, nifd=0, lenof_sign=1, with_ptrs=True):
    buf = C.create_string_buffer(256)
    n_out = C.c_int64(-1)
    dummy = C.c_void_p(16) if with_ptrs else None  # never dereferenced: the call returns before any copy
    rc = lib.neci_gpu_compress_spawns_noalloc(dummy, n, nifd, lenof_sign, 1, 1, dummy, C.byref(n_out), None, None,
                                             buf, len(buf))
    return rc, buf.value.decode(), n_out.value


def test_noalloc_limits_are_checked_before_the_device(lib):
    rc, msg, _ = _noalloc(lib, 262145)
    assert rc == capi.ERR_INVALID and "at most 262144" in msg
    rc, msg, _ = _noalloc(lib, -1)
    assert rc == capi.ERR_INVALID and "-1 spawn records" in msg
    for kw in (dict(nifd=-1), dict(nifd=4), dict(lenof_sign=0), dict(lenof_sign=3)):
        rc, msg, _ = _noalloc(lib, 8, **kw)
        assert rc == capi.ERR_INVALID and "bad argument" in msg
    rc, msg, _ = _noalloc(lib, 8, with_ptrs=False)
    assert rc == capi.ERR_INVALID and "bad argument" in msg


def test_noalloc_error_buffer_is_optional_and_bounded(lib):
    n_out = C.c_int64(0)
    assert lib.neci_gpu_compress_spawns_noalloc(None, -5, 0, 1, 1, 1, None, C.byref(n_out), None, None, None,
                                                0) == capi.ERR_INVALID
    small = C.create_string_buffer(8)
    assert lib.neci_gpu_compress_spawns_noalloc(None, -5, 0, 1, 1, 1, None, C.byref(n_out), None, None, small,
                                                len(small)) == capi.ERR_INVALID
    assert len(small.value) < len(small)  # truncated and terminated inside the caller's buffer


def test_kernel_names(lib):
    n = lib.neci_gpu_num_kernels()
    assert n >= 10
    names = [lib.neci_gpu_kernel_name(i).decode() for i in range(n)]
    assert all(names) and len(set(names)) == n
    assert {"spawn", "sweep", "ann_probe", "ann_insert", "merge_stats"} <= set(names)
    assert lib.neci_gpu_kernel_name(-1) == b"" and lib.neci_gpu_kernel_name(n) == b""


def _check(lib, rows, nifd, lenof_sign, nel, nbasis):
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    return lib.neci_gpu_check_rows(rows.ctypes.data_as(C.c_void_p), rows.shape[0], nifd, lenof_sign, nel, nbasis)


@pytest.mark.parametrize("name", ["hub4x8", "mol24", "mol80u"])
def test_upload_row_check_accepts_every_valid_determinant(lib, name):
    from helpers import make_rows, random_dets
    spec = {"hub4x8": lambda: systems.hubbard_system("square", (4, 8), 32, u=4.0),
            "mol24": lambda: _fake_molecule(48, 10, 0),
            "mol80u": lambda: _fake_molecule(160, 20, 2)}[name]()
    rng = np.random.default_rng(1)
    dets = random_dets(spec, 500, rng)
    signs = np.zeros((dets.shape[0], spec.lenof_sign))
    signs[::2, 0] = 3.0                      # zero-sign rows (holes) are uploaded too
    rows = make_rows(dets, signs, np.zeros(dets.shape[0], dtype=np.int64))
    assert _check(lib, rows, spec.nifd, spec.lenof_sign, spec.nel, spec.nbasis) == -1
    assert _check(lib, rows[:0], spec.nifd, spec.lenof_sign, spec.nel, spec.nbasis) == -1


def _fake_molecule(nbasis, nel, nifd):
    # the check needs only the layout: nel electrons, nBasis, NIfD, a reference
    ref = list(range(1, nel + 1))
    return SimpleNamespace(nbasis=nbasis, nel=nel, nifd=nifd, W=nifd + 1, lenof_sign=1, reference=ref)


def test_upload_row_check_finds_the_first_bad_row(lib):
    from helpers import make_rows
    nifd, nel, nbasis = 2, 20, 160
    good = systems.encode_det(list(range(1, nel + 1)), nifd)
    rows = make_rows(np.repeat(good[None], 6, axis=0), np.ones((6, 1)), np.zeros(6, dtype=np.int64))
    assert _check(lib, rows, nifd, 1, nel, nbasis) == -1
    few = rows.copy()
    few[3, 0] &= ~1                          # one electron short
    assert _check(lib, few, nifd, 1, nel, nbasis) == 3
    many = rows.copy()
    many[4, 1] |= 1 << 5                     # one electron too many
    assert _check(lib, many, nifd, 1, nel, nbasis) == 4
    past = rows.copy()
    past[2, 0] &= ~1
    past[2, 2] = 1 << 40                     # orbital 169 > nBasis, count still nel
    assert _check(lib, past, nifd, 1, nel, nbasis) == 2
    edge = rows.copy()
    edge[1, 0] &= ~1
    edge[1, 2] = 1 << 31                     # orbital 160 = nBasis: allowed
    assert _check(lib, edge, nifd, 1, nel, nbasis) == -1
    # flags and signs do not count
    rows[:, -1] = -1
    rows[:, nifd + 1] = -1
    assert _check(lib, rows, nifd, 1, nel, nbasis) == -1


def test_upload_row_check_arguments(lib):
    rows = np.zeros((2, 3), dtype=np.int64)
    assert _check(lib, rows, -1, 1, 2, 64) == -2
    assert _check(lib, rows, 4, 1, 2, 64) == -2
    assert _check(lib, rows, 0, 3, 2, 64) == -2
    assert lib.neci_gpu_check_rows(None, 1, 0, 1, 2, 64) == -2
    assert lib.neci_gpu_check_rows(None, -1, 0, 1, 2, 64) == -2
    assert lib.neci_gpu_check_rows(None, 0, 0, 1, 2, 64) == -1
