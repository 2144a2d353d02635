"""The allocation-free compression entry point, for hosts that may not call
cudaMalloc (code inside another program's memory pool, or a process that must
not grow its GPU footprint after start-up).

neci_gpu_compress_spawns_noalloc works in fixed file-scope device scratch;
the test hands it device buffers owned by the caller (allocated here through
torch, as such a host would own them) and checks that two calls in a row give
exactly the rows and annihilation counts of the context-based
neci_gpu_compress_spawns, for every combination of the initiator flag rules
(tTruncInitiator, tInitCoherentRule), that an empty list gives no rows, and
that a list over the size limit is refused with a message."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from neci_stable_gb300 import capi
from neci_stable_gb300.engine import Engine

from helpers import hubbard10, molecule, random_spawns, random_walkers

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 18


def ilut_sorted(rows, W):
    order = np.lexsort(tuple(rows[:, w] for w in reversed(range(W))))
    return rows[order]


def noalloc(lib, torch, spec, sp, trunc, coherent):
    """One call of the entry point on caller-owned device buffers."""
    d_in = torch.from_numpy(sp).cuda() if sp.shape[0] else torch.zeros((1, spec.W + spec.lenof_sign + 1),
                                                                      dtype=torch.int64, device="cuda")
    d_out = torch.zeros_like(d_in)
    n_out = C.c_int64(-1)
    nann = np.full(2, -1.0)
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.neci_gpu_compress_spawns_noalloc(
        C.c_void_p(d_in.data_ptr()), sp.shape[0], spec.nifd, spec.lenof_sign, trunc, coherent,
        C.c_void_p(d_out.data_ptr()), C.byref(n_out), capi.ptr(nann), C.c_void_p(stream), err, 256)
    assert rc == capi.OK, err.value
    return d_out[: n_out.value].cpu().numpy(), nann[: spec.lenof_sign]


@pytest.mark.parametrize("trunc,coherent", [(1, 1), (1, 0), (0, 1), (0, 0)])
@pytest.mark.parametrize("make", [lambda: hubbard10(), lambda: hubbard10(lenof_sign=2), lambda: molecule(40, 12)])
def test_noalloc_compression_matches_context_entry_point(make, trunc, coherent):
    torch = pytest.importorskip("torch")
    spec = make()
    eng = Engine(spec, max_walkers=100_000, max_spawned=300_000)
    # the context's flag rules are those of the last parameters it was given:
    # an annihilation of no spawns on an empty list hands them over
    eng.upload(np.zeros((0, eng.R), dtype=np.int64))
    eng.annihilate(capi.default_params(t_trunc_initiator=trunc, t_init_coherent_rule=coherent),
                   np.zeros((0, eng.R), dtype=np.int64))
    lib = capi.load()
    rng = np.random.default_rng(404 + 2 * trunc + coherent)
    walkers = random_walkers(spec, 800, rng)
    W = spec.W
    for call in range(2):
        sp = random_spawns(spec, walkers, 40_000 + 7_000 * call, rng)
        ref_rows, ref_nann = eng.compress_spawns(sp)
        got, nann = noalloc(lib, torch, spec, sp, trunc, coherent)
        assert np.array_equal(ilut_sorted(got, W), ref_rows)
        np.testing.assert_allclose(nann, ref_nann, rtol=1e-12, atol=1e-9)
    # an empty list: no rows and nothing annihilated, after the calls above
    got, nann = noalloc(lib, torch, spec, np.zeros((0, eng.R), dtype=np.int64), trunc, coherent)
    assert got.shape[0] == 0 and np.all(nann == 0.0)
    eng.close()


def test_noalloc_refuses_lists_over_the_limit():
    lib = capi.load()
    n_out = C.c_int64(-1)
    err = C.create_string_buffer(256)
    rc = lib.neci_gpu_compress_spawns_noalloc(None, MAX_ROWS + 1, 0, 1, 1, 1, None, C.byref(n_out), None, None,
                                              err, 256)
    assert rc == capi.ERR_INVALID
    assert b"at most 262144" in err.value
