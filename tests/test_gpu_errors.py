"""Error paths on the GPU that need no fault: an allocation that fails comes
back as NECI_GPU_ERR_CUDA with nothing launched, and the context stays
usable.

The PCHB alias tables are built with a scratch array of a few hundred MB
(the per-thread stacks of init_AliasTable_t, aliasSampling.F90:209-297).  The
test leaves the device just enough memory for the tables themselves, so that
the scratch allocation fails; neci_gpu_init_pchb must report it before any
kernel runs, and succeed once the memory is back."""
from __future__ import annotations

import numpy as np
import pytest

from neci_stable_gb300 import capi
from neci_stable_gb300.engine import Engine

from helpers import molecule

pytestmark = pytest.mark.gpu


def pchb_table_bytes(n_spatial):
    """Device bytes neci_gpu_init_pchb allocates for the tables (before the scratch)."""
    ij = n_spatial * (n_spatial + 1) // 2
    ntab = 3 * ij
    per_entry = 8 + 8 + 4 + 8 + 4 + 8 + 4 + 32   # bias, prob, alias, thr, prob32, inv, inv32, record
    return ntab * ij * per_entry + ntab + ij * (8 + 8 + 4 + 8 + 8 + 4 + 4) + (ij + 1) * 4


def test_pchb_scratch_allocation_failure_is_reported():
    torch = pytest.importorskip("torch")
    spec = molecule(64, 20)
    eng = Engine(spec, max_walkers=100_000, max_spawned=200_000, pchb=False)
    lib = capi.load()
    tables = pchb_table_bytes(64)
    scratch = 49 * 128 * 2 * 2080 * 4   # 49 blocks of 128 threads, 2 stacks of abMax int32 each
    assert scratch > 90 << 20
    torch.cuda.synchronize()
    free, _ = torch.cuda.mem_get_info()
    # room for the tables, their allocation granularity and the 20 KB weight
    # sums, but not for the scratch
    leave = tables + (60 << 20)
    hog = torch.empty(max(free - leave, 0), dtype=torch.uint8, device="cuda")
    try:
        rc = lib.neci_gpu_init_pchb(eng.ctx)
        msg = lib.neci_gpu_last_error().decode()
    finally:
        del hog
        torch.cuda.empty_cache()
    assert rc == capi.ERR_CUDA, (rc, msg)
    assert "PCHB table build" in msg, msg
    # nothing faulted: the context works once the memory is free again
    capi.check(lib.neci_gpu_init_pchb(eng.ctx))
    eng.start_from_reference(initial_part=50.0)
    st = eng.perform_fcimc_cyc_par(capi.default_params(tau=0.001, seed=1, iter=1))
    assert st.err == 0 and st.tot_parts[0] > 0.0
    eng.close()
