"""The oracle's annihilation of an injected spawn list pinned to an independent
restatement of NECI's rules, on the CPU.

With integer signs, every sum is exact and no OccupiedThresh rounding
applies (stochRoundSpawn, Annihilation.F90:1354-1418, and CalcHashTableStats,
load_balancer.fpp:697-722, only round |C| < 1), so the merge has a single
answer:

* CompressSpawnedList / FindResidualParticle (Annihilation.F90:249-634): the
  records of one determinant sum; the block is an initiator spawn if any
  record carries the initiator flag or, under the coherent rule, if two
  records carry non-zero signs; the annihilations of the compression add up
  to sum|s_k| - |sum s_k| (each step adds 2 min(|cum|, |new|) for opposite
  signs, which telescopes); zero blocks vanish;
* AnnihilateSpawnedParts (Annihilation.F90:965-1352): a block whose
  determinant is occupied adds to it, counting 2 min(|C|, |s|) when the
  signs are opposite, and an emptied determinant is removed; a block for an
  absent determinant is aborted when it is not an initiator spawn under
  truncinitiator (test_abort_spawn, :1462-1479), else it becomes a new
  determinant.
"""
from __future__ import annotations

from collections import defaultdict

import numpy as np
import pytest

from neci_stable_gb300 import capi, systems
from oracle.oracle import Oracle, all_determinants

INIT_BIT = capi.FLAG_INITIATOR[0]


def restated_annihilation(current, records, trunc, coherent):
    """current: {det: sign}; records: [(det, sign, initiator)].  Returns the
    new {det: sign}, nannihil and naborted."""
    blocks = defaultdict(list)
    for det, s, init in records:
        blocks[det].append((s, init))
    out = dict(current)
    nannihil = naborted = 0.0
    for det, recs in blocks.items():
        signs = [s for s, _ in recs]
        total = sum(signs)
        nannihil += sum(abs(s) for s in signs) - abs(total)
        if total == 0:
            continue
        init = any(i for _, i in recs) or (coherent and sum(1 for s in signs if s != 0) >= 2)
        if det in out:
            c = out[det]
            nannihil += abs(c) + abs(total) - abs(c + total)
            if c + total == 0:
                del out[det]
            else:
                out[det] = c + total
        elif trunc and not init:
            naborted += abs(total)
        else:
            out[det] = total
    return out, nannihil, naborted


def _rows(dets, signs, flags, W):
    rows = np.zeros((len(dets), W + 2), dtype=np.int64)
    rows[:, :W] = dets
    rows[:, W] = np.asarray(signs, dtype=np.float64).view(np.int64)
    rows[:, W + 1] = flags
    return rows


@pytest.mark.parametrize("trunc,coherent", [(1, 1), (1, 0), (0, 1)])
def test_injected_spawns_merge_by_the_rules(trunc, coherent):
    spec = systems.hubbard_system("chain", (8,), 8, u=2.0)
    W = spec.W
    orc = Oracle(spec, 8192, 65536)
    space = all_determinants(spec.nbasis, 4, 4, spec.nifd)
    rng = np.random.default_rng(11 + 2 * trunc + coherent)
    occ = rng.choice(space.shape[0], 600, replace=False)
    cur_signs = rng.integers(1, 6, occ.size) * rng.choice([-1, 1], occ.size)
    orc.upload(_rows(space[occ], cur_signs, 0, W))
    current = {tuple(space[i]): float(s) for i, s in zip(occ, cur_signs)}

    # spawns onto occupied and absent determinants, several records per determinant,
    # some blocks cancelling to zero, mixed initiator flags
    targets = rng.choice(space.shape[0], 5000)
    sp_signs = rng.integers(1, 4, targets.size) * rng.choice([-1, 1], targets.size)
    sp_init = rng.random(targets.size) < 0.3
    records = [(tuple(space[t]), float(s), bool(i)) for t, s, i in zip(targets, sp_signs, sp_init)]
    spawned = _rows(space[targets], sp_signs, np.where(sp_init, 1 << INIT_BIT, 0), W)

    p = capi.default_params(seed=5, iter=2, t_trunc_initiator=trunc, t_init_coherent_rule=coherent,
                            occupied_thresh=1.0)
    st, rc = orc.annihilate(p, spawned)
    assert rc == 0

    expect, nannihil, naborted = restated_annihilation(current, records, trunc, coherent)
    got = {tuple(r[:W]): r[W:W + 1].view(np.float64)[0] for r in orc.download()[0]}
    got = {k: v for k, v in got.items() if v != 0.0}
    assert got == expect
    assert st.nannihil[0] == nannihil
    assert st.naborted[0] == naborted
    assert st.tot_parts[0] == sum(abs(v) for v in expect.values())
    assert naborted > 0 or not trunc        # the aborts are exercised
    assert nannihil > 0


def test_compression_alone_matches_the_rules():
    spec = systems.hubbard_system("chain", (8,), 8, u=2.0)
    W = spec.W
    orc = Oracle(spec, 8192, 65536)
    space = all_determinants(spec.nbasis, 4, 4, spec.nifd)
    rng = np.random.default_rng(3)
    targets = rng.choice(space.shape[0], 3000)
    signs = rng.integers(1, 4, targets.size) * rng.choice([-1, 1], targets.size)
    init = rng.random(targets.size) < 0.2
    spawned = _rows(space[targets], signs, np.where(init, 1 << INIT_BIT, 0), W)
    p = capi.default_params(t_trunc_initiator=1, t_init_coherent_rule=1)
    out, nann = orc.compress_spawns(p, spawned)

    blocks = defaultdict(list)
    for t, s, i in zip(targets, signs, init):
        blocks[tuple(space[t])].append((float(s), bool(i)))
    expect_total, expect_init, expect_nann = {}, {}, 0.0
    for det, recs in blocks.items():
        tot = sum(s for s, _ in recs)
        expect_nann += sum(abs(s) for s, _ in recs) - abs(tot)
        if tot != 0:
            expect_total[det] = tot
            expect_init[det] = any(i for _, i in recs) or len(recs) >= 2
    got_total = {tuple(r[:W]): r[W:W + 1].view(np.float64)[0] for r in out}
    got_init = {tuple(r[:W]): bool((r[W + 1] >> INIT_BIT) & 1) for r in out}
    assert got_total == expect_total
    assert got_init == expect_init
    assert nann[0] == expect_nann
    # sorted by ilut_lt (DetBitOps.F90:431): signed 64-bit words, first word first
    keys = [tuple(int(x) for x in r[:W]) for r in out]
    assert keys == sorted(keys)


def test_compressed_list_sorts_by_signed_words():
    # 32 sites: spin orbital 64 is bit 63 of the first word, so half the
    # determinants have a negative first word; ilut_lt compares signed int64
    from helpers import random_dets
    spec = systems.hubbard_system("square", (4, 8), 32, u=4.0)
    W = spec.W
    orc = Oracle(spec, 8192, 65536)
    rng = np.random.default_rng(9)
    dets = random_dets(spec, 400, rng)
    assert (dets[:, 0] < 0).any() and (dets[:, 0] > 0).any()
    spawned = _rows(dets, np.ones(dets.shape[0]), 0, W)
    out, _ = orc.compress_spawns(capi.default_params(), spawned)
    keys = [tuple(int(x) for x in r[:W]) for r in out]
    assert keys == sorted(set(tuple(int(x) for x in d) for d in dets))
