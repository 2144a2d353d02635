"""GPU parity of the paths that a switch, the step's size or the set-up
selects, against the CPU oracle through the C ABI:

* the sort form of the annihilation (NECI_OPT_ANNIHILATION = NECI_ANN_SORT:
  CompressSpawnedList's sort, Annihilation.F90:273, and FindResidualParticle,
  :551-634): compression, injected annihilation, runs longer than one thread
  handles, determinants whose sort keys collide, and whole iterations;
* the walker-hash lookup inside the spawn kernel forced on for lattices
  (NECI_OPT_FUSE_PROBE = 1), with the separate lookup kernel shown not to run;
* a parent with more than 65536 spawn attempts (the whole-grid expansion);
* the molecule and the 6x6 lattice at about 1e5 walkers;
* the device selection of the core space (neci_gpu_select_core) against the
  host's stable argsort of the downloaded list.

Bit-exact: walker lists row for row, the estimators to FP64 summation order."""
from __future__ import annotations

import numpy as np
import pytest

from neci_stable_gb300 import capi
from neci_stable_gb300.engine import Engine
from oracle.oracle import Oracle

from helpers import canonical, canonical_with, hubbard10, hubbard_square, molecule, random_spawns, random_walkers

pytestmark = pytest.mark.gpu

SYSTEMS = {
    "hub10": lambda: hubbard10(),
    "hub10x2": lambda: hubbard10(lenof_sign=2),
    "hub6x6": lambda: hubbard_square(6, 6, 36),
    "mol12": lambda: molecule(12, 6),
    "mol12x2": lambda: molecule(12, 6, lenof_sign=2),
    "mol24": lambda: molecule(24, 10),
    "mol40": lambda: molecule(40, 12),
}

STAT_FIELDS = ("nborn", "ndied", "nannihil", "naborted", "nremoved", "tot_parts", "hf_cyc", "enum_cyc",
               "tot_parts_old")

_cache = {}


def pair(name, ann=capi.ANN_HASH, max_walkers=400_000, max_spawned=800_000):
    key = (name, max_walkers, max_spawned)
    if key not in _cache:
        spec = SYSTEMS[name]()
        eng = Engine(spec, max_walkers, max_spawned)
        orc = Oracle(spec, max_walkers, max_spawned, hii=eng.hii)
        _cache.clear()
        _cache[key] = (spec, eng, orc)
    spec, eng, orc = _cache[key]
    eng.set_option(capi.OPT_ANNIHILATION, ann)
    eng.set_option(capi.OPT_FUSE_PROBE, -1)
    return spec, eng, orc


def assert_same_list(spec, eng, orc, tag):
    W, L = spec.W, spec.lenof_sign
    rg = canonical(eng.download()[0], W)
    rc = canonical(orc.download()[0], W)
    assert rg.shape == rc.shape, (tag, rg.shape, rc.shape)
    assert np.array_equal(rg[:, :W + L], rc[:, :W + L]), tag
    assert np.array_equal(rg[:, -1] & ~1, rc[:, -1] & ~1), tag


def assert_same_stats(sg, sc, tag):
    for f in STAT_FIELDS:
        np.testing.assert_allclose(getattr(sg, f)[:], getattr(sc, f)[:], rtol=1e-9, atol=1e-7, err_msg=f"{f} {tag}")
    assert (sg.n_attempts, sg.n_spawned, sg.n_new, sg.n_occupied) == (sc.n_attempts, sc.n_spawned, sc.n_new,
                                                                     sc.n_occupied), tag
    # every slot in use is occupied or a hole (the merge sweep counts the slots
    # the step began with, the placement and the final kernel the rest)
    assert sg.n_occupied + sg.holes_in_list == sg.tot_walkers, (tag, sg.n_occupied, sg.holes_in_list, sg.tot_walkers)


def step_both(spec, eng, orc, iters, tau, seed, first_iter=1, shift=0.0, check_unique=True):
    """iters steps of engine and oracle from the same list, compared after each."""
    for it in range(first_iter, first_iter + iters):
        p = capi.default_params(tau=tau, diag_sft=[shift, shift], seed=seed, iter=it)
        sg = eng.perform_fcimc_cyc_par(p)
        sc, rc = orc.iterate(p)
        assert rc == 0 and sg.err == 0, (it, rc, sg.err)
        assert_same_list(spec, eng, orc, it)
        assert_same_stats(sg, sc, it)
        if check_unique:
            assert sg.n_unique == sc.n_unique, (it, sg.n_unique, sc.n_unique)
    return sg


# --------------------------------------------------------------- sort form
@pytest.mark.parametrize("name", ["hub10", "hub10x2", "mol24"])
def test_sort_compress_matches_oracle(name):
    spec, eng, orc = pair(name, capi.ANN_SORT)
    default_flags(eng)
    rng = np.random.default_rng(40)
    walkers = random_walkers(spec, 500, rng)
    for n in (0, 1, 17, 5000, 60000):
        sp = random_spawns(spec, walkers, n, rng)
        out_g, nann_g = eng.compress_spawns(sp)
        out_c, nann_c = orc.compress_spawns(capi.default_params(), sp)
        assert np.array_equal(out_g, out_c), n
        np.testing.assert_allclose(nann_g, nann_c, rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("name", ["hub10", "hub10x2", "mol24", "mol40"])
@pytest.mark.parametrize("trunc", [1, 0])
def test_sort_annihilate_injected(name, trunc):
    spec, eng, orc = pair(name, capi.ANN_SORT)
    rng = np.random.default_rng(50 + trunc)
    W, L = spec.W, spec.lenof_sign
    walkers = random_walkers(spec, 3000, rng)
    holes = rng.random(walkers.shape[0]) < 0.1
    walkers[holes, W:W + L] = 0
    eng.upload(walkers)
    orc.upload(walkers)
    p = capi.default_params(seed=99, iter=3, t_trunc_initiator=trunc, occupied_thresh=1.0)
    sp = random_spawns(spec, walkers, 20000, rng)
    sg = eng.annihilate(p, sp)
    sc, rc = orc.annihilate(p, sp)
    assert rc == 0 and sg.err == 0
    rg, (dg, og) = canonical_with(eng.download()[0], [eng.download()[1], eng.download()[2]], W)
    rcpu, (dc, oc) = canonical_with(orc.download()[0], [orc.download()[1], orc.download()[2]], W)
    assert rg.shape == rcpu.shape
    assert np.array_equal(rg[:, :W + L], rcpu[:, :W + L])
    assert np.array_equal(rg[:, -1] & ~1, rcpu[:, -1] & ~1)
    assert np.array_equal(dg, dc) and np.array_equal(og, oc)
    for f in ("nborn", "nannihil", "naborted", "nremoved", "tot_parts", "norm_psi_sq", "tot_parts_old"):
        np.testing.assert_allclose(getattr(sg, f)[:], getattr(sc, f)[:], rtol=1e-10, atol=1e-8, err_msg=f)
    assert sg.n_new == sc.n_new and sg.n_occupied == sc.n_occupied


@pytest.mark.parametrize("name", ["hub10", "hub10x2", "mol24"])
@pytest.mark.parametrize("ann", [capi.ANN_HASH, capi.ANN_SORT])
def test_annihilate_keeps_one_record_flag_words(name, ann):
    """A new determinant made of one spawn record keeps that record's whole
    flag word (FindResidualParticle), other flag bits and the other run's
    initiator bit included, while the initiator abort reads the bits of the
    runs that carry an amplitude: bit for bit against the oracle."""
    spec, eng, orc = pair(name, ann)
    rng = np.random.default_rng(61)
    W, L = spec.W, spec.lenof_sign
    walkers = random_walkers(spec, 2000, rng)
    eng.upload(walkers)
    orc.upload(walkers)
    sp = random_spawns(spec, walkers, 15000, rng)
    extra = rng.random(sp.shape[0]) < 0.5
    sp[extra, -1] |= np.int64(1) << 5
    if L == 2:  # the other run's initiator bit on records of one run
        cross = rng.random(sp.shape[0]) < 0.3
        sp[cross, -1] |= np.int64(1) << capi.FLAG_INITIATOR[1]
    p = capi.default_params(seed=7, iter=5, t_trunc_initiator=1, occupied_thresh=1.0)
    sg = eng.annihilate(p, sp)
    sc, rc = orc.annihilate(p, sp)
    assert rc == 0 and sg.err == 0
    rg = canonical(eng.download()[0], W)
    rcpu = canonical(orc.download()[0], W)
    assert rg.shape == rcpu.shape
    assert np.array_equal(rg[:, :W + L], rcpu[:, :W + L])
    assert np.array_equal(rg[:, -1] & ~1, rcpu[:, -1] & ~1)
    assert np.any((rg[:, -1] >> 5) & 1), "no kept flag word carries the extra bit"
    assert sg.n_new == sc.n_new and sg.n_occupied == sc.n_occupied


def default_flags(eng):
    """Hands the context NECI's default flag rules (tTruncInitiator and
    tInitCoherentRule on), which the compression applies: an annihilation of
    no spawns on an empty list."""
    empty = np.zeros((0, eng.R), dtype=np.int64)
    eng.upload(empty)
    eng.annihilate(capi.default_params(), empty)


def random_dets_one_word(spec, n, rng):
    """n random determinants of a one-word system with the reference's alpha
    and beta counts, drawn in bulk."""
    assert spec.W == 1
    norb = spec.nbasis // 2
    na = sum(1 for o in spec.reference if o % 2 == 0)
    nb = spec.nel - na
    out = np.zeros(n, dtype=np.uint64)
    for count, spin in ((na, 0), (nb, 1)):   # alpha orbital 2p (bit 2p-1), beta 2p-1 (bit 2p-2)
        pick = np.argsort(rng.random((n, norb)), axis=1)[:, :count]
        bit = (2 * (pick + 1) - 1 - spin).astype(np.uint64)
        out |= np.bitwise_or.reduce(np.left_shift(np.uint64(1), bit), axis=1)
    return out.view(np.int64)[:, None]


def colliding_dets(spec, eng, n_search, rng):
    """Pairs of different determinants whose FindWalkerHash values agree in
    the low 32 bits of their magnitude, which is all the sort key holds."""
    dets = np.unique(random_dets_one_word(spec, n_search, rng), axis=0)
    low = eng.find_walker_hash(dets, 1 << 32)  # abs(h) mod 2^32 + 1
    order = np.argsort(low, kind="stable")
    ls = low[order]
    same = np.nonzero(ls[1:] == ls[:-1])[0]
    return [(dets[order[i]], dets[order[i + 1]]) for i in same]


def test_sort_long_runs_and_key_collisions():
    """Runs of equal sort keys longer than one thread takes (a determinant
    with 500 spawns), keys shared by two determinants (interleaved in the
    sorted run), and a long run that holds two determinants: compression and
    annihilation equal the oracle's, and the hash form's."""
    spec, eng, orc = pair("mol24", capi.ANN_SORT)
    default_flags(eng)
    rng = np.random.default_rng(60)
    W, L = spec.W, spec.lenof_sign
    pairs = colliding_dets(spec, eng, 400_000, rng)
    assert len(pairs) >= 3, "no colliding keys found"
    walkers = random_walkers(spec, 2000, rng)
    # a colliding pair half in the list, so that the annihilation finds one
    # determinant of the key and inserts the other
    wrow = walkers[:1].copy()
    wrow[0, :W] = pairs[0][0]
    walkers = np.concatenate([walkers, wrow])
    walkers = walkers[np.unique(walkers[:, :W], axis=0, return_index=True)[1]]

    def records(det, n, run=0):
        r = np.zeros((n, W + L + 1), dtype=np.int64)
        r[:, :W] = det
        vals = np.round(rng.normal(0.0, 1.5, size=n) * 64) / 64
        vals[vals == 0] = 1.0 / 64
        sg = np.zeros((n, L))
        sg[:, run] = vals
        r[:, W:W + L] = sg.view(np.int64)
        init = rng.random(n) < 0.3
        r[init, -1] = np.int64(1) << capi.FLAG_INITIATOR[run]
        return r

    parts = [random_spawns(spec, walkers, 8000, rng),
             records(walkers[5, :W], 500),                      # a long run of one determinant
             records(pairs[1][0], 25), records(pairs[1][1], 20),  # a long run of two determinants
             records(pairs[0][0], 3), records(pairs[0][1], 2)]   # a short run of two
    for a, b in pairs[2:]:
        parts += [records(a, 1), records(b, 1)]
    sp = np.concatenate(parts)
    sp = sp[rng.permutation(sp.shape[0])]
    out_s, nann_s = eng.compress_spawns(sp)
    out_c, nann_c = orc.compress_spawns(capi.default_params(), sp)
    assert np.array_equal(out_s, out_c)
    np.testing.assert_allclose(nann_s, nann_c, rtol=1e-12, atol=1e-9)
    eng.set_option(capi.OPT_ANNIHILATION, capi.ANN_HASH)
    out_h, _ = eng.compress_spawns(sp)
    assert np.array_equal(out_s, out_h)
    for mode in (capi.ANN_SORT, capi.ANN_HASH):
        eng.set_option(capi.OPT_ANNIHILATION, mode)
        eng.upload(walkers)
        orc.upload(walkers)
        p = capi.default_params(seed=7, iter=2)
        sg = eng.annihilate(p, sp)
        sc, rc = orc.annihilate(p, sp)
        assert rc == 0 and sg.err == 0
        assert_same_list(spec, eng, orc, f"mode {mode}")
        for f in ("nborn", "nannihil", "naborted", "nremoved", "tot_parts"):
            np.testing.assert_allclose(getattr(sg, f)[:], getattr(sc, f)[:], rtol=1e-10, atol=1e-8, err_msg=f)
        assert sg.n_new == sc.n_new and sg.n_unique == sc.n_unique


@pytest.mark.parametrize("name,iters,pop,tau", [("hub10", 25, 50.0, 0.02), ("hub10x2", 15, 20.0, 0.02),
                                                ("hub6x6", 10, 30.0, 0.01), ("mol12x2", 15, 40.0, 0.02),
                                                ("mol24", 15, 200.0, 0.005), ("mol40", 10, 100.0, 0.005)])
def test_sort_iterations_bit_exact(name, iters, pop, tau):
    spec, eng, orc = pair(name, capi.ANN_SORT)
    eng.start_from_reference(initial_part=pop)
    orc.upload(eng.download()[0])
    st = step_both(spec, eng, orc, iters, tau, seed=33)
    assert st.n_occupied > 1


# ------------------------------------------------------- fused lookup, forced
@pytest.mark.parametrize("name,pop", [("hub10", 60.0), ("hub6x6", 40.0)])
def test_fused_lookup_forced_on_and_off(name, pop):
    """NECI_OPT_FUSE_PROBE = 1: the spawn kernel looks every child up and the
    separate lookup kernel does not run; = 0: the lookup kernel runs.  The
    lists stay bit-exact either way."""
    spec, eng, orc = pair(name)
    for mode, probe_runs in ((1, False), (0, True)):
        eng.set_option(capi.OPT_FUSE_PROBE, mode)
        eng.start_from_reference(initial_part=pop)
        orc.upload(eng.download()[0])
        eng.set_profiling(True)
        eng.kernel_times()
        try:
            step_both(spec, eng, orc, 12, 0.02, seed=71)
        finally:
            kt = eng.kernel_times()
            eng.set_profiling(False)
        assert (kt["ann_probe"][1] > 0) == probe_runs, (mode, kt["ann_probe"])
        assert kt["spawn"][1] == 12 and kt["ann_compress"][1] == 12
    eng.set_option(capi.OPT_FUSE_PROBE, -1)


def test_fused_lookup_option_is_for_lattices_only():
    spec, eng, orc = pair("mol12")
    with pytest.raises(capi.NeciGpuError) as ei:
        eng.set_option(capi.OPT_FUSE_PROBE, 1)
    assert ei.value.code == capi.ERR_UNSUPPORTED
    with pytest.raises(capi.NeciGpuError):
        eng.set_option(capi.OPT_ANNIHILATION, 7)
    with pytest.raises(capi.NeciGpuError):
        eng.set_option(99, 0)
    for bad in (0, 65537):
        with pytest.raises(capi.NeciGpuError):
            eng.set_option(capi.OPT_CORE_SEGMENT, bad)


# ------------------------------------------------- a parent of > 65536 attempts
@pytest.mark.parametrize("ann", [capi.ANN_HASH, capi.ANN_SORT])
def test_parent_with_more_than_65536_attempts(ann):
    """One determinant of |C| = 1e5 on the molecule: its attempts are expanded
    by the whole grid (more than 65536), and the steps stay bit-exact."""
    spec, eng, orc = pair("mol12", ann)
    eng.start_from_reference(initial_part=1.0e5)
    orc.upload(eng.download()[0])
    st = step_both(spec, eng, orc, 3, 0.01, seed=81)
    assert st.n_attempts > 65536


# ------------------------------------- parents expanded in several chunks
@pytest.mark.parametrize("name,pop", [("mol12", 3000.0), ("hub10x2", 2000.0)])
def test_parents_in_several_expansion_chunks(name, pop):
    """A parent of a few thousand attempts is handed to the expansion kernel in
    chunks of 512 (each a warp's work, the chunk's head carrying its first
    attempt index); with a replica pair both runs' chunks follow each other.
    The steps stay bit-exact, so every chunk wrote its entries."""
    spec, eng, orc = pair(name)
    eng.start_from_reference(initial_part=pop)
    orc.upload(eng.download()[0])
    st = step_both(spec, eng, orc, 4, 0.01, seed=83)
    assert st.n_attempts > 1024


# ---------------------------------------------------------- 1e5 walkers
@pytest.mark.parametrize("name,tau,grow,p_singles", [("mol24", 0.02, 6, 0.5), ("hub6x6", 0.002, 4, None)])
@pytest.mark.parametrize("ann", [capi.ANN_HASH, capi.ANN_SORT])
def test_1e5_walkers_bit_exact(name, tau, grow, p_singles, ann):
    """The walker list grown on the device from 1e5 walkers on the reference
    over many determinants, then 5 steps on engine and oracle from the same
    list.  The molecule runs with the excitation biases of the bench after
    the tau search (pSingles 0.5, tau 0.02), so that many spawns are written.
    With the shift at zero and little annihilation yet, the population grows
    by up to a fifth per step: the buffers are sized for it."""
    spec, eng, orc = pair(name, ann, max_walkers=2_000_000, max_spawned=4_000_000)
    if p_singles is not None:
        eng.set_excit_biases(p_singles, 0.3)
        orc.set_excit_biases(p_singles, 0.3)
    try:
        eng.start_from_reference(initial_part=1.0e5)
        for it in range(1, grow + 1):
            eng.perform_fcimc_cyc_par(capi.default_params(tau=tau, seed=90, iter=it))
        rows, dh, odh = eng.download()
        eng.upload(rows, dh, odh)
        orc.upload(rows, dh, odh)
        st = step_both(spec, eng, orc, 5, tau, seed=91, first_iter=grow + 1)
    finally:
        if p_singles is not None:
            eng.set_excit_biases(spec.p_singles, spec.p_parallel)
            orc.set_excit_biases(spec.p_singles, spec.p_parallel)
    assert st.tot_parts[0] > 1e5 and st.n_occupied > 5000 and st.n_spawned > 2e4, \
        (st.tot_parts[0], st.n_occupied, st.n_spawned)


# ------------------------------------------------------ device core selection
@pytest.mark.parametrize("name,n_core", [("hub10", 300), ("hub10x2", 200), ("mol24", 500)])
def test_select_core_matches_host_argsort(name, n_core):
    """neci_gpu_select_core picks the determinants a stable argsort of
    -sum|C| over the downloaded list picks (ties to the lower slot), in the
    same order; the core built from them is the one set_core_space builds,
    and the steps after it stay bit-exact against the oracle.  A second
    selection replaces the first."""
    spec, eng, orc = pair(name)
    W, L = spec.W, spec.lenof_sign
    eng.start_from_reference(initial_part=400.0)
    for it in range(1, 16):
        eng.perform_fcimc_cyc_par(capi.default_params(tau=0.02, seed=5, iter=it))
    rows, dh, odh = eng.download()
    pop = np.abs(rows[:, W:W + L].view(np.float64)).sum(axis=1)
    host = rows[np.argsort(-pop, kind="stable")[:n_core], :W]
    assert len(np.unique(pop)) < len(pop), "the test wants tied weights"
    got = eng.select_core(n_core)
    assert np.array_equal(got, host)
    nnz = eng.core_nnz()
    eng.upload(rows, dh, odh)
    eng.set_core_space(host)
    assert eng.core_nnz() == nnz
    # the device selection's core, stepped against the oracle's
    eng.upload(rows, dh, odh)
    eng.select_core(n_core)
    orc.upload(rows, dh, odh)
    orc.set_core_space(host)
    step_both(spec, eng, orc, 4, 0.02, seed=6, first_iter=16, check_unique=False)
    # a second selection on the stepped list replaces the core space
    n_sel = host.shape[0]   # n_core, or every occupied determinant if fewer
    rows2 = eng.download()[0]
    flags = rows2[:, W + L]
    assert np.count_nonzero((flags >> capi.FLAG_DETERMINISTIC[0]) & 1) == n_sel
    got2 = eng.select_core(n_sel // 2)
    rows3 = eng.download()[0]
    det3 = (rows3[:, W + L] >> capi.FLAG_DETERMINISTIC[0]) & 1
    assert np.count_nonzero(det3) == got2.shape[0] == n_sel // 2


def test_select_core_more_than_occupied():
    spec, eng, orc = pair("hub10")
    eng.start_from_reference(initial_part=5.0)
    got = eng.select_core(1000)
    assert got.shape[0] == 1 and np.array_equal(got[0], eng.ilut_ref)


# ------------------------------------------------------------- autotuning
@pytest.mark.parametrize("name,pop,tau", [("mol24", 300.0, 0.005), ("hub10x2", 60.0, 0.02)])
def test_autotune_steps_are_ordinary_steps(name, pop, tau):
    """neci_gpu_autotune times every candidate setting on live steps: the
    steps it runs are the run's own steps (the walker list after them equals
    the oracle's after as many iterations), and the setting it keeps is the
    one in force afterwards."""
    spec, eng, orc = pair(name)
    eng.start_from_reference(initial_part=pop)
    orc.upload(eng.download()[0])
    p = capi.default_params(tau=tau, seed=44, iter=1)
    stats, chosen = eng.autotune(p, 2)
    assert len(stats) == 7 * 3 and all(s.err == 0 for s in stats)
    for it in range(1, len(stats) + 1):
        sc, rc = orc.iterate(capi.default_params(tau=tau, seed=44, iter=it))
        assert rc == 0
        np.testing.assert_allclose(stats[it - 1].tot_parts[:spec.lenof_sign], sc.tot_parts[:spec.lenof_sign],
                                   rtol=1e-12)
    assert_same_list(spec, eng, orc, "after autotuning")
    now = eng.tuning()
    assert (now.annihilation, now.spawn_blocks_per_sm, now.table_shift, now.sort_blocks_per_sm) == \
        (chosen.annihilation, chosen.spawn_blocks_per_sm, chosen.table_shift, chosen.sort_blocks_per_sm)
    assert chosen.ns_per_update > 0.0
    # and the run goes on under it
    step_both(spec, eng, orc, 2, tau, seed=44, first_iter=len(stats) + 1)
    eng.set_tuning(capi.Tuning(capi.ANN_HASH, 8, 1, 2, 0.0))


# --------------------------------------------------- 2-RDM with a core space
@pytest.mark.parametrize("name,seg", [("hub10x2", None), ("mol12x2", None), ("mol12x2", 1)])
def test_rdm_with_core_space_matches_oracle(name, seg):
    """2-RDM sampling of a replica pair with a semistochastic core: the device
    2-RDM (spawn pairs, core pairs and the diagonal) equals the oracle's after
    every step, up to the order of the FP64 atomic sums; the walker lists stay
    bit-exact.  seg = 1: core rows summed (and their RDM pairs taken) in
    segments of one element per lane."""
    spec, eng, orc = pair(name)
    if seg is not None:
        eng.set_option(capi.OPT_CORE_SEGMENT, seg)
        orc.set_core_segment(seg)
    W, L = spec.W, spec.lenof_sign
    eng.start_from_reference(initial_part=60.0)
    for it in range(1, 11):
        eng.perform_fcimc_cyc_par(capi.default_params(tau=0.02, seed=8, iter=it))
    rows, dh, odh = eng.download()
    pop = np.abs(rows[:, W:W + L].view(np.float64)).sum(axis=1)
    core = rows[np.argsort(-pop, kind="stable")[:40], :W]
    eng.upload(rows, dh, odh)
    orc.upload(rows, dh, odh)
    eng.set_core_space(core)
    orc.set_core_space(core)
    eng.set_rdm_sampling(True)
    orc.set_rdm_sampling(True)
    eng.rdm2(reset=True)
    orc.rdm2(reset=True)
    try:
        for it in range(11, 19):
            p = capi.default_params(tau=0.02, seed=8, iter=it)
            sg = eng.perform_fcimc_cyc_par(p)
            sc, rc = orc.iterate(p)
            assert rc == 0 and sg.err == 0
            assert_same_list(spec, eng, orc, it)
            gg, gc = eng.rdm2(), orc.rdm2()
            scale = max(np.abs(gc).max(), 1.0)
            np.testing.assert_allclose(gg, gc, rtol=1e-9, atol=1e-12 * scale, err_msg=f"step {it}")
    finally:
        eng.set_rdm_sampling(False)
        orc.set_rdm_sampling(False)
