"""GPU parity tests: every kernel against the CPU oracle through the C ABI.

Integer/bit work (hashes, excitation levels, excitation generation, spawn
compression, annihilation, whole iterations) must be bit-exact; matrix
elements within 1e-12 relative (they are in fact bit-exact: the FP64
kernels are built with --fmad=false and sum in the oracle's order).
"""
from __future__ import annotations

import numpy as np
import pytest

from neci_stable_gb300 import capi
from neci_stable_gb300.engine import Engine
from oracle.oracle import Oracle

from helpers import (canonical, canonical_with, excite, hubbard10, hubbard_square, molecule, molecule_uniform,
                     random_dets, random_spawns, random_walkers)

pytestmark = pytest.mark.gpu

SYSTEMS = {
    "hub10": lambda: hubbard10(),
    "hub10x2": lambda: hubbard10(lenof_sign=2),
    "hub6x6": lambda: hubbard_square(6, 6, 36),
    "mol12": lambda: molecule(12, 6),
    "mol12x2": lambda: molecule(12, 6, lenof_sign=2),
    "mol24": lambda: molecule(24, 10),
    "mol40": lambda: molecule(40, 12),      # 80 spin orbitals: two det words
    "mol64": lambda: molecule(64, 20),      # 128 spin orbitals: three det words
    "mol12u": lambda: molecule_uniform(12, 6),   # the uniform generator (gen_rand_excit)
    "mol40u": lambda: molecule_uniform(40, 12),
    "mol32": lambda: molecule(32, 8),           # 64 spin orbitals: one orbital word in two row words
    "mol32u": lambda: molecule_uniform(32, 8),
    "mol80u": lambda: molecule_uniform(80, 10),  # 160 spin orbitals: three words
    "hub4x8": lambda: hubbard_square(4, 8, 16),
    "hub8x10": lambda: hubbard_square(8, 10, 20),
    "hub10x10": lambda: hubbard_square(10, 10, 20),  # 200 spin orbitals: four words (the any-size instance)
}

_cache = {}


def pair(name, max_walkers=200_000, max_spawned=400_000):
    key = (name, max_walkers, max_spawned)
    if key not in _cache:
        spec = SYSTEMS[name]()
        eng = Engine(spec, max_walkers, max_spawned)
        orc = Oracle(spec, max_walkers, max_spawned, hii=eng.hii)
        _cache.clear()
        _cache[key] = (spec, eng, orc)
    return _cache[key]


@pytest.mark.parametrize("name", ["hub10", "hub6x6", "mol24", "mol40", "mol64"])
def test_find_walker_hash_and_excit_level(name):
    spec, eng, orc = pair(name)
    rng = np.random.default_rng(1)
    dets = random_dets(spec, 4000, rng)
    for length in (1, 7, 1000003, 1 << 20, (1 << 31) - 1):
        assert np.array_equal(eng.find_walker_hash(dets, length), orc.find_walker_hash(dets, length))
    other = random_dets(spec, 4000, rng)
    assert np.array_equal(eng.excit_level(dets, other), orc.excit_level(dets, other))


@pytest.mark.parametrize("name", ["hub10", "hub6x6", "mol12", "mol24", "mol40", "mol64"])
def test_helement(name):
    spec, eng, orc = pair(name)
    rng = np.random.default_rng(2)
    a = random_dets(spec, 600, rng)
    b = np.array([excite(spec, d, lvl, rng) for d, lvl in zip(a, rng.integers(0, 4, size=a.shape[0]))])
    b[:50] = a[:50]
    g = eng.helement(a, b)
    c = orc.helement(a, b)
    np.testing.assert_allclose(g, c, rtol=1e-12, atol=1e-14)
    assert np.array_equal(g, c), "FP64 matrix elements are expected bit-exact"


@pytest.mark.parametrize("name", ["hub10", "hub6x6", "mol12", "mol24", "mol40", "mol64", "mol12u", "mol40u"])
def test_gen_excit(name):
    spec, eng, orc = pair(name)
    rng = np.random.default_rng(3)
    for det in random_dets(spec, 6, rng):
        for seed, it in ((7, 1), (123456789, 99)):
            cg, pg, hg = eng.gen_excit(det, 3000, seed, it)
            cc, pc, hc = orc.gen_excit(det, 3000, seed, it)
            assert np.array_equal(cg, cc)
            assert np.array_equal(pg, pc)
            assert np.array_equal(hg, hc)


@pytest.mark.parametrize("name", ["hub10", "hub10x2", "mol24"])
def test_compress_spawns(name):
    spec, eng, orc = pair(name)
    rng = np.random.default_rng(4)
    walkers = random_walkers(spec, 500, rng)
    for n in (0, 1, 17, 5000, 60000):
        sp = random_spawns(spec, walkers, n, rng)
        out_g, nann_g = eng.compress_spawns(sp)
        out_c, nann_c = orc.compress_spawns(capi.default_params(), sp)
        assert np.array_equal(out_g, out_c)
        np.testing.assert_allclose(nann_g, nann_c, rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("name", ["hub10", "hub10x2", "mol24", "mol40"])
@pytest.mark.parametrize("trunc", [1, 0])
def test_annihilate_injected(name, trunc):
    spec, eng, orc = pair(name)
    rng = np.random.default_rng(5 + trunc)
    W = spec.W
    walkers = random_walkers(spec, 3000, rng)
    # some holes in the list (zero signs) to exercise free-slot reuse
    holes = rng.random(walkers.shape[0]) < 0.1
    walkers[holes, W:W + spec.lenof_sign] = 0
    eng.upload(walkers)
    orc.upload(walkers)
    p = capi.default_params(seed=99, iter=3, t_trunc_initiator=trunc, occupied_thresh=1.0)
    sp = random_spawns(spec, walkers, 20000, rng)
    sg = eng.annihilate(p, sp)
    sc, rc = orc.annihilate(p, sp)
    assert rc == 0 and sg.err == 0
    rg, dg, og = eng.download()
    rcpu, dc, oc = orc.download()
    rg, (dg, og) = canonical_with(rg, [dg, og], W)
    rcpu, (dc, oc) = canonical_with(rcpu, [dc, oc], W)
    assert rg.shape == rcpu.shape
    # flag_removed (bit 0) bookkeeping is slot-local; compare the rest
    assert np.array_equal(rg[:, : W + spec.lenof_sign], rcpu[:, : W + spec.lenof_sign])
    assert np.array_equal(rg[:, -1] & ~1, rcpu[:, -1] & ~1)
    assert np.array_equal(dg, dc) and np.array_equal(og, oc)
    for f in ("nborn", "nannihil", "naborted", "nremoved", "tot_parts", "norm_psi_sq", "tot_parts_old"):
        np.testing.assert_allclose(getattr(sg, f)[:], getattr(sc, f)[:], rtol=1e-10, atol=1e-8, err_msg=f)
    assert sg.n_new == sc.n_new and sg.n_occupied == sc.n_occupied


def run_pair(name, iters, start_pop, tau, shift=0.0, seed=31, precision=capi.PREC_FP64, real=1, p_singles=None,
             av=1.0):
    spec, eng, orc = pair(name, 400_000, 800_000)
    if p_singles is not None:
        eng.set_excit_biases(p_singles, spec.p_parallel)
        orc.set_excit_biases(p_singles, spec.p_parallel)
    try:
        eng.start_from_reference(initial_part=start_pop)
        rows, _, _ = eng.download()
        orc.upload(rows)
        W, L = spec.W, spec.lenof_sign
        for it in range(1, iters + 1):
            p = capi.default_params(tau=tau, diag_sft=[shift, shift], seed=seed, iter=it, precision=precision,
                                    t_all_real_coeff=real, av_mc_excits=av)
            sg = eng.perform_fcimc_cyc_par(p)
            sc, rc = orc.iterate(p)
            assert rc == 0 and sg.err == 0, (it, rc, sg.err)
            rg = canonical(eng.download()[0], W)
            rcpu = canonical(orc.download()[0], W)
            assert rg.shape == rcpu.shape, (it, rg.shape, rcpu.shape)
            assert np.array_equal(rg[:, : W + L], rcpu[:, : W + L]), it
            assert np.array_equal(rg[:, -1] & ~1, rcpu[:, -1] & ~1), it
            for f in ("nborn", "ndied", "nannihil", "naborted", "nremoved", "tot_parts", "hf_cyc", "enum_cyc",
                      "tot_parts_old"):
                np.testing.assert_allclose(getattr(sg, f)[:], getattr(sc, f)[:], rtol=1e-9, atol=1e-7,
                                           err_msg=f"{f} it {it}")
            assert sg.n_attempts == sc.n_attempts and sg.n_spawned == sc.n_spawned and sg.n_new == sc.n_new
    finally:
        if p_singles is not None:
            eng.set_excit_biases(spec.p_singles, spec.p_parallel)
            orc.set_excit_biases(spec.p_singles, spec.p_parallel)
    return sg


@pytest.mark.parametrize("name,iters,pop,tau", [("hub10", 40, 50.0, 0.02), ("hub10x2", 25, 20.0, 0.02),
                                                ("hub6x6", 12, 30.0, 0.01), ("mol12", 30, 40.0, 0.02),
                                                ("mol24", 20, 200.0, 0.005), ("mol12u", 30, 40.0, 0.02),
                                                ("mol40u", 12, 100.0, 0.005)])
def test_iterations_bit_exact(name, iters, pop, tau):
    st = run_pair(name, iters, pop, tau)
    assert st.n_occupied > 1


def test_iterations_integer_walkers_and_mixed():
    run_pair("hub10", 20, 30.0, 0.02, real=0)
    run_pair("mol24", 12, 60.0, 0.01, real=0)
    run_pair("mol12", 15, 40.0, 0.02, precision=capi.PREC_MIXED)


# pSingles 0.5 takes the spawn kernel's instance that queues both classes
# (0.15 <= pSingles <= 0.85), the defaults (0.003-0.05) the one that runs
# doubles inline; the systems cover the word-count instances: one word
# (mol24), two (mol40, mol40u), three row words of which two hold orbitals
# (mol64, 128 spin orbitals)
@pytest.mark.parametrize("name,ps", [("mol24", 0.5), ("mol40", 0.5), ("mol64", 0.5), ("mol12u", 0.5),
                                     ("mol40u", 0.5), ("mol64", None), ("mol40", None)])
def test_spawn_instances_bit_exact(name, ps):
    st = run_pair(name, 12, 100.0, 0.01, p_singles=ps)
    assert st.n_spawned > 0


# The remaining word-count instances of the spawn kernel, for the molecular
# generators and the lattice one: one orbital word in two row words (64 spin
# orbitals), three words (160), and the instance for any size (200, four words)
@pytest.mark.parametrize("name,pop,tau", [("mol32", 500.0, 0.05), ("mol32u", 500.0, 0.05), ("mol80u", 500.0, 0.05),
                                          ("hub4x8", 40.0, 0.01), ("hub8x10", 40.0, 0.01), ("hub10x10", 40.0, 0.01)])
def test_word_count_instances_bit_exact(name, pop, tau):
    st = run_pair(name, 10, pop, tau)
    assert st.n_occupied > 1


def test_empty_list_and_steps_without_spawns():
    """A step on an empty walker list: no error, zero counts, an empty list.
    Steps in which nothing spawns (tau so small that every amplitude rounds
    to zero): the list still dies by the oracle's rules."""
    spec, eng, orc = pair("mol12", 400_000, 800_000)
    W, L = spec.W, spec.lenof_sign
    empty = np.zeros((0, W + L + 1), dtype=np.int64)
    eng.upload(empty)
    orc.upload(empty)
    p = capi.default_params(tau=0.01, seed=3, iter=1)
    sg = eng.perform_fcimc_cyc_par(p)
    sc, rc = orc.iterate(p)
    assert rc == 0 and sg.err == 0
    assert sg.n_attempts == 0 == sc.n_attempts and sg.n_spawned == 0 and sg.n_occupied == 0
    assert sg.tot_parts[0] == 0.0 == sc.tot_parts[0]
    assert eng.download()[0].shape[0] == 0
    eng.start_from_reference(initial_part=50.0)
    orc.upload(eng.download()[0])
    for it in range(1, 4):
        p = capi.default_params(tau=1e-12, seed=3, iter=it)
        sg = eng.perform_fcimc_cyc_par(p)
        sc, rc = orc.iterate(p)
        assert rc == 0 and sg.err == 0
        assert sg.n_attempts > 0 and sg.n_spawned == 0 == sc.n_spawned
        rg = canonical(eng.download()[0], W)
        rcpu = canonical(orc.download()[0], W)
        assert np.array_equal(rg[:, : W + L], rcpu[:, : W + L]), it


# AvMCExcits != 1: decide_num_to_spawn in FP64 (the sweep's general instance)
# and 1/AvMCExcits in the spawn amplitude
@pytest.mark.parametrize("name,av", [("mol24", 2.0), ("hub10", 0.5)])
def test_iterations_av_mc_excits(name, av):
    run_pair(name, 12, 40.0, 0.01, av=av)


def test_iterate_n_matches_single_steps():
    spec, eng, orc = pair("hub10", 100_000, 200_000)
    eng.start_from_reference(initial_part=10.0)
    p = capi.default_params(tau=0.02, seed=5, iter=1)
    a = [eng.perform_fcimc_cyc_par(capi.default_params(tau=0.02, seed=5, iter=i)) for i in range(1, 11)]
    ra = canonical(eng.download()[0], spec.W)
    eng.start_from_reference(initial_part=10.0)
    b = eng.iterate_n(p, 10)
    rb = canonical(eng.download()[0], spec.W)
    assert np.array_equal(ra, rb)
    assert [s.tot_parts[0] for s in a] == [s.tot_parts[0] for s in b]


def test_errors_are_reported_not_faulted():
    """Buffer overflows come back as NECI's err codes (no fault, context usable)."""
    spec = hubbard10()
    eng = Engine(spec, max_walkers=64, max_spawned=32)
    eng.start_from_reference(initial_part=500.0)
    with pytest.raises(capi.NeciGpuError) as ei:
        for it in range(1, 20):
            eng.perform_fcimc_cyc_par(capi.default_params(tau=0.05, seed=1, iter=it))
    assert ei.value.code in (capi.ERR_SPAWN_FULL, capi.ERR_LIST_FULL)
    # the context still works after the error
    eng.start_from_reference(initial_part=1.0)
    st = eng.perform_fcimc_cyc_par(capi.default_params(tau=0.001, seed=1, iter=1))
    assert st.err == 0


def test_list_overflow_inside_a_batch_halts_the_batch():
    """CurrentDets overflowing in the middle of a batch of graph-launched
    steps: the step reports NECI_GPU_ERR_LIST_FULL, the steps after it in the
    batch do nothing (no slot beyond the allocation is touched), and an
    upload makes the context usable again."""
    spec = hubbard10()
    eng = Engine(spec, max_walkers=4096, max_spawned=1 << 20)
    eng.start_from_reference(initial_part=3000.0)
    with pytest.raises(capi.NeciGpuError) as ei:
        eng.iterate_n(capi.default_params(tau=0.05, seed=2, iter=1), 20)
    assert ei.value.code == capi.ERR_LIST_FULL
    eng.start_from_reference(initial_part=5.0)
    st = eng.iterate_n(capi.default_params(tau=0.01, seed=2, iter=1), 5)
    assert all(s.err == 0 for s in st) and st[-1].tot_walkers <= 4096


def test_batched_steps_equal_single_steps():
    """neci_gpu_iterate_batch changes only concurrency: every instance ends
    with the walker list it has when stepped alone."""
    from neci_stable_gb300.engine import iterate_batch
    from neci_stable_gb300 import systems
    d = np.load(__import__("pathlib").Path(__file__).parent / "golden" / "hehe_fcidump.npz")
    specs = [hubbard10(), hubbard10(lenof_sign=2), molecule(12, 6),
             systems.molecular_system(d["h"], d["eri"], float(d["ecore"]), int(d["nelec"]))]
    pops = [40.0, 25.0, 60.0, 30.0]

    def fresh():
        engs = []
        for sp, pop in zip(specs, pops):
            e = Engine(sp, 200_000, 400_000)
            e.start_from_reference(initial_part=pop)
            engs.append(e)
        return engs

    params = [capi.default_params(tau=0.01 + 0.005 * i, seed=50 + i, iter=1) for i in range(len(specs))]
    batch = fresh()
    st, ms = iterate_batch(batch, params, 12)
    assert ms > 0.0 and all(len(s) == 12 for s in st)
    single = fresh()
    for e, p in zip(single, params):
        e.iterate_n(p, 12)
    for a, b, sp in zip(batch, single, specs):
        assert np.array_equal(canonical(a.download()[0], sp.W), canonical(b.download()[0], sp.W))


@pytest.mark.parametrize("name,iters,pop,tau,precision", [
    ("hub10", 15, 50.0, 0.02, capi.PREC_FP64), ("mol24", 12, 200.0, 0.005, capi.PREC_FP64),
    ("mol24", 10, 200.0, 0.005, capi.PREC_MIXED), ("mol12u", 15, 40.0, 0.02, capi.PREC_FP64)])
def test_tau_search_log_bit_exact(name, iters, pop, tau, precision):
    """log_spawn_magnitude / log_death_magnitude: the class maxima of gamma
    and max_death_cpt match the oracle bit for bit after every step, and a
    change of pSingles/pParallel (update_tau's new biases) mid-run keeps the
    walker lists identical."""
    spec, eng, orc = pair(name, 400_000, 800_000)
    eng.set_tau_search(True)
    orc.set_tau_search(True)
    eng.tau_stats(reset=True)
    orc.tau_stats(reset=True)
    try:
        eng.start_from_reference(initial_part=pop)
        orc.upload(eng.download()[0])
        W, L = spec.W, spec.lenof_sign
        for it in range(1, iters + 1):
            if it == iters // 2 and spec.kind == capi.SYS_MOLECULAR:
                ps = 0.05 if spec.generator == capi.EXGEN_PCHB else 0.2
                eng.set_excit_biases(ps, 0.3)
                orc.set_excit_biases(ps, 0.3)
            p = capi.default_params(tau=tau, diag_sft=[-0.5, -0.5], seed=77, iter=it, precision=precision)
            sg = eng.perform_fcimc_cyc_par(p)
            sc, rc = orc.iterate(p)
            assert rc == 0 and sg.err == 0
            tg, tc = eng.tau_stats().as_dict(), orc.tau_stats().as_dict()
            assert tg == tc, (it, tg, tc)
            rg = canonical(eng.download()[0], W)
            rcpu = canonical(orc.download()[0], W)
            assert np.array_equal(rg[:, : W + L], rcpu[:, : W + L]), it
        t = eng.tau_stats(reset=True)
        assert t.max_death_cpt > 0.0
        if spec.kind == capi.SYS_HUBBARD_REAL_SPACE:
            assert t.gamma_sing > 0.0 and t.gamma_doub == 0.0 and t.cnt_sing == 51
        elif spec.generator == capi.EXGEN_PCHB:
            assert t.gamma_par > 0.0 and t.gamma_opp > 0.0 and t.cnt_opp == 51
        else:
            assert t.gamma_doub > 0.0 and t.cnt_doub == 51
        z = eng.tau_stats()
        assert z.gamma_sing == 0.0 and z.max_death_cpt == 0.0 and z.cnt_opp == 0
    finally:
        eng.set_tau_search(False)
        orc.set_tau_search(False)
        if spec.kind == capi.SYS_MOLECULAR:
            eng.set_excit_biases(spec.p_singles, spec.p_parallel)
            orc.set_excit_biases(spec.p_singles, spec.p_parallel)


def test_tau_search_run_settles_tau():
    """A run with the conventional tau search (FciMCPar + update_tau on the
    device's logs) moves tau to the bloom limit and stops searching when the
    shift starts to vary."""
    from neci_stable_gb300.fcimc import CalcParams, FciMCPar
    spec = molecule(24, 10)
    eng = Engine(spec, 400_000, 800_000)
    eng.start_from_reference(initial_part=20.0)
    drv = FciMCPar(eng, CalcParams(tau=0.05, target_walkers=3000, steps_sft=10, sft_damp=0.1, seed=5,
                                   tau_search=True))
    res = drv.run(400)
    assert res.tau[0] < 0.05 and all(t > 0 for t in res.tau)
    assert drv.tau_search is None, "the search ends once the shift varies"
    t_final = res.tau[-1]
    assert drv.calc.tau == t_final


def test_popsfile_restart_on_the_engine(tmp_path):
    """Download -> binary POPSFILE -> read -> upload into a fresh context:
    the restarted run continues bit for bit like the uninterrupted one."""
    from neci_stable_gb300 import popsfile
    spec = molecule(24, 10)
    W, L = spec.W, spec.lenof_sign

    def fresh():
        e = Engine(spec, 200_000, 400_000)
        e.start_from_reference(initial_part=300.0)
        return e

    par = lambda it: capi.default_params(tau=0.005, seed=11, iter=it)  # noqa: E731
    a = fresh()
    for it in range(1, 11):
        a.perform_fcimc_cyc_par(par(it))
    rows, dh, odh = a.download()
    hdr = popsfile.PopsHeader(nel=spec.nel, lenof_sign=L, nifd=spec.nifd, cyc=10, tau=0.005,
                              p_singles=spec.p_singles, p_parallel=spec.p_parallel,
                              p_doubles=1.0 - spec.p_singles, random_hash=list(map(int, spec.random_hash2)))
    popsfile.write_popsfile(tmp_path / "POPSFILE", hdr, rows, binary=True)
    h, back = popsfile.read_popsfile(tmp_path / "POPSFILE")
    assert back.shape[0] == rows.shape[0] == h.totwalk
    b = Engine(spec, 200_000, 400_000)
    b.upload(back)  # diagonal and reference elements recomputed on the device
    assert np.array_equal(canonical_with(b.download()[0], [b.download()[1]], W)[1][0],
                          canonical_with(rows, [dh], W)[1][0])
    for it in range(11, 21):
        sa = a.perform_fcimc_cyc_par(par(it))
        sb = b.perform_fcimc_cyc_par(par(it))
        # TotParts is a reduction over slots, and the restart compacts the
        # slots: equal up to the order of the FP64 sum
        assert abs(sa.tot_parts[0] - sb.tot_parts[0]) <= 1e-12 * sa.tot_parts[0], it
        assert sa.n_occupied == sb.n_occupied and sa.n_spawned == sb.n_spawned, it
    ra, rb = canonical(a.download()[0], W), canonical(b.download()[0], W)
    assert np.array_equal(ra[:, :W + L], rb[:, :W + L])


@pytest.mark.parametrize("name", ["mol24", "hub10x2"])
def test_compaction_keeps_the_run_identical(name):
    """A list that is mostly holes is compacted at the start of the next step
    (occupied rows move into the holes below the kept count, TotWalkers
    shrinks, the walker hash is rebuilt); the walker lists stay identical to
    the oracle's, which never compacts."""
    spec, eng, orc = pair(name, 400_000, 800_000)
    rng = np.random.default_rng(21)
    W, L = spec.W, spec.lenof_sign
    rows = random_walkers(spec, 12000, rng)
    holes = rng.random(rows.shape[0]) < 0.7
    rows[holes, W:W + L] = 0
    eng.upload(rows)
    orc.upload(rows)
    p = lambda it: capi.default_params(tau=0.005, seed=4, iter=it)  # noqa: E731
    tw = []
    for it in range(1, 7):
        sg = eng.perform_fcimc_cyc_par(p(it))
        sc, rc = orc.iterate(p(it))
        assert rc == 0 and sg.err == 0
        tw.append(sg.tot_walkers)
        rg, rcpu = canonical(eng.download()[0], W), canonical(orc.download()[0], W)
        assert np.array_equal(rg[:, :W + L], rcpu[:, :W + L]), it
        assert np.array_equal(rg[:, -1] & ~1, rcpu[:, -1] & ~1), it
        np.testing.assert_allclose(sg.tot_parts[:L], sc.tot_parts[:L], rtol=1e-12)
    # TotWalkers never decreases without a compaction: the second step ran
    # on the compacted list (about 30% of the slots, then its new
    # determinants appended)
    assert tw[1] < tw[0], tw
    assert sc.tot_walkers >= rows.shape[0]   # the oracle keeps its holes


@pytest.mark.parametrize("name,pop,tau", [("hub10x2", 40.0, 0.02), ("mol12x2", 60.0, 0.02)])
def test_rdm_sampling_matches_oracle(name, pop, tau):
    """The device 2-RDM (spawn-pair and diagonal terms) equals the oracle's
    after every step, up to the order of the FP64 atomic sums; the walker
    lists stay bit-exact with sampling on."""
    spec, eng, orc = pair(name, 400_000, 800_000)
    W, L = spec.W, spec.lenof_sign
    eng.start_from_reference(initial_part=pop)
    orc.upload(eng.download()[0])
    eng.set_rdm_sampling(True)
    orc.set_rdm_sampling(True)
    eng.rdm2(reset=True)
    orc.rdm2(reset=True)
    try:
        for it in range(1, 13):
            p = capi.default_params(tau=tau, diag_sft=[0.0, 0.0], seed=8, iter=it)
            sg = eng.perform_fcimc_cyc_par(p)
            sc, rc = orc.iterate(p)
            assert rc == 0 and sg.err == 0
            rg, rcpu = canonical(eng.download()[0], W), canonical(orc.download()[0], W)
            assert np.array_equal(rg[:, :W + L], rcpu[:, :W + L]), it
            gg, gc = eng.rdm2(), orc.rdm2()
            scale = max(np.abs(gc).max(), 1.0)
            np.testing.assert_allclose(gg, gc, rtol=1e-9, atol=1e-12 * scale, err_msg=f"step {it}")
        assert np.count_nonzero(gc - np.diag(np.diag(gc))) > 0, "no off-diagonal terms were sampled"
    finally:
        eng.set_rdm_sampling(False)
        orc.set_rdm_sampling(False)
