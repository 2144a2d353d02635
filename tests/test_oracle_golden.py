"""CPU tests that pin the oracle to the reference's own known answers.

* CountBits([1234, 5678]) = 12 (unit_tests/det_bit_ops/test_countbits.F90:56-61)
* real-space Hubbard cumulative lists and generation probabilities
  (unit_tests/real_space_hubbard/test_real_space_hubbard.F90:1673-1891)
* Slater-Condon rules against an independent second-quantised Hamiltonian
  (the consistency unit_tests/sltcnd/test_sltcnd.F90 checks)
* exact diagonalisation of the reference's HeHe test input reproduces the
  Davidson "GROUND E" NECI recorded for it
* Philox-4x32-10 against the published known-answer vectors
* alias tables reproduce their target distribution
  (unit_tests/sampler/test_aliasTables.F90)
* the PCHB and uniform (gen_rand_excit) generators: sampled frequencies
  match p_gen and p_gen matches the exact get_pgen restatement
  (unit_tests/excitgen/pchb_excitgen_test_helper.F90, tolerance 0.15)
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from neci_stable_gb300 import capi, systems
from neci_stable_gb300.systems import encode_det
from oracle import oracle as orc
from oracle import second_quant as sq

from helpers import hubbard10, molecule

GOLDEN = Path(__file__).parent / "golden"


def tiny_lattice_oracle(nsites, nel, neighbours, tmat):
    spec = systems.SystemSpec(kind=capi.SYS_HUBBARD_REAL_SPACE, nel=nel, nbasis=2 * nsites,
                              tmat=np.ascontiguousarray(tmat.T), reference=list(range(1, nel + 1)),
                              random_hash2=systems.random_hash2(2 * nsites, 1), neighbours=neighbours, uhub=0.0,
                              bhub=1.0)
    return orc.Oracle(spec, 64, 64, hii=0.0)


def test_countbits_known_answer():
    spec = molecule(40, 12)  # 80 spin orbitals: two det words
    o = orc.Oracle(spec, 16, 16, pchb=False)
    a = np.array([[1234, 5678]], dtype=np.int64)
    z = np.zeros_like(a)
    assert o.excit_level(a, z)[0] == 12


def test_create_cum_list_rs_hubbard_known_answers():
    nb = np.zeros((5, 1), dtype=np.int32)
    o = tiny_lattice_oracle(5, 2, nb, np.ones((10, 10)))
    ilut = encode_det([1, 2], 0)
    cases = [([1, 2], 1, [3, 5, 7, 9], [1, 2, 3, 4], 4), ([1, 2], 2, [4, 6, 8, 10], [1, 2, 3, 4], 4),
             ([1, 2], 2, [4, 6, 8], [1, 2, 3], 3), ([1, 2], 1, [1, 3, 5], [0, 1, 2], 2),
             ([1, 2], 2, [4, 2, 6], [1, 1, 2], 2), ([1, 3], 1, [9, 3, 5, 1], [1, 1, 2, 2], 2)]
    for occ, src, neigh, cum_ref, sum_ref in cases:
        cum, s = orc.cum_list_rs_hubbard(o, encode_det(occ, 0), src, neigh)
        assert list(cum) == cum_ref and s == sum_ref
    assert ilut is not None


def test_calc_pgen_rs_hubbard_known_answers():
    nb = systems.chain_neighbours(4)
    tmat = np.zeros((8, 8))
    for s in range(1, 5):
        for n in nb[s - 1]:
            for spin in (1, 0):
                tmat[2 * s - spin - 1, 2 * n - spin - 1] = 1.0
    o = tiny_lattice_oracle(4, 2, nb, tmat)
    ilut = encode_det([1, 2], 0)
    for ic in (2, 0, -1, 3):
        assert orc.calc_pgen_rs_hubbard(o, ilut, 1, 3, ic) == 0.0
    assert orc.calc_pgen_rs_hubbard(o, ilut, 1, 3, 1) == 0.25
    assert orc.calc_pgen_rs_hubbard(o, ilut, 2, 8, 1) == 0.25
    o3 = tiny_lattice_oracle(4, 3, nb, tmat)
    assert abs(orc.calc_pgen_rs_hubbard(o3, encode_det([1, 2, 3], 0), 1, 7, 1) - 1.0 / 3.0) < 1e-15


@pytest.mark.parametrize("kind", ["molecular", "hubbard"])
def test_slater_condon_matches_second_quantisation(kind):
    if kind == "molecular":
        h, eri, ecore = systems.synthetic_fcidump(5, 3)
        spec = systems.molecular_system(h, eri, 0.25, 4)
        o = orc.Oracle(spec, 16, 16, pchb=False)
        dets = orc.all_determinants(spec.nbasis, 2, 2, spec.nifd)
        H = sq.hamiltonian([int(d[0]) for d in dets], spec.nbasis, np.asarray(spec.tmat).T, eri=eri, ecore=0.25)
    else:
        spec = systems.hubbard_system("chain", (4,), 4, u=3.0)
        o = orc.Oracle(spec, 16, 16)
        dets = orc.all_determinants(spec.nbasis, 2, 2, spec.nifd)
        H = sq.hamiltonian([int(d[0]) for d in dets], spec.nbasis, np.asarray(spec.tmat).T, uhub=3.0)
    n = dets.shape[0]
    a = np.repeat(dets, n, axis=0)
    b = np.tile(dets, (n, 1))
    Ho = o.helement(a, b).reshape(n, n)
    np.testing.assert_allclose(Ho, H.T, rtol=1e-12, atol=1e-13)


def test_hehe_exact_diagonalisation_reproduces_neci_davidson():
    d = np.load(GOLDEN / "hehe_fcidump.npz")
    spec = systems.molecular_system(d["h"], d["eri"], float(d["ecore"]), int(d["nelec"]))
    o = orc.Oracle(spec, 16, 16, pchb=False)
    e0 = orc.exact_ground_state(o, 2, 2)[0]
    assert abs(e0 - float(d["ground_e"][0])) < 5e-10  # NECI prints 10 decimals


def test_ne_frozen_core_reproduces_neci_set_up():
    """NECI's Ne PCHB run ('freeze 2 0') printed the core energy after
    freezing and <D0|H|D0>; the frozen-core fold and the Fock-ordered
    reference reproduce both, and the reference NECI printed
    ((1,2,15,16,21,22,31,32) after freezing)."""
    from helpers import ne_frozen_system
    spec, d = ne_frozen_system()
    assert spec.reference == [1, 2, 15, 16, 21, 22, 31, 32]
    assert abs(spec.ecore - float(d["ecore_frozen"][0])) < 1e-10
    o = orc.Oracle(spec, 16, 16, pchb=False)
    d0 = o.helement(o.ilut_ref[None], o.ilut_ref[None])[0]
    assert abs(d0 - float(d["d0_energy"][0])) < 1e-10


def test_philox_known_answer_vectors():
    lib = orc.lib()
    kat = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
           ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
           ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
            (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, out in kat:
        c = np.array(ctr, dtype=np.uint32)
        k = np.array(key, dtype=np.uint32)
        o = np.zeros(4, dtype=np.uint32)
        lib.orc_philox_block(c.ctypes.data_as(C.c_void_p), k.ctypes.data_as(C.c_void_p), o.ctypes.data_as(C.c_void_p))
        assert tuple(int(x) for x in o) == out


def test_alias_table_reproduces_distribution():
    rng = np.random.default_rng(5)
    for n in (1, 2, 7, 300):
        w = rng.random(n) ** 3
        w[rng.random(n) < 0.2] = 0.0
        if w.sum() == 0:
            w[0] = 1.0
        bias, alias = orc.init_alias(w)
        p = bias / n
        for i in range(n):
            p[alias[i] - 1] += (1.0 - bias[i]) / n
        np.testing.assert_allclose(p, w / w.sum(), rtol=1e-10, atol=1e-14)


@pytest.mark.parametrize("which", ["pchb", "uniform", "hubbard"])
def test_generator_pgen_diagnostic(which):
    """Draws from one determinant: every draw's p_gen equals the exact
    get_pgen restatement, and frequency / p_gen is 1 within 0.15 for
    determinants drawn often enough.  The uniform generator reaches every
    single and double of the determinant, so its p_gen sum to 1."""
    if which in ("pchb", "uniform"):
        h, eri, ecore = systems.synthetic_fcidump(8, 11)
        gen = capi.EXGEN_PCHB if which == "pchb" else capi.EXGEN_UNIFORM
        spec = systems.molecular_system(h, eri, ecore, 4, seed=12, excitgen=gen)
        o = orc.Oracle(spec, 16, 16)
        det = encode_det([1, 4, 5, 10], spec.nifd)
    else:
        spec = hubbard10()
        o = orc.Oracle(spec, 16, 16)
        det = o.ilut_ref.copy()
    n = 400_000
    child, pgen, hel = o.gen_excit(det, n, 21, 1)
    ok = pgen > 0
    keys, inv, counts = np.unique(child[ok], axis=0, return_inverse=True, return_counts=True)
    pg = np.zeros(len(keys))
    pg[inv.ravel()] = pgen[ok]
    exact = np.array([o.calc_pgen(det, k) for k in keys])
    np.testing.assert_array_equal(pg, exact)
    big = counts > 2000
    ratio = counts[big] / n / pg[big]
    assert np.all(np.abs(ratio - 1.0) < 0.15), ratio
    if which == "uniform":
        assert len(keys) == 2 * 6 + 2 * 6 + 15 + 15 + 4 * 36  # singles + aa + bb + ab doubles
        assert abs(pg.sum() - 1.0) < 1e-12
    # hel of each draw equals the Slater-Condon element between the two
    hk = np.zeros(len(keys))
    hk[inv.ravel()] = hel[ok]
    np.testing.assert_array_equal(hk, o.helement(np.repeat(det[None], len(keys), axis=0), keys))


def test_blocking_analysis_recovers_error_of_correlated_series():
    from neci_stable_gb300 import analysis
    rng = np.random.default_rng(3)
    x = np.zeros(2 ** 14)
    a = 0.9
    for i in range(1, x.size):
        x[i] = a * x[i - 1] + rng.normal()
    mean, err, corr = analysis.automatic_reblocking(x)
    true_err = np.sqrt(1.0 / (1 - a) ** 2 / x.size)  # AR(1): sigma^2/(1-a)^2 per sample
    assert 0.5 * true_err < err < 2.0 * true_err
    assert corr > 1
