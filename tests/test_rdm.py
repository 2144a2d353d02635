"""The stochastic 2-RDM of a replica pair: the host's normalisation and RDM
energy are pinned by the exact 2-RDM of an exact-diagonalisation vector
(built by applying creation/annihilation operators), and the CPU oracle's
estimator reproduces the exact energy within its statistical error."""
from __future__ import annotations

import numpy as np
import pytest

from neci_stable_gb300 import capi, rdm
from oracle import second_quant
from oracle.oracle import Oracle, exact_ground_state

from helpers import molecule


def exact_rdm(spec):
    orc = Oracle(spec, 50_000, 100_000)
    na = sum(1 for o in spec.reference if o % 2 == 0)
    e, dets, vec = exact_ground_state(orc, na, spec.nel - na)
    ints = [int(np.uint64(d[0])) for d in dets]
    return e, second_quant.rdm2_from_vector(ints, vec, spec.nbasis)


def test_rdm_energy_of_the_exact_state_is_the_exact_energy():
    spec = molecule(6, 4)
    e, G = exact_rdm(spec)
    out = rdm.rdm_energy(G, spec)
    assert abs(out["norm"] - 1.0) < 1e-10
    assert abs(out["energy"] - e) < 1e-10, (out, e)
    # Hermitian and with the right trace
    assert np.allclose(G, G.T, atol=1e-12)


def test_oracle_estimator_matches_exact_energy():
    """A replica-pair run of the CPU restatement with 2-RDM sampling: the RDM
    energy from the accumulated matrix agrees with exact diagonalisation."""
    from neci_stable_gb300.systems import encode_det, make_rows
    spec = molecule(6, 4, lenof_sign=2)
    e_exact, _ = exact_rdm(molecule(6, 4))
    orc = Oracle(spec, 100_000, 200_000)
    ref = encode_det(spec.reference, spec.nifd)
    orc.upload(make_rows(ref[None], np.array([[200.0, 200.0]]), np.array([(1 << 13) | (1 << 14)])))
    shift = [0.0, 0.0]
    old = [200.0, 200.0]
    it = 0
    for cyc in range(60):   # equilibrate: shift following each replica
        for _ in range(10):
            it += 1
            st, rc = orc.iterate(capi.default_params(tau=0.02, seed=3, iter=it, diag_sft=shift))
        for k in range(2):
            if cyc >= 5:
                shift[k] -= 0.1 * np.log(st.tot_parts[k] / old[k]) / (0.02 * 10)
            old[k] = st.tot_parts[k]
    orc.set_rdm_sampling(True)
    energies = []
    for block in range(8):
        for _ in range(100):
            it += 1
            st, rc = orc.iterate(capi.default_params(tau=0.02, seed=3, iter=it, diag_sft=shift))
            assert rc == 0
        energies.append(rdm.rdm_energy(orc.rdm2(reset=True), spec)["energy"])
    e = np.mean(energies)
    err = np.std(energies, ddof=1) / np.sqrt(len(energies))
    assert abs(e - e_exact) < max(4 * err, 2e-3), (e, err, e_exact, energies)
