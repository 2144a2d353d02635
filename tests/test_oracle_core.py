"""The oracle's semistochastic step pinned to plain linear algebra, on the CPU.

With every determinant of the Sz sector in the core space, an iteration has no
stochastic part: spawns between core determinants are not made
(the core-to-core block is applied exactly by determ_projection,
semi_stoch_procs.F90:105-241), core determinants skip walker_death, and
deterministic_annihilation (Annihilation.F90:930-963) adds
    y = tau * ( -(H - Hii) C + S C )
to the signs.  The oracle's iteration must therefore equal that dense
matrix-vector step, and its E_proj sums those of the signs before the step
(SumEContrib, fcimc_helper.F90:518-800).  The engine is checked against the
oracle bit for bit in the GPU tests; this pins the oracle's core path to an
independent computation."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from neci_stable_gb300 import capi, systems
from oracle.oracle import Oracle, all_determinants


def _hubbard6():
    return systems.hubbard_system("chain", (6,), 6, u=4.0), 3, 3


def _hehe():
    d = np.load(Path(__file__).parent / "golden" / "hehe_fcidump.npz")
    spec = systems.molecular_system(d["h"], d["eri"], float(d["ecore"]), int(d["nelec"]), name="HeHe")
    return spec, 2, 2


@pytest.mark.parametrize("make", [_hubbard6, _hehe], ids=["hubbard-chain-6", "HeHe"])
def test_full_core_step_is_the_dense_projection(make):
    spec, na, nb = make()
    orc = Oracle(spec, 8192, 16384)
    W, L = spec.W, spec.lenof_sign
    dets = all_determinants(spec.nbasis, na, nb, spec.nifd)
    n = dets.shape[0]
    rng = np.random.default_rng(5)
    c = np.round(rng.normal(0.0, 4.0, n), 3)
    c = np.where(c >= 0, c + 0.5, c - 0.5)          # every core determinant occupied
    ref = np.all(dets == orc.ilut_ref[None], axis=1)
    i_ref = int(np.argmax(ref))
    c[i_ref] = 50.0
    rows = np.zeros((n, W + L + 1), dtype=np.int64)
    rows[:, :W] = dets
    rows[:, W] = c.view(np.int64)
    orc.upload(rows)
    orc.set_core_space(dets)

    H = orc.hamiltonian(dets).toarray()
    H = 0.5 * (H + H.T)
    assert orc.core_nnz() == np.count_nonzero(H - np.diag(np.diag(H)))

    tau, shift = 0.01, -0.3
    p = capi.default_params(tau=tau, seed=3, iter=1, diag_sft=[shift])
    st, rc = orc.iterate(p)
    assert rc == 0
    assert st.n_spawned == 0 and st.n_core == n

    out = orc.download()[0]
    got = {tuple(r[:W]): r[W:W + 1].view(np.float64)[0] for r in out}
    c_new = np.array([got[tuple(d)] for d in dets])
    expect = c - tau * ((H - orc.hii * np.eye(n)) @ c - shift * c)
    np.testing.assert_allclose(c_new, expect, rtol=1e-12, atol=1e-12)

    enum = sum(H[i_ref, j] * c[j] for j in range(n) if j != i_ref)
    assert st.hf_cyc[0] == c[i_ref]
    assert st.enum_cyc[0] == pytest.approx(enum, rel=1e-12, abs=1e-12)
    assert st.tot_parts_old[0] == pytest.approx(np.abs(c).sum(), rel=1e-14)
    assert st.tot_parts[0] == pytest.approx(np.abs(expect).sum(), rel=1e-12)


def test_upload_refuses_a_determinant_without_nel_electrons():
    # a 4-site chain cannot hold a Neel reference of 8 electrons: the row has 4
    spec = systems.hubbard_system("chain", (4,), 8, u=4.0)
    W = spec.W
    orc = Oracle(spec, 64, 64)
    rows = np.zeros((1, W + 2), dtype=np.int64)
    rows[0, :W] = systems.encode_det(list(range(1, 5)), spec.nifd)
    rows[0, W] = np.array([10.0]).view(np.int64)[0]
    with pytest.raises(RuntimeError, match="does not hold nel electrons"):
        orc.upload(rows)
    rows[0, :W] = systems.encode_det(list(range(1, 9)), spec.nifd)
    orc.upload(rows)
