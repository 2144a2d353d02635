"""Host side of the conventional tau search: update_tau
(tau/tau_search_conventional.F90:274-499) on given class maxima."""
from __future__ import annotations

import math

import pytest

from neci_stable_gb300 import capi
from neci_stable_gb300.fcimc import TauSearch


def stats(**kw):
    t = capi.TauStats()
    for k, v in kw.items():
        setattr(t, k, v)
    return t


def test_par_bias_with_enough_samples_sets_all_three():
    ts = TauSearch(consider_par_bias=True, p_singles=0.1, p_parallel=0.5)
    t = stats(gamma_sing=4.0, gamma_par=10.0, gamma_opp=30.0, cnt_sing=51, cnt_par=51, cnt_opp=51)
    tau, ps, pp = ts.update(t, 0.01)
    pp_new = 10.0 / 40.0
    ps_new = 4.0 * pp_new / (10.0 + 4.0 * pp_new)
    assert pp == pytest.approx(pp_new, rel=0, abs=0)
    assert ps == pytest.approx(ps_new, rel=0, abs=0)
    assert tau == ps_new * 2.0 / 4.0 * 0.99999


def test_par_bias_too_few_samples_keeps_biases_and_takes_minimum():
    ts = TauSearch(consider_par_bias=True, p_singles=0.1, p_parallel=0.4)
    t = stats(gamma_sing=4.0, gamma_par=10.0, gamma_opp=30.0, cnt_sing=3, cnt_par=51, cnt_opp=7)
    tau, ps, pp = ts.update(t, 0.5)
    want = 2.0 * min(0.1 / 4.0, min(0.9 * 0.4 / 10.0, 0.9 * 0.6 / 30.0))
    assert (ps, pp) == (0.1, 0.4)
    assert tau == want * 0.99999  # smaller than the old tau: always taken


def test_too_few_samples_never_raise_tau():
    ts = TauSearch(consider_par_bias=True, p_singles=0.1, p_parallel=0.4)
    t = stats(gamma_sing=1e-3, gamma_par=1e-3, gamma_opp=1e-3, cnt_sing=3, cnt_par=3, cnt_opp=3)
    tau, _, _ = ts.update(t, 0.01)
    assert tau == 0.01


def test_death_caps_tau():
    ts = TauSearch(consider_par_bias=False, p_singles=0.2, p_parallel=0.5)
    t = stats(gamma_sing=1.0, gamma_doub=1.0, cnt_sing=51, cnt_doub=51, max_death_cpt=50.0)
    tau, ps, _ = ts.update(t, 0.01)
    assert tau == (1.0 / 50.0) * 0.99999
    assert ps == 0.5  # gamma_sing / (gamma_sing + gamma_doub)


def test_lattice_singles_only():
    ts = TauSearch(consider_par_bias=False, p_singles=0.0, p_parallel=0.5, lattice=True)
    t = stats(gamma_sing=8.0, cnt_sing=51)
    tau, ps, _ = ts.update(t, 0.001)
    assert tau == 2.0 * 1.0 / 8.0 * 0.99999 and ps == 0.0
    assert math.isfinite(tau)
