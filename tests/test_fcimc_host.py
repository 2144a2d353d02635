"""CPU checks of the host loop around the engine (``fcimc.FciMCPar``): the
single-particle phase, the jump of the shift to E_proj, the shift damping and
the conventional tau search's stop rule of update_shift
(fcimc_iter_utilities.F90:1027-1160) and end_of_search_reached
(tau/tau_main.F90:141-171).  A fake engine returns scripted iteration
statistics, so no device is involved."""
from __future__ import annotations

import math
from types import SimpleNamespace

import pytest

from neci_stable_gb300 import capi
from neci_stable_gb300.fcimc import CalcParams, FciMCPar


class FakeEngine:
    """Returns, for cycle k, StepsSft records whose population runs from
    cycles[k][0] to cycles[k][1]; E_proj numerator/denominator per step are
    `enum` and `hf`."""

    def __init__(self, cycles, enum=-2.0, hf=4.0, L=1, spec=None, tau_stats=None):
        self.cycles = list(cycles)
        self.enum, self.hf, self.L, self.hii = enum, hf, L, -1.0
        self.spec = spec
        self._tau_stats = tau_stats
        self.calls = []          # (diag_sft[0], tau, iter) of each iterate_n call
        self.tau_search_on = []
        self.biases = []

    def iterate_n(self, params, n):
        k = len(self.calls)
        self.calls.append((params.diag_sft[0], params.tau, params.iter))
        a, b = self.cycles[k]
        out = []
        for i in range(n):
            s = capi.IterStats()
            for r in range(self.L):
                s.tot_parts_old[r] = a + (b - a) * i / n
                s.tot_parts[r] = a + (b - a) * (i + 1) / n
            s.enum_cyc[0], s.hf_cyc[0] = self.enum, self.hf
            out.append(s)
        return out

    def set_tau_search(self, on):
        self.tau_search_on.append(bool(on))

    def tau_stats(self, reset=False):
        return self._tau_stats

    def set_excit_biases(self, ps, pp):
        self.biases.append((ps, pp))


def _calc(**kw):
    base = dict(tau=0.01, target_walkers=100, steps_sft=10, sft_damp=0.1, input_diag_sft=0.0)
    base.update(kw)
    return CalcParams(**base)


def test_shift_held_then_jumps_to_proje_then_damps():
    eng = FakeEngine([(1, 50), (50, 150), (150, 165), (165, 165), (165, 150)])
    loop = FciMCPar(eng, _calc())
    res = loop.run(50)
    proje = (10 * -2.0) / (10 * 4.0)
    damp = 0.1 / (0.01 * 10)
    s2 = proje                                # the exit cycle jumps and defers the damping
    s3 = s2 - math.log(165 / 150) * damp
    s4 = s3 - math.log(165 / 165) * damp
    s5 = s4 - math.log(150 / 165) * damp
    # the shift each cycle ran with, and the one it left
    assert [c[0] for c in eng.calls] == pytest.approx([0.0, 0.0, s2, s3, s4], abs=1e-15)
    assert res.shift == pytest.approx([0.0, s2, s3, s4, s5], abs=1e-15)
    assert res.vary_shift_cycle == 1
    # Iter advances by StepsSft per cycle
    assert [c[2] for c in eng.calls] == [1, 11, 21, 31, 41]
    assert res.proje_num == [-20.0] * 5 and res.proje_den == [40.0] * 5
    assert res.tot_parts == [50, 150, 165, 165, 150]


def test_without_jump_shift_the_exit_cycle_damps():
    eng = FakeEngine([(1, 50), (50, 150), (150, 150)])
    res = FciMCPar(eng, _calc(jump_shift=False, input_diag_sft=0.25)).run(30)
    damp = 0.1 / (0.01 * 10)
    s2 = 0.25 - math.log(150 / 50) * damp
    assert res.shift == pytest.approx([0.25, s2, s2], abs=1e-15)


def test_population_at_the_target_stays_in_the_single_particle_phase():
    # the exit needs TotParts > InitWalkers, strictly
    eng = FakeEngine([(1, 100), (100, 100)])
    res = FciMCPar(eng, _calc()).run(20)
    assert res.vary_shift_cycle is None
    assert res.shift == [0.0, 0.0]


def test_walker_updates_count_the_population_before_each_step():
    eng = FakeEngine([(10, 20)])
    res = FciMCPar(eng, _calc()).run(10)
    assert res.walker_updates == pytest.approx(sum(10 + i for i in range(10)))


def test_zero_growth_stops_the_run():
    eng = FakeEngine([(1, 150), (150, 0)])
    with pytest.raises(RuntimeError, match="growth rate is zero"):
        FciMCPar(eng, _calc(jump_shift=False)).run(20)


def test_replica_runs_leave_the_phase_separately():
    class TwoRuns(FakeEngine):
        def iterate_n(self, params, n):
            out = super().iterate_n(params, n)
            # run 2 stays small for the first two cycles
            for s in out:
                if len(self.calls) <= 2:
                    s.tot_parts_old[1] = s.tot_parts[1] = 10.0
            return out

    eng = TwoRuns([(1, 150), (150, 150), (150, 165)], L=2)
    loop = FciMCPar(eng, _calc())
    loop.run(30)
    assert loop.single_part_phase == [False, False]
    # run 1 jumped on cycle 0; run 2 jumped on cycle 2 (from 10 to 165)
    assert loop.diag_sft[1] == pytest.approx(-0.5)
    assert loop.diag_sft[0] == pytest.approx(-0.5 - math.log(165 / 150) * 0.1 / 0.1)


def test_tau_search_updates_until_the_shift_varies():
    spec = SimpleNamespace(generator=capi.EXGEN_UNIFORM, kind=capi.SYS_MOLECULAR, p_singles=0.1, p_parallel=0.3)
    t = capi.TauStats()
    t.gamma_sing, t.gamma_doub, t.cnt_sing, t.cnt_doub = 2.0, 8.0, 100, 100
    eng = FakeEngine([(1, 50), (50, 150), (150, 150)], spec=spec, tau_stats=t)
    c = _calc(tau_search=True, tau=0.5)
    res = FciMCPar(eng, c).run(30)
    # update_tau with enough samples of both classes: tau = MaxWalkerBloom / (gamma_s + gamma_d),
    # pSingles = gamma_s / (gamma_s + gamma_d), applied once while the phase lasts
    tau_new = 2.0 / 10.0 * 0.99999
    assert res.tau == pytest.approx([tau_new, tau_new])  # the cycle that ends the search logs too
    assert eng.biases == [(0.2, 0.3)]
    assert [c[1] for c in eng.calls] == pytest.approx([0.5, tau_new, tau_new])
    # the search switched on at start and off on the cycle the shift began to vary
    assert eng.tau_search_on == [True, False]
