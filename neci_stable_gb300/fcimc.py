"""Host-side driver around the engine: NECI's FciMCPar main loop.

``FciMCPar.run`` restates the part of FciMCPar (FciMCPar.F90:176-854) that
surrounds PerformFCIMCycPar: the per-iteration call, the accumulation of the
projected-energy numerator and denominator over StepsSft iterations, and the
shift update of update_shift (fcimc_iter_utilities.F90:883-1260):

* single-particle phase: the shift stays at its input value until TotParts
  exceeds the target walker number (:1057-1101);
* afterwards, every StepsSft iterations,
  DiagSft <- DiagSft - SftDamp * ln(AllGrowRate) / (tau * StepsSft)
  with AllGrowRate = TotParts / TotParts of the previous update (:1153-1160).

E_proj and the shift are reported with the blocking analysis of
ErrorAnalysis.F90 (see analysis.py).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import analysis, capi
from .engine import Engine


@dataclass
class CalcParams:
    tau: float = 0.01
    target_walkers: float = 1e4          # TOTALWALKERS
    steps_sft: int = 10                  # StepsSft
    sft_damp: float = 0.1                # SftDamp
    initial_part: float = 1.0            # InitialPart
    input_diag_sft: float = 0.0          # InputDiagSft
    seed: int = 12345
    precision: int = capi.PREC_FP64
    all_real_coeff: bool = True
    real_spawn_cutoff: float = 0.95
    initiator_walk_no: float = 3.0
    occupied_thresh: float = 1.0
    av_mc_excits: float = 1.0
    trunc_initiator: bool = True
    jump_shift: bool = True              # tJumpShift: shift <- E_proj on leaving the single-particle phase
    tau_search: bool = False             # tau-search conventional
    tau_search_max_iter: int | None = None  # stop method max_iter; None: var_shift (stop when the shift varies)


EPS = 1e-13                 # constants.F90:28
PROB_MIN_THRESH = 1e-8      # tau_search_conventional.F90:69
CNT_THRESHOLD = 50          # tau_search_conventional.F90:144


@dataclass
class TauSearch:
    """State of NECI's conventional tau search (tau/tau_search_conventional.F90).

    The device logs the class maxima of gamma = |H_ij| / (p_gen / p_class)
    and max_death_cpt every step; ``update`` restates update_tau (:274-499)
    on them and returns the new tau, pSingles and pParallel.  Searching stops
    when the shift starts to vary (the var_shift stop method,
    tau/tau_main.F90:153-158) or at a given iteration (max_iter, :159-160)."""
    consider_par_bias: bool      # PCHB with UNIF_UNIF particles (:82-95)
    p_singles: float
    p_parallel: float
    lattice: bool = False        # real-space Hubbard: singles only, pSingles = 1
    max_walker_bloom: float = 2.0  # MaxWalkerBloom (Calc.F90:134)
    min_tau: float = 0.0
    max_tau: float = float("inf")

    def update(self, t, tau: float):
        """update_tau for one set of logged maxima ``t`` (TauStats)."""
        enough_sing = t.cnt_sing > CNT_THRESHOLD
        enough_par = t.cnt_par > CNT_THRESHOLD
        enough_opp = t.cnt_opp > CNT_THRESHOLD
        enough_doub = (enough_par and enough_opp) if self.consider_par_bias else t.cnt_doub > CNT_THRESHOLD
        bloom = self.max_walker_bloom
        p_singles = 1.0 if self.lattice else self.p_singles
        p_doubles = 1.0 - p_singles
        gamma_sum = t.gamma_sing + t.gamma_doub
        if self.consider_par_bias:
            if enough_sing and enough_doub:
                pparallel_new = t.gamma_par / (t.gamma_opp + t.gamma_par)
                psingles_new = t.gamma_sing * pparallel_new / (t.gamma_par + t.gamma_sing * pparallel_new)
                tau_new = psingles_new * bloom / t.gamma_sing
            else:
                pparallel_new, psingles_new = self.p_parallel, p_singles
                if t.gamma_sing > EPS and t.gamma_par > EPS and t.gamma_opp > EPS:
                    tau_new = bloom * min(p_singles / t.gamma_sing,
                                          min(p_doubles * self.p_parallel / t.gamma_par,
                                              p_doubles * (1.0 - self.p_parallel) / t.gamma_opp))
                else:
                    tau_new = tau
            if enough_opp and enough_par:
                self.p_parallel = pparallel_new
        else:
            if enough_sing and enough_doub:
                psingles_new = max(t.gamma_sing / gamma_sum, PROB_MIN_THRESH)
                tau_new = bloom / gamma_sum
            else:
                psingles_new = p_singles
                if abs(t.gamma_doub) > EPS and abs(t.gamma_sing) > EPS:
                    tau_new = bloom * min(p_singles / t.gamma_sing, p_doubles / t.gamma_doub)
                elif abs(t.gamma_doub) > EPS:
                    tau_new = bloom * p_doubles / t.gamma_doub
                elif abs(t.gamma_sing) > EPS:
                    tau_new = bloom * p_singles / t.gamma_sing
                else:
                    tau_new = tau
        # death limits tau to 1 / max_death_cpt (:422-437)
        if abs(t.max_death_cpt) > EPS:
            tau_death = 1.0 / t.max_death_cpt
            if tau_death < tau_new:
                if tau_death < self.min_tau:
                    self.min_tau = tau_death
                tau_new = tau_death
        tau_new = min(max(tau_new, self.min_tau), self.max_tau)
        # (:455-470; .and. binds before .or., so enough singles, or the
        # Hubbard keyword's tHub, always allow the update)
        if tau_new < tau or (enough_sing and enough_doub) or enough_sing or self.lattice:
            tau = tau_new * 0.99999
        if (not self.lattice and enough_sing and enough_doub and 1e-5 < psingles_new < 1.0 - 1e-5):
            self.p_singles = psingles_new
        return tau, self.p_singles, self.p_parallel


@dataclass
class RunResult:
    proje_num: list = field(default_factory=list)   # per-cycle AllENumCyc
    proje_den: list = field(default_factory=list)   # per-cycle AllHFCyc
    shift: list = field(default_factory=list)
    tot_parts: list = field(default_factory=list)
    vary_shift_cycle: int | None = None
    walker_updates: float = 0.0
    seconds: float = 0.0
    hii: float = 0.0
    stats: list = field(default_factory=list)
    tau: list = field(default_factory=list)       # tau after each cycle (tau search)

    def energy(self, skip_cycles: int | None = None):
        start = self.vary_shift_cycle if skip_cycles is None else skip_cycles
        start = start or 0
        num = np.asarray(self.proje_num[start:])
        den = np.asarray(self.proje_den[start:])
        e, err = analysis.projected_energy(num, den, self.hii)
        s_mean, s_err, _ = analysis.automatic_reblocking(np.asarray(self.shift[start:]))
        return {"proje": e, "proje_err": err, "shift": s_mean + self.hii, "shift_err": s_err,
                "cycles": len(num)}


class FciMCPar:
    def __init__(self, engine: Engine, calc: CalcParams):
        self.engine = engine
        self.calc = calc
        L = engine.L
        self.diag_sft = [calc.input_diag_sft] * L
        self.single_part_phase = [True] * L
        self.iter = 1
        self.tau_search = None
        if calc.tau_search:
            spec = engine.spec
            self.tau_search = TauSearch(
                consider_par_bias=spec.generator == capi.EXGEN_PCHB and spec.kind == capi.SYS_MOLECULAR,
                p_singles=spec.p_singles, p_parallel=spec.p_parallel,
                lattice=spec.kind == capi.SYS_HUBBARD_REAL_SPACE)
            engine.set_tau_search(True)

    def params(self) -> capi.IterParams:
        c = self.calc
        return capi.default_params(
            tau=c.tau, diag_sft=self.diag_sft, initiator_walk_no=c.initiator_walk_no,
            occupied_thresh=c.occupied_thresh, real_spawn_cutoff=c.real_spawn_cutoff,
            av_mc_excits=c.av_mc_excits, t_trunc_initiator=int(c.trunc_initiator),
            t_all_real_coeff=int(c.all_real_coeff), precision=c.precision, seed=c.seed, iter=self.iter)

    def run(self, n_iter: int, keep_stats: bool = False) -> RunResult:
        eng, c = self.engine, self.calc
        L = eng.L
        res = RunResult(hii=eng.hii)
        old_parts = None
        t0 = time.perf_counter()
        n_cycles = n_iter // c.steps_sft
        for cyc in range(n_cycles):
            stats = eng.iterate_n(self.params(), c.steps_sft)
            self.iter += c.steps_sft
            num = sum(s.enum_cyc[0] for s in stats)
            den = sum(s.hf_cyc[0] for s in stats)
            res.walker_updates += sum(sum(s.tot_parts_old[:L]) for s in stats)
            if keep_stats:
                res.stats.extend(s.as_dict() for s in stats)
            parts = [stats[-1].tot_parts[k] for k in range(L)]
            if old_parts is None:
                old_parts = [stats[0].tot_parts_old[k] for k in range(L)]
            # update_shift (fcimc_iter_utilities.F90:883-1260)
            for k in range(L):
                jumped = False
                if self.single_part_phase[k] and parts[k] > c.target_walkers:
                    self.single_part_phase[k] = False
                    if res.vary_shift_cycle is None:
                        res.vary_shift_cycle = cyc
                    if c.jump_shift and den != 0.0:
                        # fcimc_iter_utilities.F90:1076-1079: DiagSft = proje_iter, update deferred
                        self.diag_sft[k] = num / den
                        jumped = True
                if not self.single_part_phase[k] and not jumped:
                    grow = parts[k] / old_parts[k]
                    if grow <= 0.0:
                        raise RuntimeError("Shift undefined because walker growth rate is zero")
                    self.diag_sft[k] -= math.log(grow) * c.sft_damp / (c.tau * c.steps_sft)
            old_parts = parts
            if self.tau_search is not None:
                stop_iter = c.tau_search_max_iter
                if (stop_iter is None and any(not sp for sp in self.single_part_phase)) or \
                        (stop_iter is not None and self.iter >= stop_iter):
                    # end_of_search_reached (tau/tau_main.F90:141-171): var_shift
                    # ends the search once the shift varies, max_iter at an iteration
                    self.tau_search = None
                    eng.set_tau_search(False)
                else:
                    ts = self.tau_search
                    old_biases = (ts.p_singles, ts.p_parallel)
                    c.tau, ps, pp = ts.update(eng.tau_stats(), c.tau)
                    if (ps, pp) != old_biases:
                        eng.set_excit_biases(ps, pp)
                res.tau.append(c.tau)
            res.proje_num.append(num)
            res.proje_den.append(den)
            res.shift.append(self.diag_sft[0])
            res.tot_parts.append(parts[0])
        res.seconds = time.perf_counter() - t0
        return res
