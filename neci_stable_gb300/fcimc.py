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
            res.proje_num.append(num)
            res.proje_den.append(den)
            res.shift.append(self.diag_sft[0])
            res.tot_parts.append(parts[0])
        res.seconds = time.perf_counter() - t0
        return res
