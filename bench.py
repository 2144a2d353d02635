#!/usr/bin/env python
"""Benchmark: walker updates per second of one FCIQMC step (PerformFCIMCycPar).

Workload (synthetic, seeded): molecular system from the synthetic FCIDUMP
recipe -- 24 spatial orbitals, 10 electrons, Sz = 0 (48 spin orbitals, one
64-bit determinant word), PCHB excitation generator, initiator FCIQMC with
real coefficients, 1e7 walkers; tau starts from the excitation statistics
of the reference (max |H_ij|/p_gen, walker-bloom limit 3) and is then set by
the conventional tau search on the device during equilibration.  A step is one PerformFCIMCycPar
over the whole walker list; a walker update is one unit of |C| processed
(TotParts entering the step).

  value   device time of K steps (CUDA events on the engine stream around
          each step; L2 flushed before every step; walker list resident in
          HBM)
  e2e     the same steps driven one at a time through the C ABI
          (neci_gpu_iterate: parameters host->device, stats device->host
          every step), timed on the host clock
  --impl reference   the CPU restatement of NECI's iteration (the oracle),
          one process per host core, each on a bounded sample of the same
          system (20 000 walkers), timed on the host

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "walker updates/sec on 1 GB300, mixed-batched vs plain FP64 at E_proj within 2σ"
UNIT = "walker updates/s"
N_ORB, N_EL, SEED = 24, 10, 20240601
TARGET_WALKERS = 1.0e7
BLOOM = 3.0

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum of the ncu capture
# of the spawn kernel on this workload, profiles/spawn_fp64_n24_2e6.md) per
# unit of work, for roofline.traffic when that kernel dominates the step:
# kernel -> (bytes per unit, step count that is the unit).
# The spawn kernel is bound by instruction issue, not by HBM: its issue
# figures from the same capture are reported beside its HBM roofline.
NCU_SPAWN_ISSUE = {"issue_active": 0.586, "alu_pipe": 0.541, "fp64_pipe": 0.372, "warps_active": 0.451,
                   "lanes_per_instruction": 25.2, "dram_bytes_per_attempt": 15.8}

NCU_DRAM_BYTES_PER_UNIT = {
    "spawn": (15.8, "n_attempts"),
}


def workload_spec():
    from neci_stable_gb300 import systems
    h, eri, ecore = systems.synthetic_fcidump(N_ORB, SEED)
    return systems.molecular_system(h, eri, ecore, N_EL, seed=SEED + 1, name="synthetic-fcidump-n24-e10")


def _ring10():
    from neci_stable_gb300 import systems
    return systems.hubbard_system("chain", (10,), 10, u=4.0)


def _square6x6():
    from neci_stable_gb300 import systems
    return systems.hubbard_system("square", (6, 6), 36, u=4.0)


def _fcidump64():
    from neci_stable_gb300 import systems
    h, eri, ecore = systems.synthetic_fcidump(64, SEED + 64)
    return systems.molecular_system(h, eri, ecore, 20, seed=SEED + 65, name="synthetic-fcidump-n64-e20")


# The configurations: the spec, target walkers, semistochastic core size,
# and the buffer sizes as multiples of the walker number (slots, spawn records).
WORKLOADS = {
    "n24": dict(spec=workload_spec, walkers=TARGET_WALKERS, core=0, slots=3.0, spawns=4.0, rescale=True,
                energy_steps=400,
                desc="synthetic FCIDUMP n=24 orbitals (48 spin orbitals), 10 electrons, Sz=0, PCHB, initiator "
                     "FCIQMC, real coefficients"),
    "ring10": dict(spec=_ring10, walkers=1e4, core=0, slots=10.0, spawns=100.0, start="single_part", sft_damp=0.1,
                   tau=0.01, energy_steps=400,
                   desc="1D Hubbard ring, 10 sites, 10 electrons, Sz=0, periodic, t=1, U=4, real-space, "
                        "uniform generator"),
    "hub6x6": dict(spec=_square6x6, walkers=1e8, core=10_000, slots=2.0, spawns=2.0, start="single_part",
                   sft_damp=0.3, scale_up=20.0, tau=0.003,
                   desc="2D Hubbard 6x6 periodic real-space lattice, 36 electrons, Sz=0, U/t=4, semistochastic "
                        "core of the 1e4 most populated determinants"),
    "n64": dict(spec=_fcidump64, walkers=5e8, core=50_000, slots=0.8, spawns=1.0, sft_damp=0.3, scale_up=20.0,
                tau=0.002,
                desc="synthetic FCIDUMP n=64 orbitals (128 spin orbitals, 3 determinant words), 20 electrons, "
                     "Sz=0, PCHB, semistochastic core of 5e4 determinants"),
}


def estimate_tau(eng, n_samples=200_000):
    """Conventional tau-search value from the excitation statistics of the
    reference and a few of its excitations: tau = bloom / max(|H_ij| / p_gen)."""
    import numpy as np
    det = eng.ilut_ref
    gammas = []
    child, pgen, hel = eng.gen_excit(det, n_samples, 99, 1)
    ok = pgen > 0
    gammas.append(np.max(np.abs(hel[ok]) / pgen[ok]))
    for c in child[ok][:8]:
        ch2, pg2, he2 = eng.gen_excit(c, n_samples // 4, 98, 1)
        ok2 = pg2 > 0
        gammas.append(np.max(np.abs(he2[ok2]) / pg2[ok2]))
    return float(min(0.05, BLOOM / max(gammas)))


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms by one
    nvidia-smi process that runs for the whole timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._proc = None

    def __enter__(self):
        cmd = ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
               "-lms", "50"]
        try:
            self._proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)  # the first sample lands before the timed steps start
        except OSError:
            self._proc = None
        return self

    def __exit__(self, *a):
        if self._proc is None:
            return
        self._proc.terminate()
        try:
            out, _ = self._proc.communicate(timeout=10)
        except subprocess.TimeoutExpired:
            self._proc.kill()
            out, _ = self._proc.communicate()
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) == 6:
                self.samples.append(f)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit())
        mx = max((float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[2 + k].strip() == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def algorithmic_bytes(kernel, st, W, L, nnz=0, fused=True):
    """Bytes a kernel must move per launch (per unit counts of the step).
    fused: pass 1 of the annihilation (the hash lookup of every spawn) ran
    inside the spawn kernel, which is the case unless the 2-RDM is sampled."""
    R = 8 * (W + L + 1)
    G = 16
    D = st["n_occupied"]
    S = st["n_spawned"]
    U = st["n_unique"]
    N = st["n_new"]
    slots = st["tot_walkers"]
    if kernel == "sweep":
        # rows and diagonal data read, signs written, each slot's free-list
        # mark (1 B), and each occupied slot's stream key (8 B)
        return slots * (R + G + 1) + D * 8 * L + D * 16 + D * 8
    if kernel == "spawn":
        # the 8 B attempt entries read (parent rows and tables are gathered
        # from L2); fused: per spawn a hash bucket and the row's det words
        # read and a 12 B spawn sum updated, a record written per candidate
        # (the estimate of the compression pass); else every record written
        if not fused:
            return st["n_attempts"] * 8 + S * R
        cand = max(S - (U - N), 0)
        return st["n_attempts"] * 8 + S * (4 + 8 * W + 12) + cand * (R + 12)
    if kernel == "core":
        # CSR column index and FP64 value per element, x gathered and y written
        return nnz * (4 + 8) + st["n_core"] * 16 * L
    if kernel == "ann_probe":
        return S * R + S * (4 + 8 * W) + (S - (U - N)) * 0 + U * (8 * L + 4)
    if kernel == "ann_compress":
        return max(S - (U - N), 0) * (8 * W + 12)
    if kernel == "ann_insert":
        return N * (R + G + 4)
    if kernel == "merge_stats":
        # rows, spawn counts and sums, and the free-list mark read
        return slots * (R + 12 * L + 1)
    # the sort form of the annihilation (NECI_ANN_SORT)
    if kernel == "sort_keys":
        # per record: its determinant words and amplitudes read, key, index
        # and 64-bit hash written
        return S * (8 * (W + L) + 16)
    if kernel == "sort_radix":
        # 3 passes of 8 bits over (24-bit key in 32 bits, 32-bit index): the
        # count pass reads the key, the scatter reads and writes key and index
        return S * 3 * (4 + 16)
    if kernel == "sort_group":
        # per record: key, its neighbour's key and the index read, the record
        # gathered; per unique determinant: the hash probe (bucket and row
        # words) and its sums written (acc/meta, or a new determinant's
        # candidate entry)
        return S * (12 + R) + U * (4 + 8 * W + 12 * L) + N * (24 + 12 * L)
    return 0


def combine_ranks(updates, dev_s, e2e_updates, e2e_s, device="cuda"):
    """The whole job's figures from N replicas (one per GPU, no collective on
    the data path): walker updates summed over the ranks, times the slowest
    rank's.  Returns (updates, device seconds, e2e updates, e2e seconds)."""
    import torch
    import torch.distributed as dist
    s = torch.tensor([updates, dev_s, e2e_updates, e2e_s], dtype=torch.float64, device=device)
    dist.all_reduce(s[0:1], op=dist.ReduceOp.SUM)
    dist.all_reduce(s[2:3], op=dist.ReduceOp.SUM)
    dist.all_reduce(s[1:2], op=dist.ReduceOp.MAX)
    dist.all_reduce(s[3:4], op=dist.ReduceOp.MAX)
    return tuple(float(x) for x in s.tolist())


def run_gpu(args, rank, world):
    import numpy as np
    from neci_stable_gb300 import capi
    from neci_stable_gb300.engine import Engine
    from neci_stable_gb300.fcimc import CalcParams, FciMCPar

    import torch
    wl = WORKLOADS[args.workload]
    spec = wl["spec"]()
    max_walkers = int(max(wl["slots"] * args.walkers, 1e5))
    max_spawned = int(max(wl["spawns"] * args.walkers, 2e5))
    eng = Engine(spec, max_walkers, max_spawned, device=0)
    # written between timed steps so that no step starts with a warm L2 (129 MB)
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda:0")  # 256 MB
    # a workload with a fixed tau runs without the tau search
    tau0 = wl["tau"] if "tau" in wl else estimate_tau(eng)
    # With scale_up, the walker distribution is equilibrated at 1/scale_up of
    # the target (its overshoot fits the buffers sized for the target) and the
    # list is then scaled to the target: every sign times the same factor, so
    # the shape and the shift carry over (a restart from a rescaled POPSFILE).
    # With rescale, the population is equilibrated at the target and scaled
    # back to it afterwards: once the shift varies it holds the population
    # wherever the growth stopped, which is not the target.
    scale = wl.get("scale_up", 1.0)
    target = args.walkers / scale
    # the conventional tau search runs on the device over the first half of
    # the equilibration (max_iter stop method), starting from tau0
    calc = CalcParams(tau=tau0, target_walkers=target, steps_sft=10, sft_damp=wl.get("sft_damp", 0.05),
                      seed=SEED + 1000 * rank, precision=capi.PREC_FP64, tau_search="tau" not in wl,
                      tau_search_max_iter=max(args.equil // 2, 20))
    drv = FciMCPar(eng, calc)
    if wl.get("start") == "single_part":
        # startsinglepart: a few walkers on the reference and the shift held
        # at 0 until the population reaches the target, then varied (the
        # usual start where the reference lies far above the ground state)
        eng.start_from_reference(initial_part=max(10.0, target * 1e-6))
    else:
        # the population on the reference, the shift varying from the start
        eng.start_from_reference(initial_part=target)
        drv.single_part_phase = [False] * eng.L
        drv.diag_sft = [0.0] * eng.L
    equil = drv.run(args.equil)  # untimed equilibration of the walker distribution
    scale_info = None
    if scale > 1.0 or wl.get("rescale"):
        st0 = eng.iterate_n(drv.params(), 1)[0]
        drv.iter += 1
        rows, dh, odh = eng.download(max_rows=int(st0.tot_walkers) + 1)
        factor = args.walkers / max(st0.tot_parts[0], 1.0)
        W, L = spec.W, spec.lenof_sign
        sg = rows[:, W:W + L].view(np.float64) * factor
        rows[:, W:W + L] = sg.view(np.int64)
        eng.upload(rows, dh, odh)
        scale_info = {"equilibrated_walkers": st0.tot_parts[0], "factor": factor}
        drv.calc.target_walkers = args.walkers
        # re-equilibration at the target population, with the shift damped
        # strongly enough to stop the population's drift within it
        damp = drv.calc.sft_damp
        drv.calc.sft_damp = max(damp, 0.3)
        drv.run(100)
        drv.calc.sft_damp = damp
    tau = drv.calc.tau
    tau_info = {"start": tau0, "final": tau, "cycles_searched": len(equil.tau)}
    core_info = None
    if wl["core"] > 0:
        # pops-core: the most populated determinants become the core space
        # (semi_stoch_gen.F90:103), its Hamiltonian built on the device
        t0 = time.perf_counter()
        st0 = eng.iterate_n(drv.params(), 1)[0]
        drv.iter += 1
        # selected on the device (neci_gpu_select_core): no download of the list
        core = eng.select_core(wl["core"], capi.PREC_FP64)
        core_info = {"n_core": int(core.shape[0]), "nnz": eng.core_nnz(), "set_up_s": time.perf_counter() - t0,
                     "selection": "device (neci_gpu_select_core)"}
        drv.run(20)
    p = drv.params()
    # warm-up steps (untimed)
    eng.iterate_n(p, args.warmup)
    p.iter += args.warmup
    # ---- timed region: K device-resident steps, CUDA events on the engine stream
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    eng.lib.neci_gpu_sync(eng.ctx)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        # Each step is timed alone by CUDA events on the engine stream, with
        # L2 flushed (256 MB written) before it.  Cycles of StepsSft steps
        # alternate FP64 and mixed precision, and the shift is updated after
        # every cycle (update_shift), so that both precisions step the same,
        # stationary population.
        timed = {capi.PREC_FP64: [[], 0.0], capi.PREC_MIXED: [[], 0.0]}
        steps_sft = drv.calc.steps_sft
        old = None
        k = 0
        while len(timed[capi.PREC_MIXED][0]) < args.steps:
            for prec in (capi.PREC_FP64, capi.PREC_MIXED):
                pc = drv.params()
                pc.precision = prec
                n = min(steps_sft, args.steps - len(timed[prec][0]))
                for _ in range(n):
                    flush.fill_(float(k))
                    k += 1
                    torch.cuda.synchronize()
                    st1, ms = eng.iterate_timed(pc, 1)
                    pc.iter += 1
                    timed[prec][0].extend(st1)
                    timed[prec][1] += ms
                drv.iter = pc.iter
                parts = timed[prec][0][-1].tot_parts[0]
                if old is not None:
                    drv.diag_sft[0] -= math.log(parts / old) * drv.calc.sft_damp / (drv.calc.tau * steps_sft)
                old = parts
        stats, dev_ms = timed[capi.PREC_FP64]
        mstats, mixed_ms = timed[capi.PREC_MIXED]
        p = drv.params()
        # the same number of FP64 steps back to back (CUDA graph replays, no flush)
        bb_stats, bb_ms = eng.iterate_timed(p, args.steps)
        p.iter += args.steps
        # ---- e2e: one C-ABI call per step with host buffers
        t0 = time.perf_counter()
        e2e_updates = 0.0
        for _ in range(args.steps):
            st = eng.perform_fcimc_cyc_par(p)
            p.iter += 1
            e2e_updates += st.tot_parts_old[0]
        e2e_s = time.perf_counter() - t0
    # ---- energy window (untimed): further cycles of StepsSft steps of each
    # precision, interleaved on the same population with the shift updated
    # after every cycle, so that E_proj of the two precisions has error bars
    # from many blocks
    drv.iter = p.iter
    old = st.tot_parts[0]  # the growth of the first cycle is taken from the last e2e step
    en = {capi.PREC_FP64: list(stats), capi.PREC_MIXED: list(mstats)}
    n_energy = args.energy_steps if args.energy_steps is not None else wl.get("energy_steps", 60)
    while len(en[capi.PREC_MIXED]) < args.steps + n_energy:
        for prec in (capi.PREC_FP64, capi.PREC_MIXED):
            pc = drv.params()
            pc.precision = prec
            sts = eng.iterate_n(pc, drv.calc.steps_sft)
            drv.iter += drv.calc.steps_sft
            en[prec].extend(sts)
            parts = sts[-1].tot_parts[0]
            drv.diag_sft[0] -= math.log(parts / old) * drv.calc.sft_damp / (drv.calc.tau * drv.calc.steps_sft)
            old = parts
    p = drv.params()
    updates = sum(s.tot_parts_old[0] for s in stats)
    bb_updates = sum(s.tot_parts_old[0] for s in bb_stats)
    mixed_updates = sum(s.tot_parts_old[0] for s in mstats)
    # E_proj of the FP64 and of the mixed-precision steps of the timed region
    # and the energy window (blocks of 10 steps, reblocked)
    from neci_stable_gb300 import analysis
    proje = {}
    for name, sts in (("fp64", en[capi.PREC_FP64]), ("mixed", en[capi.PREC_MIXED])):
        num = np.array([sum(x.enum_cyc[0] for x in sts[k:k + 10]) for k in range(0, len(sts), 10)])
        den = np.array([sum(x.hf_cyc[0] for x in sts[k:k + 10]) for k in range(0, len(sts), 10)])
        e, err = analysis.projected_energy(num, den, eng.hii) if len(num) >= 2 else (float(num.sum() / den.sum()) + eng.hii, None)
        proje[name] = {"e_proj": e, "err": err, "steps": len(sts)}
    if proje["fp64"]["err"] and proje["mixed"]["err"]:
        d = proje["mixed"]["e_proj"] - proje["fp64"]["e_proj"]
        proje["mixed_minus_fp64"] = {"ha": d, "sigma": abs(d) / math.hypot(proje["fp64"]["err"], proje["mixed"]["err"])}
    # ---- per-kernel timing passes (events around each kernel; not the timed
    # number): FP64, then the mixed-precision step
    def profile(prec, n=3):
        pp = drv_params_like(p, prec)
        eng.set_profiling(True)
        st = eng.iterate_n(pp, n)
        p.iter += n
        kt = eng.kernel_times()
        eng.set_profiling(False)
        return kt, st[-1].as_dict()

    def drv_params_like(base, prec):
        q = capi.default_params()
        for name, _ in capi.IterParams._fields_:
            setattr(q, name, getattr(base, name))
        q.precision = prec
        return q

    ktimes, last = profile(capi.PREC_FP64)
    ktimes_mixed, last_mixed = profile(capi.PREC_MIXED)
    # ---- the sort form of the annihilation (NECI_ANN_SORT) on the same
    # population: K steps timed alone as above, then a profiling pass
    eng.set_option(capi.OPT_ANNIHILATION, capi.ANN_SORT)
    eng.iterate_n(p, 3)
    p.iter += 3
    sort_upd, sort_ms = 0.0, 0.0
    for _ in range(args.steps):
        flush.fill_(float(k))
        k += 1
        torch.cuda.synchronize()
        st1, ms = eng.iterate_timed(p, 1)
        p.iter += 1
        sort_upd += st1[0].tot_parts_old[0]
        sort_ms += ms
    ktimes_sort, last_sort = profile(capi.PREC_FP64)
    eng.set_option(capi.OPT_ANNIHILATION, capi.ANN_HASH)
    return {
        "eng": eng, "spec": spec, "tau": tau, "tau_info": tau_info, "core_info": core_info, "proje": proje,
        "scale_info": scale_info,
        "updates": updates, "dev_ms": dev_ms, "clk": clk.summary(),
        "e2e_updates": e2e_updates, "e2e_s": e2e_s, "ktimes": ktimes, "last": last, "stats": stats,
        "first": stats[0].as_dict(),
        "equil": equil, "mixed_updates": mixed_updates, "mixed_ms": mixed_ms, "bb_updates": bb_updates,
        "bb_ms": bb_ms, "ktimes_mixed": ktimes_mixed, "last_mixed": last_mixed, "ktimes_sort": ktimes_sort,
        "last_sort": last_sort, "sort_updates": sort_upd, "sort_ms": sort_ms,
    }


def batched_specs(n_inst=64, base_seed=7000):
    """Instances of the synthetic FCIDUMP recipe with instance-indexed seeds:
    n ~ U{12..40} spatial orbitals, even nel ~ U{6..20} (Sz = 0), target
    walkers log-uniform in [1e4, 1e6], each a replica pair (lenof_sign 2)."""
    import numpy as np
    from neci_stable_gb300 import systems
    rng = np.random.default_rng(base_seed)
    out = []
    for i in range(n_inst):
        n = int(rng.integers(12, 41))
        nel = int(2 * rng.integers(3, 11))
        nel = min(nel, n)  # at most half filling of each spin
        walkers = float(10 ** rng.uniform(4.0, 6.0))
        h, eri, ecore = systems.synthetic_fcidump(n, base_seed + i)
        spec = systems.molecular_system(h, eri, ecore, nel, seed=base_seed + 1000 + i, lenof_sign=2,
                                        name=f"batch-{i}-n{n}-e{nel}")
        out.append((spec, walkers))
    return out


def run_batched(args):
    """Plain FP64 single-instance steps (each instance alone, one after the
    other) against mixed-precision batched steps (all instances side by side)."""
    from neci_stable_gb300 import capi
    from neci_stable_gb300.engine import Engine, iterate_batch
    specs = batched_specs(args.instances)
    engines, params = [], []
    for i, (spec, walkers) in enumerate(specs):
        eng = Engine(spec, max_walkers=int(max(6 * walkers, 1e5)), max_spawned=int(max(6 * walkers, 2e5)))
        eng.start_from_reference(initial_part=walkers)
        # each instance is a replica pair sampling the 2-RDM in every step
        eng.set_rdm_sampling(True)
        tau = min(0.02, estimate_tau(eng, 20_000))
        p = capi.default_params(tau=tau, seed=SEED + i, iter=1)
        engines.append(eng)
        params.append(p)
    # equilibrate all instances together, the shift following the population
    n_cyc = max(args.batch_equil // 10, 1)
    olds = [s[1] * 2 for s in specs]
    for c in range(n_cyc):
        st, _ = iterate_batch(engines, params, 10)
        for i, p in enumerate(params):
            p.iter += 10
            parts = st[i][-1].tot_parts[0] + st[i][-1].tot_parts[1]
            p.diag_sft[0] = p.diag_sft[1] = p.diag_sft[0] - 0.05 * math.log(parts / olds[i]) / (p.tau * 10)
            olds[i] = parts
    K = args.batch_steps
    # plain FP64, one instance at a time
    fp64_upd, fp64_ms = 0.0, 0.0
    for eng, p in zip(engines, params):
        p.precision = capi.PREC_FP64
        eng.iterate_n(p, 3)
        p.iter += 3
        st, ms = eng.iterate_timed(p, K)
        p.iter += K
        fp64_upd += sum(x.tot_parts_old[0] + x.tot_parts_old[1] for x in st)
        fp64_ms += ms
    # mixed precision, batched
    for p in params:
        p.precision = capi.PREC_MIXED
    iterate_batch(engines, params, 3)
    for p in params:
        p.iter += 3
    st, mixed_ms = iterate_batch(engines, params, K)
    mixed_upd = sum(x.tot_parts_old[0] + x.tot_parts_old[1] for per in st for x in per)
    # FP64 batched too (separates the batching gain from the precision gain)
    for p in params:
        p.iter += K
        p.precision = capi.PREC_FP64
    st, fb_ms = iterate_batch(engines, params, K)
    fb_upd = sum(x.tot_parts_old[0] + x.tot_parts_old[1] for per in st for x in per)
    for e in engines:
        e.close()
    v_single = fp64_upd / (fp64_ms / 1e3)
    v_mixed = mixed_upd / (mixed_ms / 1e3)
    v_fb = fb_upd / (fb_ms / 1e3)
    return {"instances": len(specs), "steps": K, "unit": UNIT, "rdm": True,
            "fp64_single_instance": v_single, "fp64_batched": v_fb, "mixed_batched": v_mixed,
            "speedup_mixed_batched_vs_fp64_single": v_mixed / v_single,
            "speedup_mixed_batched_vs_fp64_batched": v_mixed / v_fb,
            "walkers_total": sum(w for _, w in specs),
            "workload": "64 synthetic FCIDUMP instances (instance-indexed seeds), n 12..40, nel 6..20, "
                        "walkers 1e4..1e6 log-uniform, replica pairs sampling the 2-RDM every step, PCHB"}


class OracleSample:
    """The CPU restatement of the iteration (the oracle) on one core: a
    `walkers`-walker population of the workload, equilibrated for
    equil_cycles x 10 steps with the conventional tau search (update_tau on
    the oracle's own logs, as on the device) and the shift following the
    population; `step(seconds)` then runs iterations for that long."""

    def __init__(self, seed, walkers=20000.0, equil_cycles=8):
        import numpy as np
        from neci_stable_gb300.fcimc import TauSearch
        from neci_stable_gb300.systems import encode_det, make_rows
        from oracle.oracle import Oracle
        spec = workload_spec()
        self.seed = seed
        self.orc = Oracle(spec, 2_000_000, 4_000_000)
        ref = encode_det(spec.reference, spec.nifd)
        self.orc.upload(make_rows(ref[None], np.array([[walkers]]), np.array([1 << 13])))
        self.orc.set_tau_search(True)
        ts = TauSearch(consider_par_bias=True, p_singles=spec.p_singles, p_parallel=spec.p_parallel)
        self.tau, self.shift, self.old, self.it, self.n = 0.0014, 0.0, walkers, 0, 0
        for _ in range(equil_cycles):
            for _ in range(10):
                st = self._iterate()
            self.tau, ps, pp = ts.update(self.orc.tau_stats(), self.tau)
            self.orc.set_excit_biases(ps, pp)
            self._update_shift(st)
        self.orc.set_tau_search(False)
        self.p_singles, self.p_parallel = ts.p_singles, ts.p_parallel

    def _iterate(self):
        from neci_stable_gb300 import capi
        self.it += 1
        st, rc = self.orc.iterate(capi.default_params(tau=self.tau, seed=self.seed, iter=self.it,
                                                      diag_sft=[self.shift, self.shift]))
        if rc:
            raise RuntimeError(f"oracle iteration failed with {rc}")
        return st

    def _update_shift(self, st):
        self.shift -= 0.05 * math.log(st.tot_parts[0] / self.old) / (self.tau * 10)
        self.old = st.tot_parts[0]

    def step(self, seconds):
        t0 = time.perf_counter()
        upd, n = 0.0, 0
        while time.perf_counter() - t0 < seconds:
            st = self._iterate()
            upd += st.tot_parts_old[0]
            n += 1
            self.n += 1
            if self.n % 10 == 0:
                self._update_shift(st)
        return upd, time.perf_counter() - t0, n

    def describe(self):
        return f"tau {self.tau:.4g}, pSingles {self.p_singles:.3f}, pParallel {self.p_parallel:.3f}"


def cpu_baseline_sample(seconds=12.0):
    """Oracle (CPU restatement) on one core: a 20 000-walker sample of the workload."""
    smp = OracleSample(5)
    upd, dt, n = smp.step(seconds)
    return {"value": upd / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"oracle on the n24/e10 synthetic FCIDUMP, 20000-walker sample after its own tau search "
                      f"({smp.describe()}), {n} steps in {dt:.1f} s"}


_SAMPLE = None


def _ref_init(seed):
    """Pool initializer: this process's equilibrated oracle sample."""
    global _SAMPLE
    _SAMPLE = OracleSample(seed + os.getpid() % 1000)


def _ref_worker(seconds):
    upd, dt, n = _SAMPLE.step(seconds)
    return upd, dt, n, _SAMPLE.describe()


def run_reference(args, rank, world):
    """CPU restatement of the reference's iteration on all host cores: one
    equilibrated 20000-walker oracle per process; a step is one round of
    per_step seconds of iterations on every process, timed on the host clock
    around the round."""
    if rank != 0:
        return None
    import multiprocessing as mp
    from oracle import oracle as o
    o.lib()  # build/load before the workers start
    cores = os.cpu_count() or 1
    per_step = max(0.25, min(2.0, 90.0 / max(args.steps + args.warmup, 1)))
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    total_upd, total_s = 0.0, 0.0
    steps_done = 0
    desc = ""
    with ctx.Pool(cores, initializer=_ref_init, initargs=(1000,)) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_worker, [per_step] * cores, chunksize=1)
        for k in range(args.steps):
            w0 = time.perf_counter()
            res = pool.map(_ref_worker, [per_step] * cores, chunksize=1)
            total_s += time.perf_counter() - w0
            total_upd += sum(r[0] for r in res)
            steps_done += sum(r[2] for r in res)
            desc = res[0][3]
    value = total_upd / total_s
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "synthetic FCIDUMP n=24 orbitals, 10 electrons, PCHB, initiator FCIQMC, real "
                               "coefficients, conventional tau search",
                   "sample": "20000-walker population per core"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} processes x {per_step:.2f} s per step of the oracle iteration "
                                   f"(20000 walkers each, {desc}), {steps_done} iterations"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t0,
    }


def profile_case(args):
    """A short run for profilers: the headline molecule at --walkers walkers
    with the excitation biases and tau where NECI's conventional tau search
    leaves them on this workload (pSingles 0.53, pParallel 0.29, tau 0.023),
    --equil FP64 steps with the shift following the population, then --steps
    steps of the case named by --profile-case: fp64, mixed (FP32 spawn
    amplitudes) or sort (the sort form of the annihilation)."""
    import numpy as np
    from neci_stable_gb300 import build as b
    from neci_stable_gb300 import capi
    from neci_stable_gb300.engine import Engine
    b.build()
    eng = Engine(workload_spec(), int(3 * args.walkers), int(4 * args.walkers))
    eng.set_excit_biases(0.53, 0.29)
    eng.start_from_reference(initial_part=args.walkers)
    p = capi.default_params(tau=0.023, seed=5, iter=1)
    shift, old = 0.0, args.walkers
    for _ in range(args.equil // 10):
        st = eng.iterate_n(p, 10)
        p.iter += 10
        parts = st[-1].tot_parts[0]
        shift -= 0.1 * math.log(parts / old) / (p.tau * 10)
        old = parts
        p.diag_sft[0] = shift
    if args.profile_case == "mixed":
        p.precision = capi.PREC_MIXED
    if args.profile_case == "sort":
        eng.set_option(capi.OPT_ANNIHILATION, capi.ANN_SORT)
    st = eng.iterate_n(p, args.steps)[-1]
    print(json.dumps({"profile_case": args.profile_case, "walkers": st.tot_parts[0], "n_attempts": st.n_attempts,
                      "n_spawned": st.n_spawned, "n_unique": st.n_unique, "n_new": st.n_new,
                      "tot_walkers": st.tot_walkers}))
    eng.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--equil", type=int, default=600, help="untimed equilibration iterations")
    ap.add_argument("--energy-steps", type=int, default=None,
                    help="untimed steps of each precision after the timed region for E_proj (default: the workload's)")
    ap.add_argument("--walkers", type=float, default=None, help="target walker number (default: the workload's)")
    ap.add_argument("--workload", default="n24", choices=sorted(WORKLOADS),
                    help="n24: the headline configuration; ring10, hub6x6, n64: the other single-GPU configurations")
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-instances measurement")
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=20)
    ap.add_argument("--batch-equil", type=int, default=200)
    ap.add_argument("--profile-case", choices=["fp64", "mixed", "sort"], default=None,
                    help="a short run of one case for a profiler (no timing, no JSON bench line)")
    args = ap.parse_args()
    if args.profile_case:
        if args.walkers is None:
            args.walkers = 2e6
        profile_case(args)
        return
    args.warmup = max(args.warmup, 3)
    if args.walkers is None:
        args.walkers = WORKLOADS[args.workload]["walkers"]
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl" if args.impl == "native" else "gloo")

    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if rank == 0:
            print(json.dumps(out))
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    from neci_stable_gb300 import build as b
    b.build()
    r = run_gpu(args, rank, world)
    dev_s = r["dev_ms"] / 1000.0
    updates = r["updates"]
    e2e_upd, e2e_s = r["e2e_updates"], r["e2e_s"]
    if world > 1:
        updates, dev_s, e2e_upd, e2e_s = combine_ranks(updates, dev_s, e2e_upd, e2e_s)
    if rank != 0:
        dist.destroy_process_group()
        return
    eng, spec = r["eng"], r["spec"]
    W, L = spec.W, spec.lenof_sign
    kt = {k: v for k, v in r["ktimes"].items() if v[1] > 0}
    top = max(kt, key=lambda k: kt[k][0])
    top_ms = kt[top][0] / kt[top][1]
    nnz = (r["core_info"] or {}).get("nnz", 0)
    fused = "ann_probe" not in kt  # pass 1 ran inside the spawn kernel
    ab = algorithmic_bytes(top, r["last"], W, L, nnz, fused)
    hbm, peak_kind = peaks()
    achieved = ab / (top_ms / 1e3) / 1e9
    traffic = None
    if top in NCU_DRAM_BYTES_PER_UNIT:
        per_unit, unit = NCU_DRAM_BYTES_PER_UNIT[top]
        traffic = per_unit * r["last"][unit]
    # achieved GB/s of every kernel (algorithmic bytes of the last profiled step)
    kernel_gbs = {}
    for k, (ms, cnt) in kt.items():
        b = algorithmic_bytes(k, r["last"], W, L, nnz, fused)
        if b > 0:
            kernel_gbs[k] = b / (ms / cnt / 1e3) / 1e9
    ann = tuple(k for k in ("ann_probe", "ann_compress", "ann_insert") if k in kt)
    ann_ms = sum(kt[k][0] / kt[k][1] for k in ann)
    ann_bytes = sum(algorithmic_bytes(k, r["last"], W, L) for k in ann)
    # the sort form of the annihilation: per stage (keys, the 3 radix passes,
    # grouping + walker-hash lookup) and the insertion of new determinants
    kts = {k: v for k, v in r["ktimes_sort"].items() if v[1] > 0}
    sort_stages = {}
    for k in ("sort_keys", "sort_radix", "sort_group", "ann_insert"):
        if k not in kts:
            continue
        ms = kts[k][0] / kts[k][1]
        b = algorithmic_bytes(k, r["last_sort"], W, L)
        sort_stages[k] = {"ms": ms, "algorithmic_bytes": b, "gbs": b / (ms / 1e3) / 1e9,
                          "frac": b / (ms / 1e3) / 1e9 / hbm}
    sort_ms = sum(v["ms"] for v in sort_stages.values())
    sort_bytes = sum(v["algorithmic_bytes"] for v in sort_stages.values())
    ktm = {k: v for k, v in r["ktimes_mixed"].items() if v[1] > 0}
    # rehash (2, idle unless flagged), begin, sweep, expand, spawn, compress,
    # decide, place, merge, final; the probe unless the spawn kernel does it;
    # the core projection and the sum of its long rows (a compaction, when a
    # step leaves more holes than walkers, runs between calls)
    launches_per_step = 11 + (2 if r["last"]["n_core"] > 0 else 0) + (0 if fused else 1)
    line = {
        "metric": METRIC, "value": updates / dev_s, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{WORKLOADS[args.workload]['desc']}, FP64, {args.walkers:.3g} walkers",
                   "name": args.workload, "core": r["core_info"], "scaled_up": r["scale_info"],
                   "tau": r["tau"], "tau_search": r["tau_info"], "walkers": r["stats"][-1].tot_parts[0],
                   "determinants": r["stats"][-1].n_occupied,
                   "step_counts": {k: r["last"][k] for k in ("n_attempts", "n_spawned", "n_unique", "n_new",
                                                             "tot_walkers")},
                   "first_step_counts": {k: r["first"][k] for k in ("n_attempts", "n_spawned", "n_unique",
                                                                    "n_new", "tot_walkers")},
                   "l2": "flushed before every timed step (256 MB written); each step timed alone by CUDA events",
                   "parallelism": f"replica x{world}"},
        "value_back_to_back": {"value": r["bb_updates"] / (r["bb_ms"] / 1000.0), "unit": UNIT,
                               "ms_per_step": r["bb_ms"] / args.steps,
                               "note": "the same number of steps as CUDA-graph replays back to back, no flush"},
        "clocks": r["clk"],
        "e2e": {"value": e2e_upd / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 96, "d2h_bytes_per_step": 200},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": traffic,
                     "algorithmic_bytes": ab, "ms_per_launch": top_ms,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per unit of this workload"},
        "spawn_issue": dict(NCU_SPAWN_ISSUE, source="ncu --set full of k_spawn on this workload at 2e6 walkers; "
                                                   "fractions of the sustained peak, per SM"),
        "annihilation_roofline": {"kernels": list(ann), "achieved": ann_bytes / (ann_ms / 1e3) / 1e9, "peak": hbm,
                                  "unit": "GB/s", "frac": ann_bytes / (ann_ms / 1e3) / 1e9 / hbm,
                                  "ms_per_step": ann_ms, "algorithmic_bytes": ann_bytes},
        "kernel_ms_per_step": {k: v[0] / v[1] for k, v in kt.items()},
        "kernel_ms_per_step_mixed": {k: v[0] / v[1] for k, v in ktm.items()},
        "kernel_gbs": kernel_gbs,
        "sort_annihilation": {
            "value": r["sort_updates"] / (r["sort_ms"] / 1000.0), "unit": UNIT,
            "ms_per_step": r["sort_ms"] / args.steps,
            "stages": sort_stages, "ms_per_step_annihilation": sort_ms,
            "annihilation_frac": sort_bytes / (sort_ms / 1e3) / 1e9 / hbm if sort_ms > 0 else None,
            "note": "NECI_ANN_SORT on the same population: spawns radix-sorted (three 8-bit passes) by a "
                    "24-bit key of their determinant's hash and reduced as runs; the hash form is the default"},
        "proje": r["proje"],
        "mixed_precision": {"value": r["mixed_updates"] / (r["mixed_ms"] / 1000.0), "unit": UNIT,
                            "ms_per_step": r["mixed_ms"] / args.steps,
                            "speedup_vs_fp64": (r["mixed_updates"] / r["mixed_ms"]) / (updates / (dev_s * 1000.0)),
                            "note": "FP32 H_ij, p_gen and spawn amplitude; FP64 death, E_proj and signs; "
                                    "cycles of 10 steps interleaved with the FP64 steps on the same population"},
    }
    if not args.no_batched and world == 1 and args.workload == "n24":
        line["batched"] = run_batched(args)
        # against the headline: the FP64 single instance of the 1e7-walker molecule
        line["batched"]["speedup_mixed_batched_vs_n24_fp64"] = line["batched"]["mixed_batched"] / line["value"]
    if not args.no_cpu_baseline and world == 1 and args.workload == "n24":
        line["cpu_baseline"] = cpu_baseline_sample()
    print(json.dumps(line))
    eng.close()


if __name__ == "__main__":
    main()
