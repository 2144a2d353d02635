#!/usr/bin/env python
"""Benchmark: walker updates per second of one FCIQMC step (PerformFCIMCycPar).

Workload (synthetic, seeded): molecular system from the synthetic FCIDUMP
recipe -- 24 spatial orbitals, 10 electrons, Sz = 0 (48 spin orbitals, one
64-bit determinant word), PCHB excitation generator, initiator FCIQMC with
real coefficients, 1e7 walkers, tau from the excitation statistics
(max |H_ij|/p_gen, walker-bloom limit 3).  A step is one PerformFCIMCycPar
over the whole walker list; a walker update is one unit of |C| processed
(TotParts entering the step).

  value   device time of K back-to-back steps (CUDA events on the engine
          stream; walker list resident in HBM, working set > L2)
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
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "walker updates/sec on 1 GB300, mixed-batched vs plain FP64 at E_proj within 2σ"
UNIT = "walker updates/s"
N_ORB, N_EL, SEED = 24, 10, 20240601
TARGET_WALKERS = 1.0e7
BLOOM = 3.0


def workload_spec():
    from neci_stable_gb300 import systems
    h, eri, ecore = systems.synthetic_fcidump(N_ORB, SEED)
    return systems.molecular_system(h, eri, ecore, N_EL, seed=SEED + 1, name="synthetic-fcidump-n24-e10")


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
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        cmd = ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits"]
        while not self._stop.is_set():
            try:
                out = subprocess.run(cmd, capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._th.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit())
        mx = max((float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[2 + k].strip() == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def algorithmic_bytes(kernel, st, W, L):
    """Bytes a kernel must move per launch (per unit counts of the step)."""
    R = 8 * (W + L + 1)
    G = 16
    D = st["n_occupied"]
    S = st["n_spawned"]
    U = st["n_unique"]
    N = st["n_new"]
    slots = st["tot_walkers"]
    if kernel == "sweep":
        return slots * (R + G) + D * 8 * L + D * 16
    if kernel == "spawn":
        return S * R + st["n_attempts"] / 16 * (8 * W + 16)
    if kernel == "ann_probe":
        return S * R + S * (4 + 8 * W) + (S - (U - N)) * 0 + U * (8 * L + 4)
    if kernel == "ann_compress":
        return max(S - (U - N), 0) * (8 * W + 12)
    if kernel == "ann_insert":
        return N * (R + G + 4)
    if kernel == "merge_stats":
        return slots * (R + 12 * L)
    return 0


def run_gpu(args, rank, world):
    import numpy as np
    from neci_stable_gb300 import capi
    from neci_stable_gb300.engine import Engine
    from neci_stable_gb300.fcimc import CalcParams, FciMCPar

    spec = workload_spec()
    max_walkers = int(3.0e7)
    max_spawned = int(4.0e7)
    eng = Engine(spec, max_walkers, max_spawned, device=0)
    tau = estimate_tau(eng)
    calc = CalcParams(tau=tau, target_walkers=args.walkers, steps_sft=10, sft_damp=0.05,
                      seed=SEED + 1000 * rank, precision=capi.PREC_FP64)
    drv = FciMCPar(eng, calc)
    # start: the population on the reference, shift varying from the start
    eng.start_from_reference(initial_part=args.walkers)
    drv.single_part_phase = [False] * eng.L
    drv.diag_sft = [0.0] * eng.L
    equil = drv.run(args.equil)  # untimed equilibration of the walker distribution
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
        stats, dev_ms = eng.iterate_timed(p, args.steps)
    p.iter += args.steps
    updates = sum(s.tot_parts_old[0] for s in stats)
    # ---- e2e: one C-ABI call per step with host buffers
    t0 = time.perf_counter()
    e2e_updates = 0.0
    for k in range(args.steps):
        st = eng.perform_fcimc_cyc_par(p)
        p.iter += 1
        e2e_updates += st.tot_parts_old[0]
    e2e_s = time.perf_counter() - t0
    # ---- the same steps with FP32 spawn amplitudes (mixed precision)
    pm = drv.params()
    pm.iter = p.iter
    pm.precision = capi.PREC_MIXED
    eng.iterate_n(pm, 3)
    pm.iter += 3
    mstats, mixed_ms = eng.iterate_timed(pm, args.steps)
    p.iter = pm.iter + args.steps
    mixed_updates = sum(s.tot_parts_old[0] for s in mstats)
    # ---- per-kernel timing pass (events around each kernel; not the timed number)
    eng.set_profiling(True)
    prof_stats = eng.iterate_n(p, 3)
    p.iter += 3
    ktimes = eng.kernel_times()
    eng.set_profiling(False)
    last = prof_stats[-1].as_dict()
    return {
        "eng": eng, "spec": spec, "tau": tau, "updates": updates, "dev_ms": dev_ms, "clk": clk.summary(),
        "e2e_updates": e2e_updates, "e2e_s": e2e_s, "ktimes": ktimes, "last": last, "stats": stats,
        "equil": equil, "mixed_updates": mixed_updates, "mixed_ms": mixed_ms,
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
    return {"instances": len(specs), "steps": K, "unit": UNIT,
            "fp64_single_instance": v_single, "fp64_batched": fb_upd / (fb_ms / 1e3), "mixed_batched": v_mixed,
            "speedup_mixed_batched_vs_fp64_single": v_mixed / v_single,
            "walkers_total": sum(w for _, w in specs),
            "workload": "64 synthetic FCIDUMP instances (instance-indexed seeds), n 12..40, nel 6..20, "
                        "walkers 1e4..1e6 log-uniform, replica pairs, PCHB"}


def cpu_baseline_sample(seconds=12.0):
    """Oracle (CPU restatement) on one core: a 20 000-walker sample of the workload."""
    from neci_stable_gb300 import capi
    from oracle.oracle import Oracle
    from neci_stable_gb300.systems import encode_det, make_rows
    import numpy as np
    spec = workload_spec()
    orc = Oracle(spec, 2_000_000, 4_000_000)
    ref = encode_det(spec.reference, spec.nifd)
    orc.upload(make_rows(ref[None], np.array([[20000.0]]), np.array([1 << 13])))
    p = capi.default_params(tau=0.01, seed=5, iter=1)
    # short equilibration with the shift tracking the population
    shift = 0.0
    old = 20000.0
    for it in range(1, 41):
        p.iter = it
        p.diag_sft[0] = shift
        st, rc = orc.iterate(p)
        if it % 10 == 0:
            shift -= 0.05 * math.log(st.tot_parts[0] / old) / (0.01 * 10)
            old = st.tot_parts[0]
    t0 = time.perf_counter()
    upd = 0.0
    n = 0
    while time.perf_counter() - t0 < seconds:
        n += 1
        p.iter = 100 + n
        st, rc = orc.iterate(p)
        upd += st.tot_parts_old[0]
    dt = time.perf_counter() - t0
    return {"value": upd / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"oracle on the n24/e10 synthetic FCIDUMP, 20000-walker sample, {n} steps in {dt:.1f} s"}


def _ref_worker(args):
    seconds, seed = args
    import math as _m
    from neci_stable_gb300 import capi
    from oracle.oracle import Oracle
    from neci_stable_gb300.systems import encode_det, make_rows
    import numpy as np
    spec = workload_spec()
    orc = Oracle(spec, 2_000_000, 4_000_000)
    ref = encode_det(spec.reference, spec.nifd)
    orc.upload(make_rows(ref[None], np.array([[20000.0]]), np.array([1 << 13])))
    p = capi.default_params(tau=0.01, seed=seed, iter=1)
    shift, old = 0.0, 20000.0
    for it in range(1, 31):
        p.iter = it
        p.diag_sft[0] = shift
        st, rc = orc.iterate(p)
        if it % 10 == 0:
            shift -= 0.05 * _m.log(st.tot_parts[0] / old) / (0.01 * 10)
            old = st.tot_parts[0]
    t0 = time.perf_counter()
    upd, n = 0.0, 0
    while time.perf_counter() - t0 < seconds:
        n += 1
        p.iter = 100 + n
        st, rc = orc.iterate(p)
        upd += st.tot_parts_old[0]
    return upd, time.perf_counter() - t0, n


def run_reference(args, rank, world):
    """CPU restatement of the reference's iteration on all host cores."""
    if rank != 0:
        return None
    import multiprocessing as mp
    from oracle import oracle as o
    o.lib()  # build/load before forking workers
    cores = os.cpu_count() or 1
    per_step = max(0.5, min(4.0, 150.0 / max(args.steps, 1)))
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    total_upd, total_s = 0.0, 0.0
    steps_done = 0
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_worker, [(0.5, 100 + c) for c in range(cores)])
        for k in range(args.steps):
            res = pool.map(_ref_worker, [(per_step, 1000 + 17 * k + c) for c in range(cores)])
            total_upd += sum(r[0] for r in res)
            total_s += max(r[1] for r in res)
            steps_done += sum(r[2] for r in res)
    value = total_upd / total_s
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "synthetic FCIDUMP n=24 orbitals, 10 electrons, PCHB, initiator FCIQMC, real coefficients",
                   "sample": "20000-walker population per core"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} processes x {per_step:.0f} s per step of the oracle iteration "
                                   f"(20000 walkers each), {steps_done} iterations"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t0,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--equil", type=int, default=600, help="untimed equilibration iterations")
    ap.add_argument("--walkers", type=float, default=TARGET_WALKERS, help="target walker number")
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-instances measurement")
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=20)
    ap.add_argument("--batch-equil", type=int, default=200)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
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
        import torch
        import torch.distributed as dist
        t = torch.tensor([updates, dev_s, e2e_upd, e2e_s], dtype=torch.float64, device="cuda")
        s = t.clone()
        dist.all_reduce(s[0:1], op=dist.ReduceOp.SUM)
        dist.all_reduce(s[2:3], op=dist.ReduceOp.SUM)
        dist.all_reduce(s[1:2], op=dist.ReduceOp.MAX)
        dist.all_reduce(s[3:4], op=dist.ReduceOp.MAX)
        updates, dev_s, e2e_upd, e2e_s = (float(x) for x in s.tolist())
    if rank != 0:
        dist.destroy_process_group()
        return
    eng, spec = r["eng"], r["spec"]
    W, L = spec.W, spec.lenof_sign
    kt = {k: v for k, v in r["ktimes"].items() if v[1] > 0}
    top = max(kt, key=lambda k: kt[k][0])
    top_ms = kt[top][0] / kt[top][1]
    ab = algorithmic_bytes(top, r["last"], W, L)
    hbm, peak_kind = peaks()
    achieved = ab / (top_ms / 1e3) / 1e9
    traffic = None
    tp = ROOT / "profiles" / "ncu_traffic.json"
    if tp.exists():
        tj = json.loads(tp.read_text())
        if top in tj.get("bytes_per_unit", {}):
            unit = tj["unit_of"][top]
            traffic = tj["bytes_per_unit"][top] * r["last"][unit]
    launches_per_step = 11 + (1 if r["last"]["n_core"] > 0 else 0)
    line = {
        "metric": METRIC, "value": updates / dev_s, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "synthetic FCIDUMP n=24 orbitals (48 spin orbitals), 10 electrons, Sz=0, PCHB, "
                               f"initiator FCIQMC, real coefficients, FP64, {args.walkers:.3g} walkers",
                   "tau": r["tau"], "walkers": r["stats"][-1].tot_parts[0],
                   "determinants": r["stats"][-1].n_occupied, "l2": "working set larger than L2 (walker rows, "
                   "hash and spawn buffers > 129 MB); no flush", "parallelism": f"replica x{world}"},
        "clocks": r["clk"],
        "e2e": {"value": e2e_upd / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 96, "d2h_bytes_per_step": 200},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": traffic,
                     "algorithmic_bytes": ab, "ms_per_launch": top_ms},
        "kernel_ms_per_step": {k: v[0] / v[1] for k, v in kt.items()},
        "mixed_precision": {"value": r["mixed_updates"] / (r["mixed_ms"] / 1000.0), "unit": UNIT,
                            "ms_per_step": r["mixed_ms"] / args.steps,
                            "speedup_vs_fp64": (r["mixed_updates"] / r["mixed_ms"]) / (updates / (dev_s * 1000.0)),
                            "note": "FP32 H_ij, p_gen and spawn amplitude; FP64 death, E_proj and signs"},
    }
    if not args.no_batched and world == 1:
        line["batched"] = run_batched(args)
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline_sample()
    print(json.dumps(line))
    eng.close()


if __name__ == "__main__":
    main()
