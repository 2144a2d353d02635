"""Shared fixtures of the parity tests: systems, random determinants and
walker lists, and comparison of walker lists independent of slot order."""
from __future__ import annotations

import numpy as np

from neci_stable_gb300 import capi, systems
from neci_stable_gb300.systems import encode_det, make_rows


def hubbard10(lenof_sign=1):
    return systems.hubbard_system("chain", (10,), 10, u=4.0, lenof_sign=lenof_sign)


def hubbard_square(lx, ly, nel, lenof_sign=1):
    return systems.hubbard_system("square", (lx, ly), nel, u=4.0, lenof_sign=lenof_sign)


def molecule(n, nel, seed=11, lenof_sign=1):
    h, eri, ecore = systems.synthetic_fcidump(n, seed)
    return systems.molecular_system(h, eri, ecore, nel, seed=seed + 1, lenof_sign=lenof_sign, name=f"synthetic-{n}")


def molecule_uniform(n, nel, seed=11, lenof_sign=1):
    h, eri, ecore = systems.synthetic_fcidump(n, seed)
    return systems.molecular_system(h, eri, ecore, nel, seed=seed + 1, lenof_sign=lenof_sign,
                                    name=f"synthetic-{n}-uniform", excitgen=capi.EXGEN_UNIFORM)


def ne_frozen_system(lenof_sign=1):
    """NECI's Ne PCHB test input (FCIDUMP of test_suite/neci/parallel/
    Ne_FciMCPar_pchb, 'freeze 2 0'): the lowest spatial orbital by Fock
    energy is frozen, the reference fills the next four.  Returns (spec, fixture)."""
    from pathlib import Path
    d = np.load(Path(__file__).parent / "golden" / "ne_pchb_fcidump.npz")
    h, eri, ecore = d["h"], d["eri"], float(d["ecore"])
    nocc = int(d["nelec"]) // 2
    occ = systems.fock_ordered_occupation(h, eri, nocc)
    f = systems.fock_diagonal(h, eri, occ)
    frozen = [int(np.argmin(f))]
    h2, eri2, ec2, active = systems.freeze_core(h, eri, ecore, frozen)
    ref = systems.closed_shell_reference([active.index(p) for p in occ if p not in frozen])
    spec = systems.molecular_system(h2, eri2, ec2, int(d["nelec"]) - 2, reference=ref, lenof_sign=lenof_sign,
                                    name="Ne-frozen")
    return spec, d


def random_dets(spec, n, rng):
    """n random determinants with the reference's alpha/beta counts."""
    ref = spec.reference
    na = sum(1 for o in ref if o % 2 == 0)
    nb = spec.nel - na
    norb = spec.nbasis // 2
    out = np.zeros((n, spec.W), dtype=np.int64)
    for i in range(n):
        a = rng.choice(norb, size=na, replace=False) + 1
        b = rng.choice(norb, size=nb, replace=False) + 1
        out[i] = encode_det(sorted([2 * p for p in a] + [2 * p - 1 for p in b]), spec.nifd)
    return out


def excite(spec, det, level, rng):
    """A determinant `level` spin-conserving excitations away from det."""
    occ = systems.decode_det(det)
    unocc = [o for o in range(1, spec.nbasis + 1) if o not in occ]
    for _ in range(1000):
        src = list(rng.choice(occ, size=level, replace=False))
        tgt = []
        ok = True
        for s in src:
            cands = [u for u in unocc if (u % 2) == (s % 2) and u not in tgt]
            if not cands:
                ok = False
                break
            tgt.append(int(rng.choice(cands)))
        if ok:
            new = sorted((set(occ) - set(src)) | set(tgt))
            return encode_det(new, spec.nifd)
    raise RuntimeError("no excitation")


def random_walkers(spec, n, rng, scale=8.0, quantum=1.0 / 64, with_flags=True):
    """Occupied rows with signs that are multiples of `quantum` (exact in fixed point)."""
    dets = np.unique(random_dets(spec, n, rng), axis=0)
    L = spec.lenof_sign
    signs = np.round(rng.normal(0.0, scale, size=(dets.shape[0], L)) / quantum) * quantum
    signs[signs == 0] = quantum
    flags = np.zeros(dets.shape[0], dtype=np.int64)
    if with_flags:
        for k in range(L):
            flags |= (rng.random(dets.shape[0]) < 0.5).astype(np.int64) << capi.FLAG_INITIATOR[k]
    return make_rows(dets, signs, flags)


def random_spawns(spec, walkers, n, rng, quantum=1.0 / 64, p_hit=0.5):
    """Spawn records: half onto existing determinants, half onto new ones,
    with duplicates, opposite signs and random initiator flags."""
    W, L = spec.W, spec.lenof_sign
    existing = walkers[:, :W]
    fresh = random_dets(spec, max(n // 4, 1), rng)
    dets = np.zeros((n, W), dtype=np.int64)
    for i in range(n):
        if rng.random() < p_hit and existing.shape[0]:
            dets[i] = existing[rng.integers(existing.shape[0])]
        else:
            dets[i] = fresh[rng.integers(fresh.shape[0])]
    signs = np.zeros((n, L))
    run = rng.integers(L, size=n)
    vals = np.round(rng.normal(0.0, 1.5, size=n) / quantum) * quantum
    vals[vals == 0] = quantum
    signs[np.arange(n), run] = vals
    flags = np.zeros(n, dtype=np.int64)
    init = rng.random(n) < 0.4
    flags[init] = np.int64(1) << np.array([capi.FLAG_INITIATOR[r] for r in run[init]], dtype=np.int64)
    return make_rows(dets, signs, flags)


def canonical(rows, W):
    """Rows sorted by determinant words (slot order is not part of the result)."""
    rows = np.asarray(rows, dtype=np.int64)
    if rows.shape[0] == 0:
        return rows
    order = np.lexsort(tuple(rows[:, w] for w in reversed(range(W))))
    return rows[order]


def canonical_with(rows, extra, W):
    rows = np.asarray(rows, dtype=np.int64)
    order = np.lexsort(tuple(rows[:, w] for w in reversed(range(W))))
    return rows[order], [np.asarray(e)[order] for e in extra]
