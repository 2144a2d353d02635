"""Independent Hamiltonian in second quantisation -- TEST INFRASTRUCTURE.

Builds <D_i|H|D_j> by applying creation/annihilation operators to bit-string
determinants, with fermionic signs counted in NECI's spin-orbital order
(orbital p = bit p-1; odd orbitals beta).  It shares no code with the
Slater-Condon rules of the oracle or the engine, so it pins their sign and
integral-index conventions:

    H = sum_{pq} t_pq a+_p a_q + 1/2 sum_{pqrs} <pq|rs> a+_p a+_q a_s a_r,
    <pq|rs> = (pr|qs) for spin orbitals (chemist (..|..) over spatial orbitals,
    spin conserved on each electron), or U n_{i,up} n_{i,down} for Hubbard.
"""
from __future__ import annotations

import numpy as np


def _annihilate(det, q):
    if not (det >> (q - 1)) & 1:
        return None, 0
    sign = -1 if bin(det & ((1 << (q - 1)) - 1)).count("1") & 1 else 1
    return det ^ (1 << (q - 1)), sign


def _create(det, p):
    if (det >> (p - 1)) & 1:
        return None, 0
    sign = -1 if bin(det & ((1 << (p - 1)) - 1)).count("1") & 1 else 1
    return det | (1 << (p - 1)), sign


def apply_h(det, nbasis, tmat, eri=None, uhub=None, ecore=0.0):
    """Returns {det': amplitude} of H|det> (det as a Python int bit mask)."""
    out = {}

    def add(d, v):
        if v != 0.0:
            out[d] = out.get(d, 0.0) + v

    occ = [p for p in range(1, nbasis + 1) if (det >> (p - 1)) & 1]
    # one-body
    for q in occ:
        d1, s1 = _annihilate(det, q)
        for p in range(1, nbasis + 1):
            t = tmat[p - 1, q - 1]
            if t == 0.0:
                continue
            d2, s2 = _create(d1, p)
            if d2 is None:
                continue
            add(d2, t * s1 * s2)
    if uhub is not None:
        n = sum(1 for s in range(1, nbasis // 2 + 1) if (det >> (2 * s - 2)) & 1 and (det >> (2 * s - 1)) & 1)
        add(det, uhub * n)
    if eri is not None:
        spat = lambda o: (o + 1) // 2  # noqa: E731
        for r in occ:
            dr, sr = _annihilate(det, r)
            for s in occ:
                if s == r:
                    continue
                ds, ss = _annihilate(dr, s)
                for q in range(1, nbasis + 1):
                    if (q & 1) != (s & 1):
                        continue
                    dq, sq = _create(ds, q)
                    if dq is None:
                        continue
                    for p in range(1, nbasis + 1):
                        if (p & 1) != (r & 1):
                            continue
                        v = eri[spat(p) - 1, spat(r) - 1, spat(q) - 1, spat(s) - 1]
                        if v == 0.0:
                            continue
                        dp, sp = _create(dq, p)
                        if dp is None:
                            continue
                        add(dp, 0.5 * v * sr * ss * sq * sp)
    if ecore:
        add(det, ecore)
    return out


def hamiltonian(dets_int, nbasis, tmat, eri=None, uhub=None, ecore=0.0):
    index = {d: i for i, d in enumerate(dets_int)}
    H = np.zeros((len(dets_int), len(dets_int)))
    for j, d in enumerate(dets_int):
        for d2, v in apply_h(d, nbasis, tmat, eri, uhub, ecore).items():
            if d2 in index:
                H[index[d2], j] += v
    return H


def rdm2_from_vector(dets, vec, nbasis):
    """Exact spin-orbital 2-RDM of a CI vector by operators:
    G[pair(p,q), pair(r,s)] = sum_IJ c_I c_J <D_I| a+_p a+_q a_s a_r |D_J>,
    p < q, r < s, pair(p,q) = (q-1)(q-2)/2 + (p-1); dets are Python ints."""
    npair = nbasis * (nbasis - 1) // 2
    G = np.zeros((npair, npair))
    index = {d: i for i, d in enumerate(dets)}
    pair = lambda p, q: (q - 1) * (q - 2) // 2 + (p - 1)  # noqa: E731
    for j, dj in enumerate(dets):
        cj = vec[j]
        if cj == 0.0:
            continue
        occ = [p for p in range(1, nbasis + 1) if (dj >> (p - 1)) & 1]
        for ir, r in enumerate(occ):
            for s in occ[ir + 1:]:
                d1, s1 = _annihilate(dj, r)
                d2, s2 = _annihilate(d1, s)  # a_s a_r |D_J>
                for q in range(2, nbasis + 1):
                    d3, s3 = _create(d2, q)
                    if d3 is None:
                        continue
                    for p in range(1, q):
                        d4, s4 = _create(d3, p)  # a+_p a+_q a_s a_r |D_J>
                        if d4 is None or d4 not in index:
                            continue
                        G[pair(p, q), pair(r, s)] += vec[index[d4]] * cj * s1 * s2 * s3 * s4
    return G
