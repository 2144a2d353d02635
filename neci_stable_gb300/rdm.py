"""Host side of the stochastic 2-RDM: normalisation and the RDM energy.

The device accumulates, for a replica pair, the unnormalised spin-orbital
2-RDM  G[pair(p,q), pair(r,s)] ~ <Psi_1| a+_p a+_q a_s a_r |Psi_2>  with
p < q, r < s and pair(p,q) = (q-1)(q-2)/2 + (p-1) for 1-based spin orbitals
(neci_gpu_get_rdm).  As the reference does before it prints an RDM energy
(rdm_estimators.F90, calc_rdm_energy), the matrix is made Hermitian and
divided by its norm: the trace of the pair diagonal is N(N-1)/2 <Psi_1|Psi_2>.

  E_RDM = sum_pr h_pr gamma_pr + sum_{p<q, r<s} G(pq, rs) (<pq|rs> - <pq|sr>)
          + E_core,  gamma_pr = 1/(N-1) sum_q G(pq, rq)

with h = TMat2D and <pq|rs> = <ij|kl> of the spatial orbitals (UMAT) when
the spins of p, r and of q, s agree.
"""
from __future__ import annotations

import numpy as np


def pair_index(p, q):
    """pair(p, q) for 1-based spin orbitals p < q (vectorised)."""
    return (q - 1) * (q - 2) // 2 + (p - 1)


def pairs(nbasis: int):
    """All (p, q), p < q, in pair order."""
    ps, qs = [], []
    for q in range(2, nbasis + 1):
        for p in range(1, q):
            ps.append(p)
            qs.append(q)
    return np.array(ps), np.array(qs)


def _umat_ind(i, j, k, l):
    a = np.where(i > k, i * (i - 1) // 2 + k, k * (k - 1) // 2 + i)
    b = np.where(j > l, j * (j - 1) // 2 + l, l * (l - 1) // 2 + j)
    return np.where(a > b, a * (a - 1) // 2 + b, b * (b - 1) // 2 + a)


def antisym_integrals(spec) -> np.ndarray:
    """A[pair(p,q), pair(r,s)] = <pq|rs> - <pq|sr> in spin orbitals."""
    P, Q = pairs(spec.nbasis)
    sp = lambda o: (o + 1) // 2  # noqa: E731
    be = lambda o: o & 1  # noqa: E731
    u = np.asarray(spec.umat)

    def phys(p, q, r, s):  # <pq|rs> over the outer product of bra and ket pairs
        val = u[_umat_ind(sp(p)[:, None], sp(q)[:, None], sp(r)[None, :], sp(s)[None, :]) - 1]
        ok = (be(p)[:, None] == be(r)[None, :]) & (be(q)[:, None] == be(s)[None, :])
        return np.where(ok, val, 0.0)

    return phys(P, Q, P, Q) - phys(P, Q, Q, P)


def symmetrise(G: np.ndarray) -> np.ndarray:
    return 0.5 * (G + G.T)


def one_rdm(G: np.ndarray, nbasis: int, nel: int) -> np.ndarray:
    """gamma_pr = 1/(N-1) sum_q G(pq, rq), signs from the pair ordering."""
    gam = np.zeros((nbasis, nbasis))
    for p in range(1, nbasis + 1):
        for r in range(1, nbasis + 1):
            acc = 0.0
            for q in range(1, nbasis + 1):
                if q == p or q == r:
                    continue
                bra = pair_index(min(p, q), max(p, q))
                ket = pair_index(min(r, q), max(r, q))
                sgn = (1 if p < q else -1) * (1 if r < q else -1)
                acc += sgn * G[bra, ket]
            gam[p - 1, r - 1] = acc / (nel - 1)
    return gam


def rdm_energy(G: np.ndarray, spec, A: np.ndarray | None = None) -> dict:
    """Energy and norm of an unnormalised 2-RDM (made Hermitian first)."""
    nb, N = spec.nbasis, spec.nel
    Gs = symmetrise(G)
    norm = np.trace(Gs) / (N * (N - 1) / 2)
    if A is None:
        A = antisym_integrals(spec)
    e2 = float(np.sum(Gs * A))
    h = np.asarray(spec.tmat).reshape(nb, nb).T  # TMat2D is column-major: h[p, r] = TMat2D(p, r)
    gam = one_rdm(Gs, nb, N)
    e1 = float(np.sum(h * gam))
    return {"energy": (e1 + e2) / norm + spec.ecore, "norm": float(norm), "one_body": e1 / norm,
            "two_body": e2 / norm}
