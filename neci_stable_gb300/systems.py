"""Host-side system set-up: what NECI's Fortran host does before the loop.

* Real-space Hubbard lattices (``system hubbard real-space`` + ``lattice``,
  System_neci.F90:336-372, 1007-1040): neighbour tables and TMat2D
  (real_space_hubbard.F90:751 init_tmat, hopping ``bhub`` between
  neighbouring sites, same spin).
* Molecular integrals: FCIDUMP reading/writing in the format of
  readint.F90:32-238, 585-950, the 8-fold packed UMAT of UMatCache.F90:257
  (UMAT(UMatInd(i,k,j,l)) = (ij|kl), readint.F90:889) and TMat2D over spin
  orbitals, plus the seeded synthetic FCIDUMP recipe used for benchmarks.
* RandomHash2 (fcimc_initialisation.fpp:886-905): distinct integers in
  1..nBasis*1000, one per spin orbital.
* Determinant bit strings in NECI's layout (spin orbital p -> bit (p-1)%64 of
  word (p-1)//64; odd orbitals beta, even alpha).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import capi


# --------------------------------------------------------------------------- bits
def nifd_for(nbasis: int) -> int:
    """NIfD = nBasis/64 (BitReps.F90:174)."""
    return nbasis // 64


def encode_det(orbs, nifd: int) -> np.ndarray:
    """EncodeBitDet: sorted spin orbitals (1-based) -> int64 words."""
    w = np.zeros(nifd + 1, dtype=np.uint64)
    for o in orbs:
        w[(o - 1) // 64] |= np.uint64(1) << np.uint64((o - 1) % 64)
    return w.view(np.int64)


def decode_det(words) -> list[int]:
    out = []
    for wi, x in enumerate(np.asarray(words, dtype=np.int64).view(np.uint64)):
        x = int(x)
        b = 0
        while x:
            if x & 1:
                out.append(wi * 64 + b + 1)
            x >>= 1
            b += 1
    return out


def make_rows(dets: np.ndarray, signs: np.ndarray, flags: np.ndarray | None = None) -> np.ndarray:
    """CurrentDets rows from det words (n, W), signs (n, L) and flag words."""
    dets = np.atleast_2d(np.asarray(dets, dtype=np.int64))
    signs = np.asarray(signs, dtype=np.float64)
    if signs.ndim == 1:
        signs = signs[:, None]
    n, W = dets.shape
    L = signs.shape[1]
    rows = np.zeros((n, W + L + 1), dtype=np.int64)
    rows[:, :W] = dets
    rows[:, W:W + L] = np.ascontiguousarray(signs).view(np.int64)
    if flags is not None:
        rows[:, W + L] = flags
    return rows


def random_hash2(nbasis: int, seed: int) -> np.ndarray:
    """RandomHash2: distinct values in 1..nBasis*1000 (fcimc_initialisation.fpp:886)."""
    rng = np.random.default_rng(seed)
    vals = rng.choice(nbasis * 1000, size=nbasis, replace=False) + 1
    return vals.astype(np.int32)


# ----------------------------------------------------------------------- Hubbard
def chain_neighbours(nsites: int, periodic: bool = True) -> np.ndarray:
    nb = np.zeros((nsites, 2), dtype=np.int32)
    for s in range(1, nsites + 1):
        left, right = s - 1, s + 1
        if periodic:
            left = nsites if left < 1 else left
            right = 1 if right > nsites else right
        nb[s - 1, 0] = left if left >= 1 else 0
        nb[s - 1, 1] = right if right <= nsites else 0
        if nsites == 2 and periodic:
            nb[s - 1, 1] = 0  # a 2-site ring has one distinct neighbour
    return nb


def square_neighbours(lx: int, ly: int, periodic: bool = True) -> np.ndarray:
    def idx(x, y):
        return (y % ly) * lx + (x % lx) + 1

    nb = np.zeros((lx * ly, 4), dtype=np.int32)
    for y in range(ly):
        for x in range(lx):
            s = idx(x, y) - 1
            cand = [(x - 1, y), (x + 1, y), (x, y - 1), (x, y + 1)]
            for k, (cx, cy) in enumerate(cand):
                if not periodic and not (0 <= cx < lx and 0 <= cy < ly):
                    continue
                nb[s, k] = idx(cx, cy)
    return nb


def hubbard_tmat(neighbours: np.ndarray, bhub: float) -> np.ndarray:
    """TMat2D(nBasis, nBasis), Fortran order (returned as a C array of the
    transposed matrix, i.e. memory order of the Fortran array)."""
    nsites = neighbours.shape[0]
    nb = 2 * nsites
    t = np.zeros((nb, nb))
    for s in range(1, nsites + 1):
        for n in neighbours[s - 1]:
            if n <= 0:
                continue
            for spin in (1, 0):  # beta (odd), alpha (even)
                i, j = 2 * s - spin, 2 * n - spin
                t[i - 1, j - 1] = bhub
    return np.ascontiguousarray(t.T)  # column-major memory of t


def neel_reference(nsites: int, nel: int, neighbours: np.ndarray | None = None) -> list[int]:
    """A closed-shell-free Sz=0 reference: alternating spins (chain / checkerboard)."""
    if nel != nsites:
        # fill lowest sites alternately
        orbs = []
        for s in range(1, nel + 1):
            orbs.append(2 * s if s % 2 else 2 * s - 1)
        return sorted(orbs)
    side = int(round(math.sqrt(nsites)))
    orbs = []
    for s in range(1, nsites + 1):
        if neighbours is not None and neighbours.shape[1] == 4 and side * side == nsites:
            x, y = (s - 1) % side, (s - 1) // side
            up = (x + y) % 2 == 0
        else:
            up = s % 2 == 1
        orbs.append(2 * s if up else 2 * s - 1)
    return sorted(orbs)


# --------------------------------------------------------------------- integrals
def umat_index(i, j, k, l):
    """UMatInd_base (UMatCache.F90:257), vectorised, 1-based spatial indices."""
    i, j, k, l = (np.asarray(v, dtype=np.int64) for v in (i, j, k, l))
    A = np.where(i > k, i * (i - 1) // 2 + k, k * (k - 1) // 2 + i)
    B = np.where(j > l, j * (j - 1) // 2 + l, l * (l - 1) // 2 + j)
    return np.where(A > B, A * (A - 1) // 2 + B, B * (B - 1) // 2 + A)


def umat_length(n: int) -> int:
    P = n * (n + 1) // 2
    return P * (P + 1) // 2


def pack_umat(eri: np.ndarray) -> np.ndarray:
    """UMAT from chemist-notation (pq|rs): UMAT(UMatInd(i,k,j,l)) = (ij|kl)."""
    n = eri.shape[0]
    u = np.zeros(umat_length(n))
    I, J, K, Lx = np.meshgrid(*(np.arange(1, n + 1),) * 4, indexing="ij")
    idx = umat_index(I, K, J, Lx).ravel() - 1
    u[idx] = eri.ravel()
    return u


def spin_tmat(h: np.ndarray) -> np.ndarray:
    """TMat2D over spin orbitals from spatial h_pq (memory order of the Fortran array)."""
    n = h.shape[0]
    t = np.zeros((2 * n, 2 * n))
    t[0::2, 0::2] = h  # beta-beta (odd orbitals)
    t[1::2, 1::2] = h  # alpha-alpha
    return np.ascontiguousarray(t.T)


def synthetic_fcidump(n: int, seed: int):
    """Seeded synthetic molecular integrals (C1, real, PSD ERIs).

    eps_p = -1.5 + 2.5 p/(n-1); h_pq = eps_p delta_pq + N(0, 0.02) e^{-|p-q|/4}
    (symmetrised); (pq|rs) = sum_{L=1}^{3n} B^L_pq B^L_rs with symmetric B^L of
    N(0, 0.3/sqrt(n)) e^{-|p-q|/4} entries; core energy 0.
    """
    rng = np.random.default_rng(seed)
    p = np.arange(n)
    decay = np.exp(-np.abs(p[:, None] - p[None, :]) / 4.0)
    eps = -1.5 + 2.5 * p / (n - 1)
    g = rng.normal(0.0, 0.02, size=(n, n)) * decay
    h = np.diag(eps) + 0.5 * (g + g.T)
    B = rng.normal(0.0, 0.3 / math.sqrt(n), size=(3 * n, n, n)) * decay[None]
    B = 0.5 * (B + B.transpose(0, 2, 1))
    eri = np.einsum("Lpq,Lrs->pqrs", B, B, optimize=True)
    eri = 0.5 * (eri + eri.transpose(2, 3, 0, 1))  # exact (pq|rs) = (rs|pq)
    return h, eri, 0.0


def write_fcidump(path, h, eri, ecore, nelec, ms2=0, tol=1e-14):
    n = h.shape[0]
    with open(path, "w") as f:
        f.write(f" &FCI NORB={n},NELEC={nelec},MS2={ms2},\n  ORBSYM={','.join(['1'] * n)},\n  ISYM=1,\n &END\n")
        for i in range(1, n + 1):
            for j in range(1, i + 1):
                for k in range(1, n + 1):
                    for l in range(1, k + 1):
                        if (i * (i - 1) // 2 + j) < (k * (k - 1) // 2 + l):
                            continue
                        v = eri[i - 1, j - 1, k - 1, l - 1]
                        if abs(v) > tol:
                            f.write(f" {v: .16E} {i:4d} {j:4d} {k:4d} {l:4d}\n")
        for i in range(1, n + 1):
            for j in range(1, i + 1):
                v = h[i - 1, j - 1]
                if abs(v) > tol:
                    f.write(f" {v: .16E} {i:4d} {j:4d}    0    0\n")
        f.write(f" {ecore: .16E}    0    0    0    0\n")


def read_fcidump(path):
    """FCIDUMP -> (h, eri, ecore, nelec, ms2) with 8-fold symmetry (readint.F90:585)."""
    text = open(path).read()
    head, body = text.split("&END", 1) if "&END" in text else text.split("/", 1)
    hd = head.replace("\n", " ").upper()

    def grab(key):
        import re
        m = re.search(key + r"\s*=\s*(-?\d+)", hd)
        return int(m.group(1)) if m else None

    n, nelec, ms2 = grab("NORB"), grab("NELEC"), grab("MS2") or 0
    h = np.zeros((n, n))
    eri = np.zeros((n, n, n, n))
    ecore = 0.0
    for line in body.splitlines():
        parts = line.split()
        if len(parts) != 5:
            continue
        v = float(parts[0].replace("D", "E"))
        i, j, k, l = (int(x) for x in parts[1:])
        if i == j == k == l == 0:
            ecore = v
        elif j == 0 and k == 0 and l == 0:
            continue  # orbital energies (readint.F90 ignores them for the integrals)
        elif k == 0 and l == 0:
            h[i - 1, j - 1] = h[j - 1, i - 1] = v
        else:
            for a, b, c, d in ((i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                               (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)):
                eri[a - 1, b - 1, c - 1, d - 1] = v
    return h, eri, ecore, nelec, ms2


def aufbau_reference(n: int, nel: int, ms2: int = 0) -> list[int]:
    na = (nel + ms2) // 2
    nb_ = nel - na
    return sorted([2 * p for p in range(1, na + 1)] + [2 * p - 1 for p in range(1, nb_ + 1)])


def fock_diagonal(h: np.ndarray, eri: np.ndarray, occ) -> np.ndarray:
    """Closed-shell Fock diagonal f_pp = h_pp + sum_c [2 (pp|cc) - (pc|cp)] over
    the doubly occupied spatial orbitals c (0-based)."""
    occ = np.asarray(list(occ), dtype=np.int64)
    p = np.arange(h.shape[0])
    J = eri[p, p][:, occ, occ].sum(axis=1)
    K = eri[p[:, None], occ[None, :], occ[None, :], p[:, None]].sum(axis=1)
    return np.diag(h) + 2.0 * J - K


def fock_ordered_occupation(h: np.ndarray, eri: np.ndarray, nocc: int, max_iter: int = 100) -> list[int]:
    """The nocc spatial orbitals (0-based, sorted) of lowest closed-shell Fock
    energy, iterated to self-consistency of the occupation.  NECI orders its
    basis by orbital energy before filling the reference (Fermi det) and
    before choosing the orbitals to freeze (SysReadInput ... freeze)."""
    occ = tuple(sorted(np.argsort(np.diag(h), kind="stable")[:nocc].tolist()))
    for _ in range(max_iter):
        nxt = tuple(sorted(np.argsort(fock_diagonal(h, eri, occ), kind="stable")[:nocc].tolist()))
        if nxt == occ:
            break
        occ = nxt
    return list(occ)


def freeze_core(h: np.ndarray, eri: np.ndarray, ecore: float, frozen):
    """Fold doubly occupied frozen spatial orbitals (0-based) into the core
    energy and the one-electron integrals (the 'freeze' of IntFreeze,
    Integrals_neci.F90):
        E_core' = E_core + sum_c 2 h_cc + sum_cd [2 (cc|dd) - (cd|dc)]
        h'_pq  = h_pq + sum_c [2 (pq|cc) - (pc|cq)]
    and drop the frozen orbitals.  Returns (h', eri', E_core', active)."""
    frozen = np.asarray(sorted(frozen), dtype=np.int64)
    n = h.shape[0]
    active = np.array([p for p in range(n) if p not in set(frozen.tolist())], dtype=np.int64)
    ec = float(ecore)
    if frozen.size:
        ec += 2.0 * float(np.trace(h[np.ix_(frozen, frozen)]))
        ec += float(sum(2.0 * eri[c, c, d, d] - eri[c, d, d, c] for c in frozen for d in frozen))
    h2 = h.copy()
    for c in frozen:
        h2 += 2.0 * eri[:, :, c, c] - eri[:, c, c, :]
    h2 = h2[np.ix_(active, active)]
    eri2 = eri[np.ix_(active, active, active, active)]
    return np.ascontiguousarray(h2), np.ascontiguousarray(eri2), ec, active.tolist()


def closed_shell_reference(occ_spatial) -> list[int]:
    """Spin orbitals (1-based; beta odd, alpha even) of a closed-shell
    determinant on the given 0-based spatial orbitals."""
    return sorted([2 * p + 1 for p in occ_spatial] + [2 * p + 2 for p in occ_spatial])


def p_singles_from_reference(n: int, nalpha: int, nbeta: int) -> float:
    """pSingles = nSingles / (nSingles + nDoubles) counted from the reference (C1)."""
    ua, ub = n - nalpha, n - nbeta
    ns = nalpha * ua + nbeta * ub
    nd = (math.comb(nalpha, 2) * math.comb(ua, 2) + math.comb(nbeta, 2) * math.comb(ub, 2)
          + nalpha * nbeta * ua * ub)
    return ns / (ns + nd)


# ------------------------------------------------------------------ descriptions
@dataclass
class SystemSpec:
    """Everything the engine needs for one system (mirrors neci_gpu_system + tables)."""
    kind: int
    nel: int
    nbasis: int
    tmat: np.ndarray
    reference: list
    random_hash2: np.ndarray
    umat: np.ndarray | None = None
    neighbours: np.ndarray | None = None
    uhub: float = 0.0
    bhub: float = 0.0
    ecore: float = 0.0
    p_singles: float = 0.0
    p_parallel: float = 0.5
    lenof_sign: int = 1
    name: str = ""
    extra: dict = field(default_factory=dict)
    excitgen: int | None = None          # NECI_EXGEN_*; None: rs-Hubbard for lattices, PCHB for FCIDUMPs

    @property
    def generator(self) -> int:
        if self.excitgen is not None:
            return self.excitgen
        return capi.EXGEN_RS_HUBBARD if self.kind == capi.SYS_HUBBARD_REAL_SPACE else capi.EXGEN_PCHB

    @property
    def nifd(self) -> int:
        return nifd_for(self.nbasis)

    @property
    def W(self) -> int:
        return self.nifd + 1

    def c_system(self, max_walkers: int, max_spawned: int, hash_frac: float = 0.7) -> capi.System:
        s = capi.System()
        s.nel, s.nbasis, s.nifd, s.lenof_sign = self.nel, self.nbasis, self.nifd, self.lenof_sign
        s.system = self.kind
        s.excitgen = self.generator
        s.max_neighbours = 0 if self.neighbours is None else int(self.neighbours.shape[1])
        s.uhub, s.bhub, s.ecore = self.uhub, self.bhub, self.ecore
        s.p_singles, s.p_parallel = self.p_singles, self.p_parallel
        s.max_walkers, s.max_spawned = int(max_walkers), int(max_spawned)
        s.n_walker_hashes = int(max(16, hash_frac * max_walkers))
        return s


def hubbard_system(kind: str, dims, nel: int, u: float, t: float = 1.0, seed: int = 7,
                   lenof_sign: int = 1) -> SystemSpec:
    """``system hubbard real-space`` with ``lattice chain L`` or ``square Lx Ly`` (PBC), b = -t."""
    if kind == "chain":
        nb = chain_neighbours(dims[0])
    elif kind == "square":
        nb = square_neighbours(dims[0], dims[1])
    else:
        raise ValueError(kind)
    nsites = nb.shape[0]
    bhub = -t
    ref = neel_reference(nsites, nel, nb)
    return SystemSpec(kind=capi.SYS_HUBBARD_REAL_SPACE, nel=nel, nbasis=2 * nsites, tmat=hubbard_tmat(nb, bhub),
                      reference=ref, random_hash2=random_hash2(2 * nsites, seed), neighbours=nb, uhub=u,
                      bhub=bhub, lenof_sign=lenof_sign, name=f"hubbard-{kind}-{'x'.join(map(str, dims))}")


def molecular_system(h, eri, ecore, nel: int, ms2: int = 0, seed: int = 7, lenof_sign: int = 1,
                     p_parallel: float = 0.5, name: str = "fcidump", reference=None,
                     excitgen: int = capi.EXGEN_PCHB) -> SystemSpec:
    """A molecular system from spatial integrals; the reference defaults to
    the aufbau determinant in orbital index order."""
    n = h.shape[0]
    ref = sorted(reference) if reference is not None else aufbau_reference(n, nel, ms2)
    na = sum(1 for o in ref if o % 2 == 0)
    return SystemSpec(kind=capi.SYS_MOLECULAR, nel=nel, nbasis=2 * n, tmat=spin_tmat(h), reference=ref,
                      random_hash2=random_hash2(2 * n, seed), umat=pack_umat(eri), ecore=ecore,
                      p_singles=p_singles_from_reference(n, na, nel - na), p_parallel=p_parallel,
                      lenof_sign=lenof_sign, name=name, excitgen=excitgen)
