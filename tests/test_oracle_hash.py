"""The oracle's FindWalkerHash pinned to a plain-integer statement of
hash.F90:23-38, on the CPU:

    hash = 0
    do i = 1, nel:  hash = 1099511628211 * hash + RandomHash2(nI(i)) * i
    hashInd = abs(mod(hash, HashIndexLength)) + 1

over the decoded occupied orbitals nI in increasing order, with the int64
products wrapping (two's complement) and Fortran's mod taking the sign of the
dividend.  Covered: one and three determinant words, power-of-two and other
table lengths."""
from __future__ import annotations

import numpy as np
import pytest

from neci_stable_gb300 import systems
from oracle.oracle import Oracle

FNV = 1099511628211


def _wrap64(x: int) -> int:
    x &= (1 << 64) - 1
    return x - (1 << 64) if x >> 63 else x


def find_walker_hash(orbs, random_hash2, length: int) -> int:
    h = 0
    for i, o in enumerate(orbs, start=1):
        h = _wrap64(FNV * h + int(random_hash2[o - 1]) * i)
    r = abs(h) % length          # |mod(h, N)| = |h| mod N for Fortran's truncating mod
    return r + 1


@pytest.mark.parametrize("dims,nel", [((8,), 8), ((8, 8), 40)], ids=["chain-8 (1 word)", "square-8x8 (3 words)"])
@pytest.mark.parametrize("length", [1, 7, 700, 1 << 16, 1_000_003])
def test_find_walker_hash_restated(dims, nel, length):
    spec = systems.hubbard_system("chain" if len(dims) == 1 else "square", dims, nel, u=4.0)
    orc = Oracle(spec, 64, 64)
    rng = np.random.default_rng(length)
    nb = spec.nbasis
    orb_lists = [sorted(rng.choice(np.arange(1, nb + 1), nel, replace=False).tolist()) for _ in range(400)]
    dets = np.array([systems.encode_det(o, spec.nifd) for o in orb_lists], dtype=np.int64)
    got = orc.find_walker_hash(dets, length)
    expect = [find_walker_hash(o, spec.random_hash2, length) for o in orb_lists]
    assert list(map(int, got)) == expect
    assert all(1 <= e <= length for e in expect)
