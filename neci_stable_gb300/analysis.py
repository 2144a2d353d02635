"""Blocking analysis of the FCIQMC estimators (ErrorAnalysis.F90).

Restates automatic_reblocking_analysis (:374-458): the series is reblocked
by factors of two, the standard error is computed at every level
(analyze_data, :912), and the largest error among all but the last two
levels is taken (find_max_error, :1095).  The projected energy is the ratio
of the numerator and denominator means, with the error propagated through
their covariance at the longer of the two correlation lengths
(error_analysis, :27-300).
"""
from __future__ import annotations

import math

import numpy as np


def analyze_data(x: np.ndarray):
    n = x.size
    mean = float(x.sum() / n)
    mean2 = float((x * x).sum() / n)
    var = max(mean2 - mean * mean, 0.0)
    err = math.sqrt(var / (n - 1)) if n > 1 else 0.0
    eie = err / math.sqrt(2.0 * (n - 1)) if n > 1 else 0.0
    return mean, err, eie


def reblock(x: np.ndarray, b: int = 2) -> np.ndarray:
    n = (x.size // b) * b
    return x[:n].reshape(-1, b).mean(axis=1)


def automatic_reblocking(x: np.ndarray, blocklength: int = 2):
    """Returns (mean, error, correlation length in samples)."""
    x = np.asarray(x, dtype=float)
    if x.size < 4:
        m, e, _ = analyze_data(x)
        return m, e, 1
    events = int(math.log(x.size) / math.log(2.0) - 1.0)
    errs = []
    mean0, e0, _ = analyze_data(x)
    errs.append(e0)
    y = x.copy()
    for _ in range(events):
        y = reblock(y, blocklength)
        if y.size < 2:
            break
        errs.append(analyze_data(y)[1])
    best, which = errs[0], 0
    for i in range(1, len(errs) - 2):
        if errs[i] > best:
            best, which = errs[i], i
    return mean0, best, blocklength ** which


def projected_energy(num: np.ndarray, den: np.ndarray, offset: float = 0.0):
    """E_proj = offset + <num>/<den> with its blocked error."""
    num = np.asarray(num, dtype=float)
    den = np.asarray(den, dtype=float)
    mn, en, cn = automatic_reblocking(num)
    md, ed, cd = automatic_reblocking(den)
    corr = max(cn, cd)
    bn, bd = reblock(num, corr) if corr > 1 else num, reblock(den, corr) if corr > 1 else den
    nb = bn.size
    cov = float(np.mean((bn - bn.mean()) * (bd - bd.mean()))) / max(nb - 1, 1)
    e = mn / md
    en2 = analyze_data(bn)[1] if nb > 1 else en
    ed2 = analyze_data(bd)[1] if nb > 1 else ed
    rel2 = (en2 / mn) ** 2 + (ed2 / md) ** 2 - 2.0 * cov / (mn * md) if mn != 0 else 0.0
    return offset + e, abs(e) * math.sqrt(max(rel2, 0.0))
