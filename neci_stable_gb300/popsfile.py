"""POPSFILE version 4: the restart file of a NECI run (Popsfile.F90).

The engine keeps the walker list in HBM in CurrentDets layout; a POPSFILE is
written from ``Engine.download()`` and read back into ``Engine.upload()``.
Both file forms of the reference are restated:

* text: header and records in one file ``POPSFILE`` (``tBinPops`` off);
* binary: the header in ``POPSFILEHEAD`` and the records in ``POPSFILEBIN``
  as Fortran unformatted sequential records (``tBinPops``).

Header: write_popsfile_header (Popsfile.F90:1951-2052), a Fortran namelist
``&POPSHEAD ... &END`` read back by ReadPopsHeadv4 (:1309-1508).  Records:
write_pops_det (:2054-2204) -- det(0:NIfD), the lenof_sign real signs and the
flag word, formatted ``(i24)``, ``(f30.8)``, ``(i24)`` in the text form and
as one unformatted record (int64 words, real(dp) signs, int64 flags) in the
binary form.  No global determinant data is written (``gdata`` is empty
without auto-adaptive shift, scaled blooms or accumulated populations).

The text form rounds signs to 8 decimals, as the reference's does; the
binary form is exact, so a binary round trip restarts a run bit for bit.
"""
from __future__ import annotations

import math
import re
import struct
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

VERSION_LINE = "# POPSFILE VERSION 4"


@dataclass
class PopsHeader:
    """The POPSHEAD namelist (Popsfile.F90:1951-2052, names as written)."""
    nel: int
    lenof_sign: int
    nifd: int
    totwalk: int = 0
    pop64bit: bool = True
    hphf: bool = False
    lz: bool = False
    multi: bool = False                         # PopMultiSft/... instead of PopSft/...
    shift: list = field(default_factory=lambda: [0.0])          # DiagSft (relative to Hii)
    sum_noat_hf: list = field(default_factory=lambda: [0.0])    # AllSumNoatHF(1:lenof_sign)
    sum_enum: list = field(default_factory=lambda: [0.0])       # AllSumENum
    cyc: int = 0                                # Iter + PreviousCycles
    tau: float = 0.0
    blocking_iter: int = 0
    p_singles: float = 0.0
    p_parallel: float = 0.5
    p_doubles: float = 1.0
    p_triples: float = 0.0
    tot_imag_time: float = 0.0
    gamma_sing: float = 0.0
    gamma_doub: float = 0.0
    gamma_trip: float = 0.0
    gamma_opp: float = 0.0
    gamma_par: float = 0.0
    max_death_cpt: float = 0.0
    balance_blocks: int | None = None
    walkers_on_nodes: list = field(default_factory=list)
    auto_adaptive_shift: bool = False
    random_hash: list = field(default_factory=list)  # RandomOrbIndex(1:nBasis)

    @property
    def niftot(self) -> int:
        return self.nifd + self.lenof_sign + 1


# ---------------------------------------------------------------- formatting
def _l1(b: bool) -> str:
    return "T" if b else "F"


def fortran_g(x: float, w: int = 26, d: int = 17, e: int = 3) -> str:
    """Gw.dEe editing of a real (gfortran's list-directed REAL(8) output is
    G26.17E3 after a leading blank): F editing with d significant digits and
    e+2 trailing blanks when 0.1 <= |x| < 10**d, E editing otherwise."""
    if x == 0.0:
        return f"{0.0:.{d - 1}f}".rjust(w - e - 2) + " " * (e + 2)  # F(w-n).(d-1) for zero
    if 0.1 - 0.5 * 10.0 ** (-d - 1) <= abs(x) < 10.0 ** d - 0.5:
        k = math.floor(math.log10(abs(x))) + 1
        s = f"{x:.{max(d - k, 0)}f}"
        if k > 0 and len(s.replace("-", "").split(".")[0]) > k:  # rounding carried into a new digit
            s = f"{x:.{max(d - k - 1, 0)}f}"
        return s.rjust(w - e - 2) + " " * (e + 2)
    m, ex = f"{x:.{d - 1}e}".split("e")
    mant = float(m) / 10.0
    exp = int(ex) + 1
    s = f"{'-' if x < 0 else ''}0.{f'{abs(mant):.{d}f}'[2:]}E{'+' if exp >= 0 else '-'}{abs(exp):0{e}d}"
    return s.rjust(w)


def header_text(h: PopsHeader) -> str:
    """write_popsfile_header (Popsfile.F90:1951-2052) for one node."""
    L = []
    L.append(VERSION_LINE)
    L.append(f"&POPSHEAD Pop64Bit={_l1(h.pop64bit)}")
    L.append(f"PopHPHF={_l1(h.hphf)},PopLz={_l1(h.lz)},PopLensign={h.lenof_sign:2d},PopNEl={h.nel:4d},")
    L.append(f"PopTotwalk={h.totwalk:15d}")
    g = lambda v: "".join(fortran_g(float(x)) for x in v)  # noqa: E731
    if not h.multi:
        L.append(" PopSft=" + g(h.shift[:1]))
        L.append(" PopSumNoatHF=" + g(h.sum_noat_hf))
        L.append(" PopSumENum=" + g(h.sum_enum[:1]))
    else:
        L.append(" PopMultiSft=" + g(h.shift))
        L.append(" PopMultiSumNoatHF=" + g(h.sum_noat_hf))
        L.append(" PopMultiSumENum=" + g(h.sum_enum))
    L.append(f"PopCyc={h.cyc:16d},PopNIfD={h.nifd:2d},PopNifY={0:2d},PopNIfSgn={h.lenof_sign:2d},")
    L.append(f"PopNIfFlag={1:2d},PopNIfTot={h.niftot:2d},PopTau={h.tau:18.12f},")
    L.append(f"PopiBlockingIter={h.blocking_iter:16d}")
    L.append(f"PopPSingles={h.p_singles:18.12f},PopPParallel={h.p_parallel:18.12f}")
    L.append(f",PopPDoubles={h.p_doubles:18.12f},PopPTriples={h.p_triples:18.12f}")
    L.append(f",PopPSing_spindiff1={0.0:18.12f},PopPDoub_spindiff1={0.0:18.12f}")
    L.append(f",PopPDoub_spindiff2={0.0:18.12f}")
    L.append(f"PopTotImagTime={h.tot_imag_time:18.12f}")
    g18 = lambda x: fortran_g(float(x), 18, 12, 4).lstrip().ljust(18)  # noqa: E731  (g18.12)
    L.append(f"PopGammaSing={g18(h.gamma_sing)},PopGammaDoub={g18(h.gamma_doub)},PopGammaTrip={g18(h.gamma_trip)},"
             f"PopGammaOpp={g18(h.gamma_opp)},PopGammaPar={g18(h.gamma_par)},PopMaxDeathCpt={g18(h.max_death_cpt)}")
    L.append(f",PopGammaSing_spindiff1={g18(0.0)},PopGammaDoub_spindiff1={g18(0.0)},"
             f"PopGammaDoub_spindiff2={g18(0.0)}")
    if h.balance_blocks is not None:
        L.append(f"PopBalanceBlocks={h.balance_blocks:7d}")
    won = h.walkers_on_nodes or [h.totwalk]
    L.append(f"PopNNodes={len(won):6d}")
    L.append("PopWalkersOnNodes=" + "".join(f"{int(w):16d}," for w in won))
    L.append(f" tPopAutoAdaptiveShift= {_l1(h.auto_adaptive_shift)}")
    L.append("PopRandomHash= " + "".join(f"{int(r):12d}," for r in h.random_hash))
    L.append(" &END")
    return "\n".join(L) + "\n"


# ------------------------------------------------------------------ parsing
_NAME = re.compile(r"([A-Za-z_][A-Za-z0-9_]*)\s*=")


def _value(tok: str):
    tok = tok.strip()
    if tok in ("T", ".TRUE.", ".true.", "T,"):
        return True
    if tok in ("F", ".FALSE.", ".false."):
        return False
    try:
        return int(tok)
    except ValueError:
        return float(tok.replace("D", "E").replace("d", "e"))


def parse_header(text: str) -> PopsHeader:
    """ReadPopsHeadv4 (Popsfile.F90:1309-1508): the POPSHEAD namelist."""
    if not text.lstrip().startswith(VERSION_LINE):
        raise ValueError("not a version-4 POPSFILE header")
    body = text[text.index("&POPSHEAD") + len("&POPSHEAD"): text.index("&END")]
    names = list(_NAME.finditer(body))
    vals = {}
    for k, m in enumerate(names):
        end = names[k + 1].start() if k + 1 < len(names) else len(body)
        raw = [t for t in re.split(r"[,\s]+", body[m.end():end]) if t]
        vals[m.group(1).lower()] = [_value(t) for t in raw]
    one = lambda k, dflt=None: vals[k][0] if k in vals and vals[k] else dflt  # noqa: E731
    multi = "popmultisft" in vals
    h = PopsHeader(nel=int(one("popnel")), lenof_sign=int(one("poplensign")), nifd=int(one("popnifd")),
                   totwalk=int(one("poptotwalk", 0)), pop64bit=bool(one("pop64bit", True)),
                   hphf=bool(one("pophphf", False)), lz=bool(one("poplz", False)), multi=multi)
    h.shift = [float(x) for x in vals.get("popmultisft" if multi else "popsft", [0.0])]
    h.sum_noat_hf = [float(x) for x in vals.get("popmultisumnoathf" if multi else "popsumnoathf", [0.0])]
    h.sum_enum = [float(x) for x in vals.get("popmultisumenum" if multi else "popsumenum", [0.0])]
    h.cyc = int(one("popcyc", 0))
    h.tau = float(one("poptau", 0.0))
    h.blocking_iter = int(one("popiblockingiter", 0))
    h.p_singles = float(one("poppsingles", 0.0))
    h.p_parallel = float(one("poppparallel", 0.5))
    h.p_doubles = float(one("poppdoubles", 1.0 - h.p_singles))
    h.p_triples = float(one("popptriples", 0.0))
    h.tot_imag_time = float(one("poptotimagtime", 0.0))
    for nm, key in (("gamma_sing", "popgammasing"), ("gamma_doub", "popgammadoub"), ("gamma_trip", "popgammatrip"),
                    ("gamma_opp", "popgammaopp"), ("gamma_par", "popgammapar"), ("max_death_cpt", "popmaxdeathcpt")):
        setattr(h, nm, float(one(key, 0.0)))
    bb = one("popbalanceblocks")
    h.balance_blocks = None if bb is None else int(bb)
    h.walkers_on_nodes = [int(x) for x in vals.get("popwalkersonnodes", [])]
    h.auto_adaptive_shift = bool(one("tpopautoadaptiveshift", False))
    h.random_hash = [int(x) for x in vals.get("poprandomhash", [])]
    nift = one("popniftot")
    if nift is not None and int(nift) != h.niftot:
        raise ValueError(f"PopNIfTot {nift} does not match NIfD {h.nifd} + lenof_sign {h.lenof_sign} + 1")
    if int(one("popnifflag", 1)) != 1:
        raise ValueError("only one flag word per record is supported")
    return h


# ------------------------------------------------------------------ records
def _occupied(rows: np.ndarray, W: int, L: int) -> np.ndarray:
    """write_pops_det's filter: sum(abs(real_sgn)) > binarypops_min_weight (0)."""
    signs = rows[:, W:W + L].view(np.float64)
    return np.abs(signs).sum(axis=1) > 0.0


def records_text(rows: np.ndarray, W: int, L: int) -> str:
    """Text records of write_pops_det: (i24) words, (f30.8) signs, (i24) flags."""
    out = []
    signs = np.ascontiguousarray(rows[:, W:W + L]).view(np.float64)
    flags = rows[:, W + L]  # extract_flags: the whole flag word, flag_removed (bit 0) included
    for r in range(rows.shape[0]):
        out.append("".join(f"{int(x):24d}" for x in rows[r, :W]) +
                   "".join(f"{float(x):30.8f}" for x in signs[r]) + f"{int(flags[r]):24d}\n")
    return "".join(out)


def records_binary(rows: np.ndarray, W: int, L: int) -> bytes:
    """Binary records of write_pops_det: one unformatted sequential record
    per determinant (4-byte length markers around the int64 words, the
    real(dp) signs and the int64 flag word)."""
    n = rows.shape[0]
    rec = np.empty((n, W + L + 1), dtype=np.int64)
    rec[:, :] = rows[:, :W + L + 1]
    nb = 8 * (W + L + 1)
    marker = np.full((n, 1), nb, dtype="<i4").view(np.uint8)
    body = rec.astype("<i8").view(np.uint8).reshape(n, nb)
    return np.concatenate([marker, body, marker], axis=1).tobytes()


def parse_records_text(text: str, W: int, L: int) -> np.ndarray:
    rows = []
    for line in text.splitlines():
        if not line.strip():
            continue
        tok = line.split()
        if len(tok) < W + L + 1:
            raise ValueError(f"short POPSFILE record: {line!r}")
        words = [int(t) for t in tok[:W]]
        signs = np.array([float(t.replace("D", "E")) for t in tok[W:W + L]], dtype=np.float64)
        rows.append(words + list(signs.view(np.int64)) + [int(tok[W + L])])
    return np.array(rows, dtype=np.int64).reshape(-1, W + L + 1)


def parse_records_binary(data: bytes, W: int, L: int) -> np.ndarray:
    nb = 8 * (W + L + 1)
    out = []
    pos = 0
    while pos < len(data):
        (m1,) = struct.unpack_from("<i", data, pos)
        if m1 < nb:
            raise ValueError(f"POPSFILEBIN record of {m1} bytes, expected at least {nb}")
        out.append(np.frombuffer(data, dtype="<i8", count=W + L + 1, offset=pos + 4))
        (m2,) = struct.unpack_from("<i", data, pos + 4 + m1)
        if m2 != m1:
            raise ValueError("corrupt POPSFILEBIN record markers")
        pos += m1 + 8
    return np.array(out, dtype=np.int64).reshape(-1, W + L + 1)


# ------------------------------------------------------------- whole files
def write_popsfile(stem: str | Path, header: PopsHeader, rows: np.ndarray, binary: bool = True) -> list[Path]:
    """WriteToPopsfileParOneArr (Popsfile.F90:1622-1949) for one node:
    ``stem`` (text) or ``stem``HEAD + ``stem``BIN (binary).  Rows are
    CurrentDets rows; empty determinants are skipped.  Returns the paths."""
    W, L = header.nifd + 1, header.lenof_sign
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    rows = rows[_occupied(rows, W, L)]
    header.totwalk = rows.shape[0]
    header.walkers_on_nodes = [rows.shape[0]]
    stem = Path(stem)
    if binary:
        head, binp = Path(str(stem) + "HEAD"), Path(str(stem) + "BIN")
        binp.write_bytes(records_binary(rows, W, L))
        head.write_text(header_text(header))
        return [head, binp]
    stem.write_text(header_text(header) + records_text(rows, W, L))
    return [stem]


def read_popsfile(stem: str | Path) -> tuple[PopsHeader, np.ndarray]:
    """ReadFromPopsfile for a version-4 file: ``stem`` (text) or
    ``stem``HEAD/``stem``BIN (binary).  Returns the header and the rows in
    CurrentDets layout."""
    stem = Path(stem)
    head, binp = Path(str(stem) + "HEAD"), Path(str(stem) + "BIN")
    if head.exists() and binp.exists():
        h = parse_header(head.read_text())
        rows = parse_records_binary(binp.read_bytes(), h.nifd + 1, h.lenof_sign)
    else:
        text = stem.read_text()
        end = text.index("&END")
        end = text.index("\n", end) + 1
        h = parse_header(text[:end])
        rows = parse_records_text(text[end:], h.nifd + 1, h.lenof_sign)
    if rows.shape[0] != h.totwalk:
        raise ValueError(f"POPSFILE holds {rows.shape[0]} records, its header says {h.totwalk}")
    return h, rows
