"""Regenerates the golden fixtures of this directory from the reference's
own test inputs and recorded outputs (run where the reference tree exists;
the fixtures are committed so that the tests do not need it).

Usage: python make_golden.py REFERENCE_ROOT   (the root of a NECI checkout;
the environment variable NECI_REFERENCE_ROOT may give it instead).

* hehe_fcidump.npz -- integrals of test_suite/neci/serial/HeHe_Davidson_Direct_CI
  (FCIDUMP) and the exact ground-state energy NECI's Davidson printed for it
  ("GROUND E" in that directory's benchmark output).
* ne_pchb_fcidump.npz -- integrals of test_suite/neci/parallel/Ne_FciMCPar_pchb
  (FCIDUMP; the input freezes 2 spin orbitals) and the projected energy with
  its blocking error that NECI's run recorded ("Total projected energy"),
  plus the core energy after freezing ("ECORE now") and the reference
  energy ("<D0|H|D0>=") that the same run printed.
* rdm_fci_core.npz -- integrals of test_suite/dneci/rdm/full_CI+AAS+RDMs
  (FCIDUMP: 6 spatial orbitals, 6 electrons) and the 2-RDM energy that NECI's
  two recorded runs printed ("*TOTAL ENERGY* CALCULATED USING THE *REDUCED
  DENSITY MATRICES*"), with the whole space as the semistochastic core.
* pops_*.npz -- POPSFILEs that NECI wrote in its test suite (text
  test_suite/neci/tau_search/start_val/from_popsfile/POPSFILE; binary
  POPSFILEHEAD/POPSFILEBIN of test_suite/neci/serial/Ne_adi_Pops_min_si and
  test_suite/dneci/rdm/BeH_open_shell_dyn_core): the header text, the
  records as CurrentDets rows and the SHA-256 of NECI's record bytes, which
  the writer must reproduce exactly.
"""
from __future__ import annotations

import glob
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
from neci_stable_gb300.systems import read_fcidump  # noqa: E402



def reference_suite(argv) -> Path:
    """test_suite/neci of the NECI tree named on the command line or by
    NECI_REFERENCE_ROOT."""
    import os
    root = argv[1] if len(argv) > 1 else os.environ.get("NECI_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: make_golden.py REFERENCE_ROOT (or set NECI_REFERENCE_ROOT)")
    suite = Path(root) / "test_suite" / "neci"
    if not suite.is_dir():
        raise SystemExit(f"{suite} does not exist")
    return suite


def orbsym(path):
    head = open(path).read().split("&END")[0].replace("\n", " ")
    m = re.search(r"ORBSYM\s*=\s*([\d,\s]+)", head)
    return np.array([int(x) for x in m.group(1).replace(",", " ").split()], dtype=np.int32)


def save(name, src_dir, pattern, key, extra=None):
    fcidump = src_dir / "FCIDUMP"
    h, eri, ecore, nelec, ms2 = read_fcidump(fcidump)
    bench = glob.glob(str(src_dir / "benchmark*"))[0]
    text = open(bench).read()
    m = re.search(pattern, text)
    vals = [float(x) for x in m.groups()]
    more = {}
    for k, pat in (extra or {}).items():
        more[k] = np.array([float(x) for x in re.search(pat, text).groups()])
    np.savez_compressed(HERE / name, h=h, eri=eri.astype(np.float64), ecore=ecore, nelec=nelec, ms2=ms2,
                        orbsym=orbsym(fcidump), **{key: np.array(vals)}, **more)
    print(name, h.shape, vals, more)


def save_rdm(name, src_dir):
    """The FCIDUMP of an RDM test and the RDM energy of each recorded run."""
    fcidump = src_dir / "FCIDUMP"
    h, eri, ecore, nelec, ms2 = read_fcidump(fcidump)
    energies = []
    for bench in sorted(glob.glob(str(src_dir / "benchmark*"))):
        text = open(bench).read()
        m = re.search(r"\*TOTAL ENERGY\* CALCULATED USING THE \*REDUCED DENSITY MATRICES\*:\s*(-?[\d.]+E[+-]\d+)", text)
        energies.append(float(m.group(1)))
    np.savez_compressed(HERE / name, h=h, eri=eri.astype(np.float64), ecore=ecore, nelec=nelec, ms2=ms2,
                        orbsym=orbsym(fcidump), rdm_energy=np.array(energies))
    print(name, h.shape, energies)


def save_pops(name, src_dir, binary):
    import hashlib
    from neci_stable_gb300 import popsfile
    if binary:
        head = (src_dir / "POPSFILEHEAD").read_text()
        rec_bytes = (src_dir / "POPSFILEBIN").read_bytes()
        h, rows = popsfile.read_popsfile(src_dir / "POPSFILE")
    else:
        text = (src_dir / "POPSFILE").read_text()
        end = text.index("\n", text.index("&END")) + 1
        head, rec_bytes = text[:end], text[end:].encode()
        h, rows = popsfile.read_popsfile(src_dir / "POPSFILE")
    np.savez_compressed(HERE / name, header=np.array(head), rows=rows, binary=binary,
                        sha256=np.array(hashlib.sha256(rec_bytes).hexdigest()))
    print(name, rows.shape, h.totwalk, h.lenof_sign)


if __name__ == "__main__":
    REF = reference_suite(sys.argv)
    save_rdm("rdm_fci_core.npz", REF.parent / "dneci" / "rdm" / "full_CI+AAS+RDMs")
    save_pops("pops_text_li2.npz", REF / "tau_search" / "start_val" / "from_popsfile", binary=False)
    save_pops("pops_bin_ne.npz", REF / "serial" / "Ne_adi_Pops_min_si", binary=True)
    save_pops("pops_bin_beh_dneci.npz", REF.parent / "dneci" / "rdm" / "BeH_open_shell_dyn_core", binary=True)
    save("hehe_fcidump.npz", REF / "serial" / "HeHe_Davidson_Direct_CI", r"GROUND E =\s*(-?\d+\.\d+)", "ground_e")
    save("ne_pchb_fcidump.npz", REF / "parallel" / "Ne_FciMCPar_pchb",
         r"Total projected energy\s+(-?\d+\.\d+)\s+\+/-\s+(\d+\.\d+E?-?\d*)", "proje_err",
         extra={"ecore_frozen": r"ECORE now\s+(-?\d+\.\d+)", "d0_energy": r"<D0\|H\|D0>=\s+(-?\d+\.\d+)"})
