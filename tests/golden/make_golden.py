"""Regenerates the golden fixtures of this directory from the reference's
own test inputs and recorded outputs (run where the reference tree exists;
the fixtures are committed so that the tests do not need it).

* hehe_fcidump.npz -- integrals of test_suite/neci/serial/HeHe_Davidson_Direct_CI
  (FCIDUMP) and the exact ground-state energy NECI's Davidson printed for it
  ("GROUND E" in that directory's benchmark output).
* ne_pchb_fcidump.npz -- integrals of test_suite/neci/parallel/Ne_FciMCPar_pchb
  (FCIDUMP; the input freezes 2 spin orbitals) and the projected energy with
  its blocking error that NECI's run recorded ("Total projected energy"),
  plus the core energy after freezing ("ECORE now") and the reference
  energy ("<D0|H|D0>=") that the same run printed.
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

REF = Path("/root/reference/test_suite/neci")


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


if __name__ == "__main__":
    save("hehe_fcidump.npz", REF / "serial" / "HeHe_Davidson_Direct_CI", r"GROUND E =\s*(-?\d+\.\d+)", "ground_e")
    save("ne_pchb_fcidump.npz", REF / "parallel" / "Ne_FciMCPar_pchb",
         r"Total projected energy\s+(-?\d+\.\d+)\s+\+/-\s+(\d+\.\d+E?-?\d*)", "proje_err",
         extra={"ecore_frozen": r"ECORE now\s+(-?\d+\.\d+)", "d0_energy": r"<D0\|H\|D0>=\s+(-?\d+\.\d+)"})
