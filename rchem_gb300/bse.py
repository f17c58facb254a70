"""Basis-set and geometry input (the data formats either side of the hot path).

* ``load_bse(name_or_path)`` reads a Basis Set Exchange JSON document -- the
  format the reference deserialises (``src/basis.rs:14-85``) after fetching it
  through embedded Python (``src/basis.rs:87-106``).  A bare name is looked up
  among the files shipped in ``basis_sets/``.
* ``expand_shells(atomnos, bse)`` turns it into the pure-angular-momentum shell
  list the C ABI takes, in the reference's AO order (``Basis::new``,
  ``src/basis.rs:181-211``): atoms in order, shells in file order, each
  angular momentum of a shell in order.  The reference takes the coefficients
  of angular momentum ``l`` from ``coefficients[l]`` (by value, which only
  works for s and combined sp shells); here they are taken by position, which
  is the same for those shells and also handles pure p and d shells.
* ``read_xyz(path)`` reads an XYZ file; like the reference's driver
  (``src/bin/rchem.rs:29-34``) the coordinates are used as given (bohr)
  unless ``angstrom=True``.
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BASIS_DIR = os.path.join(HERE, "basis_sets")
ANGSTROM_TO_BOHR = 1.0 / 0.529177210903

_SYMBOLS = {"H": 1, "He": 2, "Li": 3, "Be": 4, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9, "Ne": 10}


def available_basis_sets():
    return sorted(f[:-5] for f in os.listdir(BASIS_DIR) if f.endswith(".json"))


def load_bse(name_or_path) -> dict:
    if isinstance(name_or_path, dict):
        return name_or_path
    path = name_or_path
    if not os.path.exists(path):
        path = os.path.join(BASIS_DIR, str(name_or_path).lower() + ".json")
    if not os.path.exists(path):
        raise FileNotFoundError("basis set %r not found (shipped: %s)" % (name_or_path, available_basis_sets()))
    with open(path) as f:
        doc = json.load(f)
    if "elements" not in doc:
        raise ValueError("%s is not a BSE JSON document (no 'elements')" % path)
    return doc


@dataclass
class Shells:
    atom: np.ndarray  # (nshell,) int32
    l: np.ndarray  # (nshell,) int32
    nprim: np.ndarray  # (nshell,) int32
    exps: np.ndarray  # (sum nprim,) f64
    coefs: np.ndarray  # (sum nprim,) f64, raw file coefficients

    @property
    def nbf(self) -> int:
        return int(sum((l + 1) * (l + 2) // 2 for l in self.l))


def expand_shells(atomnos, bse) -> Shells:
    doc = load_bse(bse)
    atom, ls, nprim, exps, coefs = [], [], [], [], []
    for ia, z in enumerate(atomnos):
        key = str(int(z))
        if key not in doc["elements"]:
            raise KeyError("basis set has no element Z=%s" % key)
        for sh in doc["elements"][key]["electron_shells"]:
            ft = sh.get("function_type", "gto")
            if ft == "sto":
                raise ValueError("Slater-type shells are not Gaussian shells")
            ex = [float(x) for x in sh["exponents"]]
            for k, l in enumerate(sh["angular_momentum"]):
                cf = [float(x) for x in sh["coefficients"][k]]
                if len(cf) != len(ex):
                    raise ValueError("shell on Z=%s: %d exponents, %d coefficients" % (key, len(ex), len(cf)))
                atom.append(ia)
                ls.append(int(l))
                nprim.append(len(ex))
                exps.extend(ex)
                coefs.extend(cf)
    return Shells(np.asarray(atom, np.int32), np.asarray(ls, np.int32), np.asarray(nprim, np.int32),
                  np.asarray(exps, np.float64), np.asarray(coefs, np.float64))


def read_xyz(path, angstrom=False):
    with open(path) as f:
        lines = f.read().splitlines()
    n = int(lines[0].split()[0])
    Z, R = [], []
    for ln in lines[2:2 + n]:
        tok = ln.split()
        sym = tok[0]
        Z.append(int(sym) if sym.isdigit() else _SYMBOLS[sym.capitalize()])
        R.append([float(t) for t in tok[1:4]])
    R = np.asarray(R, dtype=np.float64)
    if angstrom:
        R = R * ANGSTROM_TO_BOHR
    return np.asarray(Z, dtype=np.int32), R


def write_xyz(path, atomnos, coords, comment=""):
    inv = {v: k for k, v in _SYMBOLS.items()}
    with open(path, "w") as f:
        f.write("%d\n%s\n" % (len(atomnos), comment))
        for z, r in zip(atomnos, np.asarray(coords).reshape(-1, 3)):
            f.write("%-2s %20.12f %20.12f %20.12f\n" % (inv[int(z)], r[0], r[1], r[2]))
