"""Generate the golden fixtures in this directory from the reference itself.

Runs only where the reference sources are present: ``make -C oracle ref``
compiles ``libpyquante2/{cints,chgp}.c`` unmodified into
``oracle/_ref/libpyquante2_shipped.so`` (the reference's Boys function) and
``oracle/_ref/libpyquante2_exact.so`` (the same objects with an exact Boys
function bound in).  The fixtures record:

* ``eri_prims.json``   -- primitive ERIs over every angular-momentum class up
  to (dd|dd), seeded random exponents and centres: the reference's
  ``coulomb_repulsion`` (cints.c:72-115) with both Boys functions;
* ``onee_prims.json``  -- primitive overlap / kinetic / nuclear attraction
  (cints.c:152-243), both Boys functions;
* ``h2o_sto3g.npz``, ``h2o_631g.npz``, ``h2o_631gs.npz`` -- S, T, V and, for a
  fixed symmetric density, J and K with the semantics of src/basis.rs:214-428
  evaluated through the reference's integrals; the dense ERI tensor
  (src/basis.rs:430-460) for the STO-3G-shaped water; the converged RHF
  energy of src/bin/rchem.rs:40-89 for it.

Usage: ``python tests/golden/make_golden.py`` (a minute or two).
"""
from __future__ import annotations

import itertools
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

from rchem_gb300 import bse, geometry  # noqa: E402


def ijk(l):
    return O.ijk_list(l)


def random_prim_quartets(rng, n_per_class):
    out = []
    for cls in itertools.product(range(3), repeat=4):
        for _ in range(n_per_class):
            R = rng.uniform(-1.5, 1.5, (4, 3))
            if rng.random() < 0.25:
                R[1] = R[0]
            if rng.random() < 0.25:
                R[3] = R[2]
            a = rng.uniform(0.15, 4.0, 4)
            pw = [list(ijk(l)[rng.integers(len(ijk(l)))]) for l in cls]
            out.append({"R": R.tolist(), "alpha": a.tolist(), "powers": pw})
    return out


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port", "ref"], check=True)
    ex = O.ref("exact")
    sh = O.ref("shipped")
    if ex is None or sh is None:
        sys.exit("reference libraries not built (reference sources absent?)")
    rng = np.random.default_rng(20261203)

    # ---- primitive ERIs ---------------------------------------------------
    items = random_prim_quartets(rng, 2)
    # the os86 / tho66 golden geometry with high powers too (benches/bench_rchem.rs:105-113)
    base = {"R": [[1.0, 0.0, 1.0], [0.0, 1.0, 2.0], [0.0, 0.0, 3.0], [0.0, 0.0, 4.0]], "alpha": [1.1, 1.2, 1.3, 1.4]}
    for pw in ([[0, 0, 0]] * 4, [[1, 0, 0], [0, 0, 0], [0, 0, 0], [0, 0, 0]],
               [[2, 1, 0], [1, 0, 0], [1, 0, 0], [0, 1, 0]], [[1, 1, 0], [0, 1, 1], [2, 0, 0], [0, 0, 2]]):
        items.append(dict(base, powers=pw))
    for it in items:
        R, a, pw = it["R"], it["alpha"], it["powers"]
        args = []
        for k in range(4):
            args += [R[k], 1.0, pw[k], a[k]]
        it["exact"] = ex.coulomb_repulsion(*args)
        it["shipped"] = sh.coulomb_repulsion(*args)
    with open(os.path.join(HERE, "eri_prims.json"), "w") as f:
        json.dump({"source": "libpyquante2/cints.c:72-115 compiled from the reference", "items": items}, f)

    # ---- one-electron primitives -----------------------------------------
    one = []
    for la, lb in itertools.product(range(4), repeat=2):
        for _ in range(2):
            R = rng.uniform(-1.2, 1.2, (3, 3))
            a = rng.uniform(0.2, 3.0, 2)
            pa = list(ijk(la)[rng.integers(len(ijk(la)))])
            pb = list(ijk(lb)[rng.integers(len(ijk(lb)))])
            rec = {"A": R[0].tolist(), "B": R[1].tolist(), "C": R[2].tolist(), "alpha": a.tolist(), "pa": pa, "pb": pb}
            for lib, tag in ((ex, "exact"), (sh, "shipped")):
                rec["S_" + tag] = lib.overlap(a[0], a[1], R[0], R[1], pa + pb)
                rec["T_" + tag] = lib.kinetic(a[0], a[1], R[0], R[1], pa + pb)
                rec["V_" + tag] = lib.nuclear(a[0], a[1], R[0], R[1], R[2], pa + pb)
            one.append(rec)
    with open(os.path.join(HERE, "onee_prims.json"), "w") as f:
        json.dump({"source": "libpyquante2/cints.c:152-243 compiled from the reference", "items": one}, f)

    # ---- matrices --------------------------------------------------------
    Z, R = geometry.water_monomer()
    for tag, name in (("h2o_sto3g", "sto-3g-fit"), ("h2o_631g", "6-31g-fit"), ("h2o_631gs", "6-31gs-fit")):
        b = O.expand_basis(Z, R, bse.load_bse(name))
        Sm, Tm, Vm = O.S(b, ex), O.T(b, ex), O.V(b, R, Z, ex)
        Xs = O.symm_orthog(Sm)
        _, Cp = np.linalg.eigh(Xs.T @ (Tm + Vm) @ Xs)
        D = O.build_density(Xs @ Cp, 5)  # core-guess density, rchem.rs:55-59
        J, K = O.JK_direct(b, D, ex)
        rec = dict(S=Sm, T=Tm, V=Vm, D=D, J=J, K=K)
        if tag == "h2o_sto3g":
            rec["I"] = O.build_I(b, ex)
            res = O.rhf(b, Z, R, 5, jk=lambda Dm: O.JK_direct(b, Dm, ex), thresh_e=1e-12, lib=ex)
            rec["e_elec"] = np.array(res["e_elec"])
            rec["e_nuc"] = np.array(res["e_nuc"])
            rec["D_scf"] = res["D"]
        np.savez_compressed(os.path.join(HERE, tag + ".npz"), **rec)
        print("wrote", tag)


if __name__ == "__main__":
    main()
