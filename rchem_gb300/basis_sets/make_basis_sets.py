"""Generate the H/O basis-set files shipped with rchem_gb300 (BSE-JSON schema).

The Basis Set Exchange data the reference downloads at run time
(``src/basis.rs:87-106``) are not available offline, so this script builds
stand-ins with the same shell structure, primitive counts and angular momenta
as STO-3G, 6-31G, 6-31G* and 6-31G** for H and O:

* every contraction is a least-squares fit of Gaussians to a Slater-type
  orbital (the STO-nG construction: minimise the integrated squared
  difference, optimal coefficients from the normal equations, exponents by
  nonlinear minimisation);  2s and 2p share exponents (sp shells);
* orbital exponents zeta come from Slater's screening rules (O 1s 7.70,
  O 2sp 2.275), except H 1s, which uses the common molecular value 1.24;
* the "31" split-valence shells are a 4-Gaussian fit of the valence STO whose
  three tightest primitives form the inner contraction (renormalised) and whose
  most diffuse primitive is the outer function;
* polarisation functions: one Cartesian d on O (exponent 0.8) for 6-31G*,
  plus one p on H (exponent 1.1) for 6-31G**.

The numbers are NOT the published basis sets; a user with the real BSE JSON
files passes them to ``rchem_gb300.load_bse`` instead.  Output files are written
beside this script.  Run: ``python make_basis_sets.py``.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np
from scipy import integrate, optimize

HERE = os.path.dirname(os.path.abspath(__file__))


# --- radial overlaps with unit-exponent Slater functions -------------------
def _sto_norm(n, zeta):
    return math.sqrt((2 * zeta) ** (2 * n + 1) / math.factorial(2 * n))


def _radial(n_sto, l, alpha, zeta=1.0):
    """<R_STO(n,zeta) | R_GTO(l,alpha)> with both radial parts normalised
    (angular parts identical, so this is the full 3-D overlap)."""
    ns = _sto_norm(n_sto, zeta)
    ng = math.sqrt(2 * (2 * alpha) ** (l + 1.5) / math.gamma(l + 1.5))
    f = lambda r: r ** (n_sto - 1) * math.exp(-zeta * r) * r**l * math.exp(-alpha * r * r) * r * r
    val, _ = integrate.quad(f, 0, np.inf, limit=400, epsabs=1e-15, epsrel=1e-13)
    return ns * ng * val


def _gto_overlap(l, a, b):
    return (2 * math.sqrt(a * b) / (a + b)) ** (l + 1.5)


def _fit_error(logalpha, targets):
    """Sum over (n_sto, l) targets of 1 - s^T G^-1 s (the least-squares residual)."""
    al = np.exp(logalpha)
    err = 0.0
    coefs = []
    for n_sto, l in targets:
        G = np.array([[_gto_overlap(l, a, b) for b in al] for a in al])
        s = np.array([_radial(n_sto, l, a) for a in al])
        try:
            c = np.linalg.solve(G, s)
        except np.linalg.LinAlgError:
            return 10.0, None
        err += 1.0 - float(s @ c)
        coefs.append(c)
    return err, coefs


def fit(ngauss, targets, guess):
    x0 = np.log(np.asarray(guess, dtype=np.float64))
    res = optimize.minimize(lambda x: _fit_error(x, targets)[0], x0, method="Nelder-Mead",
                            options={"xatol": 1e-10, "fatol": 1e-14, "maxiter": 20000, "maxfev": 40000})
    res = optimize.minimize(lambda x: _fit_error(x, targets)[0], res.x, method="BFGS", options={"gtol": 1e-12})
    order = np.argsort(-res.x)
    al = np.exp(res.x[order])
    _, coefs = _fit_error(res.x[order], targets)
    return al, coefs, _fit_error(res.x, targets)[0]


def _renorm(l, al, c):
    G = np.array([[_gto_overlap(l, a, b) for b in al] for a in al])
    return c / math.sqrt(float(c @ G @ c))


def fmt(x):
    return f"{x:.10e}"


def shell(ams, exps, coef_lists, region=""):
    return {
        "function_type": "gto_cartesian",
        "region": region,
        "angular_momentum": list(ams),
        "exponents": [fmt(e) for e in exps],
        "coefficients": [[fmt(c) for c in cl] for cl in coef_lists],
    }


def main():
    zeta = {"H1s": 1.24, "O1s": 7.70, "O2sp": 2.275}
    g3 = [2.2, 0.4, 0.11]
    g4 = [5.0, 0.9, 0.25, 0.07]
    g6 = [24.0, 4.4, 1.2, 0.42, 0.16, 0.065]
    # unit-exponent fits
    s1_3, (c1_3,), e = fit(3, [(1, 0)], g3)
    s1_4, (c1_4,), _ = fit(4, [(1, 0)], g4)
    s1_6, (c1_6,), _ = fit(6, [(1, 0)], g6)
    sp_3, (c2s_3, c2p_3), _ = fit(3, [(2, 0), (2, 1)], [1.0, 0.23, 0.07])
    sp_4, (c2s_4, c2p_4), _ = fit(4, [(2, 0), (2, 1)], [2.0, 0.5, 0.15, 0.05])

    def scale(al, z):
        return al * z * z

    sets = {}
    # STO-3G shape: H 1s(3); O 1s(3), 2sp(3)
    sets["sto-3g-fit"] = {
        "1": [shell([0], scale(s1_3, zeta["H1s"]), [c1_3])],
        "8": [shell([0], scale(s1_3, zeta["O1s"]), [c1_3]),
              shell([0, 1], scale(sp_3, zeta["O2sp"]), [c2s_3, c2p_3])],
    }
    # 6-31G shape: H 1s(3) 1s'(1); O 1s(6), 2sp(3), 2sp'(1)
    hin = scale(s1_4[:3], zeta["H1s"])
    hout = scale(s1_4[3:], zeta["H1s"])
    oin = scale(sp_4[:3], zeta["O2sp"])
    oout = scale(sp_4[3:], zeta["O2sp"])
    h631 = [shell([0], hin, [_renorm(0, hin, c1_4[:3])]), shell([0], hout, [[1.0]])]
    o631 = [shell([0], scale(s1_6, zeta["O1s"]), [c1_6]),
            shell([0, 1], oin, [_renorm(0, oin, c2s_4[:3]), _renorm(1, oin, c2p_4[:3])]),
            shell([0, 1], oout, [[1.0], [1.0]])]
    sets["6-31g-fit"] = {"1": h631, "8": o631}
    dpol = shell([2], [0.8], [[1.0]], "polarization")
    ppol = shell([1], [1.1], [[1.0]], "polarization")
    sets["6-31gs-fit"] = {"1": h631, "8": o631 + [dpol]}
    sets["6-31gss-fit"] = {"1": h631 + [ppol], "8": o631 + [dpol]}

    for name, els in sets.items():
        doc = {
            "name": name,
            "description": "Stand-in with the shell structure of " + {
                "sto-3g-fit": "STO-3G", "6-31g-fit": "6-31G", "6-31gs-fit": "6-31G*",
                "6-31gss-fit": "6-31G**"}[name] + "; least-squares STO-nG fits, not the published numbers",
            "elements": {z: {"electron_shells": shells} for z, shells in els.items()},
        }
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(doc, f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    main()
