"""Python view of the cints-compatible entry points (include/rchem_cints.h).

The argument order of ``coulomb`` and ``overlap`` follows the reference's Rust
wrappers (src/integrals/tho66.rs:228-259): exponents, centres, norms, powers.
"""
from __future__ import annotations

import numpy as np

from . import _lib


def coulomb(za, zb, zc, zd, ra, rb, rc, rd, powers, norms=(1.0, 1.0, 1.0, 1.0)) -> float:
    p = [int(x) for x in powers]
    return _lib.lib().coulomb_repulsion(*ra, norms[0], *p[0:3], za, *rb, norms[1], *p[3:6], zb,
                                        *rc, norms[2], *p[6:9], zc, *rd, norms[3], *p[9:12], zd)


def overlap(za, zb, ra, rb, powers) -> float:
    p = [int(x) for x in powers]
    return _lib.lib().overlap(za, *p[0:3], *ra, zb, *p[3:6], *rb)


def kinetic(za, zb, ra, rb, powers) -> float:
    p = [int(x) for x in powers]
    return _lib.lib().kinetic(za, *p[0:3], *ra, zb, *p[3:6], *rb)


def nuclear(za, zb, ra, rb, rc, powers, norms=(1.0, 1.0)) -> float:
    p = [int(x) for x in powers]
    return _lib.lib().nuclear_attraction(*ra, norms[0], *p[0:3], za, *rb, norms[1], *p[3:6], zb, *rc)


def fgamma(m, x) -> float:
    return _lib.lib().Fgamma(float(m), float(x))


def boys_batch(m, x, precision=64) -> np.ndarray:
    m = np.ascontiguousarray(m, dtype=np.int32).reshape(-1)
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
    if m.size != x.size:
        raise ValueError("m and x must have the same length (%d != %d)" % (m.size, x.size))
    out = np.empty(len(m))
    _lib.check(_lib.lib().rchem_boys_batch(len(m), m.ctypes.data, x.ctypes.data, out.ctypes.data, precision,
                                           _lib.HOST))
    return out


def eri_batch(quartets) -> np.ndarray:
    """quartets: list of 4-tuples of (center(3), norm, alpha, (l,m,n))."""
    n = len(quartets)
    arr = (_lib.Prim * (4 * n))()
    for i, q in enumerate(quartets):
        for k, (r, nm, a, lmn) in enumerate(q):
            arr[4 * i + k] = _lib.Prim(r[0], r[1], r[2], nm, a, lmn[0], lmn[1], lmn[2], 0)
    out = np.empty(n)
    _lib.check(_lib.lib().rchem_eri_prim_batch(n, arr, out.ctypes.data, _lib.HOST))
    return out
