"""Seeded water geometries for the workloads this package is measured on.

* monomer: O at the origin, O-H 0.957 A, H-O-H 104.5 deg;
* clusters: n monomers, each with a uniform random rotation (normalised 4-D
  Gaussian quaternion) and a centre uniform in an L-angstrom cube, rejecting a
  placement with any O-O distance below 2.7 A; ``numpy.random.default_rng``
  with an explicit seed;
* batches of monomers, dimers and trimers with Gaussian displacements.
All coordinates returned in bohr.
"""
from __future__ import annotations

import numpy as np

ANGSTROM_TO_BOHR = 1.0 / 0.529177210903


def water_monomer():
    """(atomnos, coords_bohr) of the reference water: O, H, H."""
    half = np.deg2rad(104.5) / 2.0
    r = 0.957
    xyz = np.array([[0.0, 0.0, 0.0], [r * np.sin(half), 0.0, r * np.cos(half)], [-r * np.sin(half), 0.0, r * np.cos(half)]])
    return np.array([8, 1, 1], dtype=np.int32), xyz * ANGSTROM_TO_BOHR


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def water_cluster(n, box_angstrom, seed, min_oo_angstrom=2.7, max_tries=100000):
    """n waters, seeded rotations, centres uniform in a cube, O-O >= 2.7 A."""
    rng = np.random.default_rng(seed)
    Z0, R0 = water_monomer()
    R0 = R0 / ANGSTROM_TO_BOHR  # work in angstrom
    oxy, atoms, coords = [], [], []
    tries = 0
    while len(oxy) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place %d waters in a %.1f A cube" % (n, box_angstrom))
        rot = _rotation(rng)
        c = rng.uniform(0.0, box_angstrom, size=3)
        xyz = R0 @ rot.T + c
        if any(np.linalg.norm(xyz[0] - o) < min_oo_angstrom for o in oxy):
            continue
        oxy.append(xyz[0])
        atoms.extend(Z0.tolist())
        coords.append(xyz)
    return np.asarray(atoms, dtype=np.int32), np.concatenate(coords) * ANGSTROM_TO_BOHR


def water_batch(count, seed, sigma_bohr=0.05, box_angstrom=9.0):
    """An equal mix of monomers, dimers and trimers (count//3 each, the
    remainder added to the monomers first), each monomer displaced by
    N(0, sigma) per coordinate after placement."""
    rng = np.random.default_rng(seed)
    sizes = [1] * (count - 2 * (count // 3)) + [2] * (count // 3) + [3] * (count // 3)
    sizes = sizes[:count]
    out = []
    for k, m in enumerate(sizes):
        Z, R = water_cluster(m, box_angstrom * (m / 8.0) ** (1.0 / 3.0) if m > 1 else 1.0,
                             seed=int(rng.integers(1 << 31)))
        R = R + rng.normal(0.0, sigma_bohr, size=R.shape)
        out.append((Z, R))
    return out


# the workloads (basis-set name, geometry)
def config(name):
    if name == "h2o_sto3g":
        return ("sto-3g-fit",) + water_monomer()
    if name == "h2o8_631g":
        return ("6-31g-fit",) + water_cluster(8, 9.0, seed=1)
    if name == "h2o4_631gss":
        return ("6-31gss-fit",) + water_cluster(4, 4.5, seed=2)
    if name == "h2o32_631gs":
        return ("6-31gs-fit",) + water_cluster(32, 14.0, seed=4)
    raise KeyError(name)


CONFIGS = ("h2o_sto3g", "h2o8_631g", "h2o4_631gss", "h2o32_631gs")
