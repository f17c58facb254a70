"""Run a few Fock builds (or gradients) of a named workload for a profiler,
then print the per-class work of the plan (``python -m rchem_gb300.profile_builds``).

Workloads: the single-geometry configurations of ``rchem_gb300.geometry``
(h2o_sto3g, h2o8_631g, h2o4_631gss, h2o32_631gs) and ``batch512_631g`` (512
water monomers/dimers/trimers in one batched handle).  ``--onee`` builds S, T
and V instead; ``--scf`` (batch only) runs the library's SCF loop, one
iteration per host launch so every kernel is an ordinary launch.  The density (and, with
``--gradient``, the energy-weighted density) is a seeded random symmetric
matrix: the kernels do the same work for any density.

Example (the launch list of three FP64 builds of (H2O)8 in the 6-31G-shaped
basis)::

    ncu --metrics gpu__time_duration.sum --clock-control none --csv \\
        python -m rchem_gb300.profile_builds --workload h2o8_631g --builds 3
"""
from __future__ import annotations

import argparse
import json


def _sym(rng, n, scale):
    X = rng.normal(size=(n, n))
    return X @ X.T / n * scale


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="h2o8_631g")
    ap.add_argument("--builds", type=int, default=3)
    ap.add_argument("--fp32-tau", type=float, default=0.0)
    ap.add_argument("--emulated", action="store_true", help="double-float arithmetic for the FP64 quartets")
    ap.add_argument("--gradient", action="store_true", help="run the nuclear gradient instead of Fock builds")
    ap.add_argument("--autotune", action="store_true", help="autotune the tile shapes before the builds")
    ap.add_argument("--onee", action="store_true", help="build S, T and V (the one-electron class kernels) instead")
    ap.add_argument("--scf", action="store_true",
                    help="run the library's SCF loop (rchem_rhf) on the legacy default stream, one iteration per "
                         "host launch, instead")
    a = ap.parse_args(argv)
    import numpy as np
    import torch

    from . import _lib, batch, geometry
    from .basis import S, T, V, Basis, JK_direct
    from .scf import gradient

    L = _lib.lib()

    rng = np.random.default_rng(0)
    if a.workload == "batch512_631g":
        b = batch.BatchBasis(geometry.water_batch(512, seed=7), "6-31g-fit")
        Dh, Wh = np.zeros(b.packed), np.zeros(b.packed)
        for g in range(b.ngeom):
            n = int(b.geom_nbf[g])
            b.block(Dh, g)[:] = _sym(rng, n, 0.1)
            b.block(Wh, g)[:] = _sym(rng, n, 0.1)
        D, W = torch.from_numpy(Dh).cuda(), torch.from_numpy(Wh).cuda()
        if a.autotune:
            b.autotune(1e-12, a.fp32_tau, emulated=a.emulated)
        if a.scf:
            b.set_stream(0)
        for _ in range(a.builds):
            if a.scf:
                batch.rhf_native(b, fp32_tau=a.fp32_tau, emulated=a.emulated)
            elif a.onee:
                for fn in (L.rchem_S, L.rchem_T, L.rchem_V):
                    batch._packed_matrix(fn, b)
            elif a.gradient:
                batch.gradient_batch(b, {"D": D, "W": W})
            else:
                J, K = torch.empty_like(D), torch.empty_like(D)
                batch.jk(b, D, J, K, fp32_tau=a.fp32_tau, emulated=a.emulated)
    else:
        bname, Z, R = geometry.config(a.workload)
        b = Basis(Z, R, bname)
        n = b.nbf
        s = torch.cuda.Stream()
        b.set_stream(s.cuda_stream)
        D = torch.from_numpy(_sym(rng, n, 0.1)).cuda()
        W = torch.from_numpy(_sym(rng, n, 0.1)).cuda()
        J, K = torch.empty_like(D), torch.empty_like(D)
        if a.autotune:
            b.autotune(1e-12, a.fp32_tau, emulated=a.emulated)
        torch.cuda.synchronize()
        for _ in range(a.builds):
            if a.onee:
                S(b, device=True), T(b, device=True), V(b, device=True)
            elif a.gradient:
                gradient(b, {"D": D, "W": W})
            else:
                JK_direct(J, K, b, D, fp32_tau=a.fp32_tau, emulated=a.emulated)
    torch.cuda.synchronize()
    if not (a.gradient or a.onee or a.scf):
        print(json.dumps(b.class_stats()))
    b.close()


if __name__ == "__main__":
    main()
