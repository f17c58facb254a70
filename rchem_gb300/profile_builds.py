"""Run a few Fock builds of a named workload for a profiler, then print the
per-class work of the plan (``python -m rchem_gb300.profile_builds``).

Example (the launch list of three FP64 builds of (H2O)8 in the 6-31G-shaped
basis)::

    ncu --metrics gpu__time_duration.sum --clock-control none --csv \\
        python -m rchem_gb300.profile_builds --workload h2o8_631g --builds 3
"""
from __future__ import annotations

import argparse
import json


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="h2o8_631g")
    ap.add_argument("--builds", type=int, default=3)
    ap.add_argument("--fp32-tau", type=float, default=0.0)
    ap.add_argument("--emulated", action="store_true", help="double-float arithmetic for the FP64 quartets")
    a = ap.parse_args(argv)
    import numpy as np
    import torch

    from . import geometry
    from .basis import Basis, JK_direct

    bname, Z, R = geometry.config(a.workload)
    b = Basis(Z, R, bname)
    n = b.nbf
    s = torch.cuda.Stream()
    b.set_stream(s.cuda_stream)
    X = np.random.default_rng(0).normal(size=(n, n))
    D = torch.from_numpy(X @ X.T / n * 0.1).cuda()
    J, K = torch.empty_like(D), torch.empty_like(D)
    for _ in range(a.builds):
        JK_direct(J, K, b, D, fp32_tau=a.fp32_tau, emulated=a.emulated)
    torch.cuda.synchronize()
    print(json.dumps(b.class_stats()))
    b.close()


if __name__ == "__main__":
    main()
