"""Restricted Hartree-Fock driver around the GPU Fock build.

Follows the reference's driver (src/bin/rchem.rs:40-127) and its conventions:
symmetric orthogonalisation X = U diag(lambda^-1/2) U^T (:44-51), core-Hamiltonian
guess (:55-59), density D = C_occ C_occ^T without the factor 2 (:101-104),
F = H + 2J - K (:110-127), E_elec = sum (H + F) o D (:106-108), convergence on
|Delta E| (:84).  Added beyond the reference: DIIS extrapolation (Pulay), the
nuclear repulsion energy, a density-change criterion and the orbital energies.

Everything stays FP64 on the GPU: S^-1/2, the Fock diagonalisation (cuSOLVER
through torch.linalg.eigh) and the DIIS solve; J and K come from
librchem_gpu.so (rchem_jk_direct) on device pointers, optionally in the mixed
FP32/FP64 form or with the FP64 quartets in double-float arithmetic.
"""
from __future__ import annotations

import numpy as np

from . import basis as _b


def nuclear_repulsion(atomnos, coords) -> float:
    Z = np.asarray(atomnos, dtype=np.float64)
    R = np.asarray(coords, dtype=np.float64).reshape(-1, 3)
    e = 0.0
    for a in range(len(Z)):
        d = np.linalg.norm(R[:a] - R[a], axis=1)
        e += float(np.sum(Z[a] * Z[:a] / d))
    return e


def rhf(basis: _b.Basis, nocc: int | None = None, thresh_e: float = 1e-10, thresh_d: float = 1e-7,
        max_iter: int = 128, diis: int = 8, fp32_tau: float = 0.0, schwarz_tau: float = 1e-12, emulated=False,
        verbose=False, fp32_boys64=False, fp32_rec64=False):
    """Converge RHF for ``basis``; returns a dict with energies, D, C, eps, W."""
    import torch

    dev = torch.device("cuda")
    if nocc is None:
        nocc = int(np.sum(basis.atomnos)) // 2
    n = basis.nbf
    S = _b.S(basis, device=True)
    H = _b.T(basis, device=True) + _b.V(basis, device=True)
    w, U = torch.linalg.eigh(S)
    X = (U * w.rsqrt()) @ U.T

    def density(F):
        eps, Cp = torch.linalg.eigh(X.T @ F @ X)
        C = X @ Cp
        Co = C[:, :nocc]
        return Co @ Co.T, C, eps

    D, C, eps = density(H)
    e_new = float(torch.sum((H + H) * D))
    J = torch.empty((n, n), dtype=torch.float64, device=dev)
    K = torch.empty_like(J)
    focks, errs = [], []
    hist = []
    converged = False
    it = 0
    for it in range(1, max_iter + 1):
        _b.JK_direct(J, K, basis, D, schwarz_tau=schwarz_tau, fp32_tau=fp32_tau, emulated=emulated,
                    fp32_boys64=fp32_boys64, fp32_rec64=fp32_rec64)
        F = H + 2.0 * J - K
        e_old, e_new = e_new, float(torch.sum((H + F) * D))
        # DIIS on the orthogonalised commutator FDS - SDF
        err = X.T @ (F @ D @ S - S @ D @ F) @ X
        emax = float(err.abs().max())
        Fx = F
        if diis > 0:
            focks.append(F)
            errs.append(err)
            if len(focks) > diis:
                focks.pop(0)
                errs.pop(0)
            m = len(focks)
            if m >= 2:
                B = torch.empty((m + 1, m + 1), dtype=torch.float64, device=dev)
                B[-1, :] = -1.0
                B[:, -1] = -1.0
                B[-1, -1] = 0.0
                for i in range(m):
                    for j in range(i + 1):
                        B[i, j] = B[j, i] = torch.sum(errs[i] * errs[j])
                rhs = torch.zeros(m + 1, dtype=torch.float64, device=dev)
                rhs[-1] = -1.0
                try:
                    c = torch.linalg.solve(B, rhs)
                    Fx = sum(c[i] * focks[i] for i in range(m))
                except RuntimeError:
                    Fx = F
        D_old = D
        D, C, eps = density(Fx)
        dD = float((D - D_old).abs().max())
        hist.append((e_new, e_new - e_old, emax, dD))
        if verbose:
            print("%4d %20.12f %12.3e %10.3e %10.3e" % (it, e_new, e_new - e_old, emax, dD))
        if abs(e_new - e_old) < thresh_e and dD < thresh_d:
            converged = True
            break
    # energy at the final density with its own Fock matrix
    _b.JK_direct(J, K, basis, D, schwarz_tau=schwarz_tau, fp32_tau=fp32_tau, emulated=emulated,
                    fp32_boys64=fp32_boys64, fp32_rec64=fp32_rec64)
    F = H + 2.0 * J - K
    e_elec = float(torch.sum((H + F) * D))
    eps, Cp = torch.linalg.eigh(X.T @ F @ X)
    C = X @ Cp
    Co = C[:, :nocc]
    W = (Co * eps[:nocc]) @ Co.T  # energy-weighted density, same no-factor-2 convention as D
    e_nuc = nuclear_repulsion(basis.atomnos, basis.coords)
    return {"e_elec": e_elec, "e_nuc": e_nuc, "e_total": e_elec + e_nuc, "D": D, "C": C, "eps": eps, "W": W,
            "F": F, "H": H, "S": S, "iterations": it, "converged": converged, "history": hist}


def gradient(basis: _b.Basis, res: dict | None = None, schwarz_tau: float = 1e-12, fp32_tau: float = 0.0,
             emulated: bool = False, **scf_kw):
    """Nuclear gradient dE/dR (natoms x 3, hartree/bohr) of the converged RHF
    energy, from the adjoint kernels of librchem_gpu.so (rchem_gradient): the
    derivative integrals are contracted on the GPU with D and W = sum_i eps_i
    C_i C_i^T and never stored.  ``fp32_tau`` > 0 computes the s/p quartets
    whose Schwarz product is below it in FP32; ``emulated`` the other s/p
    quartets in double-float arithmetic.  Runs the SCF first when ``res`` is None."""
    import ctypes as C

    import torch

    from . import _lib

    if res is None:
        res = rhf(basis, schwarz_tau=schwarz_tau, **scf_kw)
    if not _b._same_kind(res["D"], res["W"]):
        raise ValueError("D and W must be CUDA tensors")
    D = res["D"].contiguous()
    W = res["W"].contiguous()
    n = basis.nbf
    _b._check_f64(D, "D", shape=(n, n))
    _b._check_f64(W, "W", shape=(n, n))
    g = torch.empty(3 * len(basis.atomnos), dtype=torch.float64, device=D.device)
    o = _lib.JKOpts(schwarz_tau=schwarz_tau if schwarz_tau > 0 else -1.0, fp32_tau=fp32_tau, where=_lib.DEVICE,
                    emulated=1 if emulated else 0)
    _b._after_torch(basis, D, W, g)
    _lib.check(_lib.lib().rchem_gradient(basis.handle, C.c_void_p(D.data_ptr()), C.c_void_p(W.data_ptr()),
                                         C.c_void_p(g.data_ptr()), C.byref(o)))
    return g.view(-1, 3)
