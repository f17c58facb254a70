"""Adjoint nuclear gradients (rchem_gradient) against central finite
differences of the GPU RHF energy, through a test-harness
torch.autograd.Function: forward = SCF energy at the given coordinates,
backward = the adjoint kernels.  FD step 1e-4 bohr; tolerance 1e-6 Eh/bohr."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H_FD = 1e-4
TOL = 1e-6


class RHFEnergy:
    """torch.autograd.Function wrapper (built lazily so importing this file
    needs no torch)."""

    @staticmethod
    def make(Z, basis_name):
        import torch

        import rchem_gb300 as rc

        class _F(torch.autograd.Function):
            @staticmethod
            def forward(ctx, coords):
                R = coords.detach().cpu().numpy().reshape(-1, 3)
                with rc.Basis(Z, R, basis_name) as b:
                    res = rc.scf.rhf(b, thresh_e=1e-12, thresh_d=1e-9)
                    g = rc.scf.gradient(b, res)
                ctx.save_for_backward(g.reshape(-1).to(coords.device))
                return torch.tensor(res["e_total"], dtype=torch.float64, device=coords.device)

            @staticmethod
            def backward(ctx, gout):
                (g,) = ctx.saved_tensors
                return gout * g.view(-1, 3) if g.numel() else None

        return _F


def _energy(Z, R, name):
    import rchem_gb300 as rc

    with rc.Basis(Z, R, name) as b:
        return rc.scf.rhf(b, thresh_e=1e-12, thresh_d=1e-9)["e_total"]


def _fd_check(Z, R, name, coords_to_check=None):
    import torch

    F = RHFEnergy.make(Z, name)
    x = torch.tensor(R, dtype=torch.float64, requires_grad=True)
    e = F.apply(x)
    e.backward()
    g = x.grad.numpy().reshape(-1)
    idx = range(R.size) if coords_to_check is None else coords_to_check
    worst = 0.0
    for k in idx:
        Rp = R.copy().reshape(-1)
        Rm = R.copy().reshape(-1)
        Rp[k] += H_FD
        Rm[k] -= H_FD
        fd = (_energy(Z, Rp.reshape(-1, 3), name) - _energy(Z, Rm.reshape(-1, 3), name)) / (2 * H_FD)
        worst = max(worst, abs(fd - g[k]))
        assert abs(fd - g[k]) < TOL, (k, fd, g[k])
    return g, worst


def test_gradient_water_sto3g_fd(gpu):
    import rchem_gb300 as rc

    Z, R = rc.geometry.water_monomer()
    R = R + np.array([[0.01, -0.02, 0.03], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]])
    g, worst = _fd_check(Z, R, "sto-3g-fit")
    assert np.abs(g.reshape(-1, 3).sum(axis=0)).max() < 1e-9  # translational invariance


def test_gradient_water_631gss_fd(gpu):
    """d on O, p on H: every integral class up to (dd|dd) and their shifts."""
    import rchem_gb300 as rc

    Z, R = rc.geometry.water_monomer()
    R = R + np.array([[0.02, 0.01, -0.01], [0.0, 0.03, 0.0], [0.0, 0.0, -0.02]])
    _fd_check(Z, R, "6-31gss-fit")


def test_gradient_h2o4_631gss_fd(gpu):
    """The (H2O)4 cluster in the 6-31G**-shaped basis (100 functions), central
    differences on all 36 coordinates."""
    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config("h2o4_631gss")
    g, worst = _fd_check(Z, R, bname)
    assert np.abs(g.reshape(-1, 3).sum(axis=0)).max() < 1e-8


def test_gradient_precision_forms_h2o4(gpu):
    """The same converged density through the FP32 (fp32_tau = 1e-6) and
    double-float forms of the gradient kernels: the emulated form within 1e-10
    of FP64, the mixed forms well inside the 1e-6 Eh/bohr finite-difference
    tolerance; every form keeps translational invariance."""
    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config("h2o4_631gss")
    with rc.Basis(Z, R, bname) as b:
        res = rc.scf.rhf(b, thresh_e=1e-12, thresh_d=1e-9)
        g64 = rc.scf.gradient(b, res)
        forms = {"emulated": rc.scf.gradient(b, res, emulated=True),
                 "mixed": rc.scf.gradient(b, res, fp32_tau=1e-6),
                 "emulated_mixed": rc.scf.gradient(b, res, fp32_tau=1e-6, emulated=True)}
    tol = {"emulated": 1e-10, "mixed": 1e-7, "emulated_mixed": 1e-7}
    for k, g in forms.items():
        assert float((g - g64).abs().max()) < tol[k], (k, float((g - g64).abs().max()))
        assert float(g.sum(dim=0).abs().max()) < 1e-8, k
