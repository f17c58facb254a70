"""The RHF driver (rchem_gb300.scf, the loop of src/bin/rchem.rs:40-127 with
DIIS) around the GPU Fock build, S^-1/2 and eigh in FP64 on the GPU."""
import numpy as np
import pytest

from conftest import load_npz

pytestmark = pytest.mark.gpu


def test_rhf_water_matches_reference_energy(gpu):
    import rchem_gb300 as rc

    g = load_npz("h2o_sto3g")
    Z, R = rc.geometry.water_monomer()
    with rc.Basis(Z, R, "sto-3g-fit") as b:
        res = rc.scf.rhf(b, thresh_e=1e-12, thresh_d=1e-9)
    assert res["converged"]
    assert abs(res["e_elec"] - float(g["e_elec"])) < 1e-10
    assert abs(res["e_nuc"] - float(g["e_nuc"])) < 1e-12
    np.testing.assert_allclose(res["D"].cpu().numpy(), g["D_scf"], atol=1e-7)


def test_rhf_mixed_precision_energy_error(gpu):
    """(H2O)8, 6-31G-shaped basis: the mixed FP32/FP64 Fock build converges to
    the FP64 energy within 1 microhartree."""
    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config("h2o8_631g")
    with rc.Basis(Z, R, bname) as b:
        e64 = rc.scf.rhf(b, thresh_e=1e-10)
        e32 = rc.scf.rhf(b, thresh_e=1e-10, fp32_tau=1e-6)
    assert e64["converged"] and e32["converged"]
    assert abs(e32["e_total"] - e64["e_total"]) < 1e-6
    assert float((e32["D"] - e64["D"]).abs().max()) < 1e-5


def test_rhf_energy_variational_and_virial(gpu):
    """Size-independent checks at full size: the converged density is
    idempotent in the S metric (D S D = D), has tr(D S) = nocc, and the
    energy is stationary (the DIIS commutator vanishes)."""
    import torch

    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config("h2o8_631g")
    with rc.Basis(Z, R, bname) as b:
        res = rc.scf.rhf(b, thresh_e=1e-11)
    D, S, F = res["D"], res["S"], res["F"]
    nocc = int(sum(Z)) // 2
    assert abs(float(torch.trace(D @ S)) - nocc) < 1e-8
    assert float((D @ S @ D - D).abs().max()) < 1e-7
    comm = F @ D @ S - S @ D @ F
    assert float(comm.abs().max()) < 1e-5


def test_rhf_emulated_fp64_energy(gpu):
    """(H2O)8, 6-31G-shaped basis: the SCF on the emulated-FP64 Fock build
    lands on the FP64 energy within 1e-9 Eh."""
    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config("h2o8_631g")
    with rc.Basis(Z, R, bname) as b:
        e64 = rc.scf.rhf(b, thresh_e=1e-11)
        eem = rc.scf.rhf(b, thresh_e=1e-11, emulated=True)
    assert e64["converged"] and eem["converged"]
    assert abs(eem["e_total"] - e64["e_total"]) < 1e-9
    assert float((eem["D"] - e64["D"]).abs().max()) < 1e-7
