"""Batched geometries: one basis handle, one Fock-build launch set for all of
them.  Each geometry's block must equal what a single-geometry handle gives."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _geoms(count=9, seed=3):
    import rchem_gb300 as rc

    return rc.geometry.water_batch(count, seed=seed)


def test_batched_fock_and_onee_match_single(gpu):
    import torch

    import rchem_gb300 as rc

    geoms = _geoms()
    bb = rc.batch.BatchBasis(geoms, "6-31g-fit")
    assert bb.ngeom == len(geoms)
    rng = np.random.default_rng(0)
    D = torch.zeros(bb.packed, dtype=torch.float64, device="cuda")
    blocks = []
    for g in range(bb.ngeom):
        n = int(bb.geom_nbf[g])
        X = rng.normal(size=(n, n)) * 0.2
        Dg = X @ X.T / n
        blocks.append(Dg)
        o = int(bb.offsets[g])
        D[o:o + n * n] = torch.from_numpy(Dg.reshape(-1)).cuda()
    J, K = torch.empty_like(D), torch.empty_like(D)
    rc.batch.jk(bb, D, J, K)
    S = rc.batch._packed_matrix(rc._lib.lib().rchem_S, bb)
    V = rc.batch._packed_matrix(rc._lib.lib().rchem_V, bb)
    for g, (Z, R) in enumerate(geoms):
        with rc.Basis(Z, R, "6-31g-fit") as b:
            n = b.nbf
            assert n == int(bb.geom_nbf[g])
            Js, Ks = np.zeros((n, n)), np.zeros((n, n))
            rc.JK_direct(Js, Ks, b, blocks[g])
            np.testing.assert_allclose(bb.block(J, g).cpu().numpy(), Js, atol=1e-12, rtol=0)
            np.testing.assert_allclose(bb.block(K, g).cpu().numpy(), Ks, atol=1e-12, rtol=0)
            np.testing.assert_allclose(bb.block(S, g).cpu().numpy(), rc.S(b), atol=1e-13, rtol=0)
            np.testing.assert_allclose(bb.block(V, g).cpu().numpy(), rc.V(b), atol=1e-12, rtol=0)
    bb.close()


def test_batched_rhf_and_gradient_match_single(gpu):
    import rchem_gb300 as rc

    geoms = _geoms(6, seed=5)
    bb = rc.batch.BatchBasis(geoms, "6-31g-fit")
    res = rc.batch.rhf_batch(bb, thresh_e=1e-11, thresh_d=1e-8)
    grads = rc.batch.gradient_batch(bb, res)
    assert res["converged"]
    for g, (Z, R) in enumerate(geoms):
        with rc.Basis(Z, R, "6-31g-fit") as b:
            r1 = rc.scf.rhf(b, thresh_e=1e-11, thresh_d=1e-8)
            g1 = rc.scf.gradient(b, r1).cpu().numpy()
        assert abs(res["e_total"][g] - r1["e_total"]) < 1e-9, g
        np.testing.assert_allclose(grads[g], g1, atol=1e-7, rtol=0)
    bb.close()


@pytest.mark.parametrize("n", [1, 2, 5, 13, 26, 39, 64])
def test_eigh_batched_vs_lapack(gpu, n):
    """rchem_eigh_batched against LAPACK (numpy) on random symmetric matrices,
    one with a degenerate spectrum and the zero matrix: eigenvalues to 1e-13 of
    the norm, A V = V diag(w), V^T V = I."""
    import torch

    import rchem_gb300 as rc

    rng = np.random.default_rng(n)
    X = rng.normal(size=(6, n, n))
    A = X + X.transpose(0, 2, 1)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    A[4] = Q @ np.diag(np.repeat(np.arange((n + 2) // 3), 3)[:n].astype(float)) @ Q.T  # triply degenerate
    A[5] = 0.0
    At = torch.from_numpy(A).cuda()
    w, V = rc.batch.eigh(At)
    torch.cuda.synchronize()
    w, V = w.cpu().numpy(), V.cpu().numpy()
    for b in range(A.shape[0]):
        scale = max(1.0, np.abs(A[b]).max())
        np.testing.assert_allclose(w[b], np.linalg.eigvalsh(A[b]), atol=1e-13 * scale * n, rtol=0)
        assert np.all(np.diff(w[b]) >= 0)
        assert np.abs(A[b] @ V[b] - V[b] * w[b]).max() < 1e-12 * scale * n
        assert np.abs(V[b].T @ V[b] - np.eye(n)).max() < 1e-13 * n


def test_eigh_batched_rejects_large_n(gpu):
    import torch

    import rchem_gb300 as rc

    with pytest.raises(rc.RchemError):
        rc.batch.eigh(torch.zeros((2, 65, 65), dtype=torch.float64, device="cuda"))


def test_batched_gradient_precision_forms(gpu):
    """Batched gradients in the emulated and mixed forms against FP64."""
    import rchem_gb300 as rc

    bb = rc.batch.BatchBasis(_geoms(6, seed=8), "6-31g-fit")
    res = rc.batch.rhf_batch(bb, thresh_e=1e-11, thresh_d=1e-8)
    g64 = np.concatenate(rc.batch.gradient_batch(bb, res))
    gem = np.concatenate(rc.batch.gradient_batch(bb, res, emulated=True))
    gmx = np.concatenate(rc.batch.gradient_batch(bb, res, fp32_tau=1e-6, emulated=True))
    assert np.abs(gem - g64).max() < 1e-10
    assert np.abs(gmx - g64).max() < 1e-7
    bb.close()


def test_native_rhf_matches_python_driver(gpu):
    """rchem_rhf (the SCF loop inside the library) against the Python batched
    driver: same energies, densities and energy-weighted densities; and the
    water monomer against the reference-generated STO-3G energy."""
    import rchem_gb300 as rc
    from conftest import load_npz

    bb = rc.batch.BatchBasis(_geoms(6, seed=9), "6-31g-fit")
    rn = rc.batch.rhf_native(bb, thresh_e=1e-12, thresh_d=1e-9)
    rp = rc.batch.rhf_batch(bb, thresh_e=1e-12, thresh_d=1e-9)
    assert rn["converged"] and rp["converged"]
    np.testing.assert_allclose(rn["e_total"], rp["e_total"], atol=1e-9, rtol=0)
    np.testing.assert_allclose(rn["e_nuc"], rp["e_nuc"], atol=1e-12, rtol=0)
    assert float((rn["D"] - rp["D"]).abs().max()) < 1e-6
    assert float((rn["W"] - rp["W"]).abs().max()) < 1e-6
    # gradients from the native densities equal the Python driver's
    g_n = np.concatenate(rc.batch.gradient_batch(bb, rn))
    g_p = np.concatenate(rc.batch.gradient_batch(bb, rp))
    assert np.abs(g_n - g_p).max() < 1e-6
    bb.close()
    g = load_npz("h2o_sto3g")
    Z, R = rc.geometry.water_monomer()
    with rc.Basis(Z, R, "sto-3g-fit") as b:
        r1 = rc.batch.rhf_native(b, thresh_e=1e-12, thresh_d=1e-9)
    assert r1["converged"]
    assert abs(r1["e_elec"][0] - float(g["e_elec"])) < 1e-10
    assert abs(r1["e_nuc"][0] - float(g["e_nuc"])) < 1e-12


def test_native_rhf_graph_loop_equals_host_loop(gpu):
    """rchem_rhf runs its loop as one graph launch (a WHILE conditional node
    whose condition the device-side convergence check clears) on a capturable
    stream, and one iteration per host launch on the legacy default stream,
    which cannot be captured: the same iterations, energies and densities."""
    import torch

    import rchem_gb300 as rc

    side = torch.cuda.Stream()  # a capturable stream of the caller's
    for emulated, tau32 in ((False, 0.0), (True, 1e-6)):
        bb = rc.batch.BatchBasis(_geoms(9, seed=4), "6-31g-fit")
        try:
            rg = rc.batch.rhf_native(bb, thresh_e=1e-11, thresh_d=1e-8, fp32_tau=tau32, emulated=emulated)
            bb.set_stream(0)  # the legacy default stream: the host-driven loop
            rh = rc.batch.rhf_native(bb, thresh_e=1e-11, thresh_d=1e-8, fp32_tau=tau32, emulated=emulated)
            assert rg["converged"] and rh["converged"]
            assert rg["iterations"] == rh["iterations"]
            np.testing.assert_allclose(rg["e_total"], rh["e_total"], atol=1e-11, rtol=0)
            assert float((rg["D"] - rh["D"]).abs().max()) < 1e-10
            # an iteration cap ends the graph loop too, unconverged
            bb.set_stream(side.cuda_stream)
            rc_ = rc.batch.rhf_native(bb, max_iter=3)
            assert rc_["iterations"] == 3 and not rc_["converged"]
        finally:
            bb.close()


def test_native_rhf_rejects_large_geometries(gpu):
    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config("h2o8_631g")  # 104 functions
    with rc.Basis(Z, R, bname) as b:
        with pytest.raises(rc.RchemError):
            rc.batch.rhf_native(b)
