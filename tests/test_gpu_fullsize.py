"""GPU parity at the benchmarked sizes, against the oracle.

* (H2O)8, 6-31G-shaped (104 functions): every element of J and K against the
  oracle's 8-fold, Schwarz-screened build over the reference's integrals;
* (H2O)32, 6-31G*-shaped (608 functions, the headline Fock build): 216 seeded
  J/K elements, chosen so that every (l_mu, l_nu) pair type -- and so every
  one of the 21 integral classes, the warp-cooperative lists included -- is
  represented, straight from the definitions of src/basis.rs:406-417;
* (H2O)4, 6-31G**-shaped (100 functions): the converged RHF energy against
  the oracle's SCF (src/bin/rchem.rs:40-127 restated, over the oracle's ERI
  tensor);
* the 512-geometry batch: a seeded sample of monomers, dimers and trimers,
  each energy of the library's batched SCF against the oracle's SCF.

The oracle runs the reference's THO integrals with an exact Boys function;
its element and tensor builds skip a contracted integral only when its
Schwarz bound Q_ab Q_cd is below 1e-15, three orders under the library's
1e-12 screen, so they stand for the unscreened sums.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ORACLE_TAU = 1e-15


def sym_density(rng, n, scale=0.2):
    X = rng.normal(size=(n, n)) * scale
    return X @ X.T / n


def pick_elements(ob, coords, rng, per=9):
    """(mu, nu) pairs: for every pair of angular momenta (l_mu >= l_nu), ``per``
    pairs on one atom, on one water, on neighbouring atoms (< 6 bohr) and
    anywhere."""
    R = np.asarray(coords).reshape(-1, 3)
    ls = ob.powers.sum(axis=1)
    atom = ob.atom
    water = atom // 3
    dist = np.linalg.norm(R[:, None, :] - R[None, :, :], axis=2)
    mus, nus = [], []
    for lm in range(3):
        for ln in range(lm + 1):
            cand_m = np.flatnonzero(ls == lm)
            cand_n = np.flatnonzero(ls == ln)
            if cand_m.size == 0 or cand_n.size == 0:
                continue
            for rule in ("atom", "water", "near", "any"):
                got = 0
                for _ in range(2000):
                    if got == per:
                        break
                    m = int(rng.choice(cand_m))
                    if rule == "atom":
                        pool = cand_n[atom[cand_n] == atom[m]]
                    elif rule == "water":
                        pool = cand_n[water[cand_n] == water[m]]
                    elif rule == "near":
                        pool = cand_n[(dist[atom[m], atom[cand_n]] < 6.0) & (water[cand_n] != water[m])]
                    else:
                        pool = cand_n
                    if pool.size == 0:
                        continue
                    mus.append(m)
                    nus.append(int(rng.choice(pool)))
                    got += 1
    return np.asarray(mus, dtype=np.int32), np.asarray(nus, dtype=np.int32)


def test_h2o8_full_jk_vs_oracle(gpu, oracle_mod):
    """Every element of J and K of (H2O)8 in the 6-31G-shaped basis, FP64 and
    emulated FP64, against the oracle's whole screened build."""
    import rchem_gb300 as rc

    O = oracle_mod
    bname, Z, R = rc.geometry.config("h2o8_631g")
    ob = O.expand_basis(Z, R, rc.load_bse(bname))
    D = sym_density(np.random.default_rng(21), ob.n)
    Q = O.schwarz(ob)
    Jr, Kr, _ = O.JK_sym_screened(ob, D, Q, ORACLE_TAU)
    with rc.Basis(Z, R, bname) as b:
        n = b.nbf
        assert n == ob.n == 104
        b.autotune(1e-12, 0.0)
        J, K = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J, K, b, D)
        assert np.abs(J - Jr).max() <= 1e-11, np.abs(J - Jr).max()
        assert np.abs(K - Kr).max() <= 1e-11, np.abs(K - Kr).max()
        b.autotune(1e-12, 0.0, emulated=True)
        rc.JK_direct(J, K, b, D, emulated=True)
        assert np.abs(J - Jr).max() <= 1e-11, np.abs(J - Jr).max()
        assert np.abs(K - Kr).max() <= 1e-11, np.abs(K - Kr).max()


@pytest.fixture(scope="module")
def h2o32_oracle(oracle_mod):
    import rchem_gb300 as rc

    O = oracle_mod
    bname, Z, R = rc.geometry.config("h2o32_631gs")
    ob = O.expand_basis(Z, R, rc.load_bse(bname))
    mus, nus = pick_elements(ob, R, np.random.default_rng(11))
    D = sym_density(np.random.default_rng(5), ob.n)
    Q = O.schwarz(ob)
    Je, Ke = O.JK_elements_screened(ob, D, Q, ORACLE_TAU, mus, nus)
    return {"bname": bname, "Z": Z, "R": R, "ob": ob, "mus": mus, "nus": nus, "D": D, "J": Je, "K": Ke}


def test_h2o32_elements_cover_every_class(h2o32_oracle):
    """The sample has every bra pair type, so every class (ab|cd) of the
    build is in some J element (its bra pair type) and in the K elements."""
    ob, mus, nus = h2o32_oracle["ob"], h2o32_oracle["mus"], h2o32_oracle["nus"]
    ls = ob.powers.sum(axis=1)
    types = {(max(a, b), min(a, b)) for a, b in zip(ls[mus], ls[nus])}
    assert types == {(0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2)}
    assert len(mus) >= 200
    # enough of them are large: the comparison is not on zeros
    assert (np.abs(h2o32_oracle["J"]) > 1e-3).sum() >= 50
    assert (np.abs(h2o32_oracle["K"]) > 1e-4).sum() >= 50


@pytest.mark.parametrize("emulated,fp32_tau,bmode,tol", [(False, 0.0, "fp32", 1e-11), (True, 0.0, "fp32", 1e-11),
                                                         (False, 1e-6, "fp32", 1e-7), (False, 1e-6, "boys64", 1e-7),
                                                         (False, 1e-6, "rec64", 1e-7)])
def test_h2o32_sampled_elements_vs_oracle(gpu, h2o32_oracle, emulated, fp32_tau, bmode, tol):
    """(H2O)32 in the 6-31G*-shaped basis with the autotuned plan the bench
    times (warp-cooperative kernels for the large classes): 216 J/K elements
    against the oracle, FP64 and emulated FP64 at 1e-11; the mixed form
    (FP32 below 1e-6, its Boys function in FP32, in FP64, or FP32 with the
    recursion in FP64) at 1e-7."""
    import torch

    import rchem_gb300 as rc

    o = h2o32_oracle
    with rc.Basis(o["Z"], o["R"], o["bname"]) as b:
        n = b.nbf
        assert n == 608
        fl = {"fp32_boys64": bmode == "boys64", "fp32_rec64": bmode == "rec64"}
        chosen = b.autotune(1e-12, fp32_tau, emulated=emulated, **fl)
        if not emulated and fp32_tau == 0.0:
            assert any(v <= 0 for (k, p), v in chosen.items() if p == 0)  # some list runs warp-cooperatively
        D = torch.from_numpy(o["D"]).cuda()
        J, K = torch.empty_like(D), torch.empty_like(D)
        rc.JK_direct(J, K, b, D, fp32_tau=fp32_tau, emulated=emulated, **fl)
        J, K = J.cpu().numpy(), K.cpu().numpy()
    dJ = np.abs(J[o["mus"], o["nus"]] - o["J"]).max()
    dK = np.abs(K[o["mus"], o["nus"]] - o["K"]).max()
    assert dJ <= tol and dK <= tol, (dJ, dK)
    assert np.abs(J - J.T).max() == 0.0 and np.abs(K - K.T).max() == 0.0


def _oracle_scf(O, ob, Z, R, nocc):
    Q = O.schwarz(ob)
    I = O.eri_packed(ob, Q, ORACLE_TAU)
    r = O.rhf(ob, Z, R, nocc, jk=lambda Dm: O.JK_packed(ob.n, I, Dm), thresh_e=1e-11, thresh_d=1e-8, diis=8,
              max_iter=200)
    assert r["converged"]
    return r["e_final"] + r["e_nuc"], r["D"]


def test_h2o4_scf_energy_vs_oracle(gpu, oracle_mod):
    """(H2O)4 in the 6-31G**-shaped basis: the converged RHF energy of the GPU
    driver (FP64) against the oracle's SCF at 1e-10 Eh; the mixed form (below
    1e-6 the Boys function in FP32, in FP64, or FP32 with its recursion in
    FP64) and emulated+mixed within 1e-9 Eh of the oracle."""
    import rchem_gb300 as rc

    O = oracle_mod
    bname, Z, R = rc.geometry.config("h2o4_631gss")
    ob = O.expand_basis(Z, R, rc.load_bse(bname))
    nocc = int(np.sum(Z)) // 2
    e_ref, D_ref = _oracle_scf(O, ob, Z, R, nocc)
    with rc.Basis(Z, R, bname) as b:
        r = rc.scf.rhf(b, thresh_e=1e-11, thresh_d=1e-8)
        assert r["converged"]
        assert abs(r["e_total"] - e_ref) < 1e-10, (r["e_total"], e_ref)
        assert float(np.abs(r["D"].cpu().numpy() - D_ref).max()) < 1e-6
        for tau32, emul, b64, r64 in ((1e-6, False, False, False), (1e-6, True, False, False),
                                      (1e-6, False, True, False), (1e-6, False, False, True)):
            r2 = rc.scf.rhf(b, thresh_e=1e-11, thresh_d=1e-8, fp32_tau=tau32, emulated=emul, fp32_boys64=b64,
                            fp32_rec64=r64)
            assert abs(r2["e_total"] - e_ref) < 1e-9, (tau32, emul, b64, r64, r2["e_total"] - e_ref)


def test_batch_sample_energies_vs_oracle(gpu, oracle_mod):
    """The 512-geometry batch (monomers, dimers, trimers in the 6-31G-shaped
    basis) through the library's batched SCF: a seeded sample of four
    geometries per size against the oracle's SCF at 1e-10 Eh."""
    import rchem_gb300 as rc

    O = oracle_mod
    geoms = rc.geometry.water_batch(512, seed=7)
    bb = rc.batch.BatchBasis(geoms, "6-31g-fit")
    try:
        r = rc.batch.rhf_native(bb, thresh_e=1e-11, thresh_d=1e-8)
        assert r["converged"]
        e = np.asarray(r["e_total"])
    finally:
        bb.close()
    sizes = np.array([len(Z) // 3 for Z, _ in geoms])
    rng = np.random.default_rng(3)
    doc = rc.load_bse("6-31g-fit")
    for m in (1, 2, 3):
        for g in rng.choice(np.flatnonzero(sizes == m), size=4, replace=False):
            Z, R = geoms[g]
            ob = O.expand_basis(Z, R, doc)
            e_ref, _ = _oracle_scf(O, ob, Z, R, int(np.sum(Z)) // 2)
            assert abs(e[g] - e_ref) < 1e-10, (g, m, e[g], e_ref)
