"""GPU parity: librchem_gpu.so through its C ABI against the oracle.

Tolerances: 1e-12 absolute per integral / matrix element for the FP64 path
(the target the hot path is built to); the reference's own Boys function is
only ~1e-7 accurate, so the as-shipped numbers are compared at that level.
"""
import itertools
import math

import numpy as np
import pytest

from conftest import load_npz

pytestmark = pytest.mark.gpu


# ---- cints-compatible scalar entry points ---------------------------------
def test_scalar_eri_golden(gpu):
    from rchem_gb300 import cints
    from test_oracle import ERI_GEOM as g
    from test_oracle import ERI_GOLDEN

    for pw, ref in ERI_GOLDEN:
        v = cints.coulomb(g["za"], g["zb"], g["zc"], g["zd"], g["ra"], g["rb"], g["rc"], g["rd"], pw)
        assert abs(v - ref) < 1e-15, (pw, v, ref)


def test_scalar_onee_golden(gpu):
    from rchem_gb300 import cints
    from test_oracle import KIN_GOLDEN, NUC_GOLDEN, OVL_GOLDEN, RA, RB, RC

    for pw, ref in OVL_GOLDEN:
        assert abs(cints.overlap(1.8, 2.8, RA, RB, pw) - ref) < 1e-16
    for pw, ref in KIN_GOLDEN:
        assert abs(cints.kinetic(1.8, 2.0, RA, RB, pw) - ref) < 1e-15
    for pw, ref in NUC_GOLDEN:
        assert abs(cints.nuclear(1.8, 2.0, RA, RB, RC, pw) - ref) < 1e-15


def test_eri_batch_vs_reference_fixture(gpu, golden_eri):
    from rchem_gb300 import cints

    quartets = [[(it["R"][k], 1.0, it["alpha"][k], it["powers"][k]) for k in range(4)] for it in golden_eri]
    v = cints.eri_batch(quartets)
    ex = np.array([it["exact"] for it in golden_eri])
    sh = np.array([it["shipped"] for it in golden_eri])
    assert np.abs(v - ex).max() < 1e-12
    # against the reference as shipped: its NR Boys function limits agreement
    assert np.all(np.abs(v - sh) <= 2e-7 * np.maximum(np.abs(sh), 1e-3))


def test_onee_batch_vs_reference_fixture(gpu, golden_onee):
    from rchem_gb300 import cints

    for it in golden_onee:
        a, pw = it["alpha"], it["pa"] + it["pb"]
        assert abs(cints.overlap(a[0], a[1], it["A"], it["B"], pw) - it["S_exact"]) < 1e-13
        assert abs(cints.kinetic(a[0], a[1], it["A"], it["B"], pw) - it["T_exact"]) < 1e-12
        assert abs(cints.nuclear(a[0], a[1], it["A"], it["B"], it["C"], pw) - it["V_exact"]) < 1e-12


def test_boys_batch(gpu, port):
    from rchem_gb300 import cints

    ms, xs = [], []
    for m in range(0, 13):
        for x in (0.0, 1e-12, 1e-3, 0.0312, 0.7, 3.3, 9.9, 17.0, 29.0, 39.97, 40.0, 40.5, 55.0, 120.0, 5000.0):
            ms.append(m)
            xs.append(x)
    ex = np.array([port.boys_exact(m, x) for m, x in zip(ms, xs)])
    v64 = cints.boys_batch(ms, xs, 64)
    v32 = cints.boys_batch(ms, xs, 32)
    assert np.all(np.abs(v64 - ex) <= 4e-15 * ex)
    # the ERI kernels' branch-free evaluation (m <= 8): Taylor rows, the power
    # law past T = 80 (both sides of the switch in the sample), L = 8 recursion
    lo = np.array(ms) <= 8
    xs_u = list(np.array(xs)[lo]) + [79.99, 80.0, 80.01, 1e4, 3.7e7]
    ms_u = list(np.array(ms)[lo]) + [8, 8, 0, 3, 1]
    ex_u = np.array([port.boys_exact(m, x) for m, x in zip(ms_u, xs_u)])
    vu = cints.boys_batch(ms_u, xs_u, 65)
    assert np.all(np.abs(vu - ex_u) <= 2e-15 * ex_u), np.max(np.abs(vu - ex_u) / ex_u)
    normal32 = ex > 1e-30  # below that the single-precision values are subnormal
    # the FP32 form (screened-weak quartets only) loses ~m ulps in the upward recursion
    assert np.all(np.abs(v32 - ex)[normal32] <= 1e-5 * ex[normal32])
    assert abs(cints.fgamma(2, 1.5) - port.boys_exact(2, 1.5)) < 1e-16


def test_contr_coulomb(gpu, port):
    import ctypes as C

    from rchem_gb300 import _lib

    L = _lib.lib()
    e = np.array([1.3, 0.4])
    c = np.array([0.6, 0.5])
    nrm = np.array([port.pgto_norm(x, 1, 0, 0) for x in e])
    args = []
    for R in ([0, 0, 0], [0, 0, 1.4], [1.0, 0, 0], [0, 1.2, 0.3]):
        args += [2, e.ctypes.data, c.ctypes.data, nrm.ctypes.data, *R, 1, 0, 0]
    v = L.contr_coulomb(*args)
    ref = 0.0
    for i, j, k, l in itertools.product(range(2), repeat=4):
        ref += c[i] * c[j] * c[k] * c[l] * port.coulomb_repulsion(
            [0, 0, 0], nrm[i], [1, 0, 0], e[i], [0, 0, 1.4], nrm[j], [1, 0, 0], e[j],
            [1.0, 0, 0], nrm[k], [1, 0, 0], e[k], [0, 1.2, 0.3], nrm[l], [1, 0, 0], e[l])
    assert abs(v - ref) < 1e-13


# ---- matrix API against the reference-generated fixtures ---------------------
@pytest.mark.parametrize("tag,name", [("h2o_sto3g", "sto-3g-fit"), ("h2o_631g", "6-31g-fit"),
                                      ("h2o_631gs", "6-31gs-fit")])
def test_matrices_vs_reference_fixture(gpu, tag, name):
    import rchem_gb300 as rc

    g = load_npz(tag)
    Z, R = rc.geometry.water_monomer()
    with rc.Basis(Z, R, name) as b:
        np.testing.assert_allclose(rc.S(b), g["S"], atol=1e-12, rtol=0)
        np.testing.assert_allclose(rc.T(b), g["T"], atol=1e-12, rtol=0)
        np.testing.assert_allclose(rc.V(b, R, Z), g["V"], atol=1e-12, rtol=0)
        n = b.nbf
        J, K = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J, K, b, g["D"], schwarz_tau=0.0)  # no screening: exact semantics
        np.testing.assert_allclose(J, g["J"], atol=1e-12, rtol=0)
        np.testing.assert_allclose(K, g["K"], atol=1e-12, rtol=0)
        rc.JK_direct(J, K, b, g["D"])  # Schwarz 1e-12
        np.testing.assert_allclose(J, g["J"], atol=1e-11, rtol=0)
        np.testing.assert_allclose(K, g["K"], atol=1e-11, rtol=0)
        if "I" in g:
            I = rc.build_I(b)
            np.testing.assert_allclose(I, g["I"], atol=1e-12, rtol=0)
            Ji, Ki = rc.JK_inmem(I, g["D"])
            np.testing.assert_allclose(Ji, g["J"], atol=1e-12, rtol=0)
            np.testing.assert_allclose(Ki, g["K"], atol=1e-12, rtol=0)


def test_device_pointers_and_torch_stream(gpu):
    torch = pytest.importorskip("torch")
    import rchem_gb300 as rc

    g = load_npz("h2o_631g")
    Z, R = rc.geometry.water_monomer()
    with rc.Basis(Z, R, "6-31g-fit") as b:
        s = torch.cuda.Stream()
        b.set_stream(s.cuda_stream)
        D = torch.from_numpy(g["D"]).cuda()
        J = torch.empty_like(D)
        K = torch.empty_like(D)
        with torch.cuda.stream(s):
            rc.JK_direct(J, K, b, D, schwarz_tau=0.0)
        torch.cuda.synchronize()
        np.testing.assert_allclose(J.cpu().numpy(), g["J"], atol=1e-12, rtol=0)
        np.testing.assert_allclose(K.cpu().numpy(), g["K"], atol=1e-12, rtol=0)
        Sd = rc.S(b, device=True)
        np.testing.assert_allclose(Sd.cpu().numpy(), g["S"], atol=1e-12, rtol=0)


def _sym_density(rng, n, scale=0.2):
    X = rng.normal(size=(n, n)) * scale
    return X @ X.T / n


@pytest.mark.parametrize("name,nw,box", [("6-31gss-fit", 2, 4.5), ("6-31gs-fit", 2, 5.0)])
def test_jk_vs_oracle_dimer(gpu, oracle_mod, name, nw, box):
    """All 21 classes in play (d on O, p on H): GPU vs the 8-fold oracle."""
    import rchem_gb300 as rc

    O = oracle_mod
    Z, R = rc.geometry.water_cluster(nw, box, seed=11)
    ob = O.expand_basis(Z, R, rc.load_bse(name))
    D = _sym_density(np.random.default_rng(1), ob.n)
    Jr, Kr = O.JK_sym(ob, D)
    with rc.Basis(Z, R, name) as b:
        n = b.nbf
        J, K = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J, K, b, D, schwarz_tau=0.0)
        assert np.abs(J - Jr).max() < 1e-12
        assert np.abs(K - Kr).max() < 1e-12
        rc.JK_direct(J, K, b, D)
        assert np.abs(J - Jr).max() < 1e-10
        assert np.abs(K - Kr).max() < 1e-10
        np.testing.assert_allclose(rc.S(b), O.S(ob), atol=1e-12, rtol=0)
        np.testing.assert_allclose(rc.T(b), O.T(ob), atol=1e-12, rtol=0)
        np.testing.assert_allclose(rc.V(b), O.V(ob, R, Z), atol=1e-11, rtol=0)


def test_jk_full_size_h2o8_sampled(gpu, oracle_mod):
    """(H2O)8 in the 6-31G-shaped basis (104 functions): sampled elements of J
    and K straight from their definitions (basis.rs:406-417) on the CPU, plus
    size-independent properties of the whole matrices."""
    import rchem_gb300 as rc

    O = oracle_mod
    bname, Z, R = rc.geometry.config("h2o8_631g")
    ob = O.expand_basis(Z, R, rc.load_bse(bname))
    D = _sym_density(np.random.default_rng(2), ob.n)
    with rc.Basis(Z, R, bname) as b:
        n = b.nbf
        assert n == 104
        J, K = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J, K, b, D)
        st = b.stats()
        # properties: symmetry, J linear in D, Tr(D J) = sum (mn|ls) D_mn D_ls >= 0
        assert np.abs(J - J.T).max() == 0.0 and np.abs(K - K.T).max() == 0.0
        assert float(np.sum(D * J)) > 0.0
        J2, K2 = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J2, K2, b, 2.0 * D)
        np.testing.assert_allclose(J2, 2.0 * J, atol=1e-11, rtol=0)
        np.testing.assert_allclose(K2, 2.0 * K, atol=1e-11, rtol=0)
        # sampled elements
        mus = [0, 5, 40, 77, 103]
        nus = [0, 17, 40, 3, 60]
        Je, Ke = O.JK_elements(ob, D, mus, nus)
        for k in range(len(mus)):
            assert abs(J[mus[k], nus[k]] - Je[k]) < 1e-10
            assert abs(K[mus[k], nus[k]] - Ke[k]) < 1e-10
        assert st["quartets_fp64"] > 0 and st["quartets_fp32"] == 0


def test_mixed_precision_close_to_fp64(gpu):
    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config("h2o8_631g")
    D = _sym_density(np.random.default_rng(2), 104)
    with rc.Basis(Z, R, bname) as b:
        n = b.nbf
        J, K = np.zeros((n, n)), np.zeros((n, n))
        Jm, Km = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J, K, b, D)
        rc.JK_direct(Jm, Km, b, D, fp32_tau=1e-6)
        st = b.stats()
        assert st["quartets_fp32"] > 0
        # every FP32 quartet is bounded by 1e-6: per-element error well below 1e-8
        assert np.abs(Jm - J).max() < 1e-8
        assert np.abs(Km - K).max() < 1e-8
        assert abs(float(np.sum(D * (Jm - J)))) < 1e-8
        # the same FP32 quartets with the Boys function and its recursion in FP64
        Jb, Kb = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(Jb, Kb, b, D, fp32_tau=1e-6, fp32_boys64=True)
        assert b.stats()["quartets_fp32"] == st["quartets_fp32"]
        assert np.abs(Jb - J).max() < 1e-8 and np.abs(Kb - K).max() < 1e-8
        assert np.abs(Jb - Jm).max() > 0.0  # a different evaluation did run
        # ... with only the Boys function's recursion in FP64 (the stated form)
        Jr, Kr = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(Jr, Kr, b, D, fp32_tau=1e-6, fp32_rec64=True)
        assert b.stats()["quartets_fp32"] == st["quartets_fp32"]
        assert np.abs(Jr - J).max() < 1e-8 and np.abs(Kr - K).max() < 1e-8
        assert np.abs(Jr - Jm).max() > 0.0
        # an unknown flag, or both FP64 Boys forms at once, is refused before any work
        from rchem_gb300 import _lib

        import ctypes as C

        for bad in (8, 6):
            o = _lib.JKOpts(schwarz_tau=1e-12, fp32_tau=1e-6, where=_lib.HOST, emulated=bad)
            assert _lib.lib().rchem_jk_direct(b.handle, D.ctypes.data, Jb.ctypes.data, Kb.ctypes.data,
                                              C.byref(o)) == _lib.RCHEM_ERR_INVALID


def test_scf_energy_with_gpu_fock(gpu, oracle_mod):
    """rchem.rs:40-89 driven by the GPU J/K and S/T/V: the fixture energy."""
    import rchem_gb300 as rc

    O = oracle_mod
    g = load_npz("h2o_sto3g")
    Z, R = rc.geometry.water_monomer()
    with rc.Basis(Z, R, "sto-3g-fit") as b:
        n = b.nbf
        H = rc.T(b) + rc.V(b)
        X = O.symm_orthog(rc.S(b))
        _, Cp = np.linalg.eigh(X.T @ H @ X)
        D = O.build_density(X @ Cp, 5)
        e = O.elec_energy(D, H, H)
        J, K = np.zeros((n, n)), np.zeros((n, n))
        for _ in range(200):
            rc.JK_direct(J, K, b, D)
            F = H + 2 * J - K
            _, Cp = np.linalg.eigh(X.T @ F @ X)
            D = O.build_density(X @ Cp, 5)
            e_old, e = e, O.elec_energy(D, H, F)
            if abs(e - e_old) < 1e-12:
                break
        assert abs(e - float(g["e_elec"])) < 1e-10


# ---- edge cases ---------------------------------------------------------
def test_single_s_function_atom(gpu, port):
    import rchem_gb300 as rc

    Z = np.array([1])
    R = np.zeros((1, 3))
    doc = {"elements": {"1": {"electron_shells": [
        {"function_type": "gto", "region": "", "angular_momentum": [0], "exponents": ["0.8"], "coefficients": [["1.0"]]}]}}}
    with rc.Basis(Z, R, doc) as b:
        assert b.nbf == 1
        S = rc.S(b)
        assert abs(S[0, 0] - 1.0) < 1e-14
        J, K = np.zeros((1, 1)), np.zeros((1, 1))
        rc.JK_direct(J, K, b, np.ones((1, 1)))
        ssss = port.coulomb_repulsion([0, 0, 0], port.pgto_norm(0.8, 0, 0, 0), [0, 0, 0], 0.8, [0, 0, 0],
                                      port.pgto_norm(0.8, 0, 0, 0), [0, 0, 0], 0.8, [0, 0, 0],
                                      port.pgto_norm(0.8, 0, 0, 0), [0, 0, 0], 0.8, [0, 0, 0],
                                      port.pgto_norm(0.8, 0, 0, 0), [0, 0, 0], 0.8)
        assert abs(J[0, 0] - ssss) < 1e-14 and abs(K[0, 0] - ssss) < 1e-14


def test_zero_density_and_errors(gpu):
    import rchem_gb300 as rc

    Z, R = rc.geometry.water_monomer()
    with rc.Basis(Z, R, "6-31gs-fit") as b:
        n = b.nbf
        J, K = np.ones((n, n)), np.ones((n, n))
        rc.JK_direct(J, K, b, np.zeros((n, n)))
        assert not J.any() and not K.any()
        with pytest.raises(ValueError):
            rc.JK_direct(J, K, b, np.zeros((n + 1, n + 1)))
    bad = {"elements": {"8": {"electron_shells": [
        {"function_type": "gto", "region": "", "angular_momentum": [3], "exponents": ["1.0"], "coefficients": [["1.0"]]}]},
        "1": {"electron_shells": [{"function_type": "gto", "region": "", "angular_momentum": [0], "exponents": ["1.0"],
                                   "coefficients": [["1.0"]]}]}}}
    with pytest.raises(rc.RchemError, match="l=3"):
        rc.Basis(Z, R, bad)


def test_autotune_keeps_results(gpu):
    """The autotuner only changes how quartets map onto lanes, never what is
    computed."""
    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config("h2o8_631g")
    D = _sym_density(np.random.default_rng(4), 104)
    with rc.Basis(Z, R, bname) as b:
        J0, K0 = np.zeros((104, 104)), np.zeros((104, 104))
        rc.JK_direct(J0, K0, b, D)
        chosen = b.autotune()
        assert len(chosen) == 42 and all(v in (0, -16, -8) or v >= 4 for v in chosen.values())
        J1, K1 = np.zeros((104, 104)), np.zeros((104, 104))
        rc.JK_direct(J1, K1, b, D)
        np.testing.assert_allclose(J1, J0, atol=1e-12, rtol=0)
        np.testing.assert_allclose(K1, K0, atol=1e-12, rtol=0)


# ---- emulated FP64: double-float arithmetic on the FP32 pipe ---------------
@pytest.mark.parametrize("name", ["6-31gss-fit", "6-31gs-fit"])
def test_emulated_fp64_vs_oracle_dimer(gpu, oracle_mod, name):
    """The emulated form keeps the FP64 form's 1e-12 bound against the 8-fold
    oracle on every class (those above total L 4 run in native FP64)."""
    import rchem_gb300 as rc

    O = oracle_mod
    Z, R = rc.geometry.water_cluster(2, 4.5, seed=11)
    ob = O.expand_basis(Z, R, rc.load_bse(name))
    D = _sym_density(np.random.default_rng(1), ob.n)
    Jr, Kr = O.JK_sym(ob, D)
    with rc.Basis(Z, R, name) as b:
        n = b.nbf
        J, K = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J, K, b, D, schwarz_tau=0.0, emulated=True)
        assert np.abs(J - Jr).max() < 1e-12
        assert np.abs(K - Kr).max() < 1e-12
        assert np.abs(J - J.T).max() == 0.0 and np.abs(K - K.T).max() == 0.0


def test_emulated_fp64_full_size_h2o8(gpu):
    """(H2O)8, 104 functions: emulated vs native FP64 J and K at 1e-12, the
    energy at fixed density at 1e-11, and the graph rebuilt when the form
    switches back and forth."""
    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config("h2o8_631g")
    D = _sym_density(np.random.default_rng(2), 104)
    with rc.Basis(Z, R, bname) as b:
        J, K = np.zeros((104, 104)), np.zeros((104, 104))
        Je, Ke = np.zeros((104, 104)), np.zeros((104, 104))
        rc.JK_direct(J, K, b, D)
        rc.JK_direct(Je, Ke, b, D, emulated=True)
        assert np.abs(Je - J).max() < 1e-12
        assert np.abs(Ke - K).max() < 1e-12
        assert abs(float(np.sum(D * (2 * (Je - J) - (Ke - K))))) < 1e-11
        J2, K2 = np.zeros((104, 104)), np.zeros((104, 104))
        rc.JK_direct(J2, K2, b, D)  # FP64 atomics: summation order varies between builds
        assert np.abs(J2 - J).max() < 1e-13 and np.abs(K2 - K).max() < 1e-13
        chosen = b.autotune(emulated=True)
        assert len(chosen) == 42
        rc.JK_direct(J2, K2, b, D, emulated=True)
        assert np.abs(J2 - J).max() < 1e-12 and np.abs(K2 - K).max() < 1e-12
        # emulated under the mixed form: FP32 below 1e-6, double-float above
        Jm, Km = np.zeros((104, 104)), np.zeros((104, 104))
        rc.JK_direct(Jm, Km, b, D, fp32_tau=1e-6, emulated=True)
        assert np.abs(Jm - J).max() < 1e-8 and np.abs(Km - K).max() < 1e-8


def test_emulated_fp64_device_and_batch(gpu):
    """Device pointers and a six-geometry batch in the emulated form."""
    import torch

    import rchem_gb300 as rc

    geoms = rc.geometry.water_batch(6, seed=3)
    bb = rc.batch.BatchBasis(geoms, "6-31g-fit")
    rng = np.random.default_rng(5)
    Dh = np.zeros(bb.packed)
    for g in range(bb.ngeom):
        n = int(bb.geom_nbf[g])
        bb.block(Dh, g)[:] = _sym_density(rng, n)
    D = torch.from_numpy(Dh).cuda()
    J, K = torch.empty_like(D), torch.empty_like(D)
    Je, Ke = torch.empty_like(D), torch.empty_like(D)
    rc.batch.jk(bb, D, J, K)
    rc.batch.jk(bb, D, Je, Ke, emulated=True)
    assert float((Je - J).abs().max()) < 1e-12
    assert float((Ke - K).abs().max()) < 1e-12
    bb.close()


@pytest.mark.parametrize("name", ["6-31gss-fit", "6-31gs-fit"])
@pytest.mark.parametrize("shape", [0, -16, -8, 16])
def test_warp_cooperative_classes_vs_oracle(gpu, oracle_mod, name, shape):
    """The warp-cooperative J/K kernel of the large classes (total L >= 4) with
    32, 16 and 8 lanes per quartet (1, 2, 4 quartets per warp), or their
    one-lane-group kernel (16 primitive quartets per lane; (dd|dd) has none and
    stays warp-cooperative), forced on every such list, FP64, emulated FP64 and
    FP32, against the 8-fold oracle."""
    import rchem_gb300 as rc

    O = oracle_mod
    Z, R = rc.geometry.water_cluster(2, 4.5, seed=11)
    ob = O.expand_basis(Z, R, rc.load_bse(name))
    D = _sym_density(np.random.default_rng(1), ob.n)
    Jr, Kr = O.JK_sym(ob, D)
    with rc.Basis(Z, R, name) as b:
        n = b.nbf
        J, K = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J, K, b, D, schwarz_tau=0.0)  # plans the work: the class table is known from here
        wc = [k for k, c in enumerate(b.class_stats()) if sum(c["class"]) >= 4]
        assert len(wc) == 13
        for k in wc:
            b.set_tile_shape(k, 0, shape)
            b.set_tile_shape(k, 1, shape)
        rc.JK_direct(J, K, b, D, schwarz_tau=0.0)
        assert np.abs(J - Jr).max() < 1e-12
        assert np.abs(K - Kr).max() < 1e-12
        rc.JK_direct(J, K, b, D, schwarz_tau=0.0, emulated=True)
        assert np.abs(J - Jr).max() < 1e-12
        assert np.abs(K - Kr).max() < 1e-12
        Jm, Km = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(Jm, Km, b, D, schwarz_tau=0.0, fp32_tau=1e30)  # every quartet in FP32
        assert np.abs(Jm - Jr).max() < 1e-5 and np.abs(Km - Kr).max() < 1e-5
        if shape <= 0:
            with pytest.raises(rc.RchemError):
                b.set_tile_shape(0, 0, shape)  # (ss|ss) has no warp-cooperative kernel
        with pytest.raises(rc.RchemError):
            b.set_tile_shape(wc[0], 0, -4)  # no 4-lane form


def test_exponent_table_on_and_off_vs_oracle(gpu, oracle_mod):
    """The (p, q) factors from the exponent table (default) and computed in
    every primitive quartet: FP64 and emulated J/K, one-lane-group and
    warp-cooperative kernels, both against the 8-fold oracle at 1e-12 and
    against each other at 1e-13; the FP64 gradient both ways to 1e-11."""
    import rchem_gb300 as rc

    O = oracle_mod
    name = "6-31gss-fit"
    Z, R = rc.geometry.water_cluster(2, 4.5, seed=11)
    ob = O.expand_basis(Z, R, rc.load_bse(name))
    D = _sym_density(np.random.default_rng(2), ob.n)
    W = _sym_density(np.random.default_rng(3), ob.n)
    Jr, Kr = O.JK_sym(ob, D)
    with rc.Basis(Z, R, name) as b:
        n = b.nbf
        out = {}
        for wc in (None, 0, -8):
            if wc is not None:
                for k, c in enumerate(b.class_stats()):
                    if sum(c["class"]) >= 4:
                        b.set_tile_shape(k, 0, wc)
            for emulated in (False, True):
                for on in (True, False):
                    b.set_exponent_table(on)
                    J, K = np.zeros((n, n)), np.zeros((n, n))
                    rc.JK_direct(J, K, b, D, schwarz_tau=0.0, emulated=emulated)
                    assert np.abs(J - Jr).max() < 1e-12 and np.abs(K - Kr).max() < 1e-12, (wc, emulated, on)
                    out[on] = (J, K)
                assert np.abs(out[True][0] - out[False][0]).max() < 1e-13
                assert np.abs(out[True][1] - out[False][1]).max() < 1e-13
        import torch

        res = {"D": torch.from_numpy(D).cuda(), "W": torch.from_numpy(W).cuda()}
        grads = []
        for on in (True, False):
            b.set_exponent_table(on)
            grads.append(rc.scf.gradient(b, res).cpu().numpy())
        assert np.abs(grads[0] - grads[1]).max() < 1e-11
        b.set_exponent_table(True)


@pytest.mark.parametrize("name", ["6-31gs-fit", "6-31gss-fit"])
def test_build_I_and_jk_inmem_d_shells_vs_oracle(gpu, oracle_mod, name):
    """The dense ERI tensor (ERI-store epilogue of all 21 classes, d on O and p
    on H) and the in-memory J/K against the oracle's build_I/JK_inmem
    (src/basis.rs:430-484)."""
    import rchem_gb300 as rc

    O = oracle_mod
    Z, R = rc.geometry.water_monomer()
    ob = O.expand_basis(Z, R, rc.load_bse(name))
    Ir = O.build_I(ob)
    D = _sym_density(np.random.default_rng(7), ob.n)
    with rc.Basis(Z, R, name) as b:
        I = rc.build_I(b)
        np.testing.assert_allclose(I, Ir, atol=1e-12, rtol=0)
        J, K = rc.JK_inmem(I, D)
        Jr, Kr = O.JK_inmem(Ir, D)
        np.testing.assert_allclose(J, Jr, atol=1e-12, rtol=0)
        np.testing.assert_allclose(K, Kr, atol=1e-12, rtol=0)


@pytest.mark.parametrize("order", [(0, 0, 0), (1, 0, 0), (0, 1, 1), (2, 0, 1), (1, 1, 1), (0, 0, 3)])
def test_moment_matrices_vs_oracle(gpu, oracle_mod, order):
    """Multipole-moment matrices (src/integrals/os86.rs:775-828) about an
    off-origin centre, d functions included."""
    import rchem_gb300 as rc

    O = oracle_mod
    Z, R = rc.geometry.water_monomer()
    center = [0.3, -0.2, 0.5]
    ob = O.expand_basis(Z, R, rc.load_bse("6-31gss-fit"))
    Mr = O.M(ob, center, list(order))
    with rc.Basis(Z, R, "6-31gss-fit") as b:
        M = rc.moment(b, center, order)
    scale = max(1.0, float(np.abs(Mr).max()))
    np.testing.assert_allclose(M, Mr, atol=1e-13 * scale, rtol=0)


@pytest.mark.parametrize("name", ["sto-3g-fit", "6-31gs-fit", "6-31gss-fit"])
def test_build_I_packed_and_jk_packed_vs_oracle(gpu, oracle_mod, name):
    """The ERI tensor in the 8-fold packed layout of ijkl2intindex
    (cints.c:375-387) against the oracle's dense build_I packed the same way,
    on host and device arrays, and J/K from it against JK_inmem."""
    torch = pytest.importorskip("torch")
    import rchem_gb300 as rc

    O = oracle_mod
    Z, R = rc.geometry.water_monomer()
    ob = O.expand_basis(Z, R, rc.load_bse(name))
    Ir = O.build_I(ob)
    Pr = O.pack_I(Ir)
    D = _sym_density(np.random.default_rng(8), ob.n)
    with rc.Basis(Z, R, name) as b:
        P = rc.build_I_packed(b)
        assert P.shape == Pr.shape
        np.testing.assert_allclose(P, Pr, atol=1e-12, rtol=0)
        Pd = rc.build_I_packed(b, device=True)
        np.testing.assert_allclose(Pd.cpu().numpy(), Pr, atol=1e-12, rtol=0)
        Jr, Kr = O.JK_inmem(Ir, D)
        J, K = rc.JK_packed(P, D)
        np.testing.assert_allclose(J, Jr, atol=1e-12, rtol=0)
        np.testing.assert_allclose(K, Kr, atol=1e-12, rtol=0)
        Jd, Kd = rc.JK_packed(Pd, torch.from_numpy(D).cuda())
        np.testing.assert_allclose(Jd.cpu().numpy(), Jr, atol=1e-12, rtol=0)
        np.testing.assert_allclose(Kd.cpu().numpy(), Kr, atol=1e-12, rtol=0)


def test_build_I_packed_matches_dense_h2o8(gpu, oracle_mod):
    """(H2O)8 in the 6-31G-shaped basis (n = 104, 14.9 M packed integrals):
    the packed tensor equals the dense one at sampled quadruples and in every
    permutation of them, and its J/K equal the dense tensor's."""
    torch = pytest.importorskip("torch")
    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config("h2o8_631g")
    with rc.Basis(Z, R, bname) as b:
        n = b.nbf
        P = rc.build_I_packed(b, device=True)
        I = rc.build_I(b, device=True)
        rng = np.random.default_rng(3)
        q = rng.integers(0, n, size=(200000, 4))
        for perm in ((0, 1, 2, 3), (1, 0, 3, 2), (2, 3, 1, 0)):
            pos = oracle_mod.ijkl2intindex(*(q[:, p] for p in perm))
            got = P[torch.from_numpy(pos).cuda()]
            ref = I[tuple(torch.from_numpy(q[:, k]).cuda() for k in range(4))]
            assert float((got - ref).abs().max()) < 1e-14  # equivalent components may round apart
        D = torch.from_numpy(_sym_density(np.random.default_rng(4), n)).cuda()
        J, K = rc.JK_packed(P, D)
        Jd, Kd = rc.JK_inmem(I, D)
        assert float((J - Jd).abs().max()) < 1e-11
        assert float((K - Kd).abs().max()) < 1e-11
