"""The CPU oracle, pinned before it is trusted.

1. Against the reference's own known-answer tests (the os86 / tho66 golden
   vectors, src/integrals/os86.rs:882-1016 and src/integrals/tho66.rs:266-321).
2. Against the reference library itself compiled from its sources
   (oracle/_ref), where those sources are present.
3. Against the committed fixtures generated from the reference
   (tests/golden/make_golden.py), which travel where the reference does not.
"""
import itertools
import math

import numpy as np
import pytest

from conftest import load_npz

# --- src/integrals/os86.rs:882-937 and tho66.rs:288-321 ----------------------
ERI_GEOM = dict(za=1.1, zb=1.2, zc=1.3, zd=1.4, ra=[1.0, 0.0, 1.0], rb=[0.0, 1.0, 2.0], rc=[0.0, 0.0, 3.0],
                rd=[0.0, 0.0, 4.0])
ERI_GOLDEN = [
    ([0] * 12, 0.08608517834596989),
    ([1] + [0] * 11, -0.046888060557776973),
    ([2, 1, 0, 1, 0, 0, 1, 0, 0, 0, 1, 0], 1.71817807954e-05),
]
# os86.rs:939-959 / tho66.rs:266-286 (za=1.8, zb=2.8)
OVL_GOLDEN = [
    ([0, 0, 0, 0, 0, 0], 0.20373275913014607),
    ([1, 0, 0, 0, 0, 0], 0.062005622343957505),
    ([1, 1, 0, 1, 1, 0], -0.00043801221837779696),
    ([2, 1, 0, 1, 1, 0], -0.0002385994651113168),
]
# os86.rs:961-978 (za=1.8, zb=2.0)
KIN_GOLDEN = [
    ([0, 0, 0, 0, 0, 0], 0.3652714583525358),
    ([1, 0, 0, 0, 0, 0], 0.2514265587836556),
    ([2, 2, 2, 2, 2, 2], -7.40057384314e-05),
]
# os86.rs:980-1002 (za=1.8, zb=2.0, rc=(0.5,0.8,0.2))
NUC_GOLDEN = [
    ([0, 0, 0, 0, 0, 0], -0.49742209545104593),
    ([1, 0, 0, 0, 0, 0], -0.15987439458254471),
    ([2, 2, 2, 0, 0, 0], -0.003801373531942607),
    ([1, 1, 1, 1, 1, 1], 8.8415484347060993e-5),
]
RA, RB, RC = [0.0, 0.0, 0.0], [0.5, 0.8, -0.2], [0.5, 0.8, 0.2]


def test_eri_golden(port):
    g = ERI_GEOM
    for pw, ref in ERI_GOLDEN:
        v = port.coulomb_os(g["za"], g["zb"], g["zc"], g["zd"], g["ra"], g["rb"], g["rc"], g["rd"], pw)
        assert abs(v - ref) < 1e-15, (pw, v, ref)


def test_eri_shipped_boys_within_reference_tolerance(port):
    """tho66.rs:288-321 checks the shipped (NR Boys) ssss at 1e-12."""
    g = ERI_GEOM
    port.set_boys(False)
    try:
        v = port.coulomb_os(g["za"], g["zb"], g["zc"], g["zd"], g["ra"], g["rb"], g["rc"], g["rd"], [0] * 12)
    finally:
        port.set_boys(True)
    assert abs(v - ERI_GOLDEN[0][1]) < 1e-12
    assert abs(v - ERI_GOLDEN[0][1]) > 1e-14  # the NR Boys error is visible


def test_onee_golden(port):
    for pw, ref in OVL_GOLDEN:
        assert abs(port.overlap(1.8, 2.8, RA, RB, pw) - ref) < 1e-16
    # the golden T values come from os86's Obara-Saika route, the port follows
    # cints.c's overlap-combination route: they agree to an ulp or two
    for pw, ref in KIN_GOLDEN:
        assert abs(port.kinetic(1.8, 2.0, RA, RB, pw) - ref) < 1e-15
    for pw, ref in NUC_GOLDEN:
        assert abs(port.nuclear(1.8, 2.0, RA, RB, RC, pw) - ref) < 1e-15


def test_moment_golden(port):
    """os86.rs:1004-1016."""
    v = port.moment(1.8, 2.0, RA, RB, [0, 0, 0], [0, 0, 2, 0, 0, 0], [0, 0, 1])
    assert abs(v - -0.01330515491323708) < 1e-16


def test_boys_exact_vs_series_identities(port):
    # F_m(0) = 1/(2m+1); downward recursion identity; large-x asymptote
    for m in range(0, 17):
        assert abs(port.boys_exact(m, 0.0) - 1.0 / (2 * m + 1)) < 1e-16
    for x in (0.3, 2.0, 11.0, 34.9, 35.1, 60.0):
        for m in range(0, 12):
            lhs = port.boys_exact(m, x)
            rhs = (2 * x * port.boys_exact(m + 1, x) + math.exp(-x)) / (2 * m + 1)
            assert abs(lhs - rhs) <= 3e-15 * abs(lhs)
    assert abs(port.boys_exact(0, 80.0) - 0.5 * math.sqrt(math.pi / 80.0)) < 1e-17


def test_boys_exact_vs_mpmath(port):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    for m in range(0, 10):
        for x in (1e-9, 0.01, 0.5, 1.0, 2.5, 5.0, 10.0, 20.0, 33.0, 50.0):
            ref = float(mp.quad(lambda t: t ** (2 * m) * mp.exp(-x * t * t), [0, 1]))
            assert abs(port.boys_exact(m, x) - ref) <= 2e-15 * ref


def test_boys_shipped_is_nr_accuracy(port):
    worst = 0.0
    for m in range(0, 9):
        for x in (1e-9, 0.01, 0.5, 1.0, 2.5, 5.0, 10.0, 20.0, 33.0, 50.0):
            ex = port.boys_exact(m, x)
            worst = max(worst, abs(port.boys_nr(m, x) - ex) / ex)
    assert 1e-9 < worst < 2e-7


def test_port_vs_golden_fixture_eri(port, golden_eri):
    for it in golden_eri:
        R, a, pw = it["R"], it["alpha"], it["powers"]
        args = []
        for k in range(4):
            args += [R[k], 1.0, pw[k], a[k]]
        v = port.coulomb_repulsion(*args)
        assert abs(v - it["exact"]) <= 1e-14 * max(1.0, abs(it["exact"])), it
        port.set_boys(False)
        try:
            v = port.coulomb_repulsion(*args)
        finally:
            port.set_boys(True)
        assert abs(v - it["shipped"]) <= 1e-14 * max(1.0, abs(it["shipped"])), it


def test_port_vs_golden_fixture_onee(port, golden_onee):
    for it in golden_onee:
        a = it["alpha"]
        pw = it["pa"] + it["pb"]
        assert abs(port.overlap(a[0], a[1], it["A"], it["B"], pw) - it["S_exact"]) < 1e-14
        assert abs(port.kinetic(a[0], a[1], it["A"], it["B"], pw) - it["T_exact"]) < 1e-13
        assert abs(port.nuclear(a[0], a[1], it["A"], it["B"], it["C"], pw) - it["V_exact"]) < 1e-14


@pytest.mark.parametrize("tag,name", [("h2o_sto3g", "sto-3g-fit"), ("h2o_631g", "6-31g-fit"),
                                      ("h2o_631gs", "6-31gs-fit")])
def test_port_matrices_vs_fixture(oracle_mod, tag, name):
    from rchem_gb300 import bse, geometry

    O = oracle_mod
    g = load_npz(tag)
    Z, R = geometry.water_monomer()
    b = O.expand_basis(Z, R, bse.load_bse(name))
    np.testing.assert_allclose(O.S(b), g["S"], atol=1e-14, rtol=0)
    np.testing.assert_allclose(O.T(b), g["T"], atol=1e-13, rtol=0)
    np.testing.assert_allclose(O.V(b, R, Z), g["V"], atol=1e-13, rtol=0)
    J, K = O.JK_sym(b, g["D"])
    np.testing.assert_allclose(J, g["J"], atol=1e-13, rtol=0)
    np.testing.assert_allclose(K, g["K"], atol=1e-13, rtol=0)
    if "I" in g:
        np.testing.assert_allclose(O.build_I(b), g["I"], atol=1e-14, rtol=0)
        Ji, Ki = O.JK_inmem(g["I"], g["D"])
        np.testing.assert_allclose(Ji, g["J"], atol=1e-13, rtol=0)
        np.testing.assert_allclose(Ki, g["K"], atol=1e-13, rtol=0)


def test_port_jk_direct_vs_sym(oracle_mod):
    """The 8-fold oracle equals the literal JK_direct loops (basis.rs:383-428)."""
    from rchem_gb300 import bse, geometry

    O = oracle_mod
    Z, R = geometry.water_monomer()
    b = O.expand_basis(Z, R, bse.load_bse("sto-3g-fit"))
    rng = np.random.default_rng(3)
    D = rng.normal(size=(b.n, b.n))
    D = D + D.T
    J1, K1 = O.JK_direct(b, D)
    J2, K2 = O.JK_sym(b, D)
    np.testing.assert_allclose(J1, J2, atol=1e-13)
    np.testing.assert_allclose(K1, K2, atol=1e-13)
    Je, Ke = O.JK_elements(b, D, [0, 3, 6], [1, 3, 2])
    np.testing.assert_allclose(Je, J1[[0, 3, 6], [1, 3, 2]], atol=1e-13)
    np.testing.assert_allclose(Ke, K1[[0, 3, 6], [1, 3, 2]], atol=1e-13)


def test_screened_jk_vs_unscreened(oracle_mod):
    """The strong CPU baseline's J/K (8-fold symmetry, Schwarz screen over
    contracted functions): with the screen off it equals the 8-fold oracle;
    at tau = 1e-12 it stays within the dropped integrals' bound; the
    count-only pass counts what the full pass evaluates; the bra pairs split
    into two subsets (one on one thread) add up to the whole build."""
    from rchem_gb300 import bse, geometry

    O = oracle_mod
    Z, R = geometry.water_cluster(2, 4.5, seed=3)
    b = O.expand_basis(Z, R, bse.load_bse("6-31g-fit"))
    rng = np.random.default_rng(1)
    X = rng.normal(size=(b.n, b.n))
    D = X @ X.T / b.n
    npair = b.n * (b.n + 1) // 2
    J0, K0 = O.JK_sym(b, D)
    Q = O.schwarz(b)
    assert Q.shape == (npair,) and np.all(Q >= 0.0)
    # Q_ii,ii is the square root of a diagonal integral
    assert abs(Q[2] ** 2 - O.port().lib.oq_contracted_eri(*b.args(), None, 1, 1, 1, 1)) < 1e-14
    J1, K1, c1 = O.JK_sym_screened(b, D, Q, 0.0)
    assert c1 == npair * (npair + 1) // 2
    np.testing.assert_allclose(J1, J0, atol=1e-13, rtol=0)
    np.testing.assert_allclose(K1, K0, atol=1e-13, rtol=0)
    J2, K2, c2 = O.JK_sym_screened(b, D, Q, 1e-12)
    assert 0 < c2 < c1
    bound = 6 * (c1 - c2) * 1e-12 * np.abs(D).max()  # each dropped |(ij|kl)| < tau feeds at most 6 elements
    assert np.abs(J2 - J0).max() <= bound and np.abs(K2 - K0).max() <= bound
    assert O.JK_sym_screened(b, D, Q, 1e-12, count_only=True)[2] == c2
    pairs = np.arange(npair)
    a, rest = pairs[::3], np.setdiff1d(pairs, pairs[::3])
    Ja, Ka, ca = O.JK_sym_screened(b, D, Q, 1e-12, pairs=a, nthreads=1)
    Jb, Kb, cb = O.JK_sym_screened(b, D, Q, 1e-12, pairs=rest)
    assert ca + cb == c2
    np.testing.assert_allclose(Ja + Jb, J2, atol=1e-13, rtol=0)
    np.testing.assert_allclose(Ka + Kb, K2, atol=1e-13, rtol=0)


def test_scf_energy_fixture(oracle_mod):
    from rchem_gb300 import bse, geometry

    O = oracle_mod
    g = load_npz("h2o_sto3g")
    Z, R = geometry.water_monomer()
    b = O.expand_basis(Z, R, bse.load_bse("sto-3g-fit"))
    res = O.rhf(b, Z, R, 5, thresh_e=1e-12)
    assert abs(res["e_elec"] - float(g["e_elec"])) < 1e-10
    assert abs(res["e_nuc"] - float(g["e_nuc"])) < 1e-12


# --- straight against the reference library, where it was compiled here -------
def test_port_vs_reference_library_random(port):
    import oracle

    ex, sh = oracle.ref("exact"), oracle.ref("shipped")
    if ex is None:
        pytest.skip("reference sources not present: oracle/_ref not built")
    rng = np.random.default_rng(7)
    for cls in itertools.product(range(3), repeat=4):
        R = rng.uniform(-1.5, 1.5, (4, 3))
        a = rng.uniform(0.2, 3.0, 4)
        pw = [oracle.ijk_list(l)[rng.integers(len(oracle.ijk_list(l)))] for l in cls]
        args = []
        for k in range(4):
            args += [R[k], 0.7, pw[k], a[k]]
        assert abs(port.coulomb_repulsion(*args) - ex.coulomb_repulsion(*args)) < 1e-15
        port.set_boys(False)
        try:
            assert abs(port.coulomb_repulsion(*args) - sh.coulomb_repulsion(*args)) < 1e-15
        finally:
            port.set_boys(True)


def test_packed_index_vs_reference_library(oracle_mod):
    """The oracle's packed 8-fold index (cints.c:375-387) against the compiled
    reference's ijkl2intindex where it was built here, and the library's own
    export (a host function, no GPU call); every permutation of a quadruple
    lands on one position and distinct unique quadruples on distinct ones."""
    import ctypes as C

    from rchem_gb300 import _lib, build

    O = oracle_mod
    n = 9
    idx = np.array(list(itertools.product(range(n), repeat=4)))
    pos = O.ijkl2intindex(idx[:, 0], idx[:, 1], idx[:, 2], idx[:, 3])
    for perm in ((1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1), (3, 2, 1, 0)):
        p2 = O.ijkl2intindex(*(idx[:, q] for q in perm))
        assert (p2 == pos).all()
    npair = n * (n + 1) // 2
    assert sorted(set(pos.tolist())) == list(range(npair * (npair + 1) // 2))
    build.build()
    L = _lib.lib()
    sample = idx[::7]
    ours = [L.ijkl2intindex(*map(int, q)) for q in sample]
    assert ours == O.ijkl2intindex(sample[:, 0], sample[:, 1], sample[:, 2], sample[:, 3]).tolist()
    ref = O.ref("shipped")
    if ref is not None:
        f = ref.lib.ijkl2intindex
        f.argtypes, f.restype = [C.c_int] * 4, C.c_int
        assert [f(*map(int, q)) for q in sample] == ours
