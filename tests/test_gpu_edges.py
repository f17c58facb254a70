"""Edge cases of the Fock build and the one-electron matrices, on the GPU,
against the oracle: the smallest systems (one atom, H2), a system whose
fragments are too far apart to interact, everything screened out, a zero
density, and empty batches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _density(n, seed):
    X = np.random.default_rng(seed).normal(size=(n, n)) * 0.2
    return X @ X.T / n


@pytest.mark.parametrize("Z,R,name", [
    ([8], [[0.0, 0.0, 0.0]], "6-31gs-fit"),                       # one atom, d shells on it
    ([1, 1], [[0.0, 0.0, 0.0], [0.0, 0.0, 1.4]], "sto-3g-fit"),    # H2: s shells only
    ([1, 1], [[0.0, 0.0, 0.0], [0.0, 0.0, 1.4]], "6-31gss-fit"),   # H2 with p on H
])
def test_smallest_systems_vs_oracle(gpu, oracle_mod, Z, R, name):
    import rchem_gb300 as rc

    O = oracle_mod
    ob = O.expand_basis(Z, R, rc.load_bse(name))
    D = _density(ob.n, 7)
    Jr, Kr = O.JK_sym(ob, D)
    with rc.Basis(Z, R, name) as b:
        n = b.nbf
        assert n == ob.n
        J, K = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J, K, b, D, schwarz_tau=0.0)
        assert np.abs(J - Jr).max() < 1e-12 and np.abs(K - Kr).max() < 1e-12
        rc.JK_direct(J, K, b, D, emulated=True)
        assert np.abs(J - Jr).max() < 1e-11 and np.abs(K - Kr).max() < 1e-11
        np.testing.assert_allclose(rc.S(b), O.S(ob), atol=1e-12, rtol=0)
        np.testing.assert_allclose(rc.V(b), O.V(ob, R, Z), atol=1e-11, rtol=0)


def test_far_apart_fragments(gpu, oracle_mod):
    """Two waters 500 bohr apart: no shell pair spans them (the Gaussian
    product factor is below the primitive cut), so every cross quartet is a
    pair on each water at long range; J and K equal the oracle's."""
    import rchem_gb300 as rc

    O = oracle_mod
    Z1, R1 = rc.geometry.water_monomer()
    R1 = np.asarray(R1, dtype=float).reshape(-1, 3)
    Z = list(Z1) + list(Z1)
    R = np.vstack([R1, R1 + np.array([500.0, 0.0, 0.0])])
    ob = O.expand_basis(Z, R, rc.load_bse("6-31g-fit"))
    D = _density(ob.n, 3)
    Jr, Kr = O.JK_sym(ob, D)
    with rc.Basis(Z, R, "6-31g-fit") as b:
        n = b.nbf
        J, K = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J, K, b, D)
        assert np.abs(J - Jr).max() < 1e-11 and np.abs(K - Kr).max() < 1e-11


def test_everything_screened_and_zero_density(gpu):
    """A screening threshold above every Schwarz product leaves no quartet (J
    and K are zero, no error); a zero density gives exact zeros; the next
    ordinary build is unaffected."""
    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config("h2o8_631g")
    D = _density(104, 5)
    with rc.Basis(Z, R, bname) as b:
        J0, K0 = np.zeros((104, 104)), np.zeros((104, 104))
        rc.JK_direct(J0, K0, b, D)
        J, K = np.full((104, 104), 7.0), np.full((104, 104), 7.0)
        rc.JK_direct(J, K, b, D, schwarz_tau=1e30)
        assert b.stats()["quartets_fp64"] == 0
        assert not J.any() and not K.any()
        rc.JK_direct(J, K, b, np.zeros((104, 104)))
        assert not J.any() and not K.any()
        rc.JK_direct(J, K, b, D)  # (FP64 atomics: the same sums in another order)
        assert np.abs(J - J0).max() < 1e-12 and np.abs(K - K0).max() < 1e-12


def test_empty_batches(gpu):
    """Zero-length batches of the bulk entry points return at once."""
    from rchem_gb300 import cints

    assert cints.boys_batch([], [], 64).size == 0
    assert cints.boys_batch([], [], 65).size == 0
    assert cints.eri_batch([]).size == 0
