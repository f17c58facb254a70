"""CPU ORACLE -- test infrastructure only.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module, and only to compare results against or as
the timed CPU reference path; the product (``rchem_gb300``) never does.

It wraps, through ctypes:

* ``libpq2_port.so`` -- the plain-C restatement in ``pq2_port.c`` of the
  reference's THO integrals (``libpyquante2/cints.c``) and matrix builders
  (``src/basis.rs:214-484``); built on any host by ``make -C oracle port``;
* ``_ref/libpyquante2_{shipped,exact}.so`` -- the reference's own C sources
  compiled unmodified by ``make -C oracle ref`` (only where the reference
  sources are present), the second with an exact Boys function bound in.

It also restates, in numpy, the reference's basis expansion
(``Basis::new``, ``src/basis.rs:181-211``, with the shell coefficients taken
by position so pure p/d shells work) and its SCF driver
(``src/bin/rchem.rs:40-127``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libpq2_port.so")
REF_DIR = os.path.join(HERE, "_ref")

_d, _i, _p = C.c_double, C.c_int, C.c_void_p
_ERI_ARGS = [_d, _d, _d, _d, _i, _i, _i, _d] * 4
_OVL_ARGS = [_d, _i, _i, _i, _d, _d, _d] * 2
_NUC_ARGS = [_d, _d, _d, _d, _i, _i, _i, _d] * 2 + [_d, _d, _d]


def build_port() -> str:
    if not os.path.exists(PORT_SO) or os.path.getmtime(PORT_SO) < os.path.getmtime(
        os.path.join(HERE, "pq2_port.c")
    ):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def _bind_cints(lib, prefix: str):
    """Bind the cints.h-signature scalar functions found under ``prefix``."""
    f = getattr(lib, prefix + "coulomb_repulsion")
    f.argtypes, f.restype = _ERI_ARGS, _d
    f = getattr(lib, prefix + "overlap")
    f.argtypes, f.restype = _OVL_ARGS, _d
    f = getattr(lib, prefix + "kinetic")
    f.argtypes, f.restype = _OVL_ARGS, _d
    f = getattr(lib, prefix + "nuclear_attraction")
    f.argtypes, f.restype = _NUC_ARGS, _d
    f = getattr(lib, "Fgamma" if prefix == "" else prefix + "fgamma")
    f.argtypes, f.restype = [_d, _d], _d


class Lib:
    """A loaded integral library with cints.h-style scalar entry points."""

    def __init__(self, path: str, prefix: str):
        self.path = path
        self.lib = C.CDLL(path)
        self.prefix = prefix
        _bind_cints(self.lib, prefix)

    def fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def addr(self, name) -> int:
        return C.cast(self.fn(name), C.c_void_p).value

    # cints.h:24-30 argument order
    def coulomb_repulsion(self, ra, na, pa, za, rb, nb, pb, zb, rc, nc, pc, zc, rd, nd, pd, zd) -> float:
        return self.fn("coulomb_repulsion")(*ra, na, *pa, za, *rb, nb, *pb, zb, *rc, nc, *pc, zc, *rd, nd, *pd, zd)

    # tho66.rs:237-259 argument order (exponents, centres, norms, 12 powers)
    def coulomb_os(self, za, zb, zc, zd, ra, rb, rc, rd, powers, norms=(1.0, 1.0, 1.0, 1.0)) -> float:
        p = list(powers)
        return self.coulomb_repulsion(ra, norms[0], p[0:3], za, rb, norms[1], p[3:6], zb,
                                      rc, norms[2], p[6:9], zc, rd, norms[3], p[9:12], zd)

    def overlap(self, za, zb, ra, rb, powers) -> float:
        p = list(powers)
        return self.fn("overlap")(za, *p[0:3], *ra, zb, *p[3:6], *rb)

    def kinetic(self, za, zb, ra, rb, powers) -> float:
        p = list(powers)
        return self.fn("kinetic")(za, *p[0:3], *ra, zb, *p[3:6], *rb)

    def nuclear(self, za, zb, ra, rb, rc, powers) -> float:
        """os86 get_nuclear semantics: unit norms, attraction to a unit charge at rc."""
        p = list(powers)
        return self.fn("nuclear_attraction")(*ra, 1.0, *p[0:3], za, *rb, 1.0, *p[3:6], zb, *rc)

    def fgamma(self, m, x) -> float:
        name = "Fgamma" if self.prefix == "" else self.prefix + "fgamma"
        return getattr(self.lib, name)(float(m), float(x))


_port = None


def port() -> "PortLib":
    global _port
    if _port is None:
        _port = PortLib(build_port())
    return _port


def ref(kind: str = "exact") -> Lib | None:
    """The reference's own C library, compiled here; None where it was not built."""
    path = os.path.join(REF_DIR, f"libpyquante2_{kind}.so")
    if not os.path.exists(path):
        return None
    return Lib(path, "")


class PortLib(Lib):
    def __init__(self, path):
        super().__init__(path, "oq_")
        L = self.lib
        L.oq_set_boys_mode.argtypes, L.oq_set_boys_mode.restype = [_i], None
        L.oq_boys_exact.argtypes, L.oq_boys_exact.restype = [_i, _d], _d
        L.oq_fgamma_nr.argtypes, L.oq_fgamma_nr.restype = [_d, _d], _d
        L.oq_pgto_norm.argtypes, L.oq_pgto_norm.restype = [_d, _i, _i, _i], _d
        L.oq_moment.argtypes = _OVL_ARGS + [_d, _d, _d, _i, _i, _i]
        L.oq_moment.restype = _d
        L.oq_num_threads.restype = _i
        bargs = [_i, _p, _p, _p, _p, _p, _p, _p]
        L.oq_contracted_eri.argtypes, L.oq_contracted_eri.restype = bargs + [_p, _i, _i, _i, _i], _d
        L.oq_S.argtypes = bargs + [_p, _p]
        L.oq_T.argtypes = bargs + [_p, _p]
        L.oq_V.argtypes = bargs + [_p, _i, _p, _p, _p]
        L.oq_M.argtypes = bargs + [_p, _i, _i, _i, _p]
        L.oq_jk_direct.argtypes = bargs + [_p, _p, _p, _p, _i, _i]
        L.oq_build_I.argtypes = bargs + [_p, _p]
        L.oq_jk_inmem.argtypes = [_i, _p, _p, _p, _p]
        L.oq_jk_sym.argtypes = bargs + [_p, _p, _p, _p]
        L.oq_jk_elements.argtypes = bargs + [_p, _p, _i, _p, _p, _p, _p]
        L.oq_jk_direct_elements.argtypes = bargs + [_p, _p, _i, _p, _p, _p, _p]
        L.oq_schwarz.argtypes = bargs + [_p, _p]
        L.oq_jk_sym_screened.argtypes = bargs + [_p, _p, _p, _d, _p, C.c_long, _i, _i, _p, _p]
        L.oq_jk_sym_screened.restype = C.c_longlong
        L.oq_jk_direct_quartets.argtypes = bargs + [_p, _p, _i, _p, _p, _p, _p, _p, _p]
        L.oq_jk_elements_screened.argtypes = bargs + [_p, _p, _p, _d, _i, _p, _p, _p, _p]
        L.oq_eri_packed.argtypes = bargs + [_p, _p, _d, _p]
        L.oq_jk_packed.argtypes = [_i, _p, _p, _p, _p]

    def set_boys(self, exact: bool):
        self.lib.oq_set_boys_mode(1 if exact else 0)

    def boys_exact(self, m, x):
        return self.lib.oq_boys_exact(int(m), float(x))

    def boys_nr(self, m, x):
        return self.lib.oq_fgamma_nr(float(m), float(x))

    def pgto_norm(self, a, l, m, n):
        return self.lib.oq_pgto_norm(a, l, m, n)

    def moment(self, za, zb, ra, rb, rc, powers, order):
        p = list(powers)
        return self.lib.oq_moment(za, *p[0:3], *ra, zb, *p[3:6], *rb, *rc, *order)

    def num_threads(self):
        return self.lib.oq_num_threads()


# ---------------------------------------------------------------------------
# basis expansion (basis.rs:181-211 restated) -- independent of the product
# ---------------------------------------------------------------------------
def ijk_list(l: int):
    """shell.rs:1-12 Cartesian order."""
    out = []
    for a in range(1, l + 2):
        for b in range(1, a + 1):
            out.append((l + 1 - a, a - b, b - 1))
    return out


@dataclass
class CGTOBasis:
    """Flat arrays of contracted Cartesian functions in AO order."""

    origin: np.ndarray  # (n,3) f64
    powers: np.ndarray  # (n,3) i32
    nprim: np.ndarray  # (n,) i32
    prim_off: np.ndarray  # (n,) i32
    exps: np.ndarray  # (P,) f64
    coefs: np.ndarray  # (P,) f64 raw contraction coefficients
    norms: np.ndarray  # (P,) f64 per-primitive norms (basis.rs:140-149)
    atom: np.ndarray = field(default=None)  # (n,) owning atom

    @property
    def n(self) -> int:
        return int(self.origin.shape[0])

    def args(self):
        return [self.n] + [a.ctypes.data for a in (self.origin, self.powers, self.nprim, self.prim_off,
                                                    self.exps, self.coefs, self.norms)]


def expand_basis(atomnos, coords, bse: dict) -> CGTOBasis:
    """Basis::new (basis.rs:181-211): atoms in order, shells in file order, each
    angular momentum of a shell in order, Cartesian components in shell.rs order;
    coefficients of the k-th angular momentum of a shell are coefficients[k]."""
    lib = port()
    origin, powers, nprim, off, exps, coefs, norms, atom = [], [], [], [], [], [], [], []
    for ia, (z, r) in enumerate(zip(atomnos, coords)):
        el = bse["elements"][str(int(z))]
        for sh in el["electron_shells"]:
            ex = [float(x) for x in sh["exponents"]]
            for k, l in enumerate(sh["angular_momentum"]):
                cf = [float(x) for x in sh["coefficients"][k]]
                assert len(cf) == len(ex)
                for pw in ijk_list(int(l)):
                    origin.append([float(c) for c in r])
                    powers.append(pw)
                    nprim.append(len(ex))
                    off.append(len(exps))
                    for e, c in zip(ex, cf):
                        exps.append(e)
                        coefs.append(c)
                        norms.append(lib.pgto_norm(e, *pw))
                    atom.append(ia)
    return CGTOBasis(
        origin=np.ascontiguousarray(origin, dtype=np.float64).reshape(-1, 3),
        powers=np.ascontiguousarray(powers, dtype=np.int32).reshape(-1, 3),
        nprim=np.ascontiguousarray(nprim, dtype=np.int32),
        prim_off=np.ascontiguousarray(off, dtype=np.int32),
        exps=np.ascontiguousarray(exps, dtype=np.float64),
        coefs=np.ascontiguousarray(coefs, dtype=np.float64),
        norms=np.ascontiguousarray(norms, dtype=np.float64),
        atom=np.ascontiguousarray(atom, dtype=np.int32),
    )


def _eri_ptr(lib: Lib | None):
    if lib is None or isinstance(lib, PortLib):
        return None
    return lib.addr("coulomb_repulsion")


def S(b: CGTOBasis, lib: Lib | None = None) -> np.ndarray:
    out = np.zeros((b.n, b.n))
    ptr = None if lib is None or isinstance(lib, PortLib) else lib.addr("overlap")
    port().lib.oq_S(*b.args(), ptr, out.ctypes.data)
    return out


def T(b: CGTOBasis, lib: Lib | None = None) -> np.ndarray:
    out = np.zeros((b.n, b.n))
    ptr = None if lib is None or isinstance(lib, PortLib) else lib.addr("kinetic")
    port().lib.oq_T(*b.args(), ptr, out.ctypes.data)
    return out


def V(b: CGTOBasis, coords, atomnos, lib: Lib | None = None) -> np.ndarray:
    out = np.zeros((b.n, b.n))
    Z = np.ascontiguousarray(atomnos, dtype=np.float64)
    R = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
    ptr = None if lib is None or isinstance(lib, PortLib) else lib.addr("nuclear_attraction")
    port().lib.oq_V(*b.args(), ptr, len(Z), Z.ctypes.data, R.ctypes.data, out.ctypes.data)
    return out


def M(b: CGTOBasis, center, order) -> np.ndarray:
    out = np.zeros((b.n, b.n))
    Cc = np.ascontiguousarray(center, dtype=np.float64)
    port().lib.oq_M(*b.args(), Cc.ctypes.data, int(order[0]), int(order[1]), int(order[2]), out.ctypes.data)
    return out


def JK_direct(b: CGTOBasis, D: np.ndarray, lib: Lib | None = None, rows=None):
    """basis.rs:383-428 semantics; ``rows=(m0,m1)`` evaluates only those rows."""
    n = b.n
    D = np.ascontiguousarray(D, dtype=np.float64)
    J = np.zeros((n, n))
    K = np.zeros((n, n))
    m0, m1 = rows if rows is not None else (0, n)
    port().lib.oq_jk_direct(*b.args(), _eri_ptr(lib), D.ctypes.data, J.ctypes.data, K.ctypes.data, m0, m1)
    return J, K


def JK_sym(b: CGTOBasis, D: np.ndarray, lib: Lib | None = None):
    n = b.n
    D = np.ascontiguousarray(D, dtype=np.float64)
    J = np.zeros((n, n))
    K = np.zeros((n, n))
    port().lib.oq_jk_sym(*b.args(), _eri_ptr(lib), D.ctypes.data, J.ctypes.data, K.ctypes.data)
    return J, K


def schwarz(b: CGTOBasis, lib: Lib | None = None) -> np.ndarray:
    """Q[ij] = sqrt(|(ij|ij)|) over contracted function pairs, ij = i(i+1)/2 + j."""
    Q = np.zeros(b.n * (b.n + 1) // 2)
    port().lib.oq_schwarz(*b.args(), _eri_ptr(lib), Q.ctypes.data)
    return Q


def JK_sym_screened(b: CGTOBasis, D: np.ndarray, Q: np.ndarray, tau: float, pairs=None, nthreads: int = 0,
                    count_only: bool = False, lib: Lib | None = None):
    """J and K with each unique contracted integral once and quartets with
    Q_ij Q_kl < tau skipped, over the bra pairs ``pairs`` (None: all, the whole
    build).  Returns (J, K, integrals evaluated); J and K are None when
    ``count_only``."""
    n = b.n
    D = np.ascontiguousarray(D, dtype=np.float64)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    assert D.shape == (n, n) and Q.shape == (n * (n + 1) // 2,)
    ijs = None if pairs is None else np.ascontiguousarray(pairs, dtype=np.int64)
    if ijs is not None:
        assert ijs.size == 0 or (ijs.min() >= 0 and ijs.max() < Q.size)
    J = np.zeros((n, n))
    K = np.zeros((n, n))
    cnt = port().lib.oq_jk_sym_screened(*b.args(), _eri_ptr(lib), D.ctypes.data, Q.ctypes.data, float(tau),
                                        None if ijs is None else ijs.ctypes.data, 0 if ijs is None else ijs.size,
                                        int(nthreads), 1 if count_only else 0, J.ctypes.data, K.ctypes.data)
    return (None, None, int(cnt)) if count_only else (J, K, int(cnt))


def JK_elements(b: CGTOBasis, D: np.ndarray, mus, nus, lib: Lib | None = None):
    D = np.ascontiguousarray(D, dtype=np.float64)
    mu = np.ascontiguousarray(mus, dtype=np.int32)
    nu = np.ascontiguousarray(nus, dtype=np.int32)
    Jo = np.zeros(len(mu))
    Ko = np.zeros(len(mu))
    port().lib.oq_jk_elements(*b.args(), _eri_ptr(lib), D.ctypes.data, len(mu), mu.ctypes.data, nu.ctypes.data,
                              Jo.ctypes.data, Ko.ctypes.data)
    return Jo, Ko


def JK_direct_elements(b: CGTOBasis, D: np.ndarray, mus, nus, lib: Lib | None = None):
    """Elements of J and K by the literal JK_direct loops (basis.rs:392-425)."""
    D = np.ascontiguousarray(D, dtype=np.float64)
    mu = np.ascontiguousarray(mus, dtype=np.int32)
    nu = np.ascontiguousarray(nus, dtype=np.int32)
    Jo = np.zeros(len(mu))
    Ko = np.zeros(len(mu))
    port().lib.oq_jk_direct_elements(*b.args(), _eri_ptr(lib), D.ctypes.data, len(mu), mu.ctypes.data,
                                     nu.ctypes.data, Jo.ctypes.data, Ko.ctypes.data)
    return Jo, Ko


def JK_direct_quartets(b: CGTOBasis, D: np.ndarray, mus, nus, las, sgs, lib: Lib | None = None):
    """The innermost block of the literal JK_direct loops (basis.rs:400-421)
    for sampled quadruples (mu, nu, lambda, sigma): their J and K
    contributions.  A whole build is the sum over all n^4 quadruples."""
    D = np.ascontiguousarray(D, dtype=np.float64)
    idx = [np.ascontiguousarray(x, dtype=np.int32) for x in (mus, nus, las, sgs)]
    m = len(idx[0])
    assert all(len(x) == m for x in idx) and all(x.size == 0 or (x.min() >= 0 and x.max() < b.n) for x in idx)
    Jo, Ko = np.zeros(m), np.zeros(m)
    port().lib.oq_jk_direct_quartets(*b.args(), _eri_ptr(lib), D.ctypes.data, m, *(x.ctypes.data for x in idx),
                                     Jo.ctypes.data, Ko.ctypes.data)
    return Jo, Ko


def JK_elements_screened(b: CGTOBasis, D: np.ndarray, Q: np.ndarray, tau: float, mus, nus,
                         lib: Lib | None = None):
    """Elements J_mn, K_mn from their definitions (basis.rs:406-417) with
    contracted integrals, skipping (ab|cd) when Q_ab Q_cd < tau (Q from
    ``schwarz``); OpenMP over the elements."""
    D = np.ascontiguousarray(D, dtype=np.float64)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    mu = np.ascontiguousarray(mus, dtype=np.int32)
    nu = np.ascontiguousarray(nus, dtype=np.int32)
    assert Q.shape == (b.n * (b.n + 1) // 2,) and D.shape == (b.n, b.n)
    assert mu.size == nu.size and (mu.size == 0 or (min(mu.min(), nu.min()) >= 0 and max(mu.max(), nu.max()) < b.n))
    Jo, Ko = np.zeros(len(mu)), np.zeros(len(mu))
    port().lib.oq_jk_elements_screened(*b.args(), _eri_ptr(lib), D.ctypes.data, Q.ctypes.data, float(tau), len(mu),
                                       mu.ctypes.data, nu.ctypes.data, Jo.ctypes.data, Ko.ctypes.data)
    return Jo, Ko


def eri_packed(b: CGTOBasis, Q: np.ndarray | None = None, tau: float = 0.0, lib: Lib | None = None) -> np.ndarray:
    """The ERI tensor in the packed 8-fold layout of ijkl2intindex; integrals
    with Q_ij Q_kl < tau stored as zero."""
    npair = b.n * (b.n + 1) // 2
    if Q is None:
        Q, tau = np.zeros(npair), 0.0
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    assert Q.shape == (npair,)
    out = np.empty(npair * (npair + 1) // 2)
    port().lib.oq_eri_packed(*b.args(), _eri_ptr(lib), Q.ctypes.data, float(tau), out.ctypes.data)
    return out


def JK_packed(n: int, I: np.ndarray, D: np.ndarray):
    """J and K (JK_inmem's definitions) from a packed tensor of ``eri_packed``."""
    npair = n * (n + 1) // 2
    I = np.ascontiguousarray(I, dtype=np.float64)
    D = np.ascontiguousarray(D, dtype=np.float64)
    assert I.shape == (npair * (npair + 1) // 2,) and D.shape == (n, n)
    J, K = np.zeros((n, n)), np.zeros((n, n))
    port().lib.oq_jk_packed(n, I.ctypes.data, D.ctypes.data, J.ctypes.data, K.ctypes.data)
    return J, K


def build_I(b: CGTOBasis, lib: Lib | None = None) -> np.ndarray:
    n = b.n
    out = np.zeros((n, n, n, n))
    port().lib.oq_build_I(*b.args(), _eri_ptr(lib), out.ctypes.data)
    return out


def JK_inmem(I: np.ndarray, D: np.ndarray):
    n = D.shape[0]
    I = np.ascontiguousarray(I, dtype=np.float64)
    D = np.ascontiguousarray(D, dtype=np.float64)
    J = np.zeros((n, n))
    K = np.zeros((n, n))
    port().lib.oq_jk_inmem(n, I.ctypes.data, D.ctypes.data, J.ctypes.data, K.ctypes.data)
    return J, K


def ijkl2intindex(i, j, k, l):
    """Packed 8-fold ERI position, restating libpyquante2/cints.c:375-387:
    order each index pair (larger first), form the pair indices ij, kl, order
    those, then the pair index of (ij, kl).  Works on numpy integer arrays."""
    i, j, k, l = (np.asarray(x, dtype=np.int64) for x in (i, j, k, l))
    ij = np.where(i >= j, i * (i + 1) // 2 + j, j * (j + 1) // 2 + i)
    kl = np.where(k >= l, k * (k + 1) // 2 + l, l * (l + 1) // 2 + k)
    return np.where(ij >= kl, ij * (ij + 1) // 2 + kl, kl * (kl + 1) // 2 + ij)


def pack_I(I: np.ndarray) -> np.ndarray:
    """A dense n^4 tensor in the packed layout of ijkl2intindex (each unique
    integral once; taken from the index quadruple with i >= j, k >= l, ij >= kl)."""
    n = I.shape[0]
    npair = n * (n + 1) // 2
    out = np.zeros(npair * (npair + 1) // 2)
    i, j, k, l = np.meshgrid(*(np.arange(n),) * 4, indexing="ij")
    out[ijkl2intindex(i, j, k, l).ravel()] = I.ravel()
    return out


def contracted_eri(b: CGTOBasis, i, j, k, l, lib: Lib | None = None) -> float:
    return port().lib.oq_contracted_eri(*b.args(), _eri_ptr(lib), i, j, k, l)


# ---------------------------------------------------------------------------
# SCF driver (src/bin/rchem.rs:40-127 restated, plus the nuclear repulsion
# energy the reference does not print)
# ---------------------------------------------------------------------------
def symm_orthog(Smat):
    """rchem.rs:44-51: X = U diag(lambda^-1/2) U^T."""
    w, U = np.linalg.eigh(Smat)
    return U @ np.diag(w ** -0.5) @ U.T


def build_density(Cmat, nocc):
    """rchem.rs:101-104: D = C_occ C_occ^T (no factor 2)."""
    Co = Cmat[:, :nocc]
    return Co @ Co.T


def elec_energy(D, H, F):
    """rchem.rs:106-108: sum (H + F) o D."""
    return float(((H + F) * D).sum())


def nuclear_repulsion(atomnos, coords):
    R = np.asarray(coords, dtype=np.float64).reshape(-1, 3)
    Z = np.asarray(atomnos, dtype=np.float64)
    e = 0.0
    for a in range(len(Z)):
        for c in range(a):
            e += Z[a] * Z[c] / np.linalg.norm(R[a] - R[c])
    return e


def rhf(b: CGTOBasis, atomnos, coords, nocc, jk=None, thresh_e=1e-11, max_iter=1024, lib=None, diis=0,
        thresh_d=None):
    """Roothaan iterations as rchem.rs:40-89 (core guess; D = C_occ C_occ^T;
    F = H + 2J - K; E = sum (H + F) o D; stop when |Delta E| < thresh_e).
    ``diis`` > 0 extrapolates the Fock matrix by Pulay's DIIS over that many
    previous iterations (error vector X^T (FDS - SDF) X), which the reference
    does not do; it changes the path to convergence, not the converged
    energy.  ``thresh_d`` also requires max |Delta D| below it.  ``e_final``
    is the energy of the last density with its own Fock matrix."""
    Smat, Tm, Vm = S(b, lib), T(b, lib), V(b, coords, atomnos, lib)
    H = Tm + Vm
    X = symm_orthog(Smat)
    _, Cp = np.linalg.eigh(X.T @ H @ X)
    D = build_density(X @ Cp, nocc)
    e_new = elec_energy(D, H, H)
    jk = jk or (lambda Dm: JK_sym(b, Dm, lib))
    focks, errs = [], []
    it = 0
    converged = False
    for it in range(max_iter):
        J, K = jk(D)
        F = H + 2.0 * J - K
        Fx = F
        if diis > 0:
            focks.append(F)
            errs.append(X.T @ (F @ D @ Smat - Smat @ D @ F) @ X)
            del focks[:-diis], errs[:-diis]
            m = len(focks)
            if m >= 2:
                B = -np.ones((m + 1, m + 1))
                B[m, m] = 0.0
                for i in range(m):
                    for j in range(m):
                        B[i, j] = float(np.sum(errs[i] * errs[j]))
                rhs = np.zeros(m + 1)
                rhs[m] = -1.0
                try:
                    c = np.linalg.solve(B, rhs)
                    Fx = sum(c[i] * focks[i] for i in range(m))
                except np.linalg.LinAlgError:
                    Fx = F
        _, Cp = np.linalg.eigh(X.T @ Fx @ X)
        D_old = D
        D = build_density(X @ Cp, nocc)
        e_old, e_new = e_new, elec_energy(D, H, F)
        if abs(e_new - e_old) < thresh_e and (thresh_d is None or np.abs(D - D_old).max() < thresh_d):
            converged = True
            break
    J, K = jk(D)
    e_final = elec_energy(D, H, H + 2.0 * J - K)
    return {"e_elec": e_new, "e_final": e_final, "e_nuc": nuclear_repulsion(atomnos, coords), "D": D,
            "iterations": it + 1, "converged": converged, "S": Smat, "T": Tm, "V": Vm}
