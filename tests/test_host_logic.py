"""Host-side logic without a GPU: AO ordering, basis files, geometry, the
C-ABI library's exported symbols."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_ijk_list_order():
    """src/shell.rs:44-60."""
    import oracle

    assert oracle.ijk_list(3) == [(3, 0, 0), (2, 1, 0), (2, 0, 1), (1, 2, 0), (1, 1, 1), (1, 0, 2), (0, 3, 0),
                                  (0, 2, 1), (0, 1, 2), (0, 0, 3)]


def test_shell4_order():
    """src/shell.rs:62-86: get_shell4(2,0,0,1) is the product order of get_ijk_list."""
    import itertools

    import oracle

    comps = [list(a) + list(b) + list(c) + list(d) for a, b, c, d in
             itertools.product(oracle.ijk_list(2), oracle.ijk_list(0), oracle.ijk_list(0), oracle.ijk_list(1))]
    assert comps[0] == [2, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0]
    assert comps[4] == [1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0]
    assert comps[-1] == [0, 0, 2, 0, 0, 0, 0, 0, 0, 0, 0, 1]
    assert len(comps) == 18


def test_generator_cartesian_order_matches_reference():
    import importlib.util

    spec = importlib.util.spec_from_file_location("g", os.path.join(ROOT, "rchem_gb300", "csrc", "gen_eri.py"))
    g = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(g)
    import oracle

    for l in range(5):
        assert g.ijk_list(l) == oracle.ijk_list(l)
    assert abs(g.comp_norm((1, 1, 0)) - 3 ** 0.5) < 1e-15
    assert g.comp_norm((2, 0, 0)) == 1.0


@pytest.mark.parametrize("name,nbf_h2o,nprim", [("sto-3g-fit", 7, 21), ("6-31g-fit", 13, 30), ("6-31gs-fit", 19, 36),
                                                ("6-31gss-fit", 25, 42)])
def test_basis_sets_shapes(name, nbf_h2o, nprim):
    from rchem_gb300 import bse, geometry

    Z, R = geometry.water_monomer()
    sh = bse.expand_shells(Z, bse.load_bse(name))
    assert sh.nbf == nbf_h2o
    # P = sum over functions of primitives
    P = sum(((l + 1) * (l + 2) // 2) * n for l, n in zip(sh.l, sh.nprim))
    assert P == nprim


def test_expand_shells_matches_oracle_expansion():
    import oracle

    from rchem_gb300 import bse, geometry

    Z, R = geometry.water_cluster(2, 5.0, seed=3)
    doc = bse.load_bse("6-31gss-fit")
    sh = bse.expand_shells(Z, doc)
    ob = oracle.expand_basis(Z, R, doc)
    # AO-by-AO: same atom, same exponents
    ao = 0
    off = 0
    for s in range(len(sh.l)):
        for k in range((sh.l[s] + 1) * (sh.l[s] + 2) // 2):
            assert ob.atom[ao] == sh.atom[s]
            assert sum(ob.powers[ao]) == sh.l[s]
            np.testing.assert_array_equal(ob.exps[ob.prim_off[ao]:ob.prim_off[ao] + ob.nprim[ao]],
                                          sh.exps[off:off + sh.nprim[s]])
            ao += 1
        off += sh.nprim[s]
    assert ao == ob.n


def test_config_sizes():
    from rchem_gb300 import bse, geometry

    sizes = {"h2o_sto3g": 7, "h2o8_631g": 104, "h2o4_631gss": 100, "h2o32_631gs": 608}
    for name, nbf in sizes.items():
        b, Z, R = geometry.config(name)
        assert bse.expand_shells(Z, bse.load_bse(b)).nbf == nbf
        O = R[Z == 8]
        d = np.linalg.norm(O[:, None] - O[None], axis=-1) + np.eye(len(O)) * 1e9
        assert d.min() >= 2.7 * geometry.ANGSTROM_TO_BOHR - 1e-9


def test_geometry_seeded_and_monomer():
    from rchem_gb300 import geometry

    Z, R = geometry.water_monomer()
    r = np.linalg.norm(R[1] - R[0]) / geometry.ANGSTROM_TO_BOHR
    assert abs(r - 0.957) < 1e-12
    v1, v2 = R[1] - R[0], R[2] - R[0]
    ang = np.degrees(np.arccos(v1 @ v2 / np.linalg.norm(v1) / np.linalg.norm(v2)))
    assert abs(ang - 104.5) < 1e-9
    a = geometry.water_cluster(8, 9.0, seed=1)[1]
    b = geometry.water_cluster(8, 9.0, seed=1)[1]
    np.testing.assert_array_equal(a, b)
    batch = geometry.water_batch(512, seed=5)
    sizes = [len(z) // 3 for z, _ in batch]
    assert len(batch) == 512 and sizes.count(1) == 172 and sizes.count(2) == 170 and sizes.count(3) == 170


def test_xyz_roundtrip(tmp_path):
    from rchem_gb300 import bse, geometry

    Z, R = geometry.water_monomer()
    p = tmp_path / "w.xyz"
    bse.write_xyz(p, Z, R)
    Z2, R2 = bse.read_xyz(p)
    np.testing.assert_array_equal(Z, Z2)
    np.testing.assert_allclose(R, R2, atol=1e-11)
    # the reference's own Crawford water file format (bohr, element symbols)
    Z3, R3 = bse.read_xyz(str(p), angstrom=True)
    np.testing.assert_allclose(R3, R2 * bse.ANGSTROM_TO_BOHR)


def _declared_symbols():
    names = set()
    for h in sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?(?:int|double|char\s*\*|const char\s*\*)\s*\*?\s*(\w+)\s*\(", src,
                             flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    """The C-ABI library loads on the host (no GPU calls) and exports every
    entry point the headers declare."""
    from rchem_gb300 import _lib, build

    build.build()
    declared = _declared_symbols()
    assert declared == set(_lib.exported_symbols())
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True, check=True)
    exported = {ln.split()[-1] for ln in out.stdout.splitlines() if " T " in ln}
    missing = declared - exported
    assert not missing, missing
    L = _lib.lib()  # dlopen succeeds without a GPU
    assert L.rchem_abi_version() == 1


def test_invalid_arguments_rejected_without_gpu():
    """Argument validation happens before any device call."""
    import ctypes as C

    from rchem_gb300 import _lib, build

    build.build()
    L = _lib.lib()
    h = C.c_void_p()
    Z = np.array([8], np.int32)
    R = np.array([0.0, 0.0, np.nan])
    one = np.array([0], np.int32)
    e = np.array([1.0])
    rc = L.rchem_basis_create(C.byref(h), 1, Z.ctypes.data, R.ctypes.data, 1, one.ctypes.data, one.ctypes.data,
                              np.array([1], np.int32).ctypes.data, e.ctypes.data, e.ctypes.data)
    assert rc == _lib.RCHEM_ERR_INVALID
    assert b"not finite" in L.rchem_last_error()
    rc = L.rchem_jk_direct(None, None, None, None, None)
    assert rc == _lib.RCHEM_ERR_INVALID
    # the native SCF driver, the packed ERI tensor and its J/K: null handles and
    # bad sizes are refused before any device work
    assert L.rchem_rhf(None, None, None, None, None, None, None, None, None) == _lib.RCHEM_ERR_INVALID
    assert L.rchem_build_I_packed(None, None, _lib.HOST) == _lib.RCHEM_ERR_INVALID
    assert L.rchem_jk_packed(0, None, None, None, None, _lib.HOST) == _lib.RCHEM_ERR_INVALID
    assert L.rchem_eigh_batched(65, 1, None, None, None, None) == _lib.RCHEM_ERR_UNSUPPORTED


def test_shell_validation_before_any_device_call():
    """Every shell is validated on the host before the library touches CUDA:
    unsupported angular momenta and primitive counts, bad exponents or
    coefficients, shells on atoms that do not exist, and (for a batch) shells
    out of geometry order are refused with a status code and a message.  On a
    host without a GPU each of these calls returns before any CUDA call."""
    import ctypes as C

    from rchem_gb300 import _lib, build

    build.build()
    L = _lib.lib()
    i32 = lambda *v: np.array(v, np.int32)  # noqa: E731
    f64 = lambda *v: np.array(v, np.float64)  # noqa: E731
    Z = i32(8, 1)
    R = f64(0.0, 0.0, 0.0, 0.0, 0.0, 1.8)

    def create(atom, l, nprim, exps, coefs):
        h = C.c_void_p()
        atom, l, nprim = i32(*atom), i32(*l), i32(*nprim)
        exps, coefs = f64(*exps), f64(*coefs)
        rc = L.rchem_basis_create(C.byref(h), 2, Z.ctypes.data, R.ctypes.data, len(atom), atom.ctypes.data,
                                  l.ctypes.data, nprim.ctypes.data, exps.ctypes.data, coefs.ctypes.data)
        assert not h.value  # no handle on failure
        return rc, L.rchem_last_error().decode()

    rc, msg = create([0, 1], [3, 0], [1, 1], [1.0, 0.5], [1.0, 1.0])  # f shell
    assert rc == _lib.RCHEM_ERR_UNSUPPORTED and "l=3" in msg
    rc, msg = create([0, 1], [-1, 0], [1, 1], [1.0, 0.5], [1.0, 1.0])
    assert rc == _lib.RCHEM_ERR_UNSUPPORTED and "l=-1" in msg
    rc, msg = create([0, 1], [0, 0], [1, 0], [1.0], [1.0])  # a shell without primitives
    assert rc == _lib.RCHEM_ERR_UNSUPPORTED and "shell 1 has 0 primitives" in msg
    rc, msg = create([0], [0], [17], [1.0] * 17, [1.0] * 17)  # more primitives than the kernels hold
    assert rc == _lib.RCHEM_ERR_UNSUPPORTED and "17 primitives" in msg
    rc, msg = create([0, 2], [0, 0], [1, 1], [1.0, 0.5], [1.0, 1.0])  # atom 2 of 2
    assert rc == _lib.RCHEM_ERR_INVALID and "on atom 2 of 2" in msg
    rc, msg = create([0, 1], [0, 0], [2, 1], [1.0, -0.5, 0.5], [1.0, 1.0, 1.0])  # negative exponent
    assert rc == _lib.RCHEM_ERR_INVALID and "shell 0 primitive 1" in msg
    rc, msg = create([0, 1], [0, 1], [1, 1], [1.0, 0.5], [1.0, np.inf])  # non-finite coefficient
    assert rc == _lib.RCHEM_ERR_INVALID and "shell 1 primitive 0" in msg
    rc, msg = create([0, 1], [0, 0], [1, 1], [1.0, np.nan], [1.0, 1.0])
    assert rc == _lib.RCHEM_ERR_INVALID and "shell 1 primitive 0" in msg

    # a batch: two one-atom geometries whose shells come in the wrong order
    h = C.c_void_p()
    gn, atom, l, npr = i32(1, 1), i32(1, 0), i32(0, 0), i32(1, 1)
    e = f64(1.0, 1.0)
    rc = L.rchem_batch_create(C.byref(h), 2, gn.ctypes.data, 2, Z.ctypes.data, R.ctypes.data, 2, atom.ctypes.data,
                              l.ctypes.data, npr.ctypes.data, e.ctypes.data, e.ctypes.data)
    assert rc == _lib.RCHEM_ERR_INVALID and b"geometry order" in L.rchem_last_error()
    # geometry atom counts that do not add up to the atoms given
    gn = i32(1, 2)
    rc = L.rchem_batch_create(C.byref(h), 2, gn.ctypes.data, 2, Z.ctypes.data, R.ctypes.data, 2, atom.ctypes.data,
                              l.ctypes.data, npr.ctypes.data, e.ctypes.data, e.ctypes.data)
    assert rc == _lib.RCHEM_ERR_INVALID and b"sum to 3, not 2" in L.rchem_last_error()


class _FakeCuda:
    """Stands in for a CUDA tensor in the wrappers' argument checks (no GPU here)."""

    is_cuda = True

    def __init__(self, shape, dtype=None, contiguous=True, device="cuda:0"):
        import torch

        self.shape = shape
        self.dtype = dtype or torch.float64
        self._c = contiguous
        self.device = device

    def is_contiguous(self):
        return self._c

    def contiguous(self):
        return _FakeCuda(self.shape, self.dtype, True, self.device)


def test_wrappers_refuse_mis_sized_or_mis_typed_arrays():
    """The Python mirror of the basis API checks every array's shape, type and
    layout before the library would read or write it as a dense float64 block;
    these all raise before any library call, so they run without a GPU."""
    import types

    import torch

    import rchem_gb300 as rc
    from rchem_gb300 import batch

    n = 7
    b = types.SimpleNamespace(nbf=n)  # only nbf is read before the checks
    ok = np.zeros((n, n))
    with pytest.raises(ValueError, match="J must be a C-contiguous float64"):
        rc.JK_direct(np.zeros((n, n), np.float32), ok, b, ok)
    with pytest.raises(ValueError, match="K must be a C-contiguous float64"):
        rc.JK_direct(ok, np.asfortranarray(np.zeros((n, n))), b, ok)
    with pytest.raises(ValueError, match=r"K: expected shape \(7, 7\), got \(8, 7\)"):
        rc.JK_direct(ok, np.zeros((n + 1, n)), b, ok)
    with pytest.raises(ValueError, match="D: expected shape"):
        rc.JK_direct(ok, ok, b, np.zeros((n, n + 1)))
    with pytest.raises(ValueError, match="all be host arrays or all CUDA"):
        rc.JK_direct(_FakeCuda((n, n)), ok, b, ok)
    with pytest.raises(ValueError, match="float64 tensor"):
        rc.JK_direct(_FakeCuda((n, n), torch.float32), _FakeCuda((n, n)), b, _FakeCuda((n, n)))
    with pytest.raises(ValueError, match="contiguous tensor"):
        rc.JK_direct(_FakeCuda((n, n), contiguous=False), _FakeCuda((n, n)), b, _FakeCuda((n, n)))
    with pytest.raises(ValueError, match="one device"):
        rc.JK_direct(_FakeCuda((n, n)), _FakeCuda((n, n), device="cuda:1"), b, _FakeCuda((n, n)))

    # the tensor-based J/K: I must hold n^4 (dense) or the packed count of elements
    npair = n * (n + 1) // 2
    with pytest.raises(ValueError, match="I: expected 2401 elements"):
        rc.JK_inmem(np.zeros(n ** 4 - 1), ok)
    with pytest.raises(ValueError, match="I: expected %d elements" % (npair * (npair + 1) // 2)):
        rc.JK_packed(np.zeros(n ** 4), ok)
    with pytest.raises(ValueError, match="square matrix"):
        rc.JK_inmem(np.zeros(n ** 4), np.zeros((n, n - 1)))
    with pytest.raises(ValueError, match="float64 tensor"):
        rc.JK_inmem(_FakeCuda((n ** 4,), torch.float32), _FakeCuda((n, n)))

    # the batched Fock build: packed device vectors of the handle's length
    bb = types.SimpleNamespace(packed=100)
    with pytest.raises(ValueError, match="must be CUDA tensors"):
        batch.jk(bb, np.zeros(100), np.zeros(100), np.zeros(100))
    with pytest.raises(ValueError, match="J: expected 100 elements"):
        batch.jk(bb, _FakeCuda((100,)), _FakeCuda((99,)), _FakeCuda((100,)))


def test_wrappers_pass_valid_arrays_through(monkeypatch):
    """Valid host arrays reach the C ABI unchanged: the wrappers pass the
    arrays' own buffers (no copies of C-contiguous float64 input), the size,
    the host/device flag and the options, here recorded by a stand-in for the
    loaded library."""
    import ctypes as C
    import types

    import rchem_gb300 as rc
    from rchem_gb300 import _lib

    calls = []

    class Recorder:
        def __getattr__(self, name):
            def f(*args):
                calls.append((name, args))
                return 0

            return f

    monkeypatch.setattr(_lib, "lib", lambda: Recorder())
    n = 5
    b = types.SimpleNamespace(nbf=n, handle="handle")
    D = np.eye(n)
    J, K = np.zeros((n, n)), np.zeros((n, n))
    rc.JK_direct(J, K, b, D, schwarz_tau=1e-10, fp32_tau=1e-6, emulated=True)
    name, a = calls[-1]
    assert name == "rchem_jk_direct" and a[0] == "handle"
    assert [x.value for x in a[1:4]] == [D.ctypes.data, J.ctypes.data, K.ctypes.data]
    o = a[4]._obj
    assert (o.schwarz_tau, o.fp32_tau, o.where, o.emulated) == (1e-10, 1e-6, _lib.HOST, 1)
    rc.JK_direct(J, K, b, D, schwarz_tau=0.0)  # no screening is passed as a negative threshold
    assert calls[-1][1][4]._obj.schwarz_tau < 0 and calls[-1][1][4]._obj.emulated == 0

    I = np.zeros(n ** 4)
    Ji, Ki = rc.JK_inmem(I, D)
    name, a = calls[-1]
    assert name == "rchem_jk_inmem" and a[0] == n and a[5] == _lib.HOST
    assert [x.value for x in a[1:5]] == [I.ctypes.data, D.ctypes.data, Ji.ctypes.data, Ki.ctypes.data]
    npair = n * (n + 1) // 2
    Ip = np.zeros(npair * (npair + 1) // 2)
    Jp, Kp = rc.JK_packed(Ip, D)
    name, a = calls[-1]
    assert name == "rchem_jk_packed" and a[0] == n and a[1].value == Ip.ctypes.data
    assert Jp.shape == Kp.shape == (n, n)
    # a float32 or strided density is converted on the host, not refused
    rc.JK_direct(J, K, b, np.eye(n, dtype=np.float32))
    rc.JK_direct(J, K, b, np.eye(2 * n)[::2, ::2])
    assert isinstance(calls[-1][1][1], C.c_void_p)


def test_gradient_and_boys_wrappers_refuse_bad_arrays():
    """The gradient wrappers check the density and energy-weighted density they
    are given (a result dict may come from the caller); the Boys batch needs
    as many orders as arguments."""
    import types

    import torch

    import rchem_gb300 as rc
    from rchem_gb300 import batch, cints

    b = types.SimpleNamespace(nbf=4, atomnos=np.array([1, 1]))
    with pytest.raises(ValueError, match="W: expected shape"):
        rc.scf.gradient(b, {"D": _FakeCuda((4, 4)), "W": _FakeCuda((5, 5))})
    with pytest.raises(ValueError, match="D and W must be CUDA tensors"):
        rc.scf.gradient(b, {"D": np.zeros((4, 4)), "W": np.zeros((4, 4))})
    with pytest.raises(ValueError, match="all be host arrays or all CUDA tensors"):
        rc.scf.gradient(b, {"D": _FakeCuda((4, 4)), "W": np.zeros((4, 4))})
    bb = types.SimpleNamespace(packed=32, atomnos=np.array([1, 1]))
    with pytest.raises(ValueError, match="float64 tensor"):
        batch.gradient_batch(bb, {"D": _FakeCuda((32,)), "W": _FakeCuda((32,), torch.float32)})
    with pytest.raises(ValueError, match="same length"):
        cints.boys_batch([0, 1, 2], [0.5, 1.0])


def test_c_consumer_links_and_calls_the_abi(tmp_path):
    """A plain C99 program (tests/abi_check.c) includes the public headers in
    strict C mode, links librchem_gpu.so and calls the entry points that need
    no GPU: the headers are valid C for a bindgen/FFI consumer and the
    exported symbols have C linkage."""
    from rchem_gb300 import _lib, build

    build.build()
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = tmp_path / "abi_check"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_check.c"), "-o", str(exe), "-L", libdir, "-lrchem_gpu",
                    "-Wl,-rpath," + libdir], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "abi_check: ok" in r.stdout
