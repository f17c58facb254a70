"""The generated HGP class code and the Boys evaluator, compiled for the host
with g++ (tests/host_eri_check.cpp), against the oracle -- no GPU needed.

This pins the code generator (csrc/gen_eri.py) and csrc/boys.cuh before any
GPU run; the GPU tests then pin the kernels that wrap them.
"""
import ctypes as C
import itertools
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "rchem_gb300", "csrc")

CLASSES = [(0, 0, 0, 0), (1, 0, 0, 0), (1, 0, 1, 0), (1, 1, 0, 0), (1, 1, 1, 0), (1, 1, 1, 1), (2, 0, 0, 0),
           (2, 0, 1, 0), (2, 0, 1, 1), (2, 0, 2, 0), (2, 1, 0, 0), (2, 1, 1, 0), (2, 1, 1, 1), (2, 1, 2, 0),
           (2, 1, 2, 1), (2, 2, 0, 0), (2, 2, 1, 0), (2, 2, 1, 1), (2, 2, 2, 0), (2, 2, 2, 1), (2, 2, 2, 2)]

# classes with a warp-cooperative program (total angular momentum >= 4)
PROG_CLASSES = [c for c in CLASSES if sum(c) >= 4]


@pytest.fixture(scope="module")
def hostlib(tmp_path_factory):
    d = tmp_path_factory.mktemp("hostcheck")
    gen = d / "gen"
    import importlib.util

    spec = importlib.util.spec_from_file_location("gen_eri", os.path.join(CSRC, "gen_eri.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.main(str(gen))
    with open(d / "eri_all.inc", "w") as f:
        for c in CLASSES:
            f.write('#include "%s/eri_class_%d%d%d%d.inc"\n' % ((str(gen),) + c))
    with open(d / "eri_prog_all.inc", "w") as f:
        for c in PROG_CLASSES:
            f.write('#include "%s/eri_prog_%d%d%d%d.inc"\n' % ((str(gen),) + c))
    so = d / "libhost.so"
    # RCHEM_SANITIZE_FLAGS: extra compiler flags (tests/test_sanitizers.py passes ASan/UBSan ones)
    extra = os.environ.get("RCHEM_SANITIZE_FLAGS", "").split()
    env = {k: v for k, v in os.environ.items() if k != "LD_PRELOAD"}  # the compiler itself runs uninstrumented
    subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", *extra, "-I", CSRC, "-I", str(d), "-o",
                    str(so), os.path.join(ROOT, "tests", "host_eri_check.cpp")], check=True, env=env)
    L = C.CDLL(str(so))
    L.host_eri_block.argtypes = [C.c_int] * 5 + [C.c_void_p] * 5
    L.host_eri_block_prog.argtypes = [C.c_int] * 4 + [C.c_void_p] * 5
    L.host_boys.restype = C.c_double
    L.host_boys.argtypes = [C.c_int, C.c_double, C.c_int]
    return L


def _block_oracle(port, oracle, cls, R, e, c):
    na = [len(oracle.ijk_list(l)) for l in cls]
    ref = np.zeros(na)
    for idx in itertools.product(*[range(x) for x in na]):
        pw = [oracle.ijk_list(cls[k])[idx[k]] for k in range(4)]
        v = 0.0
        for a, b, cc, d in itertools.product(*[range(len(x)) for x in e]):
            ps = (a, b, cc, d)
            args = []
            for k in range(4):
                args += [R[k], port.pgto_norm(e[k][ps[k]], *pw[k]), pw[k], e[k][ps[k]]]
            v += c[0][a] * c[1][b] * c[2][cc] * c[3][d] * port.coulomb_repulsion(*args)
        ref[idx] = v
    return ref


@pytest.mark.parametrize("cls", CLASSES)
def test_generated_class_vs_oracle(hostlib, port, cls):
    import oracle

    rng = np.random.default_rng(sum(cls) * 7 + cls[0])
    for trial in range(2):
        R = rng.uniform(-1.5, 1.5, (4, 3))
        if trial == 1:
            R[1] = R[0]
            R[3] = R[2]
        n = rng.integers(1, 3, 4)
        e = [rng.uniform(0.2, 3.0, k) for k in n]
        c = [rng.uniform(0.2, 1.0, k) for k in n]
        cs = np.concatenate([c[k] * np.array([port.pgto_norm(x, cls[k], 0, 0) for x in e[k]]) for k in range(4)])
        es = np.concatenate(e)
        ref = _block_oracle(port, oracle, cls, R, e, c)
        for f32, tol in ((0, 1e-14), (1, 2e-5)):
            res = np.zeros(ref.size)
            rc = hostlib.host_eri_block(*cls, f32, np.ascontiguousarray(R).ctypes.data,
                                        np.ascontiguousarray(n, dtype=np.int32).ctypes.data, es.ctypes.data,
                                        cs.ctypes.data, res.ctypes.data)
            assert rc == 0
            res = res.reshape(ref.shape)
            scale = 1.0 if f32 == 0 else np.abs(ref).max()
            assert np.abs(res - ref).max() <= tol * scale, (cls, f32, np.abs(res - ref).max())


@pytest.mark.parametrize("cls", PROG_CLASSES)
def test_warp_cooperative_program_vs_oracle(hostlib, port, cls):
    """The generated level-ordered VRR/HRR program of a large class, run term by
    term on the host, gives the oracle's contracted integrals."""
    import oracle

    rng = np.random.default_rng(sum(cls) * 11 + cls[1])
    R = rng.uniform(-1.5, 1.5, (4, 3))
    n = np.array([1, 2, 1, 2])
    e = [rng.uniform(0.2, 3.0, k) for k in n]
    c = [rng.uniform(0.2, 1.0, k) for k in n]
    cs = np.concatenate([c[k] * np.array([port.pgto_norm(x, cls[k], 0, 0) for x in e[k]]) for k in range(4)])
    es = np.concatenate(e)
    ref = _block_oracle(port, oracle, cls, R, e, c)
    res = np.zeros(ref.size)
    rc = hostlib.host_eri_block_prog(*cls, np.ascontiguousarray(R).ctypes.data,
                                     np.ascontiguousarray(n, dtype=np.int32).ctypes.data, es.ctypes.data,
                                     cs.ctypes.data, res.ctypes.data)
    assert rc == 0
    assert np.abs(res.reshape(ref.shape) - ref).max() <= 1e-14


def test_boys_evaluator(hostlib, port):
    xs = [0.0, 1e-9, 0.01, 0.03125, 0.5, 1.0, 2.5, 5.0, 10.0, 20.0, 33.0, 39.99, 40.0, 41.0, 50.0, 100.0, 1e3]
    for m in range(0, 12):
        for x in xs:
            ex = port.boys_exact(m, x)
            assert abs(hostlib.host_boys(m, x, 0) - ex) <= 4e-15 * ex, (m, x)
            assert abs(hostlib.host_boys(m, x, 1) - ex) <= 2e-6 * ex, (m, x)


def test_generated_translation_units(tmp_path):
    """One translation unit per class; the classes of total angular momentum 6
    and 7 put their one-lane-group kernel in a second one (eri_<class>_cls.cu),
    which the build compiles with ptxas -O1 and the first reaches through an
    external launcher; (dd|dd) alone is warp-cooperative only."""
    import importlib.util
    import re

    spec = importlib.util.spec_from_file_location("gen_eri_tu", os.path.join(CSRC, "gen_eri.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.main(str(tmp_path))
    from rchem_gb300 import build as B

    for c in CLASSES:
        tag = "%d%d%d%d" % c
        main = (tmp_path / ("eri_%s.cu" % tag)).read_text()
        cls_tu = tmp_path / ("eri_%s_cls.cu" % tag)
        split = sum(c) in (6, 7)
        assert cls_tu.exists() == split, c
        assert B.ptxas_extra(str(tmp_path / ("eri_%s.cu" % tag))) == []
        if split:
            assert "launch_eri_class<%d, %d, %d, %d, true>(a, fp32, epi, s, rchem_launch_eri_cls_%s)" % (c + (tag,)) \
                in main
            assert "launch_eri_cls_only<%d, %d, %d, %d>(a, prec, epi, s)" % c in cls_tu.read_text()
            assert B.ptxas_extra(str(cls_tu)) == ["-Xptxas", "-O1"]
        else:
            assert "launch_eri_class<%d, %d, %d, %d>(a, fp32, epi, s)" % c in main
        inc = (tmp_path / ("eri_class_%s.inc" % tag)).read_text()
        wc_only = re.search(r"WC_ONLY = (true|false)", inc).group(1) == "true"
        assert wc_only == (c == (2, 2, 2, 2)), c
    assert B.ptxas_extra(os.path.join(CSRC, "grad_pppp_f64.cu")) == ["-Xptxas", "-O1"]
    assert B.ptxas_extra(os.path.join(CSRC, "grad_sp_f64.cu")) == []
