"""rchem_jk_direct_noalloc: the Fock build for callers that cannot allocate
device memory where they need it (an external pooled allocator that owns the
device, or a long-running service that must not allocate in its steady-state
loop).  Called through the C
ABI on device arrays the test owns; its J and K must equal those of the
allocating entry point, rchem_jk_direct, on two calls in a row (the second
call finds the shared scratch array holding the first call's contents).

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _density(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, n)) * 0.2
    return X @ X.T / n


@pytest.mark.parametrize("fp32_tau", [0.0, 1e-6])
def test_noalloc_matches_jk_direct(gpu, fp32_tau):
    import torch

    import rchem_gb300 as rc
    from rchem_gb300 import _lib

    L = _lib.lib()
    Z, R = rc.geometry.water_cluster(3, 5.5, seed=21)
    with rc.Basis(Z, R, "6-31gs-fit") as b:
        n = b.nbf
        opts = _lib.JKOpts(schwarz_tau=1e-12, fp32_tau=fp32_tau, where=_lib.DEVICE)
        for call, seed in enumerate((5, 6)):
            D = torch.from_numpy(_density(n, seed)).cuda()
            J0, K0 = torch.empty_like(D), torch.empty_like(D)
            J1, K1 = torch.full_like(D, np.nan), torch.full_like(D, np.nan)
            torch.cuda.synchronize()  # the library runs on the handle's own stream
            # the allocating entry point (it also plans the work for these options)
            _lib.check(L.rchem_jk_direct(b.handle, C.c_void_p(D.data_ptr()), C.c_void_p(J0.data_ptr()),
                                         C.c_void_p(K0.data_ptr()), C.byref(opts)))
            _lib.check(L.rchem_jk_direct_noalloc(b.handle, C.c_void_p(D.data_ptr()), C.c_void_p(J1.data_ptr()),
                                                 C.c_void_p(K1.data_ptr()), C.byref(opts)))
            torch.cuda.synchronize()
            assert torch.isfinite(J1).all() and torch.isfinite(K1).all()
            assert (J1 - J0).abs().max().item() < 1e-12, call
            assert (K1 - K0).abs().max().item() < 1e-12, call


def test_noalloc_after_emulated_build(gpu):
    """A handle whose last Fock build (and captured graph) used the emulated
    form: the no-allocation build still runs native FP64 and equals the
    allocating entry point's FP64 result."""
    import torch

    import rchem_gb300 as rc
    from rchem_gb300 import _lib

    L = _lib.lib()
    Z, R = rc.geometry.water_cluster(3, 5.5, seed=21)
    with rc.Basis(Z, R, "6-31gs-fit") as b:
        n = b.nbf
        b.autotune(1e-12, 0.0, emulated=True)  # tile shapes chosen for the emulated form
        D = torch.from_numpy(_density(n, 7)).cuda()
        J0, K0 = torch.empty_like(D), torch.empty_like(D)
        Je, Ke = torch.empty_like(D), torch.empty_like(D)
        J1, K1 = torch.full_like(D, np.nan), torch.full_like(D, np.nan)
        ptr = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731
        fp64 = _lib.JKOpts(schwarz_tau=1e-12, where=_lib.DEVICE, emulated=0)
        emul = _lib.JKOpts(schwarz_tau=1e-12, where=_lib.DEVICE, emulated=1)
        torch.cuda.synchronize()
        _lib.check(L.rchem_jk_direct(b.handle, ptr(D), ptr(J0), ptr(K0), C.byref(fp64)))
        _lib.check(L.rchem_jk_direct(b.handle, ptr(D), ptr(Je), ptr(Ke), C.byref(emul)))
        for call in range(2):
            _lib.check(L.rchem_jk_direct_noalloc(b.handle, ptr(D), ptr(J1), ptr(K1), C.byref(emul)))
            torch.cuda.synchronize()
            assert (J1 - J0).abs().max().item() < 1e-12, call
            assert (K1 - K0).abs().max().item() < 1e-12, call
        # the emulated build itself differs from FP64 only in the last bits
        assert (Je - J0).abs().max().item() < 1e-12


def test_noalloc_rejects_what_it_cannot_do(gpu):
    import torch

    import rchem_gb300 as rc
    from rchem_gb300 import _lib

    L = _lib.lib()
    Z, R = rc.geometry.water_monomer()
    with rc.Basis(Z, R, "sto-3g-fit") as b:
        n = b.nbf
        D = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        J, K = torch.empty_like(D), torch.empty_like(D)
        args = [b.handle, C.c_void_p(D.data_ptr()), C.c_void_p(J.data_ptr()), C.c_void_p(K.data_ptr())]
        host = _lib.JKOpts(schwarz_tau=1e-12, where=_lib.HOST)
        assert L.rchem_jk_direct_noalloc(*args, C.byref(host)) == _lib.RCHEM_ERR_INVALID
        unplanned = _lib.JKOpts(schwarz_tau=1e-9, where=_lib.DEVICE)
        assert L.rchem_jk_direct_noalloc(*args, C.byref(unplanned)) == _lib.RCHEM_ERR_INVALID
        assert b"no work plan" in L.rchem_last_error()
    # more basis functions than the static scratch holds (water x34 in the 6-31G*-shaped basis: 646)
    Z, R = rc.geometry.water_cluster(34, 15.0, seed=9)
    with rc.Basis(Z, R, "6-31gs-fit") as b:
        n = b.nbf
        assert n > 640
        D = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        J, K = torch.empty_like(D), torch.empty_like(D)
        opts = _lib.JKOpts(schwarz_tau=1e-12, where=_lib.DEVICE)
        rc_ = L.rchem_jk_direct_noalloc(b.handle, C.c_void_p(D.data_ptr()), C.c_void_p(J.data_ptr()),
                                        C.c_void_p(K.data_ptr()), C.byref(opts))
        assert rc_ == _lib.RCHEM_ERR_UNSUPPORTED
        assert b"640" in L.rchem_last_error()
