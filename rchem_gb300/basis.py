"""Host-side mirror of the reference's basis API (src/basis.rs), GPU-backed.

Same names and meanings as the reference:

=====================================  =========================================
reference (src/basis.rs)               here
=====================================  =========================================
``Basis::new(atomnos, coords, name)``  ``Basis(atomnos, coords, name)``  :181
``S(&basis)``                          ``S(basis)``                      :234
``T(&basis)``                          ``T(basis)``                      :273
``V(&basis, coords, atomnos)``         ``V(basis, coords, atomnos)``     :316
``JK_direct(&mut J, &mut K, &b, &D)``  ``JK_direct(J, K, basis, D)``     :383
``build_I(&basis)``                    ``build_I(basis)``                :430
``JK_inmem(&I, &D)``                   ``JK_inmem(I, D)``                :462
=====================================  =========================================

Arrays may be numpy arrays (host) or CUDA torch tensors (device); outputs
follow the input kind.  All work runs through librchem_gpu.so: there is no
CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .bse import expand_shells, load_bse


def _is_cuda(x) -> bool:
    return hasattr(x, "is_cuda") and bool(x.is_cuda)


def _ptr(x):
    if _is_cuda(x):
        return x.data_ptr()
    return x.ctypes.data


def _check_f64(X, name, shape=None, numel=None):
    """Refuse, before any library call, an array the library would read or
    write as a dense row-major float64 block of another size or type: a
    C-contiguous float64 numpy array or a contiguous float64 CUDA tensor with
    the given shape (or number of elements)."""
    shp = tuple(int(d) for d in X.shape)
    if shape is not None and shp != tuple(shape):
        raise ValueError("%s: expected shape %s, got %s" % (name, tuple(shape), shp))
    if numel is not None and int(np.prod(shp, dtype=np.int64)) != numel:
        raise ValueError("%s: expected %d elements, got %d (shape %s)" % (name, numel, int(np.prod(shp)), shp))
    if _is_cuda(X):
        import torch

        if X.dtype != torch.float64:
            raise ValueError("%s must be a float64 tensor, got %s" % (name, X.dtype))
        if not X.is_contiguous():
            raise ValueError("%s must be a contiguous tensor" % name)
    elif not (isinstance(X, np.ndarray) and X.dtype == np.float64 and X.flags.c_contiguous):
        raise ValueError("%s must be a C-contiguous float64 numpy array or a CUDA tensor" % name)


def _same_kind(*xs):
    """All host arrays or all CUDA tensors on one device; True for CUDA."""
    dev = _is_cuda(xs[0])
    if any(_is_cuda(x) != dev for x in xs):
        raise ValueError("arrays must all be host arrays or all CUDA tensors")
    if dev and len({str(x.device) for x in xs}) != 1:
        raise ValueError("CUDA tensors must be on one device")
    return dev


def _after_torch(basis, *xs):
    """The library queues its work on the handle's own stream.  When CUDA
    tensors are passed, work still queued on torch's current stream (producing
    an input, or reading a buffer the call overwrites) must finish first,
    unless the handle already runs on that stream (Basis.set_stream)."""
    if any(_is_cuda(x) for x in xs):
        import torch

        cur = torch.cuda.current_stream()
        if getattr(basis, "_stream", None) != cur.cuda_stream:
            cur.synchronize()


class Basis:
    """A basis on the GPU: shells, shell pairs, Schwarz bounds, Boys tables."""

    def __init__(self, atomnos, coords, basis_set_name="sto-3g-fit"):
        self.atomnos = np.ascontiguousarray(atomnos, dtype=np.int32).reshape(-1)
        self.coords = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
        self.name = basis_set_name if isinstance(basis_set_name, str) else "custom"
        self.shells = expand_shells(self.atomnos, load_bse(basis_set_name))
        h = C.c_void_p()
        L = _lib.lib()
        sh = self.shells
        _lib.check(L.rchem_basis_create(C.byref(h), len(self.atomnos), self.atomnos.ctypes.data,
                                        self.coords.ctypes.data, len(sh.l), sh.atom.ctypes.data, sh.l.ctypes.data,
                                        sh.nprim.ctypes.data, sh.exps.ctypes.data, sh.coefs.ctypes.data))
        self._h = h
        self.nbf = int(L.rchem_basis_nbf(h))

    @property
    def handle(self):
        if self._h is None:
            raise ValueError("basis is closed")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            _lib.lib().rchem_basis_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_ptr: int):
        """Run this basis' work on a caller-owned CUDA stream (e.g. torch's)."""
        _lib.check(_lib.lib().rchem_basis_set_stream(self.handle, C.c_void_p(stream_ptr)))
        self._stream = stream_ptr

    def autotune(self, schwarz_tau=1e-12, fp32_tau=0.0, emulated=False, fp32_boys64=False, fp32_rec64=False):
        """Pick the Fock build's tile shape per integral class for this basis
        (rchem_autotune); returns {(class, precision): min primitive quartets per lane,
        or 0 / -16 / -8 for the warp-cooperative kernel with 32 / 16 / 8 lanes per quartet}."""
        import numpy as _np

        chosen = _np.zeros(2 * 21, dtype=_np.int32)
        o = _lib.JKOpts(schwarz_tau=schwarz_tau if schwarz_tau > 0 else -1.0, fp32_tau=fp32_tau,
                        emulated=jk_flags(emulated, fp32_boys64, fp32_rec64))
        _lib.check(_lib.lib().rchem_autotune(self.handle, C.byref(o), chosen.ctypes.data))
        return {(k, p): int(chosen[2 * k + p]) for k in range(21) for p in range(2)}

    def set_tile_shape(self, cls: int, prec: int, ppl: int):
        """Fix one class list's tile shape (rchem_set_tile_shape): ppl = minimum
        primitive quartets per lane; 0, -16, -8 = the warp-cooperative kernel with
        32, 16, 8 lanes per quartet."""
        _lib.check(_lib.lib().rchem_set_tile_shape(self.handle, cls, prec, ppl))

    def set_exponent_table(self, on: bool):
        """Read the primitive quartets' (p, q) factors from the exponent table
        (default) or compute them in every primitive quartet
        (rchem_set_exponent_table)."""
        _lib.check(_lib.lib().rchem_set_exponent_table(self.handle, 1 if on else 0))

    def class_stats(self) -> list:
        """Per integral class of the current work plan: (l_a,l_b,l_c,l_d) with the
        FP64 / FP32 shell quartets, primitive quartets and algorithmic FLOPs."""
        import numpy as _np

        cl = _np.zeros(84, dtype=_np.int32)
        q = _np.zeros(42, dtype=_np.int64)
        pq = _np.zeros(42, dtype=_np.int64)
        fl = _np.zeros(42)
        _lib.check(_lib.lib().rchem_jk_class_stats(self.handle, cl.ctypes.data, q.ctypes.data, pq.ctypes.data,
                                                   fl.ctypes.data))
        return [{"class": tuple(int(x) for x in cl[4 * k:4 * k + 4]), "quartets": (int(q[2 * k]), int(q[2 * k + 1])),
                 "prim_quartets": (int(pq[2 * k]), int(pq[2 * k + 1])), "flops": (float(fl[2 * k]), float(fl[2 * k + 1]))}
                for k in range(21)]

    def list_times(self, schwarz_tau=1e-12, fp32_tau=0.0, emulated=False):
        """Device time (ms) of every class list of the Fock build planned for
        these options, each list launched alone (rchem_jk_list_times):
        [(class, (FP64/emulated ms, FP32 ms))] in class order."""
        ms = np.zeros(42, dtype=np.float32)
        o = _lib.JKOpts(schwarz_tau=schwarz_tau if schwarz_tau > 0 else -1.0, fp32_tau=fp32_tau,
                        emulated=1 if emulated else 0)
        _lib.check(_lib.lib().rchem_jk_list_times(self.handle, C.byref(o), ms.ctypes.data))
        return [(k, (float(ms[2 * k]), float(ms[2 * k + 1]))) for k in range(21)]

    def stats(self) -> dict:
        st = _lib.JKStats()
        _lib.check(_lib.lib().rchem_jk_stats_get(self.handle, C.byref(st)))
        return st.as_dict()

    def _new(self, like=None, shape=None):
        shape = shape or (self.nbf, self.nbf)
        if like is not None and _is_cuda(like):
            import torch

            return torch.empty(shape, dtype=torch.float64, device=like.device)
        return np.empty(shape, dtype=np.float64)


def _onee(fn, basis, device=False):
    out = basis._new()
    if device:
        import torch

        out = torch.empty((basis.nbf, basis.nbf), dtype=torch.float64, device="cuda")
        _after_torch(basis, out)
    _lib.check(fn(basis.handle, C.c_void_p(_ptr(out)), _lib.DEVICE if device else _lib.HOST))
    return out


def S(basis: Basis, device=False):
    return _onee(_lib.lib().rchem_S, basis, device)


def T(basis: Basis, device=False):
    return _onee(_lib.lib().rchem_T, basis, device)


def V(basis: Basis, atomcoords=None, atomnos=None, device=False):
    """V = sum_C Z_C V_C over the basis' own atoms (the reference passes the
    same coordinates and atomic numbers it built the basis from)."""
    if atomcoords is not None and not np.allclose(np.asarray(atomcoords).reshape(-1, 3), basis.coords):
        raise ValueError("V over atoms other than the basis' own is not supported")
    return _onee(_lib.lib().rchem_V, basis, device)


def moment(basis: Basis, center, order, device=False):
    """<mu|(x-Cx)^ox (y-Cy)^oy (z-Cz)^oz|nu> (src/integrals/os86.rs:775-828)."""
    c = np.ascontiguousarray(center, dtype=np.float64)
    out = basis._new()
    if device:
        import torch

        out = torch.empty((basis.nbf, basis.nbf), dtype=torch.float64, device="cuda")
        _after_torch(basis, out)
    _lib.check(_lib.lib().rchem_moment(basis.handle, c.ctypes.data, int(order[0]), int(order[1]), int(order[2]),
                                       C.c_void_p(_ptr(out)), _lib.DEVICE if device else _lib.HOST))
    return out


def jk_flags(emulated=False, fp32_boys64=False, fp32_rec64=False) -> int:
    """rchem_jk_opts.emulated: RCHEM_JK_EMULATED (1) | RCHEM_JK_FP32_BOYS64 (2) or
    RCHEM_JK_FP32_REC64 (4)."""
    return (1 if emulated else 0) | (2 if fp32_boys64 else 0) | (4 if fp32_rec64 else 0)


def JK_direct(J, K, basis: Basis, D, schwarz_tau=1e-12, fp32_tau=0.0, emulated=False, part=0, nparts=1,
              fp32_boys64=False, fp32_rec64=False):
    """Fill J and K (in place, like the reference) from the density D.
    ``fp32_tau`` > 0 selects the mixed form; ``emulated`` computes the FP64
    quartets in double-float arithmetic on the FP32 pipe; ``fp32_boys64`` the
    FP32 quartets' Boys function and downward recursion in FP64, ``fp32_rec64``
    only their recursion.  ``nparts`` > 1
    computes only share ``part`` of the bra shell pairs (rchem_jk_direct_part):
    the sum over the nparts shares is the whole build."""
    if not (0 <= part < nparts):
        raise ValueError("part %d of %d" % (part, nparts))
    dev = _same_kind(D, J, K)
    D = D.contiguous() if dev else np.ascontiguousarray(D, dtype=np.float64)
    n = basis.nbf
    for X, name in ((D, "D"), (J, "J"), (K, "K")):
        _check_f64(X, name, shape=(n, n))
    o = _lib.JKOpts(schwarz_tau=schwarz_tau if schwarz_tau > 0 else -1.0, fp32_tau=fp32_tau,
                    where=_lib.DEVICE if dev else _lib.HOST, emulated=jk_flags(emulated, fp32_boys64, fp32_rec64))
    _after_torch(basis, D, J, K)
    if nparts == 1:
        _lib.check(_lib.lib().rchem_jk_direct(basis.handle, C.c_void_p(_ptr(D)), C.c_void_p(_ptr(J)),
                                              C.c_void_p(_ptr(K)), C.byref(o)))
    else:
        _lib.check(_lib.lib().rchem_jk_direct_part(basis.handle, C.c_void_p(_ptr(D)), C.c_void_p(_ptr(J)),
                                                   C.c_void_p(_ptr(K)), C.byref(o), int(part), int(nparts)))


def build_I(basis: Basis, device=False):
    n = basis.nbf
    if device:
        import torch

        out = torch.empty((n, n, n, n), dtype=torch.float64, device="cuda")
        _after_torch(basis, out)
    else:
        out = np.empty((n, n, n, n), dtype=np.float64)
    _lib.check(_lib.lib().rchem_build_I(basis.handle, C.c_void_p(_ptr(out)), _lib.DEVICE if device else _lib.HOST))
    return out


def build_I_packed(basis: Basis, device=False):
    """The ERI tensor in libpyquante2's 8-fold packed layout: a 1-D array with
    (ij|kl) at ijkl2intindex(i, j, k, l) (cints.c:375-387)."""
    n = basis.nbf
    npair = n * (n + 1) // 2
    length = npair * (npair + 1) // 2
    if device:
        import torch

        out = torch.empty(length, dtype=torch.float64, device="cuda")
        _after_torch(basis, out)
    else:
        out = np.empty(length, dtype=np.float64)
    _lib.check(_lib.lib().rchem_build_I_packed(basis.handle, C.c_void_p(_ptr(out)),
                                               _lib.DEVICE if device else _lib.HOST))
    return out


def ijkl2intindex(i, j, k, l):
    """cints.c:375-387: the packed position of (ij|kl)."""
    return int(_lib.lib().ijkl2intindex(int(i), int(j), int(k), int(l)))


def _jk_tensor_args(I, D, numel_of_n):
    """Checked (I, D, J, K, n, dev) for the tensor-based J/K entry points."""
    dev = _same_kind(I, D)
    if len(D.shape) != 2 or D.shape[0] != D.shape[1] or D.shape[0] < 1:
        raise ValueError("D must be a square matrix, got shape %s" % (tuple(D.shape),))
    n = int(D.shape[0])
    if dev:
        I, D = I.contiguous(), D.contiguous()
    else:
        I = np.ascontiguousarray(I, dtype=np.float64)
        D = np.ascontiguousarray(D, dtype=np.float64)
    _check_f64(D, "D", shape=(n, n))
    _check_f64(I, "I", numel=numel_of_n(n))
    if dev:
        import torch

        J = torch.empty((n, n), dtype=torch.float64, device=D.device)
        K = torch.empty_like(J)
    else:
        J, K = np.empty((n, n)), np.empty((n, n))
    return I, D, J, K, n, dev


def JK_packed(I, D):
    """J and K (JK_inmem's definitions) from the packed tensor of build_I_packed."""
    I, D, J, K, n, dev = _jk_tensor_args(I, D, lambda n: (n * (n + 1) // 2) * (n * (n + 1) // 2 + 1) // 2)
    _lib.check(_lib.lib().rchem_jk_packed(n, C.c_void_p(_ptr(I)), C.c_void_p(_ptr(D)), C.c_void_p(_ptr(J)),
                                          C.c_void_p(_ptr(K)), _lib.DEVICE if dev else _lib.HOST))
    return J, K


def JK_inmem(I, D):
    """J and K from the dense n^4 tensor of build_I (src/basis.rs:462-484)."""
    I, D, J, K, n, dev = _jk_tensor_args(I, D, lambda n: n ** 4)
    _lib.check(_lib.lib().rchem_jk_inmem(n, C.c_void_p(_ptr(I)), C.c_void_p(_ptr(D)), C.c_void_p(_ptr(J)),
                                         C.c_void_p(_ptr(K)), _lib.DEVICE if dev else _lib.HOST))
    return J, K
