"""ctypes binding of librchem_gpu.so (include/rchem_gpu.h, include/rchem_cints.h).

There is no CPU fallback: if the shared library is missing or fails to load,
importing this module raises, naming the build step.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librchem_gpu.so")

RCHEM_OK, RCHEM_ERR_INVALID, RCHEM_ERR_UNSUPPORTED, RCHEM_ERR_CUDA, RCHEM_ERR_NOMEM = range(5)
HOST, DEVICE = 0, 1


class RchemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("rchem error %d: %s" % (code, msg))
        self.code = code


class JKOpts(C.Structure):
    _fields_ = [("schwarz_tau", C.c_double), ("fp32_tau", C.c_double), ("where", C.c_int), ("emulated", C.c_int)]


class JKStats(C.Structure):
    _fields_ = [
        ("quartets_fp64", C.c_longlong), ("quartets_fp32", C.c_longlong),
        ("prim_quartets_fp64", C.c_longlong), ("prim_quartets_fp32", C.c_longlong),
        ("eris_fp64", C.c_longlong), ("eris_fp32", C.c_longlong),
        ("flops_fp64", C.c_double), ("flops_fp32", C.c_double),
        ("warp_tasks", C.c_longlong), ("kernels", C.c_int), ("reserved", C.c_int), ("gpu_ms", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class SCFOpts(C.Structure):
    _fields_ = [("thresh_e", C.c_double), ("thresh_d", C.c_double), ("max_iter", C.c_int), ("diis", C.c_int),
                ("jk", JKOpts)]


class Prim(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("norm", C.c_double), ("alpha", C.c_double),
                ("l", C.c_int), ("m", C.c_int), ("n", C.c_int), ("pad", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "librchem_gpu.so is not built (expected at %s); build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or `python -m rchem_gb300.build`" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    d, i, p, vp = C.c_double, C.c_int, C.POINTER, C.c_void_p
    L.rchem_last_error.restype = C.c_char_p
    L.rchem_abi_version.restype = i
    L.rchem_basis_create.argtypes = [p(vp), i, vp, vp, i, vp, vp, vp, vp, vp]
    L.rchem_basis_destroy.argtypes = [vp]
    L.rchem_batch_create.argtypes = [p(vp), i, vp, i, vp, vp, i, vp, vp, vp, vp, vp]
    L.rchem_basis_layout.argtypes = [vp, vp, vp, vp, vp]
    L.rchem_basis_nbf.argtypes = [vp]
    L.rchem_basis_set_stream.argtypes = [vp, vp]
    for f in ("rchem_S", "rchem_T", "rchem_V"):
        getattr(L, f).argtypes = [vp, vp, i]
    L.rchem_moment.argtypes = [vp, vp, i, i, i, vp, i]
    L.rchem_jk_direct.argtypes = [vp, vp, vp, vp, p(JKOpts)]
    L.rchem_jk_direct_noalloc.argtypes = [vp, vp, vp, vp, p(JKOpts)]
    L.rchem_jk_direct_part.argtypes = [vp, vp, vp, vp, p(JKOpts), i, i]
    L.rchem_gradient.argtypes = [vp, vp, vp, vp, p(JKOpts)]
    L.rchem_autotune.argtypes = [vp, p(JKOpts), vp]
    L.rchem_eigh_batched.argtypes = [i, i, vp, vp, vp, vp]
    L.rchem_set_tile_shape.argtypes = [vp, i, i, i]
    L.rchem_set_exponent_table.argtypes = [vp, i]
    L.rchem_rhf.argtypes = [vp, p(SCFOpts), vp, vp, vp, vp, vp, vp, vp]
    L.rchem_jk_class_stats.argtypes = [vp, vp, vp, vp, vp]
    L.rchem_jk_list_times.argtypes = [vp, p(JKOpts), vp]
    L.rchem_jk_stats_get.argtypes = [vp, p(JKStats)]
    L.rchem_build_I.argtypes = [vp, vp, i]
    L.rchem_jk_inmem.argtypes = [i, vp, vp, vp, vp, i]
    L.rchem_build_I_packed.argtypes = [vp, vp, i]
    L.rchem_jk_packed.argtypes = [i, vp, vp, vp, vp, i]
    L.ijkl2intindex.argtypes = [i, i, i, i]
    L.ijkl2intindex.restype = i
    L.rchem_eri_prim_batch.argtypes = [i, vp, vp, i]
    L.rchem_onee_prim_batch.argtypes = [i, i, vp, vp, vp, i]
    L.rchem_boys_batch.argtypes = [i, vp, vp, vp, i, i]
    L.coulomb_repulsion.argtypes = [d, d, d, d, i, i, i, d] * 4
    L.coulomb_repulsion.restype = d
    for f in ("overlap", "kinetic"):
        getattr(L, f).argtypes = [d, i, i, i, d, d, d] * 2
        getattr(L, f).restype = d
    L.nuclear_attraction.argtypes = [d, d, d, d, i, i, i, d] * 2 + [d, d, d]
    L.nuclear_attraction.restype = d
    L.Fgamma.argtypes = [d, d]
    L.Fgamma.restype = d
    L.contr_coulomb.argtypes = ([i, vp, vp, vp, d, d, d, i, i, i]) * 4
    L.contr_coulomb.restype = d
    L.rchem_peak_fma.argtypes = [i, p(d)]
    _lib = L
    return L


def check(rc: int):
    if rc != RCHEM_OK:
        raise RchemError(rc, lib().rchem_last_error().decode(errors="replace"))


def exported_symbols():
    """Names every header in include/ declares (for the symbol check)."""
    return [
        "rchem_last_error", "rchem_abi_version", "rchem_basis_create", "rchem_basis_destroy", "rchem_basis_nbf",
        "rchem_basis_set_stream", "rchem_S", "rchem_T", "rchem_V", "rchem_moment", "rchem_jk_direct",
        "rchem_jk_stats_get", "rchem_build_I", "rchem_jk_inmem", "rchem_build_I_packed", "rchem_jk_packed", "ijkl2intindex", "coulomb_repulsion", "overlap", "kinetic",
        "nuclear_attraction", "Fgamma", "contr_coulomb", "rchem_eri_prim_batch", "rchem_onee_prim_batch",
        "rchem_boys_batch", "rchem_peak_fma", "rchem_jk_direct_noalloc", "rchem_gradient", "rchem_batch_create",
        "rchem_basis_layout", "rchem_autotune", "rchem_jk_class_stats", "rchem_jk_list_times", "rchem_jk_direct_part", "rchem_eigh_batched",
        "rchem_set_tile_shape", "rchem_set_exponent_table", "rchem_rhf",
    ]
