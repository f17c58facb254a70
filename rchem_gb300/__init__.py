"""rchem_gb300 -- GB300-native (sm_103a) RHF hot path of berquist/rchem.

The compute lives in librchem_gpu.so (hand-written CUDA, C ABI in include/);
this package is the host-side mirror of the reference's basis API
(src/basis.rs) plus input readers.  Importing it loads the shared library
lazily; every compute call fails loudly if the library is not built.
"""
from . import geometry
from ._lib import RchemError
from .basis import JK_direct, JK_inmem, JK_packed, S, T, V, Basis, build_I, build_I_packed, ijkl2intindex, moment
from .bse import available_basis_sets, expand_shells, load_bse, read_xyz
from . import batch, cints, scf, shard

__all__ = [
    "Basis", "S", "T", "V", "JK_direct", "build_I", "JK_inmem", "build_I_packed", "JK_packed", "ijkl2intindex",
    "moment", "RchemError", "load_bse",
    "expand_shells", "read_xyz", "available_basis_sets", "geometry", "cints", "scf", "batch", "shard",
]
