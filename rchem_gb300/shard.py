"""Work of the hot path sharded over ranks, one process per GPU.

The batched workload (hundreds of independent molecules) has no exchange step:
quartets never couple two geometries.  Rank r takes a shard of the
geometries, runs the whole batched SCF and gradient for it on its own GPU (one
``BatchBasis`` per rank), and a single gather at the end returns every
geometry's result, in input order, on every rank.  Nothing is communicated
while the SCF runs, so the work per rank is fixed by its shard (weak scaling
as the batch grows with the ranks).

The partition balances the estimated cost of a geometry, n_g^4 for n_g basis
functions (the unscreened quartet count of its Fock builds), by
longest-processing-time-first assignment, which keeps every rank's load within
one geometry's cost of the lightest rank's.

The rank and world size come from ``torch.distributed`` when a process group
is initialised (NCCL on GPUs, gloo on CPUs; only the final gather uses it),
else the process is a world of one.  Each rank must have selected its own GPU
(``torch.cuda.set_device(local_rank)``) before creating handles.

One Fock build of a single large system shards instead by bra pairs
(``jk_sharded``): the library splits the bra shell pairs into one share per
rank of about equal cost (``rchem_jk_direct_part``, the same deterministic
split on every rank), each rank computes J and K from its share's quartets on
its GPU, and ``allreduce_sum`` adds them (2 n^2 doubles per build, the only
exchange).  ``shard`` applies the same longest-processing-time rule to any
other per-item costs.

The reference runs one molecule per process and has no distributed layer;
this is new capability around its energy conventions.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np

from .bse import expand_shells, load_bse


def geometry_cost(atomnos, basis_set) -> float:
    """Estimated Fock-build cost of one geometry: n^4, n its basis functions."""
    n = expand_shells(np.asarray(atomnos, dtype=np.int32).reshape(-1), load_bse(basis_set)).nbf
    return float(n) ** 4


def shard(costs: Sequence[float], world: int) -> list:
    """Partition item indices 0..len(costs)-1 into ``world`` shards:
    heaviest item first, each to the rank with the least load so far (ties
    to the lower rank; equal costs in index order).  Deterministic, so every
    rank computes the same partition without communicating.  Each shard is
    returned in ascending index order; ranks beyond the item count get an
    empty shard."""
    if world < 1:
        raise ValueError("world size must be >= 1, got %d" % world)
    c = np.asarray(costs, dtype=np.float64).reshape(-1)
    if c.size and (not np.all(np.isfinite(c)) or np.any(c < 0.0)):
        raise ValueError("costs must be finite and non-negative")
    order = sorted(range(c.size), key=lambda i: (-c[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += c[i]
    return [sorted(p) for p in parts]


class ShardError(RuntimeError):
    """A rank's share of a sharded computation failed (raised on every rank)."""


def _rank_world(group=None):
    try:
        import torch.distributed as dist
    except ImportError:
        return 0, 1
    if not (dist.is_available() and dist.is_initialized()):
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


def run_sharded(items: Sequence, costs: Sequence[float], compute: Callable[[list], list], group=None) -> list:
    """Run ``compute`` over this rank's shard of ``items`` and gather every
    item's result, in input order, on every rank.

    ``compute(list_of_items)`` returns one result per item, in order; results
    must be picklable (they travel through ``all_gather_object``).  A rank with
    an empty shard does not call ``compute``.

    A failure on one rank (``compute`` raising, or returning the wrong number
    of results) does not leave the others waiting: that rank still joins the
    gather, carrying its error, and every rank then raises ``ShardError``
    naming the failed ranks.  In a world of one the error propagates as it
    is."""
    if len(costs) != len(items):
        raise ValueError("%d costs for %d items" % (len(costs), len(items)))
    rank, world = _rank_world(group)
    mine = shard(costs, world)[rank]

    def run():
        local = list(compute([items[i] for i in mine])) if mine else []
        if len(local) != len(mine):
            raise ValueError("compute returned %d results for %d items" % (len(local), len(mine)))
        return local

    if world == 1:
        return run()
    import torch.distributed as dist

    try:
        local, err = run(), None
    except Exception as e:  # reported to every rank through the gather below
        local, err = [], "%s: %s" % (type(e).__name__, e)
    parts = [None] * world
    dist.all_gather_object(parts, (list(zip(mine, local)), err), group=group)
    failed = [(r, p[1]) for r, p in enumerate(parts) if p[1] is not None]
    if failed:
        raise ShardError("sharded compute failed on rank(s) " + "; ".join("%d (%s)" % f for f in failed))
    out = [None] * len(items)
    for part, _ in parts:
        for i, r in part:
            out[i] = r
    return out


def allreduce_sum(*arrays, group=None):
    """Sum each array over the ranks of the process group, in place on torch
    tensors (CPU tensors under gloo, CUDA tensors under NCCL); numpy arrays are
    summed through a tensor on the backend's device (the current CUDA device
    under NCCL, the CPU otherwise) and written back.  A world of one leaves
    them as they are.  Returns the arrays."""
    _, world = _rank_world(group)
    if world == 1:
        return arrays
    import torch
    import torch.distributed as dist

    on_gpu = str(dist.get_backend(group)).lower() == "nccl"
    for a in arrays:
        if isinstance(a, np.ndarray):
            t = torch.from_numpy(np.ascontiguousarray(a))
            if on_gpu:
                t = t.to(torch.device("cuda", torch.cuda.current_device()))
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
            a[...] = t.cpu().numpy()
        else:
            dist.all_reduce(a, op=dist.ReduceOp.SUM, group=group)
    return arrays


def rhf_gradient_sharded(geometries, basis_set_name="6-31g-fit", group=None, thresh_e=1e-10, thresh_d=1e-7,
                         max_iter=128, diis=8, fp32_tau=0.0, schwarz_tau=1e-12, emulated=False):
    """RHF energy and nuclear gradient of every geometry, sharded over the
    ranks of the process group: each rank builds one batch handle over its
    shard and runs the library's SCF loop (``rchem_rhf``, geometries of at
    most 64 basis functions) and the adjoint gradient kernels on its GPU.
    Returns, per geometry in input order, a dict with ``e_total``, ``e_elec``,
    ``e_nuc``, ``gradient`` (natoms x 3, hartree/bohr) and ``converged`` (that
    of its shard's SCF)."""
    from .batch import BatchBasis, gradient_batch, rhf_native

    costs = [geometry_cost(Z, basis_set_name) for Z, _ in geometries]

    def compute(local):
        bb = BatchBasis(local, basis_set_name)
        try:
            r = rhf_native(bb, thresh_e=thresh_e, thresh_d=thresh_d, max_iter=max_iter, diis=diis,
                           fp32_tau=fp32_tau, schwarz_tau=schwarz_tau, emulated=emulated)
            g = gradient_batch(bb, r, schwarz_tau=schwarz_tau, fp32_tau=fp32_tau, emulated=emulated)
        finally:
            bb.close()
        return [{"e_total": float(r["e_total"][k]), "e_elec": float(r["e_elec"][k]), "e_nuc": float(r["e_nuc"][k]),
                 "gradient": np.array(g[k]), "converged": bool(r["converged"])} for k in range(len(local))]

    return run_sharded(list(geometries), costs, compute, group)


def jk_sharded(basis, D, J, K, group=None, schwarz_tau=1e-12, fp32_tau=0.0, emulated=False):
    """One Fock build of ``basis`` split over the ranks of the process group:
    rank r computes J and K from share r of the bra shell pairs
    (``rchem_jk_direct_part``; every rank must hold the same basis and D),
    then one sum all-reduce of J and K gives every rank the whole build.
    Arrays as in ``JK_direct`` (host arrays: through the backend's device);
    a world of one is a plain build."""
    from .basis import JK_direct

    rank, world = _rank_world(group)
    JK_direct(J, K, basis, D, schwarz_tau=schwarz_tau, fp32_tau=fp32_tau, emulated=emulated, part=rank,
              nparts=world)
    allreduce_sum(J, K, group=group)
    return J, K
