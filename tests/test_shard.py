"""Sharding a batch of geometries over ranks (rchem_gb300/shard.py), on CPU.

The partition is checked for its properties; the gather is run with two
gloo ranks in child processes, each computing its shard's RHF energies with
the oracle's CPU SCF (the GPU path runs the same host logic with the
library's batched SCF in place of the oracle)."""
import os
import socket
import sys
import time

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shard_partition_properties():
    from rchem_gb300.shard import shard

    rng = np.random.default_rng(0)
    for n in (0, 1, 5, 37):
        costs = rng.integers(1, 100, n).astype(float) ** 2
        for world in (1, 2, 3, 5, 8):
            parts = shard(costs, world)
            assert len(parts) == world
            flat = sorted(i for p in parts for i in p)
            assert flat == list(range(n))  # a disjoint cover
            assert all(p == sorted(p) for p in parts)
            loads = [float(np.sum(costs[p])) for p in parts]
            if n:
                # longest-processing-time-first: no rank is more than one item above the lightest
                assert max(loads) - min(loads) <= costs.max()
            if world > n:
                assert sum(1 for p in parts if not p) >= world - n
            assert shard(costs, world) == parts  # deterministic
    assert shard([4, 4, 4, 4], 2) == [[0, 2], [1, 3]]
    assert shard([9, 1, 1, 1, 1, 1, 1, 1, 1, 1], 2) == [[0], list(range(1, 10))]
    with pytest.raises(ValueError):
        shard([1.0], 0)
    with pytest.raises(ValueError):
        shard([1.0, np.nan], 2)


def test_geometry_cost_and_single_rank():
    import rchem_gb300 as rc
    from rchem_gb300.shard import geometry_cost, run_sharded

    Z, _ = rc.geometry.water_monomer()
    assert geometry_cost(Z, "6-31g-fit") == 13.0 ** 4
    assert geometry_cost(np.concatenate([Z, Z]), "sto-3g-fit") == 14.0 ** 4
    # no process group: a world of one computes everything, in order
    assert run_sharded([3, 1, 2], [1, 1, 1], lambda xs: [x * 10 for x in xs]) == [30, 10, 20]
    with pytest.raises(ValueError, match="2 results for 3 items"):
        run_sharded([3, 1, 2], [1, 1, 1], lambda xs: xs[:2])
    with pytest.raises(ValueError, match="2 costs for 3 items"):
        run_sharded([3, 1, 2], [1, 1], lambda xs: xs)


def _geometries():
    import rchem_gb300 as rc

    return rc.geometry.water_batch(5, seed=11)  # monomers, dimers and a trimer: uneven costs


def _oracle_energies(geoms):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    import rchem_gb300 as rc

    O.port().set_boys(True)
    doc = rc.load_bse("sto-3g-fit")
    out = []
    for Z, R in geoms:
        b = O.expand_basis(Z, R, doc)
        r = O.rhf(b, Z, R, int(np.sum(Z)) // 2, thresh_e=1e-10)
        out.append((os.getpid(), r["e_elec"] + r["e_nuc"]))
    return out


def _gloo_worker(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    from rchem_gb300.shard import geometry_cost, run_sharded

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        geoms = _geometries()
        costs = [geometry_cost(Z, "sto-3g-fit") for Z, _ in geoms]
        res = run_sharded(geoms, costs, _oracle_energies)
        np.save(os.path.join(out_dir, "rank%d.npy" % rank),
                np.array([[pid, e] for pid, e in res] + [[os.getpid(), 0.0]]))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_batch_over_two_gloo_ranks(tmp_path):
    """Two gloo ranks: each computes only its shard, and after the gather both
    hold every geometry's energy, in input order, equal to a serial run."""
    import torch.multiprocessing as mp

    from rchem_gb300.shard import geometry_cost, shard

    world = 2
    ctx = mp.start_processes(_gloo_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=False,
                             start_method="spawn")
    deadline = time.time() + 300
    while not ctx.join(timeout=5):
        if time.time() > deadline:
            for p in ctx.processes:
                p.kill()
            pytest.fail("gloo ranks did not finish in 300 s")
    geoms = _geometries()
    serial = np.array([e for _, e in _oracle_energies(geoms)])
    parts = shard([geometry_cost(Z, "sto-3g-fit") for Z, _ in geoms], world)
    assert all(parts)  # both ranks had work
    res = [np.load(os.path.join(tmp_path, "rank%d.npy" % r)) for r in range(world)]
    pids = [int(x[-1, 0]) for x in res]
    for r in range(world):
        got = res[r][:-1]
        np.testing.assert_allclose(got[:, 1], serial, atol=1e-10, rtol=0)  # every energy on every rank
        for k in range(world):
            # geometry i was computed by the rank whose shard holds it, and only there
            assert all(int(got[i, 0]) == pids[k] for i in parts[k])


def test_rhf_gradient_sharded_plumbing(monkeypatch):
    """rhf_gradient_sharded hands each shard to one batch handle, the
    library's SCF and the gradient kernels, closes the handle, and returns one
    record per geometry in input order (here with stand-ins for the three GPU
    calls, which have their own GPU tests)."""
    from rchem_gb300 import batch, shard

    geoms = _geometries()
    made, closed = [], []

    class FakeBatch:
        def __init__(self, local, name):
            self.local = local
            made.append((len(local), name))

        def close(self):
            closed.append(True)

    def fake_rhf(bb, **kw):
        e = np.array([float(len(Z)) for Z, _ in bb.local])
        return {"e_total": e - 1.0, "e_elec": e - 2.0, "e_nuc": np.ones_like(e), "converged": True, "kw": kw}

    def fake_grad(bb, r, **kw):
        return [np.full((len(Z), 3), float(len(Z))) for Z, _ in bb.local]

    monkeypatch.setattr(batch, "BatchBasis", FakeBatch)
    monkeypatch.setattr(batch, "rhf_native", fake_rhf)
    monkeypatch.setattr(batch, "gradient_batch", fake_grad)
    res = shard.rhf_gradient_sharded(geoms, "sto-3g-fit", fp32_tau=1e-6)
    assert made == [(len(geoms), "sto-3g-fit")] and closed == [True]
    assert len(res) == len(geoms)
    for (Z, _), r in zip(geoms, res):
        assert r["e_total"] == len(Z) - 1.0 and r["e_elec"] == len(Z) - 2.0 and r["e_nuc"] == 1.0
        assert r["gradient"].shape == (len(Z), 3) and r["converged"] is True


def _jk_worker(rank, world, port, out_dir):
    """One rank of a single-system Fock build sharded by bra pairs."""
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist

    import oracle as O

    from rchem_gb300.shard import allreduce_sum, shard

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        b, D, Q, costs = _jk_problem(O)
        mine = shard(costs, world)[rank]
        J, K, cnt = O.JK_sym_screened(b, D, Q, 1e-12, pairs=mine)
        c = np.array([float(cnt)])
        allreduce_sum(J, K, c)
        np.savez(os.path.join(out_dir, "jk%d.npz" % rank), J=J, K=K, c=c, mine=np.array(mine))
    finally:
        dist.destroy_process_group()


def _jk_problem(O):
    import rchem_gb300 as rc

    O.port().set_boys(True)
    Z, R = rc.geometry.water_cluster(3, 5.0, seed=5)
    b = O.expand_basis(Z, R, rc.load_bse("6-31g-fit"))
    rng = np.random.default_rng(2)
    X = rng.normal(size=(b.n, b.n))
    D = X @ X.T / b.n
    Q = O.schwarz(b)
    # per bra pair ij: the kets kl <= ij that pass the screen
    costs = np.array([np.count_nonzero(Q[: ij + 1] * Q[ij] >= 1e-12) for ij in range(Q.size)], dtype=float)
    return b, D, Q, costs


def test_fock_build_sharded_by_bra_pairs_over_two_gloo_ranks(tmp_path):
    """A single system's J and K: bra pairs sharded by their screened ket
    counts, partial J/K per rank, one sum all-reduce -- equal on both ranks
    to the whole build, with the integral count split near evenly."""
    import torch.multiprocessing as mp

    from rchem_gb300.shard import shard

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    world = 2
    ctx = mp.start_processes(_jk_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=False,
                             start_method="spawn")
    deadline = time.time() + 300
    while not ctx.join(timeout=5):
        if time.time() > deadline:
            for p in ctx.processes:
                p.kill()
            pytest.fail("gloo ranks did not finish in 300 s")
    b, D, Q, costs = _jk_problem(O)
    J0, K0, c0 = O.JK_sym_screened(b, D, Q, 1e-12)
    loads = []
    for r in range(world):
        z = np.load(os.path.join(tmp_path, "jk%d.npz" % r))
        np.testing.assert_allclose(z["J"], J0, atol=1e-12, rtol=0)
        np.testing.assert_allclose(z["K"], K0, atol=1e-12, rtol=0)
        assert int(z["c"][0]) == c0
        loads.append(costs[z["mine"]].sum())
    assert sum(loads) == c0 and max(loads) - min(loads) <= costs.max()


def _failing_compute(rank):
    def compute(local):
        if rank == 1:
            raise RuntimeError("injected failure on rank 1")
        return [0.0 for _ in local]

    return compute


def _fail_worker(rank, world, port, out_dir):
    """Rank 1's share raises; both ranks must end with ShardError, not wait."""
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    from rchem_gb300.shard import ShardError, run_sharded

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        run_sharded(list(range(6)), [1.0] * 6, _failing_compute(rank))
        msg = "no error"
    except ShardError as e:
        msg = "ShardError: %s" % e
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out_dir, "fail%d.txt" % rank), "w") as f:
        f.write(msg)


def test_rank_failure_reported_on_every_rank(tmp_path):
    """A failure injected on the host in one rank's share (its compute raises)
    reaches every rank as ShardError naming that rank; no rank waits for it."""
    import torch.multiprocessing as mp

    world = 2
    t0 = time.time()
    ctx = mp.start_processes(_fail_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=False,
                             start_method="spawn")
    deadline = time.time() + 120
    while not ctx.join(timeout=5):
        if time.time() > deadline:
            for p in ctx.processes:
                p.kill()
            pytest.fail("ranks did not finish in 120 s")
    for r in range(world):
        msg = open(os.path.join(tmp_path, "fail%d.txt" % r)).read()
        assert msg.startswith("ShardError") and "rank(s) 1 (RuntimeError: injected failure on rank 1)" in msg, msg
    assert time.time() - t0 < 60
