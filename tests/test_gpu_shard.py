"""One Fock build split over bra-pair shares (rchem_jk_direct_part), on the GPU.

* one process: for 2 and 3 shares, the element-wise sum of every share's J
  and K is the whole build's to 1e-12, the shares' quartets add up to the
  whole build's, and no share is empty;
* two processes on cuda:0 joined by a gloo process group (the only GPU here):
  each computes its share with ``shard.jk_sharded`` and, after the one sum
  all-reduce, both hold the whole build.  The two processes' kernels never wait
  on each other; only the host-side all-reduce joins them.
"""
import os
import socket
import sys
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _problem():
    import rchem_gb300 as rc

    Z, R = rc.geometry.water_cluster(6, 7.0, seed=13)
    rng = np.random.default_rng(4)
    return Z, R, rng


def _density(rng, n):
    X = rng.normal(size=(n, n)) * 0.2
    return X @ X.T / n


@pytest.mark.parametrize("nparts", [2, 3])
def test_bra_shares_sum_to_whole_build(gpu, nparts):
    import rchem_gb300 as rc

    Z, R, rng = _problem()
    with rc.Basis(Z, R, "6-31gs-fit") as b:
        n = b.nbf
        D = _density(rng, n)
        J0, K0 = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J0, K0, b, D)
        q0 = b.stats()["quartets_fp64"]
        Js, Ks = np.zeros((n, n)), np.zeros((n, n))
        qs = []
        for part in range(nparts):
            J, K = np.zeros((n, n)), np.zeros((n, n))
            rc.JK_direct(J, K, b, D, part=part, nparts=nparts)
            qs.append(b.stats()["quartets_fp64"])
            assert np.abs(J - J.T).max() == 0.0
            Js += J
            Ks += K
        assert np.abs(Js - J0).max() < 1e-12 and np.abs(Ks - K0).max() < 1e-12
        assert sum(qs) == q0 and min(qs) > 0
        # the whole build again after the shares (the plan switches back)
        J1, K1 = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J1, K1, b, D)
        assert np.abs(J1 - J0).max() < 1e-12 and b.stats()["quartets_fp64"] == q0
        with pytest.raises(ValueError):
            rc.JK_direct(J1, K1, b, D, part=nparts, nparts=nparts)


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import rchem_gb300 as rc
    from rchem_gb300 import shard

    torch.cuda.set_device(0)
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        Z, R, rng = _problem()
        with rc.Basis(Z, R, "6-31gs-fit") as b:
            n = b.nbf
            D = _density(rng, n)
            J, K = np.zeros((n, n)), np.zeros((n, n))
            shard.jk_sharded(b, D, J, K)
            q = b.stats()["quartets_fp64"]
        np.savez(os.path.join(out_dir, "jk%d.npz" % rank), J=J, K=K, q=np.array([q]))
    finally:
        dist.destroy_process_group()


def test_jk_sharded_two_processes_gloo(gpu, tmp_path):
    import torch.multiprocessing as mp

    import rchem_gb300 as rc

    world = 2
    ctx = mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=False,
                             start_method="spawn")
    deadline = time.time() + 300
    while not ctx.join(timeout=5):
        if time.time() > deadline:
            for p in ctx.processes:
                p.kill()
            pytest.fail("ranks did not finish in 300 s")
    Z, R, rng = _problem()
    with rc.Basis(Z, R, "6-31gs-fit") as b:
        n = b.nbf
        D = _density(rng, n)
        J0, K0 = np.zeros((n, n)), np.zeros((n, n))
        rc.JK_direct(J0, K0, b, D)
        q0 = b.stats()["quartets_fp64"]
    qs = 0
    for r in range(world):
        z = np.load(os.path.join(tmp_path, "jk%d.npz" % r))
        assert np.abs(z["J"] - J0).max() < 1e-12 and np.abs(z["K"] - K0).max() < 1e-12
        qs += int(z["q"][0])
    assert qs == q0
