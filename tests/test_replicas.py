"""Replicas on CPU.  Photon split: two gloo ranks each simulate their
disjoint photon range with the oracle; the all-reduced sum of their outputs
equals the single-process run over all photons.  A rank that fails before the
reduce is reported to the others through the store instead of hanging them.
Batch mode: the configurations of a sweep are partitioned across ranks by
budget (xmimsim_gb300.replicas); the gathered per-configuration outputs equal
the single-process runs."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _spec():
    from xmimsim_gb300 import configs
    return configs.config1(n_photons_line=3001)


def _run(replica, n_replicas, spec=None):
    from oracle import oracle_api as O
    from xmimsim_gb300 import Simulation, configs, gpu_options
    spec = _spec() if spec is None else spec
    sim = Simulation(spec, options=configs.C1_OPTIONS, gpu=gpu_options(seed=7))
    r, t = sim.grid_axes(32, 32)
    sim.set_solid_angle(r, t, np.zeros((32, 32)))
    sim.prepare()
    g = O.solid_angle_points(sim.bundle_ptr(), r, t, 0, 32 * 32, 400).reshape(32, 32)
    sim.set_solid_angle(r, t, g)
    sim.set_replica(replica, n_replicas)
    sim.prepare()
    out = O.msim(sim.bundle_ptr(), spec.n_interactions_trajectory, spec.nchannels, threads=1)
    sim.close()
    return out


def _worker(rank, world, port, fail_rank, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch
    import torch.distributed as dist
    from datetime import timedelta
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=30))
    store = dist.distributed_c10d._get_default_store()
    try:
        if rank == fail_rank:
            raise RuntimeError("injected failure before the reduce")
        out = _run(rank, world)
        store.set(f"ok{rank}", "1")
        # wait for every rank to report before the collective (host-side failure detection)
        for r in range(world):
            store.wait([f"ok{r}"] if r != fail_rank else [f"failed{r}"], timedelta(seconds=20))
        if any(store.check([f"failed{r}"]) for r in range(world)):
            q.put((rank, "peer failed"))
            return
        t = torch.tensor(np.concatenate([out["channels"].ravel(), out["var_red"].ravel()]))
        dist.all_reduce(t)
        q.put((rank, t.numpy()))
    except Exception as e:
        store.set(f"failed{rank}", "1")
        q.put((rank, "error: %s" % e))
    finally:
        dist.destroy_process_group()


def _spawn(world, fail_rank=-1):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, fail_rank, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get() for _ in procs)
    for p in procs:
        p.join(60)
    return res


def test_replica_ranges_are_disjoint_and_complete():
    full = _run(0, 1)
    parts = [_run(r, 3) for r in range(3)]
    np.testing.assert_allclose(sum(p["var_red"] for p in parts), full["var_red"], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(sum(p["channels"] for p in parts), full["channels"], rtol=1e-12, atol=1e-300)


def test_two_gloo_ranks_reduce_to_single_run():
    pytest.importorskip("torch")
    res = _spawn(2)
    full = _run(0, 1)
    ref = np.concatenate([full["channels"].ravel(), full["var_red"].ravel()])
    for r in range(2):
        assert not isinstance(res[r], str), res[r]
        np.testing.assert_allclose(res[r], ref, rtol=1e-12, atol=1e-300)


def test_failed_rank_is_detected_without_hanging():
    pytest.importorskip("torch")
    res = _spawn(2, fail_rank=1)
    assert res[1].startswith("error")
    assert res[0] == "peer failed"


def _sweep():
    from xmimsim_gb300 import configs
    return [configs.config1(n_photons_line=n) for n in (900, 2500, 1200, 3100, 700)]


def _flat(out):
    return np.concatenate([out["channels"].ravel(), out["var_red"].ravel()])


def _partition_worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    from datetime import timedelta
    from xmimsim_gb300.replicas import gather_by_config, partition_by_budget, photon_budget, rank_share
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=30))
    try:
        specs = _sweep()
        mine = rank_share(specs, rank, world)
        res = [_flat(_run(0, 1, specs[i])) for i in mine]
        gathered = [None] * world
        dist.all_gather_object(gathered, res)
        parts = partition_by_budget([photon_budget(s) for s in specs], world)
        q.put((rank, (mine, gather_by_config(parts, gathered, len(specs)))))
    except Exception as e:
        q.put((rank, "error: %s" % e))
    finally:
        dist.destroy_process_group()


def test_partition_by_budget_covers_and_balances():
    from xmimsim_gb300.replicas import gather_by_config, partition_by_budget
    rng = np.random.default_rng(3)
    for n_ranks in (1, 2, 3, 8):
        budgets = (10 ** rng.uniform(6, 8, 512)).astype(np.int64)
        parts = partition_by_budget(budgets, n_ranks)
        assert sorted(i for p in parts for i in p) == list(range(len(budgets)))
        assert all(p == sorted(p) for p in parts)
        loads = [int(budgets[p].sum()) for p in parts]
        assert max(loads) <= 4 / 3 * max(budgets.sum() / n_ranks, budgets.max())
        assert parts == partition_by_budget([int(b) for b in budgets], n_ranks)  # no communication needed
        assert gather_by_config(parts, [[("cfg", i) for i in p] for p in parts], len(budgets)) == \
            [("cfg", i) for i in range(len(budgets))]
    assert partition_by_budget([5, 3], 4) == [[0], [1], [], []]
    assert partition_by_budget([], 2) == [[], []]
    with pytest.raises(ValueError):
        gather_by_config([[0], [0]], [["a"], ["b"]], 1)
    with pytest.raises(ValueError):
        gather_by_config([[0], []], [["a"], []], 2)


def test_two_gloo_ranks_partition_a_sweep():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_partition_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get() for _ in procs)
    for p in procs:
        p.join(60)
    single = [_flat(_run(0, 1, s)) for s in _sweep()]
    assert not isinstance(res[0], str), res[0]
    assert not isinstance(res[1], str), res[1]
    # each configuration ran on one rank, and both shares are non-empty
    assert sorted(res[0][0] + res[1][0]) == list(range(len(single))) and res[0][0] and res[1][0]
    for r in range(2):
        for got, want in zip(res[r][1], single):
            np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-300)
