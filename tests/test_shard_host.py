"""Multi-GPU partitioning on the host (messi_gb300.shard), exercised with
gloo ranks on the CPU (world size 2) and a stub likelihood: no GPU.

* alignments of a batch: every alignment is evaluated by exactly one rank,
  the load is balanced, and the gathered results equal a one-process run;
* replica exchange (src/MESSI.jl:1701-1775): the temperatures held by the
  ranks stay a permutation of the ladder, every rank takes the same swap
  decisions, those decisions are the reference's rule replayed from the
  gathered log-posteriors, and the B = 1 chain samples its target.
"""
import json
import math
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _units(n, seed=5):
    rng = np.random.default_rng(seed)
    L = rng.integers(80, 1500, n)
    N = rng.integers(8, 128, n)
    return [(int(a), int(b)) for a, b in zip(N, L)]


def _stub_Z(unit):
    """A stand-in for one alignment's log marginal likelihood."""
    N, L = unit
    return -float(L) * math.log(4.0) * (1.0 + 0.01 * N)


MU = np.array([1.0, 2.0, 0.5, 1.5, 3.0, 1.0, 1.2, 0.5, 2.0, 3.0, 1.5])
SD = np.array([0.1, 0.2, 0.05, 0.1, 0.3, 0.1, 0.1, 0.05, 0.2, 0.3, 0.1])


def _gauss(theta):
    from messi_gb300 import mcmc
    if not mcmc.isvalid_theta(theta):
        return -math.inf
    return float(-0.5 * np.sum(((np.asarray(theta) - MU) / SD) ** 2))


def _worker(rank, ws, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    from messi_gb300 import shard
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ag = shard.torch_allgather()
    units = _units(37)
    costs = [shard.alignment_cost(N, L, L - 1) for N, L in units]
    evaluated = []

    def evaluate(batch):
        evaluated.extend(batch)
        return [_stub_Z(u) for u in batch]
    Z = shard.evaluate_sharded(units, costs, evaluate, rank, ws, ag)
    res = shard.run_tempered(_gauss, MU.copy(), 3000, rank, ws, ag, bfactor=0.5, swap_every=10, seed=3)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(outdir, f"r{rank}.json"), "w") as f:
        json.dump({"Z": Z, "evaluated": evaluated, "temperatures": res["temperatures"],
                   "gathered": res["gathered_ll"], "final_B": res["final_B"],
                   "cold": [[it, th.tolist()] for it, th in res["cold"]],
                   "swap_accepted": res["swap_accepted"], "swap_attempted": res["swap_attempted"]}, f)


@pytest.fixture(scope="module")
def two_ranks(tmp_path_factory):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = tmp_path_factory.mktemp("shard")
    ws = 2
    mp.start_processes(_worker, args=(ws, _free_port(), str(out)), nprocs=ws, join=True, start_method="spawn")
    return [json.load(open(out / f"r{r}.json")) for r in range(ws)]


def test_every_alignment_evaluated_once_and_gathered_in_order(two_ranks):
    units = _units(37)
    done = [tuple(u) for r in two_ranks for u in r["evaluated"]]
    assert sorted(done) == sorted(units) and len(done) == len(units)
    single = [_stub_Z(u) for u in units]
    for r in two_ranks:
        assert r["Z"] == single


def test_shards_are_balanced():
    sys.path.insert(0, ROOT)
    from messi_gb300 import shard
    units = _units(256, seed=1)
    costs = [shard.alignment_cost(N, L, L - 1) for N, L in units]
    for ws in (2, 4, 8):
        plan = shard.plan_shards(costs, ws)
        assert sorted(i for s in plan for i in s) == list(range(256))
        loads = [sum(costs[i] for i in s) for s in plan]
        assert max(loads) <= 1.02 * sum(costs) / ws + max(costs)


def test_replica_exchange_rule_and_agreement(two_ranks):
    sys.path.insert(0, ROOT)
    from messi_gb300 import shard
    r0, r1 = two_ranks
    # the ranks hold a permutation of the ladder at every iteration
    for b0, b1 in zip(r0["temperatures"], r1["temperatures"]):
        assert sorted([b0, b1]) == [0.5, 1.0]
    # both ranks saw the same gathered values and took the same decisions
    assert r0["gathered"] == r1["gathered"] and r0["final_B"] == r1["final_B"]
    # replaying the reference's rule on the gathered log-posteriors gives the
    # temperature history the ranks ran with
    ladder = shard.ReplicaExchange(2, 0.5, seed=3)
    hist = []
    for lls in r0["gathered"]:
        hist.append(list(ladder.swap_round(lls)))
    for k, B in enumerate(hist[:-1]):
        it = (k + 1) * 10  # first iteration after swap round k
        assert [r0["temperatures"][it], r1["temperatures"][it]] == B
    acc = np.array(r0["swap_accepted"]).sum() / 2
    att = np.array(r0["swap_attempted"]).sum() / 2
    assert 0 < acc < att


def test_swap_acceptance_formula():
    sys.path.insert(0, ROOT)
    from messi_gb300 import shard
    # S = (B_b - B_a)(ll_a - ll_b): moving the better state to the colder
    # chain is always accepted
    rx = shard.ReplicaExchange(2, 0.25, seed=0)
    B = rx.swap_round([-100.0, -10.0])  # chain 1 (B = 0.25) is better: S > 0 for the pair
    assert B == [0.25, 1.0]
    # a much worse state is (almost) never moved to the colder chain
    rx = shard.ReplicaExchange(2, 0.25, seed=0)
    B = rx.swap_round([-10.0, -1e4])
    assert B == [1.0, 0.25]


def test_cold_chain_samples_its_target(two_ranks):
    cold = sorted((it, th) for r in two_ranks for it, th in r["cold"])
    its = [it for it, _ in cold]
    assert its == list(range(3000))  # exactly one rank holds B = 1 at each iteration
    X = np.array([th for _, th in cold[1000:]])
    z = np.abs(X.mean(axis=0) - MU) / SD
    assert np.all(z < 1.0)
