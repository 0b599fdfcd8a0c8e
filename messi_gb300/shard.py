"""Work partitioning across GPUs, one process per GPU (host side only).

One alignment's likelihood does not split usefully across GPUs: its pair
pruning is a few hundred microseconds per tree level, and the inside pass is
a wavefront over dependent span diagonals.  What shards are independent
units, and nothing on the data path is exchanged between devices:

* the alignments of a batch.  ``plan_shards`` assigns every alignment to one
  rank (longest processing time first on ``alignment_cost``, an estimate of
  the pruning and inside work), each rank evaluates its alignments on its own
  GPU (one ``messi_batch_likelihood``), and ``gather_by_index`` returns the
  per-alignment results in batch order on every rank through one all-gather
  of small host objects;
* MCMC chains.  ``ReplicaExchange`` restates the tempered chains of
  src/MESSI.jl:1701-1775: chain k runs at B = bfactor**k, the tempered
  Metropolis-Hastings ratio multiplies the log-posterior difference by B
  (src/MCMC.jl:1666), and after every round of ``swap_every`` iterations
  there are as many swap attempts as chains, each between two chains drawn
  at random, accepted when exp(S) > u with
  S = (B_b - B_a) (ll_a + lp_a - ll_b - lp_b); an accepted swap exchanges the
  two chains' temperatures (and ids).  With one chain per rank only these
  scalars cross ranks; every rank draws the swap decisions from the same
  seeded generator, so all ranks agree without a further message.

``allgather`` arguments are callables mapping this rank's Python object to
the list of every rank's object (``torch.distributed.all_gather_object`` on
any backend; the identity for one process).
"""
import math
import time

import numpy as np


def torch_allgather():
    """all-gather of small host objects over the default process group (or
    the identity when there is none)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return lambda obj: [obj]

    def gather(obj):
        out = [None] * dist.get_world_size()
        dist.all_gather_object(out, obj)
        return out
    return gather


def band_pairs(L, W):
    """Pairs (x, y) with 0 < y - x <= W in an alignment of L columns."""
    W = max(0, min(int(W), L - 1))
    return W * L - W * (W + 1) // 2


def alignment_cost(numseqs, numcols, W):
    """Relative work of one likelihood evaluation: node updates of the pair
    pruning (pairs x internal nodes, before pattern compression) plus the
    split terms of the inside pass (about L W^2 / 2), weighted by their
    measured per-unit costs on one GPU (a split term costs about a fifth of a
    node update)."""
    W = max(0, min(int(W), numcols - 1))
    return band_pairs(numcols, W) * max(1, numseqs - 1) + 0.1 * numcols * W * W


def plan_shards(costs, world_size):
    """Indices per rank: longest processing time first (each unit, largest
    first, goes to the rank with the least work so far).  Deterministic, so
    every rank computes the same plan."""
    costs = np.asarray(costs, np.float64)
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = np.zeros(world_size)
    shards = [[] for _ in range(world_size)]
    for i in order:
        r = int(np.argmin(load))
        shards[r].append(i)
        load[r] += costs[i]
    return [sorted(s) for s in shards]


def gather_by_index(indices, values, n, allgather):
    """Results of every rank, back in unit order: `indices` are this rank's
    units, `values` their results."""
    parts = allgather((list(indices), list(values)))
    out = [None] * n
    seen = 0
    for idx, vals in parts:
        for i, v in zip(idx, vals):
            if out[i] is not None:
                raise RuntimeError(f"unit {i} was evaluated by more than one rank")
            out[i] = v
            seen += 1
    if seen != n:
        raise RuntimeError(f"{n - seen} units were not evaluated by any rank")
    return out


def evaluate_sharded(units, costs, evaluate, rank, world_size, allgather):
    """evaluate(list of this rank's units) -> their results; returns every
    unit's result in order, on every rank."""
    shards = plan_shards(costs, world_size)
    mine = shards[rank]
    vals = evaluate([units[i] for i in mine]) if mine else []
    return gather_by_index(mine, vals, len(units), allgather)


class ReplicaExchange:
    """Temperature ladder and swap rule of src/MESSI.jl:1701-1775."""

    def __init__(self, nchains, bfactor, seed=1):
        self.n = int(nchains)
        self.B = [float(bfactor) ** k for k in range(self.n)]   # Bs = bfactor^(z-1), z = 1..numchains
        self.ids = list(range(self.n))
        self.rng = np.random.default_rng(seed)
        self.accepted = np.zeros((self.n, self.n))
        self.attempted = np.zeros((self.n, self.n))

    def swap_round(self, ll, lp=None):
        """One round of swap attempts given every chain's current
        log-posterior ll[k] and paired log-prior lp[k] (chain k = slot k).
        Updates and returns self.B."""
        lp = [0.0] * self.n if lp is None else lp
        for _ in range(self.n):
            if self.n < 2:
                break
            sel = self.rng.permutation(self.n)
            a, b = int(sel[0]), int(sel[1])
            S = (self.B[b] - self.B[a]) * (ll[a] + lp[a] - ll[b] - lp[b])
            u = self.rng.random()
            if math.exp(min(S, 700.0)) > u:
                self.B[a], self.B[b] = self.B[b], self.B[a]
                self.ids[a], self.ids[b] = self.ids[b], self.ids[a]
                self.accepted[self.ids[a], self.ids[b]] += 1
                self.accepted[self.ids[b], self.ids[a]] += 1
            self.attempted[self.ids[a], self.ids[b]] += 1
            self.attempted[self.ids[b], self.ids[a]] += 1
        return self.B


def run_tempered(target, theta0, iterations, rank, world_size, allgather, bfactor=0.9, swap_every=10, seed=1,
                 proposal=None, record=None):
    """One tempered chain per rank, swapping temperatures every `swap_every`
    iterations.  target(theta) -> log-posterior; proposal.propose(rng, theta)
    -> (theta', log Hastings ratio) and proposal.observe(it, theta) (the
    plain move of ``mcmc.PlainProposal`` by default).  The acceptance is
    exp((ll' - ll) B + log Hastings) > u (src/MCMC.jl:1666).  Returns a dict
    with the states this rank held while its temperature was 1 (iteration,
    state), the temperature history of this rank and the swap statistics
    (equal on every rank)."""
    from . import mcmc
    rng = np.random.default_rng(seed * 1009 + rank)
    prop = proposal if proposal is not None else mcmc.PlainProposal()
    ladder = ReplicaExchange(world_size, bfactor, seed=seed)
    theta = np.asarray(theta0, np.float64)
    ll = target(theta)
    if not math.isfinite(ll):
        raise ValueError("starting point has zero posterior density")
    cold, temps, gathered = [], [], []
    accepted = 0
    t0 = time.perf_counter()
    for it in range(iterations):
        B = ladder.B[rank]
        theta_new, hastings = prop.propose(rng, theta)
        ll_new = target(theta_new) if mcmc.isvalid_theta(theta_new) else -math.inf
        if math.isfinite(ll_new) and math.exp(min((ll_new - ll) * B + hastings, 700.0)) > rng.random():
            theta, ll = theta_new, ll_new
            accepted += 1
        prop.observe(it, theta)
        if B == 1.0:
            cold.append((it, theta.copy()))
        temps.append(B)
        if (it + 1) % swap_every == 0:
            lls = allgather(ll)
            gathered.append(list(lls))
            ladder.swap_round(lls)
        if record is not None:
            record(it, theta, ll, B)
    return {"cold": cold, "temperatures": temps, "gathered_ll": gathered, "accept": accepted / max(1, iterations),
            "swap_accepted": ladder.accepted.tolist(), "swap_attempted": ladder.attempted.tolist(),
            "final_B": list(ladder.B), "seconds": time.perf_counter() - t0}
