"""Ensembles of independent runs spread over the GPUs of one node, one rank per GPU.

The runs share nothing, so sharding them needs no exchange on the data path: each rank builds
an Ensemble of its own share and advances it; only the per-run results are gathered on the
host at the end (torch.distributed over any backend, gloo included).  The reference has no
such mode: its batch driver (dns.f90:70-101) runs the parameter sets one after another.

Shares are balanced by cost with the longest-processing-time rule: runs in decreasing cost
(ties by index), each to the rank with the least cost so far (ties by rank).  The cost of a
run is one step's work, nx ny log2(nx ny) for the transforms plus ns for the beam."""
import math


def run_cost(p):
    """One step of run p: the 2D transforms' nx ny log2(nx ny), plus the beam's ns."""
    n = p.nx * p.ny
    return n * math.log2(n) + p.ns


def partition(params_list, world):
    """The runs of each rank (lists of indices into params_list, each list ascending); the
    same on every rank for the same input."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(params_list)), key=lambda i: (-run_cost(params_list[i]), i))
    load = [0.0] * world
    share = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        share[r].append(i)
        load[r] += run_cost(params_list[i])
    return [sorted(s) for s in share]


def gather_by_index(local, share, world, total):
    """Per-run results in global order: `local` holds this rank's results in the order of
    its share; every rank receives the full list (torch.distributed.all_gather_object)."""
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, (share, list(local)))
    out = [None] * total
    for idx, vals in parts:
        for i, v in zip(idx, vals):
            out[i] = v
    return out


class ShardedEnsemble:
    """This rank's share of an ensemble (fsibe_2d_gb300.Ensemble on the rank's GPU)."""

    def __init__(self, params_list, rank, world):
        from . import Ensemble
        self.total = len(params_list)
        self.rank, self.world = rank, world
        self.share = partition(params_list, world)[rank]
        self.params = [params_list[i] for i in self.share]
        self.ens = Ensemble(self.params) if self.params else None

    @property
    def runs(self):
        return self.ens.runs if self.ens else []

    def init_fields(self, vort_of_index):
        """vort_of_index(i): the initial vorticity of global run i."""
        for i, r in zip(self.share, self.runs):
            r.init_fields(vort_of_index(i))

    def step(self, nsteps=1):
        if self.ens:
            self.ens.step(nsteps)

    def gather(self, fn):
        """fn(run) of every run of the ensemble, in global order, on every rank."""
        return gather_by_index([fn(r) for r in self.runs], self.share, self.world, self.total)

    def close(self):
        if self.ens:
            self.ens.close()
            self.ens = None
