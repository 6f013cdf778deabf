"""i-partition of a pairwise evaluation over ranks (one GPU per rank).

Each rank evaluates its contiguous slice of the i-set against the whole
j-set, which every rank holds; the per-particle outputs are then gathered.
The j-set is replicated, so the only exchange is the gather of the outputs
(none at all when each rank only needs its own slice, as in independent
replicas or cluster ensembles).
"""
import torch


def i_slice(n, rank, world):
    """Contiguous, balanced [start, stop) of the i-set for `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world: %d/%d" % (rank, world))
    return n * rank // world, n * (rank + 1) // world


def gather_rows(local, n, rank, world, group=None):
    """All-gather per-particle output rows (1-D tensors) into length-n tensors."""
    import torch.distributed as dist
    out = []
    size = max(i_slice(n, r, world)[1] - i_slice(n, r, world)[0] for r in range(world))
    for t in local:
        pad = torch.zeros(size, dtype=t.dtype, device=t.device)
        pad[:t.shape[0]] = t
        parts = [torch.empty_like(pad) for _ in range(world)]
        dist.all_gather(parts, pad, group=group)
        full = torch.cat([parts[r][:i_slice(n, r, world)[1] - i_slice(n, r, world)[0]]
                          for r in range(world)])
        out.append(full)
    return out


def sharded_calc(fn, iset, jset, rank, world, group=None):
    """Evaluate fn(i_subset, jset) -> list of 1-D tensors on this rank's slice
    of the i-set and gather the full outputs on every rank.  `iset` and
    `jset` map attribute names to 1-D tensors."""
    n = len(next(iter(iset.values())))
    a, b = i_slice(n, rank, world)
    local = fn({k: v[a:b] for k, v in iset.items()}, jset)
    return gather_rows(local, n, rank, world, group)
