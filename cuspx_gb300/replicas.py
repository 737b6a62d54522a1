"""Multi-GPU replicas: requests partition by key, with no exchange step.

A key's resident state (its table row, its midstate) lives on exactly one
GPU, so every request for that key is routed there; no rank ever needs
another rank's data, so there is no collective on the data path.  The only
communication is the host-side gather of results for reporting.

    owner = owner_of(key_id, world)          # which rank serves a key
    mine = shard_by_key(key_ids, rank, world) # request indices this rank runs
    merged = merge(world_results, n)          # back into request order
"""


def owner_of(key_id, world):
    return int(key_id) % world


def shard_by_key(key_ids, rank, world):
    """Indices of the requests whose key rank `rank` owns."""
    return [i for i, k in enumerate(key_ids) if owner_of(k, world) == rank]


def merge(per_rank, n):
    """per_rank: list over ranks of [(index, value), ...] -> values in request order."""
    out = [None] * n
    for part in per_rank:
        for i, v in part:
            if out[i] is not None:
                raise ValueError("request %d served twice" % i)
            out[i] = v
    if any(v is None for v in out):
        raise ValueError("some requests were not served")
    return out
