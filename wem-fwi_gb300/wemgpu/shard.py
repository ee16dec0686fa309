"""Shot sharding across ranks (one process per GPU).

(shot, frequency) rows are independent (propagator/src/wem_prop.cpp:11-12);
the reference shards shots over Dask workers by rewriting ``ns``/``osx`` of
each block (propagator/src/python/WEM.py:24-30).  Here every rank builds the
operators of its contiguous block of shots; data stay sharded and the only
exchange is one sum of the model-sized gradient.
"""
from __future__ import annotations

from typing import Mapping, Tuple


def shot_block(ns: int, world: int, rank: int) -> Tuple[int, int]:
    """(first shot, shot count) of rank's contiguous block; sizes differ by
    at most one."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(ns, world)
    count = base + (1 if rank < extra else 0)
    first = rank * base + min(rank, extra)
    return first, count


def block_par(par: Mapping, world: int, rank: int) -> dict:
    """Parameters of rank's block: regular geometry shifts ``osx``/``osz``
    by the block's first shot; irregular geometry slices ``sx``/``sz``."""
    p = dict(par)
    first, count = shot_block(int(p["ns"] if "sx" not in p else len(p["sx"])), world, rank)
    if "sx" in p and p["sx"] is not None:
        p["sx"] = list(p["sx"])[first:first + count]
        p["sz"] = list(p["sz"])[first:first + count]
    else:
        p["osx"] = float(p.get("osx", 0.0)) + first * float(p.get("dsx", 0.0))
        p["osz"] = float(p.get("osz", 0.0)) + first * float(p.get("dsz", 0.0))
    p["ns"] = count
    return p


def interleave_par(par: Mapping, world: int, rank: int) -> dict:
    """Weak-scaling survey: rank r keeps the block's shot count and spacing
    but shifts the regular shot line by r / world of the shot interval, so
    that the ranks together hold world x ns distinct, evenly spaced shots of
    one survey (shot interval dsx / world)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    if "sx" in par and par["sx"] is not None:
        raise ValueError("interleaving needs the regular shot geometry (ns, osx, dsx)")
    p = dict(par)
    p["osx"] = float(p.get("osx", 0.0)) + rank * float(p.get("dsx", 0.0)) / world
    return p


def survey_par(par: Mapping, world: int) -> dict:
    """The whole survey of interleave_par's ranks as one shot line."""
    p = dict(par)
    p["ns"] = int(p["ns"]) * world
    p["dsx"] = float(p.get("dsx", 0.0)) / world
    return p


def allreduce_sum(x, group=None):
    """Sum a gradient (torch tensor, any device the backend supports) over
    ranks in place."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(x, op=dist.ReduceOp.SUM, group=group)
    return x
