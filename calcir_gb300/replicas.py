"""Time origins of one job split over processes (one GPU each) and their results combined.

The reference runs its time origins one after another and only sums what each contributes:
the correlation functions, the spectral density and the frequency distributions
(calcIR.cu:360-839). A job therefore shards by origin with no exchange before one final
reduction of a few tens of KB per process. Multi-GPU in this form is replicas only: no
collective on the data path, one all-reduce at the end.

Each process runs a contiguous share of the origins through its own context, as a job of
that many origins, so its result is normalised by its own origin count. `combine` (results
gathered in one process) and `all_reduce_result` (one result per process, over
torch.distributed) weight the shares by origin count. They return what one run over every
origin returns, up to the rounding of the weighted sums:

* the damped correlation functions, the spectral density, Pw and the three lineshapes are
  averages over origins (a lineshape is linear in its correlation function): weighted means;
* Rw and Rmw are ratios to Pw (calcIR.cu:834-839): sum(w Pw R) / sum(w Pw), NaN where the
  combined Pw is 0, as the reference prints them;
* the counts of eigenvalues outside the histogram window add.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

_TCF = ("tcf_ir", "tcf_vv", "tcf_vh")
_MEAN = ("sw", "pw", "ls_ir", "ls_vv", "ls_vh")
_RATIO = ("rw", "rmw")
_SAME = ("omega", "ls_omega")


def origin_share(nsamples: int, world: int, rank: int) -> tuple[int, int]:
    """(first origin, number of origins) of process `rank` of `world`: contiguous shares
    whose sizes differ by at most one, in rank order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world} processes")
    if nsamples < world:
        raise ValueError(f"{world} processes for {nsamples} time origins: every process needs one")
    q, r = divmod(nsamples, world)
    return rank * q + min(rank, r), q + (1 if rank < r else 0)


def share_rows(frame_of_step, nsamples: int, ntcf: int, first: int, count: int) -> np.ndarray:
    """The frame-table entries (origin-major, `ntcf` per origin) of origins first .. first+count-1."""
    t = np.asarray(frame_of_step).reshape(nsamples, ntcf)
    return np.ascontiguousarray(t[first:first + count].ravel(), np.int32)


def shard_params(p, count: int):
    """A copy of the parameter block `p` for a share of `count` origins."""
    q = type(p)()
    C.memmove(C.byref(q), C.byref(p), C.sizeof(p))
    q.nsamples = int(count)
    return q


def _pack(res: dict, w: float) -> np.ndarray:
    parts = []
    for k in _TCF:
        a = np.asarray(res[k], np.complex128)
        parts += [w * a.real, w * a.imag]
    for k in _MEAN:
        parts.append(w * np.asarray(res[k], np.float64))
    pw = np.asarray(res["pw"], np.float64)
    for k in _RATIO:
        parts.append(np.where(pw > 0, w * pw * np.asarray(res[k], np.float64), 0.0))
    parts.append(np.array([float(res.get("bins_out_of_range", 0))]))
    return np.concatenate(parts)


def _unpack(vec: np.ndarray, like: dict) -> dict:
    out = {k: np.array(like[k]) for k in _SAME}
    o = 0
    for k in _TCF:
        n = len(like[k])
        out[k] = vec[o:o + n] + 1j * vec[o + n:o + 2 * n]
        o += 2 * n
    pw = None
    for k in _MEAN:
        n = len(like[k])
        if k == "pw":
            pw = vec[o:o + n]
        out[k] = vec[o:o + n].astype(np.asarray(like[k]).dtype)
        o += n
    for k in _RATIO:
        n = len(like[k])
        with np.errstate(invalid="ignore", divide="ignore"):
            r = np.where(pw > 0, vec[o:o + n] / np.where(pw > 0, pw, 1.0), np.nan)
        out[k] = r.astype(np.asarray(like[k]).dtype)
        o += n
    out["bins_out_of_range"] = int(round(vec[o]))
    return out


def combine(partials: list[dict], counts: list[int]) -> dict:
    """One result from the results of disjoint origin shares (`counts[i]` origins in
    `partials[i]`), all of the same parameters."""
    if len(partials) != len(counts) or not partials or min(counts) < 1:
        raise ValueError("one result per share, every share with at least one origin")
    for r in partials[1:]:
        for k in _SAME:
            if not np.array_equal(np.asarray(r[k]), np.asarray(partials[0][k])):
                raise ValueError(f"results of different parameters ({k} differs)")
    total = float(sum(counts))
    vec = sum(_pack(r, c / total) for r, c in zip(partials, counts))
    return _unpack(vec, partials[0])


def all_reduce_result(res: dict, count: int, group=None) -> dict:
    """The combined result on every process of `group`, each holding the result `res` of its
    own share of `count` origins (one all-reduce of the origin counts, one of the sums)."""
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    n = torch.tensor([float(count)], dtype=torch.float64, device=dev)
    dist.all_reduce(n, group=group)
    vec = torch.from_numpy(_pack(res, count / n.item())).to(dev)
    dist.all_reduce(vec, group=group)
    return _unpack(vec.cpu().numpy(), res)


def run_sharded(p, natoms: int, xyz, boxes, frame_of_step, runner=None, group=None) -> dict:
    """The job of parameters `p` with its time origins shared over the processes of `group`
    (or run whole without torch.distributed): this process runs its share and every process
    returns the combined result.

    `runner(count, rows)`, when given, replaces the share's run on this process's GPU context
    (`Engine(shard_params(p, count), natoms).run(xyz, boxes, rows)`)."""
    rank, world = 0, 1
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            rank, world = dist.get_rank(group), dist.get_world_size(group)
    except ImportError:
        pass
    first, count = origin_share(p.nsamples, world, rank)
    rows = share_rows(frame_of_step, p.nsamples, p.ntcfpoints, first, count)
    if runner is None:
        from . import Engine
        with Engine(shard_params(p, count), natoms) as eng:
            res = eng.run(xyz, boxes, rows)
    else:
        res = runner(count, rows)
    return all_reduce_result(res, count, group) if world > 1 else res
