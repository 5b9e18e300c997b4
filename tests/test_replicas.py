"""Replicas across processes (`calcir_gb300.replicas`): the time origins of one job split over
processes, each running its share as a job of that many origins, and the results combined on
the host.  Runs on the CPU: the FP64 oracle stands in for each process's run, and two gloo
processes carry the all-reduce."""
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import golden_params, load_golden
from oracle import oracle as O

KEYS_MEAN = ("tcf_ir", "tcf_vv", "tcf_vh", "sw", "pw", "ls_ir", "ls_vv", "ls_vh")


def _case(lib, nsamples=3, ntcf=12):
    """64 H2O, `nsamples` overlapping origins 0.05 ps apart, `ntcf` points each."""
    meta, _ = load_golden("small_h2o")
    prm = golden_params(meta)
    prm.update(nsamples=nsamples, ntcfpoints=ntcf, nzeros=200, sampleEvery=0.05)
    fos = np.array([O.frame_index(prm, meta["frame_dt"], s, k) for s in range(nsamples) for k in range(ntcf)])
    xyz, box = lib.synth_trajectory(meta["nmol"], int(fos.max()) + 1, seed=meta["seed"])
    return prm, xyz, [box] * len(xyz), fos


def _assert_same(got, ref, tol=1e-12):
    for k in KEYS_MEAN:
        assert O.rel_l2(got[k], ref[k]) < tol, (k, O.rel_l2(got[k], ref[k]))
    for k in ("rw", "rmw"):
        a, b = np.asarray(got[k]), np.asarray(ref[k])
        np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
        ok = ~np.isnan(b)
        assert O.rel_l2(a[ok], b[ok]) < tol, k
    np.testing.assert_array_equal(got["omega"], ref["omega"])
    np.testing.assert_array_equal(got["ls_omega"], ref["ls_omega"])
    assert int(got["bins_out_of_range"]) == int(ref["bins_out_of_range"])


def test_origin_share_partitions():
    from calcir_gb300.replicas import origin_share
    for nsamples in range(1, 13):
        for world in range(1, nsamples + 1):
            shares = [origin_share(nsamples, world, r) for r in range(world)]
            assert shares[0][0] == 0 and sum(c for _, c in shares) == nsamples
            assert all(shares[r][0] + shares[r][1] == shares[r + 1][0] for r in range(world - 1))
            assert max(c for _, c in shares) - min(c for _, c in shares) <= 1
    with pytest.raises(ValueError):
        origin_share(2, 3, 0)
    with pytest.raises(ValueError):
        origin_share(4, 2, 2)


def test_combine_equals_one_run(lib):
    from calcir_gb300.replicas import combine, origin_share, share_rows
    prm, frames, boxes, fos = _case(lib)
    whole = O.run(prm, frames, boxes, fos)
    for world in (2, 3):
        parts, counts = [], []
        for r in range(world):
            first, count = origin_share(prm["nsamples"], world, r)
            rows = share_rows(fos, prm["nsamples"], prm["ntcfpoints"], first, count)
            parts.append(O.run(dict(prm, nsamples=count), frames, boxes, rows))
            counts.append(count)
        _assert_same(combine(parts, counts), whole)


def test_combine_rejects_different_parameters(lib):
    from calcir_gb300.replicas import combine
    prm, frames, boxes, fos = _case(lib, nsamples=2, ntcf=4)
    a = O.run(dict(prm, nsamples=1), frames, boxes, fos[:4])
    b = O.run(dict(prm, nsamples=1, omegaStart=2100), frames, boxes, fos[4:])
    with pytest.raises(ValueError):
        combine([a, b], [1, 1])


def _worker(rank, world, port, prm, frames, boxes, fos, out):
    from types import SimpleNamespace

    import torch.distributed as dist

    from calcir_gb300.replicas import run_sharded
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        p = SimpleNamespace(nsamples=prm["nsamples"], ntcfpoints=prm["ntcfpoints"])
        res = run_sharded(p, 0, None, None, fos,
                          runner=lambda count, rows: O.run(dict(prm, nsamples=count), frames, boxes, rows))
        np.savez(out % rank, **{k: np.asarray(v) for k, v in res.items()})
    finally:
        dist.destroy_process_group()


def test_all_reduce_over_two_gloo_processes(lib, tmp_path):
    prm, frames, boxes, fos = _case(lib)
    whole = O.run(prm, frames, boxes, fos)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "rank%d.npz")
    mp.spawn(_worker, args=(2, port, prm, frames, boxes, fos, out), nprocs=2, join=True)
    got = [dict(np.load(out % r)) for r in range(2)]
    for k in got[0]:   # every process holds the same combined result
        np.testing.assert_array_equal(got[0][k], got[1][k])
    _assert_same(got[0], whole)


def test_shard_params_copies_every_field(lib):
    from calcir_gb300.replicas import shard_params
    p = lib.default_params(species="H2O", nsamples=7, ntcfpoints=33, precision="bf16x3", share_frames=1)
    q = shard_params(p, 3)
    assert q.nsamples == 3 and p.nsamples == 7
    for name, _ in type(p)._fields_:
        if name != "nsamples":
            assert getattr(q, name) == getattr(p, name), name


@pytest.mark.gpu
def test_run_sharded_in_one_process_on_the_gpu(lib):
    """Without torch.distributed the whole job runs in this process through a context of its
    own: the same spectra as Engine.run, within 1e-4 of the oracle like every plain run."""
    from calcir_gb300.replicas import run_sharded
    prm, frames, boxes, fos = _case(lib, nsamples=2, ntcf=16)
    keys = {k: prm[k] for k in ("ntcfpoints", "nsamples", "sampleEvery", "omegaStep", "nchrom_mol", "nzeros",
                                "map", "dt", "t1", "avef", "beginTime", "omegaStart", "omegaStop")}
    p = lib.default_params(model="tip4p2005", species="H2O", **keys)
    xyz = np.asarray(frames, np.float32)
    got = run_sharded(p, xyz.shape[1], xyz, boxes[0], fos)
    with lib.Engine(p, xyz.shape[1]) as eng:
        ref = eng.run(xyz, boxes[0], fos)
    _assert_same(got, ref, tol=1e-6)
    whole = O.run(prm, frames, boxes, fos)
    for k in KEYS_MEAN:
        assert O.rel_l2(got[k], whole[k]) < 1e-4, k
