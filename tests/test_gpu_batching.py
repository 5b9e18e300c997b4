"""The batching form: many trajectories with boxes of uneven size in one job
(cir_run_multi), the per-step launches replayed from captured CUDA graphs, and the GEMM
tile shapes picked by the autotuner.  Each trajectory's results must equal what cir_run
gives for it alone, and match the FP64 oracle."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

SPEC_TOL = 1e-4
KEYS = ("tcf_ir", "tcf_vv", "tcf_vh", "sw", "ls_ir", "ls_vv", "ls_vh")


def _params(lib, **extra):
    prm = {"natom_mol": 4, "nchrom_mol": 2, "imodel": 1, "ispecies": 0, "map": 0, "ntcfpoints": 8,
           "nsamples": 2, "sampleEvery": 0.03, "dt": 0.010, "t1": 0.260, "avef": 3415.0, "omegaStart": 1000,
           "omegaStop": 5000, "omegaStep": 1, "nzeros": 600, "beginTime": 0.0}
    keys = {k: prm[k] for k in ("ntcfpoints", "nsamples", "sampleEvery", "omegaStep", "nchrom_mol", "nzeros",
                                "map", "dt", "t1", "avef", "beginTime", "omegaStart", "omegaStop")}
    keys.update(extra)
    return prm, lib.default_params(model="tip4p2005", species="H2O", **keys)


def _trajectories(lib, prm, sizes):
    out = []
    for i, nmol in enumerate(sizes):
        xyz, box = lib.synth_trajectory(nmol, 12, seed=100 + i)
        fos = np.array([O.frame_index(prm, 0.010, s, k) for s in range(prm["nsamples"])
                        for k in range(prm["ntcfpoints"])], np.int32)
        out.append((xyz, box, fos))
    return out


def _same(a, b, tol, name):
    for k in KEYS:
        e = O.rel_l2(a[k], b[k])
        assert e < tol, (name, k, e)
    for k in ("pw", "rw", "rmw", "omega", "ls_omega"):
        np.testing.assert_allclose(np.nan_to_num(a[k]), np.nan_to_num(b[k]), rtol=1e-5, atol=1e-7, err_msg=f"{name} {k}")
    assert a["bins_out_of_range"] == b["bins_out_of_range"]


def test_run_multi_uneven_sizes_matches_single_runs(lib):
    """Three sizes (two trajectories of one of them) in one cir_run_multi call equal five
    separate cir_run calls: the batched launches compute each trajectory independently."""
    prm, p = _params(lib)
    sizes = [16, 27, 16, 40, 27]
    trajs = _trajectories(lib, prm, sizes)
    with lib.Engine(p, sizes[0] * 4) as eng:
        multi = eng.run_multi(trajs)
    for i, (xyz, box, fos) in enumerate(trajs):
        with lib.Engine(p, xyz.shape[1]) as eng:
            single = eng.run(xyz, box, fos)
        _same(multi[i], single, 1e-6, f"trajectory {i} ({sizes[i]} molecules)")


def test_run_multi_against_oracle(lib):
    """Each trajectory of an uneven batch against the FP64 oracle."""
    prm, p = _params(lib)
    sizes = [16, 32]
    trajs = _trajectories(lib, prm, sizes)
    with lib.Engine(p, 64) as eng:
        multi = eng.run_multi(trajs)
    for i, (xyz, box, fos) in enumerate(trajs):
        ref = O.run(prm, xyz, [box] * len(xyz), fos)
        for k in KEYS:
            e = O.rel_l2(multi[i][k], ref[k])
            assert e < SPEC_TOL, (sizes[i], k, e)


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_graph_replay_matches_direct_launches(lib, precision):
    """The step loop replayed from a captured CUDA graph (second call reuses the graph of the
    first) gives the results of direct launches."""
    prm, p_graph = _params(lib, precision=precision)
    _, p_direct = _params(lib, precision=precision, cuda_graphs=0)
    xyz, box, fos = _trajectories(lib, prm, [24])[0]
    with lib.Engine(p_direct, xyz.shape[1]) as eng:
        direct = eng.run(xyz, box, fos)
    with lib.Engine(p_graph, xyz.shape[1]) as eng:
        first = eng.run(xyz, box, fos)
        launches_first = eng.stats()["kernel_launches"]
        second = eng.run(xyz, box, fos)
        launches_second = eng.stats()["kernel_launches"] - launches_first
    _same(first, direct, 1e-6, "captured")
    _same(second, direct, 1e-6, "replayed")
    assert launches_second == launches_first, (launches_first, launches_second)


def test_autotuner_tile_shapes_agree(lib):
    """Both SIMT tile shapes produce the same product (the autotuner only changes speed):
    with autotune off the 128 x 128 tiles run; with it on, whichever is faster."""
    prm, p_on = _params(lib)
    _, p_off = _params(lib, autotune=0)
    xyz, box, fos = _trajectories(lib, prm, [40])[0]
    with lib.Engine(p_off, xyz.shape[1]) as eng:
        off = eng.run(xyz, box, fos)
    with lib.Engine(p_on, xyz.shape[1]) as eng:
        on = eng.run(xyz, box, fos)
    _same(on, off, 1e-6, "autotuned")


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_run_multi_config_sizes_against_oracle(lib, precision):
    """The batching configuration's sizes -- 128, 216, 343 and 512 molecules, two seeded
    trajectories each, 200 points -- in one cir_run_multi job, each trajectory against its
    FP64 oracle spectra (tests/golden/make_configs.py): the plain form within 1e-4, the
    split-BF16 form within 1e-3 per spectrum."""
    import os
    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    import make_configs as MC
    path = os.path.join(GOLDEN, "batching_2traj.npz")
    if not os.path.exists(path):
        pytest.skip("batching_2traj.npz not generated (tests/golden/make_configs.py)")
    z = np.load(path)
    q = {k: MC.BATCH_PRM[k] for k in ("ntcfpoints", "nsamples", "sampleEvery", "omegaStep", "nzeros", "map", "dt",
                                      "t1", "avef", "beginTime", "omegaStart", "omegaStop")}
    p = lib.default_params(model="tip4p2005", species="H2O", precision=precision, **q)
    trajs, names = [], []
    for nmol in MC.BATCH_SIZES:
        for t in range(MC.BATCH_TRAJ):
            xyz, box = lib.synth_trajectory(nmol, MC.BATCH_PRM["ntcfpoints"], seed=MC.batch_seed(nmol, t))
            trajs.append((xyz, box, None))
            names.append(f"n{nmol}_t{t}_")
    with lib.Engine(p, 4 * MC.BATCH_SIZES[0]) as eng:
        outs = eng.run_multi(trajs)
    tol = SPEC_TOL if precision == "fp32" else 1e-3
    worst = 0.0
    for out, key in zip(outs, names):
        ref = MC.batching_spectra(z, key)
        for k in KEYS:
            e = O.rel_l2(out[k], ref[k])
            worst = max(worst, e)
            assert e < tol, (key, k, e)
        assert out["bins_out_of_range"] == int(z[key + "oor"])
    print(f"batching config sizes {precision}: worst spectrum error {worst:.2e}")


def test_autotuner_tensor_core_forms_agree(lib):
    """In the split-BF16 form the autotuner also picks the propagation products' tile width
    (128 x 128 or 128 x 256 on the persistent tcgen05 GEMM) and the tridiagonalisation's
    thread blocks per SM; both change speed only, so the tuned run equals the untuned one."""
    keys = dict(model="tip4p2005", species="H2O", ntcfpoints=160, nsamples=2, sampleEvery=0.05, omegaStart=1000,
                omegaStop=5000, omegaStep=1, nzeros=600, precision="bf16x3")
    p_on = lib.default_params(**keys)
    p_off = lib.default_params(autotune=0, **keys)
    fos = lib.frame_table(p_on, 0.010)
    xyz, box = lib.synth_trajectory(64, int(fos.max()) + 1, seed=21)
    with lib.Engine(p_off, xyz.shape[1]) as eng:
        off = eng.run(xyz, box, fos)
        st_off = eng.stats()
    with lib.Engine(p_on, xyz.shape[1]) as eng:
        on = eng.run(xyz, box, fos)
        st = eng.stats()
    assert st_off["tuned_split_tile"] == 0 and st_off["tuned_tridiag_blocks"] == 0
    assert st["tuned_split_tile"] in (128, 256), st
    assert st["tuned_tridiag_blocks"] in (3, 4), st      # order 128: four blocks per SM by default
    print("autotuner picked", st["tuned_split_tile"], "wide tiles,", st["tuned_tridiag_blocks"], "blocks per SM")
    _same(on, off, 1e-6, "autotuned tensor-core form")


def test_run_multi_joint_split_launches_match_single_runs(lib):
    """The split-BF16 form runs the step loops of up to four box sizes jointly: each step is
    one persistent launch per product over the origins of every size.  Each trajectory's
    results equal what cir_run gives for it alone in the same form (the same products, tile
    by tile), and the joint job launches fewer kernels than the sizes one after another."""
    prm, p = _params(lib, precision="bf16x3")
    sizes = [16, 27, 16, 40, 27]
    trajs = _trajectories(lib, prm, sizes)
    with lib.Engine(p, sizes[0] * 4) as eng:
        multi = eng.run_multi(trajs)
        joint_launches = eng.stats()["kernel_launches"]
    single_launches = 0
    for i, (xyz, box, fos) in enumerate(trajs):
        with lib.Engine(p, xyz.shape[1]) as eng:
            single = eng.run(xyz, box, fos)
            single_launches += eng.stats()["kernel_launches"]
        _same(multi[i], single, 1e-5, f"trajectory {i} ({sizes[i]} molecules), joint split-BF16")
    print("kernel launches: joint", joint_launches, "one size at a time", single_launches)
    assert joint_launches < single_launches


def test_run_multi_joint_tridiagonalisation_matches_single_runs(lib):
    """With two or more box sizes of orders 257-1024 starting a chunk together, the joint
    split-BF16 run tridiagonalises all their Hamiltonians in one launch (the longest matrices
    first) before each size's eigensolver goes on; each trajectory's results equal cir_run's
    for it alone."""
    prm, p = _params(lib, precision="bf16x3")
    sizes = [144, 200, 144]            # orders 288 and 400
    trajs = _trajectories(lib, prm, sizes)
    with lib.Engine(p, sizes[0] * 4) as eng:
        multi = eng.run_multi(trajs)
    for i, (xyz, box, fos) in enumerate(trajs):
        with lib.Engine(p, xyz.shape[1]) as eng:
            single = eng.run(xyz, box, fos)
        _same(multi[i], single, 1e-5, f"trajectory {i} ({sizes[i]} molecules), joint tridiagonalisation")
