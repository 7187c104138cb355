"""GPU: ensembles of uneven members advanced by one captured CUDA graph per
step, and the autotuner's launch shapes; every member's run must be
bit-identical to the same run made alone (members are independent and all
kernels deterministic, so sharing meshes/tables, parallel graph branches
and launch shapes cannot change a result)."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    import __graft_entry__
    __graft_entry__.build()
    from cmm_gpu import ensemble, spherical_simulations, autotune, workloads, meshgen
    return ensemble, spherical_simulations, autotune, workloads, meshgen


def _alone(mods, spec, i, seed, Nt, T, lmax, rms, n_maps, precision="split_bf16", forms=True):
    ensemble, sims, _, workloads, meshgen = mods
    level, L = spec
    verts, tris = meshgen.icosahedral_mesh(level)
    pert = workloads.spectral_perturbation(lmax, seed=seed * 100003 + i, slope=-2.0, rms=rms)
    s = sims.BVESolver(verts, tris, level, L, Nt, T, sims.Vorticity(spline_sh=pert), n_maps=n_maps,
                       precision=precision, forms=forms)
    return s.run()


@pytest.mark.parametrize("persistent,precision,batch", [(False, "split_bf16", False),
                                                        (True, "split_bf16", False),
                                                        (False, "split_bf16", True),
                                                        (True, "split_bf16", True),
                                                        (True, "fp64", False)])
def test_ensemble_graph_matches_members_alone(mods, persistent, precision, batch):
    """One graph replay per step, or (persistent) the whole remaining run
    captured as one graph and launched once; FP64 members share one set of
    Pbar tables per band-limit; (batch) the same-band-limit members'
    analyses batched into one tensor-core launch per batch."""
    ensemble, sims, autotune, _, _ = mods
    kw = dict(levels=(2, 3), bandlimits=(16, 32), Nt=14, T=0.1, lmax=8, rms=3.0, n_maps=4)
    ens = ensemble.Ensemble.from_seed(5, seed=7, precision=precision, **kw).bootstrap()
    tuner = autotune.Autotuner(reps=1)
    tuner.tune_ensemble_kernels(ens)
    tuner.tune_schedule(ens, stream_counts=(1, 3), steps_each=1, batch=False)
    if batch:
        assert ens.batches()[1], "no band-limit with two split-BF16 members"
        ens.capture(streams=ens.schedule["streams"], order=ens.schedule["order"], batch=True)
        assert ens.schedule["batch"]
    if persistent:
        ens.run_persistent()
        assert ens.schedule["steps"] > 1
    else:
        ens.run(ens.members[0].Nt - 2 - ens.count)
    torch.cuda.synchronize()
    assert ens.count == ens.members[0].Nt - 2
    for i, (m, spec) in enumerate(zip(ens.members, ens.specs)):
        ref = _alone(mods, spec, i, 7, kw["Nt"], kw["T"], kw["lmax"], kw["rms"], kw["n_maps"], precision,
                     forms=m.stack_forms is not None)
        assert m.Nc == ref.Nc and m.count == ref.count
        assert torch.equal(m.omega, ref.omega), i
        for k in range(m.Nc):
            assert torch.equal(m.stack[k], ref.stack[k]), (i, k)
        assert m.mesh.status() == 0 and m.vm.status() == 0 and m.sht.status() == 0
    log = tuner.log
    assert log["schedule"]["best"]["streams"] in (1, 3)
    assert all(v["compose"]["best"] in autotune.Autotuner.BLOCKS for v in log["kernels"].values())
