"""Host-side ensemble logic (no GPU): the map-form pay-off rule that
chooses, per member, whether remapped submaps get quadratic-form records,
and the grouping of split-BF16 members into batched analyses."""
import os
import sys
import types

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "cmm-s2_gb300"))


def test_forms_pay_rule():
    """Forms pay when the sample points pass through a remapped submap more
    often than FORMS_EVALS_PER_TRIANGLE times per triangle: always for the
    1000-step level-7 / L = 1024 run, never for coarse band-limits on fine
    meshes over 100 steps, never without a remap."""
    from cmm_gpu.ensemble import forms_pay, FORMS_EVALS_PER_TRIANGLE
    assert forms_pay(7, 1024, 1000, 10)
    assert not forms_pay(7, 1024, 100, 10)
    assert forms_pay(5, 512, 100, 10) and forms_pay(6, 1024, 100, 10)
    assert not forms_pay(6, 512, 100, 10) and not forms_pay(5, 256, 100, 10)
    assert not forms_pay(5, 1024, 8, 10)          # no remap in the run
    # the threshold itself: (L+1) 2L points x mean remaining steps
    L, level, Nt, n = 64, 2, 40, 10
    later = sum(Nt - i for i in (10, 20, 30)) / 3
    assert forms_pay(level, L, Nt, n) == ((L + 1) * 2 * L * later > FORMS_EVALS_PER_TRIANGLE * (20 << (2 * level)))


def test_batches_group_split_members_by_band_limit(monkeypatch):
    """Split-BF16 members grouped by band-limit (ascending), in member
    order, in batches of at most 8; a band-limit with a single split
    member and FP64 members stay alone; the grouping is made once."""
    from cmm_gpu import ensemble, native
    made = []

    class FakeBatch:
        MAX = 8

        def __init__(self, plans):
            self.plans = list(plans)
            made.append(self)

    monkeypatch.setattr(native, "ShtBatch", FakeBatch)
    SPLIT, FP64 = native.Sht.SPLIT_BF16, native.Sht.FP64
    spec = [(1024, SPLIT)] * 10 + [(256, SPLIT), (512, FP64), (512, SPLIT), (512, SPLIT)] + [(1024, FP64)]
    members = [types.SimpleNamespace(L=L, precision_mode=mode, sht=("plan", i))
               for i, (L, mode) in enumerate(spec)]
    ens = ensemble.Ensemble.__new__(ensemble.Ensemble)
    ens.members, ens._batch_groups = members, None
    of, groups = ens.batches()
    assert [[p[1] for p in b.plans] for b in groups] == [[12, 13], list(range(8)), [8, 9]]
    assert set(of) == {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 12, 13}
    assert all(of[i] is groups[1] for i in range(8))
    assert ens.batches()[1] is groups and len(made) == 3
