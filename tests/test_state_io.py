"""On-disk state: the reference's own pickles (written by its video driver,
tests/golden/ref_video_l2_*.pkl) read by the restricted reader, the
snapshot format written back, and refusal of foreign pickle globals."""
import os
import pickle
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, os.path.join(os.path.dirname(GOLDEN), "..", "cmm-s2_gb300"))


@pytest.fixture(scope="module")
def sio():
    from cmm_gpu import state_io
    return state_io


def test_reference_snapshots_read(sio):
    for count in (3, 6, 9):
        d = sio.read_reference_snapshot(os.path.join(GOLDEN, f"ref_video_l2_run{count}.pkl"))
        assert d["vals"].shape == (3, 4, 162) and d["vals"].dtype == np.float64
        assert d["Nc"] == count // 5
        # the current map's values lie on the sphere
        np.testing.assert_allclose(np.linalg.norm(d["vals"][:, 0], axis=0), 1.0, rtol=0, atol=1e-12)


def test_reference_submaps_read(sio):
    from cmm_gpu.meshgen import icosahedral_mesh
    r = sio.reference_submaps(os.path.join(GOLDEN, "ref_video_l2_run_all_maps.pkl"))
    verts, _ = icosahedral_mesh(2)
    np.testing.assert_array_equal(r["vertices"], verts)
    assert r["simplices"].shape == (320, 3) and r["ns"] == [5, 10, 12] and r["Nc"] == 3
    assert r["vals"].shape == (3, 3, 4, 162) and r["coeffs"].shape == (3, 3, 19, 320)
    # the video driver's stack is the plain driver's (same run)
    g = np.load(os.path.join(GOLDEN, "bve_l2_L8.npz"))
    np.testing.assert_array_equal(r["vals"][:r["Nc"]], g["vals"])


def test_snapshot_round_trip_is_the_reference_format(sio, tmp_path):
    vals = np.random.default_rng(0).standard_normal((3, 4, 42))
    p = tmp_path / "snap.txt"
    sio.write_reference_snapshot(str(p), vals, 2)
    with open(p, "rb") as f:
        plain = pickle.load(f)           # what the reference's scripts do
    assert set(plain) == {"vals", "Nc"} and plain["Nc"] == 2
    np.testing.assert_array_equal(plain["vals"], vals)
    np.testing.assert_array_equal(sio.read_reference_snapshot(str(p))["vals"], vals)


class _Evil:
    def __reduce__(self):
        return (os.getpid, ())   # any callable outside numpy and the reference package


def test_reader_refuses_foreign_globals(sio, tmp_path):
    p = tmp_path / "evil.pkl"
    with open(p, "wb") as f:
        pickle.dump({"vals": _Evil()}, f)
    with pytest.raises(pickle.UnpicklingError):
        sio.read_reference_pickle(str(p))
