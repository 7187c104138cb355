"""CPU tests: the C ABI library loads and exports every declared symbol;
host-side mesh hierarchy construction and its error paths (no GPU work)."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, GOLDEN


@pytest.fixture(scope="module")
def native():
    lib = os.path.join(ROOT, "cmm-s2_gb300", "lib", "libcmmgpu.so")
    if not os.path.exists(lib):
        import __graft_entry__
        __graft_entry__.build()
    from cmm_gpu import native as nat
    return nat


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "cmm_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cmm_\w+)\s*\(", txt)))


def test_exports_every_declared_symbol(native):
    decl = declared_functions()
    assert len(decl) >= 8
    for name in decl:
        assert hasattr(native.lib, name), name
    assert set(decl) == set(native.exported_symbols())
    assert native.lib.cmm_version() >= 1


def test_split_table_derivation():
    """The device's (V,E,C) ordinate table is the reference's ordinate/corner
    tables re-ordered by corner role."""
    from oracle.spline import SPLIT_ORDINATES, SPLIT_CORNERS
    src = open(os.path.join(ROOT, "cmm-s2_gb300", "csrc", "device_common.cuh")).read()
    body = src[src.index("kSplitOrd[3][3][6] = {"):]
    body = body[body.index("{"):body.index(";")]
    dev = np.array([int(x) for x in re.findall(r"\d+", body)]).reshape(3, 3, 6)
    for lo in range(3):
        for hi in range(3):
            if lo == hi:
                continue
            o, c = SPLIT_ORDINATES[lo, hi], SPLIT_CORNERS[lo, hi]
            pv, pc = list(c).index(hi), list(c).index(3)
            pe = 3 - pv - pc
            pair = {1: o[3], 3: o[4], 2: o[5]}
            want = [o[pv], o[pe], o[pc], pair[pv + pe], pair[pe + pc], pair[pv + pc]]
            assert list(dev[lo, hi]) == want, (lo, hi)


def test_coeff_stride(native):
    assert native.lib.cmm_coeff_stride(3) == 64
    assert native.lib.cmm_coeff_stride(1) == 24
    assert native.lib.cmm_coeff_stride(2) == -1


@pytest.mark.parametrize("level", [3, 4])
def test_hierarchy_maps_onto_qhull_table(native, level):
    d = np.load(os.path.join(GOLDEN, f"mesh_l{level}.npz"))
    rows = native.mesh_check(d["verts"], d["tris"], level)
    assert np.array_equal(np.sort(rows), np.arange(len(rows)))
    # four siblings share their parent's 3 corners and 3 edge midpoints
    sib = d["tris"][rows].reshape(-1, 4 * 3)
    assert all(len(set(r)) == 6 for r in sib)


def test_arbitrary_vertex_and_row_order(native):
    from cmm_gpu.meshgen import icosahedral_mesh
    verts, tris = icosahedral_mesh(3)
    rng = np.random.default_rng(0)
    pv = rng.permutation(len(verts))
    inv = np.argsort(pv)
    v2 = verts[pv]
    t2 = inv[tris][rng.permutation(len(tris))]
    rows = native.mesh_check(v2, t2.astype(np.int32), 3)
    assert np.array_equal(np.sort(rows), np.arange(len(tris)))


def test_rejects_bad_meshes(native):
    from cmm_gpu.meshgen import icosahedral_mesh
    verts, tris = icosahedral_mesh(2)
    with pytest.raises(native.CmmError) as e:
        native.mesh_check(verts, tris, 3)
    assert e.value.code == 2
    bad = tris.copy()
    bad[5] = [0, 1, 2]
    with pytest.raises(native.CmmError):
        native.mesh_check(verts, bad, 2)
    oob = tris.copy()
    oob[0, 0] = len(verts)
    with pytest.raises(native.CmmError) as e:
        native.mesh_check(verts, oob, 2)
    assert e.value.code == 1
    moved = verts.copy()
    moved[20] += 1e-3
    moved[20] /= np.linalg.norm(moved[20])
    with pytest.raises(native.CmmError) as e:
        native.mesh_check(moved, tris, 2)
    assert e.value.code == 2
    assert "midpoint" in str(e.value)


def test_batch_and_form_entry_points_reject_bad_arguments(native):
    """Argument checks of the batched-analysis, split-step and float-float
    form entry points return CMM_ERR_ARG before any device work (null
    handles and pointers, batch sizes outside 1..8), with a message."""
    import ctypes
    lib, P = native.lib, ctypes.c_void_p
    ERR_ARG = 1
    out = P()
    assert lib.cmm_sht_batch_create(None, 2, ctypes.byref(out)) == ERR_ARG
    plans = (P * 9)()
    assert lib.cmm_sht_batch_create(plans, 0, ctypes.byref(out)) == ERR_ARG
    assert lib.cmm_sht_batch_create(plans, 9, ctypes.byref(out)) == ERR_ARG
    assert lib.cmm_sht_batch_create(plans, 2, ctypes.byref(out)) == ERR_ARG   # null plans
    assert b"plans" in lib.cmm_last_error()
    assert lib.cmm_sht_batch_analysis(None, None) == ERR_ARG
    assert lib.cmm_sht_batch_forward(None, None, None, None) == ERR_ARG
    assert lib.cmm_sht_batch_destroy(None) == 0
    assert lib.cmm_bve_step_pre(None, None) == ERR_ARG
    assert lib.cmm_bve_step_post(None, None) == ERR_ARG
    assert lib.cmm_forms_ff(None, None, None, None) == ERR_ARG
    assert native.Mesh.FORM_FF_STRIDE == 112 and native.ShtBatch.MAX == 8
