"""HDF5 trajectory files (src/Saver.cpp:184-427, src/Loader.cpp:3-267)
through the package's own reader and writer (h5.py), and the GPU step
against the trajectory the reference ships
(TrainingData/Table_2/Wind_Yarn_1_2_Plain_Size5.h5: a 5 x 5 two-yarn plain
cloth in wind, 500 steps of its simulator), extracted by
tests/golden/make_h5_golden.py.
"""
import hashlib
import os

import numpy as np
import pytest

import goldens
from pkg import gpu_available, ys
from oracle.ref.refpath import ref_file

GOLDEN = os.path.join(goldens.GOLDEN_DIR, "h5_wind_yarn12_plain5.npz")
REF_FILE = ref_file("TrainingData", "Table_2", "Wind_Yarn_1_2_Plain_Size5.h5")
KEYS = ("LPos", "LPosFix", "LVel", "EPos", "EPosBar", "EVel")


def _golden():
    return dict(np.load(GOLDEN))


def _physical(g):
    return {str(k): float(v) for k, v in zip(g["physical_names"], g["physical"])}


@pytest.mark.skipif(REF_FILE is None, reason="the reference's data file is not here")
def test_reader_reads_the_reference_file():
    g = _golden()
    assert hashlib.sha256(open(REF_FILE, "rb").read()).hexdigest() == str(g["sha256"])
    size, phy = ys.h5.cloth_property_loader_heter(REF_FILE)
    assert (size["width"], size["length"]) == (5, 5)
    assert phy == pytest.approx(_physical(g), rel=0, abs=0)
    head = ys.h5.data_loader(REF_FILE, 0, 40)
    last = ys.h5.data_loader(REF_FILE, int(g["n_steps"]) - 1, int(g["n_steps"]))
    for k in KEYS:
        assert np.array_equal(head[k], g[k]) and np.array_equal(last[k][0], g["last_" + k])


@pytest.mark.skipif(REF_FILE is None, reason="the reference's data file is not here")
def test_rewritten_reference_file_reads_back_identically(tmp_path):
    a = ys.h5.read(REF_FILE)
    p = str(tmp_path / "copy.h5")
    ys.h5.write(p, a)
    b = ys.h5.read(p)
    assert sorted(a) == sorted(b)
    for k in a:
        assert a[k].dtype == b[k].dtype and np.array_equal(a[k], b[k])


def test_save_and_load_round_trip(tmp_path):
    g = _golden()
    phy = _physical(g)
    phy["woven_pattern"] = int(phy["woven_pattern"])
    p = str(tmp_path / "traj.h5")
    ys.h5.save_trajectory(p, 5, 5, phy, {k: g[k] for k in KEYS})
    size, phy2 = ys.h5.cloth_property_loader(p)
    assert size == {"width": 5, "length": 5} and phy2 == phy
    st = ys.h5.data_loader(p, 3, 17)
    for k in KEYS:
        assert np.array_equal(st[k], g[k][3:17])
    f = ys.h5.read(p)
    assert f["/Properties/Physical properties"].dtype == ys.h5.physical_dtype(True)


def test_many_groups_round_trip(tmp_path):
    """1,600 node groups: several symbol nodes per B-tree leaf and a
    two-level B-tree."""
    W = 40
    rng = np.random.default_rng(0)
    st = {k: rng.normal(size=(3, W * W, 3 if k[0] == "L" else 2)) for k in KEYS}
    phy = {n: 1.0 for n in ys.h5.physical_dtype(False).names}
    phy["woven_pattern"] = 2
    p = str(tmp_path / "big.h5")
    ys.h5.save_trajectory(p, W, W, phy, st)
    back = ys.h5.data_loader(p, 0, 3)
    for k in KEYS:
        assert np.array_equal(back[k], st[k])
    assert ys.h5.cloth_property_loader(p)[1] == phy


def test_reader_rejects_other_files(tmp_path):
    p = tmp_path / "x.h5"
    p.write_bytes(b"not hdf5" * 20)
    with pytest.raises(ys.h5.H5Error):
        ys.h5.read(str(p))


def _spec(g, handles=None):
    phy = _physical(g)
    yarns = [ys.Yarn(R=phy["R"], rho=phy["Yarn1_rho"], Y=phy["Yarn1_Y"], B=phy["Yarn1_B"]),
             ys.Yarn(R=phy["R"], rho=phy["Yarn2_rho"], Y=phy["Yarn2_Y"], B=phy["Yarn2_B"])]
    W, L = int(g["width"]), int(g["length"])
    height = float(g["LPos"][0, 0, 2])  # node (0, 0) of the upright pose sits at the height
    spec = ys.ClothSpec.from_yarns(W, L, height, phy["L"], phy["R"], yarns, phy["kc"], phy["kf"], phy["df"],
                                   phy["mu"], phy["S"], phy["handle_stiff"], ys.WovenPattern(int(phy["woven_pattern"])),
                                   ys.InitPose.Upright)
    spec.G = (0.0, 0.0, phy["Gravity"])
    spec.wind_vel = (phy["wind_velocity_x"], phy["wind_velocity_y"], phy["wind_velocity_z"])
    spec.wind_density, spec.wind_drag = phy["wind_density"], phy["wind_drag"]
    spec.handles = [(0, 0), (W - 1, 0)] if handles is None else handles
    return spec


@pytest.mark.gpu
def test_gpu_first_step_matches_the_reference_data_file():
    """From the file's step 0, one GPU step (h = 1e-3, as the reference's
    training drivers use) against the file's step 1: positions and
    velocities to 1e-12. The file pins one step only: from step 2 on it
    follows handle springs at the top corners without their stiffness in
    the system matrix (its step 1 equals a run without handles, its later
    steps none of the current reference's set-ups), so it comes from another
    state of the reference's code; the reference's current code run on the
    same set-up (the harness) agrees with it to the same precision at step 1."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    g = _golden()
    b = ys.ClothBatch([_spec(g, handles=[])])
    st = b.get_state()
    assert np.abs(st["LPos"] - g["LPos"][0]).max() <= 1e-15  # the constructor's pose is the file's first step
    b.set_state(**{k: g[k][0] for k in KEYS})
    assert all(x["ok"] for x in b.step(1e-3))
    st = b.get_state()
    for k in ("LPos", "LVel", "EPos", "EVel"):
        scale = max(np.abs(g[k][1]).max(), 1e-300)
        assert np.abs(st[k] - g[k][1]).max() <= 1e-12 * scale, k
    b.close()


@pytest.mark.skipif(REF_FILE is None, reason="the reference's data file is not here")
def test_writer_messages_match_the_reference_files(tmp_path):
    """The writer's object-header messages for the reference's datasets equal
    the ones libhdf5 wrote (dataspace, datatype and fill value byte for byte,
    layout class and size), and its groups use the same B-tree and symbol-node
    parameters; the reference's files also carry an old-style fill value and a
    modification time, which readers do not need."""
    import struct
    p = str(tmp_path / "copy.h5")
    ys.h5.write(p, ys.h5.read(REF_FILE))
    ref = ys.h5._Reader(open(REF_FILE, "rb").read())
    ours = ys.h5._Reader(open(p, "rb").read())
    assert ref.d[:24] == ours.d[:24]  # signature, versions, sizes, group K values

    def header(r, path):
        addr = r.root[1]
        for part in [x for x in path.split("/") if x]:
            body = next(b for t, b in r.messages(addr) if t == 0x11)
            bt, hp = struct.unpack_from("<QQ", body)
            addr = r.group(bt, hp)[part]
        return {t: b for t, b in r.messages(addr)}
    for path in ("/Steps/Position/Node 3 1/LPOS", "/Steps/Velocity/Node 0 4/EVEL", "/Properties/Size",
                 "/Properties/Physical properties"):
        a, b = header(ref, path), header(ours, path)
        for t in (0x01, 0x03, 0x05):
            assert a[t] == b[t], (path, hex(t))
        assert a[0x08][:2] == b[0x08][:2] and a[0x08][10:18] == b[0x08][10:18]


def test_non_square_round_trip(tmp_path):
    """Node groups are named by (u, v) and loaded at u + v W for W != L."""
    W, L = 6, 4
    rng = np.random.default_rng(2)
    st = {k: rng.normal(size=(2, W * L, 3 if k[0] == "L" else 2)) for k in KEYS}
    phy = {n: 0.5 for n in ys.h5.physical_dtype(True).names}
    phy["woven_pattern"] = 1
    p = str(tmp_path / "ns.h5")
    ys.h5.save_trajectory(p, W, L, phy, st)
    f = ys.h5.read(p)
    assert np.array_equal(f["/Steps/Position/Node 5 1/LPOS"], st["LPos"][:, 5 + 1 * W])
    assert np.array_equal(f["/Steps/Velocity/Node 2 3/EVEL"], st["EVel"][:, 2 + 3 * W])
    back = ys.h5.data_loader(p, 1, 2)
    for k in KEYS:
        assert np.array_equal(back[k][0], st[k][1])
    assert ys.h5.cloth_property_loader_heter(p)[0] == {"width": W, "length": L}
