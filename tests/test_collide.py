"""Collision detection against the reference's own BVH and its narrow phase
(tests/golden/make_collide_golden.py: the reference's BVH.cpp and
CollisionUtil.cpp with its traversal and comp_face_impacts restated).

- CPU: the product's tree construction (csrc/ys_bvh.h) and pair / impact
  functions (csrc/ys_collide.cuh), run by the test-only emulator in the
  reference's traversal order, reproduce the reference's pair lists in the
  same order, bit for bit, and its impacts (same tests, same nodes; t,
  weights and normals to 1e-12).
- GPU: ys_collider_* finds the same pairs (as a set, with the reference's
  orientation of every pair) and the same impacts.

The collide_drop50_s* fixtures are frames of the collision benchmark scene
(a 50 x 50 cloth draping over a 1,280-face sphere, recorded on the GPU by
tests/golden/record_drop_frames.py). Their pair lists are held to the same
bit-exact standard; their impacts come from real drapes, where nearly
coplanar faces make CCD cubics rounding-sensitive, so impacts found on one
side only may be at most 0.5 % of them (each such test sits at the distance
threshold) and common impacts agree in t, weights and normal to 1e-8.
"""
import ctypes

import numpy as np
import pytest

import goldens
from emu_py import lib
from pkg import gpu_available, ys

CASES = sorted(n for n in (p for p in goldens.os.listdir(goldens.GOLDEN_DIR)) if n.startswith("collide_"))
CASES = [c[:-4] for c in CASES]


def _load(name):
    return dict(np.load(goldens.os.path.join(goldens.GOLDEN_DIR, name + ".npz")))


def _topology(W, H):
    F, E = [], []
    for i in range(W - 1):
        for j in range(H - 1):
            tl = i + j * W
            tr, bl, br = tl + 1, tl + W, tl + W + 1
            for tri in ((tl, tr, br), (tl, br, bl)):
                F.append(tri)
                E.append([sorted((tri[a], tri[(a + 1) % 3])) for a in range(3)])
    return np.array(F, np.int32), np.array(E, np.int32)


def _scene_frame(name):
    return name.startswith("collide_drop50_")


def _impacts_agree(mine, theirs, exact):
    """mine, theirs: rows (key columns..., t, w[4], n[3]) keyed by their first
    len - 8 columns. exact: same rows, values to 1e-12; else the tolerance of
    the scene frames."""
    if exact:
        assert mine.shape == theirs.shape
        assert np.array_equal(mine[:, :-8], theirs[:, :-8])
        assert np.abs(mine[:, -8:] - theirs[:, -8:]).max() <= 1e-12
        return
    A = {tuple(r[:-8]): r[-8:] for r in mine}
    B = {tuple(r[:-8]): r[-8:] for r in theirs}
    only = len(set(A) ^ set(B))
    assert only <= max(8, 0.005 * len(B)), only
    common = [k for k in A if k in B]
    assert len(common) >= 0.99 * len(B)
    assert max(np.abs(A[k] - B[k]).max() for k in common) <= 1e-8


def _obstacle(g):
    if "obs_x" in g:
        return (np.ascontiguousarray(g["obs_x"]), np.ascontiguousarray(g["obs_x_prev"]),
                np.ascontiguousarray(g["obs_faces"].astype(np.int32)))
    return np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3), np.int32)


@pytest.mark.parametrize("name", CASES)
def test_emulated_collision_matches_reference(name):
    g = _load(name)
    W, H = int(g["width"]), int(g["length"])
    F, E = _topology(W, H)
    ox, oxp, of = _obstacle(g)
    x, xp = np.ascontiguousarray(g["x"]), np.ascontiguousarray(g["x_prev"])
    L = lib()
    ip, dp, lp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_long)
    L.emu_collide.restype = ctypes.c_int
    L.emu_collide.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int, ip, ip, ctypes.c_int, dp, dp, ctypes.c_int, ip,
                              ctypes.c_double, ctypes.c_int, ip, ctypes.c_long, dp, ctypes.c_long, lp, lp]
    pc, ic = len(g["pairs"]) + 16, len(g["impacts"]) + 16
    pairs, imps = np.zeros(3 * pc, np.int32), np.zeros(15 * ic)
    npr, ni = ctypes.c_long(), ctypes.c_long()
    assert L.emu_collide(W * H, x.ctypes.data_as(dp), xp.ctypes.data_as(dp), len(F), F.ctypes.data_as(ip),
                         E.ctypes.data_as(ip), len(ox), ox.ctypes.data_as(dp), oxp.ctypes.data_as(dp), len(of),
                         of.ctypes.data_as(ip), float(g["thickness"]), 1, pairs.ctypes.data_as(ip), pc,
                         imps.ctypes.data_as(dp), ic, ctypes.byref(npr), ctypes.byref(ni)) == 0
    P = pairs[:3 * npr.value].reshape(-1, 3)
    I = imps[:15 * ni.value].reshape(-1, 15)
    assert np.array_equal(P, g["pairs"])
    gi = g["impacts"]
    if len(gi) or len(I):
        cols = lambda a: np.column_stack([a[:, 13], a[:, :5], a[:, 5:13]])  # noqa: E731
        _impacts_agree(cols(I), cols(gi), exact=not _scene_frame(name))


def test_cloth_mesh_topology_matches_reference_order():
    faces, edges = ys.cloth_mesh_topology(5, 4)
    F, E = _topology(5, 4)
    assert np.array_equal(faces, F) and np.array_equal(edges, E)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_collision_matches_reference(name):
    if not gpu_available():
        pytest.skip("no CUDA device")
    g = _load(name)
    W, H = int(g["width"]), int(g["length"])
    ox, oxp, of = _obstacle(g)
    c = ys.Collider(W, H, obstacle_faces=of if len(of) else None, n_obstacle_nodes=len(ox),
                    thickness=float(g["thickness"]))
    c.set_positions(g["x"], g["x_prev"], ox if len(ox) else None, oxp if len(ox) else None)
    P = c.pairs()
    ref = g["pairs"].astype(np.int32)
    key = lambda a: a[np.lexsort((a[:, 2], a[:, 1], a[:, 0]))]
    assert np.array_equal(key(P), key(ref))  # same pairs, each with the reference's orientation
    imp = c.impacts()
    gi = g["impacts"]
    if len(gi) or len(imp["t"]):
        # match impacts by (pair faces, test): map the reference's pair index to its faces
        def rows(pairs, pidx, typ, nodes, rest):
            pf = pairs[pidx.astype(np.int64)]
            return np.column_stack([pf, typ, nodes, rest])
        mine = rows(P, imp["pair"], imp["type"], imp["nodes"], np.column_stack([imp["t"], imp["w"], imp["n"]]))
        theirs = rows(ref, gi[:, 13], gi[:, 0], gi[:, 1:5], gi[:, 5:13])
        order = lambda a: a[np.lexsort(tuple(a[:, k] for k in range(7, -1, -1)))]
        _impacts_agree(order(mine), order(theirs), exact=not _scene_frame(name))
    c.close()


@pytest.mark.gpu
def test_gpu_obstacle_tree_reuse_matches_fresh_colliders():
    """A collider keeps an obstacle's tree while its positions are unchanged
    and rebuilds it when they move: pairs and impacts equal those of a fresh
    collider either way."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    import response_cases as RC
    s = RC.drop_scene(16, depth=1e-3)
    ox, of = s["obs_x"], s["obs_faces"]

    def fresh(x, xp, o):
        c = ys.Collider(16, 16, obstacle_faces=of, n_obstacle_nodes=len(o))
        c.set_positions(x, xp, o, o)
        out = (c.pairs(), c.impacts())
        c.close()
        return out
    c = ys.Collider(16, 16, obstacle_faces=of, n_obstacle_nodes=len(ox))
    c.set_positions(s["x"], s["x_prev"], ox, ox)
    c.pairs()
    x2 = s["x"] + 2e-4 * np.random.default_rng(0).normal(size=s["x"].shape)
    moved = ox + np.array([1e-4, 0.0, 3e-4])
    for x, o in ((x2, ox), (x2, moved), (s["x"], moved)):
        c.set_positions(x, s["x_prev"], o, o)
        P, I = c.pairs(), c.impacts()
        P0, I0 = fresh(x, s["x_prev"], o)
        assert np.array_equal(P, P0)
        assert np.array_equal(I["nodes"], I0["nodes"]) and np.array_equal(I["t"], I0["t"])
    c.close()
