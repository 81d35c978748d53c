"""CPU checks of the reverse-mode step's compression (csrc/ys_adjoint.cu).

The adjoint folds the residual r(s) = A(s) q - b(s) of one step with lambda
and obtains every column of dr/ds from one forward-mode direction per
(node colour, state component): nodes coloured (u + 9 v) mod 41 whose
neighbourhoods (L1 grid distance <= 4) never overlap. Two facts carry it:

- the colouring: two nodes of one colour are at L1 distance >= 9;
- the reach: perturbing one node's state changes the residual and the slide
  indicator only at row blocks within L1 distance 4 of it, and perturbing a
  yarn line's material only rows of that line and its two neighbours.

The reach is probed here with the CPU oracle (the reference's step restated
in C): central differences of r at a fixed q and of the slide indicator, on
a deformed cloth of each weave where every term is active (shear with
jamming, crimp bending, friction near its slide switch). The bound 4 comes
from the longest chain (normals of crimp-bent neighbours -> a crossing's
compression -> its shear segments' rows); on states where the compression is
zero the probe sees reach 3.
"""
import numpy as np
import pytest

from layout import node5_to_ref, ref_to_node5
from oracle.oracle import ClothSpec, OracleCloth

COLORS = 41


def color(u, v):
    return (u + 9 * v) % COLORS


def test_colouring_separates_neighbourhoods():
    W = H = 60
    pts = {}
    for v in range(H):
        for u in range(W):
            pts.setdefault(color(u, v), []).append((u, v))
    for c, ps in pts.items():
        a = np.array(ps)
        d = np.abs(a[:, None, :] - a[None, :, :]).sum(-1)
        d[np.arange(len(a)), np.arange(len(a))] = 99
        assert d.min() >= 9, c
    assert len(pts) == COLORS


def _deformed(weave, seed, W=12, H=12):
    rng = np.random.default_rng(seed)
    base = np.array([1e-3, 1e3, 1e-5])
    kw = dict(width=W, length=H, warp=base * (1 + 0.2 * (2 * rng.random((H, 3)) - 1)),
              weft=base * (1 + 0.2 * (2 * rng.random((W, 3)) - 1)), weave=weave, pose=0,
              handles=[(0, 0), (W - 1, 0)], wind_vel=(0.2, 1.0, 0.1), wind_density=1.0, wind_drag=0.5, S=1e-4, mu=0.3)
    oc = OracleCloth(ClothSpec(**kw))
    for _ in range(30):
        assert oc.step(1e-3)["status"] == 0
    st = oc.get_state()
    N = W * H
    st["LPos"] = st["LPos"] + 2e-5 * rng.standard_normal((N, 3))
    st["LVel"] = st["LVel"] + 1e-2 * rng.standard_normal((N, 3))
    return kw, st


def _residual(oc, st, q, h):
    oc.set_state(st)
    oc.fill()
    A, b = oc.system(h)
    d = oc.dense()
    return A @ q - b, d["slide"].copy()


@pytest.mark.parametrize("weave", [0, 1, 2])
def test_residual_reach_is_four(weave):
    kw, st = _deformed(weave, seed=weave + 3)
    W, H = kw["width"], kw["length"]
    oc = OracleCloth(ClothSpec(**kw))
    h = 1e-3
    rng = np.random.default_rng(7)
    q = node5_to_ref(rng.standard_normal((W * H, 5)), W, H)
    r0, _ = _residual(oc, st, q, h)
    assert np.abs(r0).max() > 0
    fields = [("LPos", 3, 1e-7), ("LVel", 3, 1e-5), ("EPos", 2, 1e-7), ("EVel", 2, 1e-5), ("EPosBar", 2, 1e-7)]
    worst = 0
    for (u, v) in [(5, 5), (6, 6), (2, 7), (1, 1), (9, 3)]:
        j = u + v * W
        for key, nc, eps in fields:
            for c in range(nc):
                sp = {k: x.copy() for k, x in st.items()}
                sm = {k: x.copy() for k, x in st.items()}
                sp[key][j, c] += eps
                sm[key][j, c] -= eps
                rp, _ = _residual(oc, sp, q, h)
                rm, _ = _residual(oc, sm, q, h)
                dr = ref_to_node5(np.abs(rp - rm) / (2 * eps), W, H).max(axis=1)
                thr = 1e-6 * max(dr.max(), 1e-300)
                for i in np.nonzero(dr > thr)[0]:
                    dist = abs(i % W - u) + abs(i // W - v)
                    worst = max(worst, dist)
                    assert dist <= 4, (key, c, (u, v), (i % W, i // W), dr[i] / dr.max())
    assert worst >= 3  # the probe reaches the far terms (normals through crimp bending)


def test_slide_indicator_reach_is_three():
    """The slide indicator of a crossing (the update's only other input from
    the assembly) depends on nodes within L1 distance 3."""
    kw, st = _deformed(1, seed=11)
    W, H = kw["width"], kw["length"]
    oc = OracleCloth(ClothSpec(**kw))
    n_in = (W - 2) * (H - 2)
    for (u, v) in [(5, 5), (3, 8)]:
        j = u + v * W
        for key, nc, eps in [("LPos", 3, 1e-7), ("EPos", 2, 1e-7), ("EPosBar", 2, 1e-7), ("LVel", 3, 1e-5),
                             ("EVel", 2, 1e-5)]:
            for c in range(nc):
                outs = []
                for sgn in (1, -1):
                    s2 = {k: x.copy() for k, x in st.items()}
                    s2[key][j, c] += sgn * eps
                    oc.set_state(s2)
                    oc.fill()
                    outs.append(np.asarray(oc.dense()["slide"]).reshape(-1)[:2 * n_in].reshape(n_in, 2).copy())
                d = np.abs(outs[0] - outs[1]).max(axis=1) / (2 * eps)
                if d.max() == 0:
                    continue
                for idx in np.nonzero(d > 1e-6 * d.max())[0]:
                    ui, vi = idx % (W - 2) + 1, idx // (W - 2) + 1
                    assert abs(ui - u) + abs(vi - v) <= 3, (key, c, (u, v), (ui, vi))


def test_line_material_reaches_neighbour_lines_only():
    kw, st = _deformed(2, seed=5)
    W, H = kw["width"], kw["length"]
    h = 1e-3
    rng = np.random.default_rng(9)
    q = node5_to_ref(rng.standard_normal((W * H, 5)), W, H)
    for orient, line in (("warp", 5), ("weft", 6)):
        outs = []
        for sgn in (1, -1):
            k2 = {k: (np.array(v, dtype=float) if k in ("warp", "weft") else v) for k, v in kw.items()}
            k2[orient][line] *= (1 + sgn * 1e-6)
            oc = OracleCloth(ClothSpec(**k2))
            outs.append(_residual(oc, st, q, h)[0])
        dr = ref_to_node5(np.abs(outs[0] - outs[1]), W, H).max(axis=1)
        for i in np.nonzero(dr > 1e-6 * dr.max())[0]:
            pos = (i // W) if orient == "warp" else (i % W)
            assert abs(pos - line) <= 1, (orient, line, i)
