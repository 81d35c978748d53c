"""OBJ output against the reference's own RenderCloth (src/Render.cpp): the
text for the reference's final state is byte-identical in all three forms
(fixtures from tests/golden/make_render_golden.py); on the GPU, the same text
from the device state after the same steps, to the printed precision."""
import glob
import os

import numpy as np
import pytest

import goldens
from pkg import gpu_available, spec_from_golden, ys

NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(goldens.GOLDEN_DIR, "render_*.npz")))
KINDS = [("tri", ys.RenderType.MeshTriangle), ("rect", ys.RenderType.MeshRectangle),
         ("yarn", ys.RenderType.YarnSpline)]


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("kind", KINDS, ids=[k[0] for k in KINDS])
def test_obj_text_equals_reference(name, kind):
    g = goldens.load(name)
    s = int(g["steps"])
    text = ys.obj_text(int(g["width"]), int(g["length"]), g["s%d_LPos" % s], kind[1], g["s%d_normal" % s],
                       float(g["R"]))
    assert text == str(g["obj_" + kind[0]])


def _numbers(text):
    vals = []
    for line in text.splitlines():
        parts = line.split()
        if parts and parts[0] in ("v", "vt", "vn"):
            vals += [float(x) for x in parts[1:]]
    return np.array(vals)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_state_renders_like_the_reference(name, tmp_path):
    if not gpu_available():
        pytest.skip("no CUDA device")
    g = goldens.load(name)
    b = ys.ClothBatch([spec_from_golden(g)])
    b.set_state(**goldens.init_state(g))
    for _ in range(int(g["steps"])):
        assert all(x["ok"] for x in b.step(float(g["h"]), tol=1e-12))
    for key, kind in KINDS:
        text = ys.render_batch_cloth(b, 0, str(tmp_path / (key + ".obj")), kind)
        ref = str(g["obj_" + key])
        assert [l.split()[0] for l in text.splitlines()] == [l.split()[0] for l in ref.splitlines()]
        assert [l for l in text.splitlines() if l[:1] in "fl"] == [l for l in ref.splitlines() if l[:1] in "fl"]
        assert np.abs(_numbers(text) - _numbers(ref)).max() <= 1.01e-5
    b.close()
