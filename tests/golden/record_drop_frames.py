"""Records detection inputs of the collision benchmark scene for the
reference's pair lists (step 1 of 2; needs a GPU).

Runs the 50 x 50 drop onto the 1,280-face sphere (DropOnSphere: h = 5e-4,
self-collision) for `steps` steps and saves, for a few frames -- the first
step with impacts, ten steps later, and steps 400, 700 and the last -- the
positions at the start and at the end of the step (the detection's x_prev
and x), with the sphere mesh and the thickness.

Step 2, here with the reference sources: tests/golden/make_collide_golden.py
frames <npz> runs the reference's own BVH in the harness on those frames.

    python tests/golden/record_drop_frames.py OUT.npz [steps]
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
from pkg import ys  # noqa: E402


def main(out, steps=1000):
    sc = ys.DropOnSphere(width=50, radius=0.03, levels=3, drop=0.05, h=5e-4)
    try:
        want = set(range(150, 320)) | {400, 700, steps - 1}
        log = sc.run(steps, frames=sorted(s for s in want if s < steps))
        contact = [e["step"] for e in log if e.get("impacts", 0) > 0]
        first = contact[0] if contact else None
        pick = [s for s in (first, None if first is None else first + 10, 400, 700, steps - 1)
                if s is not None and s in sc.frames]
        data = dict(width=50, length=50, thickness=sc.thickness, obs_x=sc.sphere_x, obs_faces=sc.sphere_f,
                    frames=np.array(pick), first_contact=-1 if first is None else first)
        for s in pick:
            data["x_prev_%d" % s], data["x_%d" % s] = sc.frames[s]
        np.savez_compressed(out, **data)
        print("frames", pick, "first contact", first, "all converged",
              all(e.get("converged", False) for e in log), "steps run", len(log))
    finally:
        sc.close()


if __name__ == "__main__":
    main(sys.argv[1], int(sys.argv[2]) if len(sys.argv) > 2 else 1000)
