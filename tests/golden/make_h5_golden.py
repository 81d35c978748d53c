"""Generates tests/golden/h5_wind_yarn12_plain5.npz from the trajectory file
the reference ships (TrainingData/Table_2/Wind_Yarn_1_2_Plain_Size5.h5, written
by its Saver through libhdf5): the file's SHA-256, its property records and
the first STEPS steps plus the last step of every node, read with the
package's own HDF5 reader (h5.py).

Run from the repo root:  python tests/golden/make_h5_golden.py [reference root]
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, ".."))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from pkg import ys  # noqa: E402

STEPS = 40
REL = os.path.join("TrainingData", "Table_2", "Wind_Yarn_1_2_Plain_Size5.h5")


def main():
    from oracle.ref.refpath import ref_root
    root = sys.argv[1] if len(sys.argv) > 1 else ref_root()
    if root is None:
        sys.exit("the reference checkout is not here (set REF_ROOT)")
    path = os.path.join(root, REL)
    raw = open(path, "rb").read()
    size, phy = ys.h5.cloth_property_loader_heter(path)
    head = ys.h5.data_loader(path, 0, STEPS)
    n = len(ys.h5.read(path)["/Steps/Position/Node 0 0/LPOS"])
    last = ys.h5.data_loader(path, n - 1, n)
    out = dict(sha256=np.array(hashlib.sha256(raw).hexdigest()), width=size["width"], length=size["length"],
               physical_names=np.array(list(phy)), physical=np.array([float(v) for v in phy.values()]),
               n_steps=n)
    for k in head:
        out[k] = head[k]
        out["last_" + k] = last[k][0]
    np.savez_compressed(os.path.join(HERE, "h5_wind_yarn12_plain5.npz"), **out)
    print("wrote h5_wind_yarn12_plain5.npz: %d x %d cloth, %d of %d steps" % (size["width"], size["length"], STEPS, n))


if __name__ == "__main__":
    main()
