"""Writes the regression fixtures of the FP64 oracle (test infrastructure):

* oracle_plain.npz     per-path radiance of the plain box at 8 x 8 pixels x 4 spp (depth 5, RR from
                       3, seed 7), and its kd-tree serialisation (node kinds, splits, leaf counts,
                       leaf primitives)
* oracle_textured.npz  per-path radiance of the textured box (image maps, bump map) at 6 x 6 x 4

These pin the oracle's own outputs so that a change to the restatement is seen; they are not
reference outputs (the reference has no runnable build here).  Regenerate deliberately with

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
from milton_gb300 import scenegen  # noqa: E402
from oracle import pyoracle as O  # noqa: E402


def plain_case():
    s = scenegen.plain(0)
    tree = O.Tree(s.tri_v)
    _, paths, _ = O.render(s, tree, 8, 8, 4, max_depth=5, rr_start=3, seed=7, per_path=True, threads=1)
    kind, split, count, prims = tree.serialize()
    return dict(paths=paths, kind=kind, split=split, count=count, prims=prims)


def textured_case():
    s = scenegen.textured(0)
    _, paths, _ = O.render(s, O.Tree(s.tri_v), 6, 6, 4, max_depth=5, rr_start=3, seed=3, per_path=True, threads=1)
    return dict(paths=paths)


def main():
    np.savez_compressed(HERE / "oracle_plain.npz", **plain_case())
    np.savez_compressed(HERE / "oracle_textured.npz", **textured_case())


if __name__ == "__main__":
    main()
