"""Writes small PLOT3D grid and solution files with the reference's own
Python writer (magudi_utils.plot3dnasa, unmodified) as golden fixtures for
the library's PLOT3D writer and reader. Run from the repository root:
    python tests/golden/make_plot3d_golden.py /path/to/magudi
"""
import os
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_plot3d_golden.py <path to the magudi source tree>")
root = sys.argv[1]
sys.path.insert(0, os.path.join(root, "utils", "magudi_utils", "src"))
import magudi_utils.plot3dnasa as p3d  # noqa: E402


class Arr(np.ndarray):
    """The reference writer calls ndarray.tostring, which NumPy 2 spells tobytes."""

    def tostring(self, order="C"):
        return self.tobytes(order=order)


def arr(a):
    return np.asarray(a).view(Arr)

HERE = os.path.dirname(os.path.abspath(__file__))


def fields():
    """Two 2D blocks (sizes (5, 4, 1) and (3, 6, 1)) with deterministic values;
    iblank is 0 at point b of block b."""
    sizes = [(5, 4, 1), (3, 6, 1)]
    xyz, q = [], []
    for b, (nx, ny, nz) in enumerate(sizes):
        n = nx * ny * nz
        t = np.arange(n, dtype=np.float64)
        xyz.append(np.stack([0.5 * t + b, 0.25 * t - b, np.zeros(n)]))
        q.append(np.stack([1.0 + 0.01 * t, 0.1 * t, -0.2 * t, np.zeros(n), 2.5 + 0.03 * t + b]))
    return sizes, xyz, q


def main():
    sizes, xyz, q = fields()
    g = p3d.Grid()
    g.has_iblank = True  # magudi's grid files carry iblank (src/PLOT3DFormat.c:260-267)
    g.set_size([list(s) for s in sizes], True)
    g.size = arr(g.size)
    for b, (nx, ny, nz) in enumerate(sizes):
        g.xyz[b] = arr(np.asfortranarray(xyz[b].T.reshape(nx, ny, nz, 3, order="F")))
        ib = np.ones(nx * ny * nz, dtype=np.int32)
        ib[b] = 0  # one hole per block
        g.iblank[b] = arr(np.asfortranarray(ib.reshape(nx, ny, nz, order="F")))
    g.save(os.path.join(HERE, "plot3d_two_blocks.xyz"))
    s = p3d.Solution()
    s.set_size([list(s_) for s_ in sizes], True)
    s.size = arr(s.size)
    s._format.aux_header = arr(np.zeros(4))
    s.time = 12.5
    for b, (nx, ny, nz) in enumerate(sizes):
        s.q[b] = arr(np.asfortranarray(q[b].T.reshape(nx, ny, nz, 5, order="F")))
    s.save(os.path.join(HERE, "plot3d_two_blocks.q"))


if __name__ == "__main__":
    main()
