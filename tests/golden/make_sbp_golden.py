"""Generates tests/golden/sbp48_first_derivative.npz (SBP 4-8) and
tests/golden/sbp_first_derivative_schemes.npz (SBP 1-2, 2-4, 3-6) from the reference's own
Python SBP implementation (magudi_utils/SummationByParts.py, function
`derivative`), run unmodified from the magudi source tree.

Run in a container that holds the magudi sources:
    python tests/golden/make_sbp_golden.py /path/to/magudi

`derivative` indexes arrays with lists of slices, which numpy 2 rejects; the
input is therefore wrapped in an ndarray subclass whose __getitem__ and
__setitem__ turn such a list into a tuple before numpy sees it. The
arithmetic is the reference's.
"""
import os
import sys

import numpy as np


class _TupleIndexed(np.ndarray):
    @staticmethod
    def _fix(key):
        return tuple(key) if isinstance(key, list) else key

    def __getitem__(self, key):
        return np.ndarray.__getitem__(self, self._fix(key))

    def __setitem__(self, key, value):
        return np.ndarray.__setitem__(self, self._fix(key), value)


def main(magudi_root):
    sys.path.insert(0, os.path.join(magudi_root, "utils", "magudi_utils", "src"))
    from magudi_utils.SummationByParts import derivative

    rng = np.random.default_rng(20240611)
    out = {}
    for n in (24, 37, 64):
        x = rng.standard_normal((n, 5))
        d = derivative(x.view(_TupleIndexed), order=1, axis=0, scheme="SBP 4-8")
        out[f"x_{n}"] = x
        out[f"dx_{n}"] = np.asarray(d)
    # smooth input: derivative of sin on a uniform grid with unit spacing
    t = np.arange(50, dtype=np.float64)
    s = np.sin(0.2 * t)[:, None]
    out["x_sin"] = s
    out["dx_sin"] = np.asarray(derivative(s.view(_TupleIndexed), order=1, axis=0, scheme="SBP 4-8"))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sbp48_first_derivative.npz")
    np.savez(path, **out)
    print("wrote", path)
    # the other schemes of the same function, one random input per size
    other = {}
    for scheme in ("SBP 1-2", "SBP 2-4", "SBP 3-6"):
        tag = scheme.replace("SBP ", "").replace("-", "")
        for n in (24, 37):
            x = rng.standard_normal((n, 3))
            other[f"s{tag}_x_{n}"] = x
            other[f"s{tag}_dx_{n}"] = np.asarray(derivative(x.view(_TupleIndexed), order=1, axis=0, scheme=scheme))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sbp_first_derivative_schemes.npz")
    np.savez(path, **other)
    print("wrote", path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_sbp_golden.py <path to the magudi source tree>")
    main(sys.argv[1])
