"""Copies the reference's AcousticMonopole example inputs (magudi.inp and
bc.dat, unchanged) into tests/golden/acoustic_monopole/ and writes the
fields its examples/AcousticMonopole/config.py generates for the 201 x 201
grid (coordinates, target and control mollifiers, quiescent initial state,
mean pressure), using that config.py's own functions and the reference's
magudi_utils, as acoustic_monopole/fields.npz. Run in a container that holds
the magudi sources:
    python tests/golden/make_monopole_example_golden.py /path/to/magudi
"""
import importlib.util
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(root):
    example = os.path.join(root, "examples", "AcousticMonopole")
    sys.path.insert(0, os.path.join(root, "utils", "magudi_utils", "src"))
    spec = importlib.util.spec_from_file_location("monopole_config", os.path.join(example, "config.py"))
    cfg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(cfg)
    out_dir = os.path.join(HERE, "acoustic_monopole")
    os.makedirs(out_dir, exist_ok=True)
    for name in ("magudi.inp", "bc.dat"):
        shutil.copyfile(os.path.join(example, name), os.path.join(out_dir, name))
    gamma = 1.4
    g = cfg.grid([201, 201])
    s = cfg.p3d.Solution().copy_from(g).quiescent(gamma)
    tm = cfg.target_mollifier(g)  # prints the bc.dat rows of the patches it sizes
    cm = cfg.control_mollifier(g)
    mp = cfg.mean_pressure(s)
    # Fortran order (i fastest) as the library's (N, nComponents) layout
    xyz = g.xyz[0][:, :, 0, :2]
    coords = np.stack([xyz[:, :, 0].ravel(order="F"), xyz[:, :, 1].ravel(order="F")])
    q = s.q[0][:, :, 0, :]
    state = np.stack([q[:, :, k].ravel(order="F") for k in (0, 1, 2, 4)])
    np.savez_compressed(os.path.join(out_dir, "fields.npz"), grid_size=np.array([201, 201, 1]), coordinates=coords,
                        initial_state=state, target_mollifier=tm.f[0][:, :, 0, 0].ravel(order="F"),
                        control_mollifier=cm.f[0][:, :, 0, 0].ravel(order="F"),
                        mean_pressure=mp.f[0][:, :, 0, 0].ravel(order="F"))
    print("wrote", out_dir)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_monopole_example_golden.py <path to the magudi source tree>")
    main(sys.argv[1])
