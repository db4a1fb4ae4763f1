"""Golden data from the reference's TestForcing example (a 4 x 4 periodic
grid, SBP 2-4, non-composite dissipation, viscous, thermal actuator and
sound functional over the whole grid, 8 RK4 steps): its magudi.inp, bc.dat,
initial condition (TestForcing.ic.q) and baseline control forcing
(baseline.dat) copied unchanged into tests/golden/test_forcing/; the grid
and mollifiers its config.py generates, and the initial condition read from
the PLOT3D file (whole format, 4-byte record markers), as fields.npz; and the
numbers the
reference's Fortran build printed for this case, taken from the cell outputs
of the example's notebook (examples/TestForcing/Untitled.ipynb): the cost
functional of the forward runs with control forcing A x gradient + baseline
for the 32 amplitudes of its gradient-accuracy loop, and the printed J and
adjoint sensitivity, as reference_outputs.json. Run in a container that holds
the magudi sources:
    python tests/golden/make_test_forcing_golden.py /path/to/magudi
"""
import importlib.util
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def notebook_outputs(path):
    """(printed J, printed sensitivity, [(A, J)]) from the notebook's cells:
    the outputs of the cells that print QoI0 and Grad0, and the rows
    (A, J, (J - QoI0) / A, error) of the gradient-accuracy loop."""
    nb = json.load(open(path))

    def output_of(marker):
        for cell in nb["cells"]:
            if marker in "".join(cell["source"]):
                for o in cell.get("outputs", []):
                    t = o.get("text") or o.get("data", {}).get("text/plain")
                    if t:
                        return "".join(t).strip()
        raise KeyError(marker)

    printed_j = float(output_of("print QoI0"))
    printed_grad = float(output_of("print Grad0"))
    table = output_of("Nk = 32")
    rows = [tuple(float(v) for v in line.split()[:2]) for line in table.splitlines()]
    return printed_j, printed_grad, rows


def read_plot3d_solution(path):
    """(grid size, q as (5, nk, nj, ni)) of a single-grid PLOT3D whole-format
    solution file with 4-byte record markers, native little-endian."""
    import struct
    b = open(path, "rb").read()
    pos = 0

    def record():
        nonlocal pos
        n = struct.unpack_from("<i", b, pos)[0]
        data = b[pos + 4:pos + 4 + n]
        pos += n + 8
        return data

    (n_grids,) = struct.unpack("<i", record())
    assert n_grids == 1
    dims = struct.unpack("<3i", record())
    record()  # freestream Mach number, angle of attack, Reynolds number, time
    q = np.frombuffer(record(), dtype="<f8").reshape(5, dims[2], dims[1], dims[0])
    return dims, q


def main(root):
    example = os.path.join(root, "examples", "TestForcing")
    sys.path.insert(0, os.path.join(root, "utils", "magudi_utils", "src"))
    spec = importlib.util.spec_from_file_location("test_forcing_config", os.path.join(example, "config.py"))
    cfg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(cfg)
    out_dir = os.path.join(HERE, "test_forcing")
    os.makedirs(out_dir, exist_ok=True)
    for name in ("magudi.inp", "bc.dat", "TestForcing.ic.q", "baseline.dat"):
        shutil.copyfile(os.path.join(example, name), os.path.join(out_dir, name))
    g = cfg.grid([4, 4])
    tm = cfg.target_mollifier(g)  # prints the bc.dat rows of the patches it sizes
    cm = cfg.control_mollifier(g)
    dims, q = read_plot3d_solution(os.path.join(example, "TestForcing.ic.q"))
    assert dims == (4, 4, 1)
    xyz = g.xyz[0][:, :, 0, :2]
    coords = np.stack([xyz[:, :, 0].ravel(order="F"), xyz[:, :, 1].ravel(order="F")])
    # (density, x and y momentum, energy), i fastest
    state = np.stack([q[k, 0].ravel() for k in (0, 1, 2, 4)])
    np.savez_compressed(os.path.join(out_dir, "fields.npz"), grid_size=np.array([4, 4, 1]), coordinates=coords,
                        initial_state=state, target_mollifier=tm.f[0][:, :, 0, 0].ravel(order="F"),
                        control_mollifier=cm.f[0][:, :, 0, 0].ravel(order="F"))
    printed_j, printed_grad, rows = notebook_outputs(os.path.join(example, "Untitled.ipynb"))
    json.dump({"source": "examples/TestForcing/Untitled.ipynb, cell outputs of the reference's forward and adjoint "
                         "runs (./forward, ./adjoint, ./zaxpy) of this example",
               "printed_cost": printed_j, "printed_sensitivity": printed_grad,
               "amplitudes": [a for a, _ in rows], "costs": [j for _, j in rows]},
              open(os.path.join(out_dir, "reference_outputs.json"), "w"), indent=1)
    print("wrote", out_dir)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_test_forcing_golden.py <path to the magudi source tree>")
    main(sys.argv[1])
