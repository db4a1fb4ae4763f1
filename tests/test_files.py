"""File formats around the hot path (CPU): the library's PLOT3D writer and
reader against files written by the reference's own Python writer
(tests/golden/make_plot3d_golden.py), and the actuator-patch streams."""
import ctypes as C
import os

import numpy as np

from magudi_gb300.solver import load_library

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def _fields():
    sizes = [(5, 4, 1), (3, 6, 1)]
    xyz, q, ib = [], [], []
    for b, (nx, ny, nz) in enumerate(sizes):
        n = nx * ny * nz
        t = np.arange(n, dtype=np.float64)
        xyz.append(np.ascontiguousarray(np.stack([0.5 * t + b, 0.25 * t - b])))
        q.append(np.ascontiguousarray(np.stack([1.0 + 0.01 * t, 0.1 * t, -0.2 * t, 2.5 + 0.03 * t + b])))
        i = np.ones(n, dtype=np.int32)
        i[b] = 0
        ib.append(i)
    return sizes, xyz, q, ib


def _ptrs(arrays, ctype=C.c_double):
    return (C.POINTER(ctype) * len(arrays))(*[a.ctypes.data_as(C.POINTER(ctype)) for a in arrays])


def _lib():
    L = load_library()
    L.mgd_plot3d_write_grid.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.c_int,
                                        C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.POINTER(C.c_int))]
    L.mgd_plot3d_write_solution.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.c_int,
                                            C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_double)]
    L.mgd_plot3d_read_solution.argtypes = L.mgd_plot3d_write_solution.argtypes
    L.mgd_write_patch_stream.argtypes = [C.c_char_p, C.POINTER(C.c_double), C.c_longlong, C.c_longlong,
                                         C.c_longlong, C.c_longlong]
    L.mgd_read_patch_stream.argtypes = L.mgd_write_patch_stream.argtypes
    return L


def test_plot3d_files_match_the_reference_writer(tmp_path):
    L = _lib()
    sizes, xyz, q, ib = _fields()
    gs = (C.c_int * 6)(*[s for sz in sizes for s in sz])
    grid = str(tmp_path / "g.xyz").encode()
    assert L.mgd_plot3d_write_grid(grid, 2, gs, 2, _ptrs(xyz), _ptrs(ib, C.c_int)) == 0
    assert open(grid, "rb").read() == open(os.path.join(GOLD, "plot3d_two_blocks.xyz"), "rb").read()
    sol = str(tmp_path / "s.q").encode()
    aux = (C.c_double * 4)(0.0, 0.0, 0.0, 12.5)
    assert L.mgd_plot3d_write_solution(sol, 2, gs, 4, _ptrs(q), aux) == 0
    assert open(sol, "rb").read() == open(os.path.join(GOLD, "plot3d_two_blocks.q"), "rb").read()


def test_plot3d_solution_reader_on_the_golden_file():
    L = _lib()
    sizes, _, q, _ = _fields()
    gs = (C.c_int * 6)(*[s for sz in sizes for s in sz])
    out = [np.zeros_like(a) for a in q]
    aux = (C.c_double * 4)()
    assert L.mgd_plot3d_read_solution(os.path.join(GOLD, "plot3d_two_blocks.q").encode(), 2, gs, 4,
                                      _ptrs(out), aux) == 0
    for a, b in zip(out, q):
        assert np.array_equal(a, b)
    assert aux[3] == 12.5
    wrong = (C.c_int * 6)(5, 4, 1, 3, 5, 1)
    assert L.mgd_plot3d_read_solution(os.path.join(GOLD, "plot3d_two_blocks.q").encode(), 2, wrong, 4,
                                      _ptrs(out), aux) != 0


def test_patch_streams_round_trip(tmp_path):
    """Raw entries in file order, one patch's points per entry (two patches interleaved in memory)."""
    L = _lib()
    rng = np.random.default_rng(0)
    entries = np.ascontiguousarray(rng.standard_normal((7, 10)))
    f = str(tmp_path / "p.dat").encode()
    ptr = entries.ctypes.data_as(C.POINTER(C.c_double))
    assert L.mgd_write_patch_stream(f, ptr, 7, 4, 10, 6) == 0
    raw = np.fromfile(f, dtype=np.float64).reshape(7, 4)
    assert np.array_equal(raw, entries[:, 6:10])
    back = np.zeros((7, 10))
    assert L.mgd_read_patch_stream(f, back.ctypes.data_as(C.POINTER(C.c_double)), 7, 4, 10, 6) == 0
    assert np.array_equal(back[:, 6:], entries[:, 6:]) and not back[:, :6].any()
