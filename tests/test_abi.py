"""The C-ABI library loads on a machine without a GPU and exports every
entry point that include/magudi_gb300.h declares (no compute calls)."""
import ctypes
import os
import re
import subprocess

import pytest

from magudi_gb300 import build, capi, problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "magudi_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(mgd_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_the_entry_points():
    names = declared_functions()
    for required in ("mgd_create", "mgd_destroy", "mgd_compute_rhs", "mgd_rk4_substep",
                     "mgd_run_forward", "mgd_run_adjoint", "mgd_get_gradient"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layouts_match_header(tmp_path):
    """Sizes and field offsets of the ctypes mirrors equal the C compiler's."""
    structs = (("mgd_options", capi.Options), ("mgd_block_desc", capi.BlockDesc),
               ("mgd_patch_desc", capi.PatchDesc), ("mgd_acoustic_source", capi.AcousticSource))
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void) {"]
    for cname, pyt in structs:
        lines.append(f'printf("%s size %zu\\n", "{cname}", sizeof({cname}));')
        for fname, _ in pyt._fields_:
            lines.append(f'printf("%s %s %zu\\n", "{cname}", "{fname}", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-o", str(exe), str(src)])
    out = subprocess.check_output([str(exe)], text=True).split("\n")
    got = {}
    for line in out:
        parts = line.split()
        if len(parts) == 3:
            got[(parts[0], parts[1])] = int(parts[2])
    for cname, pyt in structs:
        assert got[(cname, "size")] == ctypes.sizeof(pyt), cname
        for fname, _ in pyt._fields_:
            assert got[(cname, fname)] == getattr(pyt, fname).offset, (cname, fname)


def test_create_without_gpu_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib.mgd_last_error.restype = ctypes.c_char_p
    o = problem.Options().to_c()
    h = ctypes.c_void_p()
    rc = lib.mgd_create(ctypes.byref(o), ctypes.byref(h))
    assert rc != 0
    assert b"CUDA" in lib.mgd_last_error(None)


def test_extent_resolution_matches_bc_dat_convention():
    p = problem.Patch("s", "SPONGE", 1, -1, (-20, -1, 1, -1, 1, -1))
    assert p.resolved_extent((201, 201, 1)) == (182, 201, 1, 201, 1, 1)


@pytest.mark.parametrize("compiler,std", [("gcc", "-std=c99"), ("g++", "-std=c++11")])
def test_header_is_strict_c_and_cxx(tmp_path, compiler, std):
    """A host that binds the library compiles the header as plain C99 or C++11,
    warnings as errors."""
    ext = "c" if compiler == "gcc" else "cpp"
    src = tmp_path / f"use.{ext}"
    src.write_text(f'#include "{HEADER}"\nint main(void) {{ mgd_ctx* c = 0; (void)c; return 0; }}\n')
    subprocess.check_call([compiler, std, "-pedantic", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", str(src)])


def _fortran_types(path):
    """Fields of every bind(C) derived type in a Fortran source: name ->
    [(field, kind, count)]."""
    import re as _re
    text = open(path).read()
    out = {}
    for m in _re.finditer(r"type, bind\(C\) :: (\w+)(.*?)end type", text, _re.S):
        fields = []
        for line in m.group(2).splitlines():
            line = line.strip()
            f = _re.match(r"(integer\(c_int\)|real\(c_double\)|character\(kind=c_char\)|type\(c_ptr\)) :: (\w+)"
                          r"(?:\((\w+)\))?$", line)
            if f:
                fields.append((f.group(2), f.group(1), f.group(3)))
        out[m.group(1)] = fields
    return out


def test_fortran_binding_mirrors_the_header():
    """include/magudi_gb300.f90 (the ISO_C_BINDING module a Fortran caller
    uses): its bind(C) types list the C structs' fields in the same order
    with the same C types, and every bind(C) function names an entry point
    of the header. (No Fortran compiler here: the check is textual.)"""
    import ctypes as C
    path = os.path.join(ROOT, "include", "magudi_gb300.f90")
    types = _fortran_types(path)
    kinds = {C.c_int: "integer(c_int)", C.c_double: "real(c_double)", C.c_char: "character(kind=c_char)",
             C.c_void_p: "type(c_ptr)"}
    for cname, pyt in (("mgd_options", capi.Options), ("mgd_block_desc", capi.BlockDesc),
                       ("mgd_patch_desc", capi.PatchDesc), ("mgd_acoustic_source", capi.AcousticSource)):
        ours = types[cname]
        assert [f[0] for f in ours] == [f[0] for f in pyt._fields_], cname
        for (fname, fkind, _), (_, ctype) in zip(ours, pyt._fields_):
            if issubclass(ctype, C._Pointer):
                base = C.c_void_p
            elif issubclass(ctype, C.Array):
                base = ctype._type_
            else:
                base = ctype
            assert fkind == kinds[base], (cname, fname)
    names = set(re.findall(r'bind\(C, name="(\w+)"\)', open(path).read())) - {"strlen"}
    declared = set(declared_functions()) | {"mgd_last_error"}
    assert names and names <= declared, names - declared
    region = open(os.path.join(ROOT, "include", "RegionGB300.f90")).read()
    assert "t_Region%computeRhs" in region and "mgd_compute_rhs(" in region
