"""magudi.inp / bc.dat front end (CPU)."""
import numpy as np
import pytest

from magudi_gb300 import capi, inputs
from magudi_gb300.capi import PERIODIC_PLANE

INP = """# comment line
output_prefix = "AcousticMonopole"
include_viscous_terms = true
use_constant_CFL_mode = false
curvilinear_domain = false
Reynolds_number = 200.
Prandtl_number = 0.72   # trailing comment
add_dissipation = true
dissipation_amount = 0.01
time_step_size = 0.05
defaults/sponge_amount = 0.2
patches/farField.E/viscous_penalty_amount = 0.5
number_of_acoustic_sources = 1
acoustic_source01/amplitude = 0.01
acoustic_source01/x = -3.
grid001/dir1/periodicity_type = "PLANE"
grid001/dir1/periodic_length = 6.283185307179586
"""

BC = """# Name                 Type                  Grid normDir iMin iMax jMin jMax kMin kMax
  farField.E           SAT_FAR_FIELD            1       1    1    1    1   -1    1   -1
  sponge.E             SPONGE                   1       1    1   29    1   -1    1   -1
  controlRegion        ACTUATOR                 1       0  108  137   86  116    1   -1
"""


def test_parse_and_map(tmp_path):
    (tmp_path / "magudi.inp").write_text(INP)
    (tmp_path / "bc.dat").write_text(BC)
    d = inputs.parse_input_file(tmp_path / "magudi.inp")
    assert d.get_str("output_prefix") == "AcousticMonopole"
    o = inputs.options_from_inputs(d, 2)
    assert o.viscous and o.dissipation and not o.curvilinear and not o.use_constant_cfl
    assert o.reynolds_number == 200.0 and o.prandtl_number == 0.72
    assert o.composite_dissipation  # reference default
    assert o.viscosity_power_law_exponent == 0.666 and o.bulk_viscosity_ratio == 0.6
    rows = inputs.read_bc_dat(tmp_path / "bc.dat")
    ps = inputs.patches_from_bc(d, rows)
    assert [p.type for p in ps] == ["SAT_FAR_FIELD", "SPONGE", "ACTUATOR"]
    assert ps[0].viscous_penalty_amount == 0.5 and ps[0].inviscid_penalty_amount == 1.0
    assert ps[1].sponge_amount == 0.2 and ps[1].sponge_exponent == 2
    src = inputs.sources_from_inputs(d, 2)
    assert len(src) == 1 and src[0].location[0] == -3.0 and src[0].amplitude == 0.01
    types, lengths = inputs.block_periodicity(d, 1, 2)
    assert types[0] == PERIODIC_PLANE and abs(lengths[0] - 6.283185307179586) < 1e-15


def test_errors(tmp_path):
    (tmp_path / "bad.inp").write_text("a = b = c\n")
    with pytest.raises(inputs.InputError):
        inputs.parse_input_file(tmp_path / "bad.inp")
    (tmp_path / "dup.dat").write_text(BC + "  farField.E SAT_FAR_FIELD 1 1 1 1 1 -1 1 -1\n")
    with pytest.raises(inputs.InputError):
        inputs.read_bc_dat(tmp_path / "dup.dat")
    (tmp_path / "m.inp").write_text("add_dissipation = true\n")
    with pytest.raises(inputs.InputError):
        inputs.options_from_inputs(inputs.parse_input_file(tmp_path / "m.inp"), 2)


def test_round_trip(tmp_path):
    from magudi_gb300 import configs
    P = configs.monopole_2d(n=41)
    inputs.write_bc_dat(tmp_path / "bc.dat", P.patches)
    rows = inputs.read_bc_dat(tmp_path / "bc.dat")
    assert [r[4] for r in rows] == [tuple(p.extent) for p in P.patches]


def test_wall_and_interface_keys(tmp_path):
    """Wall and block-interface options keep the reference's key names and
    defaults (src/IsothermalWallImpl.f90:3-80, src/BlockInterfacePatchImpl.f90:72-86,
    src/InterfaceHelperImpl.f90:3-113)."""
    inp = """include_viscous_terms = true
Reynolds_number = 100.
use_constant_CFL_mode = false
time_step_size = 0.01
use_target_state = false
patches/wall.S/viscous_penalty_amount1 = 2.0
patches/wall.S/temperature = 3.5
patches/interface.1E/conforms_with = "interface.2W"
patches/interface.1E/interface_index1 = 2
patches/interface.1E/interface_index2 = -1
"""
    bc = """  wall.S          SAT_ISOTHERMAL_WALL   1   2   1 -1  1  1  1 -1
  interface.1E    SAT_BLOCK_INTERFACE   1  -1  -1 -1  1 -1  1 -1
  interface.2W    SAT_BLOCK_INTERFACE   2   1   1  1  1 -1  1 -1
  slip.N          SAT_SLIP_WALL         1  -2   1 -1 -1 -1  1 -1
"""
    (tmp_path / "magudi.inp").write_text(inp)
    (tmp_path / "bc.dat").write_text(bc)
    d = inputs.parse_input_file(tmp_path / "magudi.inp")
    ps = inputs.patches_from_bc(d, inputs.read_bc_dat(tmp_path / "bc.dat"))
    assert ps[0].viscous_penalty_amount == 2.0 and ps[0].wall_temperature == 3.5
    assert ps[1].conforms_with == "interface.2W" and ps[1].interface_index == (2, -1, 3)
    assert ps[1].viscous_penalty_amount == 0.5  # interface default
    assert ps[2].conforms_with == "" and ps[2].interface_index == (1, 2, 3)
    assert ps[3].type == "SAT_SLIP_WALL"


def test_solenoidal_excitation_keys(tmp_path):
    inp = """patches/excitationSupport/number_of_modes = 8
patches/excitationSupport/origin_x = 1.5
patches/excitationSupport/velocity_x = 0.65
patches/excitationSupport/amplitude = 1.0d-3
patches/excitationSupport/frequency = 0.3
patches/excitationSupport/radius = 2.0
patches/excitationSupport/random_seed = 12
"""
    bc = "  excitationSupport    SOLENOIDAL_EXCITATION    1       0   69  186  248  393    1   -1\n"
    (tmp_path / "magudi.inp").write_text(inp)
    (tmp_path / "bc.dat").write_text(bc)
    d = inputs.parse_input_file(tmp_path / "magudi.inp")
    (p,) = inputs.patches_from_bc(d, inputs.read_bc_dat(tmp_path / "bc.dat"))
    assert p.n_modes == 8 and p.origin == (1.5, 0.0) and p.velocity == (0.65, 0.0)
    assert p.amplitude == 1e-3 and p.frequency == 0.3 and p.radius == 2.0 and p.random_seed == 12
    w, ph = p.excitation_modes()
    # angular frequency l = 2 pi f (l + r_l - 1/2) / (n / 2), r_l in [0, 1)
    l = np.arange(1, 9)
    lo = 2 * np.pi * 0.3 * (l - 0.5) / 4.0
    hi = 2 * np.pi * 0.3 * (l + 0.5) / 4.0
    assert np.all((w >= lo) & (w < hi))
    assert ph.shape == (8, 3) and np.all((ph >= 0) & (ph < 2 * np.pi))
    c = p.to_c()
    assert c.type == capi.PATCH_SOLENOIDAL_EXCITATION and c.n_modes == 8
    assert c.angular_frequencies[3] == w[3] and c.phases[8 + 2] == ph[2, 1]
    (tmp_path / "magudi.inp").write_text(inp.replace("patches/excitationSupport/radius = 2.0\n", ""))
    d = inputs.parse_input_file(tmp_path / "magudi.inp")
    with pytest.raises(inputs.InputError):
        inputs.patches_from_bc(d, inputs.read_bc_dat(tmp_path / "bc.dat"))
