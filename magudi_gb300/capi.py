"""ctypes mirrors of the structs and enums in include/magudi_gb300.h.

The same structs describe a problem to the CUDA library (libmagudi_gb300.so)
and, in the tests, to the CPU oracle; this module only defines the layout.
"""
import ctypes as C

MGD_MAX_BLOCKS = 8
MGD_MAX_PATCHES = 64
MGD_MAX_SOURCES = 8
MGD_NAME_LEN = 64

FORWARD = 1
ADJOINT = -1
LINEARIZED = 0

FUNCTIONAL_SOUND = 0
FUNCTIONAL_TERMINAL_KINETIC_ENERGY = 1

PERIODIC_NONE = 0
PERIODIC_PLANE = 1
PERIODIC_OVERLAP = 2

PATCH_SAT_FAR_FIELD = 1
PATCH_SPONGE = 2
PATCH_ACTUATOR = 3
PATCH_COST_TARGET = 4
PATCH_SLIP_WALL = 5
PATCH_ISOTHERMAL_WALL = 6
PATCH_ADIABATIC_WALL = 7
PATCH_BLOCK_INTERFACE = 8
PATCH_SOLENOIDAL_EXCITATION = 9

PATCH_TYPES = {
    "SAT_FAR_FIELD": PATCH_SAT_FAR_FIELD,
    "SPONGE": PATCH_SPONGE,
    "ACTUATOR": PATCH_ACTUATOR,
    "COST_TARGET": PATCH_COST_TARGET,
    "SAT_SLIP_WALL": PATCH_SLIP_WALL,
    "SAT_ISOTHERMAL_WALL": PATCH_ISOTHERMAL_WALL,
    "SAT_ADIABATIC_WALL": PATCH_ADIABATIC_WALL,
    "SAT_BLOCK_INTERFACE": PATCH_BLOCK_INTERFACE,
    "SOLENOIDAL_EXCITATION": PATCH_SOLENOIDAL_EXCITATION,
}

FIELD_CONSERVED = 0
FIELD_ADJOINT = 1
FIELD_TARGET = 2
FIELD_RHS = 3
FIELD_CONTROL_MOLLIFIER = 4
FIELD_TARGET_MOLLIFIER = 5
FIELD_MEAN_PRESSURE = 6
FIELD_METRICS = 7
FIELD_JACOBIAN = 8
FIELD_NORM = 9
FIELD_PRESSURE = 10
FIELD_TEMPERATURE = 11
FIELD_ARC_LENGTHS = 12

# defaults/discretization_scheme
SBP_48 = 0
SBP_12 = 1
SBP_24 = 2
SBP_36 = 3
SBP_SCHEMES = {"SBP 4-8": SBP_48, "SBP 1-2": SBP_12, "SBP 2-4": SBP_24, "SBP 3-6": SBP_36}

# status of a run that stopped at a solution-limit violation (cost = HUGE)
SOLUTION_LIMITS = 2


class Options(C.Structure):
    _fields_ = [
        ("n_dimensions", C.c_int),
        ("viscous", C.c_int),
        ("dissipation", C.c_int),
        ("composite_dissipation", C.c_int),
        ("curvilinear", C.c_int),
        ("use_constant_cfl", C.c_int),
        ("enable_controller", C.c_int),
        ("enable_functional", C.c_int),
        ("controller_switch", C.c_int),
        ("adjoint_forcing_switch", C.c_int),
        ("ratio_of_specific_heats", C.c_double),
        ("reynolds_number", C.c_double),
        ("prandtl_number", C.c_double),
        ("viscosity_power_law_exponent", C.c_double),
        ("bulk_viscosity_ratio", C.c_double),
        ("dissipation_amount", C.c_double),
        ("time_step_size", C.c_double),
        ("cfl", C.c_double),
        ("functional_type", C.c_int),
        ("enable_solution_limits", C.c_int),
        ("minimum_density", C.c_double),
        ("maximum_density", C.c_double),
        ("minimum_temperature", C.c_double),
        ("maximum_temperature", C.c_double),
        ("discretization_scheme", C.c_int),
    ]


class BlockDesc(C.Structure):
    _fields_ = [
        ("grid_size", C.c_int * 3),
        ("periodicity_type", C.c_int * 3),
        ("periodic_length", C.c_double * 3),
    ]


class PatchDesc(C.Structure):
    _fields_ = [
        ("name", C.c_char * MGD_NAME_LEN),
        ("type", C.c_int),
        ("grid_index", C.c_int),
        ("normal_direction", C.c_int),
        ("extent", C.c_int * 6),
        ("inviscid_penalty_amount", C.c_double),
        ("viscous_penalty_amount", C.c_double),
        ("sponge_amount", C.c_double),
        ("sponge_exponent", C.c_int),
        ("wall_temperature", C.c_double),
        ("conforms_with", C.c_char * MGD_NAME_LEN),
        ("interface_index", C.c_int * 3),
        ("n_modes", C.c_int),
        ("origin", C.c_double * 2),
        ("velocity", C.c_double * 2),
        ("amplitude", C.c_double),
        ("radius", C.c_double),
        ("angular_frequencies", C.POINTER(C.c_double)),
        ("phases", C.POINTER(C.c_double)),
    ]


class AcousticSource(C.Structure):
    _fields_ = [
        ("location", C.c_double * 3),
        ("amplitude", C.c_double),
        ("frequency", C.c_double),
        ("radius", C.c_double),
        ("phase", C.c_double),
    ]


def dptr(a):
    """Pointer to the data of a C-contiguous float64 numpy array."""
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))
