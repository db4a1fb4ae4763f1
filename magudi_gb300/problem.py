"""Problem description shared by every front end of the library.

A Problem holds what magudi reads from magudi.inp, bc.dat and the PLOT3D
input files for one region: options, blocks (grid coordinates and iblank),
patches, acoustic sources and the initial, target and mollifier fields.

Array convention: a field with nc components on a block of N points is a
float64 numpy array of shape (nc, N), C-contiguous, so that component c of
point p = i + Nx*(j + Ny*k) sits at flat index p + N*c -- magudi's Fortran
column-major x(N, nc) layout.
"""
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import capi


@dataclass
class Options:
    """Hot-path keys of magudi.inp (src/SimulationFlagsImpl.f90:24-45,
    src/SolverOptionsImpl.f90:46-135). Defaults are the reference defaults."""

    n_dimensions: int = 2
    viscous: bool = False
    dissipation: bool = False
    composite_dissipation: bool = True
    curvilinear: bool = True
    use_constant_cfl: bool = True
    enable_controller: bool = False
    enable_functional: bool = False
    controller_switch: bool = False
    adjoint_forcing_switch: bool = True
    ratio_of_specific_heats: float = 1.4
    reynolds_number: float = 0.0
    prandtl_number: float = 0.72
    viscosity_power_law_exponent: float = 0.666
    bulk_viscosity_ratio: float = 0.6
    dissipation_amount: float = 0.0
    time_step_size: float = 0.0
    cfl: float = 0.5
    functional_type: int = 0  # capi.FUNCTIONAL_SOUND or FUNCTIONAL_TERMINAL_KINETIC_ENERGY
    # enable_solution_limits and its required ranges (src/SolverOptionsImpl.f90:73-78)
    enable_solution_limits: bool = False
    minimum_density: float = 0.0
    maximum_density: float = 0.0
    minimum_temperature: float = 0.0
    maximum_temperature: float = 0.0
    discretization_scheme: int = 0  # capi.SBP_*: SBP 4-8, 1-2, 2-4 or 3-6

    def to_c(self) -> capi.Options:
        o = capi.Options()
        for name, _ in capi.Options._fields_:
            v = getattr(self, name)
            setattr(o, name, int(v) if isinstance(v, bool) else v)
        return o


@dataclass
class Patch:
    """One bc.dat row and its patches/<name>/... options."""

    name: str
    type: str
    grid_index: int
    normal_direction: int
    extent: tuple  # (iMin, iMax, jMin, jMax, kMin, kMax), bc.dat convention
    inviscid_penalty_amount: float = 1.0
    viscous_penalty_amount: float = 1.0
    sponge_amount: float = 1.0
    sponge_exponent: int = 2
    wall_temperature: float = 0.0  # isothermal walls: <= 0 takes the target state's temperature
    conforms_with: str = ""        # block interfaces: name of the conforming patch
    interface_index: tuple = (0, 0, 0)  # block interfaces: index reordering (0 = 1, 2, 3)
    # solenoidal excitation (patches/<name>/number_of_modes, origin_x/y, velocity_x/y,
    # amplitude, frequency, radius, random_seed, randomize_frequency)
    n_modes: int = 0
    origin: tuple = (0.0, 0.0)
    velocity: tuple = (0.0, 0.0)
    amplitude: float = 0.0
    frequency: float = 0.0
    radius: float = 1.0
    random_seed: int = -1
    randomize_frequency: bool = True
    # explicit modes (angular frequencies (n_modes), phases (n_modes, 3)) override the seeded draw
    angular_frequencies: object = None
    phases: object = None

    def excitation_modes(self):
        """Angular frequencies (n_modes) and phases (n_modes, 3) of a solenoidal
        excitation patch: the explicit arrays when given, else `solenoidal_modes`."""
        if self.angular_frequencies is not None:
            return (np.ascontiguousarray(self.angular_frequencies, dtype=np.float64),
                    np.asarray(self.phases, dtype=np.float64).reshape(self.n_modes, 3))
        return solenoidal_modes(self.n_modes, self.frequency, self.random_seed, self.randomize_frequency)

    def to_c(self) -> capi.PatchDesc:
        p = capi.PatchDesc()
        p.name = self.name.encode()[: capi.MGD_NAME_LEN - 1]
        p.type = capi.PATCH_TYPES[self.type]
        p.grid_index = self.grid_index
        p.normal_direction = self.normal_direction
        for i in range(6):
            p.extent[i] = int(self.extent[i])
        p.inviscid_penalty_amount = self.inviscid_penalty_amount
        p.viscous_penalty_amount = self.viscous_penalty_amount
        p.sponge_amount = self.sponge_amount
        p.sponge_exponent = int(self.sponge_exponent)
        p.wall_temperature = float(self.wall_temperature)
        p.conforms_with = self.conforms_with.encode()[: capi.MGD_NAME_LEN - 1]
        for i in range(3):
            p.interface_index[i] = int(self.interface_index[i])
        if self.type == "SOLENOIDAL_EXCITATION" and self.n_modes > 0:
            w, ph = self.excitation_modes()
            # the C struct points into these arrays: keep them alive with the patch
            self._modes = (np.ascontiguousarray(w), np.ascontiguousarray(ph.T).ravel())
            p.n_modes = int(self.n_modes)
            p.angular_frequencies = capi.dptr(self._modes[0])
            p.phases = capi.dptr(self._modes[1])
        p.origin[0], p.origin[1] = (float(x) for x in self.origin)
        p.velocity[0], p.velocity[1] = (float(x) for x in self.velocity)
        p.amplitude = float(self.amplitude)
        p.radius = float(self.radius)
        return p

    def resolved_extent(self, grid_size):
        """Extent with negative indices counted from the end
        (src/PatchDescriptorImpl.f90:57-63); unused dimensions become 1..1."""
        e = list(self.extent)
        out = []
        for i in range(3):
            lo, hi = e[2 * i], e[2 * i + 1]
            if grid_size[i] == 1:
                lo, hi = 1, 1
            if lo < 0:
                lo += grid_size[i] + 1
            if hi < 0:
                hi += grid_size[i] + 1
            out += [lo, hi]
        return tuple(out)


@dataclass
class AcousticSource:
    location: tuple
    amplitude: float
    frequency: float
    radius: float
    phase: float = 0.0

    def to_c(self) -> capi.AcousticSource:
        s = capi.AcousticSource()
        for i in range(3):
            s.location[i] = self.location[i] if i < len(self.location) else 0.0
        s.amplitude, s.frequency, s.radius, s.phase = (
            self.amplitude, self.frequency, self.radius, self.phase)
        return s


@dataclass
class Block:
    grid_size: tuple  # (Nx, Ny, Nz), Nz = 1 in 2D
    coordinates: np.ndarray  # (nD, N)
    iblank: Optional[np.ndarray] = None  # (N,) int32
    periodicity_type: tuple = (0, 0, 0)
    periodic_length: tuple = (0.0, 0.0, 0.0)
    initial_state: Optional[np.ndarray] = None  # (nU, N)
    target_state: Optional[np.ndarray] = None  # (nU, N)
    control_mollifier: Optional[np.ndarray] = None  # (N,)
    target_mollifier: Optional[np.ndarray] = None  # (N,)
    mean_pressure: Optional[np.ndarray] = None  # (N,)

    @property
    def n_points(self) -> int:
        return int(np.prod(self.grid_size))

    def desc(self) -> capi.BlockDesc:
        d = capi.BlockDesc()
        for i in range(3):
            d.grid_size[i] = int(self.grid_size[i])
            d.periodicity_type[i] = int(self.periodicity_type[i])
            d.periodic_length[i] = float(self.periodic_length[i])
        return d

    def iblank_array(self) -> np.ndarray:
        if self.iblank is None:
            return np.ones(self.n_points, dtype=np.int32)
        return np.ascontiguousarray(self.iblank, dtype=np.int32)


@dataclass
class Problem:
    options: Options
    blocks: List[Block] = field(default_factory=list)
    patches: List[Patch] = field(default_factory=list)
    sources: List[AcousticSource] = field(default_factory=list)
    n_steps: int = 0
    save_interval: int = 10

    @property
    def n_unknowns(self) -> int:
        return self.options.n_dimensions + 2

    def actuator_points(self) -> int:
        n = 0
        for p in self.patches:
            if p.type == "ACTUATOR":
                e = p.resolved_extent(self.blocks[p.grid_index - 1].grid_size)
                n += (e[1] - e[0] + 1) * (e[3] - e[2] + 1) * (e[5] - e[4] + 1)
        return n


def quiescent_state(n_points: int, n_dimensions: int, gamma: float) -> np.ndarray:
    """State%makeQuiescent (src/StateImpl.f90:434-459): rho = 1, u = 0, p = 1/gamma."""
    q = np.zeros((n_dimensions + 2, n_points))
    q[0] = 1.0
    q[n_dimensions + 1] = 1.0 / gamma / (gamma - 1.0)
    return q


def solenoidal_modes(n_modes: int, frequency: float, seed: int, randomize_frequency: bool = True):
    """Modes of a solenoidal excitation patch, drawn as the reference's setup
    draws them (src/SolenoidalExcitationPatchImpl.f90:64-90): three columns of
    uniform phases r in [0, 1) (phases(:, 1..3)), then one uniform r_l per mode
    for the frequency jitter (0.5 when not randomized); phases = 2 pi r and
    angular frequency l = 2 pi frequency (l + r_l - 1/2) / (n_modes / 2).
    The reference draws from gfortran's random_number after random_seed(put =
    seed); that stream is compiler-specific, so this front end draws from
    numpy's PCG64 generator seeded with `seed` (numpy.random.default_rng).
    A Fortran caller passes its own arrays through the C ABI instead.
    Returns (angular_frequencies (n_modes), phases (n_modes, 3))."""
    if n_modes <= 0:
        return np.zeros(0), np.zeros((0, 3))
    rng = np.random.default_rng(seed)
    r = rng.random((3, n_modes))
    jitter = rng.random(n_modes) if randomize_frequency else np.full(n_modes, 0.5)
    l = np.arange(1, n_modes + 1, dtype=np.float64)
    w = 2.0 * np.pi * frequency * (l + (jitter - 0.5)) / (0.5 * n_modes)
    return w, np.ascontiguousarray((2.0 * np.pi * r).T)
