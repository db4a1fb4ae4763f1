"""magudi.inp and bc.dat front end.

parse_input_file   the `key = value` dictionary of magudi.inp
                   (InputHelper%parseInputFile, src/InputHelperImpl.f90:142-269):
                   '#' starts a comment, the first '=' splits key and value,
                   a second '=' on a line is an error, keys are case-sensitive.
read_bc_dat        the patch table of bc.dat (Region%readBoundaryConditions,
                   src/RegionImpl.f90:175-337): name, type, grid, normDir,
                   iMin iMax jMin jMax kMin kMax; duplicate names are an error.
options_from_inputs, patches_from_bc, sources_from_inputs, block_periodicity
                   map those to the library's Options / Patch / AcousticSource
                   with the reference's option names and defaults
                   (src/SimulationFlagsImpl.f90:24-45, src/SolverOptionsImpl.f90:46-135,
                   src/FarFieldPatchImpl.f90:42-63, src/SpongePatchImpl.f90:30-45,
                   src/StateImpl.f90:135-150, src/GridImpl.f90:195-214).
"""
from .capi import PATCH_TYPES, PERIODIC_NONE, PERIODIC_OVERLAP, PERIODIC_PLANE, SBP_SCHEMES
from .problem import AcousticSource, Options, Patch


class InputError(ValueError):
    pass


def _strip_comment(line, marker="#"):
    i = line.find(marker)
    return line if i < 0 else line[:i]


def parse_input_file(path, comment="#", separator="="):
    entries = {}
    with open(path) as f:
        for lineno, raw in enumerate(f, start=1):
            line = _strip_comment(raw, comment).strip()
            if not line:
                continue
            if separator not in line:
                raise InputError(f"{path}: Failed to parse input on line {lineno}!")
            key, val = line.split(separator, 1)
            key, val = key.strip(), val.strip()
            if separator in val:
                raise InputError(f"{path}: Failed to parse input on line {lineno}!")
            if not key:
                raise InputError(f"{path}: Empty parameter key on line {lineno}!")
            entries[key] = val
    if not entries:
        raise InputError(f"{path}: File is empty or does not contain any input!")
    return InputDict(entries)


class InputDict(dict):
    """Typed getters with getOption's fallback-to-default on a bad value."""

    def get_str(self, key, default=""):
        v = self.get(key)
        if v is None:
            return default
        if len(v) >= 2 and v[0] == v[-1] and v[0] in "\"'":
            return v[1:-1]
        return v

    def get_float(self, key, default):
        v = self.get(key)
        if v is None:
            return default
        try:
            return float(v.replace("d", "e").replace("D", "e"))
        except ValueError:
            return default

    def get_int(self, key, default):
        v = self.get(key)
        if v is None:
            return default
        try:
            return int(v)
        except ValueError:
            return default

    def get_bool(self, key, default):
        v = self.get(key)
        if v is None:
            return default
        t = v.strip().strip(".").lower()
        if t in ("true", "t"):
            return True
        if t in ("false", "f"):
            return False
        return default


def read_bc_dat(path):
    rows = []
    names = set()
    with open(path) as f:
        for lineno, raw in enumerate(f, start=1):
            line = _strip_comment(raw).strip()
            if not line:
                continue
            parts = line.split()
            if len(parts) < 10:
                raise InputError(f"{path}:{lineno}: Failed to parse input on this line!")
            name, ptype = parts[0], parts[1]
            try:
                grid, ndir = int(parts[2]), int(parts[3])
                ext = tuple(int(x) for x in parts[4:10])
            except ValueError:
                raise InputError(f"{path}:{lineno}: Failed to parse input on this line!")
            if name in names:
                raise InputError(f"{path}:{lineno}: A patch with name '{name}' already exists!")
            names.add(name)
            rows.append((name, ptype, grid, ndir, ext))
    return rows


def options_from_inputs(d, n_dimensions):
    o = Options(n_dimensions=n_dimensions)
    o.viscous = d.get_bool("include_viscous_terms", False)
    o.enable_controller = d.get_bool("enable_controller", False)
    o.enable_functional = d.get_bool("enable_functional", False)
    o.adjoint_forcing_switch = d.get_bool("adjoint_forcing_switch", True)
    o.dissipation = d.get_bool("add_dissipation", False)
    o.curvilinear = d.get_bool("curvilinear_domain", True)
    o.use_constant_cfl = d.get_bool("use_constant_CFL_mode", True)
    o.composite_dissipation = d.get_bool("composite_dissipation", True)
    o.controller_switch = d.get_bool("controller_switch", False)
    o.ratio_of_specific_heats = d.get_float("ratio_of_specific_heats", 1.4)
    if o.viscous:
        o.reynolds_number = max(0.0, d.get_float("Reynolds_number", 0.0))
        o.prandtl_number = max(0.0, d.get_float("Prandtl_number", 0.72))
        o.viscosity_power_law_exponent = d.get_float("viscosity_power_law_exponent", 0.666)
        o.bulk_viscosity_ratio = d.get_float("bulk_viscosity_ratio", 0.6)
    if o.dissipation:
        if "dissipation_amount" not in d:
            raise InputError("Required parameter 'dissipation_amount' not specified!")
        o.dissipation_amount = d.get_float("dissipation_amount", 0.0)
    # src/SimulationFlagsImpl.f90:34 and src/SolverOptionsImpl.f90:73-78
    o.enable_solution_limits = d.get_bool("enable_solution_limits", False)
    if o.enable_solution_limits:
        for key in ("minimum_density", "maximum_density", "minimum_temperature", "maximum_temperature"):
            if key not in d:
                raise InputError(f"Required parameter '{key}' not specified!")
            setattr(o, key, d.get_float(key, 0.0))
    if o.use_constant_cfl:
        o.cfl = d.get_float("cfl", 0.5)
    else:
        if "time_step_size" not in d:
            raise InputError("Required parameter 'time_step_size' not specified!")
        o.time_step_size = d.get_float("time_step_size", 0.0)
    scheme = d.get_str("defaults/discretization_scheme", "SBP 4-8")
    if scheme not in SBP_SCHEMES:
        raise InputError(f"discretization scheme '{scheme}' is not supported "
                         f"(one of {', '.join(sorted(SBP_SCHEMES))})")
    o.discretization_scheme = SBP_SCHEMES[scheme]
    if scheme == "SBP 1-2" and o.dissipation and not o.composite_dissipation:
        raise InputError("SBP 1-2 has no non-composite dissipation operator")
    return o


def patches_from_bc(d, rows):
    patches = []
    for name, ptype, grid, ndir, ext in rows:
        if ptype not in PATCH_TYPES:
            raise InputError(f"Invalid type for patch '{name}'!")
        key = f"patches/{name}/"
        p = Patch(name, ptype, grid, ndir, ext)
        p.inviscid_penalty_amount = d.get_float(key + "inviscid_penalty_amount",
                                                d.get_float("defaults/inviscid_penalty_amount", 1.0))
        p.viscous_penalty_amount = d.get_float(key + "viscous_penalty_amount",
                                               d.get_float("defaults/viscous_penalty_amount", 1.0))
        p.sponge_amount = d.get_float(key + "sponge_amount", d.get_float("defaults/sponge_amount", 1.0))
        p.sponge_exponent = d.get_int(key + "sponge_exponent", d.get_int("defaults/sponge_exponent", 2))
        if ptype == "SAT_BLOCK_INTERFACE":
            # src/BlockInterfacePatchImpl.f90:72-86 (viscous default 0.5) and
            # src/InterfaceHelperImpl.f90:3-113 (conforms_with, interface_index1..3)
            p.viscous_penalty_amount = d.get_float(key + "viscous_penalty_amount",
                                                   d.get_float("defaults/viscous_penalty_amount", 0.5))
            p.conforms_with = d.get_str(key + "conforms_with", "")
            p.interface_index = tuple(d.get_int(key + f"interface_index{i}", i) for i in (1, 2, 3))
        if ptype == "SOLENOIDAL_EXCITATION":
            # src/SolenoidalExcitationPatchImpl.f90:40-62: number_of_modes, amplitude,
            # frequency and radius are required; the modes are drawn from random_seed
            for req in ("number_of_modes", "amplitude", "frequency", "radius"):
                if d.get(key + req) is None:
                    raise InputError(f"Required option '{key + req}' not found!")
            p.n_modes = max(0, d.get_int(key + "number_of_modes", 0))
            p.origin = (d.get_float(key + "origin_x", 0.0), d.get_float(key + "origin_y", 0.0))
            p.velocity = (d.get_float(key + "velocity_x", 0.0), d.get_float(key + "velocity_y", 0.0))
            p.amplitude = d.get_float(key + "amplitude", 0.0)
            p.frequency = d.get_float(key + "frequency", 0.0)
            p.radius = d.get_float(key + "radius", 1.0)
            p.random_seed = d.get_int(key + "random_seed", -1)
            p.randomize_frequency = d.get_bool(key + "randomize_frequency", True)
        if ptype == "SAT_ISOTHERMAL_WALL":
            # src/IsothermalWallImpl.f90:3-80: viscous_penalty_amount1, and the wall
            # temperature from the target state unless use_target_state is off
            p.viscous_penalty_amount = d.get_float(key + "viscous_penalty_amount1",
                                                   d.get_float("defaults/viscous_penalty_amount", 1.0))
            if not d.get_bool("use_target_state", True):
                gamma = d.get_float("ratio_of_specific_heats", 1.4)
                p.wall_temperature = d.get_float(key + "temperature", 1.0 / (gamma - 1.0))
        patches.append(p)
    return patches


def sources_from_inputs(d, n_dimensions):
    n = min(d.get_int("number_of_acoustic_sources", 0), 99)
    out = []
    for i in range(1, n + 1):
        key = f"acoustic_source{i:02d}/"
        loc = tuple(d.get_float(key + c, 0.0) for c in "xyz")[:3]
        out.append(AcousticSource(loc, d.get_float(key + "amplitude", 1.0), d.get_float(key + "frequency", 1.0),
                                  d.get_float(key + "radius", 1.0), d.get_float(key + "phase", 0.0)))
    return out


def block_periodicity(d, grid_index, n_dimensions):
    types, lengths = [PERIODIC_NONE] * 3, [0.0] * 3
    for i in range(n_dimensions):
        key = f"grid{grid_index:03d}/dir{i + 1}/"
        v = d.get_str(key + "periodicity_type", "")
        if v == "PLANE":
            types[i] = PERIODIC_PLANE
            if key + "periodic_length" not in d:
                raise InputError(f"Required parameter '{key}periodic_length' not specified!")
            lengths[i] = d.get_float(key + "periodic_length", 0.0)
        elif v == "OVERLAP":
            types[i] = PERIODIC_OVERLAP
    return tuple(types), tuple(lengths)


def write_input_file(path, entries):
    with open(path, "w") as f:
        for k, v in entries.items():
            f.write(f"{k} = {v}\n")


def write_bc_dat(path, patches):
    with open(path, "w") as f:
        f.write("# Name                 Type                  Grid normDir iMin iMax jMin jMax kMin kMax\n")
        for p in patches:
            e = p.extent
            f.write(f"  {p.name:<20} {p.type:<21} {p.grid_index:>4d} {p.normal_direction:>7d}"
                    + "".join(f" {x:>4d}" for x in e) + "\n")


def problem_from_inputs(inp_path, bc_path, blocks):
    """A Problem from a magudi.inp and a bc.dat, unchanged, and the blocks'
    arrays (what the reference reads from its grid, initial-condition,
    mollifier and mean-pressure files): `blocks` is a list of
    problem.Block with grid_size and coordinates set. Options, patches and
    acoustic sources come from the two files; each block's periodicity from
    grid00N/dirM/...; a block without a target state gets the quiescent one
    (Solver%setup, src/SolverImpl.f90:509-520); number_of_timesteps and
    save_interval become the run length and the checkpoint interval
    (src/SolverImpl.f90:483-496, src/UniformCheckpointerImpl.f90:3-40)."""
    from .problem import Problem, quiescent_state
    d = parse_input_file(inp_path)
    n_dimensions = 3 if any(int(b.grid_size[2]) > 1 for b in blocks) else 2
    options = options_from_inputs(d, n_dimensions)
    for i, b in enumerate(blocks, start=1):
        b.periodicity_type, b.periodic_length = block_periodicity(d, i, n_dimensions)
        if b.target_state is None:
            b.target_state = quiescent_state(b.n_points, n_dimensions, options.ratio_of_specific_heats)
    patches = patches_from_bc(d, read_bc_dat(bc_path))
    n_steps = max(0, d.get_int("number_of_timesteps", 1000))
    save_interval = d.get_int("save_interval", -1)
    if save_interval <= 0:
        save_interval = n_steps
    return Problem(options=options, blocks=list(blocks), patches=patches,
                   sources=sources_from_inputs(d, n_dimensions), n_steps=n_steps, save_interval=save_interval)
