"""Generators for the synthetic workloads (the role of magudi's
examples/*/config.py): grids, initial states, mollifiers, bc.dat patches.

monopole_2d      2D acoustic monopole on [-14,14]^2 with far-field SATs,
                 sponges, a Gaussian cost-target mollifier at (0,10) and a
                 Gaussian control mollifier at (0,0) (sigma = 1).
taylor_green_3d  3D periodic Taylor-Green vortex on [0, 2 pi)^3.
random_state     the randomized state of test/adjoint_relation/full_rhs.f90:289-301.
"""
import math

import numpy as np

from .problem import AcousticSource, Block, Options, Patch, Problem, quiescent_state


def _extents(x, lo, hi):
    """1-based first/last index of the points of a sorted 1D coordinate in [lo, hi]."""
    idx = np.nonzero((x >= lo) & (x <= hi))[0]
    return int(idx[0]) + 1, int(idx[-1]) + 1


def uniform_grid_2d(nx, ny, lo=-14.0, hi=14.0):
    x = np.linspace(lo, hi, nx)
    y = np.linspace(lo, hi, ny)
    X, Y = np.meshgrid(x, y, indexing="xy")  # (ny, nx): p = i + nx*j
    return np.stack([X.ravel(), Y.ravel()]), x, y


def monopole_2d(n=201, ny=None, dt=0.05, n_steps=960, sponge_points=20, sponge_amount=0.2,
                dissipation_amount=0.01, reynolds=200.0, prandtl=0.72,
                power_law=0.666, bulk_viscosity_ratio=0.6, save_interval=10,
                controller_switch=False, half_width=14.0, target_center=(0.0, 10.0),
                control_center=(0.0, 0.0), mollifier_sigma=1.0, composite_dissipation=True, cfl=None):
    """Acoustic monopole: quiescent ambient rho = 1, u = 0, p = 1/gamma; pressure
    source 0.01 sin(2 pi 0.2 t) with a Gaussian of sigma 0.5 at the origin.
    magudi's source is A cos(w t + phase) exp(-9/(2 R^2) r^2)
    (src/AcousticSourceImpl.f90:27,55-62), so sin -> phase = -pi/2 and
    sigma = 0.5 -> R = 3 sigma = 1.5. The dissipation is magudi's default
    composite operator: the non-composite one at amount 0.01 is unstable at
    dt = 0.05 on this grid. With cfl set, the step size follows the
    constant-CFL rule instead of dt."""
    ny = ny or n
    gamma = 1.4
    opts = Options(
        n_dimensions=2, viscous=True, dissipation=True, composite_dissipation=composite_dissipation,
        curvilinear=False, use_constant_cfl=False, enable_controller=True,
        enable_functional=True, controller_switch=controller_switch,
        ratio_of_specific_heats=gamma, reynolds_number=reynolds, prandtl_number=prandtl,
        viscosity_power_law_exponent=power_law, bulk_viscosity_ratio=bulk_viscosity_ratio,
        dissipation_amount=dissipation_amount, time_step_size=dt)
    if cfl is not None:
        opts.use_constant_cfl = True
        opts.cfl = cfl
    coords, x, y = uniform_grid_2d(n, ny, -half_width, half_width)
    N = n * ny
    X, Y = coords
    target = quiescent_state(N, 2, gamma)
    sigma = mollifier_sigma
    tx, ty = target_center
    cx, cy = control_center
    tm = np.exp(-((X - tx) ** 2 + (Y - ty) ** 2) / (2 * sigma ** 2))
    cm = np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * sigma ** 2))
    block = Block(grid_size=(n, ny, 1), coordinates=np.ascontiguousarray(coords),
                  initial_state=target.copy(), target_state=target.copy(),
                  control_mollifier=cm, target_mollifier=tm,
                  mean_pressure=np.full(N, 1.0 / gamma))
    s = sponge_points
    patches = [
        Patch("farField.E", "SAT_FAR_FIELD", 1, 1, (1, 1, 1, -1, 1, -1)),
        Patch("farField.W", "SAT_FAR_FIELD", 1, -1, (-1, -1, 1, -1, 1, -1)),
        Patch("farField.S", "SAT_FAR_FIELD", 1, 2, (1, -1, 1, 1, 1, -1)),
        Patch("farField.N", "SAT_FAR_FIELD", 1, -2, (1, -1, -1, -1, 1, -1)),
        Patch("sponge.E", "SPONGE", 1, 1, (1, s, 1, -1, 1, -1), sponge_amount=sponge_amount),
        Patch("sponge.W", "SPONGE", 1, -1, (-s, -1, 1, -1, 1, -1), sponge_amount=sponge_amount),
        Patch("sponge.S", "SPONGE", 1, 2, (1, -1, 1, s, 1, -1), sponge_amount=sponge_amount),
        Patch("sponge.N", "SPONGE", 1, -2, (1, -1, -s, -1, 1, -1), sponge_amount=sponge_amount),
    ]
    w = 4.0 * sigma  # supports truncated at 4 sigma
    ti = _extents(x, tx - w, tx + w)
    tj = _extents(y, ty - w, ty + w)
    patches.append(Patch("targetRegion", "COST_TARGET", 1, 0, (ti[0], ti[1], tj[0], tj[1], 1, -1)))
    ci = _extents(x, cx - w, cx + w)
    cj = _extents(y, cy - w, cy + w)
    patches.append(Patch("controlRegion", "ACTUATOR", 1, 0, (ci[0], ci[1], cj[0], cj[1], 1, -1)))
    sources = [AcousticSource((0.0, 0.0), 0.01, 0.2, 1.5, -math.pi / 2)]
    return Problem(options=opts, blocks=[block], patches=patches, sources=sources,
                   n_steps=n_steps, save_interval=save_interval)


def wall_channel_2d(n=41, ny=33, wall="SAT_ISOTHERMAL_WALL", wall_temperature=0.0, dt=0.02, n_steps=20,
                    viscous=True, reynolds=200.0, mach=0.3, sponge_points=6, half_width=6.0):
    """Channel between two walls: walls of the given bc.dat type on the south
    (normal +2) and north (normal -2) faces, far-field SATs and sponges on the
    west and east faces, a uniform stream of Mach `mach` along x as target and
    initial state. wall_temperature <= 0 takes the target state's temperature
    (use_target_state)."""
    gamma = 1.4
    opts = Options(
        n_dimensions=2, viscous=viscous, dissipation=True, composite_dissipation=True,
        curvilinear=False, use_constant_cfl=False, enable_controller=False, enable_functional=False,
        ratio_of_specific_heats=gamma, reynolds_number=reynolds, prandtl_number=0.72,
        viscosity_power_law_exponent=0.666, bulk_viscosity_ratio=0.6, dissipation_amount=0.01,
        time_step_size=dt)
    coords, x, y = uniform_grid_2d(n, ny, -half_width, half_width)
    N = n * ny
    target = quiescent_state(N, 2, gamma)
    target[1] = mach * target[0]
    target[3] = target[3] + 0.5 * mach ** 2
    block = Block(grid_size=(n, ny, 1), coordinates=np.ascontiguousarray(coords),
                  initial_state=target.copy(), target_state=target.copy(),
                  control_mollifier=np.ones(N), target_mollifier=np.ones(N),
                  mean_pressure=np.full(N, 1.0 / gamma))
    s = sponge_points
    patches = [
        Patch("farField.W", "SAT_FAR_FIELD", 1, 1, (1, 1, 1, -1, 1, -1)),
        Patch("farField.E", "SAT_FAR_FIELD", 1, -1, (-1, -1, 1, -1, 1, -1)),
        Patch("wall.S", wall, 1, 2, (1, -1, 1, 1, 1, -1), wall_temperature=wall_temperature),
        Patch("wall.N", wall, 1, -2, (1, -1, -1, -1, 1, -1), wall_temperature=wall_temperature),
        Patch("sponge.W", "SPONGE", 1, 1, (1, s, 1, -1, 1, -1), sponge_amount=0.2),
        Patch("sponge.E", "SPONGE", 1, -1, (-s, -1, 1, -1, 1, -1), sponge_amount=0.2),
    ]
    return Problem(options=opts, blocks=[block], patches=patches, sources=[], n_steps=n_steps, save_interval=5)


def two_block_2d(nx1=25, nx2=29, ny=31, half_width=6.0, viscous=True, rotate_second=False, curvilinear=None,
                 interfaces=True, dt=0.02, n_steps=10, sponge_points=5, functional=False, controller_switch=False):
    """Two blocks meeting at x = 0 through SAT_BLOCK_INTERFACE patches: block 1
    covers [-w, 0] x [-w, w], block 2 covers [0, w] x [-w, w]; far-field SATs
    and sponges on the outer faces; quiescent target and initial state.
    rotate_second stores block 2 with its first index along +y and its second
    along -x (a rotation, so the Jacobian stays positive), which makes the
    interface a transposing one (interface_index 2, 1, 3). Without
    `interfaces`, the x = 0 faces carry no patch. With `functional`, an
    acoustic source and an actuator sit in block 1 at (-1.5, 0) and the cost
    target in block 2 at (1.5, 0), so that sound crosses the interface."""
    gamma = 1.4
    curv = rotate_second if curvilinear is None else curvilinear
    opts = Options(
        n_dimensions=2, viscous=viscous, dissipation=True, composite_dissipation=True,
        curvilinear=curv, use_constant_cfl=False, enable_controller=functional, enable_functional=functional,
        controller_switch=controller_switch,
        ratio_of_specific_heats=gamma, reynolds_number=200.0, prandtl_number=0.72,
        viscosity_power_law_exponent=0.666, bulk_viscosity_ratio=0.6, dissipation_amount=0.01,
        time_step_size=dt)
    w = half_width
    x1 = np.linspace(-w, 0.0, nx1)
    x2 = np.linspace(0.0, w, nx2)
    y = np.linspace(-w, w, ny)
    X1, Y1 = np.meshgrid(x1, y, indexing="xy")
    c1 = np.stack([X1.ravel(), Y1.ravel()])
    if rotate_second:
        # point (i, j): x = x2[nx2 - j], y = y[i - 1]; i fastest
        Yr, Xr = np.meshgrid(y, x2[::-1], indexing="xy")
        c2 = np.stack([Xr.ravel(), Yr.ravel()])
        gs2 = (ny, nx2, 1)
    else:
        X2, Y2 = np.meshgrid(x2, y, indexing="xy")
        c2 = np.stack([X2.ravel(), Y2.ravel()])
        gs2 = (nx2, ny, 1)
    blocks = []
    for c, gs in ((c1, (nx1, ny, 1)), (c2, gs2)):
        N = c.shape[1]
        t = quiescent_state(N, 2, gamma)
        cm = np.exp(-((c[0] + 1.5) ** 2 + c[1] ** 2) / 2.0)
        tm = np.exp(-((c[0] - 1.5) ** 2 + c[1] ** 2) / 2.0)
        blocks.append(Block(grid_size=gs, coordinates=np.ascontiguousarray(c), initial_state=t.copy(),
                            target_state=t.copy(), control_mollifier=cm, target_mollifier=tm,
                            mean_pressure=np.full(N, 1.0 / gamma)))
    s = sponge_points
    patches = [
        Patch("farField.W", "SAT_FAR_FIELD", 1, 1, (1, 1, 1, -1, 1, -1)),
        Patch("farField.S1", "SAT_FAR_FIELD", 1, 2, (1, -1, 1, 1, 1, -1)),
        Patch("farField.N1", "SAT_FAR_FIELD", 1, -2, (1, -1, -1, -1, 1, -1)),
        Patch("sponge.W", "SPONGE", 1, 1, (1, s, 1, -1, 1, -1), sponge_amount=0.2),
    ]
    if rotate_second:
        patches += [
            Patch("farField.E", "SAT_FAR_FIELD", 2, 2, (1, -1, 1, 1, 1, -1)),
            Patch("farField.S2", "SAT_FAR_FIELD", 2, 1, (1, 1, 1, -1, 1, -1)),
            Patch("farField.N2", "SAT_FAR_FIELD", 2, -1, (-1, -1, 1, -1, 1, -1)),
            Patch("sponge.E", "SPONGE", 2, 2, (1, -1, 1, s, 1, -1), sponge_amount=0.2),
        ]
        iface2 = Patch("interface.2W", "SAT_BLOCK_INTERFACE", 2, -2, (1, -1, -1, -1, 1, -1),
                       viscous_penalty_amount=0.5)
        iface1 = Patch("interface.1E", "SAT_BLOCK_INTERFACE", 1, -1, (-1, -1, 1, -1, 1, -1),
                       viscous_penalty_amount=0.5, conforms_with="interface.2W", interface_index=(2, 1, 3))
    else:
        patches += [
            Patch("farField.E", "SAT_FAR_FIELD", 2, -1, (-1, -1, 1, -1, 1, -1)),
            Patch("farField.S2", "SAT_FAR_FIELD", 2, 2, (1, -1, 1, 1, 1, -1)),
            Patch("farField.N2", "SAT_FAR_FIELD", 2, -2, (1, -1, -1, -1, 1, -1)),
            Patch("sponge.E", "SPONGE", 2, -1, (-s, -1, 1, -1, 1, -1), sponge_amount=0.2),
        ]
        iface2 = Patch("interface.2W", "SAT_BLOCK_INTERFACE", 2, 1, (1, 1, 1, -1, 1, -1),
                       viscous_penalty_amount=0.5)
        iface1 = Patch("interface.1E", "SAT_BLOCK_INTERFACE", 1, -1, (-1, -1, 1, -1, 1, -1),
                       viscous_penalty_amount=0.5, conforms_with="interface.2W")
    if interfaces:
        patches += [iface1, iface2]
    sources = []
    if functional:
        ci = _extents(x1, -3.5, -0.5)
        cj = _extents(y, -2.0, 2.0)
        patches.append(Patch("controlRegion", "ACTUATOR", 1, 0, (ci[0], ci[1], cj[0], cj[1], 1, -1)))
        ti = _extents(x2, 0.5, 3.5)
        if rotate_second:  # block 2 index 1 runs along y, index 2 along -x
            lo, hi = nx2 + 1 - ti[1], nx2 + 1 - ti[0]
            patches.append(Patch("targetRegion", "COST_TARGET", 2, 0, (cj[0], cj[1], lo, hi, 1, -1)))
        else:
            patches.append(Patch("targetRegion", "COST_TARGET", 2, 0, (ti[0], ti[1], cj[0], cj[1], 1, -1)))
        sources = [AcousticSource((-1.5, 0.0), 0.01, 0.2, 1.5, -math.pi / 2)]
    return Problem(options=opts, blocks=blocks, patches=patches, sources=sources, n_steps=n_steps, save_interval=5)


def _tanh_cluster(n, beta, left=True):
    """n points on [0, 1] clustered toward 0 (left) or 1 by a tanh mapping."""
    s = np.linspace(0.0, 1.0, n)
    if left:
        return 1.0 - np.tanh(beta * (1.0 - s)) / np.tanh(beta)
    return np.tanh(beta * s) / np.tanh(beta)


def jet_3block_3d(nx=384, ny_core=192, ny_side=171, nz=192, mach=1.3, reynolds=2500.0, theta=0.04, cfl=0.5,
                  dt=None, n_steps=1000, save_interval=None, length=20.0, core_half_width=2.0, side_extent=8.0,
                  flare=0.5, sponge_points=None, excitation_modes=8, excitation_amplitude=1e-3, seed=2022,
                  dissipation_amount=0.01, target=(2.5, 1.6, 0.3, 1.0), side_beta=1.0):
    """Three-block curvilinear jet (the 3D multi-block jet workload).

    Axial direction x (index i, `nx` points, tanh-clustered toward the inflow
    over [0, length]); cross-stream y (index j) and z (index k). Block 1 is
    the core, |y|, |z| <= core_half_width (ny_core x nz, uniform); blocks 2
    and 3 are shear-layer blocks below and above it in y out to side_extent
    (ny_side points, tanh-clustered toward the core), sharing the core's z
    points. All three blocks carry the flare mapping y, z -> (y, z)(1 + flare
    x / length), so every grid is curvilinear (non-orthogonal), and the
    blocks meet at two SAT_BLOCK_INTERFACE pairs. With the defaults the point
    count is 384 x 192 x 192 + 2 x 384 x 171 x 192 = 39.4 M, the point count
    of a 192^2 x 384 core with two 128 x 256 x 384 shear-layer blocks.

    Flow: a Mach `mach` round jet of diameter 1 along x (top hat with a tanh
    shear layer of momentum thickness theta), rho = 1 and p = 1/gamma
    everywhere, Re = `reynolds`. A SOLENOIDAL_EXCITATION patch (8 modes,
    amplitude 1e-3, seeded) forces the core near the inflow, convected at
    0.65 of the jet speed. The cost functional is the squared pressure on a
    cylindrical shell target in all blocks, target = (axial centre, radius,
    radial width, axial width) of its Gaussian mollifier; the
    control is a thermal actuator on an annulus at the nozzle lip in the
    core. Far-field SATs on every outer face, sponges on the outflow and
    lateral faces. dt defaults to `cfl` over the largest inviscid spectral
    radius sum_d (|u_d| + c) / h_d of the initial state, h_d the grid-line
    spacing.

    The composite dissipation enters the RHS as amount * D_diss q * (1/det)
    (addDissipation before the 1/det scaling, src/RhsHelperImpl.f90:10-87,
    src/RegionImpl.f90:1968-1976), so its explicit stability limit tightens
    with the cell volume. The 1D SBP 4-8 composite operator has spectral
    radius 2.42 with its boundary closures (1 in the interior), so at a corner
    where three closures meet RK4 needs about 7.3 dt amount / det < 2.8. The
    amount is capped at 0.2 det_min / dt (det estimated from the grid-line
    spacings); on the full 39.4 M-point grid that cap, not 0.01, applies.
    A cap of 0.5 det_min / dt let the closure corners at the inflow, the
    interface and a z face grow without bound.
    """
    gamma = 1.4
    U = mach  # ambient sound speed 1
    L, Yc, Ys = length, core_half_width, side_extent
    x = L * _tanh_cluster(nx, 1.2)
    yc = np.linspace(-Yc, Yc, ny_core)
    z = np.linspace(-Yc, Yc, nz)
    y_up = Yc + (Ys - Yc) * _tanh_cluster(ny_side, side_beta)
    ys = (yc, -y_up[::-1], y_up)
    opts = Options(
        n_dimensions=3, viscous=True, dissipation=True, composite_dissipation=True, curvilinear=True,
        use_constant_cfl=False, time_step_size=0.0, enable_controller=True, enable_functional=True,
        ratio_of_specific_heats=gamma, reynolds_number=reynolds, prandtl_number=0.72,
        viscosity_power_law_exponent=0.666, bulk_viscosity_ratio=0.6, dissipation_amount=dissipation_amount)
    blocks = []
    smax, vmin = 0.0, np.inf
    for yy in ys:
        Z, Y, X = np.meshgrid(z, yy, x, indexing="ij")  # (nz, ny, nx): point = i + nx (j + ny k)
        f = 1.0 + flare * X / L
        coords = np.stack([X.ravel(), (Y * f).ravel(), (Z * f).ravel()])
        N = coords.shape[1]
        r = np.sqrt(coords[1] ** 2 + coords[2] ** 2)
        u = 0.5 * U * (1.0 - np.tanh((r - 0.5) / (2.0 * theta)))
        q = quiescent_state(N, 3, gamma)
        q[1] = u
        q[4] = q[4] + 0.5 * u * u
        shape = (len(z), len(yy), len(x))
        # inviscid spectral radius sum_d (|u_d| + c) / h_d with h_d the grid-line spacing
        rad = np.zeros(shape)
        vol = np.ones(shape)
        for axis in (2, 1, 0):
            d = np.sqrt(sum(np.diff(c.reshape(shape), axis=axis) ** 2 for c in coords))
            h = np.concatenate([d, np.take(d, [-1], axis=axis)], axis=axis)
            speed = (np.abs(u.reshape(shape)) if axis == 2 else 0.0) + 1.0
            rad += speed / h
            vol *= h
        smax = max(smax, float(rad.max()))
        vmin = min(vmin, float(vol.min()))
        tm = np.exp(-((r - target[1]) / target[2]) ** 2 - ((coords[0] - target[0]) / target[3]) ** 2)
        mc = np.exp(-((r - 0.5) / 0.15) ** 2 - ((coords[0] - 0.4) / 0.25) ** 2)
        blocks.append(Block(grid_size=(nx, len(yy), nz), coordinates=np.ascontiguousarray(coords),
                            initial_state=q.copy(), target_state=q.copy(), control_mollifier=mc,
                            target_mollifier=tm, mean_pressure=np.full(N, 1.0 / gamma)))
    if dt is None:
        dt = cfl / smax
    opts.time_step_size = float(dt)
    opts.dissipation_amount = float(min(dissipation_amount, 0.2 * vmin / dt))
    s = sponge_points or max(4, nx // 24)
    sl = max(4, min(ny_side, nz) // 12)
    patches = []
    for b in (1, 2, 3):
        patches += [
            Patch(f"inflow{b}", "SAT_FAR_FIELD", b, 1, (1, 1, 1, -1, 1, -1)),
            Patch(f"outflow{b}", "SAT_FAR_FIELD", b, -1, (-1, -1, 1, -1, 1, -1)),
            Patch(f"farField.B{b}", "SAT_FAR_FIELD", b, 3, (1, -1, 1, -1, 1, 1)),
            Patch(f"farField.F{b}", "SAT_FAR_FIELD", b, -3, (1, -1, 1, -1, -1, -1)),
            Patch(f"sponge.out{b}", "SPONGE", b, -1, (-s, -1, 1, -1, 1, -1), sponge_amount=0.2),
            Patch(f"sponge.B{b}", "SPONGE", b, 3, (1, -1, 1, -1, 1, sl), sponge_amount=0.2),
            Patch(f"sponge.F{b}", "SPONGE", b, -3, (1, -1, 1, -1, -sl, -1), sponge_amount=0.2),
            Patch(f"target{b}", "COST_TARGET", b, 0, (1, -1, 1, -1, 1, -1)),
        ]
    # cross-stream (j) indices of the actuator box |y|, |z| <= 0.85 in the core
    jlo = int(np.searchsorted(yc, -0.85)) + 1
    jhi = int(np.searchsorted(yc, 0.85))
    klo = int(np.searchsorted(z, -0.85)) + 1
    khi = int(np.searchsorted(z, 0.85))
    ihi = max(2, int(np.searchsorted(x, 1.2)))
    iexc = max(2, int(np.searchsorted(x, 2.0)))
    patches += [
        Patch("farField.S", "SAT_FAR_FIELD", 2, 2, (1, -1, 1, 1, 1, -1)),
        Patch("farField.N", "SAT_FAR_FIELD", 3, -2, (1, -1, -1, -1, 1, -1)),
        Patch("sponge.S", "SPONGE", 2, 2, (1, -1, 1, sl, 1, -1), sponge_amount=0.2),
        Patch("sponge.N", "SPONGE", 3, -2, (1, -1, -sl, -1, 1, -1), sponge_amount=0.2),
        Patch("interface.1S", "SAT_BLOCK_INTERFACE", 1, 2, (1, -1, 1, 1, 1, -1), viscous_penalty_amount=0.5,
              conforms_with="interface.2N"),
        Patch("interface.2N", "SAT_BLOCK_INTERFACE", 2, -2, (1, -1, -1, -1, 1, -1), viscous_penalty_amount=0.5,
              conforms_with="interface.1S"),
        Patch("interface.1N", "SAT_BLOCK_INTERFACE", 1, -2, (1, -1, -1, -1, 1, -1), viscous_penalty_amount=0.5,
              conforms_with="interface.3S"),
        Patch("interface.3S", "SAT_BLOCK_INTERFACE", 3, 2, (1, -1, 1, 1, 1, -1), viscous_penalty_amount=0.5,
              conforms_with="interface.1N"),
        Patch("controlRegion", "ACTUATOR", 1, 0, (1, ihi, jlo, jhi, klo, khi)),
        Patch("excitationSupport", "SOLENOIDAL_EXCITATION", 1, 0, (1, iexc, 1, -1, 1, -1),
              n_modes=excitation_modes, origin=(0.75, 0.0), velocity=(0.65 * U, 0.0),
              amplitude=excitation_amplitude, frequency=0.4 * U, radius=1.0, random_seed=seed),
    ]
    S = save_interval or max(1, int(round((n_steps / 4.0) ** 0.5)))
    return Problem(options=opts, blocks=blocks, patches=patches, sources=[], n_steps=n_steps, save_interval=S)


def random_state(n_points, n_dimensions, gamma, rng):
    """full_rhs.f90:289-301: rho in U[0.01,10], u in U[-10,10], p in U[0.01,10]/gamma."""
    nU = n_dimensions + 2
    q = np.zeros((nU, n_points))
    q[0] = rng.uniform(0.01, 10.0, n_points)
    for d in range(n_dimensions):
        q[1 + d] = q[0] * rng.uniform(-10.0, 10.0, n_points)
    q[nU - 1] = (q[0] * rng.uniform(0.01, 10.0, n_points) / gamma
                 + 0.5 / q[0] * np.sum(q[1:1 + n_dimensions] ** 2, axis=0))
    return q


def smooth_perturbed_state(block, n_dimensions, gamma, rng, amplitude=1e-2):
    """A smooth non-trivial state: quiescent plus Gaussian-modulated waves."""
    N = block.n_points
    xs = block.coordinates
    q = quiescent_state(N, n_dimensions, gamma)
    phase = rng.uniform(0, 2 * np.pi, 4)
    r2 = np.sum(xs ** 2, axis=0)
    env = np.exp(-r2 / (2 * 6.0 ** 2))
    rho = 1.0 + amplitude * env * np.sin(0.7 * xs[0] + phase[0])
    u = [amplitude * env * np.cos(0.5 * xs[d % n_dimensions] + phase[1 + d % 3]) for d in range(n_dimensions)]
    p = 1.0 / gamma + amplitude * env * np.cos(0.6 * xs[n_dimensions - 1] + phase[3])
    q[0] = rho
    for d in range(n_dimensions):
        q[1 + d] = rho * u[d]
    q[n_dimensions + 1] = p / (gamma - 1.0) + 0.5 * rho * sum(ud ** 2 for ud in u)
    return q


def taylor_green_3d(n=256, mach=0.1, reynolds=1600.0, cfl=0.5, n_steps=2000,
                    dissipation_amount=0.01, power_law=0.666, bulk_viscosity_ratio=0.6, dt=None,
                    save_interval=None):
    """Taylor-Green vortex, PLANE periodicity on [0, 2 pi)^3:
    rho = 1, u = sin x cos y cos z, v = -cos x sin y cos z, w = 0,
    p = 1/(gamma M^2) + (cos 2x + cos 2y)(cos 2z + 2)/16.
    The cost functional is the kinetic energy at the final step. Constant CFL
    unless dt is given; the checkpoint interval defaults to about sqrt(n_steps)."""
    gamma = 1.4
    L = 2.0 * np.pi
    x = np.arange(n) * (L / n)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")  # (nz, ny, nx)
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()])
    N = n ** 3
    Xr, Yr, Zr = coords
    u = np.sin(Xr) * np.cos(Yr) * np.cos(Zr)
    v = -np.cos(Xr) * np.sin(Yr) * np.cos(Zr)
    w = np.zeros(N)
    p = 1.0 / (gamma * mach ** 2) + (np.cos(2 * Xr) + np.cos(2 * Yr)) * (np.cos(2 * Zr) + 2.0) / 16.0
    q = np.zeros((5, N))
    q[0] = 1.0
    q[1], q[2], q[3] = u, v, w
    q[4] = p / (gamma - 1.0) + 0.5 * (u ** 2 + v ** 2 + w ** 2)
    opts = Options(
        n_dimensions=3, viscous=True, dissipation=True, composite_dissipation=True,
        curvilinear=False, use_constant_cfl=dt is None, cfl=cfl, enable_controller=False,
        enable_functional=True, ratio_of_specific_heats=gamma, reynolds_number=reynolds,
        prandtl_number=0.72, viscosity_power_law_exponent=power_law,
        bulk_viscosity_ratio=bulk_viscosity_ratio, dissipation_amount=dissipation_amount,
        time_step_size=dt or 0.0, functional_type=1)
    block = Block(grid_size=(n, n, n), coordinates=np.ascontiguousarray(coords),
                  periodicity_type=(1, 1, 1), periodic_length=(L, L, L),
                  initial_state=q, target_state=q.copy(), mean_pressure=np.full(N, 1.0 / gamma))
    S = save_interval or max(1, int(round(n_steps ** 0.5)))
    return Problem(options=opts, blocks=[block], patches=[], sources=[], n_steps=n_steps, save_interval=S)
