"""Seeded synthetic inputs for the RS pressure path.

The reference publishes no datasets for these cases; every input is generated
here from a seed with numpy's PCG64 so that the GPU library and the CPU
oracle consume identical bytes:

* ``grf``: stationary Gaussian random field with squared-exponential
  covariance, sampled by FFT circulant embedding on a 2x padded torus;
* ``potential_case``: 2D single-phase incompressible potential problem
  (MPFA-O, full anisotropic tensor, Dirichlet columns, injector/producer);
* ``two_phase_case``: 3D oil/water black-oil problem on a perturbed hexahedral
  grid with a lognormal permeability field and a five-spot well pattern;
* ``three_phase_case``: the same grid with water, oil and gas (a gas cap over
  undersaturated oil, gas injected at the corners);
* ``compositional_case`` / ``compositional_cells``: Peng-Robinson fluids with
  water and three hydrocarbon pseudo-components, on a grid or per cell.

Units are SI as in RS (Pa, m^2, Pa*s, K, mol).
"""
import math

import numpy as np

from . import abi

MILLIDARCY = 9.869233e-16  # m^2
BAR = 1.0e5  # Pa
CENTIPOISE = 1.0e-3  # Pa*s


def rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def grf(shape, corr_len, mean, std, seed):
    """Gaussian random field on a grid of `shape` cells (1 to 3 axes)."""
    g = rng(seed)
    pad = [2 * s for s in shape]
    axes = [np.minimum(np.arange(p), p - np.arange(p)).astype(np.float64) for p in pad]
    mesh = np.meshgrid(*axes, indexing="ij")
    h2 = sum(m * m for m in mesh)
    cov = (std * std) * np.exp(-h2 / (corr_len * corr_len))
    lam = np.fft.fftn(cov).real
    lam = np.maximum(lam, 0.0)
    eps = g.standard_normal(pad) + 1j * g.standard_normal(pad)
    y = np.fft.fftn(np.sqrt(lam / lam.size) * eps)
    field = y.real[tuple(slice(0, s) for s in shape)]
    return mean + field


def _cells_ijk_to_linear(field_ijk):
    """RS numbers cells i fastest (NaturalIJKOrdering.getLinear)."""
    return np.ascontiguousarray(field_ijk.transpose(*reversed(range(field_ijk.ndim))).reshape(-1))


# --------------------------------------------------------------- 2D case ---
def potential_case(ni=64, nj=64, seed=0, corr_len=8.0, angle_deg=30.0, anisotropy=10.0, rate=1.0e-13):
    """Single-phase incompressible potential problem (numerics/PotentialCalculator).

    Returns a dict with the grid, the permeability tensors (6 per cell), the
    Dirichlet cells/values and the right-hand-side rate terms.
    """
    logk = grf((ni, nj), corr_len, 2.0, 1.0, seed)  # log10 kmax [mD]
    kmax = _cells_ijk_to_linear(10.0 ** logk) * MILLIDARCY
    kmin = kmax / anisotropy
    a = math.radians(angle_deg)
    c, s = math.cos(a), math.sin(a)
    # K = R diag(kmax, kmin) R^T
    kxx = c * c * kmax + s * s * kmin
    kyy = s * s * kmax + c * c * kmin
    kxy = c * s * (kmax - kmin)
    n = ni * nj
    perm = np.zeros((n, 6))
    perm[:, 0] = kxx
    perm[:, 1] = kyy
    perm[:, 2] = kmin  # permz must be present for RockDataParser to build a tensor
    perm[:, 3] = kxy
    dirichlet_cells = []
    dirichlet_values = []
    for j in range(nj):
        dirichlet_cells.append(0 + j * ni)
        dirichlet_values.append(1.0)
    for j in range(nj):
        dirichlet_cells.append((ni - 1) + j * ni)
        dirichlet_values.append(0.0)
    # The corner cells (0,0) and (ni-1,nj-1) are Dirichlet cells, so the
    # injector/producer pair sits one column inside: (1,0) and (ni-2,nj-1).
    rates = {1 + 0 * ni: rate, (ni - 2) + (nj - 1) * ni: -rate}
    return dict(
        dim=2, ni=ni, nj=nj, nk=0, dx=1.0, dy=1.0, dz=-1.0, perm=np.ascontiguousarray(perm),
        porosity=np.full(n, 0.2), dirichlet_cells=np.array(dirichlet_cells, dtype=np.int32),
        dirichlet_values=np.array(dirichlet_values), rates=rates, seed=seed,
    )


def potential_rhs(case):
    n = case["ni"] * case["nj"]
    b = np.zeros(n)
    for cell, q in case["rates"].items():
        b[cell] += q
    for cell, v in zip(case["dirichlet_cells"], case["dirichlet_values"]):
        b[cell] = v
    return b


# --------------------------------------------------------------- 3D case ---
def perturbed_nodes(ni, nj, nk, dx, dy, dz, frac, seed):
    """Corner points of an ni x nj x nk grid (i fastest), each displaced by
    U(-frac, frac) of the cell size along every axis."""
    g = rng(seed)
    npi, npj, npk = ni + 1, nj + 1, nk + 1
    k, j, i = np.meshgrid(np.arange(npk), np.arange(npj), np.arange(npi), indexing="ij")
    x = i * dx + g.uniform(-frac, frac, i.shape) * dx
    y = j * dy + g.uniform(-frac, frac, i.shape) * dy
    z = k * dz + g.uniform(-frac, frac, i.shape) * abs(dz)
    pts = np.stack([x.reshape(-1), y.reshape(-1), z.reshape(-1)], axis=1)
    return np.ascontiguousarray(pts)


def two_phase_fluid(keep, p_range=(20 * BAR, 600 * BAR), n_p=64, even=False):
    """Oil/water black-oil fluid: exponential compressibility tables for the
    molar densities (4e-5 /bar water, 1e-4 /bar oil), constant viscosities
    (1 cP water, 5 cP oil), no gas component, no mass transfer.  even=True
    gives the density tables as EvenLookupTables over the same ranges."""
    p0 = 200 * BAR
    ps = np.linspace(p_range[0], p_range[1], n_p)
    Ts = np.array([250.0, 450.0])
    Cs = np.array([0.0, 1.0])
    xiw0, cw = 1000.0 / 0.01801528, 4.0e-5 / BAR
    xio0, co = 800.0 / 0.2, 1.0e-4 / BAR
    xiw = np.repeat((xiw0 * np.exp(cw * (ps - p0)))[:, None], 2, axis=1)
    xio = np.repeat(np.repeat((xio0 * np.exp(co * (ps - p0)))[:, None, None], 2, axis=1), 2, axis=2)
    f = abi.rsg_blackoil()
    f.nc = 2
    f.molecular_weight[0] = 0.01801528
    f.molecular_weight[1] = 0.2
    f.group[0] = 0
    f.group[1] = 1
    if even:
        f.water_density = abi.even_table(keep, [p_range, (Ts[0], Ts[-1])], xiw)
    else:
        f.water_density = abi.table(keep, [ps, Ts], xiw)
    f.water_viscosity = abi.constant(1.0 * CENTIPOISE, 2)
    f.water_enthalpy = abi.constant(0.0, 2)
    f.bubble_point = abi.constant(0.0, 2)
    f.dew_point = abi.constant(0.0, 2)
    if even:
        f.oil_density = abi.even_table(keep, [p_range, (Cs[0], Cs[-1]), (Ts[0], Ts[-1])], xio)
    else:
        f.oil_density = abi.table(keep, [ps, Cs, Ts], xio)
    f.gas_density = abi.constant(100.0, 3)
    f.oil_viscosity = abi.constant(5.0 * CENTIPOISE, 3)
    f.gas_viscosity = abi.constant(1.0e-5, 3)
    f.oil_enthalpy = abi.constant(0.0, 3)
    f.gas_enthalpy = abi.constant(0.0, 3)
    return f


def corey(swc=0.2, sor=0.2, n=2.0):
    c = abi.rsg_corey()
    c.Sr[0], c.Sr[1], c.Sr[2] = swc, sor, 0.0
    for ph in range(3):
        c.n[ph] = n
        c.ke[ph] = 1.0
    c.aw = c.aow = c.ag = c.aog = 1.0
    return c


def rock_tables(keep, kind=abi.RF_TABULAR, swc=0.2, sor=0.2, points=21, pc_kpa=5.0):
    """Tabular rock-fluid curves (rsg_rock_tables) sampled from power laws
    with end points swc and sor: RF_TABULAR gives TabularRockFluid's 1D
    krw(Sw) (exponent 2), krg(Sg) (2), krow(So) (3), krog(So + Sw) (2) and a
    capillary pressure pcow(Sw) falling from pc_kpa kPa; RF_THREE_PHASE_TABULAR
    gives ThreePhaseTabularRockFluid's 2D krw, krg, kro and pcow of (Sw, Sg)
    on a points x points grid of [0, 1]^2 (pcgo 0)."""
    t = abi.rsg_rock_tables()
    t.kind = kind
    s = np.linspace(0.0, 1.0, points)

    def ramp(x, lo, hi, e):
        return np.clip((x - lo) / (hi - lo), 0.0, 1.0) ** e

    if kind == abi.RF_TABULAR:
        t.krw = abi.table(keep, [s], ramp(s, swc, 1 - sor, 2.0))
        t.krg = abi.table(keep, [s], ramp(s, 0.0, 1 - swc, 2.0))
        t.krow = abi.table(keep, [s], ramp(s, sor, 1 - swc, 3.0))
        t.krog = abi.table(keep, [s], ramp(s, swc + sor, 1.0, 2.0))
        t.kro = abi.constant(0.0)
        t.pcow = abi.table(keep, [s], pc_kpa * 1e3 * (1 - ramp(s, swc, 1 - sor, 1.0)))
        t.pcgo = abi.constant(0.0)
    else:
        W_, G_ = np.meshgrid(s, s, indexing="ij")
        O_ = 1 - W_ - G_
        t.krw = abi.table(keep, [s, s], ramp(W_, swc, 1 - sor, 2.0))
        t.krg = abi.table(keep, [s, s], ramp(G_, 0.0, 1 - swc, 2.0))
        t.kro = abi.table(keep, [s, s], ramp(O_, sor, 1 - swc, 2.0))
        t.krow = abi.constant(0.0, 2)
        t.krog = abi.constant(0.0, 2)
        t.pcow = abi.table(keep, [s, s], pc_kpa * 1e3 * (1 - ramp(W_, swc, 1 - sor, 1.0)))
        t.pcgo = abi.constant(0.0, 2)
    return t


def runspec(method=abi.BICGSTAB, precond=abi.PC_ILU, rtol=1e-8, atol=1e-50, max_linear=5000,
            max_newton=10, ptol=1e-6, stop_rule=0, inner_iterations=0, inner_tolerance=0.0, omega=0.0, ax=0.0,
            ay=0.0):
    """RunSpec (rs/src/no/uib/cipr/rs/numerics/RunSpec.java) as rsg_runspec;
    omega, ax, ay: the rotating frame of Field's BodyForces."""
    s = abi.rsg_runspec()
    s.max_nonlinear_pressure_iterations = max_newton
    s.pressure_tolerance = ptol
    s.linear_solver = method
    s.preconditioner = precond
    s.max_linear_iterations = max_linear
    s.relative_tolerance = rtol
    s.absolute_tolerance = atol
    s.divergence_tolerance = 1e5
    s.truncate_negative_moles = 0
    s.newton_stop_rule = stop_rule
    s.gmres_restart = 30
    s.inner_iterations = inner_iterations
    s.inner_tolerance = inner_tolerance
    s.omega = omega
    s.ax = ax
    s.ay = ay
    return s


def two_phase_case(ni=128, nj=128, nk=32, seed=1, perturb=0.1, corr_len=8.0, kz_ratio=0.1, sw0=0.25,
                   rate_m3_per_day=0.02, dt=8640.0):
    """3D oil/water case (five-spot: four corner injector columns as Regular
    sources, a centre producer column as a Fixed source)."""
    n = ni * nj * nk
    nodes = perturbed_nodes(ni, nj, nk, 1.0, 1.0, -1.0, perturb, seed)
    logk = grf((ni, nj, nk), corr_len, 2.0, 1.0, seed + 1000)
    kx = _cells_ijk_to_linear(10.0 ** logk) * MILLIDARCY
    perm = np.zeros((n, 6))
    perm[:, 0] = kx
    perm[:, 1] = kx
    perm[:, 2] = kz_ratio * kx
    poro = rng(seed + 2000).uniform(0.20, 0.30, n)
    comp = np.zeros(n)

    def column(i, j):
        return np.array([i + j * ni + k * ni * nj for k in range(nk)], dtype=np.int32)

    injectors = [column(0, 0), column(ni - 1, 0), column(0, nj - 1), column(ni - 1, nj - 1)]
    producer = column(ni // 2, nj // 2)
    # initial water/oil mole fractions giving S_w ~ sw0 at 200 bar
    xiw0, xio0 = 1000.0 / 0.01801528, 800.0 / 0.2
    nw, no = sw0 * xiw0, (1 - sw0) * xio0
    cw, co = nw / (nw + no), no / (nw + no)
    q_water = rate_m3_per_day * xiw0 / 86400.0  # mol/s per injector cell
    return dict(
        dim=3, ni=ni, nj=nj, nk=nk, nodes=nodes, perm=np.ascontiguousarray(perm), porosity=poro,
        compaction=comp, injectors=injectors, producer=producer, fractions=(cw, co), q_water=q_water,
        temperature=350.0, datum_pressure=200 * BAR, datum_depth=0.0, dt=dt, seed=seed,
    )


GAS_CONSTANT = 8.3145  # J/(mol K), util/Constants.java:23


def three_phase_fluid(keep, p_range=(20 * BAR, 600 * BAR), n_p=64, gas_swelling=0.5):
    """Water, oil and gas black-oil fluid (one component per group): the
    bubble point (gas fraction of a saturated oil) rises linearly from 0.05 at
    20 bar to 0.40 at 600 bar, the dew point (oil fraction of a saturated gas)
    is 0.02; oil molar density has 1e-4 /bar compressibility and rises with
    dissolved gas (x(1 + C)), gas molar density is p / (0.9 R T), x(1 +
    gas_swelling C) with vaporised oil fraction C; viscosities 1 cP water,
    2 cP oil, 0.02 cP gas."""
    p0 = 200 * BAR
    ps = np.linspace(p_range[0], p_range[1], n_p)
    Ts = np.array([250.0, 450.0])
    Cs = np.array([0.0, 1.0])
    xiw0, cw = 1000.0 / 0.01801528, 4.0e-5 / BAR
    xio0, co = 800.0 / 0.2, 1.0e-4 / BAR
    f = abi.rsg_blackoil()
    f.nc = 3
    for nu, (mw, grp) in enumerate(((0.01801528, 0), (0.2, 1), (0.02, 2))):
        f.molecular_weight[nu] = mw
        f.group[nu] = grp
    f.water_density = abi.table(keep, [ps, Ts], np.repeat((xiw0 * np.exp(cw * (ps - p0)))[:, None], 2, axis=1))
    f.water_viscosity = abi.constant(1.0 * CENTIPOISE, 2)
    f.water_enthalpy = abi.constant(0.0, 2)
    cb = 0.05 + 0.35 * (ps - p_range[0]) / (p_range[1] - p_range[0])
    f.bubble_point = abi.table(keep, [ps, Ts], np.repeat(cb[:, None], 2, axis=1))
    f.dew_point = abi.constant(0.02, 2)
    P, C, T = np.meshgrid(ps, Cs, Ts, indexing="ij")
    f.oil_density = abi.table(keep, [ps, Cs, Ts], xio0 * np.exp(co * (P - p0)) * (1.0 + C))
    f.gas_density = abi.table(keep, [ps, Cs, Ts], P / (0.9 * GAS_CONSTANT * T) * (1.0 + gas_swelling * C))
    f.oil_viscosity = abi.constant(2.0 * CENTIPOISE, 3)
    f.gas_viscosity = abi.constant(0.02 * CENTIPOISE, 3)
    f.oil_enthalpy = abi.constant(0.0, 3)
    f.gas_enthalpy = abi.constant(0.0, 3)
    return f


def three_phase_case(ni=12, nj=12, nk=4, seed=5, rate_m3_per_day=0.05, dt=8640.0):
    """Water, oil and gas on the two-phase case's grid: a gas cap in the top
    layer (hydrocarbons 99% gas: single-phase gas), undersaturated oil below
    (12% gas against a 16% bubble point at 200 bar: single-phase oil), gas
    injected in the four corner columns (two-phase oil/gas where it mixes
    with the oil) and the Fixed producer column holding the oil zone's
    composition."""
    case = two_phase_case(ni=ni, nj=nj, nk=nk, seed=seed, dt=dt)
    keep = abi.Keep()
    T = case["temperature"]
    xiw0, xio0 = 1000.0 / 0.01801528, 800.0 / 0.2
    xig0 = 200 * BAR / (0.9 * GAS_CONSTANT * T)

    def fractions(sw, zg, xi_hc):
        nw, nhc = sw * xiw0, (1 - sw) * xi_hc
        tot = nw + nhc
        return nw / tot, (1 - zg) * nhc / tot, zg * nhc / tot

    oil_zone = fractions(0.25, 0.12, xio0 * 1.12)
    gas_cap = fractions(0.20, 0.99, xig0 * 1.005)
    zs = [-(nk + 1.0), -1.0, -0.99, 1.0]
    case["fraction_fns"] = [abi.table(keep, [zs], [o, o, g, g]) for o, g in zip(oil_zone, gas_cap)]
    case["fractions"] = oil_zone
    case["q"] = {2: rate_m3_per_day * xig0 / 86400.0}
    case["keep"] = keep
    return case


def build_sources(keep, case):
    """Regular sources at the injector columns (case["q"]: component -> mol/s
    per cell, water by default) and a Fixed source at the producer column
    holding case["fractions"]."""
    srcs = (abi.rsg_source * (len(case["injectors"]) + 1))()
    rates = case.get("q", {0: case.get("q_water", 0.0)})
    for a, cells in enumerate(case["injectors"]):
        arr = keep.i32(cells)
        srcs[a].type = abi.SOURCE_REGULAR
        srcs[a].num_elements = len(arr)
        srcs[a].elements = abi.iptr(arr)
        for nu, q in rates.items():
            srcs[a].q[nu] = q
    arr = keep.i32(case["producer"])
    last = len(case["injectors"])
    srcs[last].type = abi.SOURCE_FIXED
    srcs[last].num_elements = len(arr)
    srcs[last].elements = abi.iptr(arr)
    srcs[last].temperature = case["temperature"]
    for nu, c in enumerate(case["fractions"]):
        srcs[last].fraction[nu] = c
    return srcs


def build_initial(case):
    """Initial values: datum, constant temperature and per-component mole
    fractions, constant or given as functions of depth (case["fraction_fns"])."""
    init = abi.rsg_initial()
    init.datum_depth = case["datum_depth"]
    init.datum_pressure = case["datum_pressure"]
    init.temperature = abi.constant(case["temperature"], 1)
    fns = case.get("fraction_fns")
    for nu in range(abi.MAX_COMPONENTS):
        if fns is not None and nu < len(fns):
            init.fraction[nu] = fns[nu]
        else:
            c = case["fractions"][nu] if nu < len(case["fractions"]) else 0.0
            init.fraction[nu] = abi.constant(c, 1)
    return init


def build_two_phase_sim(ctx, ni, nj, nk, seed=1, **spec_kw):
    """A Discretisation of the two-phase case on ctx (mesh, MPFA-O,
    initialisation); returns (sim, case).  The arrays the library reads
    through raw pointers stay referenced by the returned objects."""
    from . import api

    case = two_phase_case(ni=ni, nj=nj, nk=nk, seed=seed)
    keep = abi.Keep()
    fluid = two_phase_fluid(keep)
    srcs = build_sources(keep, case)
    mesh = api.Mesh(ctx, 3, ni, nj, nk, case["perm"], coords=case["nodes"])
    mesh.compute_mpfa()
    sim = api.Discretisation(ctx, mesh, fluid, corey(), case["porosity"], case["compaction"], srcs,
                             build_initial(case), runspec(**spec_kw))
    sim._member_keep = (keep, srcs, mesh)
    return sim, case


def ensemble_sizes(count, seed=7, lo=(32, 32, 8), hi=(96, 96, 24)):
    """Grid sizes of an ensemble, each axis uniform in [lo, hi] from a seeded draw."""
    g = np.random.Generator(np.random.PCG64(seed))
    return [tuple(int(g.integers(lo[a], hi[a] + 1)) for a in range(3)) for _ in range(count)]


def compositional_fluid(keep, seed=3, nhc=3):
    """Peng-Robinson fluid of the compositional configuration: water plus
    `nhc` hydrocarbon pseudo-components (the last standing in for CO2) with
    Tc ~ U(190, 620) K, pc ~ U(20, 50) bar, omega ~ U(0.01, 0.5) and
    symmetric binary interaction coefficients ~ U(0, 0.15), all seeded.
    Molecular weights and critical volumes follow Tc (heavier components are
    more critical); the water phase uses the same density table as the
    two-phase case and a 0.5 cP viscosity."""
    g = np.random.Generator(np.random.PCG64(seed))
    nc = nhc + 1
    f = abi.rsg_cubic_fluid()
    f.nc = nc
    f.eos = abi.EOS_PR
    Tc = np.sort(g.uniform(190.0, 620.0, nhc))
    pc = g.uniform(20.0, 50.0, nhc) * BAR
    om = g.uniform(0.01, 0.5, nhc)
    for k in range(nhc):
        i = k + 1
        f.Tc[i] = Tc[k]
        f.pc[i] = pc[k]
        f.omega[i] = om[k]
        f.Mw[i] = 0.016 + 0.25 * (Tc[k] - 190.0) / 430.0
        f.Vc[i] = 1.0e-4 + 5.0e-4 * (Tc[k] - 190.0) / 430.0
        f.shift[i] = 0.0
    f.Mw[0] = 0.01801528
    for i in range(1, nc):
        for j in range(i + 1, nc):
            d = g.uniform(0.0, 0.15)
            f.bic[i * abi.MAX_COMPONENTS + j] = f.bic[j * abi.MAX_COMPONENTS + i] = d
    f.flash_criteria = 1e4
    f.flash_tolerance = 1e-1
    f.flash_max_iterations = 100000  # the Java loop has no bound; near-critical cells take thousands
    for k, v in enumerate((0.1023, 0.023364, 0.058533, -0.040758, 0.0093324)):
        f.lbc[k] = v
    ps = np.linspace(20 * BAR, 600 * BAR, 64)
    Ts = np.array([250.0, 450.0])
    xiw = np.repeat((1000.0 / 0.01801528 * np.exp(4.0e-5 / BAR * (ps - 200 * BAR)))[:, None], 2, axis=1)
    f.water_density = abi.table(keep, [ps, Ts], xiw)
    f.water_viscosity = abi.constant(0.5 * CENTIPOISE, 2)
    return f


def compositional_cells(n, nc, seed=5, p_range=(60 * BAR, 400 * BAR), T_range=(300.0, 400.0)):
    """Seeded per-cell pressure, temperature and moles (component major) for
    flash tests: water plus hydrocarbon moles of varying composition, some
    cells without water and some with one hydrocarbon absent."""
    g = np.random.Generator(np.random.PCG64(seed))
    p = g.uniform(*p_range, n)
    T = g.uniform(*T_range, n)
    N = g.uniform(0.0, 1000.0, (nc, n))
    N[0, g.random(n) < 0.3] = 0.0
    for i in range(n):
        if g.random() < 0.15:
            N[1 + g.integers(nc - 1), i] = 0.0
    return p, T, N


def compositional_case(ni, nj, nk, seed=1, perturb=0.1, corr_len=8.0, kz_ratio=0.1, dt=8640.0,
                       rate_mol_per_s=2.0e-3, fractions=(0.3, 0.4, 0.25, 0.05)):
    """Compositional line drive on the compositional fluid: the last
    hydrocarbon (the CO2 stand-in) injected into the column (0, 0) as a
    Regular source, a Fixed producer column at (ni-1, nj-1); initial moles
    from the given overall mole fractions (water first) at 200 bar, 350 K."""
    n = ni * nj * nk
    nodes = perturbed_nodes(ni, nj, nk, 1.0, 1.0, -1.0, perturb, seed)
    logk = grf((ni, nj, nk), corr_len, 2.0, 1.0, seed + 1000)
    kx = _cells_ijk_to_linear(10.0 ** logk) * MILLIDARCY
    perm = np.zeros((n, 6))
    perm[:, 0] = kx
    perm[:, 1] = kx
    perm[:, 2] = kz_ratio * kx
    poro = rng(seed + 2000).uniform(0.20, 0.30, n)

    def column(i, j):
        return np.array([i + j * ni + k * ni * nj for k in range(nk)], dtype=np.int32)

    return dict(dim=3, ni=ni, nj=nj, nk=nk, nodes=nodes, perm=np.ascontiguousarray(perm), porosity=poro,
                compaction=np.zeros(n), injector=column(0, 0), producer=column(ni - 1, nj - 1),
                fractions=tuple(fractions), q_inject=rate_mol_per_s, temperature=350.0,
                datum_pressure=200 * BAR, datum_depth=0.0, dt=dt, seed=seed)


def build_compositional_sources(keep, case, nc):
    srcs = (abi.rsg_source * 2)()
    arr = keep.i32(case["injector"])
    srcs[0].type = abi.SOURCE_REGULAR
    srcs[0].num_elements = len(arr)
    srcs[0].elements = abi.iptr(arr)
    srcs[0].q[nc - 1] = case["q_inject"]
    arr = keep.i32(case["producer"])
    srcs[1].type = abi.SOURCE_FIXED
    srcs[1].num_elements = len(arr)
    srcs[1].elements = abi.iptr(arr)
    srcs[1].temperature = case["temperature"]
    for nu in range(nc):
        srcs[1].fraction[nu] = case["fractions"][nu]
    return srcs


def build_compositional_initial(case, nc):
    init = abi.rsg_initial()
    init.datum_depth = case["datum_depth"]
    init.datum_pressure = case["datum_pressure"]
    init.temperature = abi.constant(case["temperature"], 1)
    for nu in range(abi.MAX_COMPONENTS):
        init.fraction[nu] = abi.constant(case["fractions"][nu] if nu < nc else 0.0, 1)
    return init
