"""The reference's example Orthotope Machines as omgraph builders.

Each function restates one examples/*/Generator.hs kernel for kernel, in the
node order the Haskell builder creates (literals become imm nodes of the
operand's type, ``sum`` folds from an imm 0, ``x^2`` is ``x*x``, ``**`` is
``exp (log x * y)``), so the machine the GPU runs is the one the generator
would have been given.
"""
from __future__ import annotations

from . import omgraph as og


def hello_world(size=(10, 20), boundary="open") -> og.OM:
    """examples/HelloWorld/Generator.hs:36-68: table = x * y, total = sum."""
    om = og.OM("TableMaker", size, boundary)
    table = om.static_array("table", og.Int)
    total = om.static_scalar("total", og.Int)
    k = om.kernel("create")
    x = k.bind(k.load_index(0))
    y = k.bind(k.load_index(1))
    z = k.bind(x * y)
    k.store(table, z)
    k.store(total, k.reduce("sum", z))
    return om


def shift_example(boundary="open", n=8) -> og.OM:
    """examples/ShiftExample/Generator.hs:31-69 (1-D, size 8, open or cyclic)."""
    om = og.OM("TableMaker", (n,), boundary)
    table = om.static_array("table", og.Int)
    total = om.static_scalar("total", og.Int)
    k = om.kernel("init")
    k.store(table, k.load_index(0))
    k = om.kernel("increment")
    k.store(table, 1 + k.load(table))
    k = om.kernel("calculate")
    center = k.bind(k.load(table))
    right = k.bind(k.shift(center, -1))
    left = k.bind(k.shift(center, 1))
    ret = k.bind(10000 * left + 100 * center + right)
    k.store(table, ret)
    k.store(total, k.reduce("sum", ret))
    return om


def initial_condition(size=(500, 500), boundary="open") -> og.OM:
    """examples/InitialCondition/Generator.hs:30-63: a heart-shaped field."""
    om = og.OM("TableMaker", size, boundary)
    table = om.static_array("table", og.Double)
    k = om.kernel("create")
    d = og.Double
    x01 = k.bind(og.cast(k.load_index(0), d) / og.cast(k.broadcast(k.load_size(0)), d))
    y01 = k.bind(og.cast(k.load_index(1), d) / og.cast(k.broadcast(k.load_size(1)), d))
    x = k.bind(4 * (x01 - 0.5))
    y = k.bind(5 * (y01 - 0.5))
    third = k.imm(1, d) / k.imm(3, d)          # the Builder's 1/3: a Div of two imms
    inner = (1 - x ** 2 - (y - (x ** 2).pow_t(third)) ** 2) * 10
    z = k.bind(og.atan(inner))
    k.store(table, z)
    return om


def linear_wave(n=64, boundary="cyclic") -> og.OM:
    """examples-old/LinearWave/Convergence.hs:22-72: a 1-D linear wave
    f' = g, g' = c^2 f'' on [0, 2 pi) and its energy
    sum 0.5 (c^2 (df/dx)^2 + g^2) dx.  The earlier builder's Double-typed
    loadIndex and loadSize are the index and size cast to double."""
    import math
    om = og.OM("LinearWave", (n,), boundary)
    d = og.Double
    F = om.static_array("fieldF", d)
    G = om.static_array("fieldG", d)
    E = om.static_scalar("energy", d)
    k = om.kernel("initialize")
    i = k.bind(og.cast(k.load_index(0), d))
    nn = k.bind(og.cast(k.broadcast(k.load_size(0)), d))
    x = k.bind(k.imm(2, d) * k.imm(math.pi, d) / nn * (i + 0.5))
    k.store(F, og.sin(x))
    k.store(G, og.cos(3 * x))
    k = om.kernel("proceed")
    c = k.bind(k.imm(3.43, d))
    nn = k.bind(og.cast(k.broadcast(k.load_size(0)), d))
    f0 = k.bind(k.load(F))
    g0 = k.bind(k.load(G))
    dx = k.bind(k.imm(2, d) * k.imm(math.pi, d) / nn)
    dt = k.bind(dx / c)
    f1 = k.bind(f0 + dt * g0)
    fR = k.bind(k.shift(f1, -1))
    fL = k.bind(k.shift(f1, 1))
    g1 = k.bind(g0 + dt * c ** 2 / dx ** 2 * (fL + fR - 2 * f1))
    k.store(F, f1)
    k.store(G, g1)
    dfdx = k.bind((fR - fL) / (2 * dx))
    k.store(E, k.reduce("sum", 0.5 * (c ** 2 * dfdx ** 2 + ((g0 + g1) / 2) ** 2) * dx))
    return om


ADJ = list(zip([-1, 0, 1, -1, 1, -1, 0, 1], [-1, -1, -1, 0, 0, 1, 1, 1]))


def life(size=(80, 48), boundary="cyclic") -> og.OM:
    """examples/Life/Generator.hs:36-115: Conway's Life with population and
    generation counters."""
    om = og.OM("Life", size, boundary)
    cell = om.static_array("cell", og.Int)
    population = om.static_scalar("population", og.Int)
    generation = om.static_scalar("generation", og.Int)
    k = om.kernel("init")
    k.store(cell, 0)
    k.store(population, 0)
    k.store(generation, 0)
    k = om.kernel("proceed")
    old = k.bind(k.load(cell))
    gen = k.bind(k.load(generation))
    neighbours = [k.bind(k.shift(old, v)) for v in ADJ]
    num = k.imm(0, og.Int)                     # NumericPrelude sum = foldl (+) zero
    for nb in neighbours:
        num = num + nb
    alive = (old.eq(0) & num.eq(3)) | (old.eq(1) & ((num >= 2) & (num <= 3)))
    new = k.bind(og.select(alive, 1, 0))
    k.store(population, k.reduce("sum", new))
    k.store(generation, gen + 1)
    k.store(cell, new)
    return om


# ---------------------------------------------------------------------------
# examples/Hydro (Hydro.hs, HydroMain.hs)
# ---------------------------------------------------------------------------

class _HydroRecord:
    """A bound Hydro record (Hydro.hs:52-130): every field as a node, made
    in bindHydro's order from a primitive or a conserved triple."""

    def __init__(self, f):
        self.__dict__.update(f)


def _contract(k, terms, typ):
    acc = k.imm(0, typ)                  # foldl (+) zero
    for t in terms:
        acc = acc + t
    return acc


def _bind_hydro(k, g, typ, dens, velo=None, pres=None, mome=None, enrg=None):
    """bindHydro of a PrimitiveVar (dens, velo, pres) or a ConservedVar
    (dens, mome, enrg): the Hydrable defaults, each field bound once."""
    G = lambda: k.imm(g, typ)                           # each kGamma is an imm
    if velo is not None:                                # PrimitiveVar
        density, velocity, pressure = dens, list(velo), pres
        momentum = [density * velocity[i] for i in range(2)]
        kinetic = k.imm(0.5, typ) * _contract(k, [velocity[i] * momentum[i]
                                                  for i in range(2)], typ)
        energy = kinetic + 1 / (G() - 1) * pressure
    else:                                               # ConservedVar
        density, momentum, energy = dens, list(mome), enrg
        velocity = [momentum[i] / density for i in range(2)]
        kinetic = k.imm(0.5, typ) * _contract(k, [velocity[i] * momentum[i]
                                                  for i in range(2)], typ)
        internal = energy - kinetic
        pressure = (G() - 1) * internal
    # bindHydro's order: density, velocity, pressure, momentum, energy, ...
    enthalpy = energy + pressure
    density_flux = momentum
    momentum_flux = [[momentum[i] * velocity[j] + pressure * k.imm(1 if i == j else 0, typ)
                      for j in range(2)] for i in range(2)]
    energy_flux = [enthalpy * velocity[i] for i in range(2)]
    sound = og.sqrt(G() * pressure / density)
    return _HydroRecord(dict(density=density, velocity=velocity, pressure=pressure,
                             momentum=momentum, energy=energy, enthalpy=enthalpy,
                             density_flux=density_flux, momentum_flux=momentum_flux,
                             energy_flux=energy_flux, sound=sound))


_FIELDS = ("density", "velocity", "pressure", "momentum", "energy", "enthalpy",
           "density_flux", "momentum_flux", "energy_flux", "sound")


def _map_record(rec, f):
    out = {}
    for name in _FIELDS:
        v = getattr(rec, name)
        if name == "momentum_flux":
            out[name] = [[f(x) for x in row] for row in v]
        elif isinstance(v, list):
            out[name] = [f(x) for x in v]
        else:
            out[name] = f(v)
    return _HydroRecord(out)


def _zip_records(recs, f):
    out = {}
    for name in _FIELDS:
        vs = [getattr(r, name) for r in recs]
        if name == "momentum_flux":
            out[name] = [[f(*[v[i][j] for v in vs]) for j in range(2)] for i in range(2)]
        elif isinstance(vs[0], list):
            out[name] = [f(*[v[i] for v in vs]) for i in range(2)]
        else:
            out[name] = f(*vs)
    return _HydroRecord(out)


def hydro(size=(1024, 1024), gamma=5.0 / 3.0, boundary="open", typ=og.Double) -> og.OM:
    """examples/Hydro: HydroMain.hs:44-302 with Hydro.hs:37-130 (the
    statics, buildInit, boundaryCondition, buildProceed, proceedSingle,
    addFlux, interpolate, hllc), for gamma and Real of choice."""
    om = og.OM("Hydro", size, boundary)
    T = typ
    om.static_scalar("generation", og.Int)
    time_s = om.static_scalar("time", T)
    cfl_s = om.static_scalar("cfl", T)
    dR_s = [om.static_scalar(f"dR{i}", T) for i in range(2)]
    ext_s = [om.static_scalar(f"extent{i}", T) for i in range(2)]
    dens_s = om.static_array("density", T)
    velo_s = [om.static_array(f"velocity{i}", T) for i in range(2)]
    pres_s = om.static_array("pressure", T)

    def coords(k):
        dRG = [k.load(s) for s in dR_s]
        extG = [k.load(s) for s in ext_s]
        dR = [k.broadcast(v) for v in dRG]
        extent = [k.broadcast(v) for v in extG]
        icoord = [og.cast(k.load_index(i), T) for i in range(2)]
        return dR, extent, icoord, [dR[i] * icoord[i] for i in range(2)]

    def region_of(k, coord, extent):
        return ((coord[1] > k.imm(0.47, T) * extent[1]) & (coord[1] < k.imm(0.53, T) * extent[1])
                & (coord[0] < 0))

    # buildInit (HydroMain.hs:79-102)
    k = om.kernel("init")
    dR, extent, icoord, coord = coords(k)
    region = region_of(k, coord, extent)
    vplus, vminus = (6, 0), (0, 0)
    velo = [og.select(region, k.imm(vplus[i], T), k.imm(vminus[i], T)) for i in range(2)]
    factor = 1 + k.imm(1e-3, T) * og.sin(k.imm(6, T) * k.imm(og.PI, T) * coord[0])
    k.store(dens_s, factor * k.imm(gamma, T) * k.imm(gamma, T) *
            og.select(region, k.imm(1, T), k.imm(10, T)))
    for i in range(2):
        k.store(velo_s[i], velo[i])
    k.store(pres_s, factor * 0.6)

    # buildProceed (HydroMain.hs:134-164)
    k = om.kernel("proceed")
    dens = k.load(dens_s)
    velo = [k.load(s) for s in velo_s]
    pres = k.load(pres_s)
    timeG = k.load(time_s)
    cflG = k.load(cfl_s)
    dRG = [k.load(s) for s in dR_s]
    dR = [k.broadcast(v) for v in dRG]
    cell0 = _bind_hydro(k, gamma, T, dens, velo, pres)

    # boundaryCondition (HydroMain.hs:105-131)
    dRG2 = [k.load(s) for s in dR_s]
    extG = [k.load(s) for s in ext_s]
    dRb = [k.broadcast(v) for v in dRG2]
    extent = [k.broadcast(v) for v in extG]
    icoord = [og.cast(k.load_index(i), T) for i in range(2)]
    isize = [k.broadcast(og.cast(k.load_size(i), T)) for i in range(2)]
    coord = [dRb[i] * icoord[i] for i in range(2)]
    region = region_of(k, coord, extent)
    jet = _bind_hydro(k, gamma, T,
                      k.imm(gamma, T) * k.imm(gamma, T) *
                      og.select(region, k.imm(1, T), k.imm(10, T)),
                      [og.select(region, k.imm(vplus[i], T), k.imm(vminus[i], T))
                       for i in range(2)],
                      k.imm(0.6, T))
    out_of = ((icoord[0] < 0) | (icoord[1] < 0)) | ((icoord[0] >= isize[0]) |
                                                    (icoord[1] >= isize[1]))
    # Anot.add Alloc.Manifest <?> (select outOf a b), per field
    cell = _zip_records([jet, cell0], lambda a, b: k.manifest(og.select(out_of, a, b)))

    # CFL (HydroMain.hs:150-154)
    ts = [dR[i] / (cell.sound + og.abs_(cell.velocity[i])) for i in range(2)]
    dts = og.min_(ts[0], ts[1])
    dtG = cflG * k.reduce("min", dts)
    dt = k.broadcast(dtG)

    def interpolate(order, i, rec):
        def sh(n):
            v = [0, 0]
            v[i] = n
            return lambda x: k.shift(x, tuple(v))
        a0, a1, a2, a3 = (_map_record(rec, sh(n)) for n in (2, 1, 0, -1))

        def single(x0, x1, x2, x3):
            if order == 1:
                return (x1, x2)
            d01, d12, d23 = x1 - x0, x2 - x1, x3 - x2

            def absmaller(a, b):
                return og.select((a * b) <= 0, k.imm(0, T),
                                 og.select(og.abs_(a) < og.abs_(b), a, b))
            d1 = absmaller(d01, d12)
            d2 = absmaller(d12, d23)
            return (x1 + d1 / 2, x2 - d2 / 2)
        lr = _zip_records([a0, a1, a2, a3], single)
        left = _map_record(lr, lambda p: p[0])
        right = _map_record(lr, lambda p: p[1])

        def bp(x):
            return _bind_hydro(k, gamma, T, x.density, list(x.velocity), x.pressure)
        return bp(left), bp(right)

    def hllc(i, left, right):
        G = lambda: k.imm(gamma, T)
        dens_mid = (left.density + right.density) / 2
        sound_mid = (left.sound + right.sound) / 2
        speed_l, speed_r = left.velocity[i], right.velocity[i]
        pres_star = og.max_(k.imm(0, T), (left.pressure + right.pressure) / 2 -
                            dens_mid * sound_mid * (speed_r - speed_l))

        def q(sp, p):
            return og.select(p <= sp, k.imm(1, T),
                             og.sqrt(1 + (G() + 1) / (2 * G()) * (sp / p - 1)))
        shock_l = left.velocity[i] - left.sound * q(pres_star, left.pressure)
        shock_r = right.velocity[i] + right.sound * q(pres_star, right.pressure)
        shock_star = ((right.pressure - left.pressure
                       + left.density * speed_l * (shock_l - speed_l)
                       - right.density * speed_r * (shock_r - speed_r))
                      / (left.density * (shock_l - speed_l) -
                         right.density * (shock_r - speed_r)))

        def star(star_shock, shock, x):
            speed = x.velocity[i]
            d = x.density * (shock - speed) / (shock - star_shock)
            mome = [d * (star_shock if i == j else x.velocity[j]) for j in range(2)]
            e = d * (x.energy / x.density + (star_shock - speed) *
                     (star_shock + x.pressure / x.density / (shock - speed)))
            return _bind_hydro(k, gamma, T, d, mome=mome, enrg=e)
        lesta = star(shock_star, shock_l, left)
        rista = star(shock_star, shock_r, right)

        def selector(a, b, c, d):   # Anot.add Alloc.Manifest <?> select ...
            return k.manifest(og.select(0 < shock_l, a,
                                        og.select(0 < shock_star, b, og.select(0 < shock_r, c, d))))
        return _zip_records([left, lesta, rista, right], selector)

    def add_flux(dt_, dR_, wall, ex, rec):
        dtdx = dt_ / dR_[ex]
        left_w = wall[ex]
        back = [0, 0]
        back[ex] = -1
        right_w = _map_record(wall[ex], lambda x: k.shift(x, tuple(back)))
        dens1 = rec.density + dtdx * (left_w.density_flux[ex] - right_w.density_flux[ex])
        mome1 = [rec.momentum[j] + dtdx * (left_w.momentum_flux[j][ex] -
                                           right_w.momentum_flux[j][ex]) for j in range(2)]
        enrg1 = rec.energy + dtdx * (left_w.energy_flux[ex] - right_w.energy_flux[ex])
        return _bind_hydro(k, gamma, T, dens1, mome=mome1, enrg=enrg1)

    def proceed_single(order, dt_, dR_, cell_f, cell_s):
        wall = [hllc(i, *interpolate(order, i, cell_f)) for i in range(2)]
        # foldl1 (.) over the axes: axis 1 is added first, then axis 0
        cell_n = add_flux(dt_, dR_, wall, 0, add_flux(dt_, dR_, wall, 1, cell_s))
        return _bind_hydro(k, gamma, T, og.max_(k.imm(1e-2, T), cell_n.density),
                           list(cell_n.velocity), og.max_(k.imm(1e-2, T), cell_n.pressure))

    cell2 = proceed_single(1, dt / 2, dR, cell, cell)
    cell3 = proceed_single(2, dt, dR, cell2, cell)
    k.store(time_s, timeG + dtG)
    k.store(dens_s, cell3.density)
    for i in range(2):
        k.store(velo_s[i], cell3.velocity[i])
    k.store(pres_s, cell3.pressure)
    return om
