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
