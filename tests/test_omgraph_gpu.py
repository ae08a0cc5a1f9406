"""General OM graphs on the GPU (om_create_graph): the reference's examples
and graphs that exercise every operation, against the numpy oracle of the
same semantics (bit-exact; transcendental functions within a few ulp)."""
import numpy as np
import pytest

from oracle import omgraph_ref as R
from paraiso_gb300 import omgraph as og
from paraiso_gb300 import omgraph_examples as ex

pytestmark = pytest.mark.gpu


def both(om_lib, om, kernels, init=None):
    g = om_lib.GraphMachine(om)
    m = R.Machine(om.to_text())
    if init:
        for name, a in init.items():
            g.write(name, a)
            m.values[name] = a.copy()
    for k in kernels:
        g.run(k)
        m.run(k)
    return g, m


def assert_same(g, m, names, rtol=0.0):
    for n in names:
        realm = m.om["statics"][n][0]
        got = g.read(n) if realm == "array" else g.get_scalar(n)
        want = m.values[n]
        if realm == "array":          # a 1-D machine reads back as (1, n)
            want = np.asarray(want).reshape(np.shape(got))
        if rtol == 0.0:
            assert np.array_equal(np.asarray(got), np.asarray(want).astype(np.asarray(got).dtype)), n
        else:
            np.testing.assert_allclose(got, want, rtol=rtol, atol=rtol)


@pytest.mark.parametrize("boundary", ["open", "cyclic"])
def test_shift_example(om_lib, boundary):
    g, m = both(om_lib, ex.shift_example(boundary), [])
    assert g.om_lower_margin(0) == m.lm[0] and g.om_upper_margin(0) == m.um[0]
    for k in ("init", "increment", "calculate"):
        g.run(k)
        m.run(k)
        assert_same(g, m, ["table", "total"])
    g.close()


def test_hello_world(om_lib):
    g, m = both(om_lib, ex.hello_world(), ["create"])
    assert g.get_scalar("total") == 8550
    assert_same(g, m, ["table", "total"])
    g.close()


def test_initial_condition(om_lib):
    g, m = both(om_lib, ex.initial_condition(), ["create"])
    got, want = g.read("table"), m.values["table"]
    assert got.shape == (500, 500)
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13)
    g.close()


@pytest.mark.parametrize("size", [(256, 192), (37, 29)])
def test_life_graph_matches_life_oracle(om_lib, oracle, size):
    a = oracle.life_bernoulli(size[0], size[1], 7, 0.3)
    g = om_lib.GraphMachine(ex.life(size))
    g.write("cell", a)
    g.run("proceed", 30)           # one captured CUDA graph of 30 steps
    ref, pops = oracle.life_run(a, 30, cyclic=True)
    assert np.array_equal(g.read("cell"), ref)
    assert g.get_scalar("population") == int(pops[-1])
    assert g.get_scalar("generation") == 30
    for _ in range(3):             # single steps continue from there
        g.run("proceed")
    ref, pops = oracle.life_run(ref, 3, cyclic=True)
    assert np.array_equal(g.read("cell"), ref) and g.get_scalar("generation") == 33
    g.close()


def test_life_graph_open(om_lib, oracle):
    om = ex.life((64, 48), "open")
    a = np.zeros((50, 66), np.int32)
    a[1:-1, 1:-1] = oracle.life_bernoulli(64, 48, 3, 0.4)
    g, m = both(om_lib, om, ["proceed"] * 5, init={"cell": a})
    assert (g.om_lower_margin(0), g.om_upper_margin(1)) == (1, 1)
    assert_same(g, m, ["cell", "population", "generation"])
    g.close()


def semantics_graph(boundary, size=(61, 37)):
    """Every operation of the format, several types, two reduce stages."""
    om = og.OM("Sem", size, boundary)
    f = om.static_array("f", og.Float)
    d = om.static_array("d", og.Double)
    i = om.static_array("i", og.Int)
    b = om.static_array("b", og.Bool)
    s_min = om.static_scalar("smin", og.Float)
    s_max = om.static_scalar("smax", og.Double)
    s_sum = om.static_scalar("ssum", og.Int)
    s_flag = om.static_scalar("flag", og.Bool)
    k = om.kernel("step")
    fv, dv, iv = k.load(f), k.load(d), k.load(i)
    x = k.load_index(0)
    y = k.load_index(1)
    # integer division and modulo of mixed signs (C truncation); divisors
    # are never zero
    den1 = og.select((y - 13).eq(0), 1, y - 13)
    den2 = og.select((x - 17).eq(0), 1, x - 17)
    k.store(i, (iv - 7 * x) // den1 + (iv * 3) % den2)
    # float: shifts both ways, max/min order, abs, signum, inv, cast
    fs = k.shift(fv, (1, -1)) - k.shift(fv, (-2, 0))
    ff = og.max_(fs, fv) * 0.5 + og.min_(-fv, fs) + og.abs_(fs) * og.signum(fv)
    ff = ff + og.cast(og.cast(fv * 10, og.Int), og.Float) + og.recip(og.abs_(fv) + 1)
    k.store(f, ff)
    # double: transcendental functions and pow
    dd = og.sqrt(og.abs_(dv) + 1) + og.exp(-og.abs_(dv)) + og.log(og.abs_(dv) + 2)
    dd = dd + og.sin(dv) * og.cos(dv) + og.atan2(dv, og.cast(x, og.Double) + 1)
    dd = dd + og.pow_(og.abs_(dv) + 1, dv * 0.25) + og.tan(dv * 0.1) + og.atan(dv)
    dd = dd + og.asin(og.sin(dv) * 0.5) + og.acos(og.cos(dv) * 0.5)
    k.store(d, dd)
    # bool logic
    k.store(b, (k.load(b) & (fv > 0)) | ~(dv <= 0.5))
    # reductions, including regions that exclude cells (open: zeros join)
    k.store(s_min, k.reduce("min", fs))
    k.store(s_max, k.reduce("max", dd))
    k.store(s_sum, k.reduce("sum", og.cast(fs > 0, og.Int)))
    # second stage: a reduce result broadcast back into an array
    k2 = om.kernel("center")
    fv2 = k2.load(f)
    k2.store(f, fv2 - k2.broadcast(k2.reduce("sum", fv2) /
                                   k2.imm(float(size[0] * size[1]), og.Float, "scalar")))
    k2.store(s_flag, k2.reduce("max", og.cast(k2.load(b), og.Int)).eq(k2.imm(1, og.Int, "scalar")))
    return om


@pytest.mark.parametrize("boundary", ["cyclic", "open"])
def test_semantics_graph(om_lib, boundary):
    om = semantics_graph(boundary)
    m0 = R.Machine(om.to_text())
    rng = np.random.default_rng(11)
    shape = m0.shape
    init = {"f": rng.standard_normal(shape).astype(np.float32),
            "d": rng.standard_normal(shape),
            "i": rng.integers(-1000, 1000, shape).astype(np.int32),
            "b": rng.random(shape) < 0.5}
    g, m = both(om_lib, om, ["step", "step"], init=init)
    assert_same(g, m, ["i", "b", "smin", "ssum"])
    assert_same(g, m, ["f"])                      # + - * / max min abs cast: exact
    assert_same(g, m, ["d", "smax"], rtol=1e-12)  # transcendental: a few ulp
    g.run("center")
    m.run("center")
    np.testing.assert_allclose(g.read("f"), m.values["f"], rtol=1e-6, atol=1e-6)
    assert g.get_scalar("flag") == int(m.values["flag"])
    g.close()


@pytest.mark.parametrize("n,boundary", [(64, "cyclic"), (1024, "cyclic"), (48, "open")])
def test_linear_wave(om_lib, n, boundary):
    # examples-old/LinearWave (1-D, double, sin/cos, shifts, a sum).  The
    # start differs from numpy's sin/cos by an ulp at most; the scheme runs
    # at Courant number 1, where such differences grow, so the 40 steps start
    # both machines from the GPU's fields: + - * / agree bit for bit
    om = ex.linear_wave(n, boundary)
    g, m = both(om_lib, om, ["initialize"])
    assert_same(g, m, ["fieldF", "fieldG"], rtol=1e-15)
    for name in ("fieldF", "fieldG"):
        m.values[name] = g.read(name).reshape(np.shape(m.values[name]))
    for _ in range(40):
        g.run("proceed")
        m.run("proceed")
    assert_same(g, m, ["fieldF", "fieldG"])
    assert_same(g, m, ["energy"], rtol=1e-12)      # block-order sum
    g.close()


def test_generated_source_is_available(om_lib):
    g = om_lib.GraphMachine(ex.hello_world())
    src = g.source
    assert "om_k0_s0" in src and "__global__" in src
    g.close()


HYDRO_FIELDS = ("density", "velocity0", "velocity1", "pressure")


def hydro_graph(om_lib, state, n0, n1, gamma, boundary, typ, cfl):
    """examples/Hydro's OM, written in the builder, on the executor, with the
    scalars the Hydro drivers set (dR = extent / n, unit extent)."""
    g = om_lib.GraphMachine(ex.hydro((n0, n1), gamma, boundary, typ))
    f = np.float32 if typ == og.Float else np.float64
    for name, v in (("cfl", f(cfl)), ("dR0", f(1) / f(n0)), ("dR1", f(1) / f(n1)),
                    ("extent0", f(1)), ("extent1", f(1)), ("time", f(0))):
        g.set_scalar(name, float(v))
    for name, a in zip(HYDRO_FIELDS, state):
        g.write(name, a)
    return g


def test_hydro_graph_cyclic_fp64_matches_oracle(om_lib, oracle):
    n0, n1 = 96, 64
    st = oracle.hydro_init_kh(n0, n1, 3)
    g = hydro_graph(om_lib, st, n0, n1, 1.4, "cyclic", og.Double, 0.4)
    g.run("proceed")
    g.run("proceed", 5)              # five more steps in one captured graph
    ref, t, _ = oracle.hydro_run(st, 6, cyclic=True, gamma=1.4, cfl=0.4)
    for name, a in zip(HYDRO_FIELDS, ref):
        assert np.array_equal(g.read(name), a), name
    assert g.get_scalar("time") == t
    g.close()


def test_hydro_graph_open_matches_reference_golden(om_lib, oracle):
    # 1024^2 float, open (3-cell margins found by the executor), gamma 5/3,
    # 2 steps: bit-identical to the reference's generated float code
    import hashlib
    import os
    gold = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                "hydro_ref_jet.npz"))
    st = oracle.hydro_init_jet(1024, 1024, cyclic=False, gamma=5 / 3, dtype=np.float32)
    g = hydro_graph(om_lib, st, 1024, 1024, 5 / 3, "open", og.Float, float(gold["cfl"]))
    assert (g.om_lower_margin(0), g.om_upper_margin(1)) == (3, 3)
    g.run("proceed")
    g.run("proceed")
    got = [hashlib.sha256(np.ascontiguousarray(g.read(n)).tobytes()).hexdigest()
           for n in HYDRO_FIELDS]
    assert got == [str(s) for s in gold["sha256"]]
    assert np.float32(g.get_scalar("time")) == np.float32(gold["times"][-1])
    g.close()


def test_life_graph_four_cells_per_thread(om_lib, oracle):
    # rows of 2048 cells: each thread of the stage evaluates several
    # neighbouring cells (the generated source says so); results equal the
    # Life oracle
    a = oracle.life_bernoulli(2048, 40, 9, 0.3)
    g = om_lib.GraphMachine(ex.life((2048, 40)))
    assert "threadIdx.x * 8" in g.source or "threadIdx.x * 4" in g.source
    g.write("cell", a)
    g.run("proceed", 12)
    ref, pops = oracle.life_run(a, 12, cyclic=True)
    assert np.array_equal(g.read("cell"), ref)
    assert g.get_scalar("population") == int(pops[-1])
    g.close()


@pytest.mark.parametrize("boundary", ["cyclic", "open"])
def test_semantics_graph_long_rows(om_lib, boundary):
    # the operation mix on rows of 1024 cells (several cells per thread where
    # the stage allows it)
    om = semantics_graph(boundary, (1024, 9))
    m0 = R.Machine(om.to_text())
    rng = np.random.default_rng(12)
    shape = m0.shape
    init = {"f": rng.standard_normal(shape).astype(np.float32),
            "d": rng.standard_normal(shape),
            "i": rng.integers(-1000, 1000, shape).astype(np.int32),
            "b": rng.random(shape) < 0.5}
    g, m = both(om_lib, om, ["step"], init=init)
    assert_same(g, m, ["i", "b", "smin", "ssum", "f"])
    assert_same(g, m, ["d", "smax"], rtol=1e-12)
    g.close()


def stencil_graph(size):
    """Shifts from -9 to +9 columns and -1 to +1 rows of float, double, int
    and bool arrays and of a manifest: columns inside the thread's four,
    in the neighbouring lane's four and beyond."""
    om = og.OM("Wide", size, "cyclic")
    f = om.static_array("f", og.Float)
    d = om.static_array("d", og.Double)
    i = om.static_array("i", og.Int)
    b = om.static_array("b", og.Bool)
    s = om.static_scalar("s", og.Double)
    k = om.kernel("step")
    fv, dv, iv, bv = k.load(f), k.load(d), k.load(i), k.load(b)
    shifts = [(-9, 0), (-5, 1), (-4, -1), (-3, 0), (-1, 1), (1, -1), (3, 0), (4, 1), (5, -1),
              (7, 0), (8, 1), (9, -1)]
    ff, dd, ii = fv, dv, iv
    for n, v in enumerate(shifts):
        ff = ff * 0.75 + k.shift(fv, v) * (0.125 * (n + 1))
        dd = dd - k.shift(dv, v) * (0.0625 * (n + 1))
        ii = ii + k.shift(iv, v) * (n + 1)
    m = dd * 0.5 + og.cast(ff, og.Double)
    k.manifest(m)
    k.store(f, ff)
    k.store(i, ii % 1000003)
    k.store(b, k.shift(bv, (-1, 0)) | (k.shift(bv, (5, 1)) & (fv > 0)))
    k.store(d, k.shift(m, (-3, 0)) + k.shift(m, (6, -1)) - k.shift(m, (1, 1)) * 0.25)
    k.store(s, k.reduce("sum", dd))
    return om


@pytest.mark.parametrize("size", [(2048, 7), (1024, 3)])
def test_row_vectors_and_lane_shuffles(om_lib, size):
    # rows of whole 1024-cell chunks: four cells per thread, row vectors,
    # neighbouring columns from the lanes beside; equal to the oracle
    om = stencil_graph(size)
    m0 = R.Machine(om.to_text())
    rng = np.random.default_rng(21)
    shape = m0.shape
    init = {"f": rng.standard_normal(shape).astype(np.float32),
            "d": rng.standard_normal(shape),
            "i": rng.integers(-1000, 1000, shape).astype(np.int32),
            "b": rng.random(shape) < 0.5}
    g, m = both(om_lib, om, ["step", "step"], init=init)
    assert "*(const om_v2d *)" in g.source and "*(const om_v4f *)" in g.source
    assert "__shfl_down_sync" in g.source
    assert_same(g, m, ["f", "d", "i", "b"])
    assert_same(g, m, ["s"], rtol=1e-12)          # block-order sum
    g.close()


def tiled_graph(size):
    """Computed values read at many offsets (both axes, uneven halos) in
    double, float, int and bool: a stage that computes them once per cell of
    a shared-memory tile."""
    om = og.OM("Tiled", size, "cyclic")
    a = om.static_array("a", og.Double)
    b = om.static_array("b", og.Float)
    n = om.static_array("n", og.Int)
    f = om.static_array("f", og.Bool)
    smin = om.static_scalar("smin", og.Float)
    ssum = om.static_scalar("ssum", og.Int)
    k = om.kernel("step")
    x, y, z = k.load(a), k.load(b), k.load(n)
    u = og.sqrt(og.abs_(x) + 1) * x + og.cast(z, og.Double) * 0.25
    w = y * y - og.cast(z % 7, og.Float) * y
    c = (z * 3 + 1) % 11
    t = (x > 0) & (y < 0.5)
    offsets = [(-2, 0), (1, 0), (0, -1), (0, 3), (3, -2), (-1, 1)]
    su, sw, sc, st = u, w, c, t
    for j, o in enumerate(offsets):
        su = su + k.shift(u, o) * (0.5 + j)
        sw = sw - k.shift(w, o) * (0.25 * (j + 1))
        sc = sc + k.shift(c, o) * (j + 1)
        st = st | (k.shift(t, o) & (y > 0))
    k.store(a, su)
    k.store(b, sw)
    k.store(n, sc)
    k.store(f, st)
    k.store(smin, k.reduce("min", sw))
    k.store(ssum, k.reduce("sum", sc))
    return om


@pytest.mark.parametrize("size", [(70, 41), (64, 16), (5, 3)])
def test_tiled_stage(om_lib, size):
    # values read at several offsets come from a shared-memory tile
    # computed once per cell; meshes that are not whole tiles, and one
    # smaller than the halo; equal to the oracle bit for bit
    om = tiled_graph(size)
    m0 = R.Machine(om.to_text())
    rng = np.random.default_rng(31)
    shape = m0.shape
    init = {"a": rng.standard_normal(shape),
            "b": rng.standard_normal(shape).astype(np.float32),
            "n": rng.integers(-1000, 1000, shape).astype(np.int32),
            "f": rng.random(shape) < 0.5}
    g, m = both(om_lib, om, ["step", "step"], init=init)
    assert "__shared__ double tile" in g.source and "__shared__ float tile" in g.source
    assert "__shared__ int tile" in g.source and "__shared__ bool tile" in g.source
    assert_same(g, m, ["a", "b", "n", "f", "smin", "ssum"])
    g.close()


def manifest_graph(boundary, mark):
    """Values marked Manifest (computed once into an array) and read at
    shifts, by a second manifest, a reduce and stores; unmarked, the same
    graph recomputes them where they are used."""
    om = og.OM("Man", (70, 41), boundary)
    a = om.static_array("a", og.Double)
    b = om.static_array("b", og.Double)
    s = om.static_scalar("s", og.Double)
    k = om.kernel("step")
    x = k.load(a)
    m1 = x * 2 + k.shift(x, (1, 0))
    if mark:
        k.manifest(m1)
    m2 = k.shift(m1, (0, -1)) - k.shift(m1, (-2, 1)) * 0.5
    if mark:
        k.manifest(m2)
    r = k.reduce("sum", m2)
    k.store(b, m2 + k.broadcast(r) * 1e-3 + k.shift(m1, (1, 1)))
    k.store(a, m1)
    k.store(s, r)
    return om


@pytest.mark.parametrize("boundary", ["cyclic", "open"])
def test_manifests(om_lib, boundary):
    rng = np.random.default_rng(5)
    out = []
    for mark in (True, False):
        om = manifest_graph(boundary, mark)
        m0 = R.Machine(om.to_text())
        init = {"a": rng.standard_normal(m0.shape)} if not out else {"a": out[0][2]}
        g, m = both(om_lib, om, ["step", "step"], init=init)
        if mark:
            assert "P.tmp[" in g.source
        assert_same(g, m, ["a"])
        assert_same(g, m, ["b", "s"], rtol=1e-12)
        out.append((g.read("a"), g.read("b"), init["a"], g.get_scalar("s")))
        g.close()
    # marked or not, the executor computes the same values; the reduce's
    # sum (and b through it) may group its terms differently, because the
    # unmarked graph's stage computes shifted values in shared-memory tiles and splits
    # its cells among threads by tiles
    assert np.array_equal(out[0][0], out[1][0])
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-12, atol=1e-12)
    assert abs(out[0][3] - out[1][3]) <= 1e-12 * abs(out[0][3])
