"""General OM graphs on the CPU side: the builder's graphs, the numpy oracle
against known answers of the reference's examples, and the generated CUDA
compiled for sm_103a with NVRTC (no GPU needed)."""
import ctypes as C

import numpy as np
import pytest

from oracle import omgraph_ref as R
from paraiso_gb300 import omgraph as og
from paraiso_gb300 import omgraph_examples as ex


def run_oracle(om, kernels):
    m = R.Machine(om.to_text())
    for k in kernels:
        m.run(k)
    return m


def test_builder_follows_the_haskell_builder():
    om = og.OM("T", (4, 4), "cyclic")
    a = om.static_array("a", og.Double)
    k = om.kernel("k")
    x = k.load(a)
    k.store(a, (1 - x ** 3).pow_t(0.5))
    text = om.to_text()
    ops = [l.split()[1] for l in text.splitlines() if l[:1].isdigit()]
    # x^3 = x * (x*x) (repeated squaring); 1 - ...; ** = exp (log _ * y)
    assert ops == ["load", "mul", "mul", "imm", "sub", "log", "imm", "mul", "exp"]
    with pytest.raises(og.OMGraphError):
        k.store(a, k.load_index(0))          # int into double: needs a cast
    with pytest.raises(og.OMGraphError):
        x + k.load_size(0)                   # array + scalar: needs broadcast


def test_shift_example_known_answers():
    # examples/ShiftExample/main.cpp: init, increment, calculate on 8 cells.
    # Open: margins 1 and 1; calculate writes cells 0..7 (memory 1..8),
    # 10000*left + 100*center + right with table = index + 1; margins 0.
    m = run_oracle(ex.shift_example("open"), ["init"])
    assert (m.lm, m.um) == ([1], [1])
    assert m.values["table"].ravel().tolist() == list(range(-1, 9))
    m.run("increment")
    assert m.values["table"].ravel().tolist() == list(range(0, 10))
    m.run("calculate")
    want = [0] + [10000 * (i - 1) + 100 * i + (i + 1) for i in range(1, 9)] + [0]
    assert m.values["table"].ravel().tolist() == want
    assert int(m.values["total"]) == sum(want) == 283644
    # cyclic: no margins, neighbours wrap
    m = run_oracle(ex.shift_example("cyclic"), ["init", "increment", "calculate"])
    t = list(range(1, 9))
    want = [10000 * t[(i - 1) % 8] + 100 * t[i] + t[(i + 1) % 8] for i in range(8)]
    assert m.values["table"].ravel().tolist() == want
    assert int(m.values["total"]) == 363636


def test_hello_world_known_answer():
    m = run_oracle(ex.hello_world(), ["create"])
    assert int(m.values["total"]) == 45 * 190
    y, x = np.mgrid[0:20, 0:10]
    assert np.array_equal(m.values["table"], x * y)


def test_life_graph_matches_life_oracle(oracle):
    m = R.Machine(ex.life((40, 24)).to_text())
    a = oracle.life_bernoulli(40, 24, 5, 0.35)
    m.values["cell"] = a.copy()
    for _ in range(12):
        m.run("proceed")
    ref, pops = oracle.life_run(a, 12, cyclic=True)
    assert np.array_equal(m.values["cell"], ref)
    assert int(m.values["population"]) == int(pops[-1])
    assert int(m.values["generation"]) == 12


HYDRO_FIELDS = ("density", "velocity0", "velocity1", "pressure")


def hydro_graph_machine(state, n0, n1, gamma, boundary, typ, cfl):
    """The numpy oracle on examples/Hydro's OM written in the builder, with
    the scalars the Hydro drivers set (dR = extent / n, unit extent)."""
    m = R.Machine(ex.hydro((n0, n1), gamma, boundary, typ).to_text())
    f = np.float32 if typ == og.Float else np.float64
    for name, v in (("cfl", f(cfl)), ("dR0", f(1) / f(n0)), ("dR1", f(1) / f(n1)),
                    ("extent0", f(1)), ("extent1", f(1)), ("time", f(0))):
        m.values[name] = f(v)
    for name, a in zip(HYDRO_FIELDS, state):
        m.values[name] = a.copy()
    return m


@pytest.mark.parametrize("boundary", ["cyclic", "open"])
def test_hydro_graph_matches_hydro_oracle(oracle, boundary):
    # the builder's transcription of HydroMain.hs, run by the numpy graph
    # oracle, against the C restatement of the generated Hydro code (FP64)
    n0, n1, g = 40, 24, 1.4
    cyc = boundary == "cyclic"
    st = (oracle.hydro_init_kh(n0, n1, 5) if cyc else
          oracle.hydro_init_jet(n0, n1, cyclic=False, gamma=g, dtype=np.float64))
    m = hydro_graph_machine(st, n0, n1, g, boundary, og.Double, 0.5)
    assert m.lm == [0, 0] if cyc else m.lm == [3, 3] and m.um == [3, 3]
    for _ in range(4):
        m.run("proceed")
    ref, t, _ = oracle.hydro_run(st, 4, cyclic=cyc, gamma=g, cfl=0.5)
    for name, a in zip(HYDRO_FIELDS, ref):
        assert np.array_equal(np.asarray(m.values[name]).reshape(a.shape), a), name
    assert float(m.values["time"]) == t


def test_hydro_graph_matches_reference_golden(oracle):
    # 1024^2 float, open, gamma 5/3, the generated init, 2 steps: every
    # memory array bit-identical to the reference's generated float code
    import hashlib
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "hydro_ref_jet.npz"))
    st = oracle.hydro_init_jet(1024, 1024, cyclic=False, gamma=5 / 3, dtype=np.float32)
    m = hydro_graph_machine(st, 1024, 1024, 5 / 3, "open", og.Float, float(g["cfl"]))
    m.run("proceed")
    m.run("proceed")
    got = [hashlib.sha256(np.ascontiguousarray(m.values[n]).tobytes()).hexdigest()
           for n in HYDRO_FIELDS]
    assert got == [str(s) for s in g["sha256"]]
    assert np.float32(m.values["time"]) == np.float32(g["times"][-1])


def test_linear_wave_energy_known_answer():
    # examples-old/LinearWave: the scheme (f1 = f0 + dt g0, then g1 from the
    # Laplacian of f1) keeps its discrete energy to rounding, and that energy
    # is near the continuum value 0.5 pi (c^2 + 1) of f = sin x, g = cos 3x
    import math
    m = R.Machine(ex.linear_wave(64).to_text())
    m.run("initialize")
    es = []
    for _ in range(300):
        m.run("proceed")
        es.append(float(m.values["energy"]))
    es = np.array(es)
    assert np.abs(es - es[0]).max() <= 1e-12 * es[0]
    assert abs(es[0] / (0.5 * math.pi * (3.43 ** 2 + 1)) - 1) < 2e-3


def _check(om_lib, text):
    L = om_lib.load_library()
    src = C.c_char_p()
    status = L.om_graph_check(text.encode(), 10, 3, C.byref(src))
    return status, L.om_last_error().decode(), (src.value or b"").decode()


@pytest.mark.parametrize("make", [
    lambda: ex.hello_world(), lambda: ex.shift_example("open"),
    lambda: ex.shift_example("cyclic"), lambda: ex.initial_condition((64, 48)),
    lambda: ex.life(), lambda: ex.life((64, 64), "open"), lambda: ex.linear_wave(),
    lambda: ex.linear_wave(48, "open")])
def test_examples_compile_for_sm103a(om_lib, make):
    status, err, src = _check(om_lib, make().to_text())
    assert status == 0, err
    assert "__global__" in src


def test_row_vectors_on_rows_of_whole_chunks(om_lib):
    # rows of 16384 cells: the Life stage loads each row once as a vector of
    # four cells, takes the columns beside them from the neighbouring lanes
    # (lanes 0 and 31 load those themselves) and stores four cells at once
    status, err, src = _check(om_lib, ex.life((16384, 64)).to_text())
    assert status == 0, err
    stage = src[src.index("om_k1_s0"):src.index("om_k1_commit")]
    assert stage.count("*(const om_v4i *)") == 3
    assert stage.count("__shfl_up_sync") == 3 and stage.count("__shfl_down_sync") == 3
    assert stage.count("*(om_v4i *)") == 1
    # rows that are not whole chunks keep one cell per thread
    status, err, src = _check(om_lib, ex.life((2000, 64)).to_text())
    assert status == 0, err
    assert "om_v4i *)" not in src and "__shfl" not in src


def test_duplicates_merged_and_records_branched(om_lib):
    # examples/Hydro repeats literals, comparisons and expressions; merged,
    # the field selects of an HLLC wall record share one condition, and the
    # one-cell-per-thread wall stages branch on it once per record; the
    # stage-2 walls read the stage-1 state from a shared-memory tile
    g = ex.hydro((256, 256), gamma=1.4, boundary="cyclic", typ=og.Float)
    status, err, src = _check(om_lib, g.to_text())
    assert status == 0, err
    stages = src.split('extern "C" __global__')
    walls2 = [t for t in stages if "om_k1_s2(" in t][0]
    assert "__shared__ float tile" in walls2
    assert walls2.count("      if (v") >= 8
    assert "threadIdx.x * 4" not in walls2
    # merging keeps one node per distinct value: a graph whose two stores
    # repeat one expression computes it once
    om = og.OM("Dup", (64, 32), "cyclic")
    a = om.static_array("a", og.Double)
    b = om.static_array("b", og.Double)
    k = om.kernel("step")
    x = k.load(a)
    k.store(a, og.sqrt(og.abs_(x) + 1) * 3)
    k.store(b, og.sqrt(og.abs_(k.load(a)) + 1) * 3)
    status, err, src = _check(om_lib, om.to_text())
    assert status == 0, err
    assert src.count("sqrt(") == 1   # rows of 64 cells: one cell per thread


def test_graph_errors_are_reported(om_lib):
    bad = [
        "om T 3 4 4 4 cyclic\n",                                   # 3-D
        "om T 1 8 cyclic\nkernel k\n0 load array int nope\nend\n",  # unknown static
        "om T 1 8 cyclic\nstatic a array int\nkernel k\n0 frob array int\nend\n",
        "om T 1 8 cyclic\nstatic a array int\nkernel k\n0 load array int a\n",  # no end
        "om T 1 8 cyclic\nstatic a array double\nkernel k\n0 loadindex array int 0\n"
        "store a 0\nend\n",                                        # type mismatch
    ]
    for text in bad:
        status, err, _ = _check(om_lib, text)
        assert status != 0 and "om_create_graph" in err, text
