"""The CPU oracle, pinned against the reference's own pre-generated code.

Golden fixtures in tests/golden were produced by tests/golden/make_golden.py
from examples-old/Life-exampled/dist/Life.cpp and
examples-old/Hydro-exampled/dist/Hydro.cpp of the reference; where those
classes are compiled here (oracle/_ref), the oracle is also compared with
them directly."""
import hashlib
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load(name):
    return np.load(os.path.join(GOLDEN, name))


# ---- Life --------------------------------------------------------------

def test_life_golden_rpentomino(oracle):
    g = load("life_ref_rpentomino.npz")
    init = np.zeros((130, 130), np.int32)
    for dx, dy in ((1, 0), (2, 0), (0, 1), (1, 1), (1, 2)):  # Life.cpp sub_0
        init[1 + 64 + dy, 1 + 64 + dx] = 1
    cells, pops = oracle.life_run(init, 1000, cyclic=False)
    assert np.array_equal(pops, g["populations"])
    assert pops[-1] == 139
    assert sha(cells) == str(g["cells_sha256"])


def test_life_golden_bernoulli(oracle):
    g = load("life_ref_bernoulli.npz")
    init = oracle.life_bernoulli(128, 128, int(g["seed"]), float(g["p"]), cyclic=False)
    assert np.array_equal(init, g["init"].astype(np.int32))
    cells, pops = oracle.life_run(init, 200, cyclic=False)
    assert np.array_equal(pops, g["populations"])
    assert sha(cells) == str(g["cells_sha256"])


@pytest.mark.parametrize("n0,n1", [(8, 8), (37, 29), (1, 7), (64, 3)])
def test_life_cyclic_glider_and_invariants(oracle, n0, n1):
    # blinker / block / glider behaviour under cyclic wrap, plus the rule
    # checked cell-by-cell against a direct numpy statement of the OM program
    rng = np.random.default_rng(n0 * 100 + n1)
    a = (rng.random((n1, n0)) < 0.35).astype(np.int32)
    c, pops = oracle.life_run(a, 1, cyclic=True)
    num = sum(np.roll(np.roll(a, -dy, 0), -dx, 1)  # shift v reads x[c - v]
              for dx in (-1, 0, 1) for dy in (-1, 0, 1) if (dx, dy) != (0, 0))
    ref = (((a == 0) & (num == 3)) | ((a == 1) & (num >= 2) & (num <= 3))).astype(np.int32)
    assert np.array_equal(c, ref)
    assert pops[0] == ref.sum()


def test_life_glider_wraps(oracle):
    a = np.zeros((16, 16), np.int32)
    for x, y in ((1, 0), (2, 1), (0, 2), (1, 2), (2, 2)):
        a[y, x] = 1
    c, pops = oracle.life_run(a, 64, cyclic=True)   # 16 diagonal cells = full wrap
    assert np.array_equal(c, a)
    assert (pops == 5).all()


def test_life_nonbinary_values(oracle):
    # the generated rule is integer arithmetic: values other than 0/1 count
    a = np.zeros((5, 5), np.int32)
    a[2, 2] = 1
    a[1, 1] = 3      # one neighbour worth 3 -> num == 3 for dead cells around it
    c, _ = oracle.life_run(a, 1, cyclic=True)
    # dead (0,0) sees num 3; live (2,2) sees num 3; the value-3 cell is
    # neither 0 nor 1, so it dies
    assert c[0, 0] == 1 and c[2, 2] == 1 and c[1, 1] == 0


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref",
                                                    "libref_life.so")),
                    reason="reference classes not compiled here")
def test_life_oracle_vs_reference_build(oracle):
    for seed in (3, 4):
        init = oracle.life_bernoulli(128, 128, seed, 0.4, cyclic=False)
        rc, rp = oracle.ref_life_run(init, 150)
        oc, op = oracle.life_run(init, 150, cyclic=False)
        assert np.array_equal(rc, oc) and np.array_equal(rp, op)


# ---- Hydro -------------------------------------------------------------

def test_hydro_golden_jet(oracle):
    g = load("hydro_ref_jet.npz")
    st = oracle.hydro_init_jet(1024, 1024, cyclic=False, gamma=5 / 3, dtype=np.float32)
    out, t, dts = oracle.hydro_run(st, 2, cyclic=False, gamma=5 / 3, cfl=float(g["cfl"]),
                                   dtype=np.float32)
    assert np.float32(t) == g["times"][-1]
    assert [sha(a) for a in out] == [str(s) for s in g["sha256"]]


def test_hydro_golden_random(oracle):
    g = load("hydro_ref_random.npz")
    shape = (1030, 1030)
    ini = tuple(oracle.hash_uniform_f32(int(s), shape, float(r[0]), float(r[1]))
                for s, r in zip(g["seeds"], g["ranges"]))
    assert [sha(a) for a in ini] == [str(s) for s in g["input_sha256"]]
    out, t, dts = oracle.hydro_run(ini, 1, cyclic=False, gamma=5 / 3, cfl=float(g["cfl"]),
                                   dtype=np.float32)
    assert [sha(a) for a in out] == [str(s) for s in g["sha256"]]


def test_hydro_cyclic_conservation_f64(oracle):
    st = oracle.hydro_init_kh(64, 64, 3)
    t0 = oracle.hydro_totals(st, cyclic=True, gamma=1.4)
    out, t, dts = oracle.hydro_run(st, 20, cyclic=True, gamma=1.4, cfl=0.4)
    t1 = oracle.hydro_totals(out, cyclic=True, gamma=1.4)
    assert abs(t1[0] - t0[0]) < 1e-12 * t0[0]          # mass
    assert abs(t1[1] - t0[1]) < 1e-12 * abs(t0[0])     # x momentum
    assert abs(t1[3] - t0[3]) < 1e-12 * t0[3]          # energy
    assert t > 0 and all(d > 0 for d in dts)


def test_hydro_tangent_linear_matches_fd(oracle):
    # noise on every field breaks the ties of the CFL min (the unperturbed
    # Kelvin-Helmholtz state has thousands of cells with equal timescale,
    # where the min is not differentiable)
    rng = np.random.default_rng(0)
    st = tuple(a * (1 + 1e-3 * rng.standard_normal(a.shape))
               for a in oracle.hydro_init_kh(24, 24, 9))
    d = tuple(rng.standard_normal(a.shape) * s for a, s in zip(st, (0.1, 0.05, 0.05, 0.1)))
    _, dout, _ = oracle.hydro_tl_run(st, d, 3, gamma=1.4, cfl=0.4)
    eps = 1e-7   # small enough that no near-tied cell takes over the CFL min
    plus = tuple(a + eps * b for a, b in zip(st, d))
    minus = tuple(a - eps * b for a, b in zip(st, d))
    op, _, _ = oracle.hydro_run(plus, 3, cyclic=True, gamma=1.4, cfl=0.4)
    om_, _, _ = oracle.hydro_run(minus, 3, cyclic=True, gamma=1.4, cfl=0.4)
    for a, b, c in zip(op, om_, dout):
        fd = (a - b) / (2 * eps)
        assert np.abs(fd - c).max() <= 1e-5 * (np.abs(fd).max() + 1e-12)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref",
                                                    "libref_hydro.so")),
                    reason="reference classes not compiled here")
def test_hydro_oracle_vs_reference_build(oracle):
    st = oracle.hydro_init_jet(1024, 1024, cyclic=False, gamma=5 / 3, dtype=np.float32)
    ref, times = oracle.ref_hydro_run(None, 1, cfl=0.3)
    out, t, _ = oracle.hydro_run(st, 1, cyclic=False, gamma=5 / 3, cfl=0.3, dtype=np.float32)
    for a, b in zip(ref, out):
        assert np.array_equal(a, b)


def test_hydro_flop_count_matches_bench(oracle):
    """The flops per cell-update bench.py reports for the Hydro step are the
    ones the restatement performs (HydroMain.hs:134-276, one flux per wall):
    the same on every size of the periodic Kelvin-Helmholtz start."""
    import bench
    for n in (64, 128):
        ops = oracle.hydro_count_ops(n, n, 1, gamma=1.4, cfl=0.4)
        for k, v in bench.HYDRO_OPS_PER_CELL.items():
            # a handful of per-step scalar operations (dt, time) ride on top
            assert abs(ops[k] - v) * n * n <= 8, (n, k, ops[k], v)
        assert ops["cmp"] > 0
    assert bench.HYDRO_FLOPS_PER_CELL == sum(bench.HYDRO_OPS_PER_CELL.values())


def test_reference_arm_reports_our_config():
    """The reference arm times the same configuration our arm names."""
    import bench
    assert bench.life_config(16384, 100, 1)["workload"].startswith("life 16384x16384 cyclic")
    assert bench.life_config(16384, 100, 1) == bench.life_config(16384, 100, 1)
    assert bench.hydro_config(4096, 1)["n0"] == 4096


def _reference_present():
    from oracle import resize_ref
    return os.path.isdir(os.path.join(resize_ref.reference_tree(),
                                      "examples-old/Life-exampled/dist"))


@pytest.mark.skipif(not _reference_present(), reason="reference tree not present")
def test_resized_reference_classes(oracle):
    """oracle/resize_ref.py: resizing the generated classes to their own size
    and back through another size reproduces them byte for byte, and the
    resized classes compute what the oracle computes at the new size (Life
    96^2 open, 50 generations with populations; Hydro 192^2 float open jet,
    3 steps, gamma 5/3)."""
    import ctypes as C
    from oracle import resize_ref as RR
    for kind, via in (("life", 96), ("life", 16384), ("hydro", 192), ("hydro", 4096)):
        assert RR.check_identity(kind, via), (kind, via)
    L = C.CDLL(RR.build("life", 96))
    L.ref_life_run.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    init = oracle.life_bernoulli(96, 96, 3, 0.3, cyclic=False)
    out = np.zeros((98, 98), np.int32)
    pops = np.zeros(50, np.int32)
    L.ref_life_run(init.ctypes.data, 50, out.ctypes.data, pops.ctypes.data)
    rc, rp = oracle.life_run(init, 50, cyclic=False)
    assert np.array_equal(out, rc) and np.array_equal(pops, rp)
    H = C.CDLL(RR.build("hydro", 192))
    H.ref_hydro_run.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_void_p, C.c_void_p]
    out = np.zeros((4, 198, 198), np.float32)
    H.ref_hydro_run(None, 3, C.c_float(0.5), out.ctypes.data, None)
    st = oracle.hydro_init_jet(192, 192, cyclic=False, gamma=5 / 3, dtype=np.float32)
    ref, _, _ = oracle.hydro_run(st, 3, cyclic=False, gamma=5 / 3, cfl=0.5, dtype=np.float32)
    for a, b in zip(out, ref):
        assert np.array_equal(a, b)
