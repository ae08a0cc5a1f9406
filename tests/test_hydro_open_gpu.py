"""Hydro on an open grid (3-cell margins, the jet boundary condition of
examples/Hydro/HydroMain.hs:105-131) on the GPU.  The exact FP32 build is
checked bit for bit against outputs of the reference's own generated float
code (examples-old/Hydro-exampled/dist/Hydro.cpp, golden SHA-256 of every
memory array), FP64 against the oracle."""
import hashlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GAMMA = 5.0 / 3.0


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_open(pg, n0, n1, precision, variant, cfl):
    h = pg.Hydro((n0, n1), precision=precision, variant=variant, gamma=GAMMA,
                 boundary=pg.OPEN)
    h.set_scalar("time", 0.0)
    h.set_scalar("cfl", cfl)
    h.set_scalar("extent0", 1.0)
    h.set_scalar("extent1", 1.0)
    h.set_scalar("dR0", float(np.float32(1.0) / np.float32(n0)) if precision == 32 else 1.0 / n0)
    h.set_scalar("dR1", float(np.float32(1.0) / np.float32(n1)) if precision == 32 else 1.0 / n1)
    return h


def test_open_margins_and_sizes(om_lib):
    h = make_open(om_lib, 64, 48, 32, 2, 0.5)
    assert h.memory_shape == (54, 70)
    assert h.om_lower_margin(0) == 3 and h.om_upper_margin(1) == 3
    h.close()


@pytest.mark.parametrize("steps_per_call", [2, 1])
def test_open_jet_matches_reference_golden(om_lib, oracle, steps_per_call):
    # 1024^2 float, gamma 5/3, the generated init, 2 steps at cfl 0.5: every
    # memory array (margins included) bit-identical to the generated code's
    g = np.load(os.path.join(GOLDEN, "hydro_ref_jet.npz"))
    st = oracle.hydro_init_jet(1024, 1024, cyclic=False, gamma=GAMMA, dtype=np.float32)
    h = make_open(om_lib, 1024, 1024, 32, 2, float(g["cfl"]))
    h.set_state(st)
    for _ in range(2 // steps_per_call):
        h.proceed(steps_per_call)
    assert [sha(a) for a in h.state()] == [str(s) for s in g["sha256"]]
    assert abs(h.get_scalar("time") - float(g["times"][-1])) <= 2e-7 * float(g["times"][-1])
    h.close()


def test_open_random_matches_reference_golden(om_lib, oracle):
    # hashed random supersonic states on the whole memory array, one step
    g = np.load(os.path.join(GOLDEN, "hydro_ref_random.npz"))
    shape = (1030, 1030)
    ini = tuple(oracle.hash_uniform_f32(int(s), shape, float(r[0]), float(r[1]))
                for s, r in zip(g["seeds"], g["ranges"]))
    assert [sha(a) for a in ini] == [str(s) for s in g["input_sha256"]]
    h = make_open(om_lib, 1024, 1024, 32, 2, float(g["cfl"]))
    h.set_state(ini)
    h.proceed(1)
    assert [sha(a) for a in h.state()] == [str(s) for s in g["sha256"]]
    h.close()


@pytest.mark.parametrize("size", [(96, 80), (45, 37)])
def test_open_fp64_matches_oracle(om_lib, oracle, size):
    n0, n1 = size
    st = oracle.hydro_init_jet(n0, n1, cyclic=False, gamma=GAMMA, dtype=np.float64)
    h = make_open(om_lib, n0, n1, 64, 0, 0.4)
    h.set_state(st)
    h.proceed(7)
    ref, t, dts = oracle.hydro_run(st, 7, cyclic=False, gamma=GAMMA, cfl=0.4,
                                   dtype=np.float64)
    for a, b in zip(h.state(), ref):
        assert np.array_equal(a, b)
    assert np.array_equal(h.dt_history(7), np.array(dts))
    # conserved totals over the interior
    got, want = h.totals(), oracle.hydro_totals(ref, cyclic=False, gamma=GAMMA)
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13 * abs(want[0]))
    h.close()


def test_open_fast_fp32_close_to_oracle(om_lib, oracle):
    n0, n1 = 256, 192
    st = oracle.hydro_init_jet(n0, n1, cyclic=False, gamma=GAMMA, dtype=np.float32)
    h = make_open(om_lib, n0, n1, 32, 0, 0.5)
    h.set_state(st)
    h.proceed(20)
    ref, _, _ = oracle.hydro_run(st, 20, cyclic=False, gamma=GAMMA, cfl=0.5, dtype=np.float32)
    for a, b in zip(h.state(), ref):
        assert np.abs(a.astype(np.float64) - b).sum() <= 1e-5 * np.abs(b).sum() + 1e-12
    h.close()


def test_open_init_kernel(om_lib, oracle):
    # the generated init on the GPU (the jet in the left margin)
    n0, n1 = 128, 96
    h = make_open(om_lib, n0, n1, 64, 0, 0.4)
    h.init()
    ref = oracle.hydro_init_jet(n0, n1, cyclic=False, gamma=GAMMA, dtype=np.float64)
    for a, b in zip(h.state(), ref):
        np.testing.assert_allclose(a, b, rtol=1e-15, atol=0)
    h.close()


def test_open_unsupported_paths(om_lib):
    pg = om_lib
    with pytest.raises(pg.OMError):
        pg.Hydro((64, 64), precision=64, variant=1, gamma=GAMMA, boundary=pg.OPEN)
    h = make_open(pg, 64, 64, 64, 0, 0.4)
    with pytest.raises(pg.OMError):
        h.init_kh(1)
    h.init()
    with pytest.raises(pg.OMError):
        h.forward(2)
    h.close()
