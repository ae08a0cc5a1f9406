"""Hydro on the GPU through the C ABI, against the oracle.

FP64 (fused and plain) and the exact FP32 variant reproduce the oracle bit
for bit: their translation unit is built without multiply-add contraction
and follows the generated operation order.  The production FP32 build
(contraction allowed) is held to the benchmark spec's tolerance: relative L1 error
of density <= 1e-5 against FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAMMA = 1.4
CFL = 0.4


def make(pg, size, precision, variant=0, **kw):
    h = pg.Hydro(size, precision=precision, variant=variant, gamma=GAMMA, **kw)
    h.set_scalar("cfl", CFL)
    h.set_scalar("time", 0.0)
    h.set_scalar("extent0", 1.0)
    h.set_scalar("extent1", 1.0)
    dt = np.float64 if precision == 64 else np.float32
    # dR as the OM's Real computes extent / size
    h.set_scalar("dR0", float(dt(1.0) / dt(size[0])))
    h.set_scalar("dR1", float(dt(1.0) / dt(size[1])))
    return h


def kh_state(oracle, size, seed, dtype):
    return oracle.hydro_init_kh(size[0], size[1], seed, dtype=dtype)


def oracle_run(oracle, st, steps, size, dtype):
    d0 = dtype(1.0) / dtype(size[0])
    d1 = dtype(1.0) / dtype(size[1])
    return oracle.hydro_run(st, steps, cyclic=True, gamma=GAMMA, cfl=CFL, dR=(d0, d1),
                            dtype=dtype)


@pytest.mark.parametrize("size", [(64, 48), (37, 29), (8, 8), (96, 130)])
@pytest.mark.parametrize("variant", [0, 1])
def test_fp64_bit_exact(om_lib, oracle, size, variant):
    st = kh_state(oracle, size, 3, np.float64)
    h = make(om_lib, size, 64, variant)
    h.set_state(st)
    h.proceed(6)
    ref, t, dts = oracle_run(oracle, st, 6, size, np.float64)
    for a, b in zip(h.state(), ref):
        assert np.array_equal(a, b)
    assert np.array_equal(h.dt_history(6), np.array(dts))
    assert h.get_scalar("time") == t
    h.close()


@pytest.mark.parametrize("size", [(64, 48), (33, 17), (128, 128)])
@pytest.mark.parametrize("variant", [1, 2])
def test_fp32_exact_variants_bit_exact(om_lib, oracle, size, variant):
    st = kh_state(oracle, size, 4, np.float32)
    h = make(om_lib, size, 32, variant)
    h.set_state(st)
    h.proceed(5)
    ref, t, dts = oracle_run(oracle, st, 5, size, np.float32)
    for a, b in zip(h.state(), ref):
        assert np.array_equal(a, b)
    assert np.array_equal(h.dt_history(5).astype(np.float32), np.array(dts, np.float32))
    h.close()


@pytest.mark.parametrize("tile", [(0, 0), (16, 0), (32, 0), (0, 32), (0, 8), (0, 16), (64, 0),
                                  (64, 8), (0, -8), (0, -16), (64, -8)])
def test_fp32_fast_against_fp64(om_lib, oracle, tile):
    size = (128, 96)
    st64 = kh_state(oracle, size, 5, np.float64)
    h = make(om_lib, size, 32, 0, tile_x=tile[0], tile_y=tile[1])
    h.set_state(tuple(a.astype(np.float32) for a in st64))
    h.proceed(50)
    ref, t, _ = oracle_run(oracle, st64, 50, size, np.float64)
    got = h.state()
    l1 = np.abs(got[0] - ref[0]).mean() / np.abs(ref[0]).mean()
    assert l1 <= 1e-5, l1
    for a, b in zip(got[1:], ref[1:]):
        assert np.abs(a - b).max() < 1e-3
    assert abs(h.get_scalar("time") - t) < 1e-6 * t
    h.close()


def test_random_supersonic_states_fp64(om_lib, oracle):
    size = (48, 40)
    rng = np.random.default_rng(7)
    st = (rng.uniform(0.2, 3.0, size[::-1]), rng.uniform(-4, 4, size[::-1]),
          rng.uniform(-4, 4, size[::-1]), rng.uniform(0.05, 3.0, size[::-1]))
    h = make(om_lib, size, 64, 0)
    h.set_state(st)
    h.proceed(3)
    ref, t, dts = oracle_run(oracle, st, 3, size, np.float64)
    for a, b in zip(h.state(), ref):
        assert np.array_equal(a, b)
    h.close()


def test_totals_and_conservation(om_lib, oracle):
    size = (256, 128)
    st = kh_state(oracle, size, 8, np.float64)
    h = make(om_lib, size, 64, 0)
    h.set_state(st)
    t0 = h.totals()
    np.testing.assert_allclose(t0, oracle.hydro_totals(st, cyclic=True, gamma=GAMMA),
                               rtol=1e-14)
    h.proceed(20)
    t1 = h.totals()
    assert abs(t1[0] - t0[0]) <= 1e-12 * t0[0]
    assert abs(t1[3] - t0[3]) <= 1e-12 * t0[3]
    np.testing.assert_allclose(t1, oracle.hydro_totals(h.state(), cyclic=True, gamma=GAMMA),
                               rtol=1e-14, atol=1e-12)
    h.close()


def test_nonfinite_total_reported(om_lib, oracle):
    size = (32, 32)
    st = list(kh_state(oracle, size, 1, np.float64))
    st[3] = st[3].copy()
    st[3][5, 7] = np.nan
    h = make(om_lib, size, 64, 0)
    h.set_state(st)
    with pytest.raises(om_lib.OMError) as e:
        h.totals()
    assert e.value.status == 5
    h.close()


def test_graph_replay_and_host_writes(om_lib, oracle):
    size = (96, 64)
    st = kh_state(oracle, size, 2, np.float64)
    h = make(om_lib, size, 64, 0)
    h.set_state(st)
    ref = st
    for _ in range(3):                  # captured once, replayed twice
        h.proceed(4)
        ref, _, _ = oracle_run(oracle, ref, 4, size, np.float64)
        assert np.array_equal(h.read("density"), ref[0])
    m = h.array("pressure")             # host write invalidates the cached CFL minimum
    m[10, 10] *= 1.5
    ref = (ref[0], ref[1], ref[2], m.copy())
    h.proceed(2)
    ref, _, _ = oracle_run(oracle, ref, 2, size, np.float64)
    for a, b in zip(h.state(), ref):
        assert np.array_equal(a, b)
    h.close()


@pytest.mark.parametrize("chunks", [(3, 2), (1, 3, 1, 2), (5, 5, 1)])
def test_graph_runs_of_odd_length(om_lib, oracle, chunks):
    # a graph-captured run of odd length leaves the cached CFL minimum in the
    # other slot; the next run must read it from there
    size = (48, 32)
    st = kh_state(oracle, size, 6, np.float64)
    h = make(om_lib, size, 64, 0)
    h.set_state(st)
    for c in chunks:
        h.proceed(c)
    ref, t, _ = oracle_run(oracle, st, sum(chunks), size, np.float64)
    for a, b in zip(h.state(), ref):
        assert np.array_equal(a, b)
    assert h.get_scalar("time") == t
    h.close()


def test_init_kernels(om_lib, oracle):
    size = (64, 32)
    h = make(om_lib, size, 64, 0)
    h.init_kh(12)
    ref = oracle.hydro_init_kh(size[0], size[1], 12, dtype=np.float64)
    got = h.state()
    for a, b in zip(got, ref):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-16)
    assert h.get_scalar("dR0") == 1.0 / 64 and h.get_scalar("time") == 0.0
    h.init()                            # the reference's jet init on a periodic mesh
    ref = oracle.hydro_init_jet(size[0], size[1], cyclic=True, gamma=GAMMA, dtype=np.float64)
    for a, b in zip(h.state(), ref):
        np.testing.assert_allclose(a, b, rtol=1e-15, atol=1e-15)
    h.close()


def test_full_size_fp32_vs_fp64(om_lib):
    # 4096x4096 Kelvin-Helmholtz: FP32 fused against FP64 fused (which is
    # bit-exact with the oracle at the sizes above), 20 steps
    size = (4096, 4096)
    a = make(om_lib, size, 32, 0)
    b = make(om_lib, size, 64, 0)
    a.init_kh(1)
    b.init_kh(1)
    a.set_scalar("cfl", CFL)
    b.set_scalar("cfl", CFL)
    m0 = b.totals()
    a.proceed(20)
    b.proceed(20)
    ra, rb = a.read("density"), b.read("density")
    l1 = np.abs(ra - rb).mean() / np.abs(rb).mean()
    assert l1 <= 1e-5, l1
    ta, tb = a.totals(), b.totals()
    assert abs(tb[0] - m0[0]) <= 1e-12 * m0[0]
    assert abs(ta[0] - m0[0]) <= 1e-6 * m0[0]
    a.close()
    b.close()


@pytest.mark.parametrize("size", [(128, 96), (37, 29), (8, 8), (96, 130), (1024, 300)])
@pytest.mark.parametrize("sweep", [(0, -8), (0, -16), (64, -8)])
def test_sweep_matches_tile_kernel(om_lib, oracle, size, sweep):
    """The column sweep (strips walked in chunks of rows, halo rows kept in
    rings) evaluates every wall and cell with the tile kernel's operations:
    the production FP32 results agree bit for bit, odd and tiny grids
    included, and stay within the FP64 tolerance."""
    st = kh_state(oracle, size, 9, np.float32)
    out = []
    for tx, ty in ((0, 0), sweep):
        h = make(om_lib, size, 32, 0, tile_x=tx, tile_y=ty)
        h.set_state(st)
        h.proceed(7)
        out.append((h.state(), h.dt_history(7), h.get_scalar("time")))
        h.close()
    for a, b in zip(out[0][0], out[1][0]):
        assert np.array_equal(a, b)
    assert np.array_equal(out[0][1], out[1][1]) and out[0][2] == out[1][2]


@pytest.mark.parametrize("size,limit", [((128, 96), 0), ((128, 96), 3), ((64, 64), 0),
                                        ((256, 160), 5), ((96, 320), 2), ((1024, 768), 0),
                                        ((1024, 768), 4), ((512, 512), 2), ((256, 128), 1),
                                        ((100, 96), 0)])
def test_persistent_matches_tile_kernel(om_lib, oracle, size, limit):
    """The persistent 32 x 32 kernel (each CTA walks several tiles; the next
    tile's box is prefetched by TMA inside the grid and by wrapped 16-byte
    copies at its edges; stage-2 walls in runs of three), in its paired form
    (two walls or cells per thread with packed f32x2 instructions; 0, 0: as
    one CTA per SM of two groups running half a tile apart; 16, 0: two CTAs
    per SM) and with one wall per thread (32, 0), forms every value with
    the tile kernel's operations: the production FP32 paths agree bit for
    bit.
    grid_limit forces several tiles per CTA on small grids; 100 x 96 (not a
    multiple of 32) runs the tile kernel under all three.  The two-group
    form runs where each group gets at least 16 tiles: here with grid_limit
    4, 2 and 1 (768, 256 and 32 tiles), else (0, 0) runs the paired form."""
    st = kh_state(oracle, size, 13, np.float32)
    out = []
    for tx, ty in ((0, 0), (16, 0), (32, 0), (0, 32)):
        h = make(om_lib, size, 32, 0, tile_x=tx, tile_y=ty, grid_limit=limit)
        h.set_state(st)
        h.proceed(7)
        out.append((h.state(), h.dt_history(7), h.get_scalar("time")))
        h.close()
    for o in out[1:]:
        for a, b in zip(out[0][0], o[0]):
            assert np.array_equal(a, b)
        assert np.array_equal(out[0][1], o[1]) and out[0][2] == o[2]
