"""Checkpoint/restart of the statics (om_save / om_load) and the Hydro text
snapshot of examples/Hydro/main-kh.cpp."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_life_checkpoint_restart(om_lib, oracle, tmp_path):
    pg = om_lib
    life = pg.Life((96, 64))
    a = oracle.life_bernoulli(96, 64, 4, 0.35)
    life.write("cell", a)
    life.proceed(5)
    path = tmp_path / "life.omc"
    life.save(path)
    state, gen = life.read("cell"), life.generation
    life.proceed(7)
    life.load(path)                    # back to generation 5
    assert np.array_equal(life.read("cell"), state) and life.generation == gen == 5
    life.proceed(7)
    ref, _ = oracle.life_run(a, 12, cyclic=True)
    assert np.array_equal(life.read("cell"), ref)
    other = pg.Life((64, 96))
    with pytest.raises(pg.OMError):
        other.load(path)               # another mesh
    other.close()
    life.close()


@pytest.mark.parametrize("precision", [64, 32])
def test_hydro_checkpoint_restart_bit_identical(om_lib, tmp_path, precision):
    pg = om_lib
    h = pg.Hydro((128, 96), precision=precision, gamma=1.4)
    h.init_kh(3)
    h.set_scalar("cfl", 0.4)
    h.proceed(4)
    path = tmp_path / "hydro.omc"
    h.save(path)
    h.proceed(6)
    want, t_want = h.state(), h.get_scalar("time")
    g = pg.Hydro((128, 96), precision=precision, gamma=1.4)
    g.load(path)                        # a fresh handle continues identically
    g.proceed(6)
    for a, b in zip(g.state(), want):
        assert np.array_equal(a, b)
    assert g.get_scalar("time") == t_want
    g.close()
    h.close()


def test_hydro_text_snapshot(om_lib, tmp_path):
    pg = om_lib
    h = pg.Hydro((16, 12), precision=64, gamma=1.4)
    h.init_kh(1)
    path = tmp_path / "snapshot0000.txt"
    h.write_snapshot(path)
    rows = path.read_text().split("\n\n")
    lines = [l.split() for r in rows for l in r.split("\n") if l.strip()]
    assert len([r for r in rows if r.strip()]) == 12 and len(lines) == 16 * 12
    v = np.array(lines, float).reshape(12, 16, 6)
    x = (np.arange(16) + 0.5) / 16
    np.testing.assert_allclose(v[0, :, 0], x, rtol=1e-5)
    for k, name in enumerate(("density", "velocity0", "velocity1", "pressure")):
        np.testing.assert_allclose(v[:, :, 2 + k], h.read(name), rtol=1e-5, atol=1e-6)
    h.close()
