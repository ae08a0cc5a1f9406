"""Failure handling on the host side (no GPU fault is ever provoked): an
allocation failure injected through OM_FAIL_ALLOC_AFTER surfaces as
OM_ERR_NOMEM from every kind's constructor and leaves the device usable;
non-finite states are reported by the totals; a bounded mbarrier wait that
nothing completes gives up and reports through its error word."""
import numpy as np
import pytest

from paraiso_gb300 import omgraph_examples as ex

pytestmark = pytest.mark.gpu

NOMEM = 4


MAKERS = {
    "hydro": lambda pg: pg.Hydro((64, 48), precision=64),       # 4 arrays
    "graph": lambda pg: pg.GraphMachine(ex.life((64, 48))),     # 1 array
}


@pytest.mark.parametrize("kind,after,fails", [
    ("hydro", 0, True), ("hydro", 3, True), ("hydro", 4, False),
    ("graph", 0, True), ("graph", 1, False)])
def test_injected_allocation_failure(om_lib, monkeypatch, kind, after, fails):
    pg = om_lib
    monkeypatch.setenv("OM_FAIL_ALLOC_AFTER", str(after))
    if fails:
        with pytest.raises(pg.OMError) as e:
            MAKERS[kind](pg)
        assert e.value.status == NOMEM and "OM_FAIL_ALLOC_AFTER" in str(e.value)
    else:
        MAKERS[kind](pg).close()
    monkeypatch.delenv("OM_FAIL_ALLOC_AFTER")
    life = pg.Life((64, 48))                  # the device is still usable
    life.fill_random(1, 0.3)
    life.proceed(3)
    assert life.generation == 3
    life.close()


def test_nonfinite_state_is_reported(om_lib):
    pg = om_lib
    h = pg.Hydro((32, 32), precision=64, gamma=1.4)
    h.init_kh(1)
    rho = h.read("density")
    rho[5, 7] = np.nan
    h.write("density", rho)
    with pytest.raises(pg.OMError) as e:
        h.totals()
    assert "non-finite" in str(e.value)
    h.close()


def test_bounded_wait_reports_its_time_out(om_lib):
    # an mbarrier armed for bytes that no copy delivers (no copy is issued):
    # the wait the TMA kernels use gives up after its bound and raises the
    # error word; the device stays usable
    lib = om_lib.load_library()
    assert lib.om_selftest_wait_bound(0) == 0, lib.om_last_error()
    life = om_lib.Life((64, 64))
    life.fill_random(2, 0.3)
    life.proceed(3)
    assert life.generation == 3
    life.close()
