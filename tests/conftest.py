import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def om_lib():
    from paraiso_gb300 import build
    build.build()
    import paraiso_gb300
    return paraiso_gb300


# Figures that the parity tests at the benchmark configurations' own sizes
# measure (errors against FP64, agreement of gradients); printed at the end
# of the run so that a quiet run still shows them.
_FIGURES: list[tuple[str, dict]] = []


@pytest.fixture
def figures():
    def add(name: str, **values):
        _FIGURES.append((name, values))
    return add


def pytest_terminal_summary(terminalreporter):
    if not _FIGURES:
        return
    terminalreporter.section("figures at the benchmark configurations")
    for name, values in _FIGURES:
        parts = []
        for k, v in values.items():
            parts.append(f"{k}={v:.3g}" if isinstance(v, float) else f"{k}={v}")
        terminalreporter.write_line(f"{name}: " + ", ".join(parts))
