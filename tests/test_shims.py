"""The header-only shims rebuild the generated class over the C ABI: the
reference's own drivers compile against them unchanged, and a driver written
in the same style runs on the GPU with the oracle's results."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "paraiso_gb300")
# the reference tree the oracle recipe reads (PARAISO_REFERENCE, else its default)
REFERENCE_TREE = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref-path"],
                                capture_output=True, text=True).stdout.strip()


def compile_cpp(src, out, tmp_path):
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", src, f"-I{INC}", f"-L{LIBDIR}", "-lom_gb300",
           f"-Wl,-rpath,{LIBDIR}", "-o", str(tmp_path / out)]
    subprocess.run(cmd, check=True)
    return str(tmp_path / out)


@pytest.mark.skipif(not os.path.isdir(REFERENCE_TREE), reason="reference tree not present")
@pytest.mark.parametrize("driver", ["examples/Life/main.cpp", "examples/Hydro/main-kh.cpp"])
def test_reference_drivers_compile_unchanged(om_lib, tmp_path, driver):
    compile_cpp(os.path.join(REFERENCE_TREE, driver), "drv", tmp_path)


def test_shim_driver_compiles(om_lib, tmp_path):
    compile_cpp(os.path.join(ROOT, "tests", "cpp", "shim_driver.cpp"), "shim_driver", tmp_path)


@pytest.mark.gpu
def test_shim_driver_life_matches_oracle(om_lib, oracle, tmp_path):
    exe = compile_cpp(os.path.join(ROOT, "tests", "cpp", "shim_driver.cpp"), "shim_driver",
                      tmp_path)
    out = subprocess.run([exe, "life", "80", "48", "30"], check=True, capture_output=True,
                         text=True).stdout.split("\n")
    a = np.zeros((48, 80), np.int32)
    for x, y in ((1, 0), (2, 1), (0, 2), (1, 2), (2, 2)):
        a[y + 3, x + 3] = 1
    a[24, 40:43] = 1
    ref, pops = oracle.life_run(a, 30, cyclic=True)
    got = [tuple(map(int, l.split())) for l in out[:30]]
    assert got == [(t + 1, int(p)) for t, p in enumerate(pops)]
    assert out[30] == f"alive {ref.sum()}"


@pytest.mark.gpu
def test_shim_driver_hydro_conserves_mass(om_lib, tmp_path):
    exe = compile_cpp(os.path.join(ROOT, "tests", "cpp", "shim_driver.cpp"), "shim_driver",
                      tmp_path)
    out = subprocess.run([exe, "hydro", "64", "10"], check=True, capture_output=True,
                         text=True).stdout.split("\n")
    vals = dict(l.split() for l in out if l)
    assert float(vals["time"]) > 0
    assert abs(float(vals["mass"]) - float(vals["mass0"])) < 1e-11 * float(vals["mass0"])


@pytest.mark.gpu
def test_shim_driver_hydro_open_default(om_lib, oracle, tmp_path):
    # Hydro(n, n) is the generated class: open boundary, jet inflow, gamma 5/3
    exe = compile_cpp(os.path.join(ROOT, "tests", "cpp", "shim_driver.cpp"), "shim_driver",
                      tmp_path)
    out = subprocess.run([exe, "hydro_open", "64", "6"], check=True, capture_output=True,
                         text=True).stdout.split("\n")
    vals = dict(l.split() for l in out if l)
    assert int(vals["margin"]) == 3
    st = oracle.hydro_init_jet(64, 64, cyclic=False, gamma=5 / 3, dtype=np.float64)
    ref, t, _ = oracle.hydro_run(st, 6, cyclic=False, gamma=5 / 3, cfl=0.5, dtype=np.float64)
    rho, vx = ref[0][3:-3, 3:-3], ref[1][3:-3, 3:-3]
    assert abs(float(vals["time"]) - t) <= 1e-12 * t
    assert abs(float(vals["mass"]) - rho.sum()) <= 1e-12 * rho.sum()
    assert abs(float(vals["px"]) - (rho * vx).sum()) <= 1e-9 * abs(rho * vx).sum()


def emit(tmp_path, om, sub=""):
    from paraiso_gb300 import omgraph as og
    d = tmp_path / sub if sub else tmp_path
    d.mkdir(parents=True, exist_ok=True)
    (d / f"{om.name}.hpp").write_text(og.emit_header(om))


@pytest.mark.skipif(not os.path.isdir(REFERENCE_TREE), reason="reference tree not present")
@pytest.mark.parametrize("driver,make,sub", [
    ("examples/ShiftExample/main.cpp", "shift_example", ""),
    ("examples/HelloWorld/main.cpp", "hello_world", "dist"),
    ("examples/InitialCondition/main.cpp", "initial_condition", "dist")])
def test_reference_graph_drivers_compile_unchanged(om_lib, tmp_path, driver, make, sub):
    # the emitted class stands in for dist/TableMaker.hpp of the generator
    from paraiso_gb300 import omgraph_examples as ex
    emit(tmp_path, getattr(ex, make)(), sub)
    cmd = ["g++", "-std=c++17", "-O1", os.path.join(REFERENCE_TREE, driver), f"-I{INC}",
           f"-I{tmp_path}", f"-L{LIBDIR}", "-lom_gb300", f"-Wl,-rpath,{LIBDIR}",
           "-o", str(tmp_path / "drv")]
    subprocess.run(cmd, check=True)


@pytest.mark.skipif(not os.path.isdir(REFERENCE_TREE), reason="reference tree not present")
def test_reference_hello_gpu_driver_compiles_unchanged(om_lib, tmp_path):
    # examples/HelloGPU: the HelloWorld machine generated for CUDA, whose
    # driver is a .cu file built by nvcc
    import shutil
    from paraiso_gb300 import omgraph_examples as ex
    emit(tmp_path, ex.hello_world(), "dist")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    subprocess.run([nvcc, "-std=c++17", os.path.join(REFERENCE_TREE, "examples/HelloGPU/main.cu"),
                    f"-I{INC}", f"-I{tmp_path}", f"-L{LIBDIR}", "-lom_gb300",
                    "-Xlinker", f"-rpath={LIBDIR}", "-o", str(tmp_path / "drv")], check=True)


@pytest.mark.gpu
@pytest.mark.parametrize("boundary", ["open", "cyclic"])
def test_graph_driver_runs_shift_example(om_lib, tmp_path, boundary):
    from oracle import omgraph_ref as R
    from paraiso_gb300 import omgraph_examples as ex
    om = ex.shift_example(boundary)
    emit(tmp_path, om)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", os.path.join(ROOT, "tests", "cpp",
           "graph_driver.cpp"), f"-I{INC}", f"-I{tmp_path}", f"-L{LIBDIR}", "-lom_gb300",
           f"-Wl,-rpath,{LIBDIR}", "-o", str(tmp_path / "gd")]
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(tmp_path / "gd")], check=True, capture_output=True,
                         text=True).stdout.strip().split("\n")
    m = R.Machine(om.to_text())
    want = []
    for k in ("init", "increment", "calculate"):
        m.run(k)
        want.append("value: " + " ".join(str(v) for v in m.values["table"].ravel()))
    want.append(f"total: {int(m.values['total'])}")
    assert out == want


@pytest.mark.skipif(not os.path.isdir(REFERENCE_TREE), reason="reference tree not present")
@pytest.mark.parametrize("driver", ["examples/Life/main.cu", "examples/Hydro/main-kh.cu"])
def test_reference_earlier_api_drivers_compile_unchanged(om_lib, tmp_path, driver):
    # the drivers written against the earlier generator's class (public
    # static_<i>_<name> members, memorySize0(), ...; thrust on the host)
    import shutil
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    subprocess.run([nvcc, "-std=c++17", os.path.join(REFERENCE_TREE, driver), f"-I{INC}",
                    f"-L{LIBDIR}", "-lom_gb300", "-Xlinker", f"-rpath={LIBDIR}",
                    "-o", str(tmp_path / "drv")], check=True)


@pytest.mark.gpu
def test_earlier_api_driver_runs(om_lib, tmp_path):
    exe = compile_cpp(os.path.join(ROOT, "tests", "cpp", "old_api_driver.cpp"), "old_api",
                      tmp_path)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    assert out.strip().endswith("ok"), out
