"""The C-ABI library loads without a GPU and exports every symbol that
include/fem_gpu.h declares (no compute calls here)."""
import os
import re

import moris_gb300 as mg
from moris_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fem_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(fem_(?:gpu|hmr|cnn|lpc|xtk|gen|mg|vis)_\w+)\s*\(", src)
    return sorted(set(names))


def test_every_declared_symbol_is_exported():
    lib = mg.lib()
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header():
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_library_answers_without_gpu():
    lib = mg.lib()
    assert lib.fem_gpu_abi_version() == 3
    assert lib.fem_gpu_status_string(0) == b"ok"
    assert lib.fem_gpu_device_count() >= 0


def test_cpp_layer_compiles():
    """include/fem_gpu_solver_interface.hpp compiles as C++17 against the C ABI."""
    import shutil
    import subprocess
    import tempfile
    if not shutil.which("g++"):
        import pytest
        pytest.skip("no g++")
    src = '#include "fem_gpu_solver_interface.hpp"\nint main() { return sizeof(moris_gb300::Gpu_Solver_Interface) > 0 ? 0 : 1; }\n'
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "t.cpp")
        open(f, "w").write(src)
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), f],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_moris_adapter_links_against_the_library():
    """The integration program (tests/cpp/solver_interface_main.cpp: a
    Solver_Interface subclass over include/fem_gpu_moris_adapter.hpp, with the
    reference's signatures for Matrix, Dist_Matrix and Dist_Vector) compiles
    and links against libfem_gpu.so."""
    import shutil
    import subprocess
    import tempfile
    import pytest
    if not shutil.which("g++"):
        pytest.skip("no g++")
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
                            "-I", os.path.join(ROOT, "tests", "cpp"),
                            os.path.join(ROOT, "tests", "cpp", "solver_interface_main.cpp"),
                            "-L", os.path.join(ROOT, "moris_gb300", "_build"), "-lfem_gpu",
                            "-o", os.path.join(d, "si")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
