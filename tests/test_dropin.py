"""C++ host code over include/gbfem.hpp: a GPU run of a C++ driver, and a
compile check that dune-fem's own Krylov templates accept the GPU types."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
LIBDIR = os.path.join(ROOT, "dune-fem_gb300", "lib")


def _reference_src():
    r = subprocess.run(["sh", os.path.join(ROOT, "oracle", "ref_src.sh")], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else None


def _compile(src, out, extra=()):
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), *extra, src, "-o", out,
           "-L", LIBDIR, "-lgbfem", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_reference_krylov_templates_compile_against_gpu_types(gb, tmp_path):
    REF = _reference_src()
    if REF is None:
        pytest.skip("dune-fem sources not present")
    src = os.path.join(CPP, "ref_templates_check.cpp")
    obj = str(tmp_path / "ref_templates_check.o")
    cmd = ["g++", "-std=c++17", "-c", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle", "shim"),
           "-I", REF, src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_cpp_driver_solves_on_gpu(gb, tmp_path):
    exe = _compile(os.path.join(CPP, "dropin_main.cpp"), str(tmp_path / "dropin"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
