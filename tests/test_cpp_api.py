"""The drop-in C++ headers compile against the C ABI library; the test
program checks argument errors everywhere and bit-exact results on a GPU."""
import os
import shutil
import subprocess

import pytest

from paliwa_gb300 import _lib, build as pgbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_api_test(name="api_test", extra=()):
    pgbuild.build()
    out = os.path.join(pgbuild.BUILD, name)
    cuda = os.path.dirname(os.path.dirname(pgbuild.nvcc()))
    cmd = ["g++", "-std=c++20", "-O1", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "oracle"),
           "-I" + os.path.join(cuda, "include")] + list(extra) + [
           os.path.join(ROOT, "tests", "cpp", name + ".cpp"),
           "-o", out, "-L" + pgbuild.BUILD, "-lpaliwa_gb300",
           "-L" + os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + pgbuild.BUILD,
           "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_cpp_api_compiles_and_checks_errors():
    exe = build_api_test()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_cpp_api_on_gpu():
    exe = build_api_test()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "match the oracle" in r.stdout


DISTRIBUTED = ("-DPALIWA_WITH_MPI",
               "-I" + os.path.join(ROOT, "tests", "cpp", "fake_mpi"))


def test_distributed_dropin_compiles_and_checks_ranks():
    exe = build_api_test("distributed_test", DISTRIBUTED)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_distributed_dropin_on_gpu():
    exe = build_api_test("distributed_test", DISTRIBUTED)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "matches the oracle" in r.stdout
