"""The drop-in seen from C: a C99 program that uses include/sgemm_cuda.h the
way the reference's sgemm_test.c uses its OpenCL backend header compiles
with -std=c99 -Wall -Werror, links against libugemm_cuda.so and runs (the
host-only calls here; with a GPU, the known-answer GEMM in an arena sized by
the reference's own rule, 840 bytes for the 3 x 3 x 2 product, and a ragged
product through each of sgemm_test.c's three transpose macros)."""
import os
import shutil
import subprocess

import pytest

import ugemm_gb300 as ug

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_dropin(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    if not os.path.exists(ug.LIB_PATH):
        ug.build()
    exe = str(tmp_path / "dropin")
    libdir = os.path.dirname(ug.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "dropin.c"), "-o", exe, "-L", libdir,
                    "-lugemm_cuda", f"-Wl,-rpath,{libdir}", "-lm"], check=True)
    return exe


def test_c_caller_compiles_links_and_runs_host_calls(tmp_path):
    exe = build_dropin(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, (out.returncode, out.stderr)
    assert "dropin ok" in out.stdout


@pytest.mark.gpu
def test_c_caller_known_answer_on_gpu(tmp_path):
    exe = build_dropin(tmp_path)
    out = subprocess.run([exe, "run"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, (out.returncode, out.stderr)
