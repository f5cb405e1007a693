"""The C-ABI from plain C: tests/c_abi/abi_check.c is compiled with the
system C compiler as C99 against include/lbm_gb300.h, linked with
liblbm_gb300.so and run (argument checks only; no GPU needed)."""
import os
import shutil
import subprocess

import pytest

from pylabolt_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_c_program_against_header_and_library(lbm_lib, tmp_path):
    lib = capi.lib_path()
    exe = tmp_path / "abi_check"
    cmd = ["gcc", "-std=c99", "-Wall", "-Werror", "-pedantic",
           "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_abi", "abi_check.c"),
           "-L", os.path.dirname(lib), "-l:" + os.path.basename(lib),
           "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stderr
    assert run.stdout.strip() == "ok"
