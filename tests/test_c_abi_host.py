"""The C ABI used from C on the host (no GPU): ``tests/c_abi_host.c`` is
compiled with gcc against ``include/pjzfdtd.h``, linked with the library and
run; it creates plans, sizes a workspace, reads the launch geometry, sets
monitor boxes, creates a batch of plans of different domains and checks the
error codes of bad requests (including the run-argument checks of a batch,
which come before any device work)."""

import os
import shutil
import subprocess

import pytest

from pjz_gb300 import _build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_program_uses_the_abi(tmp_path):
  cc = shutil.which("gcc") or shutil.which("cc")
  if cc is None:
    pytest.skip("no C compiler")
  lib = _build.build()
  cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
  exe = tmp_path / "c_abi_host"
  subprocess.run([cc, "-std=c11", "-O1", "-Wall", "-Werror",
                  "-I", os.path.join(ROOT, "include"),
                  os.path.join(ROOT, "tests", "c_abi_host.c"),
                  "-o", str(exe), lib,
                  "-Wl,-rpath," + os.path.dirname(lib),
                  "-L", os.path.join(cuda, "lib64"), "-lcudart"],
                 check=True)
  env = dict(os.environ, LD_LIBRARY_PATH=os.pathsep.join(
      [os.path.dirname(lib), os.path.join(cuda, "lib64"),
       os.environ.get("LD_LIBRARY_PATH", "")]))
  out = subprocess.run([str(exe)], capture_output=True, text=True, env=env)
  print(out.stdout)
  assert out.returncode == 0, out.stdout + out.stderr
  for line in ("ok monitors", "ok batch", "ok bad region"):
    assert line in out.stdout
