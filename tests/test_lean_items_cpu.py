"""The lean kernels' item mapping (``lean_item``, ``lean_warps`` in
``csrc/lean_kernel.cuh``) compiled for the host and compared entry by entry
with the copy the shared-memory replay model uses (``lean_items`` in
``tests/test_smem_model_cpu.py``): the model checks the kernel's mapping,
not a restatement that could drift from it."""

import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from test_smem_model_cpu import lean_geom, lean_items

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
  nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
  if not os.path.exists(nvcc):
    pytest.skip("no nvcc")
  so = str(tmp_path_factory.mktemp("lean") / "liblean_items.so")
  subprocess.run([nvcc, "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
                  "-gencode", "arch=compute_103a,code=sm_103a",
                  "-I", os.path.join(ROOT, "pjz_gb300", "csrc"),
                  "-I", os.path.join(ROOT, "include"),
                  os.path.join(ROOT, "tests", "lean_items_host.cu"), "-o", so],
                 check=True)
  h = ctypes.CDLL(so)
  I, P = ctypes.c_int, ctypes.c_void_p
  h.lean_items_host.argtypes = [I, I, I, I, I, P, P, P, P, I]
  h.lean_items_host.restype = I
  h.lean_geom_host.argtypes = [I, I, I, I, P]
  h.lean_geom_host.restype = None
  return h


@pytest.mark.parametrize("esz", [4, 2])
@pytest.mark.parametrize("Z,TY", [(64, 14), (64, 28), (48, 19), (32, 29), (32, 28),
                                  (16, 5), (24, 3)])
@pytest.mark.parametrize("plo,phi", [(0, 0), (8, 8), (4, 12), (12, 4), (16, 16),
                                     (4, 24)])
def test_model_items_are_the_kernel_items(lib, esz, Z, TY, plo, phi):
  if plo + phi > Z:
    pytest.skip("slabs wider than the domain")
  for rows in (TY + 1, TY + 3):  # one-step H rows, two-step level-1 rows
    cap = 4096
    buf = [np.zeros(cap, np.int32) for _ in range(4)]
    n = lib.lean_items_host(Z, rows, plo, phi, esz, *(b.ctypes.data for b in buf),
                            cap)
    assert n > 0
    thr, rH, z0, col, pml, m = lean_items(Z, rows - 1, plo, phi, esz)
    assert m == n
    order = np.argsort(thr)
    np.testing.assert_array_equal(buf[0][:n], rH[order])
    np.testing.assert_array_equal(buf[1][:n], z0[order])
    np.testing.assert_array_equal(buf[2][:n], col[order])
    np.testing.assert_array_equal(buf[3][:n].astype(bool), pml[order])


@pytest.mark.parametrize("esz", [4, 2])
@pytest.mark.parametrize("Z,TY", [(64, 14), (64, 28), (48, 19), (32, 29), (32, 28)])
@pytest.mark.parametrize("P", [0, 8, 12, 16, 24])
def test_model_geometry_is_the_kernel_geometry(lib, esz, Z, TY, P):
  """The byte layout the alignment tests check (``lean_geom``) is the
  kernels' ``LeanGeom``."""
  out = np.zeros(10, np.int64)
  lib.lean_geom_host(TY, Z, P, esz, out.ctypes.data)
  g = lean_geom(TY, Z, P, esz)
  want = [g["e"], g["h"], g["c"], g["m"], g["p"], g["stage"], g["hn"], g["en"],
          g["pn"], g["Pp"]]
  assert out.tolist() == want
