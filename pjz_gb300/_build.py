"""Builds the in-tree native library ``libpjzfdtd.so`` for sm_103a with nvcc.

The library is a plain C ABI (``include/pjzfdtd.h``) loaded with ctypes, so
no torch extension machinery is involved.  Output stays in the package
directory (git-ignored) so the process that loads it is visible.
"""

import os
import shutil
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_PATH = os.path.join(HERE, "libpjzfdtd.so")

COMPILE_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo", "-O3", "-std=c++17",
    # Every FMA in the kernels is explicit; no contraction of a*b+c.
    "-fmad=false",
    "-Xcompiler", "-fPIC",
]
# One-command form (all sources into a shared library).
NVCC_FLAGS = COMPILE_FLAGS + ["-shared"]


def sources():
  return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                if f.endswith(".cu"))


def _stale():
  if not os.path.exists(LIB_PATH):
    return True
  t = os.path.getmtime(LIB_PATH)
  deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
  deps.append(os.path.join(ROOT, "include", "pjzfdtd.h"))
  return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
  """Compiles ``csrc/*.cu`` into ``libpjzfdtd.so`` (skipped when fresh)."""
  if not force and not _stale():
    return LIB_PATH
  nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
  tmp = LIB_PATH + f".{os.getpid()}.tmp"
  objdir = tempfile.mkdtemp(prefix="pjzfdtd_build_")
  try:
    # The kernel translation units are independent: compile them in
    # parallel, then link once.
    jobs = []
    for src in sources():
      obj = os.path.join(objdir, os.path.basename(src) + ".o")
      cmd = [nvcc, *COMPILE_FLAGS, "-I", os.path.join(ROOT, "include"), "-c",
             src, "-o", obj]
      if verbose:
        print(" ".join(cmd))
      jobs.append((obj, subprocess.Popen(cmd)))
    failed = [obj for obj, proc in jobs if proc.wait() != 0]
    if failed:
      raise RuntimeError(f"nvcc failed for {failed}")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared",
           *(obj for obj, _ in jobs), "-o", tmp]
    if verbose:
      print(" ".join(cmd))
    subprocess.run(cmd, check=True)
  finally:
    shutil.rmtree(objdir, ignore_errors=True)
  os.replace(tmp, LIB_PATH)
  return LIB_PATH
