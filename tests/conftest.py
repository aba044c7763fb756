"""Shared pytest configuration: the ``gpu`` marker and import paths."""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
  sys.path.insert(0, ROOT)


def pytest_configure(config):
  config.addinivalue_line(
      "markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the native library")


@pytest.fixture(scope="session")
def native():
  """Builds (if needed) and loads the native library; GPU tests only."""
  import torch
  from pjz_gb300 import _build, _lib
  if not torch.cuda.is_available():
    pytest.fail("gpu test collected without a CUDA device")
  _build.build()
  return _lib.load()
