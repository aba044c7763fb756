"""The JAX-facing shim imports only where jax is installed; without it the
import fails with a clear message instead of a half-working module."""

import importlib

import pytest


def test_shim_needs_jax_or_exposes_pjz_names():
  try:
    import jax  # noqa: F401
  except ImportError:
    with pytest.raises(ImportError, match="needs jax"):
      importlib.import_module("pjz_gb300.jax_shim")
    return
  shim = importlib.import_module("pjz_gb300.jax_shim")
  for name in ("fdtdz", "field", "scatter"):
    assert callable(getattr(shim, name))
