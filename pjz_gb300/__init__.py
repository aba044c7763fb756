"""GB300-native (sm_103a) FDTD engine behind pjz's simulation entry points.

Public API (mirrors pjz's ``src/pjz/_field.py``):
  * :class:`SimParams`, :func:`field` -- time-harmonic fields;
  * :func:`scatter` -- scattering values between port modes;
  * :func:`fdtdz` -- drop-in for the ``fdtdz_jax.fdtdz`` engine call;
  * :func:`epsilon` -- pjz's Yee-cell permittivity rendering
    (``src/pjz/_epsilon.py``) on the GPU;
  * :func:`field_voxel_jvp` -- forward-mode derivatives of ``field`` with
    respect to single permittivity voxels (tangent-linear solves);
  * :class:`engine.Plan` -- the plan/run API over the C ABI.
"""

from ._field import SimParams, field
from ._fdtdz import LaunchParams, fdtdz
from ._scatter import scatter
from ._epsilon import epsilon
from ._tangent import field_voxel_jvp
from . import engine

__all__ = ["SimParams", "field", "scatter", "fdtdz", "LaunchParams", "epsilon",
           "field_voxel_jvp", "engine"]
