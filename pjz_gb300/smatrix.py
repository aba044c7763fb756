"""Multi-port S-matrix and its epsilon-gradient in one batched launch.

pjz's ``scatter`` (``src/pjz/_field.py:346-442``) runs one ``field`` solve
per port in a Python loop and differentiates with reciprocity residuals
``f_i f_j / a_i`` kept for every port pair.  Here, for an objective
``L = sum_w sum_ij m_ij |S_ij|^2`` with ``S_ij = <p_j, E_t(F_i)>`` on port
j's monitor plane:

* port i's forward solve records its phasors ``F_i`` on the design box and
  on every port's monitor plane (monitor boxes, no full-field output);
* port j's *unit adjoint* solve is driven by ``i e^{3iw dt/2} p_j / w~`` on
  monitor plane j (divided by the CPML stretch where the window reaches
  into the z-PML) and records ``G_j`` on the design box.  Because the adjoint
  of forward i is ``sum_j conj(2 m_ij S_ij) x`` (unit adjoint j) by
  linearity, the adjoints do not depend on the forwards, so all 2n solves run
  in one batched, graph-captured launch;
* ``dL/d eps = sum_w Re(w~^2 e^{-2iw dt} sum_ij F_i conj(2 m_ij S_ij) G_j)``
  over the design box (the derivation is that of ``_adjoint``).

Across several GPUs (one rank each) the 2n independent solves are shared
round-robin; each rank runs its share, then one all-gather hands every rank
the recorded boxes of every solve (the design box and the monitor planes, a
few MB), and every rank assembles the same S, objective and gradient.
"""

import ctypes
from typing import List, NamedTuple, Tuple

import numpy as np
import torch

from . import _adjoint, _field, _lib, engine, replicas
from .workloads import (ABSORBER_COEFF, EPS_SI, EPS_SIO2, _blur,
                        _slab_fraction, omega_of)


class Port(NamedTuple):
  axis: int          # 0: x-normal, 1: y-normal
  center: int        # transverse centre (y for x-normal ports, x otherwise)
  source: int        # source plane index along `axis`
  monitor: int       # monitor plane index along `axis`


class SMatrixProblem(NamedTuple):
  eps: np.ndarray             # (3, X, Y, Z) float32, the whole domain
  mask: np.ndarray            # (3, X, Y) absorber
  pml_sigma: np.ndarray       # (Z, 2)
  ports: List[Port]
  omega: np.ndarray
  tt: int
  design_box: Tuple[Tuple[int, int, int], Tuple[int, int, int]]
  target: np.ndarray          # (n, n) 0/1 objective mask
  window: int                 # half-width of the port windows (cells)
  zc: float                   # slab centre (z)
  ramp: Tuple[float, float]   # pjz ramp (width, delay)
  pml: int                    # z-PML slab width (each side)


def build_c4(domain=(1024, 1024, 64), tt: int = 12000, seed: int = 3,
             device_cells: int = 100, pml: int = 8, absorber: int = 16,
             wavelengths=(1.53, 1.55, 1.57), edge: int = 40,
             monitor_inset: int = 20, window: int = 30,
             ramp_steps: int = 500) -> SMatrixProblem:
  """Config c4: 8-port 4x4 um random device (two waveguide ports per side,
  400 nm x 220 nm Si in SiO2), blurred seeded epsilon in [2.085, 12.25],
  seeded target mask over the port pairs.  The sources ramp like pjz's
  ramped sine over ``ramp_steps`` (full amplitude after ~6 ramps)."""
  X, Y, Z = domain
  rng = np.random.default_rng(seed)
  zc = Z / 2
  half = device_cells // 2
  cx, cy = X // 2, Y // 2
  offs = (-device_cells // 4, device_cells // 4)
  eps = np.empty((3, X, Y, Z), np.float64)
  for c in range(3):
    ox = 0.5 if c == 0 else 0.0
    oy = 0.5 if c == 1 else 0.0
    oz = 0.5 if c == 2 else 0.0
    fz = _slab_fraction(Z, zc - 2.75, zc + 2.75, oz)
    fill = np.zeros((X, Y))
    for d in offs:
      fy = _slab_fraction(Y, cy + d - 5, cy + d + 5, oy)
      fx = _slab_fraction(X, cx + d - 5, cx + d + 5, ox)
      fill = np.maximum(fill, np.ones(X)[:, None] * fy[None, :])   # x guides
      fill = np.maximum(fill, fx[:, None] * np.ones(Y)[None, :])   # y guides
    eps[c] = EPS_SIO2 + (EPS_SI - EPS_SIO2) * fill[:, :, None] * fz[None, None, :]
  vox = np.clip(_blur(rng.uniform(EPS_SIO2, EPS_SI, (device_cells, device_cells)),
                      2.0), EPS_SIO2, EPS_SI)
  z0, z1 = int(round(zc - 3)), int(round(zc + 3))
  eps[:, cx - half:cx + half, cy - half:cy + half, z0:z1] = vox[None, :, :, None]
  mask = _field._absorption_mask(X, Y, absorber, ABSORBER_COEFF).astype(np.float32)
  sig = _field._pml_sigma((pml, pml), Z, 0.5, 1.3).astype(np.float32)
  ports = []
  for d in offs:
    ports.append(Port(0, cy + d, edge, edge + monitor_inset))
    ports.append(Port(0, cy + d, X - 1 - edge, X - 1 - edge - monitor_inset))
  for d in offs:
    ports.append(Port(1, cx + d, edge, edge + monitor_inset))
    ports.append(Port(1, cx + d, Y - 1 - edge, Y - 1 - edge - monitor_inset))
  omega = np.array([omega_of(l) for l in wavelengths])
  n = len(ports)
  target = (rng.uniform(size=(n, n)) < 0.5).astype(np.float64)
  np.fill_diagonal(target, 0.0)
  ramp = (float(omega.mean() * 0.5 * ramp_steps), 4.0)
  return SMatrixProblem(eps.astype(np.float32), mask, sig, ports, omega, tt,
                        ((cx - half, cy - half, z0), (device_cells, device_cells,
                                                      z1 - z0)),
                        target, window, zc, ramp, pml)


def _port_profile(P: SMatrixProblem, port: Port):
  """Gaussian (sigma 7.5 cells) over the port window: (2w, Z) in
  (transverse, z)."""
  Z = P.eps.shape[3]
  t = np.arange(-P.window, P.window)[:, None] + 0.5 * (port.axis == 0)
  z = np.arange(Z)[None, :] - P.zc
  return np.exp(-(t**2 + z**2) / (2 * 7.5**2)).astype(np.float32)


def _monitor_box(P: SMatrixProblem, port: Port):
  Z = P.eps.shape[3]
  if port.axis == 0:
    return (port.monitor, port.center - P.window, 0), (1, 2 * P.window, Z)
  return (port.center - P.window, port.monitor, 0), (2 * P.window, 1, Z)


def _transverse(port: Port):
  """E component carrying a port's TE-like mode: Ey for x-normal ports."""
  return 1 if port.axis == 0 else 0


class SMatrixSolver:
  """The 2n plans (n forwards, n unit adjoints) of one S-matrix problem.
  With ``world`` > 1 this rank runs the solves ``replicas.shard`` gives it
  (plans 0..n-1 are the forwards, n..2n-1 the unit adjoints)."""

  def __init__(self, P: SMatrixProblem, device=None, launch=None, rank: int = 0,
               world: int = 1):
    self.P = P
    self.rank, self.world = rank, world
    dev = torch.device(device or "cuda")
    self.dev = dev
    X, Y, Z = P.eps.shape[1:]
    dt = 0.5
    om = P.omega
    ww = len(om)
    interval = _field._sampling_interval(om.min(), om.max(), ww, dt)
    self.steps = (P.tt - 2 * interval * ww - 1, P.tt, interval)
    self.weights = _field.projection_weights(om, self.steps, dt)
    n_t = np.arange(P.tt)
    r = _adjoint.ramp(om, dt, P.tt, *P.ramp)
    rsin = np.mean(r * np.exp(1j * om[:, None] * dt * n_t), axis=0)
    fwave = np.stack([np.imag(rsin), np.zeros(P.tt)], axis=1)
    awave = _adjoint.adjoint_waveform(om, dt, P.tt, *P.ramp)
    wt = _adjoint.discrete_omega(om, dt)
    coef = 1j * np.exp(1.5j * om * dt) / wt
    kap = np.ones_like(P.pml_sigma)
    alp = np.zeros_like(P.pml_sigma)
    knobs = launch or {}
    base = dict(domain=(X, Y, Z), offset=(0, 0, 0), region=(X, Y, Z), tt=P.tt,
                dt=dt, pml_widths=(P.pml, P.pml), pml_kappa=kap,
                pml_sigma=P.pml_sigma,
                pml_alpha=alp, output_steps=self.steps,
                out_mode=engine.OUT_PHASORS, weights=self.weights, **knobs)
    self.eps = torch.as_tensor(P.eps, device=dev)
    self.mask = torch.as_tensor(P.mask, device=dev)
    dbox = P.design_box
    mons = [_monitor_box(P, p) for p in P.ports]
    self.plans, self.inputs = [], []
    for port in P.ports:  # forwards
      prof = np.zeros((2, 3) + ((2, Y, Z) if port.axis == 0 else (X, 2, Z)),
                      np.float32)
      win = _port_profile(P, port)
      t0 = port.center - P.window
      c = _transverse(port)
      if port.axis == 0:
        prof[0, c, 1, t0:t0 + 2 * P.window, :] = win
        org = (port.source - 1, 0, 0)
      else:
        prof[0, c, t0:t0 + 2 * P.window, 1, :] = win
        org = (0, port.source - 1, 0)
      plan = engine.Plan(**base, source_origin=org, source_shape=prof.shape[2:],
                         source_ncols=2, monitors=[dbox] + mons)
      self.plans.append(plan)
      self.inputs.append(dict(source=torch.as_tensor(prof, device=dev),
                              waveform=torch.as_tensor(fwave, dtype=torch.float32,
                                                       device=dev)))
    # The port windows reach into the z-PML, where the operator is not
    # reciprocal: the unit adjoint sources are divided by the CPML stretch
    # (the S^-1 r of the adjoint; the design box lies outside the PML).
    stretch = _adjoint.cpml_stretch(om, dt, kap, P.pml_sigma, alp, (P.pml, P.pml))
    for port in P.ports:  # unit adjoints
      (mo, ms) = _monitor_box(P, port)
      win = _port_profile(P, port).reshape(ms)
      prof = np.zeros((2 * ww, 3) + ms, np.float32)
      c = _transverse(port)
      j = coef[:, None, None, None] * win[None] / stretch[:, c, None, None, :]
      prof[:ww, c] = np.real(j)
      prof[ww:, c] = np.imag(j)
      plan = engine.Plan(**base, source_origin=mo, source_shape=ms,
                         source_ncols=2 * ww, monitors=[dbox])
      self.plans.append(plan)
      self.inputs.append(dict(source=torch.as_tensor(prof, device=dev),
                              waveform=torch.as_tensor(awave, dtype=torch.float32,
                                                       device=dev)))
    for kw in self.inputs:
      kw.update(epsilon=self.eps, absorption_mask=self.mask)
    self.outs = [torch.empty(p.out_shape(), device=dev) for p in self.plans]
    self.mine = replicas.shard(range(len(self.plans)), rank, world)
    self.batch = None

  @property
  def cell_updates(self):
    """Cell-updates of the solves this rank runs."""
    X, Y, Z = self.P.eps.shape[1:]
    return len(self.mine) * X * Y * Z * self.P.tt

  def run_batched(self, graph: bool = True):
    if self.batch is None:
      self.batch = engine.Batch([self.plans[k] for k in self.mine])
    self.batch.run([dict(self.inputs[k], out=self.outs[k]) for k in self.mine],
                   graph=graph)

  def run_serial(self):
    """The per-simulation plain loop: this rank's solves one after another."""
    for k in self.mine:
      self.plans[k].run(**self.inputs[k], out=self.outs[k])

  def exchange(self):
    """Every rank gets every solve's recorded boxes (an all-gather over the
    initialised process group; nothing to do on one rank)."""
    if self.world == 1:
      return
    import torch.distributed as dist
    got = [None] * self.world
    dist.all_gather_object(got, {k: self.outs[k].cpu() for k in self.mine})
    for part in got:
      for k, t in part.items():
        self.outs[k].copy_(t)

  def results(self):
    """(S (n, n, ww) complex, objective, dL/d-eps (3, design box)); with
    several ranks every rank must call it (it starts with the exchange).

    Both reductions run on the device in the native library: S_ij is one
    weighted sum over port j's monitor plane of forward i's phasors
    (``pjzfdtd_plane_overlaps``), and dL/d-eps is
    ``sum_w Re(q_w sum_ij F_i c_ij G_j)`` over the design box
    (``pjzfdtd_smatrix_gradient``), both in FP64; only the n x n x ww
    objective and its coefficients ``c = conj(dL/dS)`` are formed on the
    host."""
    self.exchange()
    P = self.P
    lib = _lib.load()
    n, ww = len(P.ports), len(P.omega)
    dev = self.dev
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    # Overlaps: term (i, j) = forward i's phasors on port j's plane.
    blocks, profs, comps, npts = [], [], [], []
    prof_t = [torch.as_tensor(_port_profile(P, port), device=dev).reshape(-1)
              .contiguous() for port in P.ports]
    views = [self.plans[i].split(self.outs[i]) for i in range(n)]
    for i in range(n):
      for j, port in enumerate(P.ports):
        v = views[i][1 + j]
        blocks.append(v.data_ptr())
        profs.append(prof_t[j].data_ptr())
        comps.append(_transverse(port))
        npts.append(v[0, 0].numel())
    S_dev = torch.empty((n * n, ww, 2), dtype=torch.float64, device=dev)
    arr = lambda t, v: (t * len(v))(*v)
    _lib.check(lib.pjzfdtd_plane_overlaps(
        n * n, arr(ctypes.c_void_p, blocks), arr(ctypes.c_void_p, profs),
        arr(ctypes.c_int32, comps), arr(ctypes.c_int64, npts), ww,
        ctypes.c_void_p(S_dev.data_ptr()), stream))
    S = torch.view_as_complex(S_dev).reshape(n, n, ww)
    Sh = S.cpu().numpy()
    m = np.asarray(P.target, np.float64)
    L = torch.as_tensor((m[:, :, None] * np.abs(Sh) ** 2).sum(), dtype=torch.float64)
    c = np.conj(2 * m[:, :, None] * Sh)  # (n, n, ww)
    wt = _adjoint.discrete_omega(P.omega, 0.5)
    q = wt**2 * np.exp(-2j * P.omega * 0.5)
    F = [views[i][0] for i in range(n)]
    G = [self.plans[n + j].split(self.outs[n + j])[0] for j in range(n)]
    cells = int(F[0][0].numel())
    grad = torch.empty(F[0].shape[1:], dtype=torch.float32, device=dev)
    cf = np.ascontiguousarray(np.stack([c.real, c.imag], -1), np.float32)
    qf = np.ascontiguousarray(np.stack([q.real, q.imag], -1), np.float32)
    _lib.check(lib.pjzfdtd_smatrix_gradient(
        n, ww, cells, arr(ctypes.c_void_p, [t.data_ptr() for t in F]),
        arr(ctypes.c_void_p, [t.data_ptr() for t in G]), cf.ctypes.data,
        qf.ctypes.data, ctypes.c_void_p(grad.data_ptr()), stream))
    return S, L, grad
