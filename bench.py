"""Benchmark: forward FDTD throughput (Gcell-updates/s) on the c1 workload.

Workload (``--workload c1``, default): 512x512x64 Yee domain (16-cell x-y
absorber, 8-cell z-PML included), Si waveguide through a blurred random
50x50x6 design region, 10000 steps, 5 output frequencies over 1.50-1.60 um,
phasors projected inside the time loop.  One bench "step" is one full
forward solve (10000 Yee updates of every cell).  Inputs (400 MB of field
state, 200 MB of coefficients) exceed the 129 MB L2, so no flush is needed
between solves.

Output: one JSON line (rank 0).  ``value`` is device-resident throughput of
the engine plan; ``e2e`` is the same metric through ``pjz_gb300.field`` with
host inputs (H2D of epsilon/source and D2H of the complex phasors inside the
timed region).  ``roofline`` compares the step kernel's algorithmic bytes
(60 B per cell-update, times the cell-updates of one launch: two per cell
for a two-step launch) per launch time against the measured HBM copy
bandwidth; ``traffic`` is the DRAM bytes ncu counted for one launch, below
the algorithmic bytes when a launch advances two steps.
``--impl reference`` times the CPU path (the oracle's C Yee transcription
on all host cores; the reference engine is CUDA-only and not available).
The native line's ``cpu_baseline`` also carries ``torch_eager``: the same
update as eager torch ops on CPU tensors (``oracle/yee_torch.py``), all
host threads, a second CPU figure beside the C port.
"""

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("Gcell-updates/s and HBM GB/s vs roofline; batched grads/s vs plain "
          "loop at 1e-5 rel-L2")
UNIT = "Gcell-updates/s"
BYTES_PER_CELL = 60  # read E(3)+H(3)+coef(3), write E(3)+H(3), FP32
BYTES_PER_CELL_F16 = 30  # the same 15 values per cell-update, binary16


def _args():
  ap = argparse.ArgumentParser()
  ap.add_argument("--gpus", type=int, default=1)
  ap.add_argument("--steps", type=int, default=3)
  ap.add_argument("--warmup", type=int, default=3)
  ap.add_argument("--impl", default="native", choices=["native", "reference"])
  ap.add_argument("--workload", default="c1",
                  choices=["c0", "c1", "c3", "c4", "src-x", "src-y", "src-y6",
                           "render"],
                  help="src-*: one-step launches of 512x512x64 with an x-normal, "
                       "y-normal or 6-column y-normal source box (straggler "
                       "study); render: permittivity rendering of a 512x512 "
                       "stack, zz 64")
  ap.add_argument("--batch-n", type=int, default=64, help="c3: problems")
  ap.add_argument("--tune", action="store_true", help="c3: autotune per shape")
  ap.add_argument("--tt", type=int, default=0, help="override time steps")
  ap.add_argument("--cpu-seconds", type=float, default=12.0)
  ap.add_argument("--no-e2e", action="store_true")
  ap.add_argument("--no-cpu", action="store_true")
  ap.add_argument("--no-batched", action="store_true",
                  help="c1: skip the batched c4 S-matrix gradient leg")
  ap.add_argument("--no-f16", action="store_true",
                  help="c1: skip the binary16-storage leg")
  ap.add_argument("--f16-tile-y", type=int, default=-1,
                  help="c1: tile_y of the binary16 leg (-1: as --tile-y)")
  ap.add_argument("--kernel", type=int, default=0,
                  help="0 auto, 1 register-marching, 2 streamed, 3 lean streamed")
  ap.add_argument("--stages", type=int, default=0)
  ap.add_argument("--tile-y", type=int, default=0)
  ap.add_argument("--seg-x", type=int, default=0)
  ap.add_argument("--spp", type=int, default=0,
                  help="time steps per launch: 0 auto, 1, 2 (temporal blocking)")
  return ap.parse_args()


def _workload(args):
  from pjz_gb300 import workloads
  kw = {"tt": args.tt} if args.tt else {}
  if args.workload == "c0":
    wl = workloads.waveguide_c0(**kw)
  else:
    wl = workloads.design_c1(**kw)
  lp = wl.sim_params.launch_params._replace(
      kernel=getattr(args, "kernel", 0), stages=getattr(args, "stages", 0),
      tile_y=getattr(args, "tile_y", 0), seg_x=getattr(args, "seg_x", 0),
      steps_per_pass=getattr(args, "spp", 0))
  return wl._replace(sim_params=wl.sim_params._replace(launch_params=lp))


def _dist():
  rank = int(os.environ.get("RANK", 0))
  world = int(os.environ.get("WORLD_SIZE", 1))
  local = int(os.environ.get("LOCAL_RANK", 0))
  return rank, world, local


class Clocks:
  """Samples nvidia-smi SM clocks and throttle reasons during a region."""
  Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
       "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
       "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

  def __init__(self, index, path):
    self.path = path
    self.proc = None
    self.index = index
    try:
      self.f = open(path, "w")
      self.proc = subprocess.Popen(
          ["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}",
           "--format=csv,noheader,nounits", "-lms", "200"],
          stdout=self.f, stderr=subprocess.DEVNULL)
    except (OSError, FileNotFoundError):
      self.proc = None

  def stop(self):
    if self.proc is None:
      return None
    self.proc.terminate()
    try:
      self.proc.wait(timeout=5)
    except subprocess.TimeoutExpired:
      self.proc.kill()
    self.f.close()
    rows = []
    for line in open(self.path):
      parts = [p.strip() for p in line.split(",")]
      if len(parts) >= 9 and parts[1].isdigit():
        rows.append(parts)
    if not rows:
      return None
    sm = [int(r[1]) for r in rows]
    busy = [s for s in sm if s > 0.5 * max(sm)] or sm
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
             "sw_power_cap"]
    reasons = sorted({n for r in rows for n, v in zip(names, r[5:9])
                      if v.lower() == "active"})
    return {"sm_mhz": statistics.median(busy), "sm_max_mhz": int(rows[0][2]),
            "samples": len(rows), "reasons": reasons}


def _peaks():
  path = os.path.join(ROOT, "MEASURED_PEAKS.json")
  try:
    with open(path) as f:
      d = json.load(f)
    return float(d["hbm_gbs"]), "measured"
  except (OSError, KeyError, ValueError):
    return 6800.0, "fallback"


def _profile_traffic(name):
  """DRAM bytes per cell per launch of the step kernel from a committed ncu
  summary (profiles/<name>.json), or None."""
  path = os.path.join(ROOT, "profiles", f"{name}.json")
  try:
    with open(path) as f:
      d = json.load(f)
    v = d.get("dram_bytes_per_cell_per_launch")
    if v is None:
      v = d["dram_bytes_per_cell_update"]
    return float(v), d
  except (OSError, KeyError, ValueError):
    return None, None


def cpu_baseline(wl, seconds, threads=0, torch_eager=True):
  """Oracle C Yee (FP32, OpenMP) on a bounded number of steps of ``wl``;
  with ``torch_eager`` also the eager-torch CPU port of the same update."""
  import oracle
  from oracle import pjz_ref
  sp = wl.sim_params
  kw, omega = pjz_ref.field_setup(wl.epsilon, wl.source, wl.omega, wl.source_pos,
                                  pjz_ref.SimParams(*sp[:-1]), zz=wl.domain[2])
  domain = wl.domain
  org, shp, prof = oracle.plane_source_box(kw["source_field"],
                                           kw["source_position"], domain)
  threads = threads or os.cpu_count()

  def run(n):
    t0 = time.perf_counter()
    oracle.run(eps=kw["epsilon"], offset=kw["offset"], mask=kw["absorption_mask"],
               kappa=kw["pml_kappa"], sigma=kw["pml_sigma"], alpha=kw["pml_alpha"],
               dt=kw["dt"], tt=n, pml_widths=kw["pml_widths"], source_origin=org,
               source_profile=prof, waveform=kw["source_waveform"][:n],
               mode="none", nthreads=threads)
    return time.perf_counter() - t0

  t1 = run(1)
  t3 = run(3)
  per = max((t3 - t1) / 2, 1e-6)
  n = max(2, min(wl.sim_params.tt, int(seconds / per)))
  dt = run(n)
  cells = np.prod(domain) * n
  out = {"value": cells / dt / 1e9, "unit": UNIT, "cores": threads,
         "kind": "port",
         "sample": f"{n} of {wl.sim_params.tt} steps of the {domain[0]}x"
                   f"{domain[1]}x{domain[2]} domain, oracle/yee.c FP32 + "
                   f"OpenMP, {dt:.1f} s incl. set-up"}
  if not torch_eager:
    return out
  try:
    out["torch_eager"] = torch_eager_baseline(kw, org, prof, domain, wl,
                                              seconds / 2, threads)
  except Exception as e:  # a second CPU figure only; never fails the line
    out["torch_eager"] = {"error": f"{type(e).__name__}: {e}"}
  return out


def torch_eager_baseline(kw, org, prof, domain, wl, seconds, threads):
  """The same update as eager torch ops on CPU tensors (oracle/yee_torch.py,
  FP32), all host threads; per-step time from runs of 1 and 1 + n steps, so
  the set-up is excluded."""
  from oracle import yee_torch

  def run(n):
    t0 = time.perf_counter()
    yee_torch.run(eps=kw["epsilon"], offset=kw["offset"], mask=kw["absorption_mask"],
                  kappa=kw["pml_kappa"], sigma=kw["pml_sigma"], alpha=kw["pml_alpha"],
                  dt=kw["dt"], tt=n, pml_widths=kw["pml_widths"], source_origin=org,
                  source_profile=prof, waveform=kw["source_waveform"][:n],
                  threads=threads)
    return time.perf_counter() - t0

  t1 = run(1)
  per = max(run(3) - t1, 1e-6) / 2
  # 1 + n steps must fit the waveform's tt rows.
  n = max(2, min(wl.sim_params.tt - 1, int(seconds / per)))
  dt = run(1 + n) - t1
  cells = np.prod(domain) * n
  return {"value": cells / max(dt, 1e-9) / 1e9, "unit": UNIT, "cores": threads,
          "kind": "port",
          "sample": f"{n} steps of the same domain, oracle/yee_torch.py (eager "
                    f"torch {__import__('torch').__version__} on CPU tensors, "
                    f"FP32), set-up excluded"}


def run_reference(args):
  rank, world, _ = _dist()
  if rank != 0:
    return
  wl = _workload(args)
  vals = []
  for i in range(args.warmup + args.steps):
    r = cpu_baseline(wl, max(2.0, args.cpu_seconds / max(args.steps, 1)),
                     torch_eager=False)
    if i >= args.warmup:
      vals.append(r["value"])
  v = float(np.mean(vals))
  r["value"] = v
  print(json.dumps({
      "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
      "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
      "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
      "dtype": "f32", "data": "synthetic",
      "config": {"workload": wl.name, "domain": list(wl.domain),
                 "time_steps": wl.sim_params.tt, "freqs": len(wl.omega)},
      "cpu_baseline": r,
      "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
              "d2h_bytes_per_step": 0}}), flush=True)


def run_native(args):
  import torch
  import pjz_gb300
  from pjz_gb300 import _field, engine
  rank, world, local = _dist()
  torch.cuda.set_device(local)
  dev = torch.device("cuda", local)
  if world > 1:
    import torch.distributed as tdist
    tdist.init_process_group("nccl", device_id=dev)
  wl = _workload(args)
  sp = wl.sim_params
  eps = torch.as_tensor(wl.epsilon, device=dev)
  src = torch.as_tensor(wl.source, device=dev)
  kw, omega = _field._setup(eps, src, wl.omega, wl.source_pos, sp)
  plan, prof = _field.phasor_plan(kw, omega)
  run_args = dict(epsilon=eps, absorption_mask=kw["absorption_mask"],
                  source=prof, waveform=kw["source_waveform"])
  out = torch.empty(plan.out_shape(), dtype=torch.float32, device=dev)
  cells = int(np.prod(wl.domain)) * sp.tt

  def barrier():
    if world > 1:
      torch.distributed.barrier()
    torch.cuda.synchronize()

  def maxed(x):
    if world == 1:
      return x
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())

  for _ in range(args.warmup):
    plan.run(**run_args, out=out)
  barrier()
  stream = torch.cuda.current_stream(dev)
  clocks = Clocks(local, _clock_path(f"bench_{rank}"))
  e0 = torch.cuda.Event(enable_timing=True)
  e1 = torch.cuda.Event(enable_timing=True)
  e0.record(stream)
  for _ in range(args.steps):
    plan.run(**run_args, out=out)
  e1.record(stream)
  barrier()
  clk = clocks.stop()
  ms = maxed(e0.elapsed_time(e1)) / args.steps
  value = world * cells / (ms / 1e3) / 1e9

  # Step-kernel launch time: steps [1, L) skip the set-up kernels.
  nl = min(sp.tt - 1, 2000)
  plan.run(**run_args, out=out)  # leaves a valid state in the workspace
  k0 = torch.cuda.Event(enable_timing=True)
  k1 = torch.cuda.Event(enable_timing=True)
  k0.record(stream)
  plan.run(**run_args, out=out, steps=(1, 1 + nl))
  k1.record(stream)
  torch.cuda.synchronize()
  # Algorithmic bytes are 60 B per cell-update; a two-step launch
  # (temporal blocking) performs two cell-updates per cell while it reads
  # and writes the state once, so its DRAM traffic (`traffic`) falls below
  # its algorithmic bytes.  `state_gbs` is the state actually streamed (60 B
  # per cell per launch).
  cfg0 = plan.launch_config()
  launches = plan.step_launches(1, 1 + nl)
  launch_ms = k0.elapsed_time(k1) / launches
  cells_per_launch = int(np.prod(wl.domain))
  steps_per_launch = nl / launches
  alg_bytes = BYTES_PER_CELL * cells_per_launch * steps_per_launch
  achieved = alg_bytes / (launch_ms / 1e3) / 1e9
  state_gbs = BYTES_PER_CELL * cells_per_launch / (launch_ms / 1e3) / 1e9
  peak, peak_kind = _peaks()
  kname = {(3, 2): "yee_lean2", (3, 1): "yee_lean", (2, 2): "yee_stream2",
           (2, 1): "yee_stream"}.get((cfg0["kernel"], cfg0["steps_per_pass"]),
                                     "yee_step")
  bpc, prof_d = _profile_traffic(f"{kname}_{args.workload}")
  roofline = {"bound": "hbm", "achieved": achieved, "peak": peak,
              "unit": "GB/s", "frac": achieved / peak,
              "peak_source": f"hbm_gbs of {peak_kind}",
              "kernel": f"{kname}_kernel",
              "algorithmic_bytes_per_launch": alg_bytes,
              "steps_per_launch": steps_per_launch,
              "state_gbs": state_gbs,
              "launch_ms": launch_ms,
              "traffic": None if bpc is None else bpc * cells_per_launch}

  e2e = None
  if not args.no_e2e:
    eps_h = torch.as_tensor(wl.epsilon).pin_memory()
    src_h = torch.as_tensor(wl.source).pin_memory()
    # Warm-up: the same W calls as the device loop, so the caching
    # allocator holds the buffers of a call made while the previous
    # result is still alive (as in the timed loop).
    res = pjz_gb300.field(eps_h, src_h, wl.omega, wl.source_pos, sp)
    host = torch.empty(res.shape, dtype=res.dtype).pin_memory()
    for _ in range(max(1, args.warmup)):
      res = pjz_gb300.field(eps_h.to(dev, non_blocking=True),
                            src_h.to(dev, non_blocking=True), wl.omega,
                            wl.source_pos, sp)
      host.copy_(res, non_blocking=True)
    barrier()
    clk_e = Clocks(local, _clock_path(f"e2e_{rank}"))
    t0 = time.perf_counter()
    for _ in range(args.steps):
      res = pjz_gb300.field(eps_h.to(dev, non_blocking=True),
                            src_h.to(dev, non_blocking=True), wl.omega,
                            wl.source_pos, sp)
      host.copy_(res, non_blocking=True)
      torch.cuda.synchronize()
    t_e2e = maxed(time.perf_counter() - t0) / args.steps
    e2e = {"value": world * cells / t_e2e / 1e9, "unit": UNIT,
           "h2d_bytes_per_step": eps_h.numel() * 4 + src_h.numel() * 4,
           "d2h_bytes_per_step": host.numel() * host.element_size(),
           "ms_per_step": t_e2e * 1e3, "clocks": clk_e.stop()}
    del res

  f16 = None
  if args.workload == "c1" and not args.no_f16:
    f16 = f16_leg(args, wl, eps, src, stream, barrier, maxed, world, cells)

  cpu = None
  if rank == 0 and not args.no_cpu:
    cpu = cpu_baseline(wl, args.cpu_seconds)

  batched = None
  if args.workload == "c1" and not args.no_batched:
    batched = (batched_c4(local, _clock_path(f"c4_{rank}")) if world == 1 else
               {"skipped": "the c4 leg runs on one GPU (replicas only)"})

  if rank == 0:
    cfg = plan.launch_config()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded blurred random design)",
        "config": {"workload": wl.name, "domain": list(wl.domain),
                   "time_steps": sp.tt, "freqs": len(wl.omega),
                   "output": "5-frequency phasors accumulated at the sample "
                             "steps (no snapshots stored)",
                   "l2": "inputs larger than L2 (600 MB state), no flush",
                   "parallelism": "replicas" if world > 1 else "single",
                   "launch": cfg},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "batched": batched, "reduced_precision": f16,
        # per solve: the step launches of its schedule, the cb and absorber
        # set-up kernels and one record pass per sample step.
        "gpu_launches": args.steps * (plan.step_launches() + 2 + plan.num_samples),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
  if world > 1:
    torch.distributed.destroy_process_group()


def f16_leg(args, wl, eps, src, stream, barrier, maxed, world, cells):
  """The same c1 solve with pjz's use_reduced_precision=True: binary16
  storage of fields, coefficients and CPML state, FP32 arithmetic (30 B per
  cell-update instead of 60).  Timed like the main line (W warm-up solves,
  K timed, device-resident), plus its step-kernel launch time against the
  HBM roofline on the 30 B figure."""
  import torch
  from pjz_gb300 import _field
  sp = wl.sim_params._replace(use_reduced_precision=True)
  if args.f16_tile_y >= 0:
    sp = sp._replace(launch_params=sp.launch_params._replace(tile_y=args.f16_tile_y))
  kw, omega = _field._setup(eps, src, wl.omega, wl.source_pos, sp)
  plan, prof = _field.phasor_plan(kw, omega)
  run_args = dict(epsilon=eps, absorption_mask=kw["absorption_mask"],
                  source=prof, waveform=kw["source_waveform"])
  out = torch.empty(plan.out_shape(), dtype=torch.float32, device=eps.device)
  for _ in range(args.warmup):
    plan.run(**run_args, out=out)
  barrier()
  e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
  e0.record(stream)
  for _ in range(args.steps):
    plan.run(**run_args, out=out)
  e1.record(stream)
  barrier()
  ms = maxed(e0.elapsed_time(e1)) / args.steps
  nl = min(sp.tt - 1, 2000)
  k0, k1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
  k0.record(stream)
  plan.run(**run_args, out=out, steps=(1, 1 + nl))
  k1.record(stream)
  torch.cuda.synchronize()
  launch_ms = k0.elapsed_time(k1) / plan.step_launches(1, 1 + nl)
  per_launch = int(np.prod(wl.domain))
  achieved = BYTES_PER_CELL_F16 * per_launch / (launch_ms / 1e3) / 1e9
  peak, peak_kind = _peaks()
  cfg = plan.launch_config()
  bpc = None
  if cfg["kernel"] == 3 and cfg["steps_per_pass"] == 1:
    bpc, _ = _profile_traffic(f"yee_lean_f16_ty{cfg['tile_y']}_{args.workload}")
  return {"value": world * cells / (ms / 1e3) / 1e9, "unit": UNIT,
          "ms_per_step": ms, "dtype": "binary16 storage, f32 arithmetic",
          "launch": cfg,
          "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                       "unit": "GB/s", "frac": achieved / peak,
                       "peak_source": f"hbm_gbs of {peak_kind}",
                       "kernel": "yee_lean_kernel (binary16)",
                       "algorithmic_bytes_per_launch": BYTES_PER_CELL_F16 * per_launch,
                       "launch_ms": launch_ms,
                       "traffic": None if bpc is None else bpc * per_launch},
          "accuracy": "rel-L2 vs the FP64 oracle: asserted and printed by "
                      "tests/test_gpu_f16.py (c0) and "
                      "tests/test_gpu_full_length.py (c1)"}


def batched_c4(device_index, clock_path):
  """The batched half of the metric: config c4 (8-port S-matrix on
  1024x1024x64, 8 forward + 8 unit-adjoint solves, 12000 steps, 3
  frequencies) as one graph-captured batched launch against the serial
  loop of the same 16 solves (pjz's per-port loop), in gradients per
  second.  One batched warm-up run (graph capture, workspaces, clocks),
  then one serial and one batched run, timed back to back."""
  import torch
  from pjz_gb300 import smatrix
  dev = torch.device("cuda", device_index)
  s = smatrix.SMatrixSolver(smatrix.build_c4(), device=dev)
  t0 = time.perf_counter()
  s.run_batched(graph=True)
  torch.cuda.synchronize()
  t_warm = time.perf_counter() - t0
  for p in s.plans:  # the serial loop's workspaces, outside the timing
    p.workspace(dev)
  t_batch, t_serial, clk = _alternate(lambda: s.run_batched(graph=True),
                                      s.run_serial, 1, clock_path)
  s.batch.check_status()
  S, L, grad = s.results()
  cells = s.cell_updates
  return {"value": 1.0 / t_batch, "unit": "grads/s",
          "workload": "c4 8-port S-matrix gradient, 1024x1024x64, 8 forward + "
                      "8 unit-adjoint solves, 12000 steps, 3 frequencies",
          "gcell_updates_per_s": cells / t_batch / 1e9,
          "seconds_per_grad": t_batch,
          "serial_loop": {"value": 1.0 / t_serial, "unit": "grads/s",
                          "gcell_updates_per_s": cells / t_serial / 1e9,
                          "seconds_per_grad": t_serial},
          "speedup": t_serial / t_batch,
          "objective": float(L), "grad_finite": bool(torch.isfinite(grad).all()),
          "timing": f"one batched warm-up run ({t_warm:.1f} s incl. graph "
                    "capture), then one serial and one batched run timed "
                    "with the host clock around a device synchronise",
          "clocks": clk}


def _alternate(fa, fb, reps, clock_path):
  """Times ``fa`` and ``fb`` alternately ``reps`` times each (after their
  warm-up elsewhere) so that clock and power state affect both alike;
  returns (mean seconds of fa, mean seconds of fb, clock record)."""
  import torch
  clocks = Clocks(0, clock_path)
  ta, tb = [], []
  for _ in range(reps):
    for fn, acc in ((fb, tb), (fa, ta)):
      torch.cuda.synchronize()
      t0 = time.perf_counter()
      fn()
      torch.cuda.synchronize()
      acc.append(time.perf_counter() - t0)
  return statistics.mean(ta), statistics.mean(tb), clocks.stop()


def _clock_path(tag):
  """Where the nvidia-smi clock samples of a timed region are written
  (``PJZ_BENCH_CLOCKS_DIR``, default the temp directory)."""
  d = os.environ.get("PJZ_BENCH_CLOCKS_DIR", tempfile.gettempdir())
  return os.path.join(d, f"clocks_{tag}.csv")


def _timed(fn, steps, warmup):
  import torch
  for _ in range(warmup):
    fn()
  torch.cuda.synchronize()
  t0 = time.perf_counter()
  for _ in range(steps):
    fn()
  torch.cuda.synchronize()
  return (time.perf_counter() - t0) / steps


def run_batch_c3(args):
  """c3: many uneven problems in one graph-captured batched run vs the
  serial loop of the same plans."""
  import torch
  from pjz_gb300 import _field, autotune, engine, workloads
  dev = torch.device("cuda", 0)
  wls = workloads.batch_c3(n=args.batch_n, **({"tt": args.tt} if args.tt else {}))
  plans, inputs = [], []
  for wl in wls:
    sp = wl.sim_params
    if args.tune:
      sp = sp._replace(launch_params=sp.launch_params._replace(
          **autotune.knobs(wl.domain, sp.pml_widths)))
    eps = torch.as_tensor(wl.epsilon, device=dev)
    kw, om = _field._setup(eps, torch.as_tensor(wl.source, device=dev), wl.omega,
                           wl.source_pos, sp)
    plan, prof = _field.phasor_plan(kw, om)
    plans.append(plan)
    inputs.append(dict(epsilon=eps, absorption_mask=kw["absorption_mask"],
                       source=prof, waveform=kw["source_waveform"],
                       out=torch.empty(plan.out_shape(), device=dev)))
  cells = sum(wl.cell_updates for wl in wls)
  batch = engine.Batch(plans)
  run_batch = lambda: batch.run(inputs, graph=True)
  run_serial = lambda: [p.run(**kw) for p, kw in zip(plans, inputs)]
  for _ in range(args.warmup):  # graph capture, workspaces, clocks up
    run_batch()
  run_serial()
  t_batch, t_serial, clk = _alternate(run_batch, run_serial, args.steps,
                                      _clock_path("c3"))
  batch.check_status()
  print(json.dumps({
      "metric": METRIC, "value": cells / t_batch / 1e9, "unit": UNIT,
      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
      "ms_per_step": t_batch * 1e3, "higher_is_better": True,
      "scaling": "weak", "vs_baseline": None, "dtype": "f32",
      "data": "synthetic (seeded blurred random designs)",
      "config": {"workload": f"c3 {len(wls)} uneven problems, batched + graph",
                 "cell_updates": cells, "tuned": bool(args.tune),
                 "shapes": sorted({str(w.domain) for w in wls})},
      "serial_loop": {"value": cells / t_serial / 1e9, "unit": UNIT,
                      "ms_per_step": t_serial * 1e3},
      "speedup_vs_serial_loop": t_serial / t_batch,
      "timing": "batched and serial runs alternated after warm-up",
      "clocks": clk,
      # per batched run: one step launch per launch of the longest schedule
      # (a launch that mixes one- and two-step problems runs two kernels),
      # plus per problem two set-up kernels and one record pass per sample.
      "gpu_launches": args.steps * (max(p.step_launches() for p in plans) + sum(
          p.num_samples + 2 for p in plans))}), flush=True)


def run_smatrix_c4(args):
  """c4: 8 forward + 8 unit-adjoint solves of the 8-port device in one
  batched graph launch vs the serial loop; grads/s."""
  import torch
  from pjz_gb300 import smatrix
  P = smatrix.build_c4(**({"tt": args.tt} if args.tt else {}))
  s = smatrix.SMatrixSolver(P)
  dev = torch.device("cuda", 0)
  s.run_batched(graph=True)  # graph capture and batch workspace
  for p in s.plans:  # the serial loop's workspaces, outside the timing
    p.workspace(dev)
  # One repetition of each arm per 3 requested steps: a repetition of either
  # arm is 16 solves of 12000 steps on 1024x1024x64 (over two minutes).
  t_batch, t_serial, clk = _alternate(lambda: s.run_batched(graph=True),
                                      s.run_serial, max(1, args.steps // 3),
                                      _clock_path("c4"))
  S, L, grad = s.results()
  cells = s.cell_updates
  print(json.dumps({
      "metric": METRIC, "value": 1.0 / t_batch, "unit": "grads/s",
      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
      "ms_per_step": t_batch * 1e3, "higher_is_better": True,
      "scaling": "weak", "vs_baseline": None, "dtype": "f32",
      "data": "synthetic (seeded blurred random 8-port device)",
      "config": {"workload": "c4 8-port S-matrix, 8 fwd + 8 adjoint, batched",
                 "domain": list(P.eps.shape[1:]), "time_steps": P.tt,
                 "freqs": len(P.omega), "objective": float(L)},
      "gcell_updates_per_s": cells / t_batch / 1e9,
      "serial_loop": {"value": 1.0 / t_serial, "unit": "grads/s",
                      "gcell_updates_per_s": cells / t_serial / 1e9},
      "speedup_vs_serial_loop": t_serial / t_batch,
      "timing": "batched and serial runs alternated after warm-up",
      "clocks": clk}), flush=True)


SOURCE_BOXES = {  # name: (origin, box shape, waveform columns)
    "src-x": ((100, 0, 0), (2, 512, 64), 2),
    "src-y": ((0, 100, 0), (512, 2, 64), 2),
    "src-y6": ((0, 100, 0), (512, 1, 64), 6),
}


def run_source_box(args):
  """512x512x64, 8+8 z-PML, one time step per launch, uniform epsilon and a
  random source in one box orientation: 20 warm-up steps, then 300 steps
  timed with CUDA events (the run behind the source-orientation profile)."""
  import torch
  from pjz_gb300 import engine
  dev = torch.device("cuda", 0)
  X, Y, Z = 512, 512, 64
  tt = max(args.tt, 320) if args.tt else 400
  org, shp, ncols = SOURCE_BOXES[args.workload]
  sig = np.zeros((Z, 2), np.float32)
  sig[:8] = 1.0
  sig[-8:] = 1.0
  p = engine.Plan(domain=(X, Y, Z), offset=(0, 0, 0), region=(X, Y, Z), tt=tt,
                  dt=0.5, pml_widths=(8, 8), pml_kappa=np.ones((Z, 2)),
                  pml_sigma=sig, pml_alpha=np.zeros((Z, 2)), source_origin=org,
                  source_shape=shp, source_ncols=ncols, kernel=2)
  g = torch.Generator(device=dev).manual_seed(0)
  kw = dict(epsilon=torch.full((3, X, Y, Z), 2.0, device=dev),
            absorption_mask=torch.zeros((3, X, Y), device=dev),
            source=torch.randn((ncols, 3) + shp, device=dev, generator=g),
            waveform=torch.randn((tt, ncols), device=dev, generator=g))
  p.run(**kw, steps=(0, 20))
  torch.cuda.synchronize()
  e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
  e0.record()
  p.run(**kw, steps=(20, 320))
  e1.record()
  torch.cuda.synchronize()
  p.check_status()
  ms = e0.elapsed_time(e1) / 300
  print(json.dumps({
      "workload": args.workload, "domain": [X, Y, Z], "source_origin": org,
      "source_box": shp, "source_columns": ncols, "ms_per_step": ms,
      "value": X * Y * Z / ms / 1e6, "unit": UNIT,
      "launch": p.launch_config()}), flush=True)


def run_render(args):
  """pjz_gb300.epsilon on a 3-layer stack of 512 x 512 cells at 2x
  magnification, zz 64: W warm-up and K timed renders (CUDA events on the
  current stream, L2 flushed by a 256 MB write before each), against the
  algorithmic bytes ll (2m)^2 4 read + 3 zz 4 written per (x, y) column."""
  import torch
  import pjz_gb300
  dev = torch.device("cuda", 0)
  m, zz, ll, n = 2, 64, 3, 512
  g = torch.Generator(device=dev).manual_seed(0)
  layers = 2.085 + 10.165 * torch.rand((ll, 2 * m * n, 2 * m * n), device=dev,
                                        generator=g)
  pos = np.array([28.5, 35.25], np.float32)
  out = torch.empty((3, n, n, zz), device=dev)
  flush = torch.empty(64 << 20, device=dev)
  for _ in range(max(args.warmup, 3)):
    pjz_gb300.epsilon(layers, pos, m, zz, out=out)
  times = []
  for _ in range(args.steps):
    flush.fill_(1.0)
    e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
    e0.record()
    pjz_gb300.epsilon(layers, pos, m, zz, out=out)
    e1.record()
    torch.cuda.synchronize()
    times.append(e0.elapsed_time(e1) / 1e3)
  t = statistics.median(times)
  nbytes = n * n * (ll * (2 * m) ** 2 * 4 + 3 * zz * 4)
  peak, kind = _peaks()
  gbs = nbytes / t / 1e9
  print(json.dumps({
      "workload": "render 512x512 cells, 3 layers, 2x, zz 64", "ms": t * 1e3,
      "algorithmic_bytes": nbytes, "achieved_gbs": gbs,
      "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak,
                   "unit": "GB/s", "frac": gbs / peak, "peak_kind": kind},
      "steps": args.steps, "warmup": max(args.warmup, 3),
      "timing": "median of CUDA-event times, L2 flushed before each"}),
      flush=True)


if __name__ == "__main__":
  a = _args()
  if a.workload == "render":
    run_render(a)
  elif a.workload in SOURCE_BOXES:
    run_source_box(a)
  elif a.impl == "reference":
    run_reference(a)
  elif a.workload == "c3":
    run_batch_c3(a)
  elif a.workload == "c4":
    run_smatrix_c4(a)
  else:
    run_native(a)
