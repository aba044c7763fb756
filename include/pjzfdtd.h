/*
 * pjzfdtd -- C ABI of the GB300 (sm_103a) FDTD engine behind pjz.
 *
 * This library replaces the engine pjz calls at src/pjz/_field.py:254-269
 * (`fdtdz_jax.fdtdz(...)`, an XLA custom call into the third-party fdtdz
 * CUDA package, dependency `fdtdz>=1.1.3` at setup.py:26).  The problem
 * description below carries exactly the keyword arguments of that call:
 *
 *   epsilon (3,rx,ry,rz)            -> pjzfdtd_buffers.epsilon, rx/ry/rz
 *   dt                              -> pjzfdtd_problem.dt
 *   source_field, source_position   -> source box + profile (see below)
 *   source_waveform (tt,2)          -> pjzfdtd_buffers.waveform, tt, src_ncols
 *   absorption_mask (3,X,Y)         -> pjzfdtd_buffers.absorption_mask, xx/yy
 *   pml_kappa/sigma/alpha (Z,2)     -> pjzfdtd_plan_create host arrays, zz
 *   pml_widths                      -> pml_lo, pml_hi
 *   output_steps (start,stop,step)  -> out_start, out_stop, out_step
 *   offset (px,py,pz)               -> ox, oy, oz
 *   use_reduced_precision           -> storage (binary16 fields, FP32
 *                                      arithmetic) and pjz's z budget
 *   launch_params                   -> tile_y, seg_x (0 = autotuned)
 *
 * fdtdz's plane sources map onto the general source box: an x-normal source
 * (2,1,Y,Z) at position s is a 2-plane box x in [s-1, s] whose waveform
 * column 0 drives plane s and column 1 plane s-1, with the two leading
 * entries feeding (Ey, Ez); y-normal (2,X,1,Z) likewise with (Ex, Ez);
 * z-normal (2,2,X,Y,1) is a 1-plane box at z = s, column k with profile k on
 * (Ex, Ey).  The adjoint solve uses the same box with 2*ww columns.
 *
 * Conventions: device buffers are caller-owned; every call is stream-ordered
 * on the stream passed in; a plan is not thread-safe; no call throws; every
 * call returns a pjzfdtd_status and leaves a message for
 * pjzfdtd_last_error() (thread-local) when it fails.  pjz raises ValueError
 * at trace time for bad shapes (src/pjz/_field.py:288-290); the matching
 * status here is PJZFDTD_ERR_INVALID, which the Python layer raises as
 * ValueError.
 */
#ifndef PJZFDTD_H_
#define PJZFDTD_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PJZFDTD_ABI_VERSION 2

typedef enum {
  PJZFDTD_OK = 0,
  PJZFDTD_ERR_INVALID = 1,     /* bad shape or argument */
  PJZFDTD_ERR_CUDA = 2,        /* CUDA runtime error */
  PJZFDTD_ERR_WORKSPACE = 3,   /* workspace missing or too small */
  PJZFDTD_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  PJZFDTD_ERR_UNSUPPORTED = 5  /* valid request this build does not serve */
} pjzfdtd_status;

typedef enum {
  PJZFDTD_OUT_NONE = 0,
  /* E at range(out_start, out_stop, out_step): (ns,3,rx,ry,rz), the
     fdtdz return value (src/pjz/_field.py:254, 276-278). */
  PJZFDTD_OUT_SNAPSHOTS = 1,
  /* weights @ snapshots fused into the time loop: (out_rows,3,rx,ry,rz)
     with weights = pinv(P^T) of src/pjz/_field.py:272-278. */
  PJZFDTD_OUT_PHASORS = 2,
  /* adjoint: sum_j E_j * (weights[:,j] . q) over the gradient box:
     (3,gnx,gny,gnz) -- the fused dL/d-eps accumulation. */
  PJZFDTD_OUT_GRADIENT = 3
} pjzfdtd_out_mode;

typedef enum {
  /* E, H, the E-update coefficient and the z-PML state stored as FP32. */
  PJZFDTD_STORAGE_F32 = 0,
  /* Stored as IEEE binary16 (rounded to nearest even on every write), with
     all arithmetic, source sums and phasor accumulators in FP32: half the
     HBM bytes per cell-update.  fdtdz's use_reduced_precision
     (src/pjz/_field.py:52, pjz's default) selects 16-bit storage; this is
     that mode.  Served by the lean streamed kernels (kernel 3), zz in
     {64, 48, 32} and z-PML widths that are multiples of 4. */
  PJZFDTD_STORAGE_F16 = 1
} pjzfdtd_storage;

typedef struct pjzfdtd_problem {
  int32_t xx, yy, zz;          /* simulation domain in cells */
  int32_t ox, oy, oz;          /* fdtdz `offset` of the epsilon region */
  int32_t rx, ry, rz;          /* epsilon / output region shape */
  int32_t tt;                  /* time steps (rows of the waveform) */
  int32_t pml_lo, pml_hi;      /* fdtdz `pml_widths` */
  float dt;
  int32_t src_x0, src_y0, src_z0;           /* source box origin */
  int32_t src_nx, src_ny, src_nz, src_ncols; /* box shape, waveform columns */
  int32_t out_start, out_stop, out_step;    /* fdtdz `output_steps` */
  int32_t out_mode;            /* pjzfdtd_out_mode */
  int32_t out_rows;            /* rows of weights (PHASORS, GRADIENT), <= 32 */
  int32_t record_h;            /* SNAPSHOTS/PHASORS: also record H */
  int32_t grad_x0, grad_y0, grad_z0, grad_nx, grad_ny, grad_nz;
  int32_t tile_y;              /* launch params: y rows per CTA, 0 = auto */
  int32_t seg_x;               /* launch params: x planes per CTA, 0 = auto */
  int32_t steps_per_pass;      /* launch params: time steps per HBM pass, 0 = auto */
  int32_t kernel;              /* launch params: 0 auto, 1 register-marching,
                                  2 bulk-copy streamed (needs zz % 4 == 0),
                                  3 lean streamed (compile-time zz/tile_y).
                                  Auto (FP32): the lean kernel at zz 64 (two
                                  steps per pass when steps_per_pass is 0)
                                  when the source box does not ride the
                                  streamed ring, else the streamed kernel
                                  (zz % 4 == 0), else kernel 1. */
  int32_t stages;              /* launch params: streamed ring depth, 0 = auto */
  int32_t warps;               /* launch params: streamed compute warps per CTA,
                                  0 = auto (one row per warp and pass) */
  int32_t wait_limit_kcycles;  /* bound of every device-side wait in thousands
                                  of SM cycles, 0 = default (~2 s) */
  int32_t test_stall_bytes;    /* test hook, 0 in use: the streamed producer
                                  announces this many bytes more than it
                                  copies, so waits run out (no fault) */
  int32_t storage;             /* pjzfdtd_storage of the state (ABI 2) */
} pjzfdtd_problem;

typedef struct pjzfdtd_buffers {
  const float* epsilon;          /* device (3,rx,ry,rz) */
  const float* absorption_mask;  /* device (3,xx,yy) */
  const float* source;           /* device (src_ncols,3,src_nx,src_ny,src_nz) */
  const float* waveform;         /* device (tt,src_ncols) */
  const float* q;                /* device (out_rows,3,grad box), GRADIENT */
  float* out;                    /* device, shape per out_mode */
  float* out_h;                  /* device, same shape as out, if record_h */
  float* fields;                 /* device (6,xx,yy,zz) state in/out, or NULL
                                    for a zero start and no state out */
} pjzfdtd_buffers;

typedef struct pjzfdtd_plan pjzfdtd_plan;

/* ABI version of the loaded library (PJZFDTD_ABI_VERSION it was built with). */
int32_t pjzfdtd_abi_version(void);

/* Copies the calling thread's last error message into buf (NUL-terminated);
   returns the status of that error. */
int32_t pjzfdtd_last_error(char* buf, size_t len);

/* Validates `problem` and builds a plan: CPML coefficients from the host
   arrays pml_kappa/sigma/alpha (zz,2) (src/pjz/_field.py:243-251) and, for
   PHASORS/GRADIENT, the host weights (out_rows, ns).  Host-only: no CUDA
   call is made, so this can run without a GPU. */
int32_t pjzfdtd_plan_create(const pjzfdtd_problem* problem,
                            const float* pml_kappa, const float* pml_sigma,
                            const float* pml_alpha, const float* weights,
                            pjzfdtd_plan** plan);

/* Device scratch the plan needs (bytes, 256-byte aligned start). */
int32_t pjzfdtd_plan_workspace_bytes(const pjzfdtd_plan* plan, size_t* bytes);

/* Number of recorded samples ns = len(range(out_start, out_stop, out_step)). */
int32_t pjzfdtd_plan_num_samples(const pjzfdtd_plan* plan, int32_t* ns);

int32_t pjzfdtd_plan_destroy(pjzfdtd_plan* plan);

/* Forward solve: all tt steps, the fdtdz call of src/pjz/_field.py:254-269
   (SNAPSHOTS) or the whole of `field` with its pinv projection fused
   (PHASORS, src/pjz/_field.py:271-279).  Stream-ordered on `stream`
   (a cudaStream_t, NULL = legacy default stream). */
int32_t pjzfdtd_forward(pjzfdtd_plan* plan, const pjzfdtd_buffers* buffers,
                        void* workspace, size_t workspace_bytes, void* stream);

/* Adjoint solve: the same update driven by the adjoint source in `buffers`,
   accumulating dL/d-eps = sum_j E_adj(t_j) * (weights[:,j] . q) over the
   gradient box without storing any time history (plan out_mode must be
   GRADIENT).  Replaces the residual-product VJP of src/pjz/_field.py:
   380-398. */
int32_t pjzfdtd_adjoint(pjzfdtd_plan* plan, const pjzfdtd_buffers* buffers,
                        void* workspace, size_t workspace_bytes, void* stream);

/* Runs steps [step_begin, step_end) only, continuing from the state kept in
   the workspace (step_begin == 0 re-initialises it).  Lets a caller
   checkpoint (copy `fields` out between calls) or interleave work. */
int32_t pjzfdtd_run_steps(pjzfdtd_plan* plan, const pjzfdtd_buffers* buffers,
                          void* workspace, size_t workspace_bytes,
                          int32_t step_begin, int32_t step_end, void* stream);

/* Replaces the recorded region of a SNAPSHOTS or PHASORS plan by `n` boxes
   `boxes[6k..6k+5] = (x0, y0, z0, nx, ny, nz)` (domain cells).  `out` then
   holds the boxes one after another, each shaped like a single-region output
   ((ns,3,box) or (rows,3,box)); pjzfdtd_plan_output_floats gives the total.
   Lets a caller keep phasors only where it needs them (a design region and
   port planes) instead of the whole epsilon region. */
int32_t pjzfdtd_plan_set_monitors(pjzfdtd_plan* plan, int32_t n,
                                  const int32_t* boxes);

/* Number of floats of `out` (and of `out_h`) the plan writes. */
int32_t pjzfdtd_plan_output_floats(const pjzfdtd_plan* plan, size_t* floats);

/* Batches independent problems (uneven domains, sources, frequencies, step
   counts): every time step advances all of them in one launch of the
   streamed kernel, whose blocks index a work table of (problem, tile,
   segment); record passes follow at each problem's sample steps.  With
   use_graph, the whole run is captured once into a CUDA graph and replayed
   while the buffers and workspace stay the same (stream must not be the
   legacy default stream).  This is the batched scheduler for many forward
   and adjoint solves (multi-port S-matrices); pjz runs them as a Python loop
   of `field` calls (src/pjz/_field.py:354-356).  Plans must be streamed
   (zz % 4 == 0) and outlive the batch; a plan that auto selection put on
   the lean kernel joins on the streamed plan it replaced (same workspace)
   and keeps it afterwards, and one made with kernel = 3 is refused. */
typedef struct pjzfdtd_batch pjzfdtd_batch;
int32_t pjzfdtd_batch_create(pjzfdtd_plan* const* plans, int32_t n,
                             pjzfdtd_batch** batch);
int32_t pjzfdtd_batch_workspace_bytes(const pjzfdtd_batch* batch, size_t* bytes);
/* buffers: one pjzfdtd_buffers per plan, in plan order. */
int32_t pjzfdtd_batch_run(pjzfdtd_batch* batch, const pjzfdtd_buffers* buffers,
                          void* workspace, size_t workspace_bytes,
                          int32_t use_graph, void* stream);
int32_t pjzfdtd_batch_destroy(pjzfdtd_batch* batch);

/* Forward solve without any device allocation by anyone: the scratch is a
   fixed 64 MiB array inside this library instead of a caller workspace.
   No counterpart in the reference (pjz/fdtdz receive scratch from XLA).
   For callers that cannot call cudaMalloc: a host whose device memory is
   owned by another runtime's pool (for example an XLA custom call that was
   given no scratch operand), or a real-time loop that must not risk the
   implicit device synchronisation cudaMalloc/cudaFree can cause.  Plans
   whose workspace (pjzfdtd_plan_workspace_bytes) exceeds 64 MiB are
   rejected with PJZFDTD_ERR_WORKSPACE.  Each call made outside a stream
   capture looks up the array's device address (cudaGetSymbolAddress) with
   the device current and caches it per device; a call during a capture
   uses the cached address, so make one call on each device before any
   stream capture.  All calls on a device share the one array and it keeps
   the last call's contents (each solve re-initialises what it needs);
   calls that overlap on the GPU, for example on two streams, race on it.
   Otherwise it behaves as pjzfdtd_forward (same plan, buffers and
   results). */
int32_t pjzfdtd_forward_static(pjzfdtd_plan* plan,
                               const pjzfdtd_buffers* buffers, void* stream);

/* pjzfdtd_plan_status for solves run by pjzfdtd_forward_static, whose status
   word lives in the library's static array rather than a caller workspace:
   PJZFDTD_ERR_TIMEOUT if a bounded device-side wait of the work queued on
   `stream` gave up (the word is then cleared), PJZFDTD_OK otherwise.
   Synchronises `stream`.  No counterpart in the reference. */
int32_t pjzfdtd_forward_static_status(pjzfdtd_plan* plan, void* stream);

/* Reads (and clears) the device status word of `workspace` after the work
   queued on `stream` so far: PJZFDTD_ERR_TIMEOUT if a bounded device-side
   wait gave up, PJZFDTD_OK otherwise.  Synchronises `stream`. */
int32_t pjzfdtd_plan_status(pjzfdtd_plan* plan, void* workspace,
                            size_t workspace_bytes, void* stream);

/* Launch geometry the plan resolved: tile_y, seg_x (0 until the first run
   picks it for the device), threads per CTA, time steps per pass, kernel
   variant (1 register-marching, 2 streamed) and streamed ring depth. */
int32_t pjzfdtd_plan_launch_config(const pjzfdtd_plan* plan, int32_t* tile_y,
                                   int32_t* seg_x, int32_t* threads,
                                   int32_t* steps_per_pass, int32_t* kernel,
                                   int32_t* stages);

/* Weighted port-plane sums of recorded phasors, for S-matrix entries:
   out[k][w] = sum_p (blocks[k][w][comps[k]][p] + i blocks[k][ww+w][comps[k]][p])
   * profiles[k][p], FP64 accumulation in a fixed order.  blocks[k] points at
   one monitor box of a PHASORS output, (2 ww, 3, npts[k]) floats (device);
   profiles[k]: device (npts[k]); out: device (nterms, ww, 2) doubles;
   1 <= nterms <= 64, ww <= 32.  Replaces the transverse-slice overlap sums
   of pjz's scatter (src/pjz/_field.py:305-338, 367-369) on the device.
   Stream-ordered, no workspace. */
int32_t pjzfdtd_plane_overlaps(int32_t nterms, const float* const* blocks,
                               const float* const* profiles,
                               const int32_t* comps, const int64_t* npts,
                               int32_t ww, double* out, void* stream);

/* dL/d-eps of a multi-port S-matrix objective from one batched launch:
   grad[t] = sum_w Re(q[w] sum_i forward_i,w[t] sum_j coef[i][j][w]
   adjoint_j,w[t]), FP64 sums, over `cells` = 3 x (design box) cells.
   forward[i] / adjoint[j]: device phasors (2 ww, cells) of forward solve i
   and unit-adjoint solve j (host arrays of n device pointers); coef: host
   (n, n, ww, 2) floats = conj(dL/dS_ij); q: host (ww, 2) floats; grad:
   device (cells).  n <= 16, ww <= 32, n*n*ww <= 1024.  Replaces the
   reciprocity residual product of pjz's scatter VJP
   (src/pjz/_field.py:380-398).  Stream-ordered, no workspace. */
int32_t pjzfdtd_smatrix_gradient(int32_t n, int32_t ww, int64_t cells,
                                 const float* const* forward,
                                 const float* const* adjoint, const float* coef,
                                 const float* q, float* grad, void* stream);

/* Permittivity of the Yee cell from magnified layer profiles: pjz's
   `epsilon(layers, interface_positions, magnification, zz,
   use_simple_averaging)` (src/pjz/_epsilon.py:104-155) on the GPU, so a
   design -> epsilon -> solve chain stays on the device.  `layers`: device
   (ll, 2m*xx, 2m*yy) float32 with 1 <= ll <= 16 (m = magnification);
   `interface_positions`: host, ll - 1 floats, increasing; `out`: device
   (3, xx, yy, zz) float32.  Stream-ordered, no workspace. */
int32_t pjzfdtd_render_epsilon(const float* layers, int32_t ll, int32_t xx,
                               int32_t yy, int32_t zz, int32_t magnification,
                               const float* interface_positions,
                               int32_t use_simple_averaging, float* out,
                               void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PJZFDTD_H_ */
