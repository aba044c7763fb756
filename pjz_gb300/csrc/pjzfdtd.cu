// Host side of the pjzfdtd C ABI (include/pjzfdtd.h): plan validation,
// CPML coefficient set-up, workspace layout and the time loop that launches
// the sm_103a step kernels.
//
// Replaces the fdtdz engine call of src/pjz/_field.py:254-269 and, in
// PHASORS mode, the pinv projection of src/pjz/_field.py:271-279 too.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/pjzfdtd.h"
#include "step_kernel.cuh"
#include "stream_kernel.cuh"
#include "record_kernel.cuh"

using namespace pjzfdtd;

namespace {

thread_local char g_err[512] = "";
thread_local int32_t g_err_code = PJZFDTD_OK;

int32_t fail(int32_t code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  g_err_code = code;
  return code;
}

#define CUDA_TRY(expr)                                                   \
  do {                                                                   \
    cudaError_t e_ = (expr);                                             \
    if (e_ != cudaSuccess)                                               \
      return fail(PJZFDTD_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_)); \
  } while (0)

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

}  // namespace

struct pjzfdtd_plan {
  pjzfdtd_problem p;
  int ns = 0;
  int P = 0;
  long long N = 0;
  std::vector<float> zc;       // [6][Z]
  std::vector<float> weights;  // [rows][ns]
  // Resolved launch geometry.
  int tile_y = 0, seg_x = 0, threads = 0, steps_per_pass = 1;
  int kernel = 1;   // 1 register-marching, 2 bulk-copy streamed
  int stages = 0;   // streamed ring depth
  size_t smem = 0;  // dynamic shared memory per CTA
  // Workspace layout (byte offsets).
  size_t off_fa = 0, off_fb = 0, off_cb = 0, off_pa = 0, off_pb = 0,
         off_zc = 0, off_comp = 0, off_comph = 0, off_status = 0, off_mask = 0,
         bytes = 0;
  int Pp = 0;  // PML state row stride (P rounded up to 4)
  int Yp = 0;  // padded y length of the streamed kernel's absorber copy
};

namespace {

void pml_coeff(double kappa, double sigma, double alpha, double dt, double* ik,
               double* b, double* c) {
  if (std::isinf(kappa)) {
    *ik = 0.0;
    *b = std::exp(-alpha * dt);
    *c = 0.0;
    return;
  }
  *ik = 1.0 / kappa;
  *b = std::exp(-(sigma / kappa + alpha) * dt);
  *c = (sigma == 0.0) ? 0.0
                      : sigma * (*b - 1.0) / (sigma * kappa + kappa * kappa * alpha);
}

int32_t validate(const pjzfdtd_problem& p) {
  if (p.xx <= 0 || p.yy <= 0 || p.zz <= 0)
    return fail(PJZFDTD_ERR_INVALID, "domain must be positive, got (%d, %d, %d)",
                p.xx, p.yy, p.zz);
  if (p.rx <= 0 || p.ry <= 0 || p.rz <= 0)
    return fail(PJZFDTD_ERR_INVALID, "epsilon shape must be positive");
  if (p.ox < 0 || p.oy < 0 || p.oz < 0 || p.ox + p.rx > p.xx ||
      p.oy + p.ry > p.yy || p.oz + p.rz > p.zz)
    return fail(PJZFDTD_ERR_INVALID,
                "epsilon (%d, %d, %d) at offset (%d, %d, %d) does not fit the "
                "(%d, %d, %d) domain",
                p.rx, p.ry, p.rz, p.ox, p.oy, p.oz, p.xx, p.yy, p.zz);
  if (p.tt < 0) return fail(PJZFDTD_ERR_INVALID, "tt must be >= 0");
  if (p.pml_lo < 0 || p.pml_hi < 0 || p.pml_lo + p.pml_hi > p.zz)
    return fail(PJZFDTD_ERR_INVALID, "pml_widths (%d, %d) do not fit zz=%d",
                p.pml_lo, p.pml_hi, p.zz);
  if (!(p.dt > 0.f) || !std::isfinite(p.dt))
    return fail(PJZFDTD_ERR_INVALID, "dt must be positive and finite");
  if (p.src_ncols < 0 || p.src_ncols > 64)
    return fail(PJZFDTD_ERR_INVALID, "source columns must be in [0, 64]");
  if (p.src_ncols > 0) {
    if (p.src_nx <= 0 || p.src_ny <= 0 || p.src_nz <= 0 || p.src_x0 < 0 ||
        p.src_y0 < 0 || p.src_z0 < 0 || p.src_x0 + p.src_nx > p.xx ||
        p.src_y0 + p.src_ny > p.yy || p.src_z0 + p.src_nz > p.zz)
      return fail(PJZFDTD_ERR_INVALID,
                  "source box (%d, %d, %d)+(%d, %d, %d) outside the domain",
                  p.src_x0, p.src_y0, p.src_z0, p.src_nx, p.src_ny, p.src_nz);
  }
  if (p.out_mode < PJZFDTD_OUT_NONE || p.out_mode > PJZFDTD_OUT_GRADIENT)
    return fail(PJZFDTD_ERR_INVALID, "unknown out_mode %d", p.out_mode);
  if (p.out_mode != PJZFDTD_OUT_NONE) {
    if (p.out_step <= 0)
      return fail(PJZFDTD_ERR_INVALID, "output step must be positive");
    // Steps before 0 are allowed (pjz asks for them when tt is short,
    // src/pjz/_field.py:216): the field there is the zero initial state.
    if (p.out_stop > p.tt || p.out_stop <= p.out_start)
      return fail(PJZFDTD_ERR_INVALID,
                  "output_steps (%d, %d, %d) must end within tt=%d",
                  p.out_start, p.out_stop, p.out_step, p.tt);
  }
  if (p.out_mode == PJZFDTD_OUT_PHASORS || p.out_mode == PJZFDTD_OUT_GRADIENT) {
    if (p.out_rows <= 0 || p.out_rows > kMaxRows)
      return fail(PJZFDTD_ERR_INVALID, "out_rows must be in [1, %d]", kMaxRows);
  }
  if (p.out_mode == PJZFDTD_OUT_GRADIENT) {
    if (p.grad_nx <= 0 || p.grad_ny <= 0 || p.grad_nz <= 0 || p.grad_x0 < 0 ||
        p.grad_y0 < 0 || p.grad_z0 < 0 || p.grad_x0 + p.grad_nx > p.xx ||
        p.grad_y0 + p.grad_ny > p.yy || p.grad_z0 + p.grad_nz > p.zz)
      return fail(PJZFDTD_ERR_INVALID, "gradient box outside the domain");
    if (p.record_h)
      return fail(PJZFDTD_ERR_INVALID, "record_h is not defined for GRADIENT");
  }
  if (p.tile_y < 0 || p.seg_x < 0 || p.steps_per_pass < 0)
    return fail(PJZFDTD_ERR_INVALID, "launch params must be >= 0");
  return PJZFDTD_OK;
}

constexpr size_t kSmemBudget = 220 * 1024;  // of the 227 KB per CTA
constexpr int kStreamThreads = 512;

// Streamed kernel: zz % 4 == 0, one compute thread per z-pair of a row,
// compute threads = (zz / 2) * rows-per-pass rounded up to whole warps, one
// extra producer warp, and a tile height whose ring fits shared memory.
int32_t resolve_stream(pjzfdtd_plan* pl) {
  const int Z = pl->p.zz;
  const int P = pl->p.pml_lo + pl->p.pml_hi;
  const int rpt = std::max(1, (kStreamThreads - 32) / (Z / 2));
  const int S = pl->p.stages > 0 ? pl->p.stages : 4;
  if (S < 2 || S > 8)
    return fail(PJZFDTD_ERR_INVALID, "stages must be in [2, 8], got %d", S);
  int ty = pl->p.tile_y;
  if (ty == 0) {
    int best = 0;
    for (int t = 1; t <= 64; ++t) {
      if (StreamGeom(t, Z, P).bytes(S) > kSmemBudget) break;
      // Prefer heights whose H rows split evenly over the row groups.
      if ((t + 1) % rpt == 0 || t + 1 < rpt || best == 0) best = t;
    }
    ty = std::min(best, pl->p.yy);
  }
  if (ty <= 0 || StreamGeom(ty, Z, P).bytes(S) > kSmemBudget)
    return fail(PJZFDTD_ERR_INVALID,
                "streamed tile (tile_y=%d, zz=%d, stages=%d) exceeds shared "
                "memory", ty, Z, S);
  pl->tile_y = ty;
  pl->stages = S;
  const int ncomp = ((Z / 2) * std::min(rpt, ty + 1) + 31) / 32 * 32;
  pl->threads = ncomp + 32;
  pl->smem = StreamGeom(ty, Z, P).bytes(S);
  pl->kernel = 2;
  return PJZFDTD_OK;
}

// Resolves the CTA tile.  Register-marching kernel: (tile_y + 2) * zz
// cells, one thread each, at most kMaxThreads threads.
int32_t resolve_tile(pjzfdtd_plan* pl) {
  const int Z = pl->p.zz;
  if (pl->p.kernel < 0 || pl->p.kernel > 2)
    return fail(PJZFDTD_ERR_INVALID, "unknown kernel %d", pl->p.kernel);
  const int zmax = 2 * (kStreamThreads - 32);
  if (pl->p.kernel == 2 && (Z % 4 != 0 || Z > zmax))
    return fail(PJZFDTD_ERR_INVALID,
                "the streamed kernel needs zz %% 4 == 0 and zz <= %d", zmax);
  if (pl->p.kernel == 2 || (pl->p.kernel == 0 && Z % 4 == 0 && Z <= zmax))
    return resolve_stream(pl);
  pl->kernel = 1;
  int ty = pl->p.tile_y;
  const int max_rows = kMaxThreads / Z;
  if (max_rows < 3)
    return fail(PJZFDTD_ERR_UNSUPPORTED,
                "zz=%d exceeds the thin-z limit of this kernel (zz <= %d)", Z,
                kMaxThreads / 3);
  if (ty == 0) ty = max_rows - 2;
  if (ty + 2 > max_rows)
    return fail(PJZFDTD_ERR_INVALID, "tile_y=%d too large for zz=%d (max %d)",
                ty, Z, max_rows - 2);
  pl->tile_y = ty;
  pl->threads = ((ty + 2) * Z + 31) / 32 * 32;
  pl->steps_per_pass = 1;
  pl->smem = 6 * (size_t)(ty + 2) * Z * sizeof(float);
  return PJZFDTD_OK;
}

void layout(pjzfdtd_plan* pl) {
  const pjzfdtd_problem& p = pl->p;
  const size_t N = (size_t)pl->N;
  pl->Pp = round4(pl->P);
  pl->Yp = round4(p.yy);
  const size_t XYP = (size_t)p.xx * p.yy * std::max(pl->Pp, 1);
  const size_t R = (size_t)p.rx * p.ry * p.rz;
  const size_t G = (size_t)p.grad_nx * p.grad_ny * p.grad_nz;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o = align256(o + bytes);
    return at;
  };
  pl->off_fa = take(6 * N * sizeof(float));
  pl->off_fb = take(6 * N * sizeof(float));
  pl->off_cb = take(3 * N * sizeof(float));
  pl->off_pa = take(4 * XYP * sizeof(float));
  pl->off_pb = take(4 * XYP * sizeof(float));
  pl->off_zc = take(6 * (size_t)p.zz * sizeof(float));
  size_t comp = 0;
  if (p.out_mode == PJZFDTD_OUT_PHASORS) comp = (size_t)p.out_rows * 3 * R;
  if (p.out_mode == PJZFDTD_OUT_GRADIENT) comp = 3 * G;
  pl->off_comp = take(std::max<size_t>(comp, 1) * sizeof(float));
  pl->off_comph = take(std::max<size_t>(p.record_h ? comp : 0, 1) * sizeof(float));
  pl->off_status = take(sizeof(int));
  pl->off_mask = take((pl->kernel == 2 ? (size_t)p.xx * 3 * pl->Yp : 1) * sizeof(float));
  pl->bytes = o;
}

cudaError_t set_stream_smem(size_t bytes) {
  return cudaFuncSetAttribute(yee_stream_kernel,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)bytes);
}

int32_t resolve_seg_x(pjzfdtd_plan* pl) {
  if (pl->seg_x > 0) return PJZFDTD_OK;
  if (pl->p.seg_x > 0) {
    pl->seg_x = pl->p.seg_x;
    return PJZFDTD_OK;
  }
  int dev = 0, sms = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int per_sm = 1;
  if (pl->kernel == 2) {
    CUDA_TRY(set_stream_smem(pl->smem));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, yee_stream_kernel, pl->threads, pl->smem));
  } else {
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, yee_step_kernel, pl->threads, pl->smem));
  }
  per_sm = std::max(per_sm, 1);
  const int tiles_y = (pl->p.yy + pl->tile_y - 1) / pl->tile_y;
  const int slots = sms * per_sm;
  int nseg = std::max(1, slots / tiles_y);
  int seg = (pl->p.xx + nseg - 1) / nseg;
  seg = std::max(seg, std::min(pl->p.xx, 8));  // keep the halo plane cheap
  pl->seg_x = seg;
  return PJZFDTD_OK;
}

template <typename T>
T* at(void* ws, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(ws) + off);
}

int32_t check_buffers(const pjzfdtd_plan* pl, const pjzfdtd_buffers* b,
                      void* ws, size_t ws_bytes) {
  if (!b) return fail(PJZFDTD_ERR_INVALID, "buffers is NULL");
  if (!ws || ws_bytes < pl->bytes)
    return fail(PJZFDTD_ERR_WORKSPACE, "workspace of %zu bytes needed, got %zu",
                pl->bytes, ws ? ws_bytes : (size_t)0);
  if (reinterpret_cast<uintptr_t>(ws) % 256)
    return fail(PJZFDTD_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  if (!b->epsilon || !b->absorption_mask)
    return fail(PJZFDTD_ERR_INVALID, "epsilon and absorption_mask are required");
  if (pl->p.src_ncols > 0 && (!b->source || !b->waveform))
    return fail(PJZFDTD_ERR_INVALID, "source and waveform are required");
  if (pl->p.out_mode != PJZFDTD_OUT_NONE && !b->out)
    return fail(PJZFDTD_ERR_INVALID, "out is required for this out_mode");
  if (pl->p.record_h && !b->out_h)
    return fail(PJZFDTD_ERR_INVALID, "out_h is required when record_h is set");
  if (pl->p.out_mode == PJZFDTD_OUT_GRADIENT && !b->q)
    return fail(PJZFDTD_ERR_INVALID, "q is required for GRADIENT");
  return PJZFDTD_OK;
}

int32_t run_range(pjzfdtd_plan* pl, const pjzfdtd_buffers* b, void* ws,
                  size_t ws_bytes, int n0, int n1, cudaStream_t st) {
  int32_t rc = check_buffers(pl, b, ws, ws_bytes);
  if (rc) return rc;
  if (n0 < 0 || n1 > pl->p.tt || n0 > n1)
    return fail(PJZFDTD_ERR_INVALID, "step range [%d, %d) outside [0, %d)", n0,
                n1, pl->p.tt);
  rc = resolve_seg_x(pl);
  if (rc) return rc;
  const pjzfdtd_problem& p = pl->p;
  const long long N = pl->N;
  const size_t XYP = (size_t)p.xx * p.yy * std::max(pl->Pp, 1);
  float* fa = at<float>(ws, pl->off_fa);
  float* fb = at<float>(ws, pl->off_fb);
  float* cb = at<float>(ws, pl->off_cb);
  float* pa = at<float>(ws, pl->off_pa);
  float* pb = at<float>(ws, pl->off_pb);
  float* zc = at<float>(ws, pl->off_zc);
  float* comp = at<float>(ws, pl->off_comp);
  float* comph = at<float>(ws, pl->off_comph);
  const size_t R = (size_t)p.rx * p.ry * p.rz;
  const size_t G = (size_t)p.grad_nx * p.grad_ny * p.grad_nz;

  if (n0 == 0) {
    if (p.out_mode == PJZFDTD_OUT_SNAPSHOTS && p.out_start < 0) {
      const size_t n = (size_t)pl->ns * 3 * R * sizeof(float);
      CUDA_TRY(cudaMemsetAsync(b->out, 0, n, st));
      if (p.record_h) CUDA_TRY(cudaMemsetAsync(b->out_h, 0, n, st));
    }
    CUDA_TRY(cudaMemcpyAsync(zc, pl->zc.data(), pl->zc.size() * sizeof(float),
                             cudaMemcpyHostToDevice, st));
    if (b->fields)
      CUDA_TRY(cudaMemcpyAsync(fa, b->fields, 6 * N * sizeof(float),
                               cudaMemcpyDeviceToDevice, st));
    else
      CUDA_TRY(cudaMemsetAsync(fa, 0, 6 * N * sizeof(float), st));
    CUDA_TRY(cudaMemsetAsync(pa, 0, 4 * XYP * sizeof(float), st));
    CUDA_TRY(cudaMemsetAsync(pb, 0, 4 * XYP * sizeof(float), st));
    if (p.out_mode == PJZFDTD_OUT_PHASORS) {
      const size_t n = (size_t)p.out_rows * 3 * R * sizeof(float);
      CUDA_TRY(cudaMemsetAsync(b->out, 0, n, st));
      CUDA_TRY(cudaMemsetAsync(comp, 0, n, st));
      if (p.record_h) {
        CUDA_TRY(cudaMemsetAsync(b->out_h, 0, n, st));
        CUDA_TRY(cudaMemsetAsync(comph, 0, n, st));
      }
    }
    if (p.out_mode == PJZFDTD_OUT_GRADIENT) {
      CUDA_TRY(cudaMemsetAsync(b->out, 0, 3 * G * sizeof(float), st));
      CUDA_TRY(cudaMemsetAsync(comp, 0, 3 * G * sizeof(float), st));
    }
    const int threads = 256;
    const long long total = 3 * N;
    const int blocks = (int)std::min<long long>((total + threads - 1) / threads, 1 << 20);
    precompute_cb_kernel<<<blocks, threads, 0, st>>>(
        b->epsilon, b->absorption_mask, cb, p.xx, p.yy, p.zz, p.ox, p.oy, p.oz,
        p.rx, p.ry, p.rz, p.dt);
    CUDA_TRY(cudaGetLastError());
    if (pl->kernel == 2) {
      const long long nm = (long long)p.xx * 3 * pl->Yp;
      pad_mask_kernel<<<(int)std::min<long long>((nm + 255) / 256, 1 << 16), 256, 0,
                        st>>>(b->absorption_mask, at<float>(ws, pl->off_mask),
                              p.xx, p.yy, pl->Yp);
      CUDA_TRY(cudaGetLastError());
    }
  }

  StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.X = p.xx;
  a.Y = p.yy;
  a.Z = p.zz;
  a.P = pl->P;
  a.Pst = std::max(pl->Pp, 1);
  a.plo = p.pml_lo;
  a.phi = p.pml_hi;
  a.N = N;
  a.dt = p.dt;
  a.tile_y = pl->tile_y;
  a.seg_x = pl->seg_x;
  a.cb = cb;
  a.mask = b->absorption_mask;
  a.zc = zc;
  a.sx0 = p.src_x0;
  a.sy0 = p.src_y0;
  a.sz0 = p.src_z0;
  a.snx = p.src_ncols > 0 ? p.src_nx : 0;
  a.sny = p.src_ncols > 0 ? p.src_ny : 0;
  a.snz = p.src_ncols > 0 ? p.src_nz : 0;
  a.snc = p.src_ncols;
  a.src = b->source;

  const dim3 grid((p.yy + pl->tile_y - 1) / pl->tile_y,
                  (p.xx + pl->seg_x - 1) / pl->seg_x);
  const size_t smem = pl->smem;
  int* status = at<int>(ws, pl->off_status);
  if (n0 == 0) CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
  if (pl->kernel == 2) CUDA_TRY(set_stream_smem(smem));
  RecordArgs ra;
  std::memset(&ra, 0, sizeof(ra));
  ra.N = N;
  ra.X = p.xx;
  ra.Y = p.yy;
  ra.Z = p.zz;
  if (p.out_mode == PJZFDTD_OUT_GRADIENT) {
    ra.bx0 = p.grad_x0; ra.by0 = p.grad_y0; ra.bz0 = p.grad_z0;
    ra.bnx = p.grad_nx; ra.bny = p.grad_ny; ra.bnz = p.grad_nz;
  } else {
    ra.bx0 = p.ox; ra.by0 = p.oy; ra.bz0 = p.oz;
    ra.bnx = p.rx; ra.bny = p.ry; ra.bnz = p.rz;
  }
  ra.record_h = p.record_h;
  ra.out = b->out;
  ra.out_h = b->out_h;
  ra.comp = comp;
  ra.comp_h = comph;
  ra.rows = p.out_rows;
  ra.q = b->q;
  StreamArgs sa;
  sa.stages = pl->stages;
  sa.status = status;
  sa.Yp = pl->Yp;
  sa.mask_ws = at<float>(ws, pl->off_mask);
  for (int n = n0; n < n1; ++n) {
    const bool even = (n % 2) == 0;
    a.fin = even ? fa : fb;
    a.fout = even ? fb : fa;
    a.psi_in = even ? pa : pb;
    a.psi_out = even ? pb : pa;
    a.wave = p.src_ncols > 0 ? b->waveform + (size_t)n * p.src_ncols : nullptr;
    if (pl->kernel == 2) {
      sa.s = a;
      yee_stream_kernel<<<grid, pl->threads, smem, st>>>(sa);
    } else {
      yee_step_kernel<<<grid, pl->threads, smem, st>>>(a);
    }
    CUDA_TRY(cudaGetLastError());
    if (p.out_mode != PJZFDTD_OUT_NONE && n >= p.out_start && n < p.out_stop &&
        (n - p.out_start) % p.out_step == 0) {
      const int j = (n - p.out_start) / p.out_step;
      ra.f = a.fout;
      if (p.out_mode == PJZFDTD_OUT_SNAPSHOTS) {
        ra.out = b->out + (size_t)j * 3 * R;
        ra.out_h = p.record_h ? b->out_h + (size_t)j * 3 * R : nullptr;
      } else {
        for (int r = 0; r < p.out_rows; ++r)
          ra.w[r] = pl->weights[(size_t)r * pl->ns + j];
      }
      const long long nb = (long long)ra.bnx * ra.bny * ra.bnz;
      const int rblocks = (int)std::min<long long>((nb + 255) / 256, 1 << 20);
      switch (p.out_mode) {
        case PJZFDTD_OUT_SNAPSHOTS:
          record_kernel<kRecSnap><<<rblocks, 256, 0, st>>>(ra);
          break;
        case PJZFDTD_OUT_PHASORS:
          record_kernel<kRecProj><<<rblocks, 256, 0, st>>>(ra);
          break;
        default:
          record_kernel<kRecGrad><<<rblocks, 256, 0, st>>>(ra);
          break;
      }
      CUDA_TRY(cudaGetLastError());
    }
  }
  if (n1 == p.tt && b->fields) {
    float* fin = (p.tt % 2 == 0) ? fa : fb;
    CUDA_TRY(cudaMemcpyAsync(b->fields, fin, 6 * N * sizeof(float),
                             cudaMemcpyDeviceToDevice, st));
  }
  return PJZFDTD_OK;
}

}  // namespace

extern "C" {

int32_t pjzfdtd_abi_version(void) { return PJZFDTD_ABI_VERSION; }

int32_t pjzfdtd_last_error(char* buf, size_t len) {
  if (buf && len) {
    std::strncpy(buf, g_err, len - 1);
    buf[len - 1] = 0;
  }
  return g_err_code;
}

int32_t pjzfdtd_plan_create(const pjzfdtd_problem* problem,
                            const float* pml_kappa, const float* pml_sigma,
                            const float* pml_alpha, const float* weights,
                            pjzfdtd_plan** plan) {
  if (!problem || !plan) return fail(PJZFDTD_ERR_INVALID, "NULL argument");
  *plan = nullptr;
  int32_t rc = validate(*problem);
  if (rc) return rc;
  if (!pml_kappa || !pml_sigma || !pml_alpha)
    return fail(PJZFDTD_ERR_INVALID, "pml_kappa/sigma/alpha are required");
  pjzfdtd_plan* pl = new (std::nothrow) pjzfdtd_plan();
  if (!pl) return fail(PJZFDTD_ERR_INVALID, "out of host memory");
  pl->p = *problem;
  const pjzfdtd_problem& p = pl->p;
  pl->N = (long long)p.xx * p.yy * p.zz;
  pl->P = p.pml_lo + p.pml_hi;
  pl->ns = (p.out_mode != PJZFDTD_OUT_NONE && p.out_stop > p.out_start)
               ? (p.out_stop - p.out_start + p.out_step - 1) / p.out_step
               : 0;
  pl->zc.assign(6 * (size_t)p.zz, 0.f);
  for (int z = 0; z < p.zz; ++z)
    for (int col = 0; col < 2; ++col) {
      const double k = pml_kappa[2 * z + col], s = pml_sigma[2 * z + col],
                   al = pml_alpha[2 * z + col];
      if (!(k > 0.0) || !(s >= 0.0) || !(al >= 0.0) || std::isnan(k) ||
          std::isinf(s) || std::isinf(al)) {
        delete pl;
        return fail(PJZFDTD_ERR_INVALID,
                    "pml coefficients at z=%d column %d must have kappa > 0 "
                    "(inf allowed), finite sigma >= 0, alpha >= 0",
                    z, col);
      }
      double ik, b, c;
      pml_coeff(k, s, al, (double)p.dt, &ik, &b, &c);
      pl->zc[(3 * col + 0) * p.zz + z] = (float)ik;
      pl->zc[(3 * col + 1) * p.zz + z] = (float)b;
      pl->zc[(3 * col + 2) * p.zz + z] = (float)c;
    }
  if (p.out_mode == PJZFDTD_OUT_PHASORS || p.out_mode == PJZFDTD_OUT_GRADIENT) {
    if (!weights) {
      delete pl;
      return fail(PJZFDTD_ERR_INVALID, "weights are required for this out_mode");
    }
    pl->weights.assign(weights, weights + (size_t)p.out_rows * pl->ns);
  }
  rc = resolve_tile(pl);
  if (rc) {
    delete pl;
    return rc;
  }
  layout(pl);
  *plan = pl;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plan_workspace_bytes(const pjzfdtd_plan* plan, size_t* bytes) {
  if (!plan || !bytes) return fail(PJZFDTD_ERR_INVALID, "NULL argument");
  *bytes = plan->bytes;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plan_num_samples(const pjzfdtd_plan* plan, int32_t* ns) {
  if (!plan || !ns) return fail(PJZFDTD_ERR_INVALID, "NULL argument");
  *ns = plan->ns;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plan_launch_config(const pjzfdtd_plan* plan, int32_t* tile_y,
                                   int32_t* seg_x, int32_t* threads,
                                   int32_t* steps_per_pass, int32_t* kernel,
                                   int32_t* stages) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  if (tile_y) *tile_y = plan->tile_y;
  if (seg_x) *seg_x = plan->seg_x > 0 ? plan->seg_x : plan->p.seg_x;
  if (threads) *threads = plan->threads;
  if (steps_per_pass) *steps_per_pass = plan->steps_per_pass;
  if (kernel) *kernel = plan->kernel;
  if (stages) *stages = plan->stages;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plan_status(pjzfdtd_plan* plan, void* workspace,
                            size_t workspace_bytes, void* stream) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  if (!workspace || workspace_bytes < plan->bytes)
    return fail(PJZFDTD_ERR_WORKSPACE, "workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int* dev = at<int>(workspace, plan->off_status);
  int host = 0;
  CUDA_TRY(cudaMemcpyAsync(&host, dev, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (host != 0) {
    CUDA_TRY(cudaMemsetAsync(dev, 0, sizeof(int), st));
    return fail(PJZFDTD_ERR_TIMEOUT,
                "a device-side wait exceeded its limit (status %d)", host);
  }
  return PJZFDTD_OK;
}

int32_t pjzfdtd_plan_destroy(pjzfdtd_plan* plan) {
  delete plan;
  return PJZFDTD_OK;
}

int32_t pjzfdtd_forward(pjzfdtd_plan* plan, const pjzfdtd_buffers* buffers,
                        void* workspace, size_t workspace_bytes, void* stream) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  if (plan->p.out_mode == PJZFDTD_OUT_GRADIENT)
    return fail(PJZFDTD_ERR_INVALID, "GRADIENT plans run through pjzfdtd_adjoint");
  return run_range(plan, buffers, workspace, workspace_bytes, 0, plan->p.tt,
                   static_cast<cudaStream_t>(stream));
}

int32_t pjzfdtd_adjoint(pjzfdtd_plan* plan, const pjzfdtd_buffers* buffers,
                        void* workspace, size_t workspace_bytes, void* stream) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  if (plan->p.out_mode != PJZFDTD_OUT_GRADIENT)
    return fail(PJZFDTD_ERR_INVALID, "pjzfdtd_adjoint needs a GRADIENT plan");
  return run_range(plan, buffers, workspace, workspace_bytes, 0, plan->p.tt,
                   static_cast<cudaStream_t>(stream));
}

int32_t pjzfdtd_run_steps(pjzfdtd_plan* plan, const pjzfdtd_buffers* buffers,
                          void* workspace, size_t workspace_bytes,
                          int32_t step_begin, int32_t step_end, void* stream) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  return run_range(plan, buffers, workspace, workspace_bytes, step_begin,
                   step_end, static_cast<cudaStream_t>(stream));
}

}  // extern "C"

// Scratch for pjzfdtd_forward_static: a fixed device array, so a caller
// that may not allocate device memory can still run a forward solve.  Every
// GPU that loads this library holds it until the process exits.  All calls
// on a device share it and it keeps the last call's contents; the forward
// solve clears what must start at zero (fields, PML state, accumulators,
// status word) at its first step.
namespace {
constexpr size_t kStaticScratchBytes = size_t(64) << 20;  // 64 MiB
constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
void* g_static_ptr[kMaxDevices] = {};
}  // namespace

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

extern "C" {

int32_t pjzfdtd_forward_static(pjzfdtd_plan* plan,
                               const pjzfdtd_buffers* buffers, void* stream) {
  if (!plan) return fail(PJZFDTD_ERR_INVALID, "NULL plan");
  if (plan->p.out_mode == PJZFDTD_OUT_GRADIENT)
    return fail(PJZFDTD_ERR_INVALID, "GRADIENT plans run through pjzfdtd_adjoint");
  if (plan->bytes > kStaticScratchBytes)
    return fail(PJZFDTD_ERR_WORKSPACE,
                "this plan needs %zu bytes of scratch; pjzfdtd_forward_static "
                "has a fixed %zu-byte (64 MiB) array -- use pjzfdtd_forward "
                "with a caller-allocated workspace",
                plan->bytes, kStaticScratchBytes);
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return fail(PJZFDTD_ERR_UNSUPPORTED, "device %d beyond %d", dev, kMaxDevices);
  void* scratch = nullptr;
  {
    // Once per device, with that device current: the host cannot use the
    // array's symbol as a device address, so resolve the real one.
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[dev]) {
      void* p = nullptr;
      CUDA_TRY(cudaGetSymbolAddress(&p, g_static_scratch));
      g_static_ptr[dev] = p;
    }
    scratch = g_static_ptr[dev];
  }
  return run_range(plan, buffers, scratch, kStaticScratchBytes, 0, plan->p.tt,
                   static_cast<cudaStream_t>(stream));
}

}  // extern "C"
