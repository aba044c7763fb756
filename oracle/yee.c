/*
 * CPU oracle for the FDTD engine that pjz calls (test infrastructure only).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, and only as the checker; the product library never links it.
 *
 * The engine pjz drives is fdtdz (`fdtdz_jax.fdtdz`, called at
 * src/pjz/_field.py:254-269; dependency `fdtdz>=1.1.3`, setup.py:26).  Its
 * source is not part of the reference tree, so this file restates the
 * published Yee/CPML algorithm under the conventions pjz's own code fixes:
 *   - Yee staggering Ex(x+1/2,y,z), Ey(x,y+1/2,z), Ez(x,y,z+1/2)
 *     (src/pjz/_epsilon.py:10-25, 139-155: the z component uses the
 *     half-integer grid column);
 *   - E from backward differences of H, H from forward differences of E
 *     (src/pjz/_mode.py:15-19, 61-68, 92-96);
 *   - absorption_mask (3,X,Y) is a conductivity on E component c
 *     (src/pjz/_field.py:69-90, 239-241);
 *   - z-CPML with (kappa, sigma, alpha) columns 0 (integer z, E update) and
 *     1 (half-integer z, H update) (src/pjz/_field.py:98-106, 243-251);
 *     kappa = inf decouples z-layers (use_z_as_batch, :243-246);
 *   - epsilon (3,rx,ry,rz) sits at `offset` inside the domain and is
 *     edge-extended outside (src/pjz/_field.py:199-202, 268);
 *   - x/y-normal plane sources inject waveform column 0 at `source_position`
 *     and column 1 at `source_position - 1`, so pjz's even-position bump with
 *     column flip (src/pjz/_field.py:230-233) keeps the source plane; z-normal
 *     sources carry one profile per column at the same plane (:234-236);
 *   - E is recorded after the update of each step in
 *     range(*output_steps) (src/pjz/_field.py:214-216, 271-279).
 * The update arithmetic is therefore "parity unpinned" against fdtdz itself.
 *
 * Every floating-point operation is written out (fmaf / add / sub / mul in a
 * fixed order, built with -ffp-contract=off) so that the FP32 build performs
 * the same IEEE operations as the CUDA kernels; the FP64 build (REAL=double)
 * is the higher-precision reference the FP32 error is stated against.
 *
 * Reduced-precision storage (storage = 1, FP32 build only) restates pjz's
 * use_reduced_precision (src/pjz/_field.py:52) as 16-bit IEEE storage with
 * FP32 arithmetic: every stored E, H and CPML state value and the E-update
 * coefficient cb are rounded to binary16 (round to nearest even) when
 * written; reads widen them exactly; the update in between, the source sums
 * and the phasor accumulators stay FP32.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef REAL
#define REAL float
#define FMA fmaf
#define SUFFIX(name) name##_f32
/* FP32: coefficients are rounded to float exactly as the engine does. */
#define COEF(v) ((REAL)(float)(v))
#define STORE(v) (half ? (REAL)round_f16((float)(v)) : (v))
#define ORACLE_F32 1
#else
#define FMA fma
#define SUFFIX(name) name##_f64
#define COEF(v) ((REAL)(v))
#define STORE(v) (v)
#endif

typedef struct {
  int32_t xx, yy, zz;          /* simulation domain, cells */
  int32_t ox, oy, oz;          /* offset of the epsilon / output region */
  int32_t rx, ry, rz;          /* epsilon / output region shape */
  int32_t tt;                  /* time steps */
  int32_t pml_lo, pml_hi;      /* z-PML slab widths (psi storage) */
  float dt;
  int32_t sx0, sy0, sz0;       /* source box origin */
  int32_t snx, sny, snz, snc;  /* source box shape, waveform columns */
  int32_t out_start, out_stop, out_step;
  int32_t mode;                /* 0 none, 1 snapshots, 2 projection, 3 gradient */
  int32_t nrows;               /* rows of the sample weights (2 * ww) */
  int32_t record_h;            /* also record H (modes 1 and 2) */
  int32_t gx0, gy0, gz0, gnx, gny, gnz; /* gradient box (mode 3) */
  int32_t nthreads;
  int32_t storage;             /* 0 FP32, 1 binary16 (FP32 build only) */
} oracle_problem;

/* Rounds v to binary16 (round to nearest even, subnormals kept) and back. */
static inline float round_f16(float v) { return (float)(_Float16)v; }

#ifdef ORACLE_F32
float oracle_round_f16(float v) { return round_f16(v); }
#endif

static void pml_coeff(double kappa, double sigma, double alpha, double dt,
                      double* ik, double* b, double* c) {
  if (isinf(kappa)) {
    *ik = 0.0;
    *b = exp(-alpha * dt);
    *c = 0.0;
    return;
  }
  *ik = 1.0 / kappa;
  *b = exp(-(sigma / kappa + alpha) * dt);
  *c = (sigma == 0.0) ? 0.0
                      : sigma * (*b - 1.0) / (sigma * kappa + kappa * kappa * alpha);
}

static inline void kahan(REAL* s, REAL* c, REAL w, REAL e) {
  REAL y = FMA(w, e, -*c);
  REAL t = *s + y;
  *c = (t - *s) - y;
  *s = t;
}

static inline int clampi(int v, int lo, int hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

int SUFFIX(oracle_run)(const oracle_problem* p, const float* eps,
                       const float* mask, const float* kappa,
                       const float* sigma, const float* alpha,
                       const float* src, const float* wave,
                       const float* weights, const float* q, REAL* fields,
                       REAL* out, REAL* out_h) {
  const int X = p->xx, Y = p->yy, Z = p->zz;
  const long YZ = (long)Y * Z, N = (long)X * YZ;
  const int P = p->pml_lo + p->pml_hi;
  const long R = (long)p->rx * p->ry * p->rz;
  const long G = (long)p->gnx * p->gny * p->gnz;
  const REAL dt = (REAL)p->dt;
  const REAL hdt = (REAL)(0.5f * p->dt);
  const int half = p->storage == 1;
  (void)half;
  if (X <= 0 || Y <= 0 || Z <= 0 || Z > 4096 || P > Z || p->rx <= 0 ||
      p->ry <= 0 || p->rz <= 0)
    return 1;
#ifdef _OPENMP
  if (p->nthreads > 0) omp_set_num_threads(p->nthreads);
#endif

  REAL* F = fields ? fields : (REAL*)calloc(6 * N, sizeof(REAL));
  if (fields)
    for (long i = 0; i < 6 * N; ++i) F[i] = STORE(F[i]);
  REAL* cb = (REAL*)malloc(3 * N * sizeof(REAL));
  REAL* psi = (REAL*)calloc(4 * (size_t)X * Y * (P > 0 ? P : 1), sizeof(REAL));
  REAL* zc = (REAL*)malloc(6 * (size_t)Z * sizeof(REAL));
  long acc_n = 0;
  if (p->mode == 2) acc_n = (long)p->nrows * 3 * R * (p->record_h ? 2 : 1);
  if (p->mode == 3) acc_n = 3 * G;
  REAL* comp = (REAL*)calloc(acc_n > 0 ? acc_n : 1, sizeof(REAL));
  if (p->mode == 2) {
    memset(out, 0, (size_t)p->nrows * 3 * R * sizeof(REAL));
    if (p->record_h) memset(out_h, 0, (size_t)p->nrows * 3 * R * sizeof(REAL));
  }
  if (p->mode == 3) memset(out, 0, 3 * G * sizeof(REAL));

  /* Per-z CPML coefficients: [ik_e, b_e, c_e, ik_h, b_h, c_h][z]. */
  for (int z = 0; z < Z; ++z)
    for (int col = 0; col < 2; ++col) {
      double ik, b, c;
      pml_coeff(kappa[2 * z + col], sigma[2 * z + col], alpha[2 * z + col],
                (double)p->dt, &ik, &b, &c);
      zc[(3 * col + 0) * Z + z] = COEF(ik);
      zc[(3 * col + 1) * Z + z] = COEF(b);
      zc[(3 * col + 2) * Z + z] = COEF(c);
    }

  /* E-update coefficient cb = dt / (eps + sigma * dt / 2). */
  for (int c = 0; c < 3; ++c)
    for (int x = 0; x < X; ++x)
      for (int y = 0; y < Y; ++y) {
        const REAL s = (REAL)mask[((long)c * X + x) * Y + y];
        const int ex = clampi(x - p->ox, 0, p->rx - 1);
        const int ey = clampi(y - p->oy, 0, p->ry - 1);
        for (int z = 0; z < Z; ++z) {
          const int ez = clampi(z - p->oz, 0, p->rz - 1);
          const REAL e = (REAL)eps[(((long)c * p->rx + ex) * p->ry + ey) * p->rz + ez];
          cb[c * N + (x * (long)Y + y) * Z + z] = STORE(dt / FMA(s, hdt, e));
        }
      }

  REAL *Ex = F, *Ey = F + N, *Ez = F + 2 * N;
  REAL *Hx = F + 3 * N, *Hy = F + 4 * N, *Hz = F + 5 * N;
  REAL *phx = psi, *phy = psi + (long)X * Y * P;
  REAL *pex = psi + 2L * X * Y * P, *pey = psi + 3L * X * Y * P;
  const REAL *ike = zc, *be = zc + Z, *ce = zc + 2 * Z;
  const REAL *ikh = zc + 3 * Z, *bh = zc + 4 * Z, *ch = zc + 5 * Z;
  const int plo = p->pml_lo, phi = p->pml_hi;
  const int ns = (p->out_step > 0 && p->out_stop > p->out_start)
                     ? (p->out_stop - p->out_start + p->out_step - 1) / p->out_step
                     : 0;

  for (int n = 0; n < p->tt; ++n) {
    /* H^{n+1/2} from E^n. */
#pragma omp parallel for schedule(static)
    for (int x = 0; x < X; ++x)
      for (int y = 0; y < Y; ++y)
        for (int z = 0; z < Z; ++z) {
          const long i = (x * (long)Y + y) * Z + z;
          const REAL ex = Ex[i], ey = Ey[i], ez = Ez[i];
          const REAL ex_y1 = (y + 1 < Y) ? Ex[i + Z] : (REAL)0;
          const REAL ez_y1 = (y + 1 < Y) ? Ez[i + Z] : (REAL)0;
          const REAL ex_z1 = (z + 1 < Z) ? Ex[i + 1] : (REAL)0;
          const REAL ey_z1 = (z + 1 < Z) ? Ey[i + 1] : (REAL)0;
          const REAL ey_x1 = (x + 1 < X) ? Ey[i + YZ] : (REAL)0;
          const REAL ez_x1 = (x + 1 < X) ? Ez[i + YZ] : (REAL)0;
          const REAL dEz_y = ez_y1 - ez, dEy_z = ey_z1 - ey;
          const REAL dEx_z = ex_z1 - ex, dEz_x = ez_x1 - ez;
          const REAL dEy_x = ey_x1 - ey, dEx_y = ex_y1 - ex;
          REAL zEy, zEx;
          const int pz = z < plo ? z : (z >= Z - phi ? z - (Z - phi) + plo : -1);
          if (pz >= 0) {
            const long pi = (x * (long)Y + y) * P + pz;
            const REAL a = FMA(ch[z], dEy_z, bh[z] * phx[pi]);
            const REAL b = FMA(ch[z], dEx_z, bh[z] * phy[pi]);
            phx[pi] = STORE(a);
            phy[pi] = STORE(b);
            zEy = FMA(dEy_z, ikh[z], a);
            zEx = FMA(dEx_z, ikh[z], b);
          } else {
            zEy = dEy_z * ikh[z];
            zEx = dEx_z * ikh[z];
          }
          Hx[i] = STORE(FMA(-dt, dEz_y - zEy, Hx[i]));
          Hy[i] = STORE(FMA(-dt, zEx - dEz_x, Hy[i]));
          Hz[i] = STORE(FMA(-dt, dEy_x - dEx_y, Hz[i]));
        }

    /* E^{n+1} from H^{n+1/2}, source column values of step n. */
    const float* w = wave + (long)n * p->snc;
#pragma omp parallel for schedule(static)
    for (int x = 0; x < X; ++x)
      for (int y = 0; y < Y; ++y)
        for (int z = 0; z < Z; ++z) {
          const long i = (x * (long)Y + y) * Z + z;
          const REAL hx = Hx[i], hy = Hy[i], hz = Hz[i];
          const REAL hz_ym = (y > 0) ? Hz[i - Z] : (REAL)0;
          const REAL hx_ym = (y > 0) ? Hx[i - Z] : (REAL)0;
          const REAL hy_zm = (z > 0) ? Hy[i - 1] : (REAL)0;
          const REAL hx_zm = (z > 0) ? Hx[i - 1] : (REAL)0;
          const REAL hz_xm = (x > 0) ? Hz[i - YZ] : (REAL)0;
          const REAL hy_xm = (x > 0) ? Hy[i - YZ] : (REAL)0;
          const REAL dHz_y = hz - hz_ym, dHy_z = hy - hy_zm;
          const REAL dHx_z = hx - hx_zm, dHz_x = hz - hz_xm;
          const REAL dHy_x = hy - hy_xm, dHx_y = hx - hx_ym;
          REAL zHy, zHx;
          const int pz = z < plo ? z : (z >= Z - phi ? z - (Z - phi) + plo : -1);
          if (pz >= 0) {
            const long pi = (x * (long)Y + y) * P + pz;
            const REAL a = FMA(ce[z], dHy_z, be[z] * pex[pi]);
            const REAL b = FMA(ce[z], dHx_z, be[z] * pey[pi]);
            pex[pi] = STORE(a);
            pey[pi] = STORE(b);
            zHy = FMA(dHy_z, ike[z], a);
            zHx = FMA(dHx_z, ike[z], b);
          } else {
            zHy = dHy_z * ike[z];
            zHx = dHx_z * ike[z];
          }
          REAL cur[3] = {dHz_y - zHy, zHx - dHz_x, dHy_x - dHx_y};
          const int lx = x - p->sx0, ly = y - p->sy0, lz = z - p->sz0;
          if (lx >= 0 && lx < p->snx && ly >= 0 && ly < p->sny && lz >= 0 &&
              lz < p->snz) {
            const long sb = ((long)p->snx * p->sny) * p->snz;
            const long si = ((long)lx * p->sny + ly) * p->snz + lz;
            for (int c = 0; c < 3; ++c) {
              REAL j = 0;
              for (int k = 0; k < p->snc; ++k)
                j = FMA((REAL)src[((long)k * 3 + c) * sb + si], (REAL)w[k], j);
              cur[c] = cur[c] - j;
            }
          }
          for (int c = 0; c < 3; ++c) {
            REAL* E = F + c * N;
            const REAL s = (REAL)mask[((long)c * X + x) * Y + y];
            const REAL r = FMA(-s, E[i], cur[c]);
            E[i] = STORE(FMA(cb[c * N + i], r, E[i]));
          }
        }

    /* Record E^{n+1} (and H^{n+1/2}) at the output steps. */
    if (ns > 0 && n >= p->out_start && n < p->out_stop &&
        (n - p->out_start) % p->out_step == 0 && p->mode != 0) {
      const int j = (n - p->out_start) / p->out_step;
#pragma omp parallel for schedule(static)
      for (int x = 0; x < X; ++x)
        for (int y = 0; y < Y; ++y)
          for (int z = 0; z < Z; ++z) {
            const long i = (x * (long)Y + y) * Z + z;
            if (p->mode == 3) {
              const int gx = x - p->gx0, gy = y - p->gy0, gz = z - p->gz0;
              if (gx < 0 || gx >= p->gnx || gy < 0 || gy >= p->gny || gz < 0 ||
                  gz >= p->gnz)
                continue;
              const long g = ((long)gx * p->gny + gy) * p->gnz + gz;
              for (int c = 0; c < 3; ++c) {
                REAL coef = 0;
                for (int r = 0; r < p->nrows; ++r)
                  coef = FMA((REAL)weights[(long)r * ns + j],
                             (REAL)q[((long)r * 3 + c) * G + g], coef);
                kahan(&out[c * G + g], &comp[c * G + g], coef, F[c * N + i]);
              }
              continue;
            }
            const int rx = x - p->ox, ry = y - p->oy, rz = z - p->oz;
            if (rx < 0 || rx >= p->rx || ry < 0 || ry >= p->ry || rz < 0 ||
                rz >= p->rz)
              continue;
            const long ri = ((long)rx * p->ry + ry) * p->rz + rz;
            for (int c = 0; c < 3; ++c) {
              if (p->mode == 1) {
                out[((long)j * 3 + c) * R + ri] = F[c * N + i];
                if (p->record_h) out_h[((long)j * 3 + c) * R + ri] = F[(3 + c) * N + i];
              } else {
                for (int r = 0; r < p->nrows; ++r) {
                  const REAL wr = (REAL)weights[(long)r * ns + j];
                  const long ai = ((long)r * 3 + c) * R + ri;
                  kahan(&out[ai], &comp[ai], wr, F[c * N + i]);
                  if (p->record_h)
                    kahan(&out_h[ai], &comp[(long)p->nrows * 3 * R + ai], wr,
                          F[(3 + c) * N + i]);
                }
              }
            }
          }
    }
  }

  free(comp);
  free(zc);
  free(psi);
  free(cb);
  if (!fields) free(F);
  return 0;
}
