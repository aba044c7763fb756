// Host-side entry to the lean kernels' item mapping (lean_item and
// lean_warps in pjz_gb300/csrc/lean_kernel.cuh, __host__ __device__), so a
// CPU test can check the shared-memory replay model's copy of it entry by
// entry.  Built with nvcc as a shared library; no device code runs.
#include "lean_kernel.cuh"

using namespace pjzfdtd;

extern "C" int lean_items_host(int Z, int rows, int plo, int phi, int esz,
                               int* row, int* z0, int* col, int* pml, int cap) {
  const int n = 32 * lean_warps(Z, rows, plo, phi, esz);
  if (n > cap) return -1;
  for (int t = 0; t < n; ++t) {
    const LeanItem it = lean_item(t, Z, rows, plo, phi, esz);
    row[t] = it.row;
    z0[t] = it.z0;
    col[t] = it.pml ? it.col : 0;
    pml[t] = it.pml ? 1 : 0;
  }
  return n;
}

// LeanGeom<T> of a (tile_y, zz, z-PML width) shape: byte offsets e, h, c,
// m, p and the slot size, then the new-H, new-E and new-PML-state sizes.
extern "C" void lean_geom_host(int ty, int z, int p, int esz, long long* out) {
  if (esz == 2) {
    const LeanGeom<__half> g(ty, z, p);
    const long long v[] = {g.e_off, g.h_off, g.c_off, g.m_off, g.p_off, g.stage,
                           (long long)g.hn_bytes(), (long long)g.en_bytes(),
                           (long long)g.pn_bytes(), g.Pp};
    for (int i = 0; i < 10; ++i) out[i] = v[i];
  } else {
    const LeanGeom<float> g(ty, z, p);
    const long long v[] = {g.e_off, g.h_off, g.c_off, g.m_off, g.p_off, g.stage,
                           (long long)g.hn_bytes(), (long long)g.en_bytes(),
                           (long long)g.pn_bytes(), g.Pp};
    for (int i = 0; i < 10; ++i) out[i] = v[i];
  }
}
