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
