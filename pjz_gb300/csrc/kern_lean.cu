// Instantiations of the lean single-step streamed kernel (lean_kernel.cuh).
#include "kernel_table.cuh"
#include "lean_kernel.cuh"

namespace pjzfdtd {

StreamKernel lean_kernel_ptr(int zz, int tile_y, int storage) {
#define PJZ_PICK_LEAN(ZC, TYC)                                          \
  if (zz == ZC && tile_y == TYC)                                        \
    return storage == 1 ? yee_lean_kernel<ZC, TYC, __half>              \
                        : yee_lean_kernel<ZC, TYC, float>;
  PJZ_LEAN_SHAPES(PJZ_PICK_LEAN)
#undef PJZ_PICK_LEAN
#define PJZ_PICK_LEAN_F16(ZC, TYC) \
  if (zz == ZC && tile_y == TYC && storage == 1) return yee_lean_kernel<ZC, TYC, __half>;
  PJZ_LEAN_SHAPES_F16(PJZ_PICK_LEAN_F16)
#undef PJZ_PICK_LEAN_F16
  return nullptr;
}

int lean_kernel_threads(int zz, int tile_y, int storage) {
#define PJZ_BOUND_LEAN(ZC, TYC)                                              \
  if (zz == ZC && tile_y == TYC)                                             \
    return storage == 1 ? LeanBounds<ZC, TYC, __half>::threads               \
                        : LeanBounds<ZC, TYC, float>::threads;
  PJZ_LEAN_SHAPES(PJZ_BOUND_LEAN)
#undef PJZ_BOUND_LEAN
#define PJZ_BOUND_LEAN_F16(ZC, TYC) \
  if (zz == ZC && tile_y == TYC && storage == 1) return LeanBounds<ZC, TYC, __half>::threads;
  PJZ_LEAN_SHAPES_F16(PJZ_BOUND_LEAN_F16)
#undef PJZ_BOUND_LEAN_F16
  return 0;
}

int lean_tall_tile_y(int zz) {
#define PJZ_TALL_LEAN(ZC, TYC) \
  if (zz == ZC) return TYC;
  PJZ_LEAN_SHAPES_F16(PJZ_TALL_LEAN)
#undef PJZ_TALL_LEAN
  return 0;
}

}  // namespace pjzfdtd
