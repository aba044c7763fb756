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
  return nullptr;
}

}  // namespace pjzfdtd
