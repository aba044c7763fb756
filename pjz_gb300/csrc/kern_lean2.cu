// Instantiations of the lean two-step streamed kernel (lean2_kernel.cuh).
#include "kernel_table.cuh"
#include "lean2_kernel.cuh"

namespace pjzfdtd {

StreamKernel lean2_kernel_ptr(int zz, int tile_y, int storage) {
#define PJZ_PICK_LEAN2(ZC, TYC)                                         \
  if (zz == ZC && tile_y == TYC)                                        \
    return storage == 1 ? yee_lean2_kernel<ZC, TYC, __half>             \
                        : yee_lean2_kernel<ZC, TYC, float>;
  PJZ_LEAN2_SHAPES(PJZ_PICK_LEAN2)
#undef PJZ_PICK_LEAN2
  return nullptr;
}

}  // namespace pjzfdtd
