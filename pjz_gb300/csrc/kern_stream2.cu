// Instantiations of the two-step streamed kernel (stream2_kernel.cuh).
#include "kernel_table.cuh"
#include "stream2_kernel.cuh"

namespace pjzfdtd {

StreamKernel stream2_kernel_ptr(int zz, int tile_y) {
#define PJZ_PICK2(ZC, TYC) \
  if (zz == ZC && tile_y == TYC) return yee_stream2_kernel<ZC, TYC>;
  PJZ_STREAM2_SHAPES(PJZ_PICK2)
#undef PJZ_PICK2
  return yee_stream2_kernel<0, 0>;
}

}  // namespace pjzfdtd
