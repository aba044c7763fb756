// Instantiations of the single-step streamed kernel without ring-carried
// source rows (stream_kernel.cuh).
#include "kernel_table.cuh"

namespace pjzfdtd {

StreamKernel stream_kernel_plain_ptr(int zz, int tile_y) {
#define PJZ_PICK(ZC, TYC) \
  if (zz == ZC && tile_y == TYC) return yee_stream_kernel<ZC, TYC, false>;
  PJZ_STREAM_SHAPES(PJZ_PICK)
#undef PJZ_PICK
  return yee_stream_kernel<0, 0, false>;
}

}  // namespace pjzfdtd
