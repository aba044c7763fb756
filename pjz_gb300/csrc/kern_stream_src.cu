// Instantiations of the single-step streamed kernel whose ring carries the
// source rows (stream_kernel.cuh).
#include "kernel_table.cuh"

namespace pjzfdtd {

StreamKernel stream_kernel_src_ptr(int zz, int tile_y) {
#define PJZ_PICK(ZC, TYC) \
  if (zz == ZC && tile_y == TYC) return yee_stream_kernel<ZC, TYC, true>;
  PJZ_STREAM_SHAPES(PJZ_PICK)
#undef PJZ_PICK
  return yee_stream_kernel<0, 0, true>;
}

}  // namespace pjzfdtd
