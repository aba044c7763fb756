// Batched-launch kernel, one step per problem (stream_kernel.cuh).
#define PJZ_BATCH1_KERNEL
#include "kernel_table.cuh"

namespace pjzfdtd {

BatchKernel batch1_kernel_ptr() { return yee_stream_batch_kernel; }

}  // namespace pjzfdtd
