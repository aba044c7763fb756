// Batched-launch kernel, two steps per problem (stream2_kernel.cuh).
#define PJZ_BATCH2_KERNEL
#include "kernel_table.cuh"
#include "stream2_kernel.cuh"

namespace pjzfdtd {

BatchKernel batch2_kernel_ptr() { return yee_stream_batch2_kernel; }

}  // namespace pjzfdtd
