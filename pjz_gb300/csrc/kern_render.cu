// The permittivity rendering kernel (render_kernel.cuh).
#define PJZ_RENDER_KERNEL
#include "kernel_table.cuh"

namespace pjzfdtd {

RenderKernel render_kernel_ptr() { return render_epsilon_kernel; }

}  // namespace pjzfdtd
