// Entry points of the step kernels, each instantiated in its own
// translation unit (compiled in parallel) and looked up by the host code.
#pragma once

#include "render_kernel.cuh"
#include "stream_kernel.cuh"

namespace pjzfdtd {

using StreamKernel = void (*)(StreamArgs);
using BatchKernel = void (*)(BatchArgs);

// Single-step streamed kernel for (zz, tile_y): the compile-time
// specialisation when one exists, else the generic body, without
// (kern_stream.cu) or with (kern_stream_src.cu) ring-carried source rows.
StreamKernel stream_kernel_plain_ptr(int zz, int tile_y);
StreamKernel stream_kernel_src_ptr(int zz, int tile_y);
inline StreamKernel stream_kernel_ptr(int zz, int tile_y, bool sr) {
  return sr ? stream_kernel_src_ptr(zz, tile_y) : stream_kernel_plain_ptr(zz, tile_y);
}
// Two-step streamed kernel for (zz, tile_y) (kern_stream2.cu).
StreamKernel stream2_kernel_ptr(int zz, int tile_y);
// Batched launch kernels, one step (kern_batch.cu) or two steps
// (kern_batch2.cu) per problem.
BatchKernel batch1_kernel_ptr();
BatchKernel batch2_kernel_ptr();
inline BatchKernel batch_kernel_ptr(int steps) {
  return steps == 2 ? batch2_kernel_ptr() : batch1_kernel_ptr();
}
// Lean single-step streamed kernel for (zz, tile_y) and storage (0 FP32,
// 1 binary16) (kern_lean.cu), or nullptr when no compile-time shape matches.
StreamKernel lean_kernel_ptr(int zz, int tile_y, int storage);
// Block size bound of that instantiation (0 when none matches).
int lean_kernel_threads(int zz, int tile_y, int storage);
// Tile height of the tall binary16 lean shape for zz, or 0.
int lean_tall_tile_y(int zz);
// Lean two-step streamed kernel, likewise (kern_lean2.cu).
StreamKernel lean2_kernel_ptr(int zz, int tile_y, int storage);
// Block size bound of the lean two-step kernel.
constexpr int kLeanThreads = 384;
// Permittivity rendering kernel (kern_render.cu).
using RenderKernel = void (*)(RenderArgs);
RenderKernel render_kernel_ptr();

}  // namespace pjzfdtd
