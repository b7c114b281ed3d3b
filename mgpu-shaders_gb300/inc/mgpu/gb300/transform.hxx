// mgpu::gb300::launch / transform - generic kernels over a user functor.
//
// Drop-ins for vk::launch and vk::transform (vk/transform.hxx:9-36): the
// reference captured a lambda's closure into Vulkan push constants
// (vk/launch.hxx:15-30); here the closure is a kernel parameter.  Device
// lambdas need nvcc's --extended-lambda.
//   launch<nt>(num_blocks, ctx, [=] __device__ (int tid, int cta) { ... });
//   transform<nt>(count, ctx, [=] __device__ (int64_t index) { ... });
// transform runs a grid-stride loop over at most 32 CTAs per SM, so very
// large counts do not need one thread per element.
#pragma once

#include "context.hxx"

namespace mgpu {
namespace gb300 {

template<int nt, typename func_t>
__global__ void __launch_bounds__(nt) launch_kernel(func_t f) {
  f((int)threadIdx.x, (int)blockIdx.x);
}

template<int nt, typename func_t>
__global__ void __launch_bounds__(nt) transform_kernel(int64_t count, func_t f) {
  const int64_t stride = (int64_t)gridDim.x * nt;
  for(int64_t i = (int64_t)blockIdx.x * nt + threadIdx.x; i < count; i += stride) f(i);
}

template<int nt = 128, typename func_t>
status_t launch(int num_blocks, context_t& ctx, func_t f) {
  if(num_blocks < 0) return MGPU_ERR_INVALID_ARG;
  if(num_blocks == 0) return MGPU_OK;
  return ctx.launch("launch", [&] { launch_kernel<nt><<<num_blocks, nt, 0, ctx.stream>>>(f); });
}

template<int nt = 256, typename func_t>
status_t transform(int64_t count, context_t& ctx, func_t f) {
  if(count < 0) return MGPU_ERR_INVALID_ARG;
  if(count == 0) return MGPU_OK;
  int64_t blocks = std::min<int64_t>((count + nt - 1) / nt, (int64_t)ctx.sm_count * 32);
  return ctx.launch("transform", [&] {
    transform_kernel<nt><<<(unsigned)blocks, nt, 0, ctx.stream>>>(count, f);
  });
}

}  // namespace gb300
}  // namespace mgpu
