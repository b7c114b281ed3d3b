// C ABI: self test of the bounded waits (the failure path without a fault).
#include "capi.hxx"
#include "mgpu/device/common.cuh"

namespace {

// Stays zero: no code writes it.
__device__ uint32_t g_never_set = 0;

__global__ void bounded_wait_probe(int limit, int* error) {
  using namespace mgpu::device;
  __shared__ uint64_t bar;
  if(threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if(threadIdx.x == 0) {
    // A bulk-copy completion that never comes: no arrival, no bytes.
    mbar_wait_bounded(&bar, 0, error, limit);
    // A look-back status that is never published.
    int spins = 0;
    while(ld_relaxed(&g_never_set) == 0) {
      if(++spins >= limit) {
        raise_error(error, err_lookback_timeout);
        break;
      }
      __nanosleep(64);
    }
  }
}

}  // namespace

extern "C" mgpu_status_t mgpu_selftest_bounded_wait(mgpu_context_t* c, int limit) {
  MGPU_CHECK_CTX(c);
  if(limit < 1 || limit > mgpu::device::spin_limit) return MGPU_ERR_INVALID_ARG;
  return c->ctx.launch("bounded_wait_probe", [&] {
    bounded_wait_probe<<<1, 32, 0, c->ctx.stream>>>(limit, c->ctx.d_error);
  });
}

extern "C" mgpu_status_t mgpu_set_wait_limit(mgpu_context_t* c, int polls) {
  if(!c) return MGPU_ERR_INVALID_ARG;
  if(polls < 0 || polls > mgpu::device::spin_limit) return MGPU_ERR_INVALID_ARG;
  c->ctx.wait_limit = polls;
  return MGPU_OK;
}
