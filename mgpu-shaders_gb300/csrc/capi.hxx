// Shared glue of the C ABI translation units: the opaque context type and
// argument checks.  Each capi_*.cu file instantiates the mgpu::gb300
// templates for the fixed key/value types the C ABI offers.
#pragma once

#include "mgpu_gb300.h"
#include "mgpu/gb300/context.hxx"

struct mgpu_context {
  explicit mgpu_context(int device, cudaStream_t stream) : ctx(device, stream) {}
  mgpu::gb300::context_t ctx;
};

#define MGPU_CHECK_CTX(c)                                                      \
  do {                                                                         \
    if(!(c)) return MGPU_ERR_INVALID_ARG;                                      \
    if(cudaSetDevice((c)->ctx.device) != cudaSuccess) return MGPU_ERR_CUDA;    \
  } while(0)

// Calls f with a typed null pointer for the key type.
template<typename F>
mgpu_status_t dispatch_dtype(mgpu_dtype_t t, F&& f) {
  switch(t) {
    case MGPU_I32: return f((int32_t*)nullptr);
    case MGPU_U32: return f((uint32_t*)nullptr);
    case MGPU_F32: return f((float*)nullptr);
    case MGPU_I64: return f((int64_t*)nullptr);
    case MGPU_U64: return f((uint64_t*)nullptr);
    case MGPU_F64: return f((double*)nullptr);
  }
  return MGPU_ERR_INVALID_ARG;
}

template<typename T> constexpr mgpu_dtype_t dtype_of();
template<> constexpr mgpu_dtype_t dtype_of<int32_t>() { return MGPU_I32; }
template<> constexpr mgpu_dtype_t dtype_of<uint32_t>() { return MGPU_U32; }
template<> constexpr mgpu_dtype_t dtype_of<float>() { return MGPU_F32; }
template<> constexpr mgpu_dtype_t dtype_of<int64_t>() { return MGPU_I64; }
template<> constexpr mgpu_dtype_t dtype_of<uint64_t>() { return MGPU_U64; }
template<> constexpr mgpu_dtype_t dtype_of<double>() { return MGPU_F64; }
