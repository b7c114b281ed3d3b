// C ABI: element-wise transforms built on mgpu::gb300::transform, for callers
// that cannot compile device lambdas themselves.
#include "capi.hxx"
#include "mgpu/gb300/transform.hxx"

using namespace mgpu::gb300;

namespace {

template<typename T>
mgpu_status_t iota_impl(context_t& ctx, void* out, int64_t count, double start, double step) {
  T* p = (T*)out;
  if constexpr(std::is_floating_point<T>::value) {
    T s = (T)start, d = (T)step;
    return transform(count, ctx, [=] __device__(int64_t i) { p[i] = s + (T)i * d; });
  } else {
    typedef typename std::make_unsigned<T>::type U;
    U s = (U)(T)(int64_t)start, d = (U)(T)(int64_t)step;
    return transform(count, ctx, [=] __device__(int64_t i) { p[i] = (T)(s + (U)i * d); });
  }
}

template<typename T>
mgpu_status_t fill_impl(context_t& ctx, void* out, int64_t count, double value) {
  T* p = (T*)out;
  T v = std::is_floating_point<T>::value ? (T)value : (T)(int64_t)value;
  return transform(count, ctx, [=] __device__(int64_t i) { p[i] = v; });
}

template<template<typename> class F, typename... A>
mgpu_status_t by_type(mgpu_dtype_t t, A&&... a) {
  switch(t) {
    case MGPU_I32: return F<int32_t>::run(a...);
    case MGPU_U32: return F<uint32_t>::run(a...);
    case MGPU_F32: return F<float>::run(a...);
    case MGPU_I64: return F<int64_t>::run(a...);
    case MGPU_U64: return F<uint64_t>::run(a...);
    case MGPU_F64: return F<double>::run(a...);
  }
  return MGPU_ERR_INVALID_ARG;
}

template<typename T> struct iota_op {
  static mgpu_status_t run(context_t& c, void* o, int64_t n, double s, double d) {
    return iota_impl<T>(c, o, n, s, d);
  }
};
template<typename T> struct fill_op {
  static mgpu_status_t run(context_t& c, void* o, int64_t n, double v) {
    return fill_impl<T>(c, o, n, v);
  }
};

}  // namespace

extern "C" {

mgpu_status_t mgpu_transform_iota(mgpu_context_t* c, mgpu_dtype_t type, void* out,
  int64_t count, double start, double step) {
  MGPU_CHECK_CTX(c);
  if(count > 0 && !out) return MGPU_ERR_INVALID_ARG;
  return by_type<iota_op>(type, c->ctx, out, count, start, step);
}

mgpu_status_t mgpu_transform_fill(mgpu_context_t* c, mgpu_dtype_t type, void* out,
  int64_t count, double value) {
  MGPU_CHECK_CTX(c);
  if(count > 0 && !out) return MGPU_ERR_INVALID_ARG;
  return by_type<fill_op>(type, c->ctx, out, count, value);
}

mgpu_status_t mgpu_transform_saxpy_f32(mgpu_context_t* c, float a, const float* x, float* y,
  int64_t count) {
  MGPU_CHECK_CTX(c);
  if(count > 0 && (!x || !y)) return MGPU_ERR_INVALID_ARG;
  return transform(count, c->ctx, [=] __device__(int64_t i) { y[i] += a * x[i]; });
}

}  // extern "C"
