// C ABI: mgpu_scan and mgpu_reduce for I32/U32/F32/I64/U64/F64 with plus,
// max and min, in every tuned launch-shape variant.
#include "capi.hxx"
#include "mgpu/gb300/scan.hxx"

using namespace mgpu::gb300;

namespace {

template<int NT, int VT, int PERSISTENT, int MINB, typename T, typename op_t>
mgpu_status_t scan_shape(mgpu_context* c, mgpu_scan_type_t st, const T* in, T* out,
  int64_t count, T init, T* reduction, void* aux, size_t* aux_size) {
  if(st == MGPU_SCAN_EXC)
    return scan<scan_type_exc, NT, VT, PERSISTENT, MINB>(aux, aux_size, c->ctx, in, count, out, init, op_t(),
      reduction);
  if(st == MGPU_SCAN_INC)
    return scan<scan_type_inc, NT, VT, PERSISTENT, MINB>(aux, aux_size, c->ctx, in, count, out, init, op_t(),
      reduction);
  return MGPU_ERR_INVALID_ARG;
}

template<typename T, template<typename> class op_tpl>
mgpu_status_t run_scan(mgpu_context* c, mgpu_scan_type_t st, const void* in, void* out,
  int64_t count, const void* init_p, void* reduction, void* aux, size_t* aux_size, int variant) {
  typedef op_tpl<T> op_t;
  T init = op_t::identity();
  if(init_p) memcpy(&init, init_p, sizeof(T));
  const T* i = (const T*)in;
  T* o = (T*)out;
  T* r = (T*)reduction;
#define MGPU_SCAN_SHAPE(nt, vt, persistent, minb) \
  scan_shape<nt, vt, persistent, minb, T, op_t>(c, st, i, o, count, init, r, aux, aux_size)
  if constexpr(sizeof(T) == 4) {
    switch(variant) {
      case 1: return MGPU_SCAN_SHAPE(512, 32, 1, 2);
      case 2: return MGPU_SCAN_SHAPE(256, 16, 1, 6);
      case 3: return MGPU_SCAN_SHAPE(256, 32, 0, 4);
      default: return MGPU_SCAN_SHAPE(256, 32, 1, 4);
    }
  } else {
    switch(variant) {
      case 1: return MGPU_SCAN_SHAPE(256, 16, 1, 4);
      case 2: return MGPU_SCAN_SHAPE(256, 8, 1, 6);
      case 3: return MGPU_SCAN_SHAPE(256, 16, 0, 4);
      default: return MGPU_SCAN_SHAPE(512, 16, 1, 2);
    }
  }
#undef MGPU_SCAN_SHAPE
}

template<typename T, template<typename> class op_tpl>
mgpu_status_t run_reduce(mgpu_context* c, const void* in, int64_t count, const void* init_p,
  void* out, void* aux, size_t* aux_size) {
  typedef op_tpl<T> op_t;
  T init = op_t::identity();
  if(init_p) memcpy(&init, init_p, sizeof(T));
  return reduce(aux, aux_size, c->ctx, (const T*)in, count, (T*)out, init, op_t());
}

}  // namespace

extern "C" {

mgpu_status_t mgpu_scan(mgpu_context_t* c, mgpu_dtype_t type, mgpu_scan_type_t scan_type,
  mgpu_op_t op, const void* in, void* out, int64_t count, const void* init, void* reduction,
  void* aux_data, size_t* aux_size) {
  MGPU_CHECK_CTX(c);
  int variant = c->ctx.tuning.lookup(prim_scan, type, 0, count);
  return dispatch_dtype(type, [&](auto* tp) -> mgpu_status_t {
    typedef std::remove_pointer_t<decltype(tp)> T;
    switch(op) {
      case MGPU_PLUS: return run_scan<T, plus_t>(c, scan_type, in, out, count, init, reduction,
        aux_data, aux_size, variant);
      case MGPU_MAX: return run_scan<T, maximum_t>(c, scan_type, in, out, count, init, reduction,
        aux_data, aux_size, variant);
      case MGPU_MIN: return run_scan<T, minimum_t>(c, scan_type, in, out, count, init, reduction,
        aux_data, aux_size, variant);
    }
    return MGPU_ERR_INVALID_ARG;
  });
}

mgpu_status_t mgpu_reduce(mgpu_context_t* c, mgpu_dtype_t type, mgpu_op_t op, const void* in,
  int64_t count, const void* init, void* out, void* aux_data, size_t* aux_size) {
  MGPU_CHECK_CTX(c);
  return dispatch_dtype(type, [&](auto* tp) -> mgpu_status_t {
    typedef std::remove_pointer_t<decltype(tp)> T;
    switch(op) {
      case MGPU_PLUS: return run_reduce<T, plus_t>(c, in, count, init, out, aux_data, aux_size);
      case MGPU_MAX: return run_reduce<T, maximum_t>(c, in, count, init, out, aux_data, aux_size);
      case MGPU_MIN: return run_reduce<T, minimum_t>(c, in, count, init, out, aux_data, aux_size);
    }
    return MGPU_ERR_INVALID_ARG;
  });
}

}  // extern "C"
