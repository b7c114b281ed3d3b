// C ABI: mgpu_segmented_sort (keys I32/U32/F32/I64/U64/F64 with 0-, 4- or
// 8-byte values) and mgpu_segmented_scan (same types; plus, max, min).
#include "capi.hxx"
#include "mgpu/gb300/segmented.hxx"

using namespace mgpu::gb300;
using mgpu::device::no_values;

namespace {

template<typename T, template<typename> class op_tpl>
mgpu_status_t run_scan(mgpu_context* c, mgpu_scan_type_t st, const void* in, void* out,
  int64_t count, const int64_t* offsets, int64_t num_segments, const void* init_p, void* aux,
  size_t* aux_size) {
  typedef op_tpl<T> op_t;
  T init = op_t::identity();
  if(init_p) memcpy(&init, init_p, sizeof(T));
  if(st == MGPU_SCAN_EXC)
    return segmented_scan<scan_type_exc>(aux, aux_size, c->ctx, (const T*)in, count, (T*)out,
      offsets, num_segments, init, op_t());
  if(st == MGPU_SCAN_INC)
    return segmented_scan<scan_type_inc>(aux, aux_size, c->ctx, (const T*)in, count, (T*)out,
      offsets, num_segments, init, op_t());
  return MGPU_ERR_INVALID_ARG;
}

}  // namespace

extern "C" {

mgpu_status_t mgpu_segmented_sort(mgpu_context_t* c, mgpu_dtype_t key_type, void* keys,
  int val_bytes, void* vals, int64_t count, const int64_t* offsets, int64_t num_segments,
  void* aux_data, size_t* aux_size) {
  MGPU_CHECK_CTX(c);
  if(val_bytes != 0 && val_bytes != 4 && val_bytes != 8) return MGPU_ERR_INVALID_ARG;
  return dispatch_dtype(key_type, [&](auto* kp) -> mgpu_status_t {
    typedef std::remove_pointer_t<decltype(kp)> K;
    if(val_bytes == 0)
      return segmented_sort_kv(aux_data, aux_size, c->ctx, (K*)keys, (no_values*)nullptr, count,
        offsets, num_segments);
    if(val_bytes == 4)
      return segmented_sort_kv(aux_data, aux_size, c->ctx, (K*)keys, (uint32_t*)vals, count,
        offsets, num_segments);
    return segmented_sort_kv(aux_data, aux_size, c->ctx, (K*)keys, (uint64_t*)vals, count,
      offsets, num_segments);
  });
}

mgpu_status_t mgpu_segmented_scan(mgpu_context_t* c, mgpu_dtype_t type,
  mgpu_scan_type_t scan_type, mgpu_op_t op, const void* in, void* out, int64_t count,
  const int64_t* offsets, int64_t num_segments, const void* init, void* aux_data,
  size_t* aux_size) {
  MGPU_CHECK_CTX(c);
  return dispatch_dtype(type, [&](auto* tp) -> mgpu_status_t {
    typedef std::remove_pointer_t<decltype(tp)> T;
    switch(op) {
      case MGPU_PLUS: return run_scan<T, plus_t>(c, scan_type, in, out, count, offsets,
        num_segments, init, aux_data, aux_size);
      case MGPU_MAX: return run_scan<T, maximum_t>(c, scan_type, in, out, count, offsets,
        num_segments, init, aux_data, aux_size);
      case MGPU_MIN: return run_scan<T, minimum_t>(c, scan_type, in, out, count, offsets,
        num_segments, init, aux_data, aux_size);
    }
    return MGPU_ERR_INVALID_ARG;
  });
}

}  // extern "C"
