// C ABI: radix sort instantiations for 64-bit keys, every tuned variant.
#include "capi.hxx"
#include "mgpu/gb300/radix.hxx"

using namespace mgpu::gb300;
using mgpu::device::no_values;

mgpu_status_t radix_sort_w64(mgpu_context* c, mgpu_dtype_t key_type, void* keys, int val_bytes,
  void* vals, int64_t count, int variant, void* aux, size_t* aux_size, const int64_t* d_count) {
  auto go_key = [&](auto* kp) -> mgpu_status_t {
    typedef std::remove_pointer_t<decltype(kp)> K;
    auto go = [&](auto* vp) -> mgpu_status_t {
      typedef std::remove_pointer_t<decltype(vp)> V;
      if(d_count)   // count read on the device: the default shape
        return radix_sort_kv<256, 16, 3, true>(aux, aux_size, c->ctx, (K*)keys, (V*)vals, count,
          d_count);
      switch(variant) {
        case 1: return radix_sort_kv<256, 12, 3>(aux, aux_size, c->ctx, (K*)keys, (V*)vals, count);
        case 2: return radix_sort_kv<384, 10, 3>(aux, aux_size, c->ctx, (K*)keys, (V*)vals, count);
        case 3: {
          typedef radix_knobs<K, V, 256, 16, 4> R;
          return radix_sort_kv<R::NT, R::VT, R::MINB, false, 4>(aux, aux_size, c->ctx, (K*)keys,
            (V*)vals, count);
        }
        case 4: {
          typedef radix_knobs<K, V, 128, 16, 4> R;
          return radix_sort_kv<R::NT, R::VT, R::MINB, false, 4>(aux, aux_size, c->ctx, (K*)keys,
            (V*)vals, count);
        }
        default: return radix_sort_kv<256, 16, 3>(aux, aux_size, c->ctx, (K*)keys, (V*)vals, count);
      }
    };
    if(val_bytes == 0) return go((no_values*)nullptr);
    if(val_bytes == 4) return go((uint32_t*)nullptr);
    return go((uint64_t*)nullptr);
  };
  switch(key_type) {
    case MGPU_I64: return go_key((int64_t*)nullptr);
    case MGPU_U64: return go_key((uint64_t*)nullptr);
    case MGPU_F64: return go_key((double*)nullptr);
    default: break;
  }
  return MGPU_ERR_INVALID_ARG;
}
