// C ABI: mgpu_mergesort / mgpu_mergesort_indices for 32-bit keys.
#include "capi.hxx"
#include "mgpu/gb300/merge.hxx"

using namespace mgpu::gb300;
using mgpu::device::no_values;

mgpu_status_t mergesort_w32(mgpu_context* c, mgpu_dtype_t key_type, void* keys, int val_bytes,
  void* vals, int64_t count, mgpu_comp_t comp, int indices, void* aux, size_t* aux_size) {
  auto go_key = [&](auto* kp) -> mgpu_status_t {
    typedef std::remove_pointer_t<decltype(kp)> K;
    auto go = [&](auto* vp, auto idx) -> mgpu_status_t {
      typedef std::remove_pointer_t<decltype(vp)> V;
      constexpr bool I = decltype(idx)::value;
      constexpr int NT1 = sizeof(K) == 4 ? 256 : 128;
      int variant = c->ctx.tuning.lookup(prim_mergesort, key_type, I ? 4 : val_bytes, count);
      if(variant == 1) {
        if(comp == MGPU_LESS)
          return mergesort_kv<NT1, 8, I>(aux, aux_size, c->ctx, (K*)keys, (V*)vals, count,
            less_t<K>());
        return mergesort_kv<NT1, 8, I>(aux, aux_size, c->ctx, (K*)keys, (V*)vals, count,
          greater_t<K>());
      }
      constexpr int VT2 = mergesort_tuning<K, V>::vt_alt;
      if(variant == 2) {
        if(comp == MGPU_LESS)
          return mergesort_kv<256, VT2, I>(aux, aux_size, c->ctx, (K*)keys, (V*)vals, count,
            less_t<K>());
        return mergesort_kv<256, VT2, I>(aux, aux_size, c->ctx, (K*)keys, (V*)vals, count,
          greater_t<K>());
      }
      if(comp == MGPU_LESS)
        return mergesort_kv<0, 0, I>(aux, aux_size, c->ctx, (K*)keys, (V*)vals, count,
          less_t<K>());
      return mergesort_kv<0, 0, I>(aux, aux_size, c->ctx, (K*)keys, (V*)vals, count,
        greater_t<K>());
    };
    if(indices) return go((int32_t*)nullptr, std::true_type());
    if(val_bytes == 0) return go((no_values*)nullptr, std::false_type());
    if(val_bytes == 4) return go((uint32_t*)nullptr, std::false_type());
    return go((uint64_t*)nullptr, std::false_type());
  };
  switch(key_type) {
    case MGPU_I32: return go_key((int32_t*)nullptr);
    case MGPU_U32: return go_key((uint32_t*)nullptr);
    case MGPU_F32: return go_key((float*)nullptr);
    default: break;
  }
  return MGPU_ERR_INVALID_ARG;
}
