// C ABI: mgpu_merge for I32/U32/F32/I64/U64/F64 keys with 0-, 4- or 8-byte
// values and std::less / std::greater.
#include "capi.hxx"
#include "mgpu/gb300/merge.hxx"

using namespace mgpu::gb300;
using mgpu::device::no_values;

namespace {

template<typename K, typename V, typename comp_t>
mgpu_status_t run(mgpu_context* c, const void* ak, const void* av, int64_t an, const void* bk,
  const void* bv, int64_t bn, void* ck, void* cv, void* aux, size_t* aux_size) {
  int variant = c->ctx.tuning.lookup(prim_merge, (int)dtype_of<K>(), (int)sizeof(V) *
    !std::is_same<V, no_values>::value, an + bn);
  constexpr int NT1 = sizeof(K) == 4 ? 256 : 128;
  if(variant == 1)
    return merge_kv<NT1, 8>(aux, aux_size, c->ctx, (const K*)ak, (const V*)av, an, (const K*)bk,
      (const V*)bv, bn, (K*)ck, (V*)cv, comp_t());
  // The even shape (stride-16 or -8 shared-memory accesses per thread).
  constexpr int VT_EVEN = sizeof(K) == 4 ? 16 : 8;
  if(variant == 2)
    return merge_kv<256, VT_EVEN>(aux, aux_size, c->ctx, (const K*)ak, (const V*)av, an,
      (const K*)bk, (const V*)bv, bn, (K*)ck, (V*)cv, comp_t());
  return merge_kv(aux, aux_size, c->ctx, (const K*)ak, (const V*)av, an, (const K*)bk,
    (const V*)bv, bn, (K*)ck, (V*)cv, comp_t());
}

}  // namespace

extern "C" mgpu_status_t mgpu_merge(mgpu_context_t* c, mgpu_dtype_t key_type,
  const void* a_keys, const void* a_vals, int64_t a_count, const void* b_keys,
  const void* b_vals, int64_t b_count, void* c_keys, void* c_vals, int val_bytes,
  mgpu_comp_t comp, void* aux_data, size_t* aux_size) {
  MGPU_CHECK_CTX(c);
  if(val_bytes != 0 && val_bytes != 4 && val_bytes != 8) return MGPU_ERR_INVALID_ARG;
  if(comp != MGPU_LESS && comp != MGPU_GREATER) return MGPU_ERR_INVALID_ARG;
  return dispatch_dtype(key_type, [&](auto* kp) -> mgpu_status_t {
    typedef std::remove_pointer_t<decltype(kp)> K;
    auto go = [&](auto* vp) -> mgpu_status_t {
      typedef std::remove_pointer_t<decltype(vp)> V;
      if(comp == MGPU_LESS)
        return run<K, V, less_t<K>>(c, a_keys, a_vals, a_count, b_keys, b_vals, b_count, c_keys,
          c_vals, aux_data, aux_size);
      return run<K, V, greater_t<K>>(c, a_keys, a_vals, a_count, b_keys, b_vals, b_count, c_keys,
        c_vals, aux_data, aux_size);
    };
    if(val_bytes == 0) return go((no_values*)nullptr);
    if(val_bytes == 4) return go((uint32_t*)nullptr);
    return go((uint64_t*)nullptr);
  });
}
