// C ABI: radix sort instantiations for 32-bit keys, every tuned variant.
#include "capi.hxx"
#include "mgpu/gb300/radix.hxx"

using namespace mgpu::gb300;
using mgpu::device::no_values;

// Shapes are given for 4-byte values (and keys-only); with 8-byte values
// the staged elements are twice as wide, so a tile holds half the keys.
template<int NT, int VT4, int MINB, bool DEV = false, typename K, typename V>
mgpu_status_t sort_shape(mgpu_context* c, K* keys, V* vals, int64_t count, void* aux,
  size_t* aux_size, const int64_t* d_count) {
  constexpr int VT = radix_elem_bytes<K, V>() == 8 ? VT4 / 2 : VT4;
  return radix_sort_kv<NT, VT, MINB, DEV>(aux, aux_size, c->ctx, keys, vals, count, d_count);
}

// A 4-bit-digit shape (eight passes over 4-byte keys), CTAs per SM as the
// C++ knobs derive them.
template<int NT, int VT4, typename K, typename V>
mgpu_status_t sort_shape4(mgpu_context* c, K* keys, V* vals, int64_t count, void* aux,
  size_t* aux_size) {
  constexpr int VT = radix_elem_bytes<K, V>() == 8 ? VT4 / 2 : VT4;
  typedef radix_knobs<K, V, NT, VT, 4> R;
  return radix_sort_kv<R::NT, R::VT, R::MINB, false, 4>(aux, aux_size, c->ctx, keys, vals, count);
}

mgpu_status_t radix_sort_w32(mgpu_context* c, mgpu_dtype_t key_type, void* keys, int val_bytes,
  void* vals, int64_t count, int variant, void* aux, size_t* aux_size, const int64_t* d_count) {
  auto go_key = [&](auto* kp) -> mgpu_status_t {
    typedef std::remove_pointer_t<decltype(kp)> K;
    auto go = [&](auto* vp) -> mgpu_status_t {
      typedef std::remove_pointer_t<decltype(vp)> V;
      K* k = (K*)keys;
      V* v = (V*)vals;
      // Odd item counts: a half-warp's run starts 16 banks from its
      // neighbour's.
      constexpr int V0 = radix_tuning<4>::vt, V1 = 31, V2 = 23;
      if(d_count)   // count read on the device: the default shape
        return sort_shape<384, V0, 3, true>(c, k, v, count, aux, aux_size, d_count);
      switch(variant) {
        case 1: return sort_shape<256, V1, 3>(c, k, v, count, aux, aux_size, nullptr);
        case 2: return sort_shape<256, V2, 3>(c, k, v, count, aux, aux_size, nullptr);
        case 3: return sort_shape4<256, 16>(c, k, v, count, aux, aux_size);
        case 4: return sort_shape4<128, 16>(c, k, v, count, aux, aux_size);
        default: return sort_shape<384, V0, 3>(c, k, v, count, aux, aux_size, nullptr);
      }
    };
    if(val_bytes == 0) return go((no_values*)nullptr);
    if(val_bytes == 4) return go((uint32_t*)nullptr);
    return go((uint64_t*)nullptr);
  };
  switch(key_type) {
    case MGPU_I32: return go_key((int32_t*)nullptr);
    case MGPU_U32: return go_key((uint32_t*)nullptr);
    case MGPU_F32: return go_key((float*)nullptr);
    default: break;
  }
  return MGPU_ERR_INVALID_ARG;
}

// Failure-path self test of the production look-back (mgpu_gb300.h): the
// default u32 key-value pass kernel over two tiles of zero keys, tile counter
// advanced to 1, one CTA.  That CTA claims tile 1 and waits on tile 0's
// look-back row, which stays zero; the wait gives up after the context's
// limit.  Tile 1 then stores at offsets 0 .. tile-1 (the look-back prefix it
// could not read counts as 0), inside the two-tile output buffers.
extern "C" mgpu_status_t mgpu_selftest_lookback_timeout(mgpu_context_t* c) {
  MGPU_CHECK_CTX(c);
  using namespace mgpu::device;
  typedef radix_tuning<4> T;
  constexpr int nt = T::nt, vt = T::vt, minb = T::min_blocks;
  typedef onesweep_layout<uint32_t, uint32_t, nt, vt> L;
  constexpr int64_t n = 2 * (int64_t)nt * vt;
  auto kernel = onesweep_pass<uint32_t, uint32_t, nt, vt, minb, 4, false>;
  context_t& ctx = c->ctx;
  if(!ctx.allow_smem(kernel, L::bytes)) return MGPU_ERR_CUDA;
  // keys in/out, values in/out, 256 digit counts, two look-back rows, counter
  const size_t words = 4 * n + radix_bins + 2 * radix_bins + 1;
  uint32_t* buf = nullptr;
  if(ctx.check(cudaMalloc(&buf, sizeof(uint32_t) * words))) return MGPU_ERR_OOM;
  const uint32_t digit0 = (uint32_t)n, one = 1;
  uint32_t* hist = buf + 4 * n;
  uint32_t* lookback = hist + radix_bins;
  uint32_t* counter = lookback + 2 * radix_bins;
  mgpu_status_t st = MGPU_OK;
  if(ctx.check(cudaMemsetAsync(buf, 0, sizeof(uint32_t) * words, ctx.stream)) ||
     ctx.check(cudaMemcpyAsync(hist, &digit0, 4, cudaMemcpyHostToDevice, ctx.stream)) ||
     ctx.check(cudaMemcpyAsync(counter, &one, 4, cudaMemcpyHostToDevice, ctx.stream))) {
    st = MGPU_ERR_CUDA;
  } else {
    onesweep_args<uint32_t, uint32_t> a;
    a.keys_in = buf;
    a.keys_out = buf + n;
    a.vals_in = buf + 2 * n;
    a.vals_out = buf + 3 * n;
    a.count = n;
    a.shift = 0;
    a.hist = hist;
    a.lookback = lookback;
    a.tile_counter = counter;
    a.error = ctx.d_error;
    a.wait_limit = ctx.wait_limit > 0 ? ctx.wait_limit : spin_limit;
    a.first = 1;
    a.last = 0;
    a.tma = 1;
    st = ctx.launch("onesweep_pass", [&] {
      kernel<<<1, nt, L::bytes, ctx.stream>>>(a);
    });
  }
  if(ctx.check(cudaStreamSynchronize(ctx.stream)) && !st) st = MGPU_ERR_CUDA;
  cudaFree(buf);
  return st;
}
