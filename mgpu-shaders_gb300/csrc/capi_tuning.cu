// C ABI: tuning table access and the autotuner.  The autotuner times every
// compiled variant of a primitive on device-generated data of the requested
// type and size (CUDA events, median of `reps` runs, each on an unsorted
// copy) and records the fastest in the context's table for that size bucket.
#include "capi.hxx"
#include "variants.hxx"
#include "mgpu/gb300/transform.hxx"

#include <algorithm>
#include <cstring>
#include <vector>

using namespace mgpu::gb300;

namespace {

int variant_count(int prim, int bytes) {
  switch(prim) {
    case prim_radix: return variants::radix_count(bytes);
    case prim_scan: return variants::scan_count(bytes);
    case prim_merge: case prim_mergesort: return variants::merge_count(bytes);
  }
  return 0;
}

const char* variant_name(int prim, int bytes, int v) {
  switch(prim) {
    case prim_radix: return variants::radix_name(bytes, v);
    case prim_scan: return variants::scan_name(bytes, v);
    case prim_merge: return variants::merge_name(bytes, v);
    case prim_mergesort: return variants::mergesort_name(bytes, v);
  }
  return "";
}

__host__ __device__ inline uint64_t mix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// Fills `bytes`-wide elements with hashed bits; floats get values in [0, 1).
mgpu_status_t fill_random(context_t& ctx, void* p, int64_t n, int bytes, bool fp, uint64_t seed) {
  if(bytes == 4) {
    uint32_t* q = (uint32_t*)p;
    if(fp) return transform(n, ctx, [=] __device__(int64_t i) {
      float f = (float)(mix64(i ^ seed) >> 40) * (1.0f / 16777216.0f);
      q[i] = __float_as_uint(f);
    });
    return transform(n, ctx, [=] __device__(int64_t i) { q[i] = (uint32_t)mix64(i ^ seed); });
  }
  uint64_t* q = (uint64_t*)p;
  if(fp) return transform(n, ctx, [=] __device__(int64_t i) {
    double f = (double)(mix64(i ^ seed) >> 11) * (1.0 / 9007199254740992.0);
    q[i] = (uint64_t)__double_as_longlong(f);
  });
  return transform(n, ctx, [=] __device__(int64_t i) { q[i] = mix64(i ^ seed); });
}

mgpu_status_t iota32(context_t& ctx, void* p, int64_t n) {
  uint32_t* q = (uint32_t*)p;
  return transform(n, ctx, [=] __device__(int64_t i) { q[i] = (uint32_t)i; });
}

}  // namespace

extern "C" {

int mgpu_tuning_variants(int primitive, mgpu_dtype_t key_type, char* names, size_t names_bytes) {
  int bytes = variants::dtype_bytes(key_type);
  int n = variant_count(primitive, bytes);
  if(names && names_bytes) {
    names[0] = 0;
    size_t used = 0;
    for(int v = 0; v < n; ++v) {
      const char* s = variant_name(primitive, bytes, v);
      size_t len = strlen(s);
      if(used + len + 2 > names_bytes) break;
      memcpy(names + used, s, len);
      used += len;
      names[used++] = '\n';
      names[used] = 0;
    }
  }
  return n;
}

mgpu_status_t mgpu_tuning_set(mgpu_context_t* c, int primitive, mgpu_dtype_t key_type,
  int val_bytes, int size_bucket, int variant) {
  MGPU_CHECK_CTX(c);
  int n = variant_count(primitive, variants::dtype_bytes(key_type));
  if(variant < 0 || variant >= n || size_bucket < -1 || size_bucket > 62) return MGPU_ERR_INVALID_ARG;
  c->ctx.tuning.set(primitive, key_type, val_bytes, size_bucket, variant);
  return MGPU_OK;
}

int mgpu_tuning_get(mgpu_context_t* c, int primitive, mgpu_dtype_t key_type, int val_bytes,
  int64_t count) {
  if(!c) return -1;
  return c->ctx.tuning.lookup(primitive, key_type, val_bytes, count);
}

mgpu_status_t mgpu_tuning_save(mgpu_context_t* c, const char* path) {
  MGPU_CHECK_CTX(c);
  if(!path) return MGPU_ERR_INVALID_ARG;
  return c->ctx.tuning.save(path) ? MGPU_OK : MGPU_ERR_INVALID_ARG;
}

mgpu_status_t mgpu_tuning_load(mgpu_context_t* c, const char* path) {
  MGPU_CHECK_CTX(c);
  if(!path) return MGPU_ERR_INVALID_ARG;
  // Read into a scratch table and take it only if every entry names a
  // compiled variant and a valid bucket, so a bad file changes nothing.
  tuning_table_t t;
  if(!t.load(path)) return MGPU_ERR_INVALID_ARG;
  for(auto& e : t.entries) {
    const int prim = std::get<0>(e.first), type = std::get<1>(e.first);
    const int bucket = std::get<3>(e.first);
    if(type < 0 || type > MGPU_F64 || bucket < -1 || bucket > 62 || e.second < 0 ||
       e.second >= variant_count(prim, variants::dtype_bytes((mgpu_dtype_t)type)))
      return MGPU_ERR_INVALID_ARG;
  }
  for(auto& e : t.entries) c->ctx.tuning.entries[e.first] = e.second;
  return MGPU_OK;
}

mgpu_status_t mgpu_autotune(mgpu_context_t* c, int primitive, mgpu_dtype_t key_type,
  int val_bytes, int64_t count, int reps, int* best_variant, double* best_ms) {
  MGPU_CHECK_CTX(c);
  context_t& ctx = c->ctx;
  if(count <= 0 || reps <= 0 || ctx.capturing) return MGPU_ERR_INVALID_ARG;
  if(val_bytes != 0 && val_bytes != 4 && val_bytes != 8) return MGPU_ERR_INVALID_ARG;
  const int kb = variants::dtype_bytes(key_type);
  const bool fp = key_type == MGPU_F32 || key_type == MGPU_F64;
  const int nvar = variant_count(primitive, kb);
  if(nvar <= 0) return MGPU_ERR_INVALID_ARG;
  if(primitive == prim_scan) val_bytes = 0;
  if(primitive == prim_mergesort && val_bytes == 8) val_bytes = 8;
  const int vb = val_bytes;

  // Scratch: source and working copies of keys (and values); merge also
  // needs an output.
  char* buf[6] = {};
  size_t kbytes = (size_t)kb * count, vbytes = (size_t)(vb ? vb : 4) * count;
  size_t sizes[6] = { kbytes, kbytes, vbytes, vbytes, kbytes, vbytes };
  mgpu_status_t st = MGPU_OK;
  for(int i = 0; i < 6 && !st; ++i)
    if(ctx.check(cudaMalloc((void**)&buf[i], std::max<size_t>(sizes[i], 16)))) st = MGPU_ERR_OOM;
  char *src_k = buf[0], *wk = buf[1], *src_v = buf[2], *wv = buf[3], *out_k = buf[4],
       *out_v = buf[5];
  if(!st) st = fill_random(ctx, src_k, count, kb, fp, 0x6d677075ull + primitive);
  if(!st && vb) st = iota32(ctx, src_v, count * vb / 4);
  const int64_t a_count = count / 2, b_count = count - a_count;
  if(!st && primitive == prim_merge) {
    // Two sorted halves: radix order equals numeric order for these keys.
    st = mgpu_radix_sort(c, key_type, src_k, 0, nullptr, a_count, nullptr, nullptr);
    if(!st) st = mgpu_radix_sort(c, key_type, src_k + (size_t)kb * a_count, 0, nullptr,
      b_count, nullptr, nullptr);
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if(!st && (ctx.check(cudaEventCreate(&e0)) || ctx.check(cudaEventCreate(&e1))))
    st = MGPU_ERR_CUDA;

  const int bucket = size_bucket(count);
  int best = 0;
  double best_t = 1e30;
  auto run_once = [&]() -> mgpu_status_t {
    switch(primitive) {
      case prim_radix:
        return mgpu_radix_sort(c, key_type, wk, vb, vb ? wv : nullptr, count, nullptr, nullptr);
      case prim_scan:
        return mgpu_scan(c, key_type, MGPU_SCAN_INC, MGPU_PLUS, wk, out_k, count, nullptr,
          nullptr, nullptr, nullptr);
      case prim_merge:
        return mgpu_merge(c, key_type, wk, vb ? wv : nullptr, a_count,
          wk + (size_t)kb * a_count, vb ? wv + (size_t)vb * a_count : nullptr, b_count,
          out_k, vb ? out_v : nullptr, vb, MGPU_LESS, nullptr, nullptr);
      case prim_mergesort:
        return mgpu_mergesort(c, key_type, wk, vb, vb ? wv : nullptr, count, MGPU_LESS, nullptr,
          nullptr);
    }
    return MGPU_ERR_INVALID_ARG;
  };
  auto restore = [&]() -> mgpu_status_t {
    if(ctx.check(cudaMemcpyAsync(wk, src_k, kbytes, cudaMemcpyDeviceToDevice, ctx.stream)))
      return MGPU_ERR_CUDA;
    if(vb && ctx.check(cudaMemcpyAsync(wv, src_v, (size_t)vb * count, cudaMemcpyDeviceToDevice,
      ctx.stream))) return MGPU_ERR_CUDA;
    return MGPU_OK;
  };
  for(int v = 0; v < nvar && !st; ++v) {
    ctx.tuning.set(primitive, key_type, vb, bucket, v);
    std::vector<float> times;
    for(int r = -1; r < reps && !st; ++r) {       // r == -1: warm-up
      st = restore();
      if(!st && ctx.check(cudaEventRecord(e0, ctx.stream))) st = MGPU_ERR_CUDA;
      if(!st) st = run_once();
      if(!st && ctx.check(cudaEventRecord(e1, ctx.stream))) st = MGPU_ERR_CUDA;
      if(!st) st = ctx.synchronize();
      float ms = 0;
      if(!st && r >= 0 && !ctx.check(cudaEventElapsedTime(&ms, e0, e1))) times.push_back(ms);
    }
    if(st) break;
    std::sort(times.begin(), times.end());
    double med = times.empty() ? 1e30 : times[times.size() / 2];
    if(med < best_t) { best_t = med; best = v; }
  }
  if(!st) {
    ctx.tuning.set(primitive, key_type, vb, bucket, best);
    if(best_variant) *best_variant = best;
    if(best_ms) *best_ms = best_t;
  }
  ctx.synchronize();
  if(e0) cudaEventDestroy(e0);
  if(e1) cudaEventDestroy(e1);
  for(char* p : buf) if(p) cudaFree(p);
  return st;
}

}  // extern "C"
