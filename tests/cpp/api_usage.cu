// Drop-in usage of the mgpu::gb300 C++ templates, written the way the
// reference's examples drive mgpu::vk (examples/vk_transform, vk_sort,
// vk_merge, vk_scan, vk_radix2): two-phase aux sizing, a context standing in
// for cmd_buffer_t, device lambdas for launch/transform, and a user
// comparator for mergesort.  Prints one "ok <name>" line per check and exits
// non-zero on the first mismatch.
#include "mgpu/gb300/merge.hxx"
#include "mgpu/gb300/radix.hxx"
#include "mgpu/gb300/scan.hxx"
#include "mgpu/gb300/transform.hxx"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace mgpu::gb300;

#define CHECK(cond, name)                                                      \
  do {                                                                         \
    if(!(cond)) { printf("FAIL %s\n", name); return 1; }                       \
    printf("ok %s\n", name);                                                   \
  } while(0)

// A user comparator: descending by absolute value (ties keep input order).
struct abs_greater_t {
  __device__ bool operator()(float a, float b) const { return fabsf(a) > fabsf(b); }
};

int main() {
  context_t context;
  cmd_buffer_t cmd_buffer(context);

  // launch + transform (examples/vk_transform/vk_transform.cxx:36-63).
  {
    const int count = 100, NT = 64;
    float a = 1.618f;
    float* x = context.alloc_gpu<float>(count);
    float* y = context.alloc_gpu<float>(count);
    transform(count, context, [=] __device__(int64_t i) { x[i] = 2 * i; y[i] = 2 * i + 1; });
    launch<NT>((count + NT - 1) / NT, context, [=] __device__(int tid, int cta) {
      int gid = tid + NT * cta;
      if(gid < count) y[gid] += a * x[gid];
    });
    transform(count, context, [=] __device__(int64_t i) { x[i] *= sqrtf(y[i]); });
    std::vector<float> host(count);
    context.memcpy(host.data(), x, sizeof(float) * count);
    if(context.synchronize()) return 2;
    bool ok = true;
    for(int i = 0; i < count; ++i) {
      float xi = 2.0f * i, yi = 2.0f * i + 1 + a * xi;
      ok &= fabsf(host[i] - xi * sqrtf(yi)) <= 1e-4f * fabsf(xi * sqrtf(yi)) + 1e-5f;
    }
    CHECK(ok, "launch_transform");
  }

  // mergesort_keys with a user comparator (stable), in the reference's
  // default launch shape <128, 7> (vk/mergesort.hxx).
  {
    const int count = 10000;
    std::vector<float> h(count);
    srand(1);
    for(auto& v : h) v = (float)(rand() % 2001 - 1000) / 8;
    float* gpu = context.alloc_gpu<float>(count);
    context.memcpy(gpu, h.data(), sizeof(float) * count);
    void* aux_data = nullptr;
    size_t aux_size = 0;
    mergesort_keys<128, 7>(aux_data, aux_size, cmd_buffer, gpu, count, abs_greater_t());
    aux_data = context.alloc_gpu(aux_size);
    mergesort_keys<128, 7>(aux_data, aux_size, cmd_buffer, gpu, count, abs_greater_t());
    std::vector<float> got(count);
    context.memcpy(got.data(), gpu, sizeof(float) * count);
    if(context.synchronize()) return 2;
    std::stable_sort(h.begin(), h.end(), [](float a, float b) { return fabsf(a) > fabsf(b); });
    CHECK(got == h, "mergesort_user_comparator");
  }

  // merge keys-only (examples/vk_merge/vk_merge.cxx:19-62).
  {
    const int a_count = 10000, b_count = 10000, count = a_count + b_count;
    std::vector<float> ah(a_count), bh(b_count);
    for(auto& v : ah) v = rand() % 100000;
    for(auto& v : bh) v = rand() % 100000;
    std::sort(ah.begin(), ah.end());
    std::sort(bh.begin(), bh.end());
    float* a = context.alloc_gpu<float>(a_count);
    float* b = context.alloc_gpu<float>(b_count);
    float* c = context.alloc_gpu<float>(count);
    context.memcpy(a, ah.data(), sizeof(float) * a_count);
    context.memcpy(b, bh.data(), sizeof(float) * b_count);
    void* aux_data = nullptr;
    size_t aux_size = 0;
    merge<128, 7>(aux_data, aux_size, cmd_buffer, a, a_count, b, b_count, c, less_t<float>());
    aux_data = context.alloc_gpu(aux_size);
    merge<128, 7>(aux_data, aux_size, cmd_buffer, a, a_count, b, b_count, c, less_t<float>());
    std::vector<float> got(count), ref(count);
    context.memcpy(got.data(), c, sizeof(float) * count);
    if(context.synchronize()) return 2;
    std::merge(ah.begin(), ah.end(), bh.begin(), bh.end(), ref.begin());
    CHECK(got == ref, "merge_keys");
  }

  // In-place exclusive scan (examples/vk_scan/vk_scan.cxx:13-61).
  {
    const int count = 10000;
    std::vector<int> h(count);
    for(int i = 0; i < count; ++i) h[i] = i;
    int* gpu = context.alloc_gpu<int>(count);
    context.memcpy(gpu, h.data(), sizeof(int) * count);
    void* aux_data = nullptr;
    size_t aux_size = 0;
    scan(aux_data, aux_size, context, gpu, count);
    aux_data = context.alloc_gpu(aux_size);
    scan(aux_data, aux_size, context, gpu, count);
    context.memcpy(h.data(), gpu, sizeof(int) * count);
    if(context.synchronize()) return 2;
    bool ok = true;
    for(int i = 0; i < count; ++i) ok &= h[i] == (int)((int64_t)i * (i - 1) / 2);
    CHECK(ok, "scan_exclusive_in_place");
    // The same call with the reference's explicit launch knobs and operator:
    // a different launch shape, so it is sized with its own first call.
    for(int i = 0; i < count; ++i) h[i] = i;
    context.memcpy(gpu, h.data(), sizeof(int) * count);
    void* aux_knobs = nullptr;
    size_t aux_knobs_size = 0;
    scan<128, 7>(aux_knobs, aux_knobs_size, context, gpu, count, 0, plus_t<int>());
    aux_knobs = context.alloc_gpu(aux_knobs_size);
    if(scan<128, 7>(aux_knobs, aux_knobs_size, context, gpu, count, 0, plus_t<int>())) return 3;
    context.memcpy(h.data(), gpu, sizeof(int) * count);
    if(context.synchronize()) return 2;
    ok = true;
    for(int i = 0; i < count; ++i) ok &= h[i] == (int)((int64_t)i * (i - 1) / 2);
    CHECK(ok, "scan_reference_template_shape");
  }

  // Keys-only radix sort, sorted six times (examples/vk_radix2/vk_radix2.cxx).
  {
    const int count = 256 * 32 * 32;
    std::vector<uint32_t> h(count), ref;
    for(auto& v : h) v = (uint32_t)rand();
    ref = h;
    std::sort(ref.begin(), ref.end());
    uint32_t* gpu = context.alloc_gpu<uint32_t>(count);
    context.memcpy(gpu, h.data(), sizeof(uint32_t) * count);
    void* aux_data = nullptr;
    size_t aux_size = 0;
    // The reference's benchmarked call shape (examples/vk_radix/vk_radix.cxx).
    radix_sort<256, 16, 8>(aux_data, aux_size, context, gpu, count);
    aux_data = context.alloc_gpu(aux_size);
    for(int i = 0; i < 6; ++i) radix_sort<256, 16, 8>(aux_data, aux_size, context, gpu, count);
    context.memcpy(h.data(), gpu, sizeof(uint32_t) * count);
    if(context.synchronize()) return 2;
    CHECK(h == ref, "radix_sort_keys");
  }

  // The reference's default radix_sort template, <128, 15, 4>: 4-bit digits
  // (eight passes), 128 threads, 16 keys per thread; the same permutation.
  {
    const int count = 1000003;
    std::vector<uint32_t> h(count), ref;
    for(auto& v : h) v = (uint32_t)rand() * 2654435761u;
    ref = h;
    std::sort(ref.begin(), ref.end());
    uint32_t* gpu = context.alloc_gpu<uint32_t>(count);
    context.memcpy(gpu, h.data(), sizeof(uint32_t) * count);
    void* aux_data = nullptr;
    size_t aux_size = 0;
    radix_sort<128, 15, 4>(aux_data, aux_size, context, gpu, count);
    aux_data = context.alloc_gpu(aux_size);
    const int64_t launches0 = context.launches;
    if(radix_sort<128, 15, 4>(aux_data, aux_size, context, gpu, count)) return 3;
    const int64_t launches = context.launches - launches0;
    context.memcpy(h.data(), gpu, sizeof(uint32_t) * count);
    if(context.synchronize()) return 2;
    CHECK(h == ref, "radix_sort_keys_4bit");
    // Histogram + eight 4-bit passes, where the 8-bit shape runs four.
    CHECK(launches == 9, "radix_sort_4bit_passes");
  }

  // merge_path_partitions with both bounds (vk/partition.hxx:9-20) into
  // buffers from a memcache_t (vk/context.hxx:110-134), against a host merge
  // path of the same bound.
  {
    const int na = 5000, nb = 3000, spacing = 128;
    std::vector<int> ha(na), hb(nb);
    srand(11);
    for(int& x : ha) x = rand() % 1000;
    for(int& x : hb) x = rand() % 1000;
    std::sort(ha.begin(), ha.end());
    std::sort(hb.begin(), hb.end());
    memcache_t cache(context);
    auto bufs = cache.allocate<4>({ sizeof(int) * na, sizeof(int) * nb, 0, 0 });
    const int np = (int)num_merge_partitions(na + nb, spacing);
    int* mp = (int*)context.alloc_gpu<int>(2 * np);
    int* da = (int*)bufs[0];
    int* db = (int*)bufs[1];
    context.memcpy(da, ha.data(), sizeof(int) * na);
    context.memcpy(db, hb.data(), sizeof(int) * nb);
    merge_path_partitions<bounds_lower>(cmd_buffer, da, na, db, nb, mp, spacing, less_t<int>());
    merge_path_partitions<bounds_upper>(context, da, na, db, nb, mp + np, spacing, less_t<int>());
    std::vector<int> hmp(2 * np);
    context.memcpy(hmp.data(), mp, sizeof(int) * 2 * np);
    if(context.synchronize()) return 2;
    bool ok = bufs[0] != nullptr && ((uintptr_t)bufs[1] & 255) == 0;
    for(int u = 0; u < 2; ++u) {
      for(int i = 0; i < np; ++i) {
        const int diag = std::min(i * spacing, na + nb);
        int lo = std::max(0, diag - nb), hi = std::min(diag, na);
        while(lo < hi) {
          const int mid = (lo + hi) / 2;
          const bool pred = u ? ha[mid] < hb[diag - 1 - mid] : !(hb[diag - 1 - mid] < ha[mid]);
          if(pred) lo = mid + 1; else hi = mid;
        }
        ok &= hmp[u * np + i] == lo;
      }
    }
    CHECK(ok, "merge_path_partitions_memcache");
  }
  return 0;
}
