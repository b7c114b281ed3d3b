// Launch-parameter tuning table: which compiled (nt, vt) variant a primitive
// uses for a (key type, value width, size bucket).  The reference fixes these
// as template arguments per call site (radix_sort<nt, vt, num_bits>,
// vk/radix.hxx:195; mergesort/merge/scan <nt = 128, vt = 7>); here the C ABI
// carries several instantiations and the table picks one per call.  The
// autotuner (capi_tuning.cu) times the variants on the device and records the
// fastest; tables persist as text (one entry per line).
#pragma once

#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <tuple>

namespace mgpu {
namespace gb300 {

enum primitive_t : int { prim_radix = 0, prim_scan = 1, prim_merge = 2, prim_mergesort = 3,
  prim_count = 4 };

// Size bucket: ceil(log2(count)), 0 for count <= 1.
inline int size_bucket(int64_t count) {
  int b = 0;
  while(b < 62 && ((int64_t)1 << b) < count) ++b;
  return b;
}

struct tuning_table_t {
  // (primitive, key type, value bytes, bucket) -> variant; bucket -1 = any size.
  std::map<std::tuple<int, int, int, int>, int> entries;

  int lookup(int prim, int type, int val_bytes, int64_t count) const {
    auto it = entries.find(std::make_tuple(prim, type, val_bytes, size_bucket(count)));
    if(it != entries.end()) return it->second;
    it = entries.find(std::make_tuple(prim, type, val_bytes, -1));
    return it != entries.end() ? it->second : 0;
  }

  void set(int prim, int type, int val_bytes, int bucket, int variant) {
    entries[std::make_tuple(prim, type, val_bytes, bucket)] = variant;
  }

  bool save(const char* path) const {
    FILE* f = fopen(path, "w");
    if(!f) return false;
    fprintf(f, "# mgpu_gb300 tuning table: primitive key_type val_bytes size_bucket variant\n");
    for(auto& e : entries)
      fprintf(f, "%d %d %d %d %d\n", std::get<0>(e.first), std::get<1>(e.first),
        std::get<2>(e.first), std::get<3>(e.first), e.second);
    return fclose(f) == 0;
  }

  bool load(const char* path) {
    FILE* f = fopen(path, "r");
    if(!f) return false;
    char line[256];
    while(fgets(line, sizeof(line), f)) {
      if(line[0] == '#') continue;
      int p, t, v, b, var;
      if(sscanf(line, "%d %d %d %d %d", &p, &t, &v, &b, &var) == 5) set(p, t, v, b, var);
    }
    fclose(f);
    return true;
  }
};

}  // namespace gb300
}  // namespace mgpu
