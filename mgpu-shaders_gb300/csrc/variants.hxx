// Compiled launch-shape variants of each primitive, selected at run time by
// the context's tuning table (mgpu/gb300/tuning.hxx).  Variant 0 is the
// default.  Names are "<threads>x<items per thread>".
#pragma once

#include "mgpu_gb300.h"

namespace variants {

// radix_sort onesweep tiles: 8-bit digits at 3 CTAs/SM, 4-byte keys
// {384x19, 256x31, 256x23} (with 8-byte values each holds half the keys per
// thread), 8-byte keys {256x16, 256x12, 384x10}; then 4-bit digits (twice
// the passes, ranking in registers) {256x16/4b, 128x16/4b} for both.  The
// tuner thus picks the digit width as well as the shape.
inline int radix_count(int) { return 5; }
inline const char* radix_name(int key_bytes, int v) {
  static const char* n4[] = { "384x19", "256x31", "256x23", "256x16/4b", "128x16/4b" };
  static const char* n8[] = { "256x16", "256x12", "384x10", "256x16/4b", "128x16/4b" };
  return key_bytes == 4 ? n4[v] : n8[v];
}
inline int radix_digit_bits(int v) { return v >= 3 ? 4 : 8; }

// scan: threads x elements per thread, b = CTAs per SM; "p" = persistent
// with deferred look-back, "t" = one tile per CTA.
inline int scan_count(int) { return 4; }
inline const char* scan_name(int bytes, int v) {
  static const char* n4[] = { "256x32b4p", "512x32b2p", "256x16b6p", "256x32b4t" };
  static const char* n8[] = { "512x16b2p", "256x16b4p", "256x8b6p", "256x16b4t" };
  return bytes == 4 ? n4[v] : n8[v];
}

// merge / mergesort: 4-byte keys {256x15, 256x8, 256x16}; 8-byte keys
// {256x7, 128x8, 256x8} (odd shapes keep shared-memory strides odd).
inline int merge_count(int) { return 3; }
inline const char* merge_name(int bytes, int v) {
  static const char* n4[] = { "256x15", "256x8", "256x16" };
  static const char* n8[] = { "256x7", "128x8", "256x8" };
  return bytes == 4 ? n4[v] : n8[v];
}
// mergesort: 4-byte keys {256x15, 256x8, 256x17 (256x15 with 8-byte values,
// whose tile would not fit the blocksort's 48 KB of static shared memory)};
// 8-byte keys as merge.
inline const char* mergesort_name(int bytes, int v) {
  static const char* n4[] = { "256x15", "256x8", "256x17" };
  return bytes == 4 ? n4[v] : merge_name(bytes, v);
}

inline int dtype_bytes(mgpu_dtype_t t) {
  return (t == MGPU_I64 || t == MGPU_U64 || t == MGPU_F64) ? 8 : 4;
}

}  // namespace variants
