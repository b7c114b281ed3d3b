// Host-only checks of the launch-shape tuning table (no CUDA needed): size
// buckets, lookup precedence, and the text format's save / load round trip.
#include "mgpu/gb300/tuning.hxx"

#include <cstdio>
#include <cstdlib>

using mgpu::gb300::size_bucket;
using mgpu::gb300::tuning_table_t;

static int failures = 0;
#define CHECK(x) do { if(!(x)) { std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #x); \
  ++failures; } } while(0)

int main(int argc, char** argv) {
  const char* path = argc > 1 ? argv[1] : "tuning_table.txt";

  CHECK(size_bucket(0) == 0);
  CHECK(size_bucket(1) == 0);
  CHECK(size_bucket(2) == 1);
  CHECK(size_bucket(3) == 2);
  CHECK(size_bucket(1 << 20) == 20);
  CHECK(size_bucket((1 << 20) + 1) == 21);
  CHECK(size_bucket(int64_t(1) << 62) == 62);
  CHECK(size_bucket(INT64_MAX) == 62);

  tuning_table_t t;
  CHECK(t.lookup(0, 1, 4, 1000) == 0);            // empty: the default shape
  t.set(0, 1, 4, -1, 2);                           // any size
  t.set(0, 1, 4, 20, 3);                           // 2^19 < count <= 2^20
  CHECK(t.lookup(0, 1, 4, 1 << 20) == 3);          // the size's own entry wins
  CHECK(t.lookup(0, 1, 4, (1 << 20) + 1) == 2);    // else the any-size entry
  CHECK(t.lookup(0, 1, 0, 1 << 20) == 0);          // other value width: default
  CHECK(t.lookup(3, 1, 4, 1 << 20) == 0);          // other primitive: default
  t.set(0, 1, 4, 20, 1);                           // replaces
  CHECK(t.lookup(0, 1, 4, 1 << 20) == 1);

  CHECK(t.save(path));
  tuning_table_t u;
  CHECK(u.load(path));
  CHECK(u.entries == t.entries);

  // Comment lines and lines that are not five integers are skipped.
  FILE* f = std::fopen(path, "w");
  CHECK(f != nullptr);
  if(f) {
    std::fputs("# header\n2 5 8 -1 1\nnot a line\n2 5 8\n\n1 0 0 12 3\n", f);
    std::fclose(f);
  }
  tuning_table_t w;
  CHECK(w.load(path));
  CHECK(w.entries.size() == 2);
  CHECK(w.lookup(2, 5, 8, 77) == 1);
  CHECK(w.lookup(1, 0, 0, 4096) == 3);
  CHECK(!w.load("/nonexistent/dir/tuning_table.txt"));

  if(!failures) std::printf("ok tuning_table\n");
  return failures ? 1 : 0;
}
