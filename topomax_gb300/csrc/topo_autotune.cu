// Process-wide table of the march kernels' tuned segment lengths (MG<T>::autotune).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "topo_mg.h"
#include "topomax_gb300.h"

namespace topo {
std::mutex& seg_mutex() {
  static std::mutex m;
  return m;
}
std::map<std::tuple<int, int, int>, int>& seg_table() {
  static std::map<std::tuple<int, int, int>, int> t;
  return t;
}

int tuned_segment(int family, int nx, int ny) {
  std::lock_guard<std::mutex> g(seg_mutex());
  auto it = seg_table().find({family, nx, ny});
  return it == seg_table().end() ? 0 : it->second;
}

void set_tuned_segment(int family, int nx, int ny, int seg) {
  std::lock_guard<std::mutex> g(seg_mutex());
  seg_table()[{family, nx, ny}] = seg;
}

bool autotune_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("TOPO_AUTOTUNE");
    return !(e && e[0] == '0');
  }();
  return on;
}
}  // namespace topo

// The tuned tiles as text, one line per kernel family and grid:
// "family<TAB>nx<TAB>ny<TAB>segment<LF>" (family: P2 or P1 march, precision, components).
extern "C" int64_t topo_march_tiles_report(char* buf, int64_t len) {
  std::string s;
  {
    std::lock_guard<std::mutex> g(topo::seg_mutex());
    for (const auto& kv : topo::seg_table()) {
      const int fam = std::get<0>(kv.first);
      char name[64];
      std::snprintf(name, sizeof(name), "%s %s NC=%d", (fam & 8) ? "P1 march" : "P2 march", (fam & 4) ? "FP64" : "FP32",
                    fam & 3);
      char line[160];
      std::snprintf(line, sizeof(line), "%s\t%d\t%d\t%d\n", name, std::get<1>(kv.first), std::get<2>(kv.first),
                    kv.second);
      s += line;
    }
  }
  const int64_t need = int64_t(s.size()) + 1;
  if (buf && len >= need) std::memcpy(buf, s.c_str(), size_t(need));
  return need;
}
