// Process-wide table of the march kernels' tuned segment lengths (MG<T>::autotune).
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include "topo_mg.h"

namespace topo {
namespace {
std::mutex& seg_mutex() {
  static std::mutex m;
  return m;
}
std::map<std::tuple<int, int, int>, int>& seg_table() {
  static std::map<std::tuple<int, int, int>, int> t;
  return t;
}
}  // namespace

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
