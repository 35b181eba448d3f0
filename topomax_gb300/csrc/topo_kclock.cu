// The kernel clock's process-wide state and its C ABI (topo_kclock.h).
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>

#include "topo_kclock.h"
#include "topomax_gb300.h"

namespace topo {
KClockState& kclock() {
  static KClockState k;
  return k;
}
}  // namespace topo

namespace {
struct Tot {
  long long launches = 0;
  double ms = 0.0, bytes = 0.0;
};
std::map<std::pair<std::string, int>, Tot>& totals() {
  static std::map<std::pair<std::string, int>, Tot> t;
  return t;
}
std::string& report_text() {
  static std::string r;
  return r;
}
// fold the recorded launches into the totals (waits for their events)
int fold() {
  auto& k = topo::kclock();
  int rc = TOPO_OK;
  for (auto& r : k.recs) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.e1) != cudaSuccess || cudaEventElapsedTime(&ms, r.e0, r.e1) != cudaSuccess)
      rc = TOPO_ERR_CUDA;
    Tot& t = totals()[{r.family, r.level}];
    t.launches += 1;
    t.ms += ms;
    t.bytes += r.bytes;
    cudaEventDestroy(r.e0);
    cudaEventDestroy(r.e1);
  }
  k.recs.clear();
  return rc;
}
}  // namespace

extern "C" int topo_kernel_clock(int enable) {
  auto& k = topo::kclock();
  if (enable) {
    fold();
    totals().clear();
    k.on = true;
  } else {
    k.on = false;
  }
  return TOPO_OK;
}

extern "C" int64_t topo_kernel_clock_report(char* buf, int64_t len) {
  if (fold() != TOPO_OK) return TOPO_ERR_CUDA;
  std::string& s = report_text();
  s.clear();
  char line[256];
  for (const auto& kv : totals()) {
    std::snprintf(line, sizeof(line), "%s\t%d\t%lld\t%.6f\t%.0f\n", kv.first.first.c_str(), kv.first.second,
                  kv.second.launches, kv.second.ms, kv.second.bytes);
    s += line;
  }
  const int64_t need = int64_t(s.size()) + 1;
  if (buf && len >= need) std::memcpy(buf, s.c_str(), size_t(need));
  return need;
}
