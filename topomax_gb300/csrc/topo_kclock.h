// Opt-in kernel clock for per-family bandwidth figures (a measurement hook, off
// by default).  While it is on (topo_kernel_clock), every launch wrapped in a
// KClock scope is bracketed by two CUDA events on its stream and recorded with
// its family name, its level and its algorithmic bytes; topo_kernel_clock_report
// sums them per (family, level).  Meant for host-driven runs (TOPO_GRAPHS=0): a
// scope on a stream that is being captured records nothing, so graph-recorded
// solves are never touched.
#pragma once

#include <cuda_runtime.h>

#include <vector>

namespace topo {

struct KClockRec {
  const char* family;
  int level;
  double bytes;
  cudaEvent_t e0, e1;
};

struct KClockState {
  bool on = false;
  std::vector<KClockRec> recs;
};

KClockState& kclock();  // process-wide (topo_kclock.cu)

class KClock {
 public:
  KClock(cudaStream_t s, const char* family, int level, double bytes) : s_(s) {
    KClockState& k = kclock();
    if (!k.on) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
    rec_ = KClockRec{family, level, bytes, nullptr, nullptr};
    if (cudaEventCreate(&rec_.e0) != cudaSuccess) return;
    if (cudaEventCreate(&rec_.e1) != cudaSuccess) {
      cudaEventDestroy(rec_.e0);
      return;
    }
    cudaEventRecord(rec_.e0, s);
    active_ = true;
  }
  ~KClock() {
    if (!active_) return;
    cudaEventRecord(rec_.e1, s_);
    kclock().recs.push_back(rec_);
  }
  KClock(const KClock&) = delete;
  KClock& operator=(const KClock&) = delete;

 private:
  cudaStream_t s_;
  KClockRec rec_{};
  bool active_ = false;
};

}  // namespace topo
