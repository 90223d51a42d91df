// Autotuner of the serving engine's solver launches: warps per k-mode (1, 2
// or 4) from measured seconds per mode-step.  Host-only code (no CUDA),
// included by engine.cu and compiled on its own by the CPU tests.
#pragma once

#include <algorithm>
#include <cmath>

namespace bolt {

// Seconds per mode-step by warps per mode, in two tables.  An isolated
// launch (the GPU otherwise idle, nothing waiting) is keyed by its own size:
// a small one is bound by its longest mode's chain of dependent steps, where
// more warps per mode win.  A shared launch (other lanes' modes in flight or
// requests waiting) is keyed by the whole load -- its modes, the other lanes'
// and the waiting ones -- because the GPU stays full and the FP64 issue
// rate, where one warp per mode wins, sets the pace.
struct Tuner {
  double sps[2][48][3];
  int n[2][48][3];
  int picks[2][48];
  Tuner() {
    for (int t = 0; t < 2; ++t)
      for (int b = 0; b < 48; ++b) {
        picks[t][b] = 0;
        for (int v = 0; v < 3; ++v) { sps[t][b][v] = 0.0; n[t][b][v] = 0; }
      }
  }
  static int bucket(int nmodes) {
    int b = 0;
    while ((1 << (b + 1)) <= nmodes && b < 47) ++b;
    return b;
  }
  static int vidx(int wpm) { return wpm == 1 ? 0 : (wpm == 2 ? 1 : 2); }
  // Prior relative cost per mode-step of 4 / 2 / 1 warps per mode.  Isolated:
  // against the launch size in modes per SM, interpolated in log size
  // between two measurements (N = 473: 7.9 modes/SM -> 1.00 / 1.20 / 1.69,
  // 31.6 modes/SM -> 1.00 / 0.73 / 0.64).  Shared: the saturated ratios
  // (the 31.6 modes/SM figures).
  static void prior(bool shared, double r, double* c) {
    double t = shared ? 1.0 : (std::log(std::max(r, 1e-3)) - std::log(7.9)) / (std::log(31.6) - std::log(7.9));
    t = std::min(1.0, std::max(-1.0, t));
    c[2] = 1.0;                           // 4 warps
    c[1] = 1.20 + (0.73 - 1.20) * t;      // 2 warps
    c[0] = 1.69 + (0.64 - 1.69) * t;      // 1 warp
  }
  // The variant with the lowest estimated cost: measured seconds per
  // mode-step in this bucket where available, else the prior scaled by a
  // measured variant; every eighth launch of a bucket tries the runner-up so
  // the estimates keep up with the workload.  key = own modes (isolated) or
  // the whole load (shared).
  int pick(bool shared, int key, int nsm) {
    const double r = double(key) / double(nsm);
    // one wave onto an otherwise idle GPU: the lowest-latency variant.  Not
    // for a shared launch: one that starts small keeps its variant while the
    // GPU fills up and then runs as the slow tail of the load.
    if (!shared && r <= 2.0) return 4;
    double c[3];
    prior(shared, r, c);
    const int t = shared ? 1 : 0, b = bucket(key);
    double base = 0.0;
    for (int v = 0; v < 3; ++v)
      if (n[t][b][v] > 0) { base = sps[t][b][v] / c[v]; break; }
    double est[3];
    for (int v = 0; v < 3; ++v) est[v] = n[t][b][v] > 0 ? sps[t][b][v] : (base > 0 ? base * c[v] : c[v]);
    int order[3] = {0, 1, 2};
    std::sort(order, order + 3, [&](int x, int y) { return est[x] < est[y]; });
    const int v = (++picks[t][b] % 8 == 0) ? order[1] : order[0];
    return v == 0 ? 1 : (v == 1 ? 2 : 4);
  }
  void update(bool shared, int key, int wpm, double secs, double steps) {
    if (!(steps > 0) || !(secs > 0)) return;
    const int t = shared ? 1 : 0, b = bucket(key), v = vidx(wpm);
    double x = secs / steps;
    sps[t][b][v] = n[t][b][v] == 0 ? x : 0.7 * sps[t][b][v] + 0.3 * x;
    ++n[t][b][v];
  }
};

}  // namespace bolt
