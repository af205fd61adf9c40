// Planning-latency breakdown of this engine -- MEASUREMENT DRIVER ONLY.
//
// For every problem of a case file (one per line: rank, element bytes, dims,
// permutation), with the analytic and then the learned selector and the plan
// cache off, it times
//   describe  librett_c_describe: host-only planning (fusion, candidate
//             enumeration, selection, completion of the chosen candidate);
//   plan      librett_c_plan: the same plus the plan's device tables (the
//             librettPlan path);
// warm (best of 10 repeats of the same problem) and cold (once, after a
// 64 MiB host sweep that evicts the caches), and the cold plan call followed
// by a stream synchronize.  After the cold plan, its first librett_c_execute
// and a second one are timed to completion (host clock around the call and a
// stream synchronize), so that work deferred from planning to the first
// execute would show as their difference.  Two controls: the first and
// second execute of a plan made warm (no sweep), and a third execute of the
// cold plan after another sweep (an executed plan, cold host caches).  Then
// librett_c_plan_measure, cold with the synchronize, on every 4th problem.
// Medians are printed.
//
// Build and run (from the repository root, after python -m librett_gb300.build):
//   python -c "from librett_gb300.learn import data
//   for d, p, es in data.problems(200, 424242): print(len(d), es, *d, *p)" > cases.txt
//   g++ -O2 -std=c++17 oracle/ref_bench/plan_latency.cpp -Iinclude \
//       -I/usr/local/cuda/include librett_gb300/librett.so \
//       -Wl,-rpath,$PWD/librett_gb300 -L/usr/local/cuda/lib64 -lcudart -o plan_latency
//   ./plan_latency cases.txt
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <fstream>
#include <vector>

#include <cuda_runtime.h>

#include "librett_c.h"

namespace {

using Clock = std::chrono::steady_clock;

double micros(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::micro>(b - a).count();
}

std::vector<char> sweepBuffer(64 << 20);
volatile long sweepSink;

void sweep() {
  long s = 0;
  for (size_t i = 0; i < sweepBuffer.size(); i += 64) {
    sweepBuffer[i]++;
    s += sweepBuffer[i];
  }
  sweepSink = s;
}

double median(std::vector<double> v) {
  std::sort(v.begin(), v.end());
  return v[v.size() / 2];
}

struct Case {
  int rank = 0, es = 0;
  std::vector<int> dim, perm;
};

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <cases>\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1]);
  std::vector<Case> cases;
  Case c;
  while (in >> c.rank >> c.es) {
    c.dim.resize(c.rank);
    c.perm.resize(c.rank);
    for (int& x : c.dim) in >> x;
    for (int& x : c.perm) in >> x;
    cases.push_back(c);
  }
  if (cases.empty()) return 2;
  cudaStream_t s;
  if (cudaStreamCreate(&s) != cudaSuccess) return 1;
  size_t maxBytes = 0;
  for (const Case& k : cases) {
    size_t v = (size_t)k.es;
    for (int d : k.dim) v *= (size_t)d;
    maxBytes = std::max(maxBytes, v);
  }
  void *a = nullptr, *b = nullptr;
  if (cudaMalloc(&a, maxBytes) != cudaSuccess || cudaMalloc(&b, maxBytes) != cudaSuccess) return 1;
  librett_c_set_plan_cache(0);
  for (int mode : {1, 2}) {
    librett_c_set_plan_selector(mode);
    std::vector<double> dWarm, dCold, pWarm, pCold, pColdSync, exFirst, exSecond, exDelta, warmDelta,
        sweptDelta;
    for (const Case& k : cases) {
      librett_plan_info info;
      double bd = 1e30, bp = 1e30;
      for (int r = 0; r < 10; ++r) {
        auto t0 = Clock::now();
        librett_c_describe(k.rank, k.dim.data(), k.perm.data(), k.es, 152, -1, &info);
        bd = std::min(bd, micros(t0, Clock::now()));
        librettHandle h;
        auto t1 = Clock::now();
        if (librett_c_plan(&h, k.rank, k.dim.data(), k.perm.data(), k.es, s) != 0) return 1;
        bp = std::min(bp, micros(t1, Clock::now()));
        librett_c_destroy(h);
        cudaStreamSynchronize(s);
      }
      dWarm.push_back(bd);
      pWarm.push_back(bp);
      sweep();
      auto t0 = Clock::now();
      librett_c_describe(k.rank, k.dim.data(), k.perm.data(), k.es, 152, -1, &info);
      dCold.push_back(micros(t0, Clock::now()));
      sweep();
      librettHandle h;
      auto t1 = Clock::now();
      if (librett_c_plan(&h, k.rank, k.dim.data(), k.perm.data(), k.es, s) != 0) return 1;
      auto t2 = Clock::now();
      cudaStreamSynchronize(s);
      pCold.push_back(micros(t1, t2));
      pColdSync.push_back(micros(t1, Clock::now()));
      double ex[2];
      for (double& e : ex) {
        auto t3 = Clock::now();
        if (librett_c_execute(h, a, b) != 0 || cudaStreamSynchronize(s) != cudaSuccess) return 1;
        e = micros(t3, Clock::now());
      }
      exFirst.push_back(ex[0]);
      exSecond.push_back(ex[1]);
      exDelta.push_back(ex[0] - ex[1]);
      sweep();
      auto t5 = Clock::now();
      if (librett_c_execute(h, a, b) != 0 || cudaStreamSynchronize(s) != cudaSuccess) return 1;
      sweptDelta.push_back(micros(t5, Clock::now()) - ex[1]);
      librett_c_destroy(h);
      cudaStreamSynchronize(s);
      // control: a plan made with warm caches, its first and second execute
      if (librett_c_plan(&h, k.rank, k.dim.data(), k.perm.data(), k.es, s) != 0) return 1;
      cudaStreamSynchronize(s);
      for (double& e : ex) {
        auto t3 = Clock::now();
        if (librett_c_execute(h, a, b) != 0 || cudaStreamSynchronize(s) != cudaSuccess) return 1;
        e = micros(t3, Clock::now());
      }
      warmDelta.push_back(ex[0] - ex[1]);
      librett_c_destroy(h);
      cudaStreamSynchronize(s);
    }
    std::printf("%s: describe warm %.1f cold %.1f | plan warm %.1f cold %.1f cold+sync %.1f us"
                " | first execute %.1f second %.1f first-second %.1f us | controls: warm plan"
                " first-second %.1f, executed plan after a sweep minus second %.1f us\n",
                mode == 1 ? "analytic" : "learned ", median(dWarm), median(dCold), median(pWarm),
                median(pCold), median(pColdSync), median(exFirst), median(exSecond),
                median(exDelta), median(warmDelta), median(sweptDelta));
  }
  std::vector<double> m;
  for (size_t i = 0; i < cases.size(); i += 4) {
    const Case& k = cases[i];
    sweep();
    librettHandle h;
    auto t0 = Clock::now();
    if (librett_c_plan_measure(&h, k.rank, k.dim.data(), k.perm.data(), k.es, s, a, b) != 0)
      return 1;
    cudaStreamSynchronize(s);
    m.push_back(micros(t0, Clock::now()));
    librett_c_destroy(h);
  }
  std::printf("plan_measure cold+sync %.1f us (median of %zu)\n", median(m), m.size());
  cudaFree(a);
  cudaFree(b);
  return 0;
}
