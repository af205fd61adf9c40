// Host cost of the device operations a plan's activation could make -- a
// MEASUREMENT DRIVER ONLY: a stream-ordered allocation from a memory pool
// (what plan tables used before the table arena) and a small kernel launch
// (the table writer), each warm and after a 64 MiB host sweep that evicts
// the caches; also cudaFreeAsync and cudaStreamQuery.  Medians of 200.
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O2 \
//       oracle/ref_bench/activation_cost.cu -o activation_cost && ./activation_cost
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <vector>

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

__global__ void fill(int* p, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = i;
}

}  // namespace

int main() {
  cudaStream_t s;
  if (cudaStreamCreate(&s) != cudaSuccess) return 1;
  cudaMemPool_t pool;
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = 0;
  if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) return 1;
  unsigned long long keep = 256ull << 20;
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  int* target = nullptr;
  if (cudaMalloc(&target, 1 << 20) != cudaSuccess) return 1;
  for (int cold = 0; cold < 2; ++cold) {
    std::vector<double> alloc, launch, release, query;
    for (int it = 0; it < 200; ++it) {
      void* d = nullptr;
      if (cold) sweep();
      auto t0 = Clock::now();
      cudaMallocFromPoolAsync(&d, 24576, pool, s);
      alloc.push_back(micros(t0, Clock::now()));
      if (cold) sweep();
      auto t1 = Clock::now();
      fill<<<24, 256, 0, s>>>(target, 6144);
      launch.push_back(micros(t1, Clock::now()));
      if (cold) sweep();
      auto t2 = Clock::now();
      cudaFreeAsync(d, s);
      release.push_back(micros(t2, Clock::now()));
      if (cold) sweep();
      auto t3 = Clock::now();
      cudaStreamQuery(s);
      query.push_back(micros(t3, Clock::now()));
      cudaStreamSynchronize(s);
    }
    std::printf("%s: pool allocation %.2f  launch %.2f  cudaFreeAsync %.2f  cudaStreamQuery %.2f us\n",
                cold ? "cold" : "warm", median(alloc), median(launch), median(release),
                median(query));
  }
  cudaFree(target);
  return 0;
}
