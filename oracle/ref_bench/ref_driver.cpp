// Driver for LibreTT's own CUDA build -- TEST INFRASTRUCTURE ONLY.
//
// Links against the LibreTT library compiled unmodified from its sources by
// oracle/ref_bench/run_ref.py, and calls it only through its public API
// (librettPlan / librettPlanMeasure / librettExecute / librettDestroy,
// LibreTT src/librett.h:57-121).  Three modes:
//
//   ref_driver golden <cases> <outdir>
//       for each case, fill the input (LibreTT's test conventions: element i
//       holds i, or 32-bit word w holds w), plan with librettPlan, execute,
//       and write the output bytes to <outdir>/out_<n>.bin;
//   ref_driver bench <cases> <steps> <warmup> <measure:0|1>
//       for each case, plan (librettPlan, or librettPlanMeasure when
//       measure=1), then time <steps> executes after <warmup> untimed ones
//       with CUDA events on the plan's stream; print one JSON line per case;
//   ref_driver loop <cases> <steps> <warmup>
//       plan every case, then time the per-tensor loop (librettExecute on
//       every case in turn, each tensor at its own offset of one buffer);
//       print one JSON line;
//   ref_driver random <cases>
//       for each case (kind 3), fill the input on the device with the
//       seeded random words of oracle/vectors.py, plan with librettPlan,
//       execute, and write the output to standard output as an 8-byte
//       little-endian length followed by the bytes (the caller digests it).
//
// Case file: one case per line, "rank d0 .. d{r-1} p0 .. p{r-1} es kind"
// (kind 0 = value pattern, 1 = word pattern, 2 = leave memory as is,
// 3 = seeded random words; kind 3 is followed by the 64-bit key).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "librett.h"

namespace {

struct Case {
  std::vector<int> dim, perm;
  int es = 8;
  int kind = 0;
  unsigned long long key = 0;  // kind 3
};

std::vector<Case> readCases(const char* path) {
  std::vector<Case> out;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    int r;
    if (!(is >> r)) continue;
    Case c;
    c.dim.resize(r);
    c.perm.resize(r);
    for (int i = 0; i < r; ++i) is >> c.dim[i];
    for (int i = 0; i < r; ++i) is >> c.perm[i];
    is >> c.es >> c.kind;
    if (c.kind == 3) is >> c.key;
    out.push_back(c);
  }
  return out;
}

#define CHECK(x)                                                                     \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess) {                                                         \
      std::fprintf(stderr, "%s failed: %s\n", #x, cudaGetErrorString(e_));           \
      std::exit(2);                                                                  \
    }                                                                                \
  } while (0)

size_t volumeOf(const Case& c) {
  size_t v = 1;
  for (int d : c.dim) v *= (size_t)d;
  return v;
}

void fillHost(const Case& c, std::vector<unsigned char>& buf) {
  const size_t vol = volumeOf(c);
  buf.assign(vol * c.es, 0);
  if (c.kind == 1) {
    uint32_t* w = reinterpret_cast<uint32_t*>(buf.data());
    for (size_t i = 0; i < buf.size() / 4; ++i) w[i] = (uint32_t)i;
  } else if (c.es == 4) {
    int32_t* p = reinterpret_cast<int32_t*>(buf.data());
    for (size_t i = 0; i < vol; ++i) p[i] = (int32_t)i;
  } else if (c.es == 8) {
    int64_t* p = reinterpret_cast<int64_t*>(buf.data());
    for (size_t i = 0; i < vol; ++i) p[i] = (int64_t)i;
  } else {
    std::complex<double>* p = reinterpret_cast<std::complex<double>*>(buf.data());
    for (size_t i = 0; i < vol; ++i) p[i] = std::complex<double>((double)i, 0.0);
  }
}

// Word i of a seeded random input: SplitMix64's output function of
// key + (i + 1) * golden ratio (the definition in oracle/vectors.py).
__global__ void fillRandomKernel(unsigned long long* w, size_t n, unsigned long long key) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    unsigned long long z = key + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    w[i] = z ^ (z >> 31);
  }
}

int randomMode(const char* casePath) {
  std::vector<Case> cases = readCases(casePath);
  size_t maxBytes = 0;
  for (auto& c : cases) maxBytes = std::max(maxBytes, volumeOf(c) * c.es);
  const size_t maxWords = (maxBytes + 7) / 8;
  unsigned long long* din;
  void* dout;
  CHECK(cudaMalloc(&din, maxWords * 8));
  CHECK(cudaMalloc(&dout, maxBytes));
  unsigned char* host = nullptr;
  CHECK(cudaMallocHost(&host, maxBytes));
  cudaStream_t s;
  CHECK(cudaStreamCreate(&s));
  for (size_t n = 0; n < cases.size(); ++n) {
    Case& c = cases[n];
    if (c.kind != 3) {
      std::fprintf(stderr, "case %zu: random mode needs kind 3\n", n);
      return 3;
    }
    const size_t bytes = volumeOf(c) * c.es;
    fillRandomKernel<<<1024, 256, 0, s>>>(din, (bytes + 7) / 8, c.key);
    CHECK(cudaGetLastError());
    CHECK(cudaMemsetAsync(dout, 0xA5, bytes, s));
    librettHandle h;
    librettResult r = librettPlan(&h, (int)c.dim.size(), c.dim.data(), c.perm.data(), c.es, s);
    if (r == LIBRETT_SUCCESS) r = librettExecute(h, din, dout);
    if (r != LIBRETT_SUCCESS) {
      std::fprintf(stderr, "case %zu: plan/execute -> %d\n", n, (int)r);
      return 3;
    }
    CHECK(cudaStreamSynchronize(s));
    CHECK(cudaMemcpy(host, dout, bytes, cudaMemcpyDeviceToHost));
    librettDestroy(h);
    unsigned char len[8];
    for (int b = 0; b < 8; ++b) len[b] = (unsigned char)((unsigned long long)bytes >> (8 * b));
    if (std::fwrite(len, 1, 8, stdout) != 8 || std::fwrite(host, 1, bytes, stdout) != bytes)
      return 4;
    std::fflush(stdout);
  }
  CHECK(cudaFreeHost(host));
  CHECK(cudaFree(din));
  CHECK(cudaFree(dout));
  CHECK(cudaStreamDestroy(s));
  return 0;
}

int golden(const char* casePath, const char* outDir) {
  std::vector<Case> cases = readCases(casePath);
  cudaStream_t s;
  CHECK(cudaStreamCreate(&s));
  for (size_t n = 0; n < cases.size(); ++n) {
    Case& c = cases[n];
    const size_t bytes = volumeOf(c) * c.es;
    std::vector<unsigned char> host;
    fillHost(c, host);
    void *din, *dout;
    CHECK(cudaMalloc(&din, bytes));
    CHECK(cudaMalloc(&dout, bytes));
    CHECK(cudaMemcpy(din, host.data(), bytes, cudaMemcpyHostToDevice));
    librettHandle h;
    librettResult r = librettPlan(&h, (int)c.dim.size(), c.dim.data(), c.perm.data(), c.es, s);
    if (r != LIBRETT_SUCCESS) {
      std::fprintf(stderr, "case %zu: librettPlan -> %d\n", n, (int)r);
      return 3;
    }
    r = librettExecute(h, din, dout);
    if (r != LIBRETT_SUCCESS) {
      std::fprintf(stderr, "case %zu: librettExecute -> %d\n", n, (int)r);
      return 3;
    }
    CHECK(cudaStreamSynchronize(s));
    CHECK(cudaMemcpy(host.data(), dout, bytes, cudaMemcpyDeviceToHost));
    librettDestroy(h);
    CHECK(cudaFree(din));
    CHECK(cudaFree(dout));
    std::string path = std::string(outDir) + "/out_" + std::to_string(n) + ".bin";
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f || std::fwrite(host.data(), 1, bytes, f) != bytes) return 4;
    std::fclose(f);
  }
  CHECK(cudaStreamDestroy(s));
  return 0;
}

int bench(const char* casePath, int steps, int warmup, int measure) {
  std::vector<Case> cases = readCases(casePath);
  size_t maxBytes = 0;
  for (auto& c : cases) maxBytes = std::max(maxBytes, volumeOf(c) * c.es);
  void *din, *dout;
  CHECK(cudaMalloc(&din, maxBytes));
  CHECK(cudaMalloc(&dout, maxBytes));
  CHECK(cudaMemset(din, 0x3c, maxBytes));
  cudaStream_t s;
  CHECK(cudaStreamCreate(&s));
  cudaEvent_t e0, e1;
  CHECK(cudaEventCreate(&e0));
  CHECK(cudaEventCreate(&e1));
  for (size_t n = 0; n < cases.size(); ++n) {
    Case& c = cases[n];
    const size_t bytes = volumeOf(c) * c.es;
    librettHandle h;
    CHECK(cudaDeviceSynchronize());
    auto t0 = std::chrono::steady_clock::now();
    librettResult r =
        measure ? librettPlanMeasure(&h, (int)c.dim.size(), c.dim.data(), c.perm.data(), c.es, s,
                                     din, dout)
                : librettPlan(&h, (int)c.dim.size(), c.dim.data(), c.perm.data(), c.es, s);
    CHECK(cudaStreamSynchronize(s));
    double planMs =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (r != LIBRETT_SUCCESS) {
      std::fprintf(stderr, "case %zu: plan -> %d\n", n, (int)r);
      return 3;
    }
    for (int w = 0; w < warmup; ++w) librettExecute(h, din, dout);
    CHECK(cudaStreamSynchronize(s));
    CHECK(cudaEventRecord(e0, s));
    for (int k = 0; k < steps; ++k) librettExecute(h, din, dout);
    CHECK(cudaEventRecord(e1, s));
    CHECK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CHECK(cudaEventElapsedTime(&ms, e0, e1));
    ms /= steps;
    std::ostringstream js;
    js << "{\"case\": " << n << ", \"dims\": [";
    for (size_t i = 0; i < c.dim.size(); ++i) js << (i ? ", " : "") << c.dim[i];
    js << "], \"perm\": [";
    for (size_t i = 0; i < c.perm.size(); ++i) js << (i ? ", " : "") << c.perm[i];
    js << "], \"es\": " << c.es << ", \"measure\": " << measure << ", \"ms\": " << ms
       << ", \"gbs\": " << (2.0 * bytes / (ms * 1e-3) / 1e9) << ", \"plan_ms\": " << planMs << "}";
    std::printf("%s\n", js.str().c_str());
    std::fflush(stdout);
    librettDestroy(h);
  }
  return 0;
}

// All cases planned up front, each tensor at its own 256-byte-aligned offset
// of one input and one output buffer; one step = librettExecute on every
// case in order (the per-tensor loop a grouped execution replaces).
int loop(const char* casePath, int steps, int warmup) {
  std::vector<Case> cases = readCases(casePath);
  std::vector<size_t> off(cases.size());
  size_t total = 0, algBytes = 0;
  for (size_t n = 0; n < cases.size(); ++n) {
    off[n] = total;
    const size_t b = volumeOf(cases[n]) * cases[n].es;
    algBytes += 2 * b;
    total += (b + 255) / 256 * 256;
  }
  unsigned char *din, *dout;
  CHECK(cudaMalloc(&din, total + 256));
  CHECK(cudaMalloc(&dout, total + 256));
  CHECK(cudaMemset(din, 0x3c, total + 256));
  cudaStream_t s;
  CHECK(cudaStreamCreate(&s));
  std::vector<librettHandle> h(cases.size());
  auto t0 = std::chrono::steady_clock::now();
  for (size_t n = 0; n < cases.size(); ++n) {
    Case& c = cases[n];
    librettResult r = librettPlan(&h[n], (int)c.dim.size(), c.dim.data(), c.perm.data(), c.es, s);
    if (r != LIBRETT_SUCCESS) {
      std::fprintf(stderr, "case %zu: plan -> %d\n", n, (int)r);
      return 3;
    }
  }
  CHECK(cudaStreamSynchronize(s));
  const double planS =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  auto step = [&]() {
    for (size_t n = 0; n < cases.size(); ++n)
      if (librettExecute(h[n], din + off[n], dout + off[n]) != LIBRETT_SUCCESS) return false;
    return true;
  };
  for (int w = 0; w < warmup; ++w)
    if (!step()) return 3;
  CHECK(cudaStreamSynchronize(s));
  cudaEvent_t e0, e1;
  CHECK(cudaEventCreate(&e0));
  CHECK(cudaEventCreate(&e1));
  CHECK(cudaEventRecord(e0, s));
  for (int k = 0; k < steps; ++k)
    if (!step()) return 3;
  CHECK(cudaEventRecord(e1, s));
  CHECK(cudaEventSynchronize(e1));
  float ms = 0.f;
  CHECK(cudaEventElapsedTime(&ms, e0, e1));
  ms /= steps;
  std::printf("{\"mode\": \"loop\", \"transposes\": %zu, \"ms_per_step\": %.4f, "
              "\"transposes_per_s\": %.1f, \"gbs\": %.3f, \"plan_s\": %.3f}\n",
              cases.size(), ms, cases.size() / (ms * 1e-3), algBytes / (ms * 1e-3) / 1e9, planS);
  std::fflush(stdout);
  for (librettHandle x : h) librettDestroy(x);
  CHECK(cudaFree(din));
  CHECK(cudaFree(dout));
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc >= 5 && std::strcmp(argv[1], "loop") == 0)
    return loop(argv[2], std::atoi(argv[3]), std::atoi(argv[4]));
  if (argc >= 4 && std::strcmp(argv[1], "golden") == 0) return golden(argv[2], argv[3]);
  if (argc >= 3 && std::strcmp(argv[1], "random") == 0) return randomMode(argv[2]);
  if (argc >= 6 && std::strcmp(argv[1], "bench") == 0)
    return bench(argv[2], std::atoi(argv[3]), std::atoi(argv[4]), std::atoi(argv[5]));
  std::fprintf(stderr,
               "usage: ref_driver golden <cases> <outdir> | bench <cases> <steps> <warmup> "
               "<measure> | loop <cases> <steps> <warmup> | random <cases>\n");
  return 1;
}
