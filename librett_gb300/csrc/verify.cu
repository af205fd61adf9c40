// Device-side verifier: compares every output element of a transpose with
// the input element the transpose formula names, on the GPU, without a host
// copy of the tensors.  The role of LibreTT's device checker
// (src/TensorTester.cpp:47-126, checkTransposeKernel), which compares the
// output with an index pattern; this one compares with the actual input, so
// any input data works.
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "librett.h"
#include "librett_c.h"
#include "plan.h"

namespace lt {
namespace {

struct VerifyParams {
  int rank;
  unsigned long long vol;
  unsigned long long outD[MAXR];  // output-order dims (fused; may exceed 2^31)
  FastDiv outDim[MAXR];           // their fast dividers (dims below 2^31)
  long long inStride[MAXR];       // input stride of output rank i (elements)
};

// result[0]: mismatching elements; result[1]: smallest mismatching output index
template <int ES>
__global__ void __launch_bounds__(256)
verifyKernel(const __grid_constant__ VerifyParams p, const typename Word<ES>::T* __restrict__ in,
             const typename Word<ES>::T* __restrict__ out, unsigned long long* result) {
  using T = typename Word<ES>::T;
  unsigned long long bad = 0, first = ~0ull;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long q = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; q < p.vol;
       q += stride) {
    unsigned long long rem = q;
    long long src = 0;
    for (int i = 0; i < p.rank; ++i) {
      const unsigned long long d = p.outD[i];
      unsigned long long c;
      if (rem < (1ull << 31) && d < (1ull << 31)) {
        const uint32_t qq = fdiv((uint32_t)rem, p.outDim[i]);
        c = rem - (unsigned long long)qq * d;
        rem = qq;
      } else {
        c = rem % d;
        rem /= d;
      }
      src += (long long)c * p.inStride[i];
    }
    T a = in[src], b = out[q];
    bool same;
    if constexpr (ES == 4) {
      same = a == b;
    } else if constexpr (ES == 8) {
      same = a.x == b.x && a.y == b.y;
    } else {
      same = a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w;
    }
    if (!same) {
      ++bad;
      if (q < first) first = q;
    }
  }
  if (bad) {
    atomicAdd(result, bad);
    atomicMin(result + 1, first);
  }
}

}  // namespace
}  // namespace lt

extern "C" int librett_c_verify(int rank, const int* dim, const int* permutation,
                                size_t sizeofType, const void* idata, const void* odata,
                                void* stream, unsigned long long* mismatches,
                                long long* first_bad) {
  if (lt::checkInput(rank, dim, permutation, sizeofType) != 0 || idata == nullptr ||
      odata == nullptr || mismatches == nullptr)
    return LIBRETT_INVALID_PARAMETER;
  const size_t a = sizeofType < 16 ? sizeofType : 16;
  if ((uintptr_t)idata % a || (uintptr_t)odata % a) return LIBRETT_INVALID_PARAMETER;
  lt::Fused f;
  lt::fuseRanks(rank, dim, permutation, (int)sizeofType, f);
  lt::VerifyParams p{};
  p.rank = f.rank;
  p.vol = (unsigned long long)f.vol;
  for (int i = 0; i < f.rank; ++i) {
    const int r = f.perm[i];
    p.outD[i] = (unsigned long long)f.dim[r];
    p.outDim[i] = lt::makeFastDiv(f.dim[r] < (int64_t(1) << 31) ? (uint32_t)f.dim[r] : 1u);
    p.inStride[i] = f.sin[r];
  }
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long* d = nullptr;
  if (cudaMallocAsync(&d, 2 * sizeof(unsigned long long), s) != cudaSuccess)
    return LIBRETT_INTERNAL_ERROR;
  const unsigned long long init[2] = {0ull, ~0ull};
  unsigned long long host[2] = {0ull, ~0ull};
  cudaError_t err = cudaMemcpyAsync(d, init, sizeof(init), cudaMemcpyHostToDevice, s);
  int sms = 0, dev = 0;
  if (err == cudaSuccess) err = cudaGetDevice(&dev);
  if (err == cudaSuccess) err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (err == cudaSuccess) {
    unsigned long long blocks = (p.vol + 255) / 256;
    const unsigned long long cap = (unsigned long long)sms * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    switch (sizeofType) {
      case 4:
        lt::verifyKernel<4><<<(unsigned)blocks, 256, 0, s>>>(
            p, (const lt::Word<4>::T*)idata, (const lt::Word<4>::T*)odata, d);
        break;
      case 8:
        lt::verifyKernel<8><<<(unsigned)blocks, 256, 0, s>>>(
            p, (const lt::Word<8>::T*)idata, (const lt::Word<8>::T*)odata, d);
        break;
      default:
        lt::verifyKernel<16><<<(unsigned)blocks, 256, 0, s>>>(
            p, (const lt::Word<16>::T*)idata, (const lt::Word<16>::T*)odata, d);
        break;
    }
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = cudaMemcpyAsync(host, d, sizeof(host), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return LIBRETT_INTERNAL_ERROR;
  *mismatches = host[0];
  if (first_bad) *first_bad = host[0] ? (long long)host[1] : -1;
  return LIBRETT_SUCCESS;
}
