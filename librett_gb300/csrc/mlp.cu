// Training and batch-inference kernels of the plan-selection MLP
// (NFEAT -> 128 -> 128 -> 128 -> 1, ReLU), exposed through the C-ABI on
// device pointers so that a driver (Python or C++) can run the training
// loop while every forward, backward, loss and optimiser step runs in these
// kernels.  The sizes are small (batch <= a few thousand rows, 128-wide
// layers), so a plain tiled SIMT GEMM is used; there is no tensor-core path.
//
// Parameter layout (also used by the host inference in select.cpp): W1
// [128][NFEAT], b1 [128], W2 [128][128], b2, W3 [128][128], b3, W4 [1][128],
// b4 [1]; weights row-major [out][in].
#include <cuda_runtime.h>

#include <cmath>

#include "librett.h"
#include "librett_c.h"
#include "select.h"

namespace lt {
namespace {

constexpr int H = MLP_HIDDEN;
constexpr int BM = 64, BN = 64, BK = 16;

// C[M][N] = alpha * op(A) * op(B) + beta * C, row-major.
// op(A)(m,k) = TA ? A[k*lda + m] : A[m*lda + k]
// op(B)(k,n) = TB ? B[n*ldb + k] : B[k*ldb + n]
template <bool TA, bool TB>
__global__ void __launch_bounds__(256)
sgemmKernel(int M, int N, int K, float alpha, const float* __restrict__ A, int lda,
            const float* __restrict__ B, int ldb, float beta, float* __restrict__ C, int ldc) {
  __shared__ float As[BK][BM + 4];
  __shared__ float Bs[BK][BN + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int i = threadIdx.x; i < BM * BK; i += 256) {
      const int mm = i % BM, kk = i / BM;
      const int m = m0 + mm, k = k0 + kk;
      float v = 0.f;
      if (m < M && k < K) v = TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
      As[kk][mm] = v;
    }
    for (int i = threadIdx.x; i < BN * BK; i += 256) {
      const int nn = i % BN, kk = i / BN;
      const int n = n0 + nn, k = k0 + kk;
      float v = 0.f;
      if (n < N && k < K) v = TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n];
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx * 4 + j;
      if (n >= N) continue;
      float* c = C + (size_t)m * ldc + n;
      *c = alpha * acc[i][j] + (beta == 0.f ? 0.f : beta * *c);
    }
  }
}

cudaError_t sgemm(bool ta, bool tb, int M, int N, int K, float alpha, const float* A, int lda,
                  const float* B, int ldb, float beta, float* C, int ldc, cudaStream_t s) {
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
  if (ta && tb) sgemmKernel<true, true><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  else if (ta) sgemmKernel<true, false><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  else if (tb) sgemmKernel<false, true><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  else sgemmKernel<false, false><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  return cudaGetLastError();
}

// Y[b][o] = act(Y[b][o] + bias[o])
__global__ void biasActKernel(float* Y, const float* bias, int rows, int cols, int relu) {
  const size_t n = (size_t)rows * cols;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    float v = Y[i] + bias[i % cols];
    Y[i] = (relu && v < 0.f) ? 0.f : v;
  }
}

// dZ = dA where the layer's activation A is positive, else 0 (ReLU').
__global__ void reluMaskKernel(float* dA, const float* A, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    if (!(A[i] > 0.f)) dA[i] = 0.f;
}

// out[o] = sum_b D[b][o]; one block per column.
__global__ void colSumKernel(const float* D, int rows, int cols, float* out) {
  __shared__ float red[256];
  const int o = blockIdx.x;
  float s = 0.f;
  for (int b = threadIdx.x; b < rows; b += blockDim.x) s += D[(size_t)b * cols + o];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[o] = red[0];
}

// dout[b] = 2 (out[b] - y[b]) / batch; *loss += sum (out - y)^2 / batch.
__global__ void mseGradKernel(const float* out, const float* y, int batch, float* dout,
                              float* loss) {
  __shared__ float red[256];
  float s = 0.f;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < batch; b += gridDim.x * blockDim.x) {
    const float d = out[b] - y[b];
    dout[b] = 2.f * d / batch;
    s += d * d / batch;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0 && loss != nullptr) atomicAdd(loss, red[0]);
}

// Adam (Kingma & Ba, 2015) with bias correction.
__global__ void adamKernel(float* p, const float* g, float* m, float* v, int n, float lr,
                           float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

int gridFor(size_t n) {
  size_t g = (n + 255) / 256;
  return (int)(g > 4096 ? 4096 : (g < 1 ? 1 : g));
}

struct Layout {
  const float *W1, *b1, *W2, *b2, *W3, *b3, *W4, *b4;
};

Layout layout(const float* p) {
  Layout L;
  L.W1 = p;
  L.b1 = L.W1 + H * NFEAT;
  L.W2 = L.b1 + H;
  L.b2 = L.W2 + H * H;
  L.W3 = L.b2 + H;
  L.b3 = L.W3 + H * H;
  L.W4 = L.b3 + H;
  L.b4 = L.W4 + H;
  return L;
}

}  // namespace
}  // namespace lt

extern "C" {

int librett_c_mlp_param_count(void) { return lt::mlpParamCount(); }

int librett_c_mlp_feature_count(void) { return lt::NFEAT; }

int librett_c_mlp_workspace_floats(int batch) { return 5 * batch * lt::H; }

int librett_c_mlp_forward(const float* params, const float* X, int batch, float* ws, float* out,
                          void* stream) {
  using namespace lt;
  if (!params || !X || !ws || !out || batch < 1) return LIBRETT_INVALID_PARAMETER;
  cudaStream_t s = (cudaStream_t)stream;
  const Layout L = layout(params);
  float* A1 = ws;
  float* A2 = A1 + (size_t)batch * H;
  float* A3 = A2 + (size_t)batch * H;
  const int g = gridFor((size_t)batch * H);
  if (sgemm(false, true, batch, H, NFEAT, 1.f, X, NFEAT, L.W1, NFEAT, 0.f, A1, H, s)) return LIBRETT_INTERNAL_ERROR;
  biasActKernel<<<g, 256, 0, s>>>(A1, L.b1, batch, H, 1);
  if (sgemm(false, true, batch, H, H, 1.f, A1, H, L.W2, H, 0.f, A2, H, s)) return LIBRETT_INTERNAL_ERROR;
  biasActKernel<<<g, 256, 0, s>>>(A2, L.b2, batch, H, 1);
  if (sgemm(false, true, batch, H, H, 1.f, A2, H, L.W3, H, 0.f, A3, H, s)) return LIBRETT_INTERNAL_ERROR;
  biasActKernel<<<g, 256, 0, s>>>(A3, L.b3, batch, H, 1);
  if (sgemm(false, true, batch, 1, H, 1.f, A3, H, L.W4, H, 0.f, out, 1, s)) return LIBRETT_INTERNAL_ERROR;
  biasActKernel<<<gridFor(batch), 256, 0, s>>>(out, L.b4, batch, 1, 0);
  return cudaGetLastError() == cudaSuccess ? LIBRETT_SUCCESS : LIBRETT_INTERNAL_ERROR;
}

int librett_c_mlp_backward(const float* params, const float* X, int batch, float* ws,
                           const float* dout, float* grads, void* stream) {
  using namespace lt;
  if (!params || !X || !ws || !dout || !grads || batch < 1) return LIBRETT_INVALID_PARAMETER;
  cudaStream_t s = (cudaStream_t)stream;
  const Layout L = layout(params);
  float* gW1 = grads;
  float* gb1 = gW1 + H * NFEAT;
  float* gW2 = gb1 + H;
  float* gb2 = gW2 + H * H;
  float* gW3 = gb2 + H;
  float* gb3 = gW3 + H * H;
  float* gW4 = gb3 + H;
  float* gb4 = gW4 + H;
  const float* A1 = ws;
  const float* A2 = A1 + (size_t)batch * H;
  const float* A3 = A2 + (size_t)batch * H;
  float* dA = ws + 3 * (size_t)batch * H;
  float* dB = dA + (size_t)batch * H;
  const size_t n = (size_t)batch * H;
  const int g = gridFor(n);
  // output layer
  if (sgemm(true, false, 1, H, batch, 1.f, dout, 1, A3, H, 0.f, gW4, H, s)) return LIBRETT_INTERNAL_ERROR;
  colSumKernel<<<1, 256, 0, s>>>(dout, batch, 1, gb4);
  if (sgemm(false, false, batch, H, 1, 1.f, dout, 1, L.W4, H, 0.f, dA, H, s)) return LIBRETT_INTERNAL_ERROR;
  reluMaskKernel<<<g, 256, 0, s>>>(dA, A3, n);
  // layer 3
  if (sgemm(true, false, H, H, batch, 1.f, dA, H, A2, H, 0.f, gW3, H, s)) return LIBRETT_INTERNAL_ERROR;
  colSumKernel<<<H, 256, 0, s>>>(dA, batch, H, gb3);
  if (sgemm(false, false, batch, H, H, 1.f, dA, H, L.W3, H, 0.f, dB, H, s)) return LIBRETT_INTERNAL_ERROR;
  reluMaskKernel<<<g, 256, 0, s>>>(dB, A2, n);
  // layer 2
  if (sgemm(true, false, H, H, batch, 1.f, dB, H, A1, H, 0.f, gW2, H, s)) return LIBRETT_INTERNAL_ERROR;
  colSumKernel<<<H, 256, 0, s>>>(dB, batch, H, gb2);
  if (sgemm(false, false, batch, H, H, 1.f, dB, H, L.W2, H, 0.f, dA, H, s)) return LIBRETT_INTERNAL_ERROR;
  reluMaskKernel<<<g, 256, 0, s>>>(dA, A1, n);
  // layer 1
  if (sgemm(true, false, H, NFEAT, batch, 1.f, dA, H, X, NFEAT, 0.f, gW1, NFEAT, s)) return LIBRETT_INTERNAL_ERROR;
  colSumKernel<<<H, 256, 0, s>>>(dA, batch, H, gb1);
  return cudaGetLastError() == cudaSuccess ? LIBRETT_SUCCESS : LIBRETT_INTERNAL_ERROR;
}

int librett_c_mlp_mse_grad(const float* out, const float* y, int batch, float* dout, float* loss,
                           void* stream) {
  if (!out || !y || !dout || batch < 1) return LIBRETT_INVALID_PARAMETER;
  lt::mseGradKernel<<<lt::gridFor(batch), 256, 0, (cudaStream_t)stream>>>(out, y, batch, dout,
                                                                            loss);
  return cudaGetLastError() == cudaSuccess ? LIBRETT_SUCCESS : LIBRETT_INTERNAL_ERROR;
}

int librett_c_mlp_adam(float* params, const float* grads, float* m, float* v, int n, float lr,
                       float beta1, float beta2, float eps, int step, void* stream) {
  if (!params || !grads || !m || !v || n < 1 || step < 1) return LIBRETT_INVALID_PARAMETER;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  lt::adamKernel<<<lt::gridFor(n), 256, 0, (cudaStream_t)stream>>>(params, grads, m, v, n, lr,
                                                                     beta1, beta2, eps, c1, c2);
  return cudaGetLastError() == cudaSuccess ? LIBRETT_SUCCESS : LIBRETT_INTERNAL_ERROR;
}

}  // extern "C"
