// A small fully-connected network (FP32) trained on the GPU by hand-written
// kernels: forward, backward and Adam.  It predicts the next Newton initial
// guess of a parameter continuation from (node coordinates, parameter); the
// reference's own predictor (ac_conti.c ALC_ZEROTH / ALC_FIRST,
// src/ac_conti.c:759-784) stays the fallback and the converged Newton
// solve always decides.
//
// Layout: layer l maps width_in -> width_out with W_l [out][in] row-major and
// b_l [out]; hidden layers use tanh, the last is linear.  All parameters
// live in one flat FP32 buffer (and gradients / Adam moments in three more),
// so the host can read, write and checksum them in one copy.
//
// GEMMs are tiled SIMT FP32 (64 x 64 tiles, 4 x 4 per thread): at width 256
// and batches of a few thousand points one training step is a few GFLOP, far
// below the time of one Newton solve.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gb_newton.h"
#include "gb_context.h"

namespace gb {

constexpr int TM = 64, TN = 64, TK = 16;
constexpr int kMaxSplit = 32;  // batch splits of the weight-gradient product

// C[M][N] = A[M][K] * B^T where B is [N][K]  (i.e. X W^T), + bias[N],
// optional tanh.  Row-major everything.
__global__ void __launch_bounds__(256)
    gemm_xwT_kernel(int M, int N, int K, const float *__restrict__ A, const float *__restrict__ B,
                    const float *__restrict__ bias, float *__restrict__ C, int act) {
  __shared__ float As[TK][TM + 4];
  __shared__ float Bs[TK][TN + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += TK) {
    for (int t = threadIdx.x; t < TM * TK; t += 256) {
      const int mm = t / TK, kk = t % TK;
      const int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[(int64_t)gm * K + gk] : 0.f;
      const int gn = n0 + mm;
      Bs[kk][mm] = (gn < N && gk < K) ? B[(int64_t)gn * K + gk] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float v = acc[i][j] + (bias ? bias[gn] : 0.f);
      if (act) v = tanhf(v);
      C[(int64_t)gm * N + gn] = v;
    }
  }
}

// C[M][N] = A[M][K] * B[K][N]   (dH = dZ W)
__global__ void __launch_bounds__(256)
    gemm_xw_kernel(int M, int N, int K, const float *__restrict__ A, const float *__restrict__ B,
                   float *__restrict__ C) {
  __shared__ float As[TK][TM + 4];
  __shared__ float Bs[TK][TN + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += TK) {
    for (int t = threadIdx.x; t < TM * TK; t += 256) {
      const int mm = t / TK, kk = t % TK;
      const int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[(int64_t)gm * K + gk] : 0.f;
      const int kb = t / TN, nb = t % TN;
      const int gkb = k0 + kb, gnb = n0 + nb;
      Bs[kb][nb] = (gkb < K && gnb < N) ? B[(int64_t)gkb * N + gnb] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int gn = n0 + tx * 4 + j;
      if (gn < N) C[(int64_t)gm * N + gn] = acc[i][j];
    }
  }
}

// G[N][K] = D^T[N][M] * X[M][K]  (weight gradient dW = dZ^T H).  The batch
// M is split over blockIdx.z in chunks of mchunk rows; split z writes its
// partial sum to G + z N K (reduce_splits_kernel adds them in a fixed
// order, so the result is deterministic).
__global__ void __launch_bounds__(256)
    gemm_dTx_kernel(int M, int N, int K, const float *__restrict__ D, const float *__restrict__ X,
                    float *__restrict__ G, int mchunk) {
  __shared__ float Ds[TK][TM + 4];
  __shared__ float Xs[TK][TN + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int n0 = blockIdx.y * TM, k0c = blockIdx.x * TN;
  const int mb = blockIdx.z * mchunk, me = min(M, mb + mchunk);
  G += (int64_t)blockIdx.z * N * K;
  float acc[4][4] = {};
  for (int m0 = mb; m0 < me; m0 += TK) {
    for (int t = threadIdx.x; t < TM * TK; t += 256) {
      const int mm = t / TM, nn = t % TM;
      const int gm = m0 + mm;
      Ds[mm][nn] = (gm < me && n0 + nn < N) ? D[(int64_t)gm * N + n0 + nn] : 0.f;
      Xs[mm][nn] = (gm < me && k0c + nn < K) ? X[(int64_t)gm * K + k0c + nn] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int mm = 0; mm < TK; mm++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = Ds[mm][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Xs[mm][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int gn = n0 + ty * 4 + i;
    if (gn >= N) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int gk = k0c + tx * 4 + j;
      if (gk < K) G[(int64_t)gn * K + gk] = acc[i][j];
    }
  }
}

// g[i] = sum over the splits z (in order) of P[z][i]
__global__ void reduce_splits_kernel(int nsplit, int n, const float *__restrict__ P,
                                     float *__restrict__ g) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < nsplit; z++) s += P[(int64_t)z * n + i];
    g[i] = s;
  }
}

// column sums of D[M][N] -> g[N] (bias gradient), one block per column tile
__global__ void colsum_kernel(int M, int N, const float *__restrict__ D, float *__restrict__ g) {
  __shared__ float sh[256];
  const int n = blockIdx.x;
  float s = 0.f;
  for (int m = threadIdx.x; m < M; m += blockDim.x) s += D[(int64_t)m * N + n];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) g[n] = sh[0];
}

// dY = 2 mask (Y - T) / msum ; per-block partial of sum mask (Y-T)^2
__global__ void loss_grad_kernel(int n, const float *__restrict__ Y, const float *__restrict__ T,
                                 const float *__restrict__ mask, float inv_msum,
                                 float *__restrict__ dY, float *__restrict__ part) {
  __shared__ float sh[256];
  float s = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float d = (Y[i] - T[i]) * mask[i];
    dY[i] = 2.f * d * inv_msum;
    s += d * d;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// dZ = dH * (1 - H^2)
__global__ void tanh_back_kernel(int64_t n, const float *__restrict__ H, float *__restrict__ d) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    d[i] *= 1.f - H[i] * H[i];
}

__global__ void adam_kernel(int n, float *__restrict__ w, const float *__restrict__ g,
                            float *__restrict__ m, float *__restrict__ v, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// gather rows idx[b] of X[n][k] -> Xb[b][k]
__global__ void gather_rows_kernel(int B, int k, const int *__restrict__ idx,
                                   const float *__restrict__ X, float *__restrict__ Xb) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < B * k; t += gridDim.x * blockDim.x) {
    const int b = t / k, j = t - b * k;
    Xb[t] = X[(int64_t)idx[b] * k + j];
  }
}

struct Mlp {
  std::vector<int> width;  // n_in, hidden..., n_out
  int nparam = 0;
  std::vector<int> woff, boff;
  float *d_w = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;
  int cap = 0;                       // batch capacity of the activations
  std::vector<float *> act;          // per layer output [cap][width]
  float *d_dA = nullptr, *d_dB = nullptr;  // backward scratch [cap][maxw]
  float *d_part = nullptr, *h_part = nullptr;
  float *d_xb = nullptr, *d_tb = nullptr, *d_mb = nullptr;
  float *d_split = nullptr;          // weight-gradient partial sums [kMaxSplit][maxw][maxw]
  int *d_idx = nullptr;
  int adam_t = 0;
  int dev = 0;                       // the device the network lives on
  cudaStream_t st = nullptr;
  // orders a caller's stream after the network's own stream and back
  cudaEvent_t ev_own = nullptr, ev_caller = nullptr;
  ~Mlp() {
    cudaFree(d_w);
    cudaFree(d_g);
    cudaFree(d_m);
    cudaFree(d_v);
    for (float *a : act) cudaFree(a);
    cudaFree(d_dA);
    cudaFree(d_dB);
    cudaFree(d_part);
    cudaFree(d_xb);
    cudaFree(d_tb);
    cudaFree(d_mb);
    cudaFree(d_idx);
    cudaFree(d_split);
    if (h_part) cudaFreeHost(h_part);
    if (ev_own) cudaEventDestroy(ev_own);
    if (ev_caller) cudaEventDestroy(ev_caller);
    if (st) cudaStreamDestroy(st);
  }
  int maxw() const {
    int m = 0;
    for (int w : width) m = w > m ? w : m;
    return m;
  }
  int layers() const { return (int)width.size() - 1; }
  int ensure(int B) {
    if (B <= cap) return 0;
    for (float *a : act) cudaFree(a);
    act.assign(layers(), nullptr);
    cudaFree(d_dA);
    cudaFree(d_dB);
    cudaFree(d_xb);
    cudaFree(d_tb);
    cudaFree(d_mb);
    cudaFree(d_idx);
    for (int l = 0; l < layers(); l++)
      if (cudaMalloc(&act[l], sizeof(float) * (size_t)B * width[l + 1]) != cudaSuccess)
        return fail("MLP activations");
    const size_t mw = (size_t)B * maxw();
    if (cudaMalloc(&d_dA, sizeof(float) * mw) != cudaSuccess ||
        cudaMalloc(&d_dB, sizeof(float) * mw) != cudaSuccess ||
        cudaMalloc(&d_xb, sizeof(float) * (size_t)B * width[0]) != cudaSuccess ||
        cudaMalloc(&d_tb, sizeof(float) * (size_t)B * width.back()) != cudaSuccess ||
        cudaMalloc(&d_mb, sizeof(float) * (size_t)B * width.back()) != cudaSuccess ||
        cudaMalloc(&d_idx, sizeof(int) * (size_t)B) != cudaSuccess)
      return fail("MLP scratch");
    if (!d_split &&
        cudaMalloc(&d_split, sizeof(float) * (size_t)kMaxSplit * maxw() * maxw()) != cudaSuccess)
      return fail("MLP scratch");
    cap = B;
    return 0;
  }
  void forward(const float *X, int B) {
    const float *in = X;
    for (int l = 0; l < layers(); l++) {
      const int K = width[l], N = width[l + 1];
      dim3 grid((N + TN - 1) / TN, (B + TM - 1) / TM);
      gemm_xwT_kernel<<<grid, 256, 0, st>>>(B, N, K, in, d_w + woff[l], d_w + boff[l], act[l],
                                            l + 1 < layers() ? 1 : 0);
      in = act[l];
    }
  }
  // gradient of sum mask (Y - T)^2 / sum(mask) into d_g; with loss != NULL
  // also waits for and returns the loss (host)
  int backward(const float *X, const float *T, const float *Mk, int B, float msum, float *loss) {
    const int nl = layers(), no = width.back();
    const int nb = 64;
    loss_grad_kernel<<<nb, 256, 0, st>>>(B * no, act[nl - 1], T, Mk, 1.f / msum, d_dA, d_part);
    float *dcur = d_dA, *dnext = d_dB;
    for (int l = nl - 1; l >= 0; l--) {
      const int K = width[l], N = width[l + 1];
      const float *Hin = l == 0 ? X : act[l - 1];
      // dW_l = dZ^T Hin  [N][K], the batch split over up to kMaxSplit CTA
      // layers so that the grid covers the GPU; db_l = colsum dZ
      const int nsplit = std::max(1, std::min(kMaxSplit, B / 128));
      const int mchunk = ((B + nsplit - 1) / nsplit + TK - 1) / TK * TK;
      dim3 g1((K + TN - 1) / TN, (N + TM - 1) / TM, nsplit);
      if (nsplit == 1) {
        gemm_dTx_kernel<<<g1, 256, 0, st>>>(B, N, K, dcur, Hin, d_g + woff[l], mchunk);
      } else {
        gemm_dTx_kernel<<<g1, 256, 0, st>>>(B, N, K, dcur, Hin, d_split, mchunk);
        reduce_splits_kernel<<<(N * K + 255) / 256, 256, 0, st>>>(nsplit, N * K, d_split,
                                                                  d_g + woff[l]);
      }
      colsum_kernel<<<N, 256, 0, st>>>(B, N, dcur, d_g + boff[l]);
      if (l == 0) break;
      // dH_{l-1} = dZ W_l  [B][K]; dZ_{l-1} = dH * (1 - H^2)
      dim3 g2((K + TN - 1) / TN, (B + TM - 1) / TM);
      gemm_xw_kernel<<<g2, 256, 0, st>>>(B, K, N, dcur, d_w + woff[l], dnext);
      tanh_back_kernel<<<304, 256, 0, st>>>((int64_t)B * K, act[l - 1], dnext);
      float *t = dcur;
      dcur = dnext;
      dnext = t;
    }
    if (!loss) return 0;  // no loss wanted: nothing to wait for
    cudaMemcpyAsync(h_part, d_part, sizeof(float) * nb, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "MLP backward");
    double s = 0.0;
    for (int b = 0; b < nb; b++) s += h_part[b];
    if (loss) *loss = (float)(s / msum);
    return 0;
  }
  void adam(float lr, float b1, float b2, float eps) {
    adam_t++;
    const float c1 = 1.f - powf(b1, (float)adam_t), c2 = 1.f - powf(b2, (float)adam_t);
    adam_kernel<<<304, 256, 0, st>>>(nparam, d_w, d_g, d_m, d_v, lr, b1, b2, eps, c1, c2);
  }
};

}  // namespace gb

struct gb_mlp {
  gb::Mlp m;
};

extern "C" {

int gb_mlp_create(int n_in, int width, int hidden_layers, int n_out, unsigned long long seed,
                  gb_mlp **out) {
  if (!out || n_in <= 0 || width <= 0 || hidden_layers < 1 || n_out <= 0)
    return gb::fail("invalid MLP shape");
  *out = nullptr;
  gb_mlp *h = new (std::nothrow) gb_mlp;
  if (!h) return gb::fail("out of host memory");
  gb::Mlp &M = h->m;
  M.width.push_back(n_in);
  for (int l = 0; l < hidden_layers; l++) M.width.push_back(width);
  M.width.push_back(n_out);
  int off = 0;
  for (int l = 0; l < M.layers(); l++) {
    M.woff.push_back(off);
    off += M.width[l] * M.width[l + 1];
    M.boff.push_back(off);
    off += M.width[l + 1];
  }
  M.nparam = off;
  // Glorot-uniform weights from a fixed integer hash (splitmix64), zero biases
  std::vector<float> w(off, 0.f);
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + 1;
  auto next = [&]() {
    z += 0x9E3779B97F4A7C15ull;
    uint64_t r = z;
    r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ull;
    r = (r ^ (r >> 27)) * 0x94D049BB133111EBull;
    r ^= r >> 31;
    return (double)(r >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < M.layers(); l++) {
    const int fi = M.width[l], fo = M.width[l + 1];
    const double a = std::sqrt(6.0 / (fi + fo));
    for (int i = 0; i < fi * fo; i++) w[M.woff[l] + i] = (float)((2.0 * next() - 1.0) * a);
  }
  cudaError_t e = cudaGetDevice(&M.dev);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&M.st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&M.ev_own, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&M.ev_caller, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&M.d_w, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&M.d_g, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&M.d_m, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&M.d_v, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&M.d_part, sizeof(float) * 64);
  if (e == cudaSuccess) e = cudaMallocHost(&M.h_part, sizeof(float) * 64);
  if (e == cudaSuccess) e = cudaMemcpy(M.d_w, w.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(M.d_m, 0, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMemset(M.d_v, 0, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMemset(M.d_g, 0, sizeof(float) * off);
  if (e != cudaSuccess) {
    delete h;
    return gb::cuda_fail(e, "MLP create");
  }
  *out = h;
  return 0;
}

void gb_mlp_destroy(gb_mlp *m) { delete m; }

int gb_mlp_num_params(const gb_mlp *m) { return m ? m->m.nparam : -1; }

int gb_mlp_get_params(const gb_mlp *m, float *host) {
  if (!m || !host) return gb::fail("NULL argument");
  cudaError_t e = cudaMemcpy(host, m->m.d_w, sizeof(float) * m->m.nparam, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? 0 : gb::cuda_fail(e, "MLP params");
}

int gb_mlp_set_params(gb_mlp *m, const float *host) {
  if (!m || !host) return gb::fail("NULL argument");
  cudaError_t e = cudaMemcpy(m->m.d_w, host, sizeof(float) * m->m.nparam, cudaMemcpyHostToDevice);
  m->m.adam_t = 0;
  cudaMemset(m->m.d_m, 0, sizeof(float) * m->m.nparam);
  cudaMemset(m->m.d_v, 0, sizeof(float) * m->m.nparam);
  return e == cudaSuccess ? 0 : gb::cuda_fail(e, "MLP params");
}

int gb_mlp_get_grads(const gb_mlp *m, float *host) {
  if (!m || !host) return gb::fail("NULL argument");
  cudaError_t e = cudaMemcpy(host, m->m.d_g, sizeof(float) * m->m.nparam, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? 0 : gb::cuda_fail(e, "MLP grads");
}

int gb_mlp_forward_device(gb_mlp *m, const float *d_x, int B, float *d_y) {
  if (!m || !d_x || !d_y || B <= 0) return gb::fail("invalid argument");
  gb::Mlp &M = m->m;
  if (M.ensure(B)) return -1;
  M.forward(d_x, B);
  cudaError_t e = cudaMemcpyAsync(d_y, M.act.back(), sizeof(float) * (size_t)B * M.width.back(),
                                  cudaMemcpyDeviceToDevice, M.st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(M.st);
  return e == cudaSuccess ? 0 : gb::cuda_fail(e, "MLP forward");
}

int gb_mlp_loss_grad_device(gb_mlp *m, const float *d_x, const float *d_t, const float *d_mask,
                            int B, float *loss) {
  if (!m || !d_x || !d_t || !d_mask || B <= 0) return gb::fail("invalid argument");
  gb::Mlp &M = m->m;
  if (M.ensure(B)) return -1;
  // sum of the mask (host side would need a copy; compute on device)
  std::vector<float> hm((size_t)B * M.width.back());
  cudaError_t e = cudaMemcpy(hm.data(), d_mask, sizeof(float) * hm.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return gb::cuda_fail(e, "mask");
  double ms = 0.0;
  for (float v : hm) ms += v;
  if (ms <= 0.0) return gb::fail("empty loss mask");
  M.forward(d_x, B);
  return M.backward(d_x, d_t, d_mask, B, (float)ms, loss);
}

int gb_mlp_adam_step(gb_mlp *m, float lr, float beta1, float beta2, float eps) {
  if (!m) return gb::fail("NULL argument");
  m->m.adam(lr, beta1, beta2, eps);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : gb::cuda_fail(e, "Adam");
}

int gb_mlp_train_device(gb_mlp *m, const float *d_x, const float *d_t, const float *d_mask,
                        int n_points, int steps, int batch, float lr, unsigned long long seed,
                        float *final_loss) {
  if (!m || !d_x || !d_t || !d_mask || n_points <= 0 || steps <= 0 || batch <= 0)
    return gb::fail("invalid argument");
  gb::Mlp &M = m->m;
  const int B = batch < n_points ? batch : n_points;
  if (M.ensure(B)) return -1;
  const int ni = M.width[0], no = M.width.back();
  std::vector<int> idx(B);
  std::vector<float> hm((size_t)n_points * no);
  cudaError_t e = cudaMemcpy(hm.data(), d_mask, sizeof(float) * hm.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return gb::cuda_fail(e, "mask");
  uint64_t z = seed * 0xD1B54A32D192ED03ull + 7;
  float loss = 0.f;
  for (int s = 0; s < steps; s++) {
    // minibatch: B indices from a fixed integer hash stream
    double ms = 0.0;
    for (int b = 0; b < B; b++) {
      z += 0x9E3779B97F4A7C15ull;
      uint64_t r = z;
      r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ull;
      r = (r ^ (r >> 27)) * 0x94D049BB133111EBull;
      r ^= r >> 31;
      idx[b] = B == n_points ? b : (int)(r % (uint64_t)n_points);
      for (int o = 0; o < no; o++) ms += hm[(size_t)idx[b] * no + o];
    }
    if (ms <= 0.0) continue;
    e = cudaMemcpyAsync(M.d_idx, idx.data(), sizeof(int) * B, cudaMemcpyHostToDevice, M.st);
    if (e != cudaSuccess) return gb::cuda_fail(e, "batch");
    gb::gather_rows_kernel<<<304, 256, 0, M.st>>>(B, ni, M.d_idx, d_x, M.d_xb);
    gb::gather_rows_kernel<<<304, 256, 0, M.st>>>(B, no, M.d_idx, d_t, M.d_tb);
    gb::gather_rows_kernel<<<304, 256, 0, M.st>>>(B, no, M.d_idx, d_mask, M.d_mb);
    M.forward(M.d_xb, B);
    // the loss is read back on the last step only: no per-step host wait
    if (M.backward(M.d_xb, M.d_tb, M.d_mb, B, (float)ms, s + 1 == steps ? &loss : nullptr))
      return -1;
    M.adam(lr, 0.9f, 0.999f, 1e-8f);
  }
  e = cudaStreamSynchronize(M.st);
  if (e != cudaSuccess) return gb::cuda_fail(e, "MLP training");
  if (final_loss) *final_loss = loss;
  return 0;
}

}  // extern "C"

// ------------------------------------------------- allocation-free inference
//
// gb_mlp_forward_device keeps its hidden activations in buffers it
// allocates (and grows) on demand.  gb_mlp_forward_noalloc runs the same
// kernels with the activations in the fixed array below instead, for callers
// that cannot allocate device memory at that point.

namespace gb {

// Two ping-pong activation buffers of GB_MLP_NOALLOC_MAX_ACT floats each.
// Every GPU that loads the library holds this array until the process ends.
static __device__ __align__(256) float g_mlp_noalloc_scratch[2 * (size_t)GB_MLP_NOALLOC_MAX_ACT];

constexpr int kNoallocMaxDevices = 64;
static float *g_noalloc_addr[kNoallocMaxDevices];  // device address, per device
static std::mutex g_noalloc_mutex;

// Device address of the scratch array on the current device.  Host code only
// sees a host-side stand-in under the array's name, so the address is
// looked up once per device, with that device current.
static int noalloc_scratch(float **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kNoallocMaxDevices) return fail("device index beyond the scratch table");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_mlp_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
    g_noalloc_addr[dev] = static_cast<float *>(p);
  }
  *out = g_noalloc_addr[dev];
  return 0;
}

}  // namespace gb

extern "C" int gb_mlp_forward_noalloc(gb_mlp *m, const float *d_x, int B, float *d_y,
                                      void *stream) {
  if (!m || !d_x || !d_y) return gb::fail("NULL argument");
  if (B <= 0) return gb::fail("batch size must be positive");
  gb::Mlp &M = m->m;
  {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return gb::cuda_fail(e, "cudaGetDevice");
    if (dev != M.dev) {
      char msg[160];
      snprintf(msg, sizeof msg,
               "current device %d is not the network's device %d; make device %d current", dev,
               M.dev, M.dev);
      return gb::fail(msg);
    }
  }
  int widest = 0;
  for (int l = 1; l + 1 < (int)M.width.size(); l++) widest = M.width[l] > widest ? M.width[l] : widest;
  if ((long long)B * widest > (long long)GB_MLP_NOALLOC_MAX_ACT) {
    char msg[200];
    snprintf(msg, sizeof msg,
             "batch %d x hidden width %d exceeds the static scratch of %d floats per activation "
             "buffer; split the batch",
             B, widest, (int)GB_MLP_NOALLOC_MAX_ACT);
    return gb::fail(msg);
  }
  float *base = nullptr;
  if (gb::noalloc_scratch(&base)) return -1;
  float *buf[2] = {base, base + (size_t)GB_MLP_NOALLOC_MAX_ACT};
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  // after the network's own queued work (training, parameter updates) ...
  cudaError_t e = cudaEventRecord(M.ev_own, M.st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, M.ev_own, 0);
  if (e != cudaSuccess) return gb::cuda_fail(e, "MLP forward (no allocation): ordering");
  const float *in = d_x;
  const int L = M.layers();
  for (int l = 0; l < L; l++) {
    const int K = M.width[l], N = M.width[l + 1];
    float *out = l + 1 == L ? d_y : buf[l & 1];
    dim3 grid((N + gb::TN - 1) / gb::TN, (B + gb::TM - 1) / gb::TM);
    gb::gemm_xwT_kernel<<<grid, 256, 0, cs>>>(B, N, K, in, M.d_w + M.woff[l], M.d_w + M.boff[l],
                                              out, l + 1 < L ? 1 : 0);
    in = out;
  }
  e = cudaGetLastError();
  // ... and the network's later work after this pass
  if (e == cudaSuccess) e = cudaEventRecord(M.ev_caller, cs);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(M.st, M.ev_caller, 0);
  return e == cudaSuccess ? 0 : gb::cuda_fail(e, "MLP forward (no allocation)");
}
