// mlp.cu — the tau / block-shape predictor: a 64-128-128-12 FP32 MLP
// (ReLU hidden layers) with two softmax heads, logits 0..8 for tau in
// {0.1, ..., 0.9} and 9..11 for the block shape {8x8, 16x16, 32x16}, trained
// with the sum of the two heads' cross-entropies (mean over the batch) and
// Adam, all in hand-written kernels: the batch is small and the layers
// narrow, so each output element is one thread's dot product.
//
// Parameters, one FP32 array: W1[64][128], b1[128], W2[128][128], b2[128],
// W3[128][12], b3[12] (W[in][out], y = x W + b).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "smat_internal.h"

namespace smat {
namespace dev {

constexpr int kIn = 64, kH = 128, kOut = 12, kTau = 9;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + kIn * kH, OFF_W2 = OFF_B1 + kH, OFF_B2 = OFF_W2 + kH * kH,
              OFF_W3 = OFF_B2 + kH, OFF_B3 = OFF_W3 + kH * kOut, NPARAM = OFF_B3 + kOut;

// Y[b][o] = act(sum_i X[b][i] W[i][o] + bias[o])
__global__ void linear_fwd(const float* __restrict__ X, const float* __restrict__ W, const float* __restrict__ bias,
                           float* __restrict__ Y, int B, int In, int Out, int relu) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * Out) return;
  const int b = idx / Out, o = idx % Out;
  float acc = bias[o];
  for (int i = 0; i < In; i++) acc = fmaf(X[b * In + i], W[i * Out + o], acc);
  Y[idx] = relu ? fmaxf(acc, 0.0f) : acc;
}

// Softmax cross-entropy of both heads; dL[b][o] = (p - onehot) / B.
__global__ void heads_loss(const float* __restrict__ L, const int* __restrict__ ytau, const int* __restrict__ yblk,
                           float* __restrict__ dL, float* __restrict__ loss, int B) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float* l = L + b * kOut;
  float* d = dL + b * kOut;
  float total = 0.0f;
  const int seg0[2] = {0, kTau}, seg1[2] = {kTau, kOut};
  const int y[2] = {ytau[b], kTau + yblk[b]};
  for (int h = 0; h < 2; h++) {
    float m = -INFINITY;
    for (int o = seg0[h]; o < seg1[h]; o++) m = fmaxf(m, l[o]);
    float s = 0.0f;
    for (int o = seg0[h]; o < seg1[h]; o++) s += expf(l[o] - m);
    const float lse = m + logf(s);
    for (int o = seg0[h]; o < seg1[h]; o++) d[o] = (expf(l[o] - lse) - (o == y[h] ? 1.0f : 0.0f)) / (float)B;
    total += lse - l[y[h]];
  }
  atomicAdd(loss, total / (float)B);
}

// dX[b][i] = (sum_o dY[b][o] W[i][o]) * (H[b][i] > 0), H the layer input (post-ReLU)
__global__ void linear_bwd_x(const float* __restrict__ dY, const float* __restrict__ W, const float* __restrict__ H,
                             float* __restrict__ dX, int B, int In, int Out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * In) return;
  const int b = idx / In, i = idx % In;
  float acc = 0.0f;
  for (int o = 0; o < Out; o++) acc = fmaf(dY[b * Out + o], W[i * Out + o], acc);
  dX[idx] = H[idx] > 0.0f ? acc : 0.0f;
}

// dW[i][o] = sum_b X[b][i] dY[b][o]; db[o] = sum_b dY[b][o] (thread i == In)
__global__ void linear_bwd_w(const float* __restrict__ X, const float* __restrict__ dY, float* __restrict__ dW,
                             float* __restrict__ db, int B, int In, int Out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (In + 1) * Out) return;
  const int i = idx / Out, o = idx % Out;
  float acc = 0.0f;
  if (i < In) {
    for (int b = 0; b < B; b++) acc = fmaf(X[b * In + i], dY[b * Out + o], acc);
    dW[i * Out + o] = acc;
  } else {
    for (int b = 0; b < B; b++) acc += dY[b * Out + o];
    db[o] = acc;
  }
}

__global__ void adam_step(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ m,
                          float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = G[i];
  const float mi = b1 * m[i] + (1.0f - b1) * g;
  const float vi = b2 * v[i] + (1.0f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  P[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace dev
}  // namespace smat

using namespace smat;
using namespace smat::dev;

struct smat_mlp {
  int device = 0;
  int64_t step = 0;
  float *P = nullptr, *G = nullptr, *m = nullptr, *v = nullptr;
  int cap = 0;  // batch capacity of the buffers below
  float *X = nullptr, *H1 = nullptr, *H2 = nullptr, *L = nullptr, *dL = nullptr, *dH2 = nullptr, *dH1 = nullptr,
        *loss = nullptr;
  int *yt = nullptr, *yb = nullptr;
};

static void mlp_free_batch(smat_mlp* n) {
  for (float* p : {n->X, n->H1, n->H2, n->L, n->dL, n->dH2, n->dH1, n->loss}) cudaFree(p);
  cudaFree(n->yt);
  cudaFree(n->yb);
  n->X = n->H1 = n->H2 = n->L = n->dL = n->dH2 = n->dH1 = n->loss = nullptr;
  n->yt = n->yb = nullptr;
  n->cap = 0;
}

static smat_status mlp_reserve(smat_mlp* n, int B) {
  if (B <= n->cap) return SMAT_OK;
  mlp_free_batch(n);
  bool ok = cudaMalloc(&n->X, (size_t)B * kIn * 4) == cudaSuccess && cudaMalloc(&n->H1, (size_t)B * kH * 4) == cudaSuccess &&
            cudaMalloc(&n->H2, (size_t)B * kH * 4) == cudaSuccess && cudaMalloc(&n->L, (size_t)B * kOut * 4) == cudaSuccess &&
            cudaMalloc(&n->dL, (size_t)B * kOut * 4) == cudaSuccess && cudaMalloc(&n->dH2, (size_t)B * kH * 4) == cudaSuccess &&
            cudaMalloc(&n->dH1, (size_t)B * kH * 4) == cudaSuccess && cudaMalloc(&n->loss, 4) == cudaSuccess &&
            cudaMalloc(&n->yt, (size_t)B * 4) == cudaSuccess && cudaMalloc(&n->yb, (size_t)B * 4) == cudaSuccess;
  if (!ok) {
    mlp_free_batch(n);
    return fail(SMAT_ERR_NOMEM, "MLP batch buffers");
  }
  n->cap = B;
  return SMAT_OK;
}

static inline int nblk(int n) { return (n + 255) / 256; }

// Forward pass of n->X (batch B) into H1, H2, L.
static void mlp_forward(smat_mlp* n, int B) {
  linear_fwd<<<nblk(B * kH), 256>>>(n->X, n->P + OFF_W1, n->P + OFF_B1, n->H1, B, kIn, kH, 1);
  linear_fwd<<<nblk(B * kH), 256>>>(n->H1, n->P + OFF_W2, n->P + OFF_B2, n->H2, B, kH, kH, 1);
  linear_fwd<<<nblk(B * kOut), 256>>>(n->H2, n->P + OFF_W3, n->P + OFF_B3, n->L, B, kH, kOut, 0);
}

// Loss and gradients into n->G for the batch already in X / yt / yb.
static void mlp_backward(smat_mlp* n, int B) {
  cudaMemsetAsync(n->loss, 0, 4);
  heads_loss<<<nblk(B), 256>>>(n->L, n->yt, n->yb, n->dL, n->loss, B);
  linear_bwd_w<<<nblk((kH + 1) * kOut), 256>>>(n->H2, n->dL, n->G + OFF_W3, n->G + OFF_B3, B, kH, kOut);
  linear_bwd_x<<<nblk(B * kH), 256>>>(n->dL, n->P + OFF_W3, n->H2, n->dH2, B, kH, kOut);
  linear_bwd_w<<<nblk((kH + 1) * kH), 256>>>(n->H1, n->dH2, n->G + OFF_W2, n->G + OFF_B2, B, kH, kH);
  linear_bwd_x<<<nblk(B * kH), 256>>>(n->dH2, n->P + OFF_W2, n->H1, n->dH1, B, kH, kH);
  linear_bwd_w<<<nblk((kIn + 1) * kH), 256>>>(n->X, n->dH1, n->G + OFF_W1, n->G + OFF_B1, B, kIn, kH);
}

static smat_status mlp_load_batch(smat_mlp* n, const float* X, const int32_t* yt, const int32_t* yb, int B) {
  smat_status st = mlp_reserve(n, B);
  if (st != SMAT_OK) return st;
  if (cudaMemcpy(n->X, X, (size_t)B * kIn * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(SMAT_ERR_CUDA, "MLP input copy");
  if (yt && yb) {
    for (int b = 0; b < B; b++)
      if (yt[b] < 0 || yt[b] >= kTau || yb[b] < 0 || yb[b] >= kOut - kTau)
        return fail(SMAT_ERR_INVALID, "label out of range");
    if (cudaMemcpy(n->yt, yt, (size_t)B * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(n->yb, yb, (size_t)B * 4, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(SMAT_ERR_CUDA, "MLP label copy");
  }
  return SMAT_OK;
}

struct DevScope {
  int prev = -1;
  explicit DevScope(int d) {
    cudaGetDevice(&prev);
    if (prev != d) cudaSetDevice(d);
  }
  ~DevScope() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

extern "C" {

smat_status smat_mlp_create(int32_t device, uint64_t seed, smat_mlp** out) {
  if (!out) return fail(SMAT_ERR_INVALID, "null argument");
  *out = nullptr;
  DevScope ds(device);
  smat_mlp* n = new smat_mlp();
  n->device = device;
  bool ok = cudaMalloc(&n->P, NPARAM * 4) == cudaSuccess && cudaMalloc(&n->G, NPARAM * 4) == cudaSuccess &&
            cudaMalloc(&n->m, NPARAM * 4) == cudaSuccess && cudaMalloc(&n->v, NPARAM * 4) == cudaSuccess &&
            cudaMemset(n->m, 0, NPARAM * 4) == cudaSuccess && cudaMemset(n->v, 0, NPARAM * 4) == cudaSuccess &&
            cudaMemset(n->G, 0, NPARAM * 4) == cudaSuccess;
  // He-normal weights, zero biases
  std::vector<float> p(NPARAM, 0.0f);
  std::mt19937_64 rng(seed);
  auto init = [&](int off, int fan_in, int cnt) {
    std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / fan_in));
    for (int i = 0; i < cnt; i++) p[off + i] = nd(rng);
  };
  init(OFF_W1, kIn, kIn * kH);
  init(OFF_W2, kH, kH * kH);
  init(OFF_W3, kH, kH * kOut);
  ok = ok && cudaMemcpy(n->P, p.data(), NPARAM * 4, cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    smat_mlp_destroy(n);
    return fail(SMAT_ERR_NOMEM, "MLP parameters");
  }
  *out = n;
  return SMAT_OK;
}

int32_t smat_mlp_num_params(void) { return NPARAM; }

smat_status smat_mlp_get_params(const smat_mlp* n, float* params) {
  if (!n || !params) return fail(SMAT_ERR_INVALID, "null argument");
  DevScope ds(n->device);
  if (cudaMemcpy(params, n->P, NPARAM * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return fail(SMAT_ERR_CUDA, "copy");
  return SMAT_OK;
}

smat_status smat_mlp_set_params(smat_mlp* n, const float* params) {
  if (!n || !params) return fail(SMAT_ERR_INVALID, "null argument");
  DevScope ds(n->device);
  if (cudaMemcpy(n->P, params, NPARAM * 4, cudaMemcpyHostToDevice) != cudaSuccess) return fail(SMAT_ERR_CUDA, "copy");
  return SMAT_OK;
}

smat_status smat_mlp_gradients(smat_mlp* n, const float* X, const int32_t* y_tau, const int32_t* y_block, int32_t batch,
                               float* grads, float* loss) {
  if (!n || !X || !y_tau || !y_block || batch <= 0) return fail(SMAT_ERR_INVALID, "bad argument");
  DevScope ds(n->device);
  smat_status st = mlp_load_batch(n, X, y_tau, y_block, batch);
  if (st != SMAT_OK) return st;
  mlp_forward(n, batch);
  mlp_backward(n, batch);
  if (cudaGetLastError() != cudaSuccess) return fail(SMAT_ERR_CUDA, "MLP kernels");
  if (grads && cudaMemcpy(grads, n->G, NPARAM * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(SMAT_ERR_CUDA, "copy");
  if (loss && cudaMemcpy(loss, n->loss, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return fail(SMAT_ERR_CUDA, "copy");
  return SMAT_OK;
}

smat_status smat_mlp_train_step(smat_mlp* n, const float* X, const int32_t* y_tau, const int32_t* y_block,
                                int32_t batch, float lr, float* loss) {
  smat_status st = smat_mlp_gradients(n, X, y_tau, y_block, batch, nullptr, loss);
  if (st != SMAT_OK) return st;
  DevScope ds(n->device);
  n->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - std::pow(b1, (float)n->step), c2 = 1.0f - std::pow(b2, (float)n->step);
  adam_step<<<nblk(NPARAM), 256>>>(n->P, n->G, n->m, n->v, NPARAM, lr, b1, b2, 1e-8f, c1, c2);
  if (cudaGetLastError() != cudaSuccess) return fail(SMAT_ERR_CUDA, "Adam kernel");
  return SMAT_OK;
}

smat_status smat_mlp_predict(smat_mlp* n, const float* X, int32_t batch, float* logits) {
  if (!n || !X || !logits || batch <= 0) return fail(SMAT_ERR_INVALID, "bad argument");
  DevScope ds(n->device);
  smat_status st = mlp_load_batch(n, X, nullptr, nullptr, batch);
  if (st != SMAT_OK) return st;
  mlp_forward(n, batch);
  if (cudaMemcpy(logits, n->L, (size_t)batch * kOut * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(SMAT_ERR_CUDA, "MLP output copy");
  return SMAT_OK;
}

smat_status smat_mlp_destroy(smat_mlp* n) {
  if (!n) return SMAT_OK;
  DevScope ds(n->device);
  mlp_free_batch(n);
  cudaFree(n->P);
  cudaFree(n->G);
  cudaFree(n->m);
  cudaFree(n->v);
  delete n;
  return SMAT_OK;
}

}  // extern "C"
