// Active-set predictor for parametric QP families: a multilayer perceptron
// theta -> one logit per inequality constraint (positive: predicted active at
// the optimum), whose prediction seeds the batched NASOQ solve as a warm start
// (nqg_batch_warm_start_from_scores); the active-set iteration then corrects
// it and alone decides whether the final tolerance is met.  The reference has no
// learned component; its warm-start entry is Nasoq::set_warm_start
// (src/nasoq.cpp:413-436).
//
// Weights are kept as FP32 master copies (the optimizer's) and as BF16 copies
// that the forward and backward products read; every product accumulates in
// FP32.  Kernels (all hand-written):
//  * k_gemm: C[M x N] = sum_k A(m, k) B(k, n) over 64 x 64 output tiles with
//    16-deep K slices staged in shared memory (4 x 4 outputs per thread); A
//    and B are addressed through strides, so one kernel gives X W^T (forward),
//    dY^T X (weight gradient) and dY W (input gradient); epilogues: bias +
//    ReLU, ReLU mask of the layer below, plain store;
//  * k_colsum (bias gradient), k_bce (weighted sigmoid cross-entropy and its
//    gradient), k_adam (Adam step, BF16 refresh), k_gather (mini-batch rows).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <string>
#include <vector>

#include "../../include/nasoq_gb300.h"

namespace {

constexpr int GT = 64;   // output tile
constexpr int GK = 16;   // K slice

enum { EPI_STORE = 0, EPI_BIAS_RELU = 1, EPI_BIAS = 2, EPI_RELU_MASK = 3 };

template <class TB> __device__ __forceinline__ float ldf(const TB *p) { return (float)*p; }
template <> __device__ __forceinline__ float ldf<__nv_bfloat16>(const __nv_bfloat16 *p) { return __bfloat162float(*p); }

// C[m * ldc + n] = epi(sum_k A[m * sam + k * sak] * B[k * sbk + n * sbn]).
template <class TB>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float *A, long sam, long sak, const TB *B,
                                              long sbk, long sbn, float *C, int ldc, int epi, const float *bias,
                                              const float *mask) {
  __shared__ float As[GK][GT + 1];
  __shared__ float Bs[GK][GT + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += GK) {
    for (int e = threadIdx.x; e < GK * GT; e += 256) {
      const int kk = e / GT, mm = e % GT;
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < K) ? A[(long)m * sam + (long)k * sak] : 0.f;
      const int n = n0 + mm;
      Bs[kk][mm] = (n < N && k < K) ? ldf(B + (long)k * sbk + (long)n * sbn) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
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
      float v = acc[i][j];
      if (epi == EPI_BIAS_RELU) v = fmaxf(v + bias[n], 0.f);
      else if (epi == EPI_BIAS) v = v + bias[n];
      else if (epi == EPI_RELU_MASK) v = mask[(long)m * ldc + n] > 0.f ? v : 0.f;
      C[(long)m * ldc + n] = v;
    }
  }
}

__global__ void k_colsum(int M, int N, const float *Y, float *out) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int m = 0; m < M; ++m) s += Y[(long)m * N + n];
    out[n] = s;
  }
}

// Weighted sigmoid cross-entropy, mean over the batch rows:
//   l = -(pw y log s(z) + (1 - y) log(1 - s(z))),  dl/dz = s(z) (pw y + 1 - y) - pw y
// (computed with log1p(exp(-|z|)) for stability); grad = dl/dz / M.
__global__ void k_bce(long total, int M, const float *Z, const float *Y, float pw, float *grad, double *loss) {
  double part = 0.0;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const float z = Z[e], y = Y[e];
    const float sp_neg = fmaxf(-z, 0.f) + log1pf(expf(-fabsf(z)));  // -log s(z)
    const float sp_pos = fmaxf(z, 0.f) + log1pf(expf(-fabsf(z)));   // -log(1 - s(z))
    part += (double)(pw * y * sp_neg + (1.f - y) * sp_pos);
    const float s = 1.f / (1.f + expf(-z));
    grad[e] = (s * (pw * y + 1.f - y) - pw * y) / (float)M;
  }
  __shared__ double red[256];
  red[threadIdx.x] = part;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0] / M);
}

__global__ void k_adam(long n, float *w, __nv_bfloat16 *wb, const float *g, float *m, float *v, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
  }
}

__global__ void k_to_bf16(long n, const float *w, __nv_bfloat16 *wb) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    wb[i] = __float2bfloat16(w[i]);
}

__global__ void k_gather(int rows, int cols, const int *idx, const float *src, float *dst) {
  const long total = (long)rows * cols;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long r = e / cols, c = e % cols;
    dst[e] = src[(long)idx[r] * cols + c];
  }
}

inline int blocks_for(long n) { return (int)std::max<long>(1, std::min<long>((n + 255) / 256, 4096)); }

}  // namespace

struct nqg_mlp {
  std::vector<int> sizes;  // sizes[0] inputs, ..., sizes[L] outputs
  int L = 0;
  std::vector<float *> W, b, gW, gb, mW, vW, mb, vb;
  std::vector<__nv_bfloat16 *> Wb;
  std::vector<float *> act;  // act[0]: input rows, act[l]: output of layer l (act[L]: logits)
  std::vector<float *> dact;
  int cap = 0;               // rows the activation buffers hold
  float *d_X = nullptr, *d_Y = nullptr;  // training set (device)
  int n_train = 0;
  float *d_lab = nullptr;    // labels of the current mini-batch
  int *d_idx = nullptr;
  double *d_loss = nullptr;
  long step = 0;
  cudaStream_t stream = nullptr;
  std::string err;
};

namespace {

#define MQ(call)                                                         \
  do {                                                                   \
    cudaError_t e_ = (call);                                             \
    if (e_ != cudaSuccess) {                                             \
      m->err = std::string(#call) + ": " + cudaGetErrorString(e_);       \
      return NQG_ERR_CUDA;                                               \
    }                                                                    \
  } while (0)

int ensure_rows(nqg_mlp *m, int rows) {
  if (rows <= m->cap) return NQG_OK;
  for (auto *p : m->act) cudaFree(p);
  for (auto *p : m->dact) cudaFree(p);
  cudaFree(m->d_lab);
  cudaFree(m->d_idx);
  m->act.assign(m->L + 1, nullptr);
  m->dact.assign(m->L + 1, nullptr);
  for (int l = 0; l <= m->L; ++l) {
    MQ(cudaMalloc(&m->act[l], (size_t)rows * m->sizes[l] * sizeof(float)));
    MQ(cudaMalloc(&m->dact[l], (size_t)rows * m->sizes[l] * sizeof(float)));
  }
  MQ(cudaMalloc(&m->d_lab, (size_t)rows * m->sizes[m->L] * sizeof(float)));
  MQ(cudaMalloc(&m->d_idx, (size_t)rows * sizeof(int)));
  m->cap = rows;
  return NQG_OK;
}

void gemm(cudaStream_t st, int M, int N, int K, const float *A, long sam, long sak, const float *B, long sbk,
          long sbn, float *C, int ldc, int epi, const float *bias, const float *mask) {
  dim3 grid((N + GT - 1) / GT, (M + GT - 1) / GT);
  k_gemm<float><<<grid, 256, 0, st>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, epi, bias, mask);
}
void gemm(cudaStream_t st, int M, int N, int K, const float *A, long sam, long sak, const __nv_bfloat16 *B, long sbk,
          long sbn, float *C, int ldc, int epi, const float *bias, const float *mask) {
  dim3 grid((N + GT - 1) / GT, (M + GT - 1) / GT);
  k_gemm<__nv_bfloat16><<<grid, 256, 0, st>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, epi, bias, mask);
}

// Forward over rows already in act[0]; act[L] receives the logits.
void forward(nqg_mlp *m, int rows) {
  for (int l = 0; l < m->L; ++l) {
    const int in = m->sizes[l], out = m->sizes[l + 1];
    // act[l+1][r, o] = sum_i act[l][r, i] W[o, i]  (+ b, ReLU below the last layer)
    gemm(m->stream, rows, out, in, m->act[l], in, 1, m->Wb[l], 1, in, m->act[l + 1], out,
         l + 1 < m->L ? EPI_BIAS_RELU : EPI_BIAS, m->b[l], nullptr);
  }
}

// Backward from dact[L] (dloss/dlogits); fills gW, gb.
void backward(nqg_mlp *m, int rows) {
  for (int l = m->L - 1; l >= 0; --l) {
    const int in = m->sizes[l], out = m->sizes[l + 1];
    // gW[o, i] = sum_r dact[l+1][r, o] act[l][r, i]
    gemm(m->stream, out, in, rows, m->dact[l + 1], 1, out, m->act[l], in, 1, m->gW[l], in, EPI_STORE, nullptr,
         nullptr);
    k_colsum<<<blocks_for(out), 256, 0, m->stream>>>(rows, out, m->dact[l + 1], m->gb[l]);
    if (l > 0)  // dact[l][r, i] = sum_o dact[l+1][r, o] W[o, i], masked by the ReLU of layer l
      gemm(m->stream, rows, in, out, m->dact[l + 1], out, 1, m->Wb[l], in, 1, m->dact[l], in, EPI_RELU_MASK, nullptr,
           m->act[l]);
  }
}

}  // namespace

extern "C" int nqg_mlp_create(int nsizes, const int *sizes, unsigned long long seed, nqg_mlp **out) {
  if (!out || nsizes < 2 || !sizes) return NQG_ERR_ARG;
  for (int l = 0; l < nsizes; ++l)
    if (sizes[l] <= 0) return NQG_ERR_ARG;
  auto *m = new nqg_mlp;
  m->sizes.assign(sizes, sizes + nsizes);
  m->L = nsizes - 1;
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete m;
    return NQG_ERR_CUDA;
  }
  std::mt19937_64 rng(seed);
  for (int l = 0; l < m->L; ++l) {
    const int in = sizes[l], o = sizes[l + 1];
    const long nw = (long)in * o;
    // He initialisation for the ReLU layers
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / in));
    std::vector<float> w(nw), z(std::max<long>(nw, o), 0.f);
    for (auto &v : w) v = nd(rng);
    float *p;
    for (auto *vec : {&m->W, &m->gW, &m->mW, &m->vW}) {
      if (cudaMalloc(&p, nw * sizeof(float)) != cudaSuccess) return NQG_ERR_CUDA;
      vec->push_back(p);
    }
    for (auto *vec : {&m->b, &m->gb, &m->mb, &m->vb}) {
      if (cudaMalloc(&p, o * sizeof(float)) != cudaSuccess) return NQG_ERR_CUDA;
      vec->push_back(p);
    }
    __nv_bfloat16 *pb;
    if (cudaMalloc(&pb, nw * sizeof(__nv_bfloat16)) != cudaSuccess) return NQG_ERR_CUDA;
    m->Wb.push_back(pb);
    cudaMemcpy(m->W[l], w.data(), nw * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(m->b[l], z.data(), o * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(m->mW[l], z.data(), nw * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(m->vW[l], z.data(), nw * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(m->mb[l], z.data(), o * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(m->vb[l], z.data(), o * sizeof(float), cudaMemcpyHostToDevice);
    k_to_bf16<<<blocks_for(nw), 256, 0, m->stream>>>(nw, m->W[l], m->Wb[l]);
  }
  if (cudaMalloc(&m->d_loss, sizeof(double)) != cudaSuccess) return NQG_ERR_CUDA;
  if (cudaStreamSynchronize(m->stream) != cudaSuccess) return NQG_ERR_CUDA;
  *out = m;
  return NQG_OK;
}

extern "C" int nqg_mlp_num_params(const nqg_mlp *m, long *n_weights, long *n_biases) {
  if (!m) return NQG_ERR_ARG;
  long nw = 0, nb = 0;
  for (int l = 0; l < m->L; ++l) {
    nw += (long)m->sizes[l] * m->sizes[l + 1];
    nb += m->sizes[l + 1];
  }
  if (n_weights) *n_weights = nw;
  if (n_biases) *n_biases = nb;
  return NQG_OK;
}

// Host copies of every layer's FP32 master weights (row-major out x in,
// layer after layer) and biases; set also refreshes the BF16 copies and
// restarts the optimizer.
extern "C" int nqg_mlp_set_weights(nqg_mlp *m, const float *w_all, const float *b_all) {
  if (!m || !w_all || !b_all) return NQG_ERR_ARG;
  long ow = 0, ob = 0;
  for (int l = 0; l < m->L; ++l) {
    const long nw = (long)m->sizes[l] * m->sizes[l + 1];
    const int o = m->sizes[l + 1];
    MQ(cudaMemcpy(m->W[l], w_all + ow, nw * sizeof(float), cudaMemcpyHostToDevice));
    MQ(cudaMemcpy(m->b[l], b_all + ob, o * sizeof(float), cudaMemcpyHostToDevice));
    MQ(cudaMemset(m->mW[l], 0, nw * sizeof(float)));
    MQ(cudaMemset(m->vW[l], 0, nw * sizeof(float)));
    MQ(cudaMemset(m->mb[l], 0, o * sizeof(float)));
    MQ(cudaMemset(m->vb[l], 0, o * sizeof(float)));
    k_to_bf16<<<blocks_for(nw), 256, 0, m->stream>>>(nw, m->W[l], m->Wb[l]);
    ow += nw;
    ob += o;
  }
  m->step = 0;
  MQ(cudaStreamSynchronize(m->stream));
  return NQG_OK;
}

extern "C" int nqg_mlp_get_weights(nqg_mlp *m, float *w_all, float *b_all) {
  if (!m) return NQG_ERR_ARG;
  long ow = 0, ob = 0;
  MQ(cudaStreamSynchronize(m->stream));
  for (int l = 0; l < m->L; ++l) {
    const long nw = (long)m->sizes[l] * m->sizes[l + 1];
    const int o = m->sizes[l + 1];
    if (w_all) MQ(cudaMemcpy(w_all + ow, m->W[l], nw * sizeof(float), cudaMemcpyDeviceToHost));
    if (b_all) MQ(cudaMemcpy(b_all + ob, m->b[l], o * sizeof(float), cudaMemcpyDeviceToHost));
    ow += nw;
    ob += o;
  }
  return NQG_OK;
}

// Logits of `rows` inputs (device pointers, row-major), on `stream` (NULL:
// the model's own stream, synchronised before returning).
extern "C" int nqg_mlp_forward_device(nqg_mlp *m, int rows, const float *d_x, float *d_logits, void *stream) {
  if (!m || rows <= 0 || !d_x || !d_logits) return NQG_ERR_ARG;
  int rc = ensure_rows(m, rows);
  if (rc) return rc;
  cudaStream_t st = stream ? (cudaStream_t)stream : m->stream;
  cudaStream_t keep = m->stream;
  m->stream = st;
  MQ(cudaMemcpyAsync(m->act[0], d_x, (size_t)rows * m->sizes[0] * sizeof(float), cudaMemcpyDeviceToDevice, st));
  forward(m, rows);
  MQ(cudaMemcpyAsync(d_logits, m->act[m->L], (size_t)rows * m->sizes[m->L] * sizeof(float),
                     cudaMemcpyDeviceToDevice, st));
  m->stream = keep;
  if (!stream) MQ(cudaStreamSynchronize(st));
  return NQG_OK;
}

// Host-buffer variant of nqg_mlp_forward_device.
extern "C" int nqg_mlp_forward(nqg_mlp *m, int rows, const float *x, float *logits) {
  if (!m || rows <= 0 || !x || !logits) return NQG_ERR_ARG;
  int rc = ensure_rows(m, rows);
  if (rc) return rc;
  MQ(cudaMemcpyAsync(m->act[0], x, (size_t)rows * m->sizes[0] * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  forward(m, rows);
  MQ(cudaMemcpyAsync(logits, m->act[m->L], (size_t)rows * m->sizes[m->L] * sizeof(float), cudaMemcpyDeviceToHost,
                     m->stream));
  MQ(cudaStreamSynchronize(m->stream));
  return NQG_OK;
}

// Loss and gradients of one batch (host buffers): loss = mean over rows of
// the weighted cross-entropy summed over outputs; gradients copied to the
// host (layer after layer, as in nqg_mlp_get_weights) when the pointers are
// non-null.  No optimizer step.
extern "C" int nqg_mlp_loss_grad(nqg_mlp *m, int rows, const float *x, const float *y, float pos_weight,
                                 double *loss, float *gw_all, float *gb_all) {
  if (!m || rows <= 0 || !x || !y) return NQG_ERR_ARG;
  int rc = ensure_rows(m, rows);
  if (rc) return rc;
  const int out = m->sizes[m->L];
  MQ(cudaMemcpyAsync(m->act[0], x, (size_t)rows * m->sizes[0] * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MQ(cudaMemcpyAsync(m->d_lab, y, (size_t)rows * out * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MQ(cudaMemsetAsync(m->d_loss, 0, sizeof(double), m->stream));
  forward(m, rows);
  const long tot = (long)rows * out;
  k_bce<<<blocks_for(tot), 256, 0, m->stream>>>(tot, rows, m->act[m->L], m->d_lab, pos_weight, m->dact[m->L],
                                                 m->d_loss);
  backward(m, rows);
  double h = 0.0;
  MQ(cudaMemcpyAsync(&h, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  MQ(cudaStreamSynchronize(m->stream));
  if (loss) *loss = h;
  long ow = 0, ob = 0;
  for (int l = 0; l < m->L; ++l) {
    const long nw = (long)m->sizes[l] * m->sizes[l + 1];
    const int o = m->sizes[l + 1];
    if (gw_all) MQ(cudaMemcpy(gw_all + ow, m->gW[l], nw * sizeof(float), cudaMemcpyDeviceToHost));
    if (gb_all) MQ(cudaMemcpy(gb_all + ob, m->gb[l], o * sizeof(float), cudaMemcpyDeviceToHost));
    ow += nw;
    ob += o;
  }
  return NQG_OK;
}

// Training set (host buffers, row-major): n rows of inputs and of 0/1 labels.
extern "C" int nqg_mlp_set_data(nqg_mlp *m, int n, const float *x, const float *y) {
  if (!m || n <= 0 || !x || !y) return NQG_ERR_ARG;
  cudaFree(m->d_X);
  cudaFree(m->d_Y);
  MQ(cudaMalloc(&m->d_X, (size_t)n * m->sizes[0] * sizeof(float)));
  MQ(cudaMalloc(&m->d_Y, (size_t)n * m->sizes[m->L] * sizeof(float)));
  MQ(cudaMemcpy(m->d_X, x, (size_t)n * m->sizes[0] * sizeof(float), cudaMemcpyHostToDevice));
  MQ(cudaMemcpy(m->d_Y, y, (size_t)n * m->sizes[m->L] * sizeof(float), cudaMemcpyHostToDevice));
  m->n_train = n;
  return NQG_OK;
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8) over shuffled mini-batches of the
// training set; epoch_loss (nullable, `epochs` entries) receives the mean
// mini-batch loss of each epoch.
extern "C" int nqg_mlp_train(nqg_mlp *m, int epochs, int batch, float lr, float pos_weight, unsigned long long seed,
                             double *epoch_loss) {
  if (!m || epochs <= 0 || batch <= 0 || m->n_train <= 0) return NQG_ERR_ARG;
  batch = std::min(batch, m->n_train);
  int rc = ensure_rows(m, batch);
  if (rc) return rc;
  const int in = m->sizes[0], out = m->sizes[m->L];
  std::mt19937_64 rng(seed);
  std::vector<int> perm(m->n_train);
  for (int i = 0; i < m->n_train; ++i) perm[i] = i;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs; ++ep) {
    std::shuffle(perm.begin(), perm.end(), rng);
    MQ(cudaMemsetAsync(m->d_loss, 0, sizeof(double), m->stream));
    int nb = 0;
    for (int s0 = 0; s0 + batch <= m->n_train; s0 += batch, ++nb) {
      MQ(cudaMemcpyAsync(m->d_idx, perm.data() + s0, batch * sizeof(int), cudaMemcpyHostToDevice, m->stream));
      k_gather<<<blocks_for((long)batch * in), 256, 0, m->stream>>>(batch, in, m->d_idx, m->d_X, m->act[0]);
      k_gather<<<blocks_for((long)batch * out), 256, 0, m->stream>>>(batch, out, m->d_idx, m->d_Y, m->d_lab);
      forward(m, batch);
      const long tot = (long)batch * out;
      k_bce<<<blocks_for(tot), 256, 0, m->stream>>>(tot, batch, m->act[m->L], m->d_lab, pos_weight, m->dact[m->L],
                                                     m->d_loss);
      backward(m, batch);
      m->step++;
      const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
      for (int l = 0; l < m->L; ++l) {
        const long nw = (long)m->sizes[l] * m->sizes[l + 1];
        const int o = m->sizes[l + 1];
        k_adam<<<blocks_for(nw), 256, 0, m->stream>>>(nw, m->W[l], m->Wb[l], m->gW[l], m->mW[l], m->vW[l], lr, b1, b2,
                                                       eps, c1, c2);
        k_adam<<<blocks_for(o), 256, 0, m->stream>>>(o, m->b[l], nullptr, m->gb[l], m->mb[l], m->vb[l], lr, b1, b2,
                                                      eps, c1, c2);
      }
      // the host index buffer of the next batch must not change before the copy ran
      MQ(cudaStreamSynchronize(m->stream));
    }
    double h = 0.0;
    MQ(cudaMemcpyAsync(&h, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    MQ(cudaStreamSynchronize(m->stream));
    if (epoch_loss) epoch_loss[ep] = nb ? h / nb : 0.0;
  }
  MQ(cudaGetLastError());
  return NQG_OK;
}

extern "C" const char *nqg_mlp_last_error(const nqg_mlp *m) { return m ? m->err.c_str() : ""; }

extern "C" int nqg_mlp_destroy(nqg_mlp *m) {
  if (!m) return NQG_ERR_ARG;
  cudaStreamSynchronize(m->stream);
  for (auto *vec : {&m->W, &m->b, &m->gW, &m->gb, &m->mW, &m->vW, &m->mb, &m->vb, &m->act, &m->dact})
    for (float *p : *vec) cudaFree(p);
  for (auto *p : m->Wb) cudaFree(p);
  cudaFree(m->d_X);
  cudaFree(m->d_Y);
  cudaFree(m->d_lab);
  cudaFree(m->d_idx);
  cudaFree(m->d_loss);
  cudaStreamDestroy(m->stream);
  delete m;
  return NQG_OK;
}
