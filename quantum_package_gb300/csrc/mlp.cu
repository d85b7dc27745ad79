// Learned Davidson preconditioner: a small MLP (8 -> 64 -> 64 -> 1, GELU,
// FP32) that maps per-determinant features to a multiplier g of the
// reference's diagonal correction d = (lambda u - W)(...)/max(H_II - lambda,
// 1e-2) (src/Davidson/diagonalization_hs2.irp.f:386-391).  g acts as a learned
// per-determinant shift of the diagonal denominator.  Training pairs come from
// Davidson runs on earlier determinant sets (captured in davidson.cu); the
// forward, backward and Adam kernels below are the whole training stack.
// The reference has no learned component: this file has no counterpart there.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "qpgpu_internal.cuh"

namespace {

constexpr int MT = QP_MLP_H;  // threads of the training CTA: one per hidden unit

inline unsigned gsz(int64_t n, int tpb = 256) {
  int64_t g = (n + tpb - 1) / tpb;
  if (g < 1) g = 1;
  if (g > 65535LL * 16) g = 65535LL * 16;
  return (unsigned)g;
}

// static features of each determinant (bilinear order): excitation rank of the
// alpha and beta strings relative to the reference, sum of h_pp over particles
// minus holes (orbital-energy change); .w is set by k_row_coupling
template <int NINT>
__global__ void k_det_features(DevTables t, const u64* alpha, const u64* beta, const int* rows, const int* cols,
                               float4* out, int64_t N) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x) {
    const u64* a = alpha + (int64_t)rows[k] * NINT;
    const u64* b = beta + (int64_t)cols[k] * NINT;
    int ra = 0, rb = 0;
    double e = 0.0;
    for (int w = 0; w < NINT; ++w) {
      const u64 xa = a[w] ^ t.ref[w], xb = b[w] ^ t.ref[NINT + w];
      ra += popc64(xa);
      rb += popc64(xb);

      for (u64 x = xa; x; x &= x - 1) {
        const int p = ctz64(x) + 1 + 64 * w;
        const double hp = tab2(t.h, t.n, p, p);
        e += ((a[w] >> (p - 1 - 64 * w)) & 1ull) ? hp : -hp;
      }
      for (u64 x = xb; x; x &= x - 1) {
        const int p = ctz64(x) + 1 + 64 * w;
        const double hp = tab2(t.h, t.n, p, p);
        e += ((b[w] >> (p - 1 - 64 * w)) & 1ull) ? hp : -hp;
      }
    }
    out[k] = make_float4(0.5f * ra, 0.5f * rb, (float)e, 0.f);
  }
}

// coupling strength of each row: log10(sum_J H_IJ^2) / 4 (the scale of the
// second-order shift of the diagonal denominator), one warp per row, into .w
__global__ void k_row_coupling(const int64_t* rowptr, const double* val, float4* out, int64_t N) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t k = warp; k < N; k += nwarp) {
    double s = 0.0;
    for (int64_t e = rowptr[k] + lane; e < rowptr[k + 1]; e += 32) s = fma(val[e], val[e], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[k].w = (float)(log10(s + 1e-30) * 0.25);
  }
}

// one gradient evaluation: CTA of 64 threads (thread j = hidden unit j) runs
// the samples idx[s] for s = blockIdx.x, +gridDim.x, ... one after the other;
// per-CTA gradient sums are written to partial[blockIdx.x][NPARAM + 1 (loss)]
__global__ void __launch_bounds__(MT) k_mlp_grad(const float* __restrict__ P, const float* __restrict__ X,
                                                  const float* __restrict__ G, const float* __restrict__ Wt,
                                                  const int* __restrict__ idx, int nb, float* partial) {
  __shared__ float W2s[QP_MLP_H * QP_MLP_H];
  __shared__ float h1s[QP_MLP_H], d2s[QP_MLP_H], red[2];
  const int j = threadIdx.x;
  for (int i = j; i < QP_MLP_H * QP_MLP_H; i += MT) W2s[i] = P[QP_MLP_W2 + i];
  float w1[QP_MLP_IN];
#pragma unroll
  for (int i = 0; i < QP_MLP_IN; ++i) w1[i] = P[QP_MLP_W1 + j * QP_MLP_IN + i];
  const float b1 = P[QP_MLP_B1 + j], b2 = P[QP_MLP_B2 + j], w3 = P[QP_MLP_W3 + j], b3 = P[QP_MLP_B3];
  float gW1[QP_MLP_IN], gW2[QP_MLP_H], gb1 = 0.f, gb2 = 0.f, gW3 = 0.f, gb3 = 0.f, loss = 0.f;
#pragma unroll
  for (int i = 0; i < QP_MLP_IN; ++i) gW1[i] = 0.f;
#pragma unroll
  for (int i = 0; i < QP_MLP_H; ++i) gW2[i] = 0.f;
  __syncthreads();
  for (int s = blockIdx.x; s < nb; s += gridDim.x) {
    const int64_t q = idx[s];
    float x[QP_MLP_IN];
#pragma unroll
    for (int i = 0; i < QP_MLP_IN; ++i) x[i] = X[q * QP_MLP_IN + i];
    float pre1 = b1;
#pragma unroll
    for (int i = 0; i < QP_MLP_IN; ++i) pre1 = fmaf(w1[i], x[i], pre1);
    h1s[j] = qp_gelu(pre1);
    __syncthreads();
    float pre2 = b2;
#pragma unroll 16
    for (int i = 0; i < QP_MLP_H; ++i) pre2 = fmaf(W2s[j * QP_MLP_H + i], h1s[i], pre2);
    const float a2 = qp_gelu(pre2);
    // y = b3 + sum_j w3_j a2_j (two warps)
    float t = w3 * a2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((j & 31) == 0) red[j >> 5] = t;
    __syncthreads();
    const float y = b3 + red[0] + red[1];
    const float err = y - G[q];
    const float wq = Wt[q];
    const float dy = 2.f * wq * err;
    if (j == 0) {
      loss = fmaf(wq * err, err, loss);
      gb3 += dy;
    }
    gW3 = fmaf(dy, a2, gW3);
    const float dp2 = dy * w3 * qp_gelu_grad(pre2);
    d2s[j] = dp2;
    gb2 += dp2;
#pragma unroll 16
    for (int i = 0; i < QP_MLP_H; ++i) gW2[i] = fmaf(dp2, h1s[i], gW2[i]);
    __syncthreads();
    float dh1 = 0.f;
#pragma unroll 16
    for (int k = 0; k < QP_MLP_H; ++k) dh1 = fmaf(W2s[k * QP_MLP_H + j], d2s[k], dh1);
    const float dp1 = dh1 * qp_gelu_grad(pre1);
    gb1 += dp1;
#pragma unroll
    for (int i = 0; i < QP_MLP_IN; ++i) gW1[i] = fmaf(dp1, x[i], gW1[i]);
    __syncthreads();
  }
  float* out = partial + (int64_t)blockIdx.x * (QP_MLP_NPARAM + 1);
#pragma unroll
  for (int i = 0; i < QP_MLP_IN; ++i) out[QP_MLP_W1 + j * QP_MLP_IN + i] = gW1[i];
  out[QP_MLP_B1 + j] = gb1;
#pragma unroll 16
  for (int i = 0; i < QP_MLP_H; ++i) out[QP_MLP_W2 + j * QP_MLP_H + i] = gW2[i];
  out[QP_MLP_B2 + j] = gb2;
  out[QP_MLP_W3 + j] = gW3;
  if (j == 0) {
    out[QP_MLP_B3] = gb3;
    out[QP_MLP_NPARAM] = loss;
  }
}

// grad[p] = sum over CTAs (fixed order) / nb; optional Adam update of P
__global__ void k_mlp_reduce_adam(const float* partial, int ncta, int nb, float* grad, float* P, float* m, float* v,
                                  int64_t step, float lr, int update) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > QP_MLP_NPARAM) return;
  float s = 0.f;
  for (int c = 0; c < ncta; ++c) s += partial[(int64_t)c * (QP_MLP_NPARAM + 1) + p];
  s /= (float)nb;
  if (grad) grad[p] = s;
  if (!update || p == QP_MLP_NPARAM) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float mm = b1 * m[p] + (1.f - b1) * s;
  const float vv = b2 * v[p] + (1.f - b2) * s * s;
  m[p] = mm;
  v[p] = vv;
  const float mh = mm / (1.f - powf(b1, (float)step)), vh = vv / (1.f - powf(b2, (float)step));
  P[p] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void __launch_bounds__(256) k_mlp_predict(const float* P, const float* X, float* y, int64_t n) {
  __shared__ __align__(16) float Ps[QP_MLP_NPARAM];
  for (int i = threadIdx.x; i < QP_MLP_NPARAM; i += blockDim.x) Ps[i] = P[i];
  __syncthreads();
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    float f[QP_MLP_IN];
    for (int i = 0; i < QP_MLP_IN; ++i) f[i] = X[q * QP_MLP_IN + i];
    y[q] = qp_mlp_forward(Ps, f);
  }
}

}  // namespace

// y[q] = MLP(X[q]) for n samples (inference of the learned Davidson step)
void qp_mlp_eval(const float* P, const float* X, float* y, int64_t n, cudaStream_t st, int n_sm) {
  const int64_t g = std::min<int64_t>(gsz(n), (int64_t)n_sm * 8);
  k_mlp_predict<<<(unsigned)std::max<int64_t>(g, 1), 256, 0, st>>>(P, X, y, n);
}

namespace {

int ensure_mlp(qpgpu_ctx* c) {
  if (c->mlp.params) return 0;
  QP_CUDA(c, dev_alloc(&c->mlp.params, QP_MLP_NPARAM));
  QP_CUDA(c, dev_alloc(&c->mlp.adam_m, QP_MLP_NPARAM));
  QP_CUDA(c, dev_alloc(&c->mlp.adam_v, QP_MLP_NPARAM));
  return 0;
}

// gradient over samples idx[0..nb) into grad (device, NPARAM+1 with the loss)
int mlp_gradient(qpgpu_ctx* c, const int* d_idx, int nb, float* d_partial, int ncta, float* d_grad, bool update,
                 float lr) {
  k_mlp_grad<<<ncta, MT, 0, c->stream>>>(c->mlp.params, c->mlp.X, c->mlp.G, c->mlp.Wt, d_idx, nb, d_partial);
  if (update) ++c->mlp.adam_t;
  k_mlp_reduce_adam<<<gsz(QP_MLP_NPARAM + 1), 256, 0, c->stream>>>(d_partial, ncta, nb, d_grad, c->mlp.params,
                                                                   c->mlp.adam_m, c->mlp.adam_v, c->mlp.adam_t, lr,
                                                                   update ? 1 : 0);
  QP_CUDA(c, cudaGetLastError());
  return 0;
}

struct Lk {
  std::mutex& m;
  explicit Lk(std::mutex& mm) : m(mm) { m.lock(); }
  ~Lk() { m.unlock(); }
};

}  // namespace

int qp_det_features(qpgpu_ctx* c) {
  dev_free(c->d_detfeat);
  c->d_detfeat = nullptr;
  QP_CUDA(c, cudaMalloc((void**)&c->d_detfeat, c->N * sizeof(float4)));
  if (c->nint == 1)
    k_det_features<1><<<gsz(c->N), 256, 0, c->stream>>>(c->tab, c->d_alpha, c->d_beta, c->d_rows, c->d_cols,
                                                        (float4*)c->d_detfeat, c->N);
  else
    k_det_features<2><<<gsz(c->N), 256, 0, c->stream>>>(c->tab, c->d_alpha, c->d_beta, c->d_rows, c->d_cols,
                                                        (float4*)c->d_detfeat, c->N);
  // coupling feature from the stored elements (left at 0 with the direct sigma)
  if (!c->direct)
    k_row_coupling<<<gsz(c->N * 32), 256, 0, c->stream>>>(c->d_rowptr, c->d_val64, (float4*)c->d_detfeat, c->N);
  QP_CUDA(c, cudaGetLastError());
  return 0;
}

// append n samples (host or device arrays) to the training set
int qp_mlp_append(qpgpu_ctx* c, const float* X, const float* G, const float* W, int64_t n, bool device_src) {
  if (n <= 0) return 0;
  MlpState& m = c->mlp;
  if (m.n + n > m.cap) {
    const int64_t cap = std::max<int64_t>(2 * (m.n + n), 1 << 16);
    float *nX = nullptr, *nG = nullptr, *nW = nullptr;
    if (cudaMalloc((void**)&nX, cap * QP_MLP_IN * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void**)&nG, cap * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void**)&nW, cap * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      dev_free(nX);
      dev_free(nG);
      dev_free(nW);
      return qpgpu_fail(c, QPGPU_ERR_NOMEM, "training set does not fit on the device");
    }
    if (m.n) {
      QP_CUDA(c, cudaMemcpyAsync(nX, m.X, m.n * QP_MLP_IN * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
      QP_CUDA(c, cudaMemcpyAsync(nG, m.G, m.n * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
      QP_CUDA(c, cudaMemcpyAsync(nW, m.Wt, m.n * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
      QP_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    dev_free(m.X);
    dev_free(m.G);
    dev_free(m.Wt);
    m.X = nX;
    m.G = nG;
    m.Wt = nW;
    m.cap = cap;
  }
  const cudaMemcpyKind k = device_src ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  QP_CUDA(c, cudaMemcpyAsync(m.X + m.n * QP_MLP_IN, X, n * QP_MLP_IN * sizeof(float), k, c->stream));
  QP_CUDA(c, cudaMemcpyAsync(m.G + m.n, G, n * sizeof(float), k, c->stream));
  QP_CUDA(c, cudaMemcpyAsync(m.Wt + m.n, W, n * sizeof(float), k, c->stream));
  QP_CUDA(c, cudaStreamSynchronize(c->stream));
  m.n += n;
  return 0;
}

extern "C" {

int qpgpu_mlp_init(qpgpu_ctx* c, uint64_t seed) {
  if (!c) return QPGPU_ERR_ARG;
  Lk l(c->mu);
  int rc = ensure_mlp(c);
  if (rc) return rc;
  // Glorot-uniform weights, zero biases, output bias 1 (g = 1: the diagonal step)
  std::mt19937_64 gen(seed);
  std::vector<float> P(QP_MLP_NPARAM, 0.f);
  auto fill = [&](int off, int fan_out, int fan_in) {
    const float lim = std::sqrt(6.f / (fan_in + fan_out));
    std::uniform_real_distribution<float> u(-lim, lim);
    for (int i = 0; i < fan_out * fan_in; ++i) P[off + i] = u(gen);
  };
  fill(QP_MLP_W1, QP_MLP_H, QP_MLP_IN);
  fill(QP_MLP_W2, QP_MLP_H, QP_MLP_H);
  fill(QP_MLP_W3, 1, QP_MLP_H);
  for (int i = 0; i < QP_MLP_H; ++i) P[QP_MLP_W3 + i] *= 0.1f;
  P[QP_MLP_B3] = 1.f;
  QP_CUDA(c, cudaMemcpyAsync(c->mlp.params, P.data(), P.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  QP_CUDA(c, cudaMemsetAsync(c->mlp.adam_m, 0, QP_MLP_NPARAM * sizeof(float), c->stream));
  QP_CUDA(c, cudaMemsetAsync(c->mlp.adam_v, 0, QP_MLP_NPARAM * sizeof(float), c->stream));
  QP_CUDA(c, cudaStreamSynchronize(c->stream));
  c->mlp.adam_t = 0;
  c->mlp.ready = true;
  return QPGPU_OK;
}

int qpgpu_mlp_set_weights(qpgpu_ctx* c, const float* w) {
  if (!c || !w) return QPGPU_ERR_ARG;
  Lk l(c->mu);
  int rc = ensure_mlp(c);
  if (rc) return rc;
  QP_CUDA(c, cudaMemcpyAsync(c->mlp.params, w, QP_MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  QP_CUDA(c, cudaMemsetAsync(c->mlp.adam_m, 0, QP_MLP_NPARAM * sizeof(float), c->stream));
  QP_CUDA(c, cudaMemsetAsync(c->mlp.adam_v, 0, QP_MLP_NPARAM * sizeof(float), c->stream));
  QP_CUDA(c, cudaStreamSynchronize(c->stream));
  c->mlp.adam_t = 0;
  c->mlp.ready = true;
  return QPGPU_OK;
}

int qpgpu_mlp_get_weights(qpgpu_ctx* c, float* w) {
  if (!c || !w) return QPGPU_ERR_ARG;
  if (!c->mlp.ready) return qpgpu_fail(c, QPGPU_ERR_STATE, "MLP not initialised");
  Lk l(c->mu);
  QP_CUDA(c, cudaMemcpyAsync(w, c->mlp.params, QP_MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  QP_CUDA(c, cudaStreamSynchronize(c->stream));
  return QPGPU_OK;
}

int qpgpu_mlp_add_samples(qpgpu_ctx* c, const float* X, const float* G, const float* W, int64_t n) {
  if (!c || !X || !G || !W || n < 0) return QPGPU_ERR_ARG;
  Lk l(c->mu);
  return qp_mlp_append(c, X, G, W, n, false);
}

int qpgpu_mlp_clear_samples(qpgpu_ctx* c) {
  if (!c) return QPGPU_ERR_ARG;
  Lk l(c->mu);
  c->mlp.n = 0;
  return QPGPU_OK;
}

int64_t qpgpu_mlp_n_samples(qpgpu_ctx* c) { return c ? c->mlp.n : -1; }

// Gradient (and weighted loss) of the current parameters over host samples
// X[n][8], G[n], W[n]: loss = mean(W (y - G)^2).  grad has NPARAM entries.
int qpgpu_mlp_gradient(qpgpu_ctx* c, const float* X, const float* G, const float* W, int64_t n, float* grad,
                       float* loss) {
  if (!c || !X || !G || !W || !grad || n < 1 || n > (1 << 24)) return QPGPU_ERR_ARG;
  if (!c->mlp.ready) return qpgpu_fail(c, QPGPU_ERR_STATE, "MLP not initialised");
  Lk l(c->mu);
  const int64_t keep = c->mlp.n;
  int rc = qp_mlp_append(c, X, G, W, n, false);
  if (rc) return rc;
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), (int)keep);
  const int ncta = 256;
  int* d_idx = nullptr;
  float *d_part = nullptr, *d_grad = nullptr;
  QP_CUDA(c, cudaMalloc((void**)&d_idx, n * sizeof(int)));
  QP_CUDA(c, cudaMalloc((void**)&d_part, (size_t)ncta * (QP_MLP_NPARAM + 1) * sizeof(float)));
  QP_CUDA(c, cudaMalloc((void**)&d_grad, (QP_MLP_NPARAM + 1) * sizeof(float)));
  QP_CUDA(c, cudaMemcpyAsync(d_idx, idx.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  rc = mlp_gradient(c, d_idx, (int)n, d_part, ncta, d_grad, false, 0.f);
  std::vector<float> g(QP_MLP_NPARAM + 1);
  if (!rc) {
    QP_CUDA(c, cudaMemcpyAsync(g.data(), d_grad, g.size() * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    QP_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  cudaFree(d_idx);
  cudaFree(d_part);
  cudaFree(d_grad);
  c->mlp.n = keep;  // the probe samples are not kept
  if (rc) return rc;
  std::memcpy(grad, g.data(), QP_MLP_NPARAM * sizeof(float));
  if (loss) *loss = g[QP_MLP_NPARAM];
  return QPGPU_OK;
}

int qpgpu_mlp_predict(qpgpu_ctx* c, const float* X, int64_t n, float* y) {
  if (!c || !X || !y || n < 1) return QPGPU_ERR_ARG;
  if (!c->mlp.ready) return qpgpu_fail(c, QPGPU_ERR_STATE, "MLP not initialised");
  Lk l(c->mu);
  float *dX = nullptr, *dy = nullptr;
  QP_CUDA(c, cudaMalloc((void**)&dX, n * QP_MLP_IN * sizeof(float)));
  QP_CUDA(c, cudaMalloc((void**)&dy, n * sizeof(float)));
  QP_CUDA(c, cudaMemcpyAsync(dX, X, n * QP_MLP_IN * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  k_mlp_predict<<<gsz(n), 256, 0, c->stream>>>(c->mlp.params, dX, dy, n);
  cudaError_t e = cudaMemcpyAsync(y, dy, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(dX);
  cudaFree(dy);
  if (e != cudaSuccess) return qpgpu_fail(c, QPGPU_ERR_CUDA, cudaGetErrorString(e));
  return QPGPU_OK;
}

// Adam training on the stored samples: `epochs` passes over a seeded shuffle,
// minibatches of `batch`.  Returns the mean loss of the last epoch in *loss.
int qpgpu_mlp_train(qpgpu_ctx* c, int epochs, int batch, float lr, uint64_t seed, float* loss) {
  if (!c || epochs < 1 || batch < 1) return QPGPU_ERR_ARG;
  if (!c->mlp.ready) return qpgpu_fail(c, QPGPU_ERR_STATE, "MLP not initialised");
  Lk l(c->mu);
  const int64_t n = c->mlp.n;
  if (n < 1) return qpgpu_fail(c, QPGPU_ERR_STATE, "no training samples");
  const int ncta = 256;
  int* d_idx = nullptr;
  float *d_part = nullptr, *d_grad = nullptr;
  QP_CUDA(c, cudaMalloc((void**)&d_idx, n * sizeof(int)));
  QP_CUDA(c, cudaMalloc((void**)&d_part, (size_t)ncta * (QP_MLP_NPARAM + 1) * sizeof(float)));
  QP_CUDA(c, cudaMalloc((void**)&d_grad, (QP_MLP_NPARAM + 1) * sizeof(float)));
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::mt19937_64 gen(seed);
  double last = 0.0;
  int rc = 0;
  for (int ep = 0; ep < epochs && !rc; ++ep) {
    std::shuffle(idx.begin(), idx.end(), gen);
    QP_CUDA(c, cudaMemcpyAsync(d_idx, idx.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    std::vector<float> losses;
    for (int64_t b0 = 0; b0 < n && !rc; b0 += batch) {
      const int nb = (int)std::min<int64_t>(batch, n - b0);
      rc = mlp_gradient(c, d_idx + b0, nb, d_part, ncta, d_grad, true, lr);
    }
    if (ep == epochs - 1 && !rc) {
      // loss of the final parameters over all samples
      rc = mlp_gradient(c, d_idx, (int)std::min<int64_t>(n, 1 << 20), d_part, ncta, d_grad, false, 0.f);
      float g = 0.f;
      QP_CUDA(c, cudaMemcpyAsync(&g, d_grad + QP_MLP_NPARAM, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
      QP_CUDA(c, cudaStreamSynchronize(c->stream));
      last = g;
    }
  }
  QP_CUDA(c, cudaStreamSynchronize(c->stream));
  cudaFree(d_idx);
  cudaFree(d_part);
  cudaFree(d_grad);
  if (loss) *loss = (float)last;
  return rc;
}

}  // extern "C"
