// Small fully connected network for the learned local solver, trained on the GPU.
//
// Layers: n_in -> n_hidden (tanh) -> ... -> n_hidden (tanh) -> n_out (linear), FP32. The
// widths are small (tens of units), so every layer is a plain CUDA-core kernel with one
// thread per output element and a fixed summation order (results do not depend on the
// launch); the batched products are far too small for tensor-core tiles to pay.
// Training minimizes the mean squared error over all outputs with Adam (Kingma & Ba 2015:
// beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected moments), mini-batches in a seeded
// permutation per epoch.
// Parameter vector: for every layer l, W_l [out][in] row-major, then b_l [out].
#include "internal.h"

#include <cmath>
#include <numeric>

struct tpss_mlp
{
  int n_in = 0, n_hidden = 0, n_hidden_layers = 0, n_out = 0;
  std::vector<int> width;      // n_layers + 1 widths, width[0] = n_in
  std::vector<int64_t> w_off;  // offset of W_l in the parameter vector
  std::vector<int64_t> b_off;
  int64_t n_params = 0;
  tpss::DeviceBuffer<float> params, grads, adam_m, adam_v;
  int64_t adam_step = 0;
  // activations of the last forward pass (for backward): one buffer per layer output
  std::vector<tpss::DeviceBuffer<float>> act;
  tpss::DeviceBuffer<float> delta0, delta1, partial, xb, yb;
  int64_t act_rows = 0;
  int n_layers() const { return (int)width.size() - 1; }
};

namespace tpss
{
namespace
{
constexpr int kLossBlocks = 256;

__global__ void layer_fwd_kernel(const float *__restrict__ W, const float *__restrict__ b,
                                 const float *__restrict__ x, float *__restrict__ y, int64_t rows,
                                 int n_in, int n_out, int tanh_act)
{
  const int64_t total = rows * n_out;
  for(int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
      t += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t r = t / n_out;
    const int o = int(t % n_out);
    const float *xr = x + r * n_in, *wo = W + (int64_t)o * n_in;
    float acc = b[o];
    for(int i = 0; i < n_in; ++i) acc = fmaf(wo[i], xr[i], acc);
    y[t] = tanh_act ? tanhf(acc) : acc;
  }
}

// delta = 2 (y - target) / (rows * n_out); per-block partial sums of the squared error
__global__ void mse_kernel(const float *__restrict__ y, const float *__restrict__ target,
                           int64_t total, float scale, float *__restrict__ delta,
                           float *__restrict__ partial)
{
  __shared__ float red[256];
  float s = 0.f;
  for(int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
      t += (int64_t)gridDim.x * blockDim.x)
  {
    const float e = y[t] - target[t];
    s += e * e;
    if(delta) delta[t] = 2.f * scale * e;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for(int w = blockDim.x / 2; w > 0; w /= 2)
  {
    if(threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if(threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// dW[o][i] = sum_r delta[r][o] x[r][i], db[o] = sum_r delta[r][o]
__global__ void layer_wgrad_kernel(const float *__restrict__ delta, const float *__restrict__ x,
                                   int64_t rows, int n_in, int n_out, float *__restrict__ dW,
                                   float *__restrict__ db)
{
  const int64_t total = (int64_t)n_out * (n_in + 1);
  for(int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
      t += (int64_t)gridDim.x * blockDim.x)
  {
    const int o = int(t / (n_in + 1)), i = int(t % (n_in + 1));
    float acc = 0.f;
    if(i < n_in)
    {
      for(int64_t r = 0; r < rows; ++r) acc = fmaf(delta[r * n_out + o], x[r * n_in + i], acc);
      dW[(int64_t)o * n_in + i] = acc;
    }
    else
    {
      for(int64_t r = 0; r < rows; ++r) acc += delta[r * n_out + o];
      db[o] = acc;
    }
  }
}

// dx[r][i] = (sum_o W[o][i] delta[r][o]) * (1 - a[r][i]^2)   (a = tanh output of the layer below)
__global__ void layer_dgrad_kernel(const float *__restrict__ W, const float *__restrict__ delta,
                                   const float *__restrict__ a, int64_t rows, int n_in, int n_out,
                                   float *__restrict__ dx)
{
  const int64_t total = rows * n_in;
  for(int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
      t += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t r = t / n_in;
    const int i = int(t % n_in);
    float acc = 0.f;
    for(int o = 0; o < n_out; ++o) acc = fmaf(W[(int64_t)o * n_in + i], delta[r * n_out + o], acc);
    const float ai = a[t];
    dx[t] = acc * (1.f - ai * ai);
  }
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, int64_t n, float lr, float c1, float c2)
{
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
      i += (int64_t)gridDim.x * blockDim.x)
  {
    const float gi = g[i];
    const float mi = 0.9f * m[i] + 0.1f * gi;
    const float vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
  }
}

__global__ void gather_rows_kernel(const float *__restrict__ src, const int64_t *__restrict__ idx,
                                   int64_t rows, int width, float *__restrict__ dst)
{
  const int64_t total = rows * width;
  for(int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
      t += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t r = t / width;
    dst[t] = src[idx[r] * width + t % width];
  }
}

unsigned grid_of(int64_t n)
{
  const int64_t b = (n + 255) / 256, cap = (int64_t)num_sms() * 8;
  return (unsigned)(b < 1 ? 1 : (b < cap ? b : cap));
}

// splitmix64 (Steele, Lea, Flood 2014) for the seeded initialisation and shuffles
uint64_t splitmix(uint64_t &s)
{
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
double uniform01(uint64_t &s) { return (splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }
}  // namespace
}  // namespace tpss

namespace tpss
{
namespace
{
void ensure_rows(tpss_mlp &m, int64_t rows)
{
  if(rows <= m.act_rows) return;
  const int L = m.n_layers();
  m.act.resize(L);
  int wmax = 0;
  for(int w : m.width) wmax = std::max(wmax, w);
  for(int l = 0; l < L; ++l) m.act[l].resize((size_t)(rows * m.width[l + 1]));
  m.delta0.resize((size_t)(rows * wmax));
  m.delta1.resize((size_t)(rows * wmax));
  m.act_rows = rows;
}

// forward pass of `rows` inputs; the output is m.act[L-1]
void mlp_forward(tpss_mlp &m, const float *x, int64_t rows, cudaStream_t s)
{
  ensure_rows(m, rows);
  const int L = m.n_layers();
  const float *in = x;
  for(int l = 0; l < L; ++l)
  {
    const int ni = m.width[l], no = m.width[l + 1];
    layer_fwd_kernel<<<grid_of(rows * no), 256, 0, s>>>(m.params.ptr + m.w_off[l], m.params.ptr + m.b_off[l],
                                                        in, m.act[l].ptr, rows, ni, no, l + 1 < L);
    in = m.act[l].ptr;
  }
  TPSS_CUDA(cudaGetLastError());
}

// MSE loss of the last forward pass against `target` and its gradient in m.grads
void mlp_loss_backward(tpss_mlp &m, const float *x, const float *target, int64_t rows, cudaStream_t s,
                       bool want_loss, double *loss)
{
  const int L = m.n_layers();
  const int64_t total = rows * m.n_out;
  if(m.partial.n < (size_t)kLossBlocks) m.partial.resize(kLossBlocks);
  mse_kernel<<<kLossBlocks, 256, 0, s>>>(m.act[L - 1].ptr, target, total, 1.f / float(total),
                                         m.delta0.ptr, m.partial.ptr);
  TPSS_CUDA(cudaGetLastError());
  float *delta = m.delta0.ptr, *other = m.delta1.ptr;
  for(int l = L - 1; l >= 0; --l)
  {
    const int ni = m.width[l], no = m.width[l + 1];
    const float *in = l == 0 ? x : m.act[l - 1].ptr;
    layer_wgrad_kernel<<<grid_of((int64_t)no * (ni + 1)), 256, 0, s>>>(
      delta, in, rows, ni, no, m.grads.ptr + m.w_off[l], m.grads.ptr + m.b_off[l]);
    if(l > 0)
    {
      layer_dgrad_kernel<<<grid_of(rows * ni), 256, 0, s>>>(m.params.ptr + m.w_off[l], delta,
                                                            m.act[l - 1].ptr, rows, ni, no, other);
      std::swap(delta, other);
    }
  }
  TPSS_CUDA(cudaGetLastError());
  if(want_loss)
  {
    std::vector<float> h(kLossBlocks);
    TPSS_CUDA(cudaMemcpyAsync(h.data(), m.partial.ptr, sizeof(float) * kLossBlocks, cudaMemcpyDeviceToHost, s));
    TPSS_CUDA(cudaStreamSynchronize(s));
    double t = 0.0;
    for(float v : h) t += v;
    *loss = t / double(total);
  }
}

double mlp_loss_only(tpss_mlp &m, const float *x, const float *target, int64_t rows, cudaStream_t s)
{
  mlp_forward(m, x, rows, s);
  const int64_t total = rows * m.n_out;
  if(m.partial.n < (size_t)kLossBlocks) m.partial.resize(kLossBlocks);
  mse_kernel<<<kLossBlocks, 256, 0, s>>>(m.act[m.n_layers() - 1].ptr, target, total, 1.f, nullptr, m.partial.ptr);
  TPSS_CUDA(cudaGetLastError());
  std::vector<float> h(kLossBlocks);
  TPSS_CUDA(cudaMemcpyAsync(h.data(), m.partial.ptr, sizeof(float) * kLossBlocks, cudaMemcpyDeviceToHost, s));
  TPSS_CUDA(cudaStreamSynchronize(s));
  double t = 0.0;
  for(float v : h) t += v;
  return t / double(total);
}
}  // namespace

void mlp_infer(const tpss_mlp &mc, const float *x_dev, int64_t rows, float *y_dev, cudaStream_t s)
{
  tpss_mlp &m = const_cast<tpss_mlp &>(mc);  // activation scratch only
  mlp_forward(m, x_dev, rows, s);
  TPSS_CUDA(cudaMemcpyAsync(y_dev, m.act[m.n_layers() - 1].ptr, sizeof(float) * rows * m.n_out,
                            cudaMemcpyDeviceToDevice, s));
}

int mlp_n_in(const tpss_mlp &m) { return m.n_in; }
int mlp_n_out(const tpss_mlp &m) { return m.n_out; }
}  // namespace tpss

using namespace tpss;

extern "C" int tpss_mlp_create(const tpss_mlp_desc *d, tpss_mlp **out)
{
  return guarded([&] {
    TPSS_REQUIRE(d && out, "null argument");
    *out = nullptr;
    TPSS_REQUIRE(d->n_in >= 1 && d->n_out >= 1 && d->n_hidden >= 1 && d->n_hidden_layers >= 0 &&
                   d->n_in <= 4096 && d->n_out <= 4096 && d->n_hidden <= 4096 && d->n_hidden_layers <= 16,
                 "invalid network sizes");
    auto m = std::make_unique<tpss_mlp>();
    m->n_in = d->n_in;
    m->n_hidden = d->n_hidden;
    m->n_hidden_layers = d->n_hidden_layers;
    m->n_out = d->n_out;
    m->width.push_back(d->n_in);
    for(int l = 0; l < d->n_hidden_layers; ++l) m->width.push_back(d->n_hidden);
    m->width.push_back(d->n_out);
    const int L = m->n_layers();
    int64_t off = 0;
    for(int l = 0; l < L; ++l)
    {
      m->w_off.push_back(off);
      off += (int64_t)m->width[l] * m->width[l + 1];
      m->b_off.push_back(off);
      off += m->width[l + 1];
    }
    m->n_params = off;
    // Glorot-uniform weights, zero biases
    std::vector<float> p(off, 0.f);
    uint64_t st = d->seed;
    for(int l = 0; l < L; ++l)
    {
      const double a = std::sqrt(6.0 / (m->width[l] + m->width[l + 1]));
      for(int64_t i = 0; i < (int64_t)m->width[l] * m->width[l + 1]; ++i)
        p[m->w_off[l] + i] = float(a * (2.0 * uniform01(st) - 1.0));
    }
    m->params.upload(p.data(), p.size());
    m->grads.resize(off);
    std::vector<float> z(off, 0.f);
    m->adam_m.upload(z.data(), z.size());
    m->adam_v.upload(z.data(), z.size());
    *out = m.release();
  });
}

extern "C" int tpss_mlp_n_params(const tpss_mlp *m, int64_t *n)
{
  return guarded([&] {
    TPSS_REQUIRE(m && n, "null argument");
    *n = m->n_params;
  });
}

extern "C" int tpss_mlp_get_params(const tpss_mlp *m, float *host)
{
  return guarded([&] {
    TPSS_REQUIRE(m && host, "null argument");
    TPSS_CUDA(cudaMemcpy(host, m->params.ptr, sizeof(float) * m->n_params, cudaMemcpyDeviceToHost));
  });
}

extern "C" int tpss_mlp_set_params(tpss_mlp *m, const float *host)
{
  return guarded([&] {
    TPSS_REQUIRE(m && host, "null argument");
    for(int64_t i = 0; i < m->n_params; ++i) TPSS_REQUIRE(std::isfinite(host[i]), "parameters must be finite");
    TPSS_CUDA(cudaMemcpy(m->params.ptr, host, sizeof(float) * m->n_params, cudaMemcpyHostToDevice));
    m->adam_step = 0;
    TPSS_CUDA(cudaMemset(m->adam_m.ptr, 0, sizeof(float) * m->n_params));
    TPSS_CUDA(cudaMemset(m->adam_v.ptr, 0, sizeof(float) * m->n_params));
  });
}

extern "C" int tpss_mlp_forward(tpss_mlp *m, const float *x, int64_t rows, float *y, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(m && x && y && rows >= 0, "invalid argument");
    if(rows) mlp_infer(*m, x, rows, y, as_stream(stream));
  });
}

extern "C" int tpss_mlp_loss_grad(tpss_mlp *m, const float *x, const float *target, int64_t rows,
                                  double *loss, float *grad_host)
{
  return guarded([&] {
    TPSS_REQUIRE(m && x && target && loss && rows >= 1, "invalid argument");
    mlp_forward(*m, x, rows, nullptr);
    mlp_loss_backward(*m, x, target, rows, nullptr, true, loss);
    if(grad_host)
      TPSS_CUDA(cudaMemcpy(grad_host, m->grads.ptr, sizeof(float) * m->n_params, cudaMemcpyDeviceToHost));
  });
}

extern "C" int tpss_mlp_train(tpss_mlp *m, const float *x, const float *target, int64_t rows, int epochs,
                              int batch, double lr, uint64_t seed, double *loss_per_epoch, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(m && x && target && rows >= 1 && epochs >= 0 && batch >= 1 && lr > 0.0,
                 "invalid argument");
    cudaStream_t s = as_stream(stream);
    const int64_t B = std::min<int64_t>(batch, rows);
    if(m->xb.n < (size_t)(B * m->n_in)) m->xb.resize((size_t)(B * m->n_in));
    if(m->yb.n < (size_t)(B * m->n_out)) m->yb.resize((size_t)(B * m->n_out));
    std::vector<int64_t> perm(rows);
    DeviceBuffer<int64_t> dperm(rows);
    uint64_t st = seed;
    for(int ep = 0; ep < epochs; ++ep)
    {
      std::iota(perm.begin(), perm.end(), int64_t(0));
      for(int64_t i = rows - 1; i > 0; --i)  // Fisher-Yates
        std::swap(perm[i], perm[(int64_t)(splitmix(st) % uint64_t(i + 1))]);
      TPSS_CUDA(cudaMemcpyAsync(dperm.ptr, perm.data(), sizeof(int64_t) * rows, cudaMemcpyHostToDevice, s));
      for(int64_t b0 = 0; b0 + B <= rows; b0 += B)
      {
        gather_rows_kernel<<<grid_of(B * m->n_in), 256, 0, s>>>(x, dperm.ptr + b0, B, m->n_in, m->xb.ptr);
        gather_rows_kernel<<<grid_of(B * m->n_out), 256, 0, s>>>(target, dperm.ptr + b0, B, m->n_out, m->yb.ptr);
        mlp_forward(*m, m->xb.ptr, B, s);
        mlp_loss_backward(*m, m->xb.ptr, m->yb.ptr, B, s, false, nullptr);
        ++m->adam_step;
        const float c1 = float(1.0 - std::pow(0.9, double(m->adam_step)));
        const float c2 = float(1.0 - std::pow(0.999, double(m->adam_step)));
        adam_kernel<<<grid_of(m->n_params), 256, 0, s>>>(m->params.ptr, m->grads.ptr, m->adam_m.ptr,
                                                          m->adam_v.ptr, m->n_params, float(lr), c1, c2);
        TPSS_CUDA(cudaGetLastError());
      }
      // perm (pageable host memory) is reshuffled next epoch: wait for its copy and the epoch
      TPSS_CUDA(cudaStreamSynchronize(s));
      if(loss_per_epoch) loss_per_epoch[ep] = mlp_loss_only(*m, x, target, rows, s);
    }
  });
}

extern "C" int tpss_mlp_eval_loss(tpss_mlp *m, const float *x, const float *target, int64_t rows,
                                  double *loss)
{
  return guarded([&] {
    TPSS_REQUIRE(m && x && target && loss && rows >= 1, "invalid argument");
    *loss = mlp_loss_only(*m, x, target, rows, nullptr);
  });
}

extern "C" int tpss_mlp_sizes(const tpss_mlp *m, int *n_in, int *n_out)
{
  return guarded([&] {
    TPSS_REQUIRE(m, "null argument");
    if(n_in) *n_in = m->n_in;
    if(n_out) *n_out = m->n_out;
  });
}

extern "C" void tpss_mlp_destroy(tpss_mlp *m) { delete m; }
