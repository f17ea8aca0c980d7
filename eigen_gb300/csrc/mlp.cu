// The precision router's network: a 3-layer MLP in -> 64 -> 64 -> 1 (ReLU),
// FP32, trained on the GPU with Adam on the mean squared error, by the
// kernels below (no library): a fused forward + backward kernel (one thread
// per sample, parameters in shared memory, per-CTA gradient sums), a reduction
// + Adam kernel (fixed summation order over CTAs), and a prediction kernel.
//
// Parameter layout (floats): W1[in][64], b1[64], W2[64][64], b2[64], W3[64], b3.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "dense_driver.cuh"
#include "gbs_common.cuh"
#include "gbs_profile.cuh"

namespace gbs {
namespace {

constexpr int kW = 64;            // hidden width
constexpr int kMaxIn = 16;
constexpr int kSamplesPerCTA = 128;

__host__ __device__ constexpr int param_count(int in) { return in * kW + kW + kW * kW + kW + kW + 1; }

struct Layout {
  int w1, b1, w2, b2, w3, b3, total;
  __host__ __device__ explicit Layout(int in)
      : w1(0), b1(in * kW), w2(in * kW + kW), b2(in * kW + kW + kW * kW), w3(in * kW + 2 * kW + kW * kW),
        b3(in * kW + 3 * kW + kW * kW), total(param_count(in))
  {
  }
};

// Forward + backward for the CTA's chunk of samples; gradient sums (over the
// chunk) to part[blockIdx.x][P] and the chunk's summed squared error to
// lossp[blockIdx.x].  idx (optional) selects the samples (a shuffled
// minibatch).  Gradients are of mean((y - t)^2) over `total` samples.
// Shared memory: parameters, then per-sample rows (stride kW + 1, no bank
// conflicts): X, H1, H2, D2 = dL/d(pre-activation 2), D1 = dL/d(pre-act. 1), dy.
constexpr int kLd = kW + 1;
__host__ __device__ constexpr size_t grad_smem_floats(int in)
{
  return (size_t)param_count(in) + (size_t)kSamplesPerCTA * (kMaxIn + 1) + 4 * (size_t)kSamplesPerCTA * kLd +
         kSamplesPerCTA;
}

__global__ void __launch_bounds__(kSamplesPerCTA)
mlp_grad_kernel(int in, const float* __restrict__ params, const float* __restrict__ X, const float* __restrict__ T,
                const int* __restrict__ idx, int count, int total, float* __restrict__ part, double* __restrict__ lossp)
{
  extern __shared__ float sm[];
  const Layout L(in);
  float* p = sm;
  float* Xs = p + L.total;                          // [S][kMaxIn + 1]
  float* H1 = Xs + kSamplesPerCTA * (kMaxIn + 1);   // [S][kLd]
  float* H2 = H1 + kSamplesPerCTA * kLd;
  float* D2 = H2 + kSamplesPerCTA * kLd;
  float* D1 = D2 + kSamplesPerCTA * kLd;
  float* DY = D1 + kSamplesPerCTA * kLd;            // [S]
  for (int e = threadIdx.x; e < L.total; e += blockDim.x) p[e] = params[e];
  __syncthreads();
  const int t = threadIdx.x;
  const int s = blockIdx.x * kSamplesPerCTA + t;
  const bool live = s < count;
  const int row = live ? (idx ? idx[s] : s) : 0;
  float* xr = Xs + t * (kMaxIn + 1);
  float* h1 = H1 + t * kLd;
  float* h2 = H2 + t * kLd;
  float* d2 = D2 + t * kLd;
  float* d1 = D1 + t * kLd;
  for (int i = 0; i < kMaxIn; ++i) xr[i] = (live && i < in) ? X[(int64_t)row * in + i] : 0.f;
  // forward
  for (int j = 0; j < kW; ++j) {
    float a = p[L.b1 + j];
    for (int i = 0; i < in; ++i) a = fmaf(xr[i], p[L.w1 + i * kW + j], a);
    h1[j] = a > 0.f ? a : 0.f;
  }
  for (int j = 0; j < kW; ++j) {
    float a = p[L.b2 + j];
    for (int i = 0; i < kW; ++i) a = fmaf(h1[i], p[L.w2 + i * kW + j], a);
    h2[j] = a > 0.f ? a : 0.f;
  }
  float y = p[L.b3];
  for (int i = 0; i < kW; ++i) y = fmaf(h2[i], p[L.w3 + i], y);
  const float err = live ? y - T[row] : 0.f;
  const double sq = (double)err * err;
  const float dy = 2.f * err / (float)total;
  DY[t] = dy;
  // backward through the activations
  for (int j = 0; j < kW; ++j) d2[j] = h2[j] > 0.f ? dy * p[L.w3 + j] : 0.f;
  for (int i = 0; i < kW; ++i) {
    float a = 0.f;
    for (int j = 0; j < kW; ++j) a = fmaf(p[L.w2 + i * kW + j], d2[j], a);
    d1[i] = h1[i] > 0.f ? a : 0.f;
  }
  __syncthreads();
  // weight gradients: dot products over the CTA's samples, one parameter per
  // thread at a time (fixed order, no atomics)
  for (int e = t; e < L.total; e += kSamplesPerCTA) {
    float acc = 0.f;
    if (e < L.b1) {                    // W1[i][j] : sum_s x[s][i] d1[s][j]
      const int i = e / kW, j = e % kW;
      for (int q = 0; q < kSamplesPerCTA; ++q) acc = fmaf(Xs[q * (kMaxIn + 1) + i], D1[q * kLd + j], acc);
    } else if (e < L.w2) {             // b1[j]
      const int j = e - L.b1;
      for (int q = 0; q < kSamplesPerCTA; ++q) acc += D1[q * kLd + j];
    } else if (e < L.b2) {             // W2[i][j] : sum_s h1[s][i] d2[s][j]
      const int i = (e - L.w2) / kW, j = (e - L.w2) % kW;
      for (int q = 0; q < kSamplesPerCTA; ++q) acc = fmaf(H1[q * kLd + i], D2[q * kLd + j], acc);
    } else if (e < L.w3) {             // b2[j]
      const int j = e - L.b2;
      for (int q = 0; q < kSamplesPerCTA; ++q) acc += D2[q * kLd + j];
    } else if (e < L.b3) {             // W3[i] : sum_s h2[s][i] dy[s]
      const int i = e - L.w3;
      for (int q = 0; q < kSamplesPerCTA; ++q) acc = fmaf(H2[q * kLd + i], DY[q], acc);
    } else {                           // b3
      for (int q = 0; q < kSamplesPerCTA; ++q) acc += DY[q];
    }
    part[(int64_t)blockIdx.x * L.total + e] = acc;
  }
  // per-CTA squared error, fixed order
  __shared__ double sq_s[kSamplesPerCTA];
  sq_s[t] = sq;
  __syncthreads();
  if (t == 0) {
    double tot = 0.0;
    for (int i = 0; i < kSamplesPerCTA; ++i) tot += sq_s[i];
    lossp[blockIdx.x] = tot;
  }
}

// grad[p] = sum over CTAs (in order); optional Adam step on params.
__global__ void mlp_reduce_adam_kernel(int P, int nparts, const float* __restrict__ part, float* __restrict__ grad,
                                       float* __restrict__ params, float* __restrict__ m, float* __restrict__ v,
                                       float lr, float b1, float b2, float eps, int step, int apply)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  float gs = 0.f;
  for (int c = 0; c < nparts; ++c) gs += part[(int64_t)c * P + i];
  grad[i] = gs;
  if (!apply) return;
  const float mi = b1 * m[i] + (1.f - b1) * gs;
  const float vi = b2 * v[i] + (1.f - b2) * gs * gs;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.f - powf(b1, (float)step));
  const float vh = vi / (1.f - powf(b2, (float)step));
  params[i] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void __launch_bounds__(kSamplesPerCTA)
mlp_predict_kernel(int in, const float* __restrict__ params, const float* __restrict__ X, int count,
                   float* __restrict__ Y)
{
  extern __shared__ float sm[];
  const Layout L(in);
  for (int e = threadIdx.x; e < L.total; e += blockDim.x) sm[e] = params[e];
  __syncthreads();
  const float* p = sm;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < count; s += gridDim.x * blockDim.x) {
    float x[kMaxIn];
#pragma unroll
    for (int i = 0; i < kMaxIn; ++i) x[i] = i < in ? X[(int64_t)s * in + i] : 0.f;
    float h1[kW];
#pragma unroll
    for (int j = 0; j < kW; ++j) {
      float a = p[L.b1 + j];
#pragma unroll
      for (int i = 0; i < kMaxIn; ++i)
        if (i < in) a = fmaf(x[i], p[L.w1 + i * kW + j], a);
      h1[j] = a > 0.f ? a : 0.f;
    }
    float y = p[L.b3];
#pragma unroll 4
    for (int j = 0; j < kW; ++j) {
      float a = p[L.b2 + j];
#pragma unroll
      for (int i = 0; i < kW; ++i) a = fmaf(h1[i], p[L.w2 + i * kW + j], a);
      y = fmaf(a > 0.f ? a : 0.f, p[L.w3 + j], y);
    }
    Y[s] = y;
  }
}

// predicted log10 kappa -> tier: 1 = FP32 LU + refinement, 2 = FP32 LU +
// GMRES-IR, 0 = FP64 LU
__global__ void router_route_kernel(const float* __restrict__ pred, int count, float t_ir, float t_gmres,
                                    int* __restrict__ tier)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) {
    const float v = pred[i];
    tier[i] = v <= t_ir ? 1 : (v <= t_gmres ? 2 : 0);
  }
}

uint64_t splitmix(uint64_t& s)
{
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

}  // namespace
}  // namespace gbs

using namespace gbs;

struct gbs_mlp {
  int in = 0;
  int P = 0;
  int step = 0;
  DevBuf params, grad, m, v, part, lossp, idx;
  cudaStream_t stream = nullptr;
};

extern "C" int gbs_mlp_create(gbs_mlp** out, int in_dim, int width, uint64_t seed)
{
  if (!out || in_dim < 1 || in_dim > kMaxIn || width != kW) return GBS_INVALID_ARGUMENT;
  *out = nullptr;
  GBS_TRY(ensure_device());
  gbs_mlp* o = new gbs_mlp();
  o->in = in_dim;
  o->P = param_count(in_dim);
  int rc;
  if ((rc = o->params.reserve(sizeof(float) * o->P)) || (rc = o->grad.reserve(sizeof(float) * o->P)) ||
      (rc = o->m.reserve(sizeof(float) * o->P)) || (rc = o->v.reserve(sizeof(float) * o->P))) {
    delete o;
    return rc;
  }
  // He-uniform initialisation from a seeded splitmix64 stream; zero biases
  const Layout L(in_dim);
  std::vector<float> h((size_t)o->P, 0.f);
  uint64_t s = seed;
  auto uni = [&](float bound) { return (float)(((splitmix(s) >> 11) * 0x1.0p-53) * 2.0 - 1.0) * bound; };
  for (int i = 0; i < in_dim * kW; ++i) h[(size_t)L.w1 + i] = uni(std::sqrt(6.f / in_dim));
  for (int i = 0; i < kW * kW; ++i) h[(size_t)L.w2 + i] = uni(std::sqrt(6.f / kW));
  for (int i = 0; i < kW; ++i) h[(size_t)L.w3 + i] = uni(std::sqrt(3.f / kW));
  cudaMemcpy(o->params.p, h.data(), sizeof(float) * o->P, cudaMemcpyHostToDevice);
  cudaMemset(o->m.p, 0, sizeof(float) * o->P);
  cudaMemset(o->v.p, 0, sizeof(float) * o->P);
  cudaStreamCreateWithFlags(&o->stream, cudaStreamDefault);
  *out = o;
  return GBS_SUCCESS;
}

extern "C" int gbs_mlp_destroy(gbs_mlp* o)
{
  if (!o) return GBS_SUCCESS;
  if (o->stream) {
    cudaStreamSynchronize(o->stream);
    cudaStreamDestroy(o->stream);
  }
  delete o;
  return GBS_SUCCESS;
}

extern "C" int gbs_mlp_param_count(const gbs_mlp* o) { return o ? o->P : 0; }

extern "C" int gbs_mlp_get_params(const gbs_mlp* o, float* host)
{
  if (!o || !host) return GBS_INVALID_ARGUMENT;
  GBS_CUDA_TRY(cudaMemcpy(host, o->params.p, sizeof(float) * o->P, cudaMemcpyDeviceToHost));
  return GBS_SUCCESS;
}

extern "C" int gbs_mlp_set_params(gbs_mlp* o, const float* host)
{
  if (!o || !host) return GBS_INVALID_ARGUMENT;
  GBS_CUDA_TRY(cudaMemcpy(o->params.p, host, sizeof(float) * o->P, cudaMemcpyHostToDevice));
  GBS_CUDA_TRY(cudaMemset(o->m.p, 0, sizeof(float) * o->P));
  GBS_CUDA_TRY(cudaMemset(o->v.p, 0, sizeof(float) * o->P));
  o->step = 0;
  return GBS_SUCCESS;
}

// One pass over `count` samples (optionally gathered through d_idx): gradient
// of the mean squared error; with apply != 0 an Adam step follows.
static int grad_pass(gbs_mlp* o, const float* d_x, const float* d_t, const int* d_idx, int count, float lr, int apply,
                     double* loss)
{
  const int nparts = (count + kSamplesPerCTA - 1) / kSamplesPerCTA;
  GBS_TRY(o->part.reserve(sizeof(float) * (size_t)nparts * o->P));
  GBS_TRY(o->lossp.reserve(sizeof(double) * (size_t)nparts));
  cudaStream_t s = o->stream;
  const size_t smem = sizeof(float) * grad_smem_floats(o->in);
  static const cudaError_t attr = cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        (int)(sizeof(float) * grad_smem_floats(kMaxIn)));
  GBS_CUDA_TRY(attr);
  {
    PhaseScope ps(s, PH_ROUTER, 6.0 * count * (double)o->P, 4.0 * count * (o->in + 1));
    mlp_grad_kernel<<<nparts, kSamplesPerCTA, smem, s>>>(o->in, o->params.as<float>(), d_x, d_t, d_idx, count, count,
                                                          o->part.as<float>(), o->lossp.as<double>());
    GBS_CUDA_TRY(cudaGetLastError());
  }
  if (apply) ++o->step;
  count_launch();
  mlp_reduce_adam_kernel<<<(o->P + 255) / 256, 256, 0, s>>>(o->P, nparts, o->part.as<float>(), o->grad.as<float>(),
                                                           o->params.as<float>(), o->m.as<float>(), o->v.as<float>(), lr,
                                                           0.9f, 0.999f, 1e-8f, o->step, apply);
  GBS_CUDA_TRY(cudaGetLastError());
  if (loss) {
    std::vector<double> h((size_t)nparts);
    GBS_CUDA_TRY(cudaMemcpyAsync(h.data(), o->lossp.p, sizeof(double) * nparts, cudaMemcpyDeviceToHost, s));
    GBS_CUDA_TRY(cudaStreamSynchronize(s));
    double t = 0;
    for (double v : h) t += v;
    *loss = t / std::max(count, 1);
  }
  return GBS_SUCCESS;
}

extern "C" int gbs_mlp_gradients(gbs_mlp* o, const float* d_x, const float* d_t, int count, float* h_grad, double* loss)
{
  if (!o || count <= 0 || !d_x || !d_t) return GBS_INVALID_ARGUMENT;
  GBS_TRY(grad_pass(o, d_x, d_t, nullptr, count, 0.f, 0, loss));
  if (h_grad) {
    GBS_CUDA_TRY(cudaStreamSynchronize(o->stream));
    GBS_CUDA_TRY(cudaMemcpy(h_grad, o->grad.p, sizeof(float) * o->P, cudaMemcpyDeviceToHost));
  }
  return GBS_SUCCESS;
}

extern "C" int gbs_mlp_train_step(gbs_mlp* o, const float* d_x, const float* d_t, int count, float lr, double* loss)
{
  if (!o || count <= 0 || !d_x || !d_t) return GBS_INVALID_ARGUMENT;
  return grad_pass(o, d_x, d_t, nullptr, count, lr, 1, loss);
}

// Minibatch Adam over `epochs` passes of a seeded shuffle of the samples.
extern "C" int gbs_mlp_fit(gbs_mlp* o, const float* d_x, const float* d_t, int count, int epochs, int batch, float lr,
                           uint64_t seed, double* final_loss)
{
  if (!o || count <= 0 || epochs < 0 || batch <= 0 || !d_x || !d_t) return GBS_INVALID_ARGUMENT;
  GBS_TRY(o->idx.reserve(sizeof(int) * (size_t)count));
  std::vector<int> perm((size_t)count);
  for (int i = 0; i < count; ++i) perm[(size_t)i] = i;
  uint64_t s = seed;
  double loss = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    for (int i = count - 1; i > 0; --i) std::swap(perm[(size_t)i], perm[(size_t)(splitmix(s) % (uint64_t)(i + 1))]);
    GBS_CUDA_TRY(cudaMemcpyAsync(o->idx.p, perm.data(), sizeof(int) * count, cudaMemcpyHostToDevice, o->stream));
    for (int b0 = 0; b0 < count; b0 += batch) {
      const int nb = std::min(batch, count - b0);
      GBS_TRY(grad_pass(o, d_x, d_t, o->idx.as<int>() + b0, nb, lr, 1,
                        (ep == epochs - 1 && b0 + batch >= count) ? &loss : nullptr));
    }
  }
  GBS_CUDA_TRY(cudaStreamSynchronize(o->stream));
  if (final_loss) *final_loss = loss;
  return GBS_SUCCESS;
}

extern "C" int gbs_mlp_predict(const gbs_mlp* o, const float* d_x, int count, float* d_y, void* stream)
{
  if (!o || count < 0 || (count > 0 && (!d_x || !d_y))) return GBS_INVALID_ARGUMENT;
  if (count == 0) return GBS_SUCCESS;
  cudaStream_t s = (cudaStream_t)stream;     // NULL: the legacy default stream
  const int grid = std::min((count + kSamplesPerCTA - 1) / kSamplesPerCTA, 8 * device_sm_count());
  PhaseScope ps(s, PH_ROUTER, 2.0 * count * (double)o->P, 4.0 * count * (o->in + 1));
  mlp_predict_kernel<<<grid, kSamplesPerCTA, sizeof(float) * o->P, s>>>(o->in, o->params.as<float>(), d_x, count, d_y);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

extern "C" int gbs_router_route(const float* d_pred, int count, float t_ir, float t_gmres, int* d_tier, void* stream)
{
  if (count < 0 || (count > 0 && (!d_pred || !d_tier))) return GBS_INVALID_ARGUMENT;
  if (count == 0) return GBS_SUCCESS;
  count_launch();
  router_route_kernel<<<(count + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_pred, count, t_ir, t_gmres, d_tier);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}
