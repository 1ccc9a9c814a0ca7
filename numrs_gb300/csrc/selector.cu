// Learned tile selector: a small MLP cost model trained on autotuner timings
// (no reference counterpart).
//
// features[F] -> Linear(F,H) -> ReLU -> Linear(H,H) -> ReLU -> Linear(H,V):
// one predicted log2(microseconds per problem) per grouped-kernel tile
// variant. Parameters live as an fp32 master copy (Adam updates) and a BF16
// copy that every forward pass reads; products accumulate in fp32. Training,
// inference and gradients run on the GPU in this file's kernels:
//   mlp_forward      one CTA per sample, activations kept for backward;
//   mlp_backward     per-sample deltas (dL/dz of every layer) and the loss;
//   mlp_grad         one thread per parameter, summing over the minibatch in
//                    sample order (deterministic, no atomics);
//   adam_step        fp32 Adam update + BF16 refresh.
// The selector never changes numerics: it only picks among tile variants that
// all pass the same parity tests.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include <cuda_bf16.h>

#include "nrs_internal.cuh"

struct nrs_selector {
  int F = 0, H = 0, V = 0;
  int64_t n_params = 0;
  int64_t off_w1, off_b1, off_w2, off_b2, off_w3, off_b3;
  float* master = nullptr;           // fp32 parameters
  __nv_bfloat16* wbf = nullptr;      // bf16 copy read by the forward pass
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  float* grads = nullptr;            // scratch gradient buffer
  int64_t step = 0;
  // per-batch scratch (grown on demand)
  int64_t cap = 0;
  float *h1 = nullptr, *h2 = nullptr, *y = nullptr, *d1 = nullptr, *d2 = nullptr, *d3 = nullptr;
  float* loss = nullptr;
  float *bx = nullptr, *bt = nullptr, *bm = nullptr;  // gathered minibatch
};

namespace {

constexpr int kMaxH = 128;
constexpr int kMaxF = 16;
constexpr int kMaxV = 16;

__global__ void mlp_forward(int64_t B, int F, int H, int V, const float* __restrict__ x,
                            const __nv_bfloat16* __restrict__ w, int64_t ow1, int64_t ob1,
                            int64_t ow2, int64_t ob2, int64_t ow3, int64_t ob3,
                            float* __restrict__ h1, float* __restrict__ h2, float* __restrict__ y) {
  __shared__ float sx[kMaxF], s1[kMaxH], s2[kMaxH];
  const int64_t b = blockIdx.x;
  if (b >= B) return;
  const int t = threadIdx.x;
  if (t < F) sx[t] = x[b * F + t];
  __syncthreads();
  if (t < H) {
    float acc = 0.f;
    for (int i = 0; i < F; ++i) acc += sx[i] * __bfloat162float(w[ow1 + (int64_t)t * F + i]);
    acc += __bfloat162float(w[ob1 + t]);
    acc = acc > 0.f ? acc : 0.f;
    s1[t] = acc;
    h1[b * H + t] = acc;
  }
  __syncthreads();
  if (t < H) {
    float acc = 0.f;
    for (int i = 0; i < H; ++i) acc += s1[i] * __bfloat162float(w[ow2 + (int64_t)t * H + i]);
    acc += __bfloat162float(w[ob2 + t]);
    acc = acc > 0.f ? acc : 0.f;
    s2[t] = acc;
    h2[b * H + t] = acc;
  }
  __syncthreads();
  if (t < V) {
    float acc = 0.f;
    for (int i = 0; i < H; ++i) acc += s2[i] * __bfloat162float(w[ow3 + (int64_t)t * H + i]);
    acc += __bfloat162float(w[ob3 + t]);
    y[b * V + t] = acc;
  }
}

// Mask sum of the minibatch (one CTA, fixed order).
__global__ void mask_total(int64_t n, const float* __restrict__ mask, float* out) {
  __shared__ float sh[256];
  float acc = 0.f;
  for (int64_t i = threadIdx.x; i < n; i += 256) acc += mask[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int i = 0; i < 256; ++i) s += sh[i];
    out[0] = s > 0.f ? s : 1.f;
  }
}

// Per-sample deltas. d3 = dL/dy, d2 = dL/dz2, d1 = dL/dz1 (ReLU gates).
__global__ void mlp_backward(int64_t B, int F, int H, int V, const float* __restrict__ t,
                             const float* __restrict__ mask, const float* __restrict__ denom,
                             const __nv_bfloat16* __restrict__ w, int64_t ow2, int64_t ow3,
                             const float* __restrict__ h1, const float* __restrict__ h2,
                             const float* __restrict__ y, float* __restrict__ d1,
                             float* __restrict__ d2, float* __restrict__ d3) {
  __shared__ float s3[kMaxV], s2[kMaxH];
  const int64_t b = blockIdx.x;
  if (b >= B) return;
  const int th = threadIdx.x;
  const float dn = denom[0];
  if (th < V) {
    const float diff = y[b * V + th] - t[b * V + th];
    const float g = 2.f * mask[b * V + th] * diff / dn;
    s3[th] = g;
    d3[b * V + th] = g;
  }
  __syncthreads();
  if (th < H) {
    float acc = 0.f;
    for (int o = 0; o < V; ++o) acc += s3[o] * __bfloat162float(w[ow3 + (int64_t)o * H + th]);
    const float g = h2[b * H + th] > 0.f ? acc : 0.f;
    s2[th] = g;
    d2[b * H + th] = g;
  }
  __syncthreads();
  if (th < H) {
    float acc = 0.f;
    for (int o = 0; o < H; ++o) acc += s2[o] * __bfloat162float(w[ow2 + (int64_t)o * H + th]);
    d1[b * H + th] = h1[b * H + th] > 0.f ? acc : 0.f;
  }
}

// Loss = sum(mask * (y - t)^2) / denom, one CTA, fixed order.
__global__ void mlp_loss(int64_t n, const float* __restrict__ y, const float* __restrict__ t,
                         const float* __restrict__ mask, const float* __restrict__ denom, float* out) {
  __shared__ float sh[256];
  float acc = 0.f;
  for (int64_t i = threadIdx.x; i < n; i += 256) {
    const float d = y[i] - t[i];
    acc += mask[i] * d * d;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int i = 0; i < 256; ++i) s += sh[i];
    out[0] = s / denom[0];
  }
}

// One thread per parameter: dW[o,i] = sum_b delta[b,o] * act[b,i],
// db[o] = sum_b delta[b,o], in sample order.
__global__ void mlp_grad(int64_t B, int F, int H, int V, const float* __restrict__ x,
                         const float* __restrict__ h1, const float* __restrict__ h2,
                         const float* __restrict__ d1, const float* __restrict__ d2,
                         const float* __restrict__ d3, int64_t ow1, int64_t ob1, int64_t ow2,
                         int64_t ob2, int64_t ow3, int64_t ob3, int64_t n_params,
                         float* __restrict__ g) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n_params) return;
  const float* delta;
  const float* act = nullptr;
  int dO, aI, o, i = 0;
  if (p < ob1) {
    o = (int)((p - ow1) / F); i = (int)((p - ow1) % F); delta = d1; dO = H; act = x; aI = F;
  } else if (p < ow2) {
    o = (int)(p - ob1); delta = d1; dO = H; aI = 0;
  } else if (p < ob2) {
    o = (int)((p - ow2) / H); i = (int)((p - ow2) % H); delta = d2; dO = H; act = h1; aI = H;
  } else if (p < ow3) {
    o = (int)(p - ob2); delta = d2; dO = H; aI = 0;
  } else if (p < ob3) {
    o = (int)((p - ow3) / H); i = (int)((p - ow3) % H); delta = d3; dO = V; act = h2; aI = H;
  } else {
    o = (int)(p - ob3); delta = d3; dO = V; aI = 0;
  }
  float acc = 0.f;
  if (act) {
    for (int64_t b = 0; b < B; ++b) acc += delta[b * dO + o] * act[b * aI + i];
  } else {
    for (int64_t b = 0; b < B; ++b) acc += delta[b * dO + o];
  }
  g[p] = acc;
}

__global__ void adam_step(int64_t n, float* __restrict__ p, const float* __restrict__ g,
                          float* __restrict__ m, float* __restrict__ v, __nv_bfloat16* __restrict__ pb,
                          float lr, float b1c, float b2c) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  const float gi = g[i];
  const float mi = beta1 * m[i] + (1.f - beta1) * gi;
  const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float upd = lr * (mi / b1c) / (sqrtf(vi / b2c) + eps);
  const float np = p[i] - upd;
  p[i] = np;
  pb[i] = __float2bfloat16_rn(np);
}

__global__ void to_bf16(int64_t n, const float* __restrict__ p, __nv_bfloat16* __restrict__ pb) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) pb[i] = __float2bfloat16_rn(p[i]);
}

// Gathers rows idx[b] of x/t/mask into the minibatch buffers.
__global__ void gather_rows(int64_t B, const int64_t* __restrict__ idx, int F, int V,
                            const float* __restrict__ x, const float* __restrict__ t,
                            const float* __restrict__ mask, float* bx, float* bt, float* bm) {
  const int64_t b = blockIdx.x;
  if (b >= B) return;
  const int64_t r = idx[b];
  for (int j = threadIdx.x; j < F; j += blockDim.x) bx[b * F + j] = x[r * F + j];
  for (int j = threadIdx.x; j < V; j += blockDim.x) {
    bt[b * V + j] = t[r * V + j];
    bm[b * V + j] = mask[r * V + j];
  }
}

int ensure_cap(nrs_handle* h, nrs_selector* s, int64_t B) {
  if (B <= s->cap) return NRS_OK;
  float** bufs[] = {&s->h1, &s->h2, &s->y, &s->d1, &s->d2, &s->d3, &s->bx, &s->bt, &s->bm};
  for (auto b : bufs) {
    cudaFree(*b);
    *b = nullptr;
  }
  const size_t sizes[] = {(size_t)B * s->H, (size_t)B * s->H, (size_t)B * s->V, (size_t)B * s->H,
                          (size_t)B * s->H, (size_t)B * s->V, (size_t)B * s->F, (size_t)B * s->V,
                          (size_t)B * s->V};
  for (int i = 0; i < 9; ++i)
    if (cudaMalloc(bufs[i], sizes[i] * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      s->cap = 0;
      return nrs_fail(h, NRS_ERR_ALLOC, "selector scratch");
    }
  s->cap = B;
  return NRS_OK;
}

int forward(nrs_handle* h, nrs_selector* s, int64_t B, const float* x) {
  mlp_forward<<<(unsigned)B, kMaxH, 0, h->stream>>>(B, s->F, s->H, s->V, x, s->wbf, s->off_w1,
                                                    s->off_b1, s->off_w2, s->off_b2, s->off_w3,
                                                    s->off_b3, s->h1, s->h2, s->y);
  return nrs_after_launch(h, "mlp_forward");
}

// forward + backward + gradient on a minibatch already in device buffers.
int fwd_bwd(nrs_handle* h, nrs_selector* s, int64_t B, const float* x, const float* t,
            const float* mask) {
  int st = forward(h, s, B, x);
  if (st) return st;
  mask_total<<<1, 256, 0, h->stream>>>(B * s->V, mask, s->loss + 1);
  mlp_backward<<<(unsigned)B, kMaxH, 0, h->stream>>>(B, s->F, s->H, s->V, t, mask, s->loss + 1,
                                                     s->wbf, s->off_w2, s->off_w3, s->h1, s->h2,
                                                     s->y, s->d1, s->d2, s->d3);
  mlp_loss<<<1, 256, 0, h->stream>>>(B * s->V, s->y, t, mask, s->loss + 1, s->loss);
  mlp_grad<<<(unsigned)((s->n_params + 127) / 128), 128, 0, h->stream>>>(
      B, s->F, s->H, s->V, x, s->h1, s->h2, s->d1, s->d2, s->d3, s->off_w1, s->off_b1, s->off_w2,
      s->off_b2, s->off_w3, s->off_b3, s->n_params, s->grads);
  return nrs_after_launch(h, "mlp backward");
}

}  // namespace

bool nrs_handle_has_selector(nrs_handle* h) { return h && h->selector != nullptr; }

extern "C" int nrs_selector_create(nrs_handle* h, int F, int H, int V, uint64_t seed,
                                   nrs_selector** out) {
  if (!h || !out || F < 1 || F > kMaxF || H < 1 || H > kMaxH || V < 1 || V > kMaxV)
    return NRS_ERR_INVALID;
  *out = nullptr;
  nrs_selector* s = new nrs_selector();
  s->F = F;
  s->H = H;
  s->V = V;
  s->off_w1 = 0;
  s->off_b1 = s->off_w1 + (int64_t)H * F;
  s->off_w2 = s->off_b1 + H;
  s->off_b2 = s->off_w2 + (int64_t)H * H;
  s->off_w3 = s->off_b2 + H;
  s->off_b3 = s->off_w3 + (int64_t)V * H;
  s->n_params = s->off_b3 + V;
  // He-uniform initialisation from the seed (host), then upload.
  std::vector<float> p((size_t)s->n_params, 0.f);
  std::mt19937_64 rng(seed);
  auto fill = [&](int64_t off, int64_t count, int fan_in) {
    const float lim = std::sqrt(6.f / (float)fan_in);
    std::uniform_real_distribution<float> U(-lim, lim);
    for (int64_t i = 0; i < count; ++i) p[(size_t)(off + i)] = U(rng);
  };
  fill(s->off_w1, (int64_t)H * F, F);
  fill(s->off_w2, (int64_t)H * H, H);
  fill(s->off_w3, (int64_t)V * H, H);
  const size_t nb = (size_t)s->n_params * sizeof(float);
  if (cudaMalloc(&s->master, nb) || cudaMalloc(&s->wbf, (size_t)s->n_params * 2) ||
      cudaMalloc(&s->adam_m, nb) || cudaMalloc(&s->adam_v, nb) || cudaMalloc(&s->grads, nb) ||
      cudaMalloc(&s->loss, 4 * sizeof(float))) {
    cudaGetLastError();
    nrs_selector_destroy(s);
    return nrs_fail(h, NRS_ERR_ALLOC, "selector parameters");
  }
  cudaMemcpy(s->master, p.data(), nb, cudaMemcpyHostToDevice);
  cudaMemset(s->adam_m, 0, nb);
  cudaMemset(s->adam_v, 0, nb);
  to_bf16<<<(unsigned)((s->n_params + 255) / 256), 256, 0, h->stream>>>(s->n_params, s->master, s->wbf);
  int st = nrs_after_launch(h, "to_bf16");
  if (st) {
    nrs_selector_destroy(s);
    return st;
  }
  *out = s;
  return NRS_OK;
}

extern "C" int nrs_selector_destroy(nrs_selector* s) {
  if (!s) return NRS_ERR_INVALID;
  float* bufs[] = {s->master, s->adam_m, s->adam_v, s->grads, s->h1, s->h2, s->y,
                   s->d1, s->d2, s->d3, s->loss, s->bx, s->bt, s->bm};
  for (float* b : bufs) cudaFree(b);
  cudaFree(s->wbf);
  delete s;
  return NRS_OK;
}

extern "C" int64_t nrs_selector_num_params(nrs_selector* s) { return s ? s->n_params : -1; }

int nrs_selector_shape(nrs_selector* s, int* F, int* H, int* V) {
  if (!s) return NRS_ERR_INVALID;
  *F = s->F;
  *H = s->H;
  *V = s->V;
  return NRS_OK;
}

extern "C" int nrs_selector_get_params(nrs_handle* h, nrs_selector* s, float* host) {
  if (!h || !s || !host) return NRS_ERR_INVALID;
  int st = nrs_cuda_check(h, cudaStreamSynchronize(h->stream), "sync");
  if (st) return st;
  return nrs_cuda_check(h, cudaMemcpy(host, s->master, (size_t)s->n_params * 4, cudaMemcpyDeviceToHost),
                        "cudaMemcpy(params)");
}

extern "C" int nrs_selector_set_params(nrs_handle* h, nrs_selector* s, const float* host) {
  if (!h || !s || !host) return NRS_ERR_INVALID;
  int st = nrs_cuda_check(h, cudaMemcpyAsync(s->master, host, (size_t)s->n_params * 4,
                                             cudaMemcpyHostToDevice, h->stream),
                          "cudaMemcpy(params)");
  if (st) return st;
  to_bf16<<<(unsigned)((s->n_params + 255) / 256), 256, 0, h->stream>>>(s->n_params, s->master, s->wbf);
  st = nrs_after_launch(h, "to_bf16");
  if (st) return st;
  return nrs_cuda_check(h, cudaStreamSynchronize(h->stream), "sync");
}

extern "C" int nrs_selector_forward_backward(nrs_handle* h, nrs_selector* s, int64_t B,
                                             const float* x, const float* t, const float* mask,
                                             float* y, float* grads, float* loss) {
  if (!h || !s || B < 1 || !x || !t || !mask) return NRS_ERR_INVALID;
  h->last_error.clear();
  int st = ensure_cap(h, s, B);
  if (st) return st;
  if ((st = fwd_bwd(h, s, B, x, t, mask))) return st;
  if (y) cudaMemcpyAsync(y, s->y, (size_t)B * s->V * 4, cudaMemcpyDeviceToDevice, h->stream);
  if (grads) cudaMemcpyAsync(grads, s->grads, (size_t)s->n_params * 4, cudaMemcpyDeviceToDevice, h->stream);
  if (loss) {
    st = nrs_cuda_check(h, cudaMemcpyAsync(loss, s->loss, 4, cudaMemcpyDeviceToHost, h->stream), "loss");
    if (st) return st;
    return nrs_cuda_check(h, cudaStreamSynchronize(h->stream), "sync");
  }
  return nrs_after_launch(h, "forward_backward");
}

extern "C" int nrs_selector_train(nrs_handle* h, nrs_selector* s, int64_t n, const float* x,
                                  const float* t, const float* mask, int epochs, int64_t batch,
                                  float lr, uint64_t seed, float* loss) {
  if (!h || !s || n < 1 || !x || !t || !mask || epochs < 1 || batch < 1) return NRS_ERR_INVALID;
  h->last_error.clear();
  int st = ensure_cap(h, s, batch);
  if (st) return st;
  int64_t* d_idx = nullptr;
  if ((st = nrs_cuda_check(h, cudaMalloc(&d_idx, (size_t)n * 8), "cudaMalloc(perm)"))) return st;
  std::vector<int64_t> perm((size_t)n);
  std::iota(perm.begin(), perm.end(), 0);
  std::mt19937_64 rng(seed);
  double last_epoch_loss = 0.0;
  std::vector<float> batch_losses;
  for (int ep = 0; ep < epochs && !st; ++ep) {
    std::shuffle(perm.begin(), perm.end(), rng);
    cudaMemcpyAsync(d_idx, perm.data(), (size_t)n * 8, cudaMemcpyHostToDevice, h->stream);
    const bool last = (ep == epochs - 1);
    int nb = 0;
    double acc = 0.0;
    for (int64_t b0 = 0; b0 < n; b0 += batch) {
      const int64_t B = (n - b0) < batch ? (n - b0) : batch;
      gather_rows<<<(unsigned)B, 32, 0, h->stream>>>(B, d_idx + b0, s->F, s->V, x, t, mask, s->bx,
                                                     s->bt, s->bm);
      if ((st = fwd_bwd(h, s, B, s->bx, s->bt, s->bm))) break;
      ++s->step;
      const float b1c = 1.f - std::pow(0.9f, (float)s->step);
      const float b2c = 1.f - std::pow(0.999f, (float)s->step);
      adam_step<<<(unsigned)((s->n_params + 255) / 256), 256, 0, h->stream>>>(
          s->n_params, s->master, s->grads, s->adam_m, s->adam_v, s->wbf, lr, b1c, b2c);
      if (last) {
        float l = 0.f;
        cudaMemcpyAsync(&l, s->loss, 4, cudaMemcpyDeviceToHost, h->stream);
        cudaStreamSynchronize(h->stream);
        acc += l;
        ++nb;
      }
    }
    // the pageable copy of perm above must finish before perm is reshuffled
    if (!st) st = nrs_cuda_check(h, cudaStreamSynchronize(h->stream), "train epoch");
    if (last && nb) last_epoch_loss = acc / nb;
  }
  cudaFree(d_idx);
  if (loss) *loss = (float)last_epoch_loss;
  return st;
}

extern "C" int nrs_selector_predict(nrs_handle* h, nrs_selector* s, int64_t n, const float* x,
                                    float* y) {
  if (!h || !s || n < 1 || !x || !y) return NRS_ERR_INVALID;
  h->last_error.clear();
  int st = ensure_cap(h, s, n);
  if (st) return st;
  if ((st = forward(h, s, n, x))) return st;
  return nrs_cuda_check(h, cudaMemcpyAsync(y, s->y, (size_t)n * s->V * 4, cudaMemcpyDeviceToDevice,
                                           h->stream),
                        "predict copy");
}

extern "C" int nrs_tuner_set_selector(nrs_handle* h, nrs_selector* s) {
  if (!h) return NRS_ERR_INVALID;
  h->selector = s;
  return NRS_OK;
}

// Picks the variant with the smallest predicted time among those of each
// problem's dtype (plan creation for shapes the tuner table lacks).
int nrs_selector_choose(nrs_handle* h, int n, const float* host_feat, const int* dtypes,
                        int* variant_out) {
  nrs_selector* s = h->selector;
  if (!s || s->F != 7 || s->V != NRS_TILE_VARIANTS) return NRS_ERR_UNSUPPORTED;
  float *dx = nullptr, *dy = nullptr;
  if (cudaMalloc(&dx, (size_t)n * 7 * 4) || cudaMalloc(&dy, (size_t)n * s->V * 4)) {
    cudaGetLastError();
    cudaFree(dx);
    return NRS_ERR_ALLOC;
  }
  std::vector<float> y((size_t)n * s->V);
  cudaMemcpyAsync(dx, host_feat, (size_t)n * 7 * 4, cudaMemcpyHostToDevice, h->stream);
  int st = nrs_selector_predict(h, s, n, dx, dy);
  if (!st) st = nrs_cuda_check(h, cudaMemcpyAsync(y.data(), dy, y.size() * 4, cudaMemcpyDeviceToHost, h->stream), "copy");
  if (!st) st = nrs_cuda_check(h, cudaStreamSynchronize(h->stream), "sync");
  cudaFree(dx);
  cudaFree(dy);
  if (st) return st;
  for (int i = 0; i < n; ++i) {
    int best = -1;
    float bt = 1e30f;
    for (int v = 0; v < s->V; ++v) {
      int vd = 0;
      nrs_tile_variant_info(v, nullptr, nullptr, nullptr, &vd);
      if (vd != dtypes[i]) continue;
      if (y[(size_t)i * s->V + v] < bt) {
        bt = y[(size_t)i * s->V + v];
        best = v;
      }
    }
    variant_out[i] = best;
  }
  return NRS_OK;
}
