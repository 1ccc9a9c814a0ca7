// Grouped persistent launch: thousands of uneven GEMMs and row reductions in
// ONE kernel launch (no reference counterpart; the reference's analogue is a
// caller loop over Array::matmul / batched_gemm, src/array/linalg.rs:56-136,
// and over kernels::reduce::sum_*).
//
// nrs_plan_create turns the problems into a work queue of GEMM tiles (tile
// shape and split-K from the autotuner table, else the learned selector, else
// a size heuristic) and row-reduction tasks, ordered longest first. The
// persistent kernel's CTAs pull items from an atomic counter. GEMM tiles run
// the same tile bodies as the standalone GEMM kernels (gemm_tiles.cuh), and a
// row reduction follows the flat-reduction order of nrs_reduce
// (reduce_common.cuh), so grouped results equal the one-by-one results bit
// for bit (split-K tiles excepted: their K order differs by construction).
//
// Split-K is deterministic without any waiting: every split writes its
// partial tile to workspace and bumps a per-tile counter; the CTA that
// arrives last sums the partials in split order 0..S-1, writes C and resets
// the counter for the next replay. No CTA ever waits on another.
#include <algorithm>
#include <cmath>
#include <map>
#include <tuple>
#include <vector>

#include "gemm_tiles.cuh"
#include "reduce_common.cuh"

using namespace nrs_tiles;
using namespace nrs_red;

namespace {

struct WorkItem {
  int32_t kind;     // 0 = GEMM tile, 1 = row reduction
  int32_t prob;     // problem index
  int32_t variant;  // tile variant (GEMM)
  int32_t tm, tn;   // tile coordinates
  int32_t split, nsplit;
  int32_t slot;     // split-K tile slot, -1 if unsplit
};

struct VariantDesc {
  int bm, bn, split, dtype;
};
// Tile variants of the grouped kernel (index = variant id).
constexpr VariantDesc kVariants[NRS_TILE_VARIANTS] = {
    {64, 64, 1, NRS_F32}, {32, 32, 1, NRS_F32}, {32, 32, 4, NRS_F32},
    {64, 64, 1, NRS_F64}, {32, 32, 1, NRS_F64}, {32, 32, 4, NRS_F64}};

using TileF32L = Simt<float, 64, 64, 16, 4, 4>;
using TileF32S = Simt<float, 32, 32, 16, 2, 2>;
using TileF64L = Dmma<64, 64, 2, 4>;
using TileF64S = Dmma<32, 32, 2, 4>;
constexpr int kSmem = TileF64L::kSmem > TileF32L::kSmem ? TileF64L::kSmem : TileF32L::kSmem;
constexpr int kThreads = 256;
// Workspace bytes of one split-K tile slot: nsplit partial tiles.
constexpr int kSlotBytes = 4 * 32 * 32 * 8;
static_assert(kVariants[2].split * kVariants[2].bm * kVariants[2].bn * 4 <= kSlotBytes, "slot size");
static_assert(kVariants[5].split * kVariants[5].bm * kVariants[5].bn * 8 <= kSlotBytes, "slot size");

template <typename T, typename Tile, int BM, int BN>
__device__ void gemm_item(const nrs_gemm_desc& g, const WorkItem& w, uint8_t* smem,
                          unsigned* tile_cnt, uint8_t* partials, int* s_last) {
  const int64_t m0 = (int64_t)w.tm * BM, n0 = (int64_t)w.tn * BN;
  int64_t k0 = 0, k1 = g.k;
  if (w.nsplit > 1) {
    const int64_t kc = ((g.k + w.nsplit - 1) / w.nsplit + 15) / 16 * 16;
    k0 = w.split * kc < g.k ? w.split * kc : g.k;
    k1 = k0 + kc < g.k ? k0 + kc : g.k;
  }
  const bool ta = g.flags & NRS_GEMM_TRANS_A, tb = g.flags & NRS_GEMM_TRANS_B;
  const int64_t rsa = ta ? 1 : g.lda, csa = ta ? g.lda : 1;
  const int64_t rsb = tb ? 1 : g.ldb, csb = tb ? g.ldb : 1;
  Tile t;
  t.run((const T*)g.A, rsa, csa, (const T*)g.B, rsb, csb, g.m, g.n, m0, n0, k0, k1, smem);
  const bool acc = g.flags & NRS_GEMM_ACCUMULATE;
  if (w.nsplit <= 1) {
    tile_store<T>(t, (T*)g.C, g.ldc, g.m, g.n, m0, n0, acc);
    return;
  }
  T* base = reinterpret_cast<T*>(partials + (size_t)w.slot * kSlotBytes);
  T* mine = base + (size_t)w.split * BM * BN;
#pragma unroll
  for (int e = 0; e < Tile::kPerThread; ++e) {
    int r, c;
    t.coords(e, r, c);
    mine[r * BN + c] = (T)t.value(e);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned old = atomicAdd(&tile_cnt[w.slot], 1u);
    *s_last = (old == (unsigned)(w.nsplit - 1));
  }
  __syncthreads();
  if (*s_last) {
    __threadfence();
    for (int idx = threadIdx.x; idx < BM * BN; idx += blockDim.x) {
      const int r = idx / BN, c = idx % BN;
      const int64_t gi = m0 + r, gj = n0 + c;
      if (gi >= g.m || gj >= g.n) continue;
      T s = __ldcg(base + idx);
      for (int sp = 1; sp < w.nsplit; ++sp) s = s + __ldcg(base + (size_t)sp * BM * BN + idx);
      T* p = (T*)g.C + gi * g.ldc + gj;
      *p = acc ? (*p + s) : s;
    }
    if (threadIdx.x == 0) tile_cnt[w.slot] = 0;  // ready for the next replay
  }
}

// One row, the flat-reduction order of nrs_reduce: chunks of 8192 (SUM/MEAN
// below 10000 elements: one chunk), lane-striped tree per chunk, chunk
// partials folded in order by thread 0.
template <typename T, int OP>
__device__ void row_reduce_t(const T* __restrict__ x, int64_t len, void* out, uint8_t* smem) {
  T* sh = reinterpret_cast<T*>(smem);
  const int64_t chunk = ((OP == NRS_SUM || OP == NRS_MEAN) && len < 10000) ? (len > 0 ? len : 1) : 8192;
  T total = Fold<T, OP>::init();
  int nan = 0;
  for (int64_t c0 = 0; c0 < len; c0 += chunk) {
    const int64_t clen = (len - c0) < chunk ? (len - c0) : chunk;
    T acc = Fold<T, OP>::init();
    int tn = 0;
    for (int64_t i = threadIdx.x; i < clen; i += kThreads) {
      const T v = x[c0 + i];
      if constexpr (OP == NRS_MAX || OP == NRS_MIN) {
        tn |= (v != v);
        if (v == v) acc = Fold<T, OP>::step(acc, v);
      } else {
        acc = Fold<T, OP>::step(acc, v);
      }
    }
    T r = block_combine<T, OP>(acc, sh);
    const int anynan = __syncthreads_or(tn);
    if constexpr (std::is_floating_point<T>::value && (OP == NRS_MAX || OP == NRS_MIN)) {
      // An extreme of zero: the left-to-right fold keeps the chunk's first
      // zero (-0.0 and +0.0 tie), which the striped tree does not track.
      __shared__ int zflag;
      __shared__ unsigned long long fzs;
      if (threadIdx.x == 0) {
        zflag = r == T(0);
        fzs = (unsigned long long)clen;
      }
      __syncthreads();
      if (zflag) {
        for (int64_t i = threadIdx.x; i < clen; i += kThreads)
          if (x[c0 + i] == T(0)) {
            atomicMin(&fzs, (unsigned long long)i);
            break;
          }
        __syncthreads();
        if (threadIdx.x == 0) r = x[c0 + (int64_t)fzs];
      }
      __syncthreads();  // zflag / fzs are free for the next chunk
    }
    if (threadIdx.x == 0) {
      total = Fold<T, OP>::step(total, Fold<T, OP>::step(Fold<T, OP>::init(), r));
      nan |= anynan;
    }
  }
  if (threadIdx.x == 0) {
    if constexpr (OP == NRS_MAX || OP == NRS_MIN) {
      if constexpr (std::is_floating_point<T>::value) {
        if (nan) total = (T)NAN;
      }
      static_cast<T*>(out)[0] = len == 0 ? T(0) : total;
    } else if constexpr (OP == NRS_MEAN) {
      if constexpr (std::is_floating_point<T>::value)
        static_cast<T*>(out)[0] = len == 0 ? T(0) : total / (T)len;
      else
        static_cast<double*>(out)[0] = len == 0 ? 0.0 : (double)total / (double)len;
    } else {
      static_cast<T*>(out)[0] = total;
    }
  }
  __syncthreads();
}

template <typename T>
__device__ void row_reduce_ops(const nrs_rowreduce_desc& r, uint8_t* smem) {
  const T* x = static_cast<const T*>(r.x);
  switch (r.op) {
    case NRS_SUM: row_reduce_t<T, NRS_SUM>(x, r.len, r.out, smem); break;
    case NRS_MEAN: row_reduce_t<T, NRS_MEAN>(x, r.len, r.out, smem); break;
    case NRS_MAX: row_reduce_t<T, NRS_MAX>(x, r.len, r.out, smem); break;
    default: row_reduce_t<T, NRS_MIN>(x, r.len, r.out, smem); break;
  }
}

__global__ void __launch_bounds__(kThreads)
    grouped_kernel(const nrs_gemm_desc* __restrict__ gp, const nrs_rowreduce_desc* __restrict__ rp,
                   const WorkItem* __restrict__ items, int n_items, unsigned* queue,
                   unsigned* tile_cnt, uint8_t* partials) {
  __shared__ __align__(16) uint8_t smem[kSmem];
  __shared__ int s_item, s_last;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(queue, 1u);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= n_items) return;
    const WorkItem w = items[it];
    if (w.kind == 1) {
      const nrs_rowreduce_desc r = rp[w.prob];
      if (r.dtype == NRS_F32) row_reduce_ops<float>(r, smem);
      else if (r.dtype == NRS_F64) row_reduce_ops<double>(r, smem);
      else row_reduce_ops<int64_t>(r, smem);
      continue;
    }
    const nrs_gemm_desc g = gp[w.prob];
    switch (w.variant) {
      case 0: gemm_item<float, TileF32L, 64, 64>(g, w, smem, tile_cnt, partials, &s_last); break;
      case 1:
      case 2: gemm_item<float, TileF32S, 32, 32>(g, w, smem, tile_cnt, partials, &s_last); break;
      case 3: gemm_item<double, TileF64L, 64, 64>(g, w, smem, tile_cnt, partials, &s_last); break;
      default: gemm_item<double, TileF64S, 32, 32>(g, w, smem, tile_cnt, partials, &s_last); break;
    }
    __syncthreads();
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct nrs_plan {
  nrs_handle* h = nullptr;
  int64_t n_items = 0, gemm_tiles = 0;
  // f64 / f32 GEMMs on the tensor cores (nrs_plan_options.f64_mode /
  // f32_mode = OZAKI); they run before the persistent kernel, which then
  // holds none of them.
  nrs_ozaki_group* oz = nullptr;
  int64_t oz_gemms = 0;
  nrs_ozaki_group* oz32 = nullptr;
  int64_t oz32_gemms = 0;
  nrs_gemm_desc* d_gemm = nullptr;
  nrs_rowreduce_desc* d_red = nullptr;
  WorkItem* d_items = nullptr;
  unsigned* d_counters = nullptr;  // [0] = queue, [1..] = split-K tile counters
  uint8_t* d_partials = nullptr;
  int grid = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
};

int nrs_selector_choose(nrs_handle* h, int n, const float* host_feat, const int* dtypes,
                        int* variant_out);
bool nrs_handle_has_selector(nrs_handle* h);

namespace {

// Size heuristic used when neither the tuner nor the selector has an answer.
int heuristic_variant(int dtype, int64_t m, int64_t k, int64_t n) {
  const int64_t mx = m > n ? m : n;
  if (dtype == NRS_F32) {
    if (m * n >= 128 * 128) return 0;
    return (k >= 8 * mx && m * n <= 64 * 64) ? 2 : 1;
  }
  if (m * n >= 256 * 256) return 3;
  return (k >= 8 * mx && m * n <= 64 * 64) ? 5 : 4;
}

void selector_features(const nrs_gemm_desc& d, int64_t batch, float* f) {
  auto lg = [](double v) { return (float)(std::log2(v < 1 ? 1.0 : v) / 14.0); };
  f[0] = lg((double)d.m);
  f[1] = lg((double)d.n);
  f[2] = lg((double)d.k);
  f[3] = d.dtype == NRS_F64 ? 1.f : 0.f;
  f[4] = (d.flags & NRS_GEMM_TRANS_A) ? 1.f : 0.f;
  f[5] = (d.flags & NRS_GEMM_TRANS_B) ? 1.f : 0.f;
  f[6] = lg((double)batch);
}

void plan_free(nrs_plan* p) {
  if (!p) return;
  nrs_ozaki_group_free(p->oz);
  nrs_ozaki_group_free(p->oz32);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->ev_in) cudaEventDestroy(p->ev_in);
  if (p->ev_out) cudaEventDestroy(p->ev_out);
  cudaFree(p->d_gemm);
  cudaFree(p->d_red);
  cudaFree(p->d_items);
  cudaFree(p->d_counters);
  cudaFree(p->d_partials);
  delete p;
}

// forced >= 0 forces every GEMM onto that variant (autotuning).
int plan_build(nrs_handle* h, int64_t n_gemm, const nrs_gemm_desc* gemms, int64_t n_red,
               const nrs_rowreduce_desc* reds, int forced, const nrs_plan_options* opt, nrs_plan** out) {
  *out = nullptr;
  if (opt && (opt->f64_mode != NRS_PLAN_F64_DMMA && opt->f64_mode != NRS_PLAN_F64_OZAKI))
    return nrs_fail(h, NRS_ERR_INVALID, "unknown f64 mode");
  if (opt && (opt->f32_mode != NRS_PLAN_F32_FMA && opt->f32_mode != NRS_PLAN_F32_OZAKI))
    return nrs_fail(h, NRS_ERR_INVALID, "unknown f32 mode");
  std::vector<int> var((size_t)n_gemm, -1);
  std::vector<int> need_sel;
  for (int64_t i = 0; i < n_gemm; ++i) {
    const nrs_gemm_desc& d = gemms[i];
    if (d.dtype != NRS_F32 && d.dtype != NRS_F64)
      return nrs_fail(h, NRS_ERR_DTYPE, "grouped GEMMs take f32 or f64");
    if (d.m < 0 || d.k < 0 || d.n < 0) return nrs_fail(h, NRS_ERR_SHAPE, "negative GEMM dimension");
    if (d.flags & ~(NRS_GEMM_ACCUMULATE | NRS_GEMM_TRANS_A | NRS_GEMM_TRANS_B))
      return nrs_fail(h, NRS_ERR_INVALID, "unknown GEMM flag");
    const bool ta = d.flags & NRS_GEMM_TRANS_A, tb = d.flags & NRS_GEMM_TRANS_B;
    if (d.ldc < (d.n > 0 ? d.n : 1) || d.lda < ((ta ? d.m : d.k) > 0 ? (ta ? d.m : d.k) : 1) ||
        d.ldb < ((tb ? d.k : d.n) > 0 ? (tb ? d.k : d.n) : 1))
      return nrs_fail(h, NRS_ERR_SHAPE, "leading dimension too small");
    if (d.m * d.n > 0 && (!d.C || (d.k > 0 && (!d.A || !d.B))))
      return nrs_fail(h, NRS_ERR_INVALID, "null operand");
    if (forced >= 0) {
      if (kVariants[forced].dtype != d.dtype) return nrs_fail(h, NRS_ERR_DTYPE, "variant/dtype mismatch");
      var[i] = forced;
      continue;
    }
    const int t = nrs_tuner_get(h, d.dtype, d.m, d.k, d.n);
    if (t >= 0 && kVariants[t].dtype == d.dtype) var[i] = t;
    else need_sel.push_back((int)i);
  }
  if (!need_sel.empty()) {
    bool done = false;
    if (nrs_handle_has_selector(h)) {
      std::vector<float> feat(need_sel.size() * 7);
      std::vector<int> dts(need_sel.size()), choice(need_sel.size());
      for (size_t j = 0; j < need_sel.size(); ++j) {
        selector_features(gemms[need_sel[j]], n_gemm, &feat[j * 7]);
        dts[j] = gemms[need_sel[j]].dtype;
      }
      if (nrs_selector_choose(h, (int)need_sel.size(), feat.data(), dts.data(), choice.data()) == NRS_OK) {
        for (size_t j = 0; j < need_sel.size(); ++j) var[need_sel[j]] = choice[j];
        done = true;
      }
    }
    if (!done)
      for (int i : need_sel) var[i] = heuristic_variant(gemms[i].dtype, gemms[i].m, gemms[i].k, gemms[i].n);
  }
  for (int64_t i = 0; i < n_red; ++i) {
    const nrs_rowreduce_desc& r = reds[i];
    if (r.dtype != NRS_F32 && r.dtype != NRS_F64 && r.dtype != NRS_I64)
      return nrs_fail(h, NRS_ERR_DTYPE, "grouped reductions take f32, f64 or i64");
    if (r.op != NRS_SUM && r.op != NRS_MEAN && r.op != NRS_MAX && r.op != NRS_MIN)
      return nrs_fail(h, NRS_ERR_INVALID, "grouped reductions: SUM, MEAN, MAX or MIN");
    if (r.len < 0 || !r.out || (r.len > 0 && !r.x)) return nrs_fail(h, NRS_ERR_INVALID, "bad row reduction");
  }
  // f64 / f32 GEMMs on the tensor cores: each group takes what it can, the
  // rest stays on DMMA / FMA tiles.
  std::vector<int> on_tc((size_t)n_gemm, 0), on_tc32((size_t)n_gemm, 0);
  nrs_ozaki_group* oz = nullptr;
  nrs_ozaki_group* oz32 = nullptr;
  if (opt && opt->f64_mode == NRS_PLAN_F64_OZAKI && forced < 0 && n_gemm > 0) {
    int st = nrs_ozaki_group_build(h, n_gemm, gemms, NRS_F64, opt->f64_slices, opt->f64_digit_bits, on_tc.data(),
                                   &oz);
    if (st) return st;
  }
  if (opt && opt->f32_mode == NRS_PLAN_F32_OZAKI && forced < 0 && n_gemm > 0) {
    int st = nrs_ozaki_group_build(h, n_gemm, gemms, NRS_F32, 0, 0, on_tc32.data(), &oz32);
    if (st) {
      nrs_ozaki_group_free(oz);
      return st;
    }
  }
  // Work items with a cost estimate (ns on one SM) for longest-first order.
  struct Costed {
    double cost;
    WorkItem w;
  };
  std::vector<Costed> items;
  int slots = 0;
  const double sms = h->num_sms > 0 ? h->num_sms : 1;
  const double f64_rate = 1.2e12 / sms, f32_rate = 60e12 / sms, bw = 6.5e12 / sms;
  int64_t gemm_tiles = 0;
  int64_t oz_gemms = 0, oz32_gemms = 0;
  for (int64_t i = 0; i < n_gemm; ++i) {
    const nrs_gemm_desc& d = gemms[i];
    if (on_tc[i] || on_tc32[i]) {
      ++(on_tc[i] ? oz_gemms : oz32_gemms);
      continue;
    }
    if (d.m == 0 || d.n == 0) continue;
    const VariantDesc& v = kVariants[var[i]];
    const int tm = (int)((d.m + v.bm - 1) / v.bm), tn = (int)((d.n + v.bn - 1) / v.bn);
    const int ns = (d.k > 0) ? v.split : 1;
    const double kk = (double)(d.k > 0 ? d.k : 1) / ns;
    const double cost = 2.0 * v.bm * v.bn * kk / (d.dtype == NRS_F64 ? f64_rate : f32_rate) * 1e9 + 500;
    for (int a = 0; a < tm; ++a)
      for (int b = 0; b < tn; ++b) {
        const int slot = ns > 1 ? slots++ : -1;
        for (int s = 0; s < ns; ++s) {
          items.push_back({cost, WorkItem{0, (int32_t)i, var[i], a, b, s, ns, slot}});
          ++gemm_tiles;
        }
      }
  }
  for (int64_t i = 0; i < n_red; ++i) {
    const double cost = (double)reds[i].len * 8 / bw * 1e9 + 500;
    items.push_back({cost, WorkItem{1, (int32_t)i, -1, 0, 0, 0, 1, -1}});
  }
  std::stable_sort(items.begin(), items.end(), [](const Costed& a, const Costed& b) { return a.cost > b.cost; });
  if (items.size() > 0x7fffffff) {
    nrs_ozaki_group_free(oz);
    nrs_ozaki_group_free(oz32);
    return nrs_fail(h, NRS_ERR_TOO_LARGE, "too many work items");
  }

  nrs_plan* p = new nrs_plan();
  p->h = h;
  p->oz = oz;
  p->oz_gemms = oz_gemms;
  p->oz32 = oz32;
  p->oz32_gemms = oz32_gemms;
  p->n_items = (int64_t)items.size();
  p->gemm_tiles = gemm_tiles;
  std::vector<WorkItem> wi(items.size());
  for (size_t i = 0; i < items.size(); ++i) wi[i] = items[i].w;
  const size_t partial_bytes = (size_t)slots * kSlotBytes + 256;
  auto fail = [&](cudaError_t e, const char* what) {
    int s = nrs_cuda_check(h, e, what);
    plan_free(p);
    return s;
  };
  cudaError_t e;
  if ((e = cudaMalloc(&p->d_gemm, sizeof(nrs_gemm_desc) * (n_gemm > 0 ? n_gemm : 1)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&p->d_red, sizeof(nrs_rowreduce_desc) * (n_red > 0 ? n_red : 1)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&p->d_items, sizeof(WorkItem) * (wi.size() > 0 ? wi.size() : 1)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&p->d_counters, sizeof(unsigned) * (1 + slots)))) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&p->d_partials, partial_bytes))) return fail(e, "cudaMalloc");
  if (n_gemm && (e = cudaMemcpy(p->d_gemm, gemms, sizeof(nrs_gemm_desc) * n_gemm, cudaMemcpyHostToDevice)))
    return fail(e, "cudaMemcpy");
  if (n_red && (e = cudaMemcpy(p->d_red, reds, sizeof(nrs_rowreduce_desc) * n_red, cudaMemcpyHostToDevice)))
    return fail(e, "cudaMemcpy");
  if (!wi.empty() && (e = cudaMemcpy(p->d_items, wi.data(), sizeof(WorkItem) * wi.size(), cudaMemcpyHostToDevice)))
    return fail(e, "cudaMemcpy");
  if ((e = cudaMemset(p->d_counters, 0, sizeof(unsigned) * (1 + slots)))) return fail(e, "cudaMemset");
  int blocks_per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, grouped_kernel, kThreads, 0);
  if (blocks_per_sm < 1) blocks_per_sm = 1;
  int64_t want = (int64_t)h->num_sms * blocks_per_sm;
  p->grid = (int)(want < (p->n_items > 0 ? p->n_items : 1) ? want : (p->n_items > 0 ? p->n_items : 1));
  if ((e = cudaEventCreateWithFlags(&p->ev_in, cudaEventDisableTiming))) return fail(e, "cudaEventCreate");
  if ((e = cudaEventCreateWithFlags(&p->ev_out, cudaEventDisableTiming))) return fail(e, "cudaEventCreate");
  *out = p;
  return NRS_OK;
}

int plan_launch(nrs_handle* h, nrs_plan* p, cudaStream_t s) {
  for (nrs_ozaki_group* g : {p->oz, p->oz32}) {
    if (!g) continue;
    int st = nrs_ozaki_group_launch(h, g, s);
    if (st) return st;
  }
  if (p->n_items == 0) return NRS_OK;
  cudaMemsetAsync(p->d_counters, 0, sizeof(unsigned), s);
  grouped_kernel<<<p->grid, kThreads, 0, s>>>(p->d_gemm, p->d_red, p->d_items, (int)p->n_items,
                                              p->d_counters, p->d_counters + 1, p->d_partials);
  return nrs_after_launch(h, "grouped_kernel");
}

}  // namespace

extern "C" int nrs_plan_create(nrs_handle* h, int64_t n_gemm, const nrs_gemm_desc* gemms,
                               int64_t n_red, const nrs_rowreduce_desc* reds, nrs_plan** out) {
  if (!h || !out || n_gemm < 0 || n_red < 0 || (n_gemm && !gemms) || (n_red && !reds))
    return NRS_ERR_INVALID;
  h->last_error.clear();
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;
  return plan_build(h, n_gemm, gemms, n_red, reds, -1, nullptr, out);
}

extern "C" int nrs_plan_create_ex(nrs_handle* h, int64_t n_gemm, const nrs_gemm_desc* gemms, int64_t n_red,
                                  const nrs_rowreduce_desc* reds, const nrs_plan_options* opt, nrs_plan** out) {
  if (!h || !out || n_gemm < 0 || n_red < 0 || (n_gemm && !gemms) || (n_red && !reds))
    return NRS_ERR_INVALID;
  h->last_error.clear();
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;
  return plan_build(h, n_gemm, gemms, n_red, reds, -1, opt, out);
}

extern "C" int nrs_plan_f64_info(nrs_plan* p, int64_t* on_tensor_cores, int* slices, int* digit_bits) {
  if (!p) return NRS_ERR_INVALID;
  int s = 0, b = 0;
  if (p->oz) nrs_ozaki_group_info(p->oz, &s, &b, nullptr);
  if (on_tensor_cores) *on_tensor_cores = p->oz_gemms;
  if (slices) *slices = s;
  if (digit_bits) *digit_bits = b;
  return NRS_OK;
}

extern "C" int nrs_plan_f32_info(nrs_plan* p, int64_t* on_tensor_cores, int* slices, int* digit_bits) {
  if (!p) return NRS_ERR_INVALID;
  int s = 0, b = 0;
  if (p->oz32) nrs_ozaki_group_info(p->oz32, &s, &b, nullptr);
  if (on_tensor_cores) *on_tensor_cores = p->oz32_gemms;
  if (slices) *slices = s;
  if (digit_bits) *digit_bits = b;
  return NRS_OK;
}

extern "C" int nrs_plan_run(nrs_handle* h, nrs_plan* p, int use_graph) {
  if (!h || !p || p->h != h) return NRS_ERR_INVALID;
  h->last_error.clear();
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;
  if (p->n_items == 0 && !p->oz && !p->oz32) return NRS_OK;
  if (!use_graph) return plan_launch(h, p, h->stream);
  cudaStream_t gs = h->own_stream;
  if (!p->exec) {
    cudaError_t e = cudaStreamBeginCapture(gs, cudaStreamCaptureModeThreadLocal);
    if (e) return nrs_cuda_check(h, e, "cudaStreamBeginCapture");
    plan_launch(h, p, gs);
    e = cudaStreamEndCapture(gs, &p->graph);
    if (e) return nrs_cuda_check(h, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&p->exec, p->graph, 0);
    if (e) return nrs_cuda_check(h, e, "cudaGraphInstantiate");
  }
  if (gs != h->stream) {
    cudaEventRecord(p->ev_in, h->stream);
    cudaStreamWaitEvent(gs, p->ev_in, 0);
  }
  st = nrs_cuda_check(h, cudaGraphLaunch(p->exec, gs), "cudaGraphLaunch");
  if (st) return st;
  if (gs != h->stream) {
    cudaEventRecord(p->ev_out, gs);
    cudaStreamWaitEvent(h->stream, p->ev_out, 0);
  }
  return NRS_OK;
}

extern "C" int nrs_plan_stats(nrs_plan* p, int64_t* work_items, int64_t* gemm_tiles) {
  if (!p) return NRS_ERR_INVALID;
  if (work_items) *work_items = p->n_items;
  if (gemm_tiles) *gemm_tiles = p->gemm_tiles;
  return NRS_OK;
}

extern "C" int nrs_plan_destroy(nrs_plan* p) {
  if (!p) return NRS_ERR_INVALID;
  cudaSetDevice(p->h->device);
  cudaStreamSynchronize(p->h->stream);
  cudaStreamSynchronize(p->h->own_stream);
  plan_free(p);
  return NRS_OK;
}

extern "C" int nrs_tile_variant_info(int v, int* tile_m, int* tile_n, int* split_k, int* dtype) {
  if (v < 0 || v >= NRS_TILE_VARIANTS) return NRS_ERR_INVALID;
  if (tile_m) *tile_m = kVariants[v].bm;
  if (tile_n) *tile_n = kVariants[v].bn;
  if (split_k) *split_k = kVariants[v].split;
  if (dtype) *dtype = kVariants[v].dtype;
  return NRS_OK;
}

// Exhaustive autotuning of one problem shape: every variant of its dtype is
// timed as a grouped launch of `batch` copies (CUDA events on the handle's
// stream, one warm-up, `reps` timed launches), per-problem microseconds out.
extern "C" int nrs_tune_gemm(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n,
                             unsigned flags, int64_t batch, int reps, float* times_us, int* best) {
  if (!h || !times_us || m < 1 || k < 1 || n < 1 || batch < 1 || reps < 1) return NRS_ERR_INVALID;
  if (dtype != NRS_F32 && dtype != NRS_F64) return nrs_fail(h, NRS_ERR_DTYPE, "tuning takes f32 or f64");
  if (flags & ~(NRS_GEMM_TRANS_A | NRS_GEMM_TRANS_B)) return nrs_fail(h, NRS_ERR_INVALID, "flags");
  h->last_error.clear();
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;
  const size_t es = nrs_dtype_size(dtype);
  const size_t a_b = (size_t)m * k * es, b_b = (size_t)k * n * es, c_b = (size_t)m * n * es * batch;
  void *A = nullptr, *B = nullptr, *Cm = nullptr;
  cudaError_t e = cudaMalloc(&A, a_b);
  if (!e) e = cudaMalloc(&B, b_b);
  if (!e) e = cudaMalloc(&Cm, c_b);
  if (e) {
    cudaFree(A);
    cudaFree(B);
    cudaFree(Cm);
    cudaGetLastError();
    return nrs_fail(h, NRS_ERR_ALLOC, "tuning buffers");
  }
  nrs_fill_random(h, dtype, NRS_RNG_UNIFORM, 77, (int64_t)(a_b / es), -1.0, 1.0, A);
  nrs_fill_random(h, dtype, NRS_RNG_UNIFORM, 78, (int64_t)(b_b / es), -1.0, 1.0, B);
  std::vector<nrs_gemm_desc> descs((size_t)batch);
  const bool ta = flags & NRS_GEMM_TRANS_A, tb = flags & NRS_GEMM_TRANS_B;
  for (int64_t i = 0; i < batch; ++i)
    descs[i] = nrs_gemm_desc{dtype, flags, m, k, n, A, ta ? m : k, B, tb ? k : n,
                             (uint8_t*)Cm + (size_t)i * m * n * es, n};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best_t = 1e30f;
  int best_v = -1;
  for (int v = 0; v < NRS_TILE_VARIANTS; ++v) {
    times_us[v] = -1.f;
    if (kVariants[v].dtype != dtype) continue;
    nrs_plan* p = nullptr;
    if ((st = plan_build(h, batch, descs.data(), 0, nullptr, v, nullptr, &p)) != NRS_OK) break;
    plan_launch(h, p, h->stream);
    cudaEventRecord(e0, h->stream);
    for (int r = 0; r < reps; ++r) plan_launch(h, p, h->stream);
    cudaEventRecord(e1, h->stream);
    st = nrs_cuda_check(h, cudaEventSynchronize(e1), "tuning run");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    plan_free(p);
    if (st) break;
    times_us[v] = ms * 1000.f / reps / (float)batch;
    if (times_us[v] < best_t) {
      best_t = times_us[v];
      best_v = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(A);
  cudaFree(B);
  cudaFree(Cm);
  if (best) *best = best_v;
  return st;
}

// ---------------------------------------------------------------------------
// Plan-level autotuning
// ---------------------------------------------------------------------------
// Tuning one shape bucket in isolation (nrs_tune_gemm: a launch of copies of
// one problem) misses what decides a mixed launch: which tiles share the
// machine and how the queue balances. nrs_plan_autotune therefore judges
// every candidate by timing the caller's whole group:
//   1. the untuned plan (selector or size heuristic), f64 on DMMA tiles,
//   2. if the caller allows it, the f64 GEMMs on the tensor cores (grouped
//      Ozaki) at each digit width -- 8, 7 or 6 bits, the slice count
//      following from the width at the same accuracy -- kept if faster,
//   3. every remaining bucket tuned in isolation,
//   4. starting from the faster of 1-2 and 3, a greedy pass over the buckets
//      with the most estimated work: each alternative variant is kept only
//      if the whole group gets faster.
// The final choice is never slower than the untuned plan as measured.
namespace {

struct TuneBucket {
  int dtype;
  int64_t m, k, n;  // a member's shape (every member maps to this bucket)
  double work;      // estimated seconds at the pipe's rate
  int64_t count;
};

int time_group(nrs_handle* h, const std::vector<nrs_gemm_desc>& g, int64_t n_red,
               const nrs_rowreduce_desc* reds, int reps, cudaEvent_t e0, cudaEvent_t e1, const nrs_plan_options* opt,
               double* ms) {
  nrs_plan* p = nullptr;
  int st = plan_build(h, (int64_t)g.size(), g.data(), n_red, reds, -1, opt, &p);
  if (st) return st;
  st = plan_launch(h, p, h->stream);  // warm-up
  std::vector<float> ts;
  for (int r = 0; r < reps && st == NRS_OK; ++r) {
    cudaEventRecord(e0, h->stream);
    st = plan_launch(h, p, h->stream);
    cudaEventRecord(e1, h->stream);
    if (st == NRS_OK) st = nrs_cuda_check(h, cudaEventSynchronize(e1), "autotune run");
    float t = 0.f;
    if (st == NRS_OK) cudaEventElapsedTime(&t, e0, e1);
    ts.push_back(t);
  }
  cudaStreamSynchronize(h->stream);
  plan_free(p);
  if (st) return st;
  std::sort(ts.begin(), ts.end());
  *ms = ts[ts.size() / 2];
  return NRS_OK;
}

}  // namespace

extern "C" int nrs_plan_autotune(nrs_handle* h, int64_t n_gemm, const nrs_gemm_desc* gemms, int64_t n_red,
                                 const nrs_rowreduce_desc* reds, const nrs_plan_options* opt, int max_trials,
                                 int reps, nrs_autotune_report* rep) {
  if (!h || n_gemm < 0 || n_red < 0 || (n_gemm && !gemms) || (n_red && !reds) || max_trials < 0 || reps < 1)
    return NRS_ERR_INVALID;
  h->last_error.clear();
  int st = nrs_cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (st) return st;
  // The group runs repeatedly: accumulating GEMMs are tuned as overwriting
  // ones (same tiles, same reads of A and B).
  std::vector<nrs_gemm_desc> g(gemms, gemms + n_gemm);
  for (auto& d : g) d.flags &= ~NRS_GEMM_ACCUMULATE;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto done = [&](int s2) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return s2;
  };
  auto key_of = [](const nrs_gemm_desc& d) {
    auto lg = [](int64_t v) { return (int)std::lround(std::log2((double)(v < 1 ? 1 : v))); };
    return std::make_tuple((int)d.dtype, lg(d.m), lg(d.k), lg(d.n));
  };
  // Buckets of the GEMMs the persistent kernel runs (row-major f64 / f32
  // ones leave it when they go to the tensor cores).
  auto make_buckets = [&](bool skip_f64, bool skip_f32) {
    std::map<std::tuple<int, int, int, int>, TuneBucket> bm;
    for (const auto& d : g) {
      if (d.m == 0 || d.n == 0 || d.k == 0 || (d.dtype != NRS_F32 && d.dtype != NRS_F64)) continue;
      const bool row_major = !(d.flags & (NRS_GEMM_TRANS_A | NRS_GEMM_TRANS_B));
      if (row_major && ((skip_f64 && d.dtype == NRS_F64) || (skip_f32 && d.dtype == NRS_F32))) continue;
      auto& b = bm[key_of(d)];
      if (b.count == 0) b = TuneBucket{d.dtype, d.m, d.k, d.n, 0.0, 0};
      b.work += 2.0 * d.m * d.n * d.k / (d.dtype == NRS_F64 ? 1.1e12 : 70e12);
      b.count++;
    }
    std::vector<TuneBucket> out;
    for (auto& kv : bm) out.push_back(kv.second);
    std::sort(out.begin(), out.end(), [](const TuneBucket& a, const TuneBucket& b) { return a.work > b.work; });
    return out;
  };
  // 1. untuned, f64 on DMMA tiles
  for (const auto& b : make_buckets(false, false)) nrs_tuner_forget(h, b.dtype, b.m, b.k, b.n);
  double t_untuned = 0.0, t_isolated = 0.0;
  if ((st = time_group(h, g, n_red, reds, reps, e0, e1, nullptr, &t_untuned))) return done(st);
  // 2. the f64 mode: DMMA tiles, or the tensor cores at each digit width;
  //    then the f32 GEMMs on the tensor cores on top of the best
  nrs_plan_options best_opt{NRS_PLAN_F64_DMMA, 0, 0, NRS_PLAN_F32_FMA};
  double t_mode = t_untuned, t_oz_best = -1.0, t_oz32 = -1.0;
  if (opt && opt->f64_mode == NRS_PLAN_F64_OZAKI) {
    for (int bits : {0, 7, 6}) {
      if (opt->f64_digit_bits != 0 && bits != 0) continue;  // the caller fixed the width
      nrs_plan_options o{NRS_PLAN_F64_OZAKI, opt->f64_slices, bits ? bits : opt->f64_digit_bits, NRS_PLAN_F32_FMA};
      double t = 0.0;
      if ((st = time_group(h, g, n_red, reds, reps, e0, e1, &o, &t))) return done(st);
      if (t_oz_best < 0 || t < t_oz_best) t_oz_best = t;
      if (t < t_mode) {
        t_mode = t;
        best_opt = o;
      }
    }
  }
  if (opt && opt->f32_mode == NRS_PLAN_F32_OZAKI) {
    nrs_plan_options o = best_opt;
    o.f32_mode = NRS_PLAN_F32_OZAKI;
    if ((st = time_group(h, g, n_red, reds, reps, e0, e1, &o, &t_oz32))) return done(st);
    if (t_oz32 < t_mode) {
      t_mode = t_oz32;
      best_opt = o;
    }
  }
  const std::vector<TuneBucket> buckets =
      make_buckets(best_opt.f64_mode == NRS_PLAN_F64_OZAKI, best_opt.f32_mode == NRS_PLAN_F32_OZAKI);
  // 3. every bucket tuned in isolation
  std::vector<int> untuned(buckets.size()), isolated(buckets.size());
  for (size_t i = 0; i < buckets.size(); ++i) {
    const auto& b = buckets[i];
    untuned[i] = heuristic_variant(b.dtype, b.m, b.k, b.n);
    float times[NRS_TILE_VARIANTS];
    int best = -1;
    if ((st = nrs_tune_gemm(h, b.dtype, b.m, b.k, b.n, 0, b.count < 64 ? b.count : 64, 2, times, &best)))
      return done(st);
    isolated[i] = best;
    nrs_tuner_set(h, b.dtype, b.m, b.k, b.n, best);
  }
  if ((st = time_group(h, g, n_red, reds, reps, e0, e1, &best_opt, &t_isolated))) return done(st);
  // 4. greedy refinement from the faster start
  std::vector<int> cur = isolated;
  double t_best = t_isolated;
  if (t_mode < t_isolated) {
    cur = untuned;
    for (size_t i = 0; i < buckets.size(); ++i)
      nrs_tuner_set(h, buckets[i].dtype, buckets[i].m, buckets[i].k, buckets[i].n, cur[i]);
    if ((st = time_group(h, g, n_red, reds, reps, e0, e1, &best_opt, &t_best))) return done(st);
    if (t_best > t_mode) {
      // the representative shapes' variants lost to the per-problem untuned
      // choices: keep those (no table entries) as the starting point
      for (const auto& b : buckets) nrs_tuner_forget(h, b.dtype, b.m, b.k, b.n);
      std::fill(cur.begin(), cur.end(), -1);
      t_best = t_mode;
    }
  }
  int trials = 0;
  for (size_t i = 0; i < buckets.size() && trials < max_trials; ++i) {
    const auto& b = buckets[i];
    for (int v = 0; v < NRS_TILE_VARIANTS && trials < max_trials; ++v) {
      if (kVariants[v].dtype != b.dtype || v == cur[i]) continue;
      nrs_tuner_set(h, b.dtype, b.m, b.k, b.n, v);
      double t = 0.0;
      if ((st = time_group(h, g, n_red, reds, reps, e0, e1, &best_opt, &t))) return done(st);
      ++trials;
      if (t < t_best * 0.997) {
        t_best = t;
        cur[i] = v;
      }
    }
    if (cur[i] >= 0) nrs_tuner_set(h, b.dtype, b.m, b.k, b.n, cur[i]);
    else nrs_tuner_forget(h, b.dtype, b.m, b.k, b.n);
  }
  if (rep) {
    rep->untuned_ms = t_untuned;
    rep->isolated_ms = t_isolated;
    rep->final_ms = t_best;
    rep->ozaki_ms = t_oz_best;
    rep->buckets = (int32_t)buckets.size();
    rep->trials = trials;
    rep->options = best_opt;
    rep->ozaki_f32_ms = t_oz32;
  }
  return done(NRS_OK);
}
