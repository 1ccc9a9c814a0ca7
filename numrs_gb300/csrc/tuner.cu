// Autotuner table: shape bucket -> tile variant of the grouped kernel.
//
// Buckets are (dtype, round(log2 m), round(log2 k), round(log2 n)) so one
// tuned shape covers its neighbours within a factor of sqrt(2). The table is
// filled by nrs_tune_gemm / nrs_tuner_set and read by nrs_plan_create.
#include <cmath>
#include <map>
#include <tuple>

#include "nrs_internal.cuh"

struct nrs_tuner_table {
  std::map<std::tuple<int, int, int, int>, int> best;
};

static std::tuple<int, int, int, int> bucket(int dtype, int64_t m, int64_t k, int64_t n) {
  auto lg = [](int64_t v) { return (int)std::lround(std::log2((double)(v < 1 ? 1 : v))); };
  return {dtype, lg(m), lg(k), lg(n)};
}

void nrs_tuner_free(nrs_handle* h) {
  delete h->tuner;
  h->tuner = nullptr;
}

extern "C" int nrs_tuner_set(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n, int variant) {
  if (!h || variant < 0 || variant >= NRS_TILE_VARIANTS) return NRS_ERR_INVALID;
  if (!h->tuner) h->tuner = new nrs_tuner_table();
  h->tuner->best[bucket(dtype, m, k, n)] = variant;
  return NRS_OK;
}

extern "C" int nrs_tuner_get(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n) {
  if (!h || !h->tuner) return -1;
  auto it = h->tuner->best.find(bucket(dtype, m, k, n));
  return it == h->tuner->best.end() ? -1 : it->second;
}

extern "C" int nrs_tuner_clear(nrs_handle* h) {
  if (!h) return NRS_ERR_INVALID;
  if (h->tuner) h->tuner->best.clear();
  return NRS_OK;
}
