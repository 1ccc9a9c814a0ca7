// Autotuner table: shape bucket -> tile variant of the grouped kernel.
//
// Buckets are (dtype, round(log2 m), round(log2 k), round(log2 n)) so one
// tuned shape covers its neighbours within a factor of sqrt(2). The table is
// filled by nrs_tune_gemm / nrs_tuner_set and read by nrs_plan_create.
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include <tuple>
#include <vector>

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

void nrs_tuner_forget(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n) {
  if (h && h->tuner) h->tuner->best.erase(bucket(dtype, m, k, n));
}

extern "C" int nrs_tuner_clear(nrs_handle* h) {
  if (!h) return NRS_ERR_INVALID;
  if (h->tuner) h->tuner->best.clear();
  return NRS_OK;
}

// ---------------------------------------------------------------------------
// Persistence: tuned tables and selector weights are valid for one GPU model,
// driver and build of this library; files carry that key and are refused
// when any part differs.
// ---------------------------------------------------------------------------
#ifndef NRS_SOURCE_HASH
#define NRS_SOURCE_HASH "unknown"
#endif

namespace {

struct DeviceKey {
  std::string gpu;
  int driver = 0;
  std::string source = NRS_SOURCE_HASH;
};

int device_key(nrs_handle* h, DeviceKey* k) {
  cudaDeviceProp prop;
  int st = nrs_cuda_check(h, cudaGetDeviceProperties(&prop, h->device), "cudaGetDeviceProperties");
  if (st) return st;
  k->gpu = prop.name;
  for (auto& c : k->gpu)
    if (c == ' ' || c == '\t' || c == '\n') c = '_';
  return nrs_cuda_check(h, cudaDriverGetVersion(&k->driver), "cudaDriverGetVersion");
}

void write_key(FILE* f, const char* kind, int version, const DeviceKey& k) {
  std::fprintf(f, "numrs_gb300-%s %d\ngpu %s\ndriver %d\nsource %s\n", kind, version, k.gpu.c_str(),
               k.driver, k.source.c_str());
}

// Reads and checks the header; NRS_OK when it names this device/driver/build.
int read_key(nrs_handle* h, FILE* f, const char* kind, int version) {
  DeviceKey want;
  int st = device_key(h, &want);
  if (st) return st;
  char k1[64], gpu[256], src[128];
  int ver = 0, drv = 0;
  if (std::fscanf(f, "%63s %d gpu %255s driver %d source %127s", k1, &ver, gpu, &drv, src) != 5)
    return nrs_fail(h, NRS_ERR_IO, "not a numrs_gb300 file");
  if (std::string(k1) != std::string("numrs_gb300-") + kind || ver != version)
    return nrs_fail(h, NRS_ERR_UNSUPPORTED, std::string("not a version-") + std::to_string(version) + " " + kind + " file");
  if (want.gpu != gpu || want.driver != drv || want.source != src)
    return nrs_fail(h, NRS_ERR_UNSUPPORTED,
                    std::string("file was made for ") + gpu + " / driver " + std::to_string(drv) + " / build " + src +
                        "; this is " + want.gpu + " / driver " + std::to_string(want.driver) + " / build " + want.source);
  return NRS_OK;
}

}  // namespace

extern "C" int nrs_tuner_save(nrs_handle* h, const char* path) {
  if (!h || !path) return NRS_ERR_INVALID;
  h->last_error.clear();
  DeviceKey k;
  int st = device_key(h, &k);
  if (st) return st;
  FILE* f = std::fopen(path, "w");
  if (!f) return nrs_fail(h, NRS_ERR_IO, std::string("cannot write ") + path);
  write_key(f, "tuner", 1, k);
  const size_t n = h->tuner ? h->tuner->best.size() : 0;
  std::fprintf(f, "entries %zu\n", n);
  if (h->tuner)
    for (const auto& kv : h->tuner->best)
      std::fprintf(f, "%d %d %d %d %d\n", std::get<0>(kv.first), std::get<1>(kv.first), std::get<2>(kv.first),
                   std::get<3>(kv.first), kv.second);
  const bool ok = std::fclose(f) == 0;
  return ok ? NRS_OK : nrs_fail(h, NRS_ERR_IO, std::string("cannot write ") + path);
}

extern "C" int nrs_tuner_load(nrs_handle* h, const char* path) {
  if (!h || !path) return NRS_ERR_INVALID;
  h->last_error.clear();
  FILE* f = std::fopen(path, "r");
  if (!f) return nrs_fail(h, NRS_ERR_IO, std::string("cannot read ") + path);
  int st = read_key(h, f, "tuner", 1);
  size_t n = 0;
  if (st == NRS_OK && std::fscanf(f, " entries %zu", &n) != 1) st = nrs_fail(h, NRS_ERR_IO, "bad tuner file");
  std::vector<std::pair<std::tuple<int, int, int, int>, int>> rows;
  for (size_t i = 0; st == NRS_OK && i < n; ++i) {
    int d, a, b, c, v;
    if (std::fscanf(f, "%d %d %d %d %d", &d, &a, &b, &c, &v) != 5 || v < 0 || v >= NRS_TILE_VARIANTS)
      st = nrs_fail(h, NRS_ERR_IO, "bad tuner file entry");
    else
      rows.push_back({std::make_tuple(d, a, b, c), v});
  }
  std::fclose(f);
  if (st) return st;  // nothing is changed by a refused or broken file
  if (!h->tuner) h->tuner = new nrs_tuner_table();
  for (const auto& r : rows) h->tuner->best[r.first] = r.second;
  return NRS_OK;
}

extern "C" int nrs_selector_save(nrs_handle* h, nrs_selector* s, const char* path) {
  if (!h || !s || !path) return NRS_ERR_INVALID;
  h->last_error.clear();
  const int64_t np = nrs_selector_num_params(s);
  int F = 0, H = 0, V = 0;
  int st = nrs_selector_shape(s, &F, &H, &V);
  if (st) return st;
  std::vector<float> p((size_t)np);
  if ((st = nrs_selector_get_params(h, s, p.data()))) return st;
  DeviceKey k;
  if ((st = device_key(h, &k))) return st;
  FILE* f = std::fopen(path, "wb");
  if (!f) return nrs_fail(h, NRS_ERR_IO, std::string("cannot write ") + path);
  write_key(f, "selector", 1, k);
  std::fprintf(f, "shape %d %d %d params %lld\n", F, H, V, (long long)np);
  const bool ok = std::fwrite(p.data(), sizeof(float), p.size(), f) == p.size();
  return (std::fclose(f) == 0 && ok) ? NRS_OK : nrs_fail(h, NRS_ERR_IO, std::string("cannot write ") + path);
}

extern "C" int nrs_selector_load(nrs_handle* h, nrs_selector* s, const char* path) {
  if (!h || !s || !path) return NRS_ERR_INVALID;
  h->last_error.clear();
  FILE* f = std::fopen(path, "rb");
  if (!f) return nrs_fail(h, NRS_ERR_IO, std::string("cannot read ") + path);
  int st = read_key(h, f, "selector", 1);
  int F = 0, H = 0, V = 0, f2 = 0, h2 = 0, v2 = 0;
  long long np = 0;
  if (st == NRS_OK && (std::fscanf(f, " shape %d %d %d params %lld", &F, &H, &V, &np) != 4 || std::fgetc(f) != '\n'))
    st = nrs_fail(h, NRS_ERR_IO, "bad selector file");
  if (st == NRS_OK && ((st = nrs_selector_shape(s, &f2, &h2, &v2)) == NRS_OK) &&
      (F != f2 || H != h2 || V != v2 || np != nrs_selector_num_params(s)))
    st = nrs_fail(h, NRS_ERR_SHAPE, "selector file has another network shape");
  std::vector<float> p(st == NRS_OK ? (size_t)np : 0);
  if (st == NRS_OK && std::fread(p.data(), sizeof(float), p.size(), f) != p.size())
    st = nrs_fail(h, NRS_ERR_IO, "selector file is truncated");
  std::fclose(f);
  if (st) return st;
  return nrs_selector_set_params(h, s, p.data());
}
