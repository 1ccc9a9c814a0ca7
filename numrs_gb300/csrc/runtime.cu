// Handle, stream, workspace, memory and input-generator entry points.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "nrs_internal.cuh"

extern "C" int nrs_abi_version(void) { return NRS_ABI_VERSION; }

extern "C" const char* nrs_status_string(int s) {
  switch (s) {
    case NRS_OK: return "ok";
    case NRS_ERR_INVALID: return "invalid argument";
    case NRS_ERR_SHAPE: return "shape mismatch";
    case NRS_ERR_DTYPE: return "unsupported dtype for this operation";
    case NRS_ERR_AXIS: return "axis out of bounds";
    case NRS_ERR_EMPTY: return "operation on an empty array";
    case NRS_ERR_STRIDE: return "invalid stride";
    case NRS_ERR_CUDA: return "CUDA error";
    case NRS_ERR_TIMEOUT: return "device-side wait timed out";
    case NRS_ERR_ALLOC: return "allocation failed";
    case NRS_ERR_UNSUPPORTED: return "unsupported";
    case NRS_ERR_TOO_LARGE: return "size beyond the supported maximum";
    case NRS_ERR_IO: return "file I/O error";
    default: return "unknown status";
  }
}

int nrs_fail(nrs_handle* h, int status, const std::string& msg) {
  if (h) h->last_error = msg;
  return status;
}

int nrs_cuda_check(nrs_handle* h, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return NRS_OK;
  return nrs_fail(h, NRS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int nrs_after_launch(nrs_handle* h, const char* what) {
  return nrs_cuda_check(h, cudaGetLastError(), what);
}

size_t nrs_dtype_size(int dtype) {
  switch (dtype) {
    case NRS_F32: return 4;
    case NRS_F64: return 8;
    case NRS_I32: return 4;
    case NRS_I64: return 8;
    default: return 0;
  }
}

void* nrs_workspace(nrs_handle* h, size_t bytes, int* status) {
  *status = NRS_OK;
  if (bytes <= h->workspace_bytes) return h->workspace;
  size_t want = bytes < (1u << 20) ? (1u << 20) : bytes;
  want = (want + 255) & ~size_t(255);
  if (h->workspace) {
    // The old workspace may still be read by queued work on this stream.
    cudaStreamSynchronize(h->stream);
    cudaFree(h->workspace);
    h->workspace = nullptr;
    h->workspace_bytes = 0;
  }
  if (cudaMalloc(&h->workspace, want) != cudaSuccess) {
    cudaGetLastError();
    *status = nrs_fail(h, NRS_ERR_ALLOC, "workspace cudaMalloc failed");
    return nullptr;
  }
  h->workspace_bytes = want;
  return h->workspace;
}

nrs_encode_tiled_fn nrs_get_encode_tiled() {
  static nrs_encode_tiled_fn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<nrs_encode_tiled_fn>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

extern "C" int nrs_create(int device, nrs_handle** out) {
  if (!out) return NRS_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return NRS_ERR_CUDA;
  }
  nrs_handle* h = new nrs_handle();
  h->device = device;
  int st = nrs_cuda_check(h, cudaSetDevice(device), "cudaSetDevice");
  if (st == NRS_OK)
    st = nrs_cuda_check(h, cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device),
                        "cudaDeviceGetAttribute");
  if (st == NRS_OK)
    st = nrs_cuda_check(h, cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking),
                        "cudaStreamCreate");
  if (st == NRS_OK)
    st = nrs_cuda_check(h, cudaMalloc(&h->dev_error, 256), "cudaMalloc(error word)");
  if (st == NRS_OK) st = nrs_cuda_check(h, cudaMemset(h->dev_error, 0, 256), "cudaMemset");
  if (st != NRS_OK) {
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    if (h->dev_error) cudaFree(h->dev_error);
    delete h;
    return st;
  }
  h->hw_sms = h->num_sms;
  h->stream = h->own_stream;
  *out = h;
  return NRS_OK;
}

extern "C" int nrs_set_sm_budget(nrs_handle* h, int sms) {
  if (!h || sms < 0) return NRS_ERR_INVALID;
  h->num_sms = (sms == 0 || sms > h->hw_sms) ? h->hw_sms : sms;
  return NRS_OK;
}

void nrs_tuner_free(nrs_handle* h);

extern "C" int nrs_destroy(nrs_handle* h) {
  if (!h) return NRS_ERR_INVALID;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  if (h->workspace) cudaFree(h->workspace);
  if (h->dev_error) cudaFree(h->dev_error);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  nrs_tuner_free(h);
  nrs_stage_free(h);
  delete h;
  return NRS_OK;
}

extern "C" int nrs_set_stream(nrs_handle* h, void* s) {
  if (!h) return NRS_ERR_INVALID;
  // NULL is CUDA's default stream (the one a framework's "current stream"
  // usually is), not the handle's own stream.
  h->stream = static_cast<cudaStream_t>(s);
  return NRS_OK;
}

extern "C" int nrs_use_own_stream(nrs_handle* h) {
  if (!h) return NRS_ERR_INVALID;
  h->stream = h->own_stream;
  return NRS_OK;
}

extern "C" void* nrs_get_stream(nrs_handle* h) { return h ? (void*)h->stream : nullptr; }

extern "C" int nrs_synchronize(nrs_handle* h) {
  if (!h) return NRS_ERR_INVALID;
  int st = nrs_cuda_check(h, cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
  if (st != NRS_OK) return st;
  uint32_t word = 0;
  st = nrs_cuda_check(h, cudaMemcpy(&word, h->dev_error, sizeof(word), cudaMemcpyDeviceToHost),
                      "cudaMemcpy(error word)");
  if (st != NRS_OK) return st;
  if (word != 0) {
    cudaMemset(h->dev_error, 0, sizeof(uint32_t));
    char buf[96];
    snprintf(buf, sizeof buf, "device-side bounded wait gave up (site 0x%08x)", word);
    return nrs_fail(h, NRS_ERR_TIMEOUT, buf);
  }
  return NRS_OK;
}

extern "C" int nrs_test_expire_next_wait(nrs_handle* h, uint32_t probes) {
  if (!h || probes == 0) return NRS_ERR_INVALID;
  // Word 1 of the error block is read (and cleared) by the next column-fold
  // launch on this handle's stream.
  return nrs_cuda_check(h, cudaMemcpyAsync(h->dev_error + 1, &probes, sizeof(probes),
                                           cudaMemcpyHostToDevice, h->stream),
                        "cudaMemcpyAsync(test hook)") ||
         nrs_cuda_check(h, cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
}

extern "C" const char* nrs_last_error(nrs_handle* h) { return h ? h->last_error.c_str() : ""; }

extern "C" int nrs_malloc(nrs_handle* h, size_t bytes, void** p) {
  if (!h || !p) return NRS_ERR_INVALID;
  *p = nullptr;
  if (bytes == 0) return NRS_OK;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return nrs_fail(h, NRS_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  return NRS_OK;
}

extern "C" int nrs_free(nrs_handle* h, void* p) {
  if (!h) return NRS_ERR_INVALID;
  if (!p) return NRS_OK;
  return nrs_cuda_check(h, cudaFree(p), "cudaFree");
}

extern "C" int nrs_host_alloc(nrs_handle* h, size_t bytes, void** p) {
  if (!h || !p) return NRS_ERR_INVALID;
  *p = nullptr;
  if (bytes == 0) return NRS_OK;
  cudaError_t e = cudaMallocHost(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return nrs_fail(h, NRS_ERR_ALLOC, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
  }
  return NRS_OK;
}

extern "C" int nrs_host_free(nrs_handle* h, void* p) {
  if (!h) return NRS_ERR_INVALID;
  if (!p) return NRS_OK;
  return nrs_cuda_check(h, cudaFreeHost(p), "cudaFreeHost");
}

extern "C" int nrs_memcpy_h2d(nrs_handle* h, void* dst, const void* src, size_t bytes) {
  if (!h || (bytes && (!dst || !src))) return NRS_ERR_INVALID;
  if (!bytes) return NRS_OK;
  return nrs_cuda_check(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream),
                        "cudaMemcpyAsync(H2D)");
}

extern "C" int nrs_memcpy_d2h(nrs_handle* h, void* dst, const void* src, size_t bytes) {
  if (!h || (bytes && (!dst || !src))) return NRS_ERR_INVALID;
  if (!bytes) return NRS_OK;
  return nrs_cuda_check(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream),
                        "cudaMemcpyAsync(D2H)");
}

// ---------------------------------------------------------------------------
// SplitMix64 input generator
// ---------------------------------------------------------------------------
namespace {
constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ULL;

__device__ __forceinline__ uint64_t sm64_at(uint64_t seed, uint64_t i) {
  uint64_t z = (seed ^ kGamma) + (i + 1) * kGamma;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double u01(uint64_t x) {
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

// Standard normal from draws (2i, 2i+1): Box-Muller, cosine branch.
__device__ __forceinline__ double normal_at(uint64_t seed, uint64_t i) {
  double u1 = 1.0 - u01(sm64_at(seed, 2 * i));  // (0, 1]
  double u2 = u01(sm64_at(seed, 2 * i + 1));
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

template <typename T>
__global__ void fill_kernel(T* out, int64_t n, int dist, uint64_t seed, double p0, double p1,
                            int shift) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v;
    if (dist == NRS_RNG_UNIFORM) {
      v = p0 + (p1 - p0) * u01(sm64_at(seed, i));
      out[i] = (T)v;
    } else if (dist == NRS_RNG_NORMAL) {
      v = p0 + p1 * normal_at(seed, i);
      out[i] = (T)v;
    } else if (dist == NRS_RNG_OZAKI) {
      double u = u01(sm64_at(seed, 3 * i)) - 0.5;
      double u1 = 1.0 - u01(sm64_at(seed, 3 * i + 1));
      double u2 = u01(sm64_at(seed, 3 * i + 2));
      double z = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
      out[i] = (T)(u * exp(p0 * z));
    } else {
      out[i] = (T)((int64_t)(sm64_at(seed, i) >> shift) + (int64_t)p0);
    }
  }
}
}  // namespace

extern "C" int nrs_fill_random(nrs_handle* h, int dtype, int dist, uint64_t seed, int64_t n,
                               double p0, double p1, void* out) {
  if (!h || n < 0 || (n && !out)) return NRS_ERR_INVALID;
  if (n == 0) return NRS_OK;
  int grid = h->num_sms * 8;
  int shift = 0;
  if (dist == NRS_RNG_INT) {
    // p1 = range width, a power of two: (x >> (64 - log2 p1)) + p0.
    if (!(p1 >= 2.0) || p1 > 9.223372036854775807e18) return NRS_ERR_INVALID;
    int b = 0;
    while ((double)(1ULL << (b + 1)) <= p1 && b < 62) ++b;
    shift = 64 - b;
    if (dtype == NRS_I64)
      fill_kernel<int64_t><<<grid, 256, 0, h->stream>>>((int64_t*)out, n, dist, seed, p0, p1, shift);
    else if (dtype == NRS_I32)
      fill_kernel<int32_t><<<grid, 256, 0, h->stream>>>((int32_t*)out, n, dist, seed, p0, p1, shift);
    else
      return NRS_ERR_DTYPE;
  } else if (dist == NRS_RNG_UNIFORM || dist == NRS_RNG_NORMAL || dist == NRS_RNG_OZAKI) {
    if (dtype == NRS_F32)
      fill_kernel<float><<<grid, 256, 0, h->stream>>>((float*)out, n, dist, seed, p0, p1, 0);
    else if (dtype == NRS_F64)
      fill_kernel<double><<<grid, 256, 0, h->stream>>>((double*)out, n, dist, seed, p0, p1, 0);
    else
      return NRS_ERR_DTYPE;
  } else {
    return NRS_ERR_INVALID;
  }
  return nrs_after_launch(h, "fill_kernel");
}
