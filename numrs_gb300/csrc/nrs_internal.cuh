// Internal definitions shared by the CUDA translation units of libnumrs_gb300.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/numrs_gpu.h"

// ---------------------------------------------------------------------------
// Handle
// ---------------------------------------------------------------------------
// Device-side error word layout: the low byte names the kernel family whose
// bounded wait gave up, the rest is a site code. 0 = no error.
enum : uint32_t {
  NRS_DEVERR_NONE = 0,
  NRS_DEVERR_REDUCE_TMA = 0x01,
  NRS_DEVERR_GEMM_TC = 0x02,
  NRS_DEVERR_GROUPED = 0x03,
};

struct nrs_tuner_table;
struct nrs_host_stage;  // pinned staging slots for file I/O (npy.cu)

// SM count that every result-affecting plan is computed for (a GEMM's k
// split, a flattened scan's segments): GB300's 152. Grids are sized from
// the handle's num_sms, plans from this constant, so results do not depend
// on the device or on the handle's SM budget.
constexpr int NRS_PLAN_SMS = 152;

struct nrs_handle {
  int device = 0;
  int num_sms = 0;   // SMs grids are sized for (the budget, nrs_set_sm_budget)
  int hw_sms = 0;    // the device's SM count
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // Grow-only device workspace for kernels that need scratch memory.
  void* workspace = nullptr;
  size_t workspace_bytes = 0;
  // Device error word written by kernels whose waits are bounded.
  uint32_t* dev_error = nullptr;
  std::string last_error;
  nrs_tuner_table* tuner = nullptr;
  // Learned selector consulted for shapes the tuner table lacks (not owned).
  nrs_selector* selector = nullptr;
  // Pinned staging for NPY reads/writes, allocated on first use.
  nrs_host_stage* stage = nullptr;
};

// ---------------------------------------------------------------------------
// Helpers (runtime.cu)
// ---------------------------------------------------------------------------
int nrs_fail(nrs_handle* h, int status, const std::string& msg);
int nrs_cuda_check(nrs_handle* h, cudaError_t e, const char* what);
// Ensures the workspace holds at least `bytes`; returns its pointer or null.
void* nrs_workspace(nrs_handle* h, size_t bytes, int* status);
size_t nrs_dtype_size(int dtype);
// Checks launch errors right after a launch.
int nrs_after_launch(nrs_handle* h, const char* what);
// Frees the handle's pinned staging slots (npy.cu).
void nrs_stage_free(nrs_handle* h);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda).
typedef CUresult (*nrs_encode_tiled_fn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                        const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                        const cuuint32_t*, CUtensorMapInterleave,
                                        CUtensorMapSwizzle, CUtensorMapL2promotion,
                                        CUtensorMapFloatOOBfill);
nrs_encode_tiled_fn nrs_get_encode_tiled();

// Grouped Ozaki (ozaki.cu): the tensor-core form of many f64 (or f32)
// GEMMs. build decides which problems of element type `dtype` it takes
// (accepted[i] = 1: row-major operands and a spread the slice count covers)
// and allocates every buffer; launch enqueues the whole group without host
// synchronisation.
struct nrs_ozaki_group;
int nrs_ozaki_group_build(nrs_handle* h, int64_t count, const nrs_gemm_desc* descs, int dtype, int slices,
                          int digit_bits, int* accepted, nrs_ozaki_group** out);
int nrs_ozaki_group_launch(nrs_handle* h, nrs_ozaki_group* g, cudaStream_t s);
int nrs_ozaki_group_info(const nrs_ozaki_group* g, int* slices, int* bits, int64_t* tiles);
void nrs_ozaki_group_free(nrs_ozaki_group* g);
// Network shape of a selector (selector.cu).
int nrs_selector_shape(nrs_selector* s, int* F, int* H, int* V);
// Removes a shape bucket's entry from the tuner table (tuner.cu).
void nrs_tuner_forget(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n);

// Host-side entry points of the other translation units.
int nrs_plain_gemm_launch(nrs_handle* h, int dtype, int64_t m, int64_t k, int64_t n,
                          const void* A, int64_t rsa, int64_t csa, const void* B, int64_t rsb,
                          int64_t csb, void* C, int64_t ldc, bool accumulate, int variant);

// ---------------------------------------------------------------------------
// Device helpers: mbarrier and TMA (inline PTX, sm_90+ forms valid on sm_103a)
// ---------------------------------------------------------------------------
#define NRS_DEV __device__ __forceinline__

// 16-byte moves between a shared-memory tile and registers, as one vector
// access (a byte-pointer memcpy may be split into narrow loads). Callers'
// tile addresses are 16-byte aligned by construction.
template <typename T>
NRS_DEV void lds16(T* dst, const uint8_t* src) {
  const uint4 q = *reinterpret_cast<const uint4*>(src);
  memcpy(dst, &q, 16);
}
template <typename T>
NRS_DEV void sts16(uint8_t* dst, const T* src) {
  uint4 q;
  memcpy(&q, src, 16);
  *reinterpret_cast<uint4*>(dst) = q;
}

NRS_DEV uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

NRS_DEV void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

NRS_DEV void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

NRS_DEV void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

NRS_DEV void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

NRS_DEV void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// One try_wait probe on `phase`; true once the phase has completed.
NRS_DEV bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Bounded wait: gives up after `limit` probes (each probe itself may suspend
// the thread for a hardware-defined time). Returns false on give-up.
NRS_DEV bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}

NRS_DEV void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int32_t x, int32_t y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

NRS_DEV void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int32_t x, int32_t y,
                         int32_t z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

// Tiled TMA store (shared -> global) of one box at (x, y, z); elements
// outside the tensor are not written. Tracked by the issuing thread's bulk
// async-groups: commit, then wait (reads of shared memory done / complete).
NRS_DEV void tma_store_3d(const CUtensorMap* map, const void* src, int32_t x, int32_t y, int32_t z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
      : "memory");
}
// Untiled bulk copies (no tensor map): both addresses 16-byte aligned and
// `bytes` a multiple of 16. The load signals `bar` with complete_tx; the store
// joins the issuing thread's bulk async-group like tma_store_3d.
NRS_DEV void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
NRS_DEV void bulk_store(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(
                   reinterpret_cast<uint64_t>(dst)),
               "r"(smem_u32(src)), "r"(bytes)
               : "memory");
}
NRS_DEV void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int N>
NRS_DEV void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
template <int N>
NRS_DEV void bulk_wait() {
  asm volatile("cp.async.bulk.wait_group %0;" ::"n"(N) : "memory");
}

NRS_DEV void prefetch_tensormap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Bounded-wait budget: ~2^22 probes is several seconds of a stalled copy,
// far beyond any legitimate wait.
#define NRS_WAIT_LIMIT (1u << 22)
