// Bulk asynchronous copies (cp.async.bulk, the TMA's untiled form) into
// shared memory, completed on mbarriers, with bounded waits; and the tile
// ring the streaming vector kernels use.
//
// Every wait polls a bounded number of times: on expiry the kernel's error
// flag is set and the caller drains the copies it still has in flight
// (again bounded) before it leaves, so a CTA never exits under a copy.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace pg {
namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// 16-byte aligned addresses, size a multiple of 16
__device__ __forceinline__ void bulk_load(void *dst, const void *src,
                                          uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], "
      "%2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
constexpr int kWaitLimit = 1 << 22;  // try_wait polls before giving up

// Bounded wait on the phase `parity` of a barrier.  On expiry the error
// flag is set and the copy still in flight is waited for once more
// (bounded) so the CTA does not exit under it.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, int *err,
                                                  uint32_t parity = 0) {
  for (int it = 0; it < kWaitLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  if (err) atomicExch(err, 1);
  for (int it = 0; it < kWaitLimit; ++it)
    if (mbar_try_wait(bar, parity)) break;
  return false;
}
// orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (bulk copy) writes to the same memory
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ int al16(int b) { return (b + 15) & ~15; }

// ---- streamed tiles of the Krylov vector kernels ----
// A CTA of kTileN threads owns the tiles blockIdx.x + k * gridDim.x
// (k = 0, 1, ...) and keeps up to S of them in flight in a ring of stages
// (tile k in stage k % S, completed on that stage's mbarrier in phase
// (k / S) & 1); thread 0 issues the bulk copies, every thread waits, a
// block barrier frees a stage before it is refilled.  Thread t handles
// element (row) t of each tile, so each thread's sums run in a fixed order.
constexpr int kTileN = 256;

// elements of tile j (of 8-byte elements) that the bulk copies move: the
// tile's elements below n rounded down to even, a 16-byte multiple; a
// thread whose element lies past that count reads global memory
__device__ __forceinline__ int tile_bulk_count(int n, int j) {
  const int rem = n - j * kTileN;
  return (rem < kTileN ? rem : kTileN) & ~1;
}

// tile j of NV vectors of 8-byte elements into stg (vector q at
// q * kTileN * 8 bytes); the vectors are 16-byte aligned
template <int NV>
__device__ __forceinline__ void issue_vec_tile(uint8_t *stg,
                                               const void *const (&src)[NV],
                                               int n, int j, uint64_t *bar) {
  const int cnt = tile_bulk_count(n, j);
  const uint32_t bytes = (uint32_t)cnt * 8u;
  mbar_expect_tx(bar, NV * bytes);
  if (bytes)
#pragma unroll
    for (int q = 0; q < NV; ++q)
      bulk_load(stg + q * kTileN * 8,
                static_cast<const uint8_t *>(src[q]) + (size_t)j * kTileN * 8,
                bytes, bar);
}

// Stage of a sliced-ELLPACK tile (the 8 slices of 32 rows of tile j, at
// most W entries per row): the slices' 8-byte values, their int32 columns,
// then NV 8-byte vector tiles.
__host__ __device__ constexpr size_t sell_stage_bytes(int W, int NV) {
  return (size_t)kTileN * W * 12 + (size_t)NV * kTileN * 8;
}
// entries [a, b) of the sliced arrays are tile j's (a, b multiples of 32,
// so both copies are 16-byte multiples from 16-byte aligned addresses)
template <int NV>
__device__ __forceinline__ void issue_sell_tile(uint8_t *stg, int W,
                                                const void *vals,
                                                const int32_t *cols, int a,
                                                int b,
                                                const void *const (&src)[NV],
                                                int n, int j, uint64_t *bar) {
  const uint32_t ent = (uint32_t)(b - a);
  const int cnt = tile_bulk_count(n, j);
  const uint32_t vbytes = (uint32_t)cnt * 8u;
  mbar_expect_tx(bar, ent * 12u + NV * vbytes);
  if (ent) {
    bulk_load(stg, static_cast<const uint8_t *>(vals) + (size_t)a * 8, ent * 8u, bar);
    bulk_load(stg + (size_t)kTileN * W * 8, cols + a, ent * 4u, bar);
  }
  if (vbytes)
#pragma unroll
    for (int q = 0; q < NV; ++q)
      bulk_load(stg + (size_t)kTileN * W * 12 + q * kTileN * 8,
                static_cast<const uint8_t *>(src[q]) + (size_t)j * kTileN * 8,
                vbytes, bar);
}

}  // namespace

// CTAs of a streamed-tile kernel: as many as fit on the device at once
// (persistent), at most the tiles and the reduction workspace's grid
inline int stream_grid(const void *kern, size_t smem, int n_tiles, int cap) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTileN, smem);
  int g = per_sm * sms;
  if (g > n_tiles) g = n_tiles;
  if (g > cap) g = cap;
  return g < 1 ? 1 : g;
}
inline bool aligned16(const void *p) {
  return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

}  // namespace pg
