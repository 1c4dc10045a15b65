// szp_pipe.cuh -- pieces shared by the persistent, warp-specialised kernels.
//
// A CTA of such a kernel runs until the tile tickets run out: a producer
// thread draws tickets and fills shared-memory slots by bulk copy, 8 compute
// warps (256 threads, named barrier 1) work on the slots in order, and
// control warps finish each tile once the decoupled look-back has given its
// prefix.  Slots are handed between the roles with mbarriers; every wait is
// bounded and, on timeout, flags the launch instead of hanging.
#pragma once
#include "szp_device.cuh"
#include "szp_tma.cuh"

namespace szp {

constexpr uint32_t kStopTile = 0xFFFFFFFFu;  // slot marker: no more tiles for this CTA
constexpr uint32_t kWaitLimit = 1u << 24;    // mbarrier polls before a wait gives up

// Barrier over the 256 compute threads (warps 0-7) only.
__device__ __forceinline__ void compute_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// Waits for an mbarrier phase; on timeout flags the launch and waits once more.
__device__ __forceinline__ void mbar_wait_or_flag(uint64_t* bar, uint32_t parity, uint32_t* err) {
  if (!mbar_wait_bounded(bar, parity, kWaitLimit)) {
    atomicOr(err, kErrLookbackTimeout);
    mbar_wait_bounded(bar, parity, kWaitLimit);
  }
}

// A control warp's wait for slot phase `parity` of its k-th tile, or for the
// producer's stop at an earlier or equal k; true when the slot is full.
__device__ __forceinline__ bool control_wait_full(uint64_t* full, uint32_t parity, uint32_t k,
                                                  const volatile uint32_t* s_stop_k, uint32_t* err) {
  bool got = false;
  for (uint32_t i = 0; i < kWaitLimit; i++) {
    if ((got = mbar_try_wait(full, parity))) break;
    if (*s_stop_k <= k) break;
  }
  if (!__all_sync(0xffffffffu, got)) {
    if ((threadIdx.x & 31) == 0 && *s_stop_k > k) atomicOr(err, kErrLookbackTimeout);
    return false;
  }
  return true;
}

// Draws the next tile ticket for a persistent launch of `grid` CTAs over
// `ntiles` tiles.  Every CTA draws until it gets one >= ntiles, so the launch
// draws ntiles + grid tickets; the last draw resets the counter and advances
// the epoch for the next launch (every CTA read the epoch before its first draw).
__device__ __forceinline__ uint32_t draw_ticket_persistent(LaunchState* ls, uint32_t ntiles) {
  const uint32_t t = atomicAdd(&ls->ticket, 1u);
  if (t == ntiles + gridDim.x - 1) {
    ls->ticket = 0;
    __threadfence();
    atomicAdd(&ls->epoch, 1u);
  }
  return t;
}

// Bulk-copies bytes [g0, g1) of a buffer [buf, buf + buf_len) into shared
// memory so that byte g lands at sdst + (g - floor16(g0)): the 16-byte-aligned
// part by TMA (completing on bar), bytes outside it by plain loads.  Returns
// the byte count the caller must expect on bar (0: nothing in flight).  One
// thread.
__device__ __forceinline__ uint32_t stage_range(uint8_t* sdst, const uint8_t* buf, uint64_t buf_len,
                                                uintptr_t g0, uintptr_t g1) {
  if (g1 <= g0) return 0;
  const uintptr_t ba = (uintptr_t)buf;
  const uintptr_t a0 = g0 & ~(uintptr_t)15;
  const uintptr_t b0 = max(a0, (ba + 15) & ~(uintptr_t)15);
  const uintptr_t b1 = min((g1 + 15) & ~(uintptr_t)15, (ba + buf_len) & ~(uintptr_t)15);
  if (b1 > b0) {
    for (uintptr_t p = g0; p < b0; p++) sdst[p - a0] = __ldg(reinterpret_cast<const uint8_t*>(p));
    for (uintptr_t p = max(b1, g0); p < g1; p++) sdst[p - a0] = __ldg(reinterpret_cast<const uint8_t*>(p));
    return (uint32_t)(b1 - b0);
  }
  for (uintptr_t p = g0; p < g1; p++) sdst[p - a0] = __ldg(reinterpret_cast<const uint8_t*>(p));
  return 0;
}

// Issues the TMA part of a stage_range (after the expect_tx on bar).
__device__ __forceinline__ void stage_range_issue(uint8_t* sdst, const uint8_t* buf, uint64_t buf_len,
                                                  uintptr_t g0, uintptr_t g1, uint64_t* bar) {
  if (g1 <= g0) return;
  const uintptr_t ba = (uintptr_t)buf;
  const uintptr_t a0 = g0 & ~(uintptr_t)15;
  const uintptr_t b0 = max(a0, (ba + 15) & ~(uintptr_t)15);
  const uintptr_t b1 = min((g1 + 15) & ~(uintptr_t)15, (ba + buf_len) & ~(uintptr_t)15);
  if (b1 > b0) bulk_load(sdst + (b0 - a0), reinterpret_cast<const void*>(b0), (uint32_t)(b1 - b0), bar);
}

}  // namespace szp
