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
constexpr uint32_t kWaitLimit = 1u << 24;    // polls of a shared-memory counter (with a 64 ns pause each)
constexpr uint64_t kWaitNs = 2000000000ull;  // an mbarrier wait gives up after about two seconds

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for an mbarrier phase for at most `ns` nanoseconds; false if it did
// not complete.
__device__ __forceinline__ bool mbar_wait_ns(uint64_t* bar, uint32_t parity, uint64_t ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (globaltimer_ns() - t0 < ns)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Barrier over the 256 compute threads (warps 0-7) only.
__device__ __forceinline__ void compute_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// Waits for an mbarrier phase; after about two seconds flags the launch as
// given up.  Once the launch is flagged, waits return after their first 256
// polls.  The flag and the clock are read out of line, after 256 polls: a
// read of the flag is a trip to L2, which would delay every short wait.
static __device__ __noinline__ void mbar_wait_long(uint64_t* bar, uint32_t parity, uint32_t* err) {
  if (launch_gave_up(err)) return;
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t i = 1;; i++) {
    if (mbar_try_wait(bar, parity)) return;
    if ((i & 255) == 0 && (launch_gave_up(err) || globaltimer_ns() - t0 > kWaitNs)) break;
  }
  if (!launch_gave_up(err)) atomicOr(err, kErrLookbackTimeout);
}
__device__ __forceinline__ void mbar_wait_or_flag(uint64_t* bar, uint32_t parity, uint32_t* err) {
#pragma unroll 1
  for (int i = 0; i < 256; i++)
    if (mbar_try_wait(bar, parity)) return;
  mbar_wait_long(bar, parity, err);  // out of line: the clock and the flag stay off short waits
}

// A control warp's wait for slot phase `parity` of its k-th tile, or for the
// producer's stop at an earlier or equal k; true when the slot is full.
__device__ __forceinline__ bool control_wait_full(uint64_t* full, uint32_t parity, uint32_t k,
                                                  const volatile uint32_t* s_stop_k, uint32_t* err) {
  bool got = false;
  uint64_t t0 = 0;  // first read at the 256th poll
  for (uint32_t i = 1; !(got = mbar_try_wait(full, parity)) && *s_stop_k > k; i++) {
    if ((i & 255) == 0) {
      if (launch_gave_up(err)) break;
      const uint64_t t = globaltimer_ns();
      if (t0 == 0) {
        t0 = t;
      } else if (t - t0 > kWaitNs) {
        break;
      }
    }
  }
  if (!__all_sync(0xffffffffu, got)) {
    if ((threadIdx.x & 31) == 0 && *s_stop_k > k) atomicOr(err, kErrLookbackTimeout);
    return false;
  }
  return true;
}

// Called by a producer before it returns at position `k` (its stop): waits
// until the bulk copies of its last NS positions have landed, so no copy
// outlives the CTA even when a launch gave up its hand-offs.
template <int NS>
__device__ __forceinline__ void drain_copies(uint64_t* full, uint32_t k) {
  for (uint32_t j = k >= (uint32_t)NS ? k - NS : 0u; j < k; j++) mbar_wait_ns(&full[j % NS], (j / NS) & 1, kWaitNs);
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

// Offset of segment t, after an eb header of hb bytes (4 float, 8 double).
__device__ __forceinline__ void write_offset(uint8_t* out, uint32_t t, uint64_t off, uint32_t hb = 4) {
  uint8_t* p = out + hb + 8ull * t;
  for (int i = 0; i < 8; i++) p[i] = (uint8_t)(off >> (8 * i));
}

// eb (big-endian) and, when every segment but the last is empty (n < T),
// their zero offsets (szp_float.cc:164,280-289); one warp.
__device__ __forceinline__ void write_header_warp(uint8_t* out, float eb, const Segments& sg, int lane) {
  const uint32_t b = __float_as_uint(eb);
  if (lane < 4) out[lane] = (uint8_t)(b >> (24 - 8 * lane));
  if (sg.tsz == 0) {
    const uint32_t nz = 8 * (sg.n == 0 ? sg.T : sg.T - 1);
    for (uint32_t i = lane; i < nz; i += 32) out[4 + i] = 0;
  }
}

// The float64 stream's header: eb as 8 big-endian bytes, zero offsets as above.
__device__ __forceinline__ void write_header_warp(uint8_t* out, double eb, const Segments& sg, int lane) {
  const uint64_t b = (uint64_t)__double_as_longlong(eb);
  if (lane < 8) out[lane] = (uint8_t)(b >> (56 - 8 * lane));
  if (sg.tsz == 0) {
    const uint32_t nz = 8 * (sg.n == 0 ? sg.T : sg.T - 1);
    for (uint32_t i = lane; i < nz; i += 32) out[8 + i] = 0;
  }
}

// One warp copies len bytes from shared memory src (16-byte aligned, readable
// for len + 16 bytes) to global dst (any alignment): 16-byte stores for the
// aligned middle, the bytes shifted into place with funnel shifts; byte
// stores for the ragged ends, which neighbouring tiles share.
__device__ __forceinline__ void warp_store_span(uint8_t* __restrict__ dst, const uint8_t* __restrict__ src,
                                                uint32_t len, int lane) {
  if (len == 0) return;
  const uint32_t a = (uint32_t)((uintptr_t)dst & 15);
  uint8_t* g0 = dst - a;                             // 16-byte aligned
  const uint32_t end = a + len;                      // the span is [a, end) from g0
  const uint32_t c0 = (a + 15) >> 4, c1 = end >> 4;  // whole 16-byte chunks [c0, c1)
  if (c0 >= c1) {
    for (uint32_t b = a + (uint32_t)lane; b < end; b += 32) g0[b] = src[b - a];
    return;
  }
  if ((uint32_t)lane < 16 * c0 - a) g0[a + lane] = src[lane];
  if ((uint32_t)lane < end - 16 * c1) g0[16 * c1 + lane] = src[16 * c1 + lane - a];
  const uint32_t sh = (16 - a) & 15;  // chunk c starts at src byte 16c - a = 16(c - 1) + sh when a != 0
  if (sh == 0) {
    for (uint32_t c = c0 + lane; c < c1; c += 32)
      *reinterpret_cast<uint4*>(g0 + 16 * c) = *reinterpret_cast<const uint4*>(src + 16 * c);
    return;
  }
  const uint32_t q = sh >> 2, bs = 8 * (sh & 3);
  // two chunks per lane per pass: their shared-memory loads are in flight together
  for (uint32_t cb = c0; cb < c1; cb += 64) {
    uint4 o[2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const uint32_t c = min(cb + lane + 32 * k, c1 - 1);  // clamped: always a readable chunk
      const uint4* line = reinterpret_cast<const uint4*>(src + 16 * (c - 1));
      const uint4 u = line[0], v = line[1];
      const uint32_t w[8] = {u.x, u.y, u.z, u.w, v.x, v.y, v.z, v.w};
#define SZP_FS(i) __funnelshift_r(w[(i)], w[(i) + 1], bs)
      switch (q) {
        case 0: o[k] = make_uint4(SZP_FS(0), SZP_FS(1), SZP_FS(2), SZP_FS(3)); break;
        case 1: o[k] = make_uint4(SZP_FS(1), SZP_FS(2), SZP_FS(3), SZP_FS(4)); break;
        case 2: o[k] = make_uint4(SZP_FS(2), SZP_FS(3), SZP_FS(4), SZP_FS(5)); break;
        default: o[k] = make_uint4(SZP_FS(3), SZP_FS(4), SZP_FS(5), SZP_FS(6)); break;
      }
#undef SZP_FS
    }
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const uint32_t c = cb + lane + 32 * k;
      if (c < c1) *reinterpret_cast<uint4*>(g0 + 16 * c) = o[k];
    }
  }
}

}  // namespace szp
