// szp_device.cuh -- device-side helpers shared by the SZp fastmode1/2 kernels.
//
// Stream format (byte-identical to SZp's, SZp/src/szp_float.cc:148-309):
//   [eb f32 big-endian][T x u64 segment offsets][segment 0]...[segment T-1]
//   segment = [i32 seed] {block}*  (fastmode1), blocks start at lo+1 step L
//   block   = [u8 bc] if bc>0: [sign bits MSB-first ceil(m/8)]
//             [m x (bc/8) bytes of v>>(bc%8), little-endian]
//             [low bc%8 bits of each v, one MSB-first bit string]
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace szp {

constexpr int kMaxBitCount = 33;

// Error bits written by kernels into Workspace::err (never a trap).
enum : uint32_t {
  kErrLookbackTimeout = 1u << 0,   // a wait (look-back or pipeline hand-off) gave up
  kErrCapacity = 1u << 1,          // stream larger than the caller's buffer
  kErrCorrupt = 1u << 2,           // malformed stream (bad bc, walk past end)
  kErrBlockCount = 1u << 3,        // segment did not hold the expected blocks
  kErrQuantRange = 1u << 4,        // |x/eb| >= 2^31 or NaN (reference UB; INT_MIN used)
};

// Bit-count thresholds: thr[k] = smallest m with (int)log2f((float)m)+1 >= k.
// Filled from the host libm once per process (see api.cu).
struct BitcountTable {
  uint32_t thr[36];
};

// bc = (int)log2f((float)max)+1 (szp_float.cc:261) without calling log2f on the
// device: the true width k = 32-clz(max) is exact and the reference's value is
// k or k+1, k+1 exactly when max >= thr[k+1].
__device__ __forceinline__ int bitcount_from_table(uint32_t max, const uint32_t* __restrict__ thr) {
  if (max == 0) return 0;
  int k = 32 - __clz(max);
  return k + (max >= thr[k + 1] ? 1 : 0);
}

// Exact q = (int)((double)x * (double)inv) of szp_float.cc:209,228 in FP32.
// The double product of two floats is exact, so trunc() of it equals trunc()
// of the round-toward-zero float product whenever |product| < 2^24 (every
// integer below 2^24 is a float, so RZ never crosses one).  Larger products
// take the FP64 path; out of range and NaN give INT32_MIN like x86's
// cvttsd2si, and raise kErrQuantRange.
__device__ __forceinline__ int32_t quantize_slow(float x, float inv, uint32_t& flags) {
  double p = __dmul_rn((double)x, (double)inv);
  if (p > -2147483649.0 && p < 2147483648.0) return __double2int_rz(p);
  flags |= kErrQuantRange;
  return INT32_MIN;
}

__device__ __forceinline__ int32_t quantize(float x, float inv, uint32_t& flags) {
  float p = __fmul_rz(x, inv);
  if (fabsf(p) < 16777216.0f) return __float2int_rz(p);
  return quantize_slow(x, inv, flags);
}

// q = (int)(x * inv) for float64 data (szp_double.cc:209,228): the double
// product rounds to nearest, the conversion truncates; out of range and NaN
// give INT32_MIN like x86's cvttsd2si, and raise kErrQuantRange.
__device__ __forceinline__ int32_t quantize_d(double x, double inv, uint32_t& flags) {
  const double p = __dmul_rn(x, inv);
  if (p > -2147483649.0 && p < 2147483648.0) return __double2int_rz(p);
  flags |= kErrQuantRange;
  return INT32_MIN;
}

// NaN results follow x86 SSE, where the reference's fixtures come from: a NaN
// operand propagates (quieted), an invalid operation (0*inf, inf-inf) gives
// the default NaN 0xFFC00000.  The GPU would return 0x7FFFFFFF.
__device__ __forceinline__ float x86_nan_fix(float r, float a, float b) {
  if (r == r) return r;
  uint32_t u = (a != a) ? __float_as_uint(a) : ((b != b) ? __float_as_uint(b) : 0xFFC00000u);
  return __uint_as_float(u | 0x00400000u);
}
// The same rule for double results (default NaN 0xFFF8000000000000).
__device__ __forceinline__ double x86_nan_fix_d(double r, double a, double b) {
  if (r == r) return r;
  const unsigned long long u = (a != a) ? (unsigned long long)__double_as_longlong(a)
                                        : ((b != b) ? (unsigned long long)__double_as_longlong(b)
                                                    : 0xFFF8000000000000ull);
  return __longlong_as_double((long long)(u | 0x0008000000000000ull));
}

// Byte size of an encoded block of m elements (1 <= m) with bit count bc.
__host__ __device__ __forceinline__ uint32_t block_bytes(uint32_t m, uint32_t bc) {
  if (bc == 0) return 1;
  uint32_t B = bc >> 3, r = bc & 7;
  return 1 + ((m + 7) >> 3) + B * m + ((r * m + 7) >> 3);
}

__host__ __device__ __forceinline__ uint32_t max_block_bytes(uint32_t L) {
  return block_bytes(L, kMaxBitCount);
}

// Geometry of the T contiguous segments (szp_float.cc:186,194-199).
struct Segments {
  uint64_t n;
  uint64_t tsz;  // floor(n / T)
  uint32_t T;
  uint32_t L;
  __host__ __device__ __forceinline__ uint64_t lo(uint32_t t) const { return (uint64_t)t * tsz; }
  __host__ __device__ __forceinline__ uint64_t hi(uint32_t t) const {
    return t + 1 == T ? n : (uint64_t)(t + 1) * tsz;
  }
  __host__ __device__ __forceinline__ uint64_t len(uint32_t t) const { return hi(t) - lo(t); }
  // fastmode1 blocks of segment t: ceil((len-1)/L) (the seed element excluded)
  __host__ __device__ __forceinline__ uint64_t blocks_fm1(uint32_t t) const {
    uint64_t l = len(t);
    return l > 1 ? (l - 1 + L - 1) / L : 0;
  }
};

// 64-bit look-back status word: [epoch:20][flag:2][value:42].
constexpr int kStatusValueBits = 42;
constexpr uint64_t kStatusValueMask = (1ull << kStatusValueBits) - 1;
constexpr uint64_t kFlagAggregate = 1, kFlagInclusive = 2;

__device__ __forceinline__ uint64_t make_status(uint32_t epoch, uint64_t flag, uint64_t value) {
  return ((uint64_t)(epoch & 0xFFFFF) << 44) | (flag << 42) | (value & kStatusValueMask);
}
__device__ __forceinline__ uint32_t status_epoch(uint64_t s) { return (uint32_t)(s >> 44); }
__device__ __forceinline__ uint64_t status_flag(uint64_t s) { return (s >> 42) & 3; }
__device__ __forceinline__ uint64_t status_value(uint64_t s) { return s & kStatusValueMask; }

__device__ __forceinline__ uint64_t ld_volatile_u64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(uint64_t* p, uint64_t v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// Look-back words carry their value, so publishing one orders nothing else:
// a relaxed store, which does not wait for the thread's earlier global writes
// to drain (a release store held the publishing warp, and with it the CTA at
// the next barrier, for that long).
__device__ __forceinline__ void st_relaxed_u64(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_acquire_u64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Per-launch ordering state.  Tiles are numbered by an atomic ticket so that
// every predecessor of a tile has started before it (look-back never waits
// on a CTA that is not resident).  The CTA that draws the last ticket resets
// the counter and bumps the epoch, so no memset is needed between launches
// and a captured graph can be replayed.
struct alignas(8) LaunchState {
  uint32_t ticket;  // low word of the pair
  uint32_t epoch;
};

// Draw a tile ticket; returns (tile, epoch) broadcast to the CTA.  One 64-bit
// atomic on (epoch, ticket) returns the ticket with the epoch it belongs to;
// the launch's last draw adds 2^32 - ntiles, which takes the ticket back to 0
// and carries into the epoch.
__device__ __forceinline__ void draw_ticket(LaunchState* ls, uint32_t ntiles, uint32_t& tile, uint32_t& epoch,
                                            uint32_t* smem2) {
  if (threadIdx.x == 0) {
    unsigned long long* w = reinterpret_cast<unsigned long long*>(ls);
    const unsigned long long old = atomicAdd(w, 1ull);
    const uint32_t t = (uint32_t)old;
    if (t == ntiles - 1) atomicAdd(w, (1ull << 32) - ntiles);
    smem2[0] = t;
    smem2[1] = (uint32_t)(old >> 32);
  }
  __syncthreads();
  tile = smem2[0];
  epoch = smem2[1];
  __syncthreads();
}

constexpr uint32_t kSpinLimit = 1u << 20;  // look-back polls (about a second) before giving up

// True once a wait of the launch has given up: later waits then return at
// once, so a launch that lost its hand-offs runs to its end with an error
// instead of waiting out every later wait.
__device__ __forceinline__ bool launch_gave_up(const uint32_t* err) {
  return (*(const volatile uint32_t*)err & kErrLookbackTimeout) != 0;
}

// Decoupled look-back over an additive 42-bit quantity, by one full warp.
// Each lane reads LB_K predecessors per round trip (lane l, slot k holds the
// tile at distance 1 + l + 32k), so a window covers 32*LB_K tiles: a tile whose
// nearest finished predecessor is D tiles back waits ceil(D / (32*LB_K)) round
// trips.  Tiles < stop_at are not consulted (a chain can restart at a segment
// boundary).  Returns the exclusive prefix; on timeout sets
// kErrLookbackTimeout and returns 0.  One window per round trip with a
// 500 ns pause between polls: polling competes with the compute warps for
// issue slots, and wider windows or tighter polling measured slower on both
// pipelines (a 512^3 field: compress 0.300 ms with one window, 0.325 with four,
// 0.446 with sixteen).
constexpr int LB_K = 1;

__device__ __forceinline__ uint64_t lookback_sum(const uint64_t* status, uint32_t tile, uint32_t stop_at,
                                                 uint32_t epoch, uint32_t* err) {
  const int lane = threadIdx.x & 31;
  const uint32_t ep = epoch & 0xFFFFF;
  uint64_t excl = 0;
  int64_t base = (int64_t)tile - 1;  // distance 1
  uint32_t spins = 0;
  while (base >= (int64_t)stop_at) {
    uint64_t s[LB_K];
    uint32_t incl[LB_K], nready[LB_K];
#pragma unroll
    for (int k = 0; k < LB_K; k++) {
      const int64_t idx = base - lane - 32 * k;
      s[k] = idx >= (int64_t)stop_at ? ld_volatile_u64(status + idx) : 0;
    }
    int dstar = 32 * LB_K;  // nearest inclusive (distance index), none yet
#pragma unroll
    for (int k = 0; k < LB_K; k++) {
      const int64_t idx = base - lane - 32 * k;
      const bool inr = idx >= (int64_t)stop_at;
      const bool ready = !inr || (status_epoch(s[k]) == ep && status_flag(s[k]) != 0);
      incl[k] = __ballot_sync(0xffffffffu, inr && ready && status_flag(s[k]) == kFlagInclusive);
      nready[k] = __ballot_sync(0xffffffffu, !ready);
      if (dstar == 32 * LB_K && incl[k]) dstar = 32 * k + __ffs(incl[k]) - 1;
    }
    // every predecessor closer than (and at) the nearest inclusive must be ready
    bool wait = false;
#pragma unroll
    for (int k = 0; k < LB_K; k++) {
      const int lo = 32 * k;
      if (lo > dstar) break;
      uint32_t rel = dstar - lo >= 31 ? 0xffffffffu : ((2u << (dstar - lo)) - 1u);
      if (nready[k] & rel) wait = true;
    }
    if (wait) {
      __nanosleep(500);  // a predecessor is still working: leave the issue slots to the compute warps
      if (++spins > kSpinLimit || ((spins & 63) == 0 && launch_gave_up(err))) {
        if (lane == 0) atomicOr(err, kErrLookbackTimeout);
        return 0;
      }
      continue;
    }
    uint64_t v = 0;
#pragma unroll
    for (int k = 0; k < LB_K; k++) {
      const int64_t idx = base - lane - 32 * k;
      if (idx >= (int64_t)stop_at && lane + 32 * k <= dstar) v += status_value(s[k]);
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    excl += v;
    if (dstar < 32 * LB_K) break;
    base -= 32 * LB_K;
  }
  return excl;
}


}  // namespace szp
