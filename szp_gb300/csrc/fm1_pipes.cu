// fm1_pipes.cu -- the fastmode1 float32 compressor specialised for blockSize 32,
// the configuration of SZp's benchmark drivers (szp_compress(..., blockSize 32)
// with SZP_NONRANDOMACCESS, SZp/src/szp_float.cc:148-309).
//
// A persistent, warp-specialised pipeline like compress_pipe (a producer
// thread stages each tile's input window by TMA, 8 compute warps analyse and
// pack it, a control warp finds its stream position by decoupled look-back),
// with two changes of structure and the compute cut down to what this one
// configuration needs.
//
// Structure: a tile's input slot is freed as soon as its analysis is done,
// and its packed bytes go to a ring in shared memory.  The control warp only
// places tiles (decoupled look-back, header and segment offsets); the compute
// warps copy a tile from the ring to the stream two tiles later, all 256
// threads at once.  A tile's position waits for its slowest predecessor
// anywhere on the GPU; with the ring that wait holds no input slot, and the
// compute warps only wait when a position is still unknown two tiles on, or
// the ring is full.
//
// Compute:
//   * the analysis is compiled once per 16-byte phase of the tile's input in
//     shared memory (the phase is constant within a segment), so every lane
//     loads its 8 elements with 2 or 3 16-byte loads and no selects;
//   * the quantization range check is one NaN-propagating max per element
//     (|x/eb| < 2^24 keeps the round-toward-zero float product exact);
//   * the previous element's code comes from a shuffle of the round before;
//   * sign bits enter with one funnel shift per element; the bit count is the
//     exact width 32-clz(max), with the log2f rule's extra bit applied on a
//     rare, warp-uniform path (max >= 2^20);
//   * two rounds' block sizes share one 32-bit scan (16-bit halves);
//   * remainder bits accumulate by multiply-add (v < 2^r when bc < 8).
// Tiles other than full ones (a segment's last, short tile) take a masked,
// exact path.  Every other blockSize, fastmode2, float64 codes and the
// batched launches stay on compress_pipe.
#include <atomic>
#include <cstring>

#include "szp_device.cuh"
#include "szp_kernels.h"
#include "szp_pipe.cuh"
#include "szp_tma.cuh"

namespace szp {
namespace {

constexpr uint32_t kL = 32;             // blockSize
constexpr int kW = 8;                   // compute warps
constexpr int kR = 4;                   // rounds per compute warp
constexpr uint32_t kTB = kW * kR * 8;   // blocks per tile (8 blocks of 4 lanes per round)
constexpr uint32_t kTE = kTB * kL;      // elements of a full tile
constexpr int kNS = 2;                  // input slots
constexpr int kThreads = (kW + 2) * 32; // compute warps, control warp, producer warp

// An input slot holds a tile's window (kTE + 1 floats from a 16-byte
// boundary, and the 16-byte loads past its end).  Packed tiles go to a ring
// of kRing bytes (16-byte-aligned starts, kRingPad bytes of padding for the
// shifted copy's reads past a tile's end); the largest tile, 4 + kTB blocks
// of 137 bytes, fits it.  At most kRecs tiles wait in the ring.
constexpr uint32_t kSlotBytes = 4 * (kTE + 8);
constexpr uint32_t kRing = 45056;
constexpr uint32_t kRingPad = 32;
constexpr int kRecs = 16;
static_assert(4 + kTB * 137 <= kRing, "the ring holds the largest tile");
static_assert(kSlotBytes % 16 == 0 && kRing % 16 == 0, "16-byte-aligned regions");

struct C32Meta {
  uint64_t lo, hi, e0;  // segment element range; first element of the tile's first block
  uint32_t tile;        // launch tile; kStopTile: no more tiles
  uint32_t seg;         // segment
  uint32_t nblk, nel;   // blocks of the tile and their elements
  uint32_t d;           // slot float index of element e0 - 1
  uint32_t first;       // first tile of its segment: the seed goes in front
  uint32_t has_seg;     // the stream has elements
};

// What the control warp needs of a tile, written by compute thread 0 once the
// tile's packed size is known (before it is packed); the control warp's
// stream position comes back in gpos.
struct C32Rec {
  uint64_t end;    // ring bytes allocated up to and including this tile
  uint64_t gpos;   // stream position, written by the control warp (~0: does not fit)
  uint32_t tile;   // launch tile
  uint32_t seg;    // segment
  uint32_t first;  // first tile of its segment (the stream has elements)
  uint32_t agg;    // packed bytes
  uint32_t rpos;   // ring offset of the packed bytes
};

// Producer: one thread.  Draws tile tickets in order and, for each, stages
// the input window [e0 - 1, e0 + nel) in a free slot (element e at slot float
// e - (e0 - 1) + d): the 16-byte-aligned middle by one bulk copy, issued
// first, the ragged ends by plain loads.
__device__ __forceinline__ void c32_producer(const CompressArgs& a, uint8_t* slots, C32Meta* meta, uint64_t* full,
                                             uint64_t* empty, uint32_t* s_epoch, volatile uint32_t* s_stop_k) {
  *s_epoch = *(volatile uint32_t*)&a.ls->epoch;
  __threadfence();
  const Segments sg = a.seg;
  for (uint32_t k = 0;; k++) {
    const int s = (int)(k % kNS);
    if (k >= (uint32_t)kNS) mbar_wait_or_flag(&empty[s], ((k / kNS) - 1) & 1, a.err);
    const uint32_t tile = draw_ticket_persistent(a.ls, a.ntiles);
    C32Meta& m = meta[s];
    if (tile >= a.ntiles) {
      drain_copies<kNS>(full, k);
      m.tile = kStopTile;
      *s_stop_k = k;
      mbar_arrive(&full[s]);
      return;
    }
    float* sx = reinterpret_cast<float*>(slots + (size_t)s * kSlotBytes);
    // segment and position of the tile (the host's tile_counts geometry)
    uint32_t t = sg.T - 1, ts = tile;
    if (a.tiles_per_seg) {
      t = tile / a.tiles_per_seg;
      if (t > sg.T - 1) t = sg.T - 1;
      ts = tile - t * a.tiles_per_seg;
    }
    const uint64_t lo = (uint64_t)t * sg.tsz, hi = t + 1 == sg.T ? sg.n : lo + sg.tsz;
    const uint64_t nb = t + 1 == sg.T ? a.nb_last : a.nb_reg;
    const uint64_t blk0 = (uint64_t)ts * kTB;
    const uint32_t nblk = nb > blk0 ? (uint32_t)min((uint64_t)kTB, nb - blk0) : 0u;
    const uint64_t e0 = lo + 1 + blk0 * kL;
    const uint32_t nel = nblk ? (uint32_t)min((uint64_t)nblk * kL, hi - e0) : 0u;
    m.lo = lo;
    m.hi = hi;
    m.e0 = e0;
    m.seg = t;
    m.nblk = nblk;
    m.nel = nel;
    m.first = ts == 0;
    m.has_seg = sg.n > 0;
    m.d = 0;
    if (sg.n > 0 && (nblk || (ts == 0 && hi > lo))) {  // a lone seed still needs x[lo]
      const uintptr_t xa = (uintptr_t)a.x;
      const uintptr_t w0 = xa + 4 * (e0 - 1), w1 = xa + 4 * (e0 + nel);
      const uintptr_t a0 = w0 & ~(uintptr_t)15;
      m.d = (uint32_t)((w0 - a0) >> 2);
      const uintptr_t b0 = max(a0, (xa + 15) & ~(uintptr_t)15);
      const uintptr_t b1 = min((w1 + 15) & ~(uintptr_t)15, (xa + 4 * sg.n) & ~(uintptr_t)15);
      if (b1 > b0) {
        fence_async_smem();
        mbar_expect_tx(&full[s], (uint32_t)(b1 - b0));
        bulk_load(reinterpret_cast<uint8_t*>(sx) + (b0 - a0), reinterpret_cast<const void*>(b0), (uint32_t)(b1 - b0),
                  &full[s]);
        for (uintptr_t p = w0; p < b0; p += 4) sx[(p - a0) >> 2] = __ldg(reinterpret_cast<const float*>(p));
        for (uintptr_t p = max(b1, w0); p < w1; p += 4) sx[(p - a0) >> 2] = __ldg(reinterpret_cast<const float*>(p));
      } else {
        for (uintptr_t p = w0; p < w1; p += 4) sx[(p - a0) >> 2] = __ldg(reinterpret_cast<const float*>(p));
      }
    }
    m.tile = tile;
    mbar_arrive(&full[s]);
  }
}

// Control warp: for each of the CTA's tiles in order, the stream position
// (the eb header for the first tile, the decoupled look-back for the others),
// the segment offset of a segment's first tile and the stream size after the
// last tile.  The position goes back to the compute warps in the record.
__device__ __forceinline__ void c32_control(const CompressArgs& a, C32Rec* rec, uint64_t* recb, uint64_t* based,
                                            const uint32_t* s_epoch, const volatile uint32_t* s_stop_k, float eb) {
  const int lane = threadIdx.x & 31;
  const uint64_t head = 4 + 8ull * a.seg.T;
  for (uint32_t k = 0;; k++) {
    const int p = (int)(k % kRecs);
    if (!control_wait_full(&recb[p], (k / kRecs) & 1, k, s_stop_k, a.err)) return;
    C32Rec& r = rec[p];
    const uint32_t tile = r.tile, agg = r.agg;
    const uint32_t epoch = *s_epoch;
    uint64_t excl = 0;
    if (tile == 0) {
      write_header_warp(a.out, eb, a.seg, lane);
    } else {
      excl = lookback_sum(a.status, tile, 0, epoch, a.err);
      if (lane == 0) st_relaxed_u64(a.status + tile, make_status(epoch, kFlagInclusive, excl + agg));
    }
    if (lane == 0) {
      const uint64_t gpos = head + excl;
      const bool fits = gpos + agg <= a.cap;
      if (tile == a.ntiles - 1) *a.out_size = gpos + agg;
      if (r.first && fits) write_offset(a.out, r.seg, excl);
      if (!fits) atomicOr(a.err, kErrCapacity);
      r.gpos = fits ? gpos : ~0ull;
      mbar_arrive(&based[p]);
    }
    __syncwarp();
  }
}

// The 256 compute threads copy len bytes staged at src (16-byte aligned,
// readable for len + 16 bytes) to global dst (any alignment): 16-byte stores
// of the aligned middle, each chunk funnel-shifted out of two aligned lines;
// byte stores at the ragged ends, which neighbouring tiles share.
__device__ __forceinline__ void cta_store_span(uint8_t* __restrict__ dst, const uint8_t* __restrict__ src, uint32_t len,
                                               uint32_t tid) {
  if (len == 0) return;
  const uint32_t a = (uint32_t)((uintptr_t)dst & 15);
  uint8_t* g0 = dst - a;                             // 16-byte aligned
  const uint32_t end = a + len;                      // the span is [a, end) from g0
  const uint32_t c0 = (a + 15) >> 4, c1 = end >> 4;  // whole 16-byte chunks [c0, c1)
  if (c0 >= c1) {
    if (tid < len) g0[a + tid] = src[tid];
    return;
  }
  if (tid < 16 * c0 - a) g0[a + tid] = src[tid];
  if (tid >= 32 && tid - 32 < end - 16 * c1) g0[16 * c1 + tid - 32] = src[16 * c1 + tid - 32 - a];
  const uint32_t sh = (16 - a) & 15;  // chunk c starts at src byte 16c - a = 16(c - 1) + sh when a != 0
  if (sh == 0) {
    for (uint32_t c = c0 + tid; c < c1; c += kW * 32)
      *reinterpret_cast<uint4*>(g0 + 16 * c) = *reinterpret_cast<const uint4*>(src + 16 * c);
    return;
  }
  const uint32_t q = sh >> 2, bs = 8 * (sh & 3);
  for (uint32_t c = c0 + tid; c < c1; c += kW * 32) {
    const uint4* line = reinterpret_cast<const uint4*>(src + 16 * (c - 1));
    const uint4 u = line[0], v = line[1];
    const uint32_t w[8] = {u.x, u.y, u.z, u.w, v.x, v.y, v.z, v.w};
    uint4 o;
#define SZP_FS(i) __funnelshift_r(w[(i)], w[(i) + 1], bs)
    switch (q) {
      case 0: o = make_uint4(SZP_FS(0), SZP_FS(1), SZP_FS(2), SZP_FS(3)); break;
      case 1: o = make_uint4(SZP_FS(1), SZP_FS(2), SZP_FS(3), SZP_FS(4)); break;
      case 2: o = make_uint4(SZP_FS(2), SZP_FS(3), SZP_FS(4), SZP_FS(5)); break;
      default: o = make_uint4(SZP_FS(3), SZP_FS(4), SZP_FS(5), SZP_FS(6)); break;
    }
#undef SZP_FS
    *reinterpret_cast<uint4*>(g0 + 16 * c) = o;
  }
}

// max(m, |p|) that keeps a NaN (max.NaN), so one compare after the tile
// catches both |x/eb| >= 2^24 and NaN inputs.
__device__ __forceinline__ float maxabs_nan(float m, float p) {
  float r;
  asm("{\n .reg .f32 t;\n abs.f32 t, %2;\n max.NaN.f32 %0, %1, t;\n}" : "=f"(r) : "f"(m), "f"(p));
  return r;
}

// Per lane and round: the 8 magnitudes, the sign byte (element 0 in bit 7),
// the block's max and then bit count (the same in the block's 4 lanes).
struct C32Analysis {
  uint32_t v[kR][8];
  uint32_t sb[kR];
  uint32_t bc[kR];
};

// Full tile, input phase PH = (slot index of tile element 0) mod 4.  Fast
// quantization q = trunc(x * inv) by the round-toward-zero float product,
// exact while |x * inv| < 2^24; returns false when some element of the lane's
// share (or the element before the warp's first) fails that or is NaN.
template <int PH>
__device__ __forceinline__ bool c32_analyse_fast(const float* __restrict__ sx, uint32_t sh, float inv, int warp,
                                                 int lane, C32Analysis& an) {
  const int sub = lane & 3, grp = lane >> 2;
  float pm = 0.0f;
  // code of the element before the warp's first one
  const float pb = __fmul_rz(sx[sh + (uint32_t)warp * (kR * 8 * kL) - 1], inv);
  pm = maxabs_nan(pm, pb);
  int32_t carry = __float2int_rz(pb);
#pragma unroll
  for (int r = 0; r < kR; r++) {
    const uint32_t k0 = ((uint32_t)(warp * kR + r) * 8 + grp) * kL + 8 * sub;
    const uint32_t i = sh + k0;  // i % 4 == PH
    const float4* q4 = reinterpret_cast<const float4*>(sx + (i - PH));
    float x[8];
    const float4 A = q4[0], B = q4[1];
    if constexpr (PH == 0) {
      x[0] = A.x; x[1] = A.y; x[2] = A.z; x[3] = A.w; x[4] = B.x; x[5] = B.y; x[6] = B.z; x[7] = B.w;
    } else {
      const float4 C = q4[2];
      const float w[12] = {A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w, C.x, C.y, C.z, C.w};
#pragma unroll
      for (int j = 0; j < 8; j++) x[j] = w[PH + j];
    }
    int32_t q[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const float p = __fmul_rz(x[j], inv);
      pm = maxabs_nan(pm, p);
      q[j] = __float2int_rz(p);
    }
    int32_t prev = __shfl_up_sync(0xffffffffu, q[7], 1);
    if (lane == 0) prev = carry;
    carry = __shfl_sync(0xffffffffu, q[7], 31);
    uint32_t sb = 0, lmax = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int32_t d = (int32_t)((uint32_t)q[j] - (uint32_t)prev);  // wrapping, as the compiled reference
      prev = q[j];
      const uint32_t v = (uint32_t)abs(d);  // |INT_MIN| is 2^31 as in the reference
      sb = __funnelshift_l((uint32_t)d, sb, 1);
      lmax = max(lmax, v);
      an.v[r][j] = v;
    }
    an.sb[r] = sb;
    lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, 1));
    lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, 2));
    an.bc[r] = lmax;  // the block max for now; the caller turns it into a bit count
  }
  return pm < 16777216.0f;
}

// Any tile, exact quantization and per-element masks (a segment's last tile,
// a warp whose fast pass failed).  ml: elements of the lane in round r.
__device__ __forceinline__ void c32_analyse_exact(const float* __restrict__ sx, uint32_t sh, float inv,
                                                  const C32Meta& g, int warp, int lane, C32Analysis& an,
                                                  uint32_t& flags) {
  const int sub = lane & 3, grp = lane >> 2;
#pragma unroll
  for (int r = 0; r < kR; r++) {
    const uint32_t bt = (uint32_t)(warp * kR + r) * 8 + grp;
    const uint32_t k0 = bt * kL + 8 * sub;
    const uint32_t ml = (bt < g.nblk && k0 < g.nel) ? min(8u, g.nel - k0) : 0u;
    int32_t q[8];
#pragma unroll
    for (int j = 0; j < 8; j++) q[j] = (uint32_t)j < ml ? quantize(sx[sh + k0 + j], inv, flags) : 0;
    // the element before the lane's first (a block's first lane takes it
    // from the block before, which may be another warp's)
    int32_t prev = __shfl_up_sync(0xffffffffu, q[7], 1);
    if (sub == 0 && bt < g.nblk) prev = quantize(sx[sh + k0 - 1], inv, flags);
    uint32_t sb = 0, lmax = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int32_t d = (int32_t)((uint32_t)q[j] - (uint32_t)prev);
      prev = q[j];
      const bool valid = (uint32_t)j < ml;
      const uint32_t v = valid ? (uint32_t)abs(d) : 0u;
      sb = (sb << 1) | (valid ? ((uint32_t)d >> 31) : 0u);
      lmax = max(lmax, v);
      an.v[r][j] = v;
    }
    an.sb[r] = sb;
    lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, 1));
    lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, 2));
    an.bc[r] = lmax;
  }
}

// Packs a full block's lane share (8 elements) at dst (the block's bit-count
// byte): bc and sign bytes, the byte planes, the remainder bits MSB first
// (szp_TypeManager.cc:13-94,122-434,820-844).  bmax/rmax: the warp's largest
// B and r this round (loop bounds; the stores are predicated per lane).
__device__ __forceinline__ void c32_pack_full(uint8_t* dst, const uint32_t (&v)[8], uint32_t sb, uint32_t bc, int sub,
                                              uint32_t bmax, uint32_t rmax) {
  if (sub == 0) dst[0] = (uint8_t)bc;
  if (bc == 0) return;
  dst[1 + sub] = (uint8_t)sb;
  const uint32_t B = bc >> 3, rr = bc & 7;
  const uint32_t pw = 1u << rr;
  uint32_t hi4, lo4;  // elements 0-3 and 4-7, rr bits each, element 0 on top
  if (bmax == 0) {    // v < 2^rr: no masking
    hi4 = ((v[0] * pw + v[1]) * pw + v[2]) * pw + v[3];
    lo4 = ((v[4] * pw + v[5]) * pw + v[6]) * pw + v[7];
  } else {
    const uint32_t mk = pw - 1u;
    hi4 = (((v[0] & mk) * pw + (v[1] & mk)) * pw + (v[2] & mk)) * pw + (v[3] & mk);
    lo4 = (((v[4] & mk) * pw + (v[5] & mk)) * pw + (v[6] & mk)) * pw + (v[7] & mk);
    uint8_t* q8 = dst + 5 + 8 * B * sub;
    for (uint32_t b = 0; b < bmax; b++) {
      if (b < B) {
#pragma unroll
        for (int j = 0; j < 8; j++) q8[j * B + b] = (uint8_t)((v[j] >> rr) >> (8 * b));
      }
    }
  }
  if (rmax == 0 || rr == 0) return;
  // 8*rr bits, element 0 first, moved to the top of 64 bits
  const uint64_t top = (((uint64_t)hi4 << (4 * rr)) | lo4) << (64 - 8 * rr);
  const uint32_t th = (uint32_t)(top >> 32), tl = (uint32_t)top;
  uint8_t* rp = dst + 5 + 32 * B + rr * sub;
#pragma unroll
  for (uint32_t i = 0; i < 7; i++) {
    if (i < rmax && i < rr) rp[i] = (uint8_t)(i < 4 ? th >> (24 - 8 * i) : tl >> (56 - 8 * i));
  }
}

// Packs any block's lane share with its element count m (a short last block).
__device__ __forceinline__ void c32_pack_masked(uint8_t* dst, const uint32_t (&v)[8], uint32_t sb, uint32_t bc, int sub,
                                                uint32_t m) {
  const uint32_t ml = m > 8u * sub ? min(8u, m - 8u * sub) : 0u;
  if (sub == 0) dst[0] = (uint8_t)bc;
  if (bc == 0 || ml == 0) return;
  const uint32_t ns = (m + 7) >> 3, B = bc >> 3, rr = bc & 7;
  dst[1 + sub] = (uint8_t)sb;  // sign bits, szp_TypeManager.cc:820-844
  if (B) {                     // byte planes, szp_TypeManager.cc:36-52
    uint8_t* q8 = dst + 1 + ns + 8 * B * sub;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      if ((uint32_t)j < ml) {
        const uint32_t h = v[j] >> rr;
        for (uint32_t b = 0; b < B; b++) q8[j * B + b] = (uint8_t)(h >> (8 * b));
      }
    }
  }
  if (rr) {  // remainder bits, MSB first, szp_TypeManager.cc:122-434
    const uint32_t mask = (1u << rr) - 1u;
    uint32_t hi4 = 0, lo4 = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) hi4 = (hi4 << rr) | ((uint32_t)j < ml ? (v[j] & mask) : 0u);
#pragma unroll
    for (int j = 4; j < 8; j++) lo4 = (lo4 << rr) | ((uint32_t)j < ml ? (v[j] & mask) : 0u);
    const uint64_t acc = ((uint64_t)hi4 << (4 * rr)) | lo4;  // 8*rr bits, element 0 on top
    uint8_t* rp = dst + 1 + ns + B * m + rr * sub;
    const uint32_t nb = (ml * rr + 7) >> 3;
    const uint32_t top = 8 * rr - 8;
#pragma unroll
    for (uint32_t kk = 0; kk < 7; kk++)
      if (kk < nb) rp[kk] = (uint8_t)(acc >> (top - 8 * kk));
  }
}

__global__ void __launch_bounds__(kThreads, 2) compress32_pipe(const __grid_constant__ CompressArgs a) {
  extern __shared__ __align__(16) uint8_t s_dyn[];
  uint8_t* s_slots = s_dyn;                    // kNS input slots
  uint8_t* s_ring = s_dyn + kNS * kSlotBytes;  // kRing + kRingPad bytes
  __shared__ C32Meta s_meta[kNS];
  __shared__ C32Rec s_rec[kRecs];
  __shared__ uint32_t s_wtot[2][kW];  // compute warps' packed bytes, by tile parity
  __shared__ uint32_t s_thr[36];
  __shared__ uint32_t s_epoch;
  __shared__ volatile uint32_t s_stop_k;    // the producer's stop position
  __shared__ volatile uint32_t s_cstop_k;   // the compute warps' stop position (for the control warp)
  __shared__ __align__(8) uint64_t s_full[kNS], s_empty[kNS], s_recb[kRecs], s_based[kRecs];

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x < 36) s_thr[threadIdx.x] = a.thr.thr[threadIdx.x];
  if (threadIdx.x < kNS) s_meta[threadIdx.x].tile = kStopTile;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kNS; s++) {
      mbar_init(&s_full[s], 1);
      mbar_init(&s_empty[s], 1);
    }
    for (int p = 0; p < kRecs; p++) {
      mbar_init(&s_recb[p], 1);  // compute thread 0, once the tile's size is known
      mbar_init(&s_based[p], 1);
    }
    s_stop_k = kStopTile;
    s_cstop_k = kStopTile;
  }
  __syncthreads();
  const float eb = a.eb_dev ? *a.eb_dev : a.eb;

  if (warp == kW + 1) {
    if (lane == 0) c32_producer(a, s_slots, s_meta, s_full, s_empty, &s_epoch, &s_stop_k);
    return;
  }
  if (warp == kW) {
    c32_control(a, s_rec, s_recb, s_based, &s_epoch, &s_cstop_k, eb);
    return;
  }

  // ---- compute warps ----
  const float inv = __fdiv_rn(1.0f, eb);
  const int sub = lane & 3, grp = lane >> 2;
  const uint32_t tid = threadIdx.x;
  // Ring state, the same in every compute thread: bytes allocated and
  // released, the next position to copy out, and the end of a copied tile
  // whose space is released at the next barrier.
  uint64_t rhead = 0, rtail = 0, pend_end = 0;
  uint32_t ncopy = 0;
  // Copies position j out of the ring once the control warp has placed it.
  auto copy_out = [&](uint32_t j) {
    const int pj = (int)(j % kRecs);
    mbar_wait_or_flag(&s_based[pj], (j / kRecs) & 1, a.err);
    const uint64_t gpos = s_rec[pj].gpos;
    if (gpos != ~0ull) cta_store_span(a.out + gpos, s_ring + s_rec[pj].rpos, s_rec[pj].agg, tid);
    pend_end = s_rec[pj].end;
  };
  constexpr uint32_t kDefer = 2;  // tiles between packing a tile and copying it out
  for (uint32_t k = 0;; k++) {
    const int s = (int)(k % kNS);
    mbar_wait_or_flag(&s_full[s], (k / kNS) & 1, a.err);
    const C32Meta g = s_meta[s];
    if (g.tile >= a.ntiles) {
      if (tid == 0) s_cstop_k = k;  // the control warp ends after the tiles before k
      // a tile's position does not mean it is packed: every warp has packed
      // tile k - 1 after this barrier (the tiles before it are older than
      // one barrier already)
      compute_sync();
      for (; ncopy < k; ncopy++) copy_out(ncopy);
      return;
    }
    const float* sx = reinterpret_cast<const float*>(s_slots + (size_t)s * kSlotBytes);
    const bool seed = g.has_seg && g.first && g.hi > g.lo;  // the segment's seed element x[lo]
    uint32_t flags = 0;
    int32_t seedv = 0;
    if (seed && tid == 0) seedv = quantize(sx[g.d], inv, flags);  // window element 0

    // ---- analysis ----
    C32Analysis an;
    const uint32_t sh = 1 + g.d;  // slot index of tile element 0
    const bool full = g.nblk == kTB && g.nel == kTE;
    bool exact = !full;
    if (full) {
      bool ok;
      switch (sh & 3) {
        case 0: ok = c32_analyse_fast<0>(sx, sh, inv, warp, lane, an); break;
        case 1: ok = c32_analyse_fast<1>(sx, sh, inv, warp, lane, an); break;
        case 2: ok = c32_analyse_fast<2>(sx, sh, inv, warp, lane, an); break;
        default: ok = c32_analyse_fast<3>(sx, sh, inv, warp, lane, an); break;
      }
      exact = !__all_sync(0xffffffffu, ok);
    }
    if (exact) c32_analyse_exact(sx, sh, inv, g, warp, lane, an, flags);
    if (__any_sync(0xffffffffu, flags != 0) && lane == 0) atomicOr(a.err, kErrQuantRange);
    // block max -> bit count (int)log2f(max)+1 (szp_float.cc:253-262): the
    // exact width, one more at and above the libm thresholds (max >= 2^20)
    bool big = false;
#pragma unroll
    for (int r = 0; r < kR; r++) big |= an.bc[r] >= (1u << 20);
    const bool anybig = __any_sync(0xffffffffu, big);
#pragma unroll
    for (int r = 0; r < kR; r++) {
      const uint32_t lmax = an.bc[r];
      uint32_t bc = 32 - __clz(lmax);
      if (anybig && bc >= 21) bc += lmax >= s_thr[bc + 1] ? 1 : 0;
      an.bc[r] = bc;
    }

    // ---- block offsets: the warp's blocks in round order; two rounds per
    // 32-bit scan word (a round's 8 blocks hold at most 8 * 137 bytes) ----
    uint32_t sz[kR];
#pragma unroll
    for (int r = 0; r < kR; r++) {
      const uint32_t bt = (uint32_t)(warp * kR + r) * 8 + grp;
      const uint32_t m = bt < g.nblk ? min(kL, g.nel - bt * kL) : 0u;
      sz[r] = m == kL ? (an.bc[r] ? 4 * an.bc[r] + 5 : 1u) : (m ? block_bytes(m, an.bc[r]) : 0u);
    }
    uint32_t z01 = sz[0] | (sz[1] << 16), z23 = sz[2] | (sz[3] << 16);
#pragma unroll
    for (int o = 4; o < 32; o <<= 1) {
      const uint32_t y01 = __shfl_up_sync(0xffffffffu, z01, o), y23 = __shfl_up_sync(0xffffffffu, z23, o);
      if (lane >= o) {
        z01 += y01;
        z23 += y23;
      }
    }
    const uint32_t t01 = __shfl_sync(0xffffffffu, z01, 31), t23 = __shfl_sync(0xffffffffu, z23, 31);
    const uint32_t tot0 = t01 & 0xFFFFu, tot1 = t01 >> 16, tot2 = t23 & 0xFFFFu, tot3 = t23 >> 16;
    uint32_t off[kR];
    off[0] = (z01 & 0xFFFFu) - sz[0];
    off[1] = tot0 + (z01 >> 16) - sz[1];
    off[2] = tot0 + tot1 + (z23 & 0xFFFFu) - sz[2];
    off[3] = tot0 + tot1 + tot2 + (z23 >> 16) - sz[3];
    // warp totals, alternating buffers: a warp writes a buffer again only
    // after the next tile's barrier, which every reader of it has passed
    uint32_t* wtot = s_wtot[k & 1];
    if (lane == 0) wtot[warp] = tot0 + tot1 + tot2 + tot3;
    compute_sync();  // also ends every read of the input slot and of the last copied tile
    rtail = pend_end;
    const uint32_t front = seed ? 4u : 0u;
    uint32_t wexcl = front, agg = front;
#pragma unroll
    for (int w = 0; w < kW; w++) {
      const uint32_t t = wtot[w];
      wexcl += w < warp ? t : 0u;
      agg += t;
    }
    if (tid == 0) {
      const bool head = g.tile == 0;  // the stream's first tile has no predecessor
      st_relaxed_u64(a.status + g.tile, make_status(s_epoch, head ? kFlagInclusive : kFlagAggregate, agg));
      mbar_arrive(&s_empty[s]);  // the input slot is free for the producer
    }

    // ---- ring space: 16-byte-aligned and contiguous (a tile that would
    // wrap starts over at offset 0); when the older tiles leave too little,
    // they are copied out now ----
    uint64_t start = rhead;
    const uint32_t pos0 = (uint32_t)(start % kRing);
    if (pos0 + agg > kRing) start += kRing - pos0;
    const uint64_t end = start + ((agg + 15) & ~15u);
    const uint32_t rpos = (uint32_t)(start % kRing);
    while (end - rtail > kRing) {
      if (ncopy == k) {  // nothing waits in the ring: the skipped bytes belong to no tile
        rtail = start;
        break;
      }
      copy_out(ncopy++);
      compute_sync();  // the copied bytes are read before they are overwritten
      rtail = pend_end;
    }
    rhead = end;
    uint8_t* out = s_ring + rpos;
    const int p = (int)(k % kRecs);
    if (tid == 0) {
      C32Rec& r = s_rec[p];
      r.end = end;
      r.tile = g.tile;
      r.seg = g.seg;
      r.first = g.has_seg && g.first;
      r.agg = agg;
      r.rpos = rpos;
      mbar_arrive(&s_recb[p]);  // the control warp can place the tile while it is packed
      if (seed) {
        out[0] = (uint8_t)seedv;
        out[1] = (uint8_t)((uint32_t)seedv >> 8);
        out[2] = (uint8_t)((uint32_t)seedv >> 16);
        out[3] = (uint8_t)((uint32_t)seedv >> 24);
      }
    }

    // ---- pack into the ring ----
    if (full) {
#pragma unroll
      for (int r = 0; r < kR; r++) {
        const uint32_t bc = an.bc[r];
        const uint32_t bmax = __reduce_max_sync(0xffffffffu, bc >> 3);
        const uint32_t rmax = __reduce_max_sync(0xffffffffu, bc & 7);
        c32_pack_full(out + wexcl + off[r], an.v[r], an.sb[r], bc, sub, bmax, rmax);
      }
    } else {
#pragma unroll
      for (int r = 0; r < kR; r++) {
        const uint32_t bt = (uint32_t)(warp * kR + r) * 8 + grp;
        if (bt >= g.nblk) continue;
        c32_pack_masked(out + wexcl + off[r], an.v[r], an.sb[r], an.bc[r], sub, min(kL, g.nel - bt * kL));
      }
    }
    // ---- copy out the tile packed kDefer tiles ago (every warp packed it
    // before the last barrier; its space is released at the next one) ----
    if (ncopy + kDefer <= k) copy_out(ncopy++);
  }
}

}  // namespace

bool compress32_supported(const CompressArgs& a) { return a.seg.L == kL && a.fields == nullptr; }

cudaError_t launch_compress32(const CompressArgs& a, cudaStream_t st) {
  auto k = compress32_pipe;
  const size_t smem = (size_t)kNS * kSlotBytes + kRing + kRingPad;
  // resident CTAs, cached per device as (device + 1) << 32 | CTAs
  static std::atomic<uint64_t> s_cache{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  uint64_t c = s_cache.load(std::memory_order_relaxed);
  if ((c >> 32) != (uint64_t)dev + 1) {
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kThreads, smem);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    c = ((uint64_t)dev + 1) << 32 | (uint32_t)((occ < 1 ? 1 : occ) * sms);
    s_cache.store(c, std::memory_order_relaxed);
  }
  const uint32_t s_grid = (uint32_t)c;
  const uint32_t grid = a.ntiles < s_grid ? a.ntiles : s_grid;
  if (grid == 0) return cudaSuccess;
  k<<<grid, kThreads, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace szp
