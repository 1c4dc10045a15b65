// compress.cu -- SZp fastmode1 / fastmode2 float32 compressors for sm_103a.
//
// blockSize 8..256 (a power of two): compress_pipe, a persistent,
// warp-specialised pipeline (a producer warp stages tile inputs by TMA, eight
// compute warps quantize, analyse and pack each tile in shared memory, control
// warps find the tile's stream offset by decoupled look-back and write it with
// 16-byte stores).  Other blockSizes: compress_generic, one warp per block.
// The REL range pass (rel_bound_bulk over large inputs, rel_bound_kernel over
// small ones, rel_batch_kernel for batches) runs first.  HBM traffic: 4n
// bytes read (twice with REL), stream bytes written.
//
// Reference semantics followed (SZp/src/szp_float.cc):
//   quantize  (int)(x * (double)(1.0f/eb))                    :185,209,228
//   fastmode1 delta carried across blocks of a segment         :226-251
//   bit count (int)log2f(max)+1                                :253-262
//   sign bitmap / fixed-length packing   szp_TypeManager.cc:13-94,820-844
//   fastmode2 per-block seed                                   :812-864
#include <atomic>
#include <type_traits>

#include "szp_device.cuh"
#include "szp_f64.h"
#include "szp_kernels.h"
#include "szp_pipe.cuh"
#include "szp_tma.cuh"

namespace szp {

// Copy `len` bytes staged in shared memory starting at s_out[align] to global
// dst (where (uintptr_t)dst % 16 == align).  16-byte stores for whole
// chunks, byte stores at the ragged ends so neighbouring tiles never share a
// store.
__device__ __forceinline__ void flush_span(uint8_t* __restrict__ gdst, const uint8_t* __restrict__ s_out,
                                           uint32_t align, uint32_t len) {
  if (len == 0) return;
  uint8_t* gbase = gdst - align;  // 16-byte aligned
  const uint32_t end = align + len;
  const uint32_t nchunks = (end + 15) >> 4;
  for (uint32_t c = threadIdx.x; c < nchunks; c += blockDim.x) {
    uint32_t b0 = c << 4;
    if (b0 >= align && b0 + 16 <= end) {
      *reinterpret_cast<uint4*>(gbase + b0) = *reinterpret_cast<const uint4*>(s_out + b0);
    } else {
      uint32_t lo = b0 < align ? align : b0;
      uint32_t hi = b0 + 16 < end ? b0 + 16 : end;
      for (uint32_t b = lo; b < hi; b++) gbase[b] = s_out[b];
    }
  }
}

// Tile geometry shared by the compressors.
struct TileInfo {
  uint32_t seg;       // segment index
  uint64_t blk0;      // first block (segment-relative)
  uint32_t nblk;      // blocks in this tile
  bool first;         // first tile of its segment (carries the seed)
  bool has_seg;       // false for the header-only tile of an empty stream
};

__device__ __forceinline__ TileInfo tile_info(const Segments& sg, uint32_t tile, uint32_t tiles_per_seg,
                                              uint32_t tb, bool fm2) {
  TileInfo ti;
  if (sg.n == 0) {
    ti.seg = sg.T - 1;
    ti.blk0 = 0;
    ti.nblk = 0;
    ti.first = false;
    ti.has_seg = false;
    return ti;
  }
  uint32_t t, ts;
  if (tiles_per_seg) {
    t = tile / tiles_per_seg;
    if (t > sg.T - 1) t = sg.T - 1;
    ts = tile - t * tiles_per_seg;
  } else {
    t = sg.T - 1;
    ts = tile;
  }
  uint64_t nb = fm2 ? (sg.len(t) + sg.L - 1) / sg.L : sg.blocks_fm1(t);
  ti.seg = t;
  ti.blk0 = (uint64_t)ts * tb;
  uint64_t rem = nb > ti.blk0 ? nb - ti.blk0 : 0;
  ti.nblk = (uint32_t)(rem < tb ? rem : tb);
  ti.first = ts == 0;
  ti.has_seg = true;
  return ti;
}

// Writes eb (big-endian) and, when every segment but the last is empty
// (n < T), their zero offsets (szp_float.cc:164,280-289).
__device__ __forceinline__ void write_header_common(uint8_t* out, float eb, const Segments& sg) {
  uint32_t b = __float_as_uint(eb);
  for (int i = threadIdx.x; i < 4; i += blockDim.x) out[i] = (uint8_t)(b >> (24 - 8 * i));
  if (sg.tsz == 0) {
    uint32_t nz = 8 * (sg.n == 0 ? sg.T : sg.T - 1);
    for (uint32_t i = threadIdx.x; i < nz; i += blockDim.x) out[4 + i] = 0;
  }
}

// eb as a big-endian double (szp_double.cc:164, szp_CompressionToolkit.h:539-546)
// and the zero offsets of empty segments after it; float64 streams.
__device__ __forceinline__ void write_header_common(uint8_t* out, double eb, const Segments& sg) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(eb);
  for (int i = threadIdx.x; i < 8; i += blockDim.x) out[i] = (uint8_t)(b >> (56 - 8 * i));
  if (sg.tsz == 0) {
    uint32_t nz = 8 * (sg.n == 0 ? sg.T : sg.T - 1);
    for (uint32_t i = threadIdx.x; i < nz; i += blockDim.x) out[8 + i] = 0;
  }
}

// CTA-wide exclusive scan of per-warp byte counts; returns the tile aggregate.
template <int WARPS>
__device__ __forceinline__ uint32_t scan_warps(uint32_t* s_w, uint32_t mine, int warp, int lane, uint32_t& excl,
                                               uint32_t extra_front) {
  if (lane == 0) s_w[warp] = mine;
  __syncthreads();
  if (warp == 0) {
    uint32_t x = lane < WARPS ? s_w[lane] : 0;
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane < WARPS) s_w[lane] = incl - x + extra_front;
    if (lane == 31) s_w[WARPS] = incl + extra_front;
  }
  __syncthreads();
  excl = s_w[warp];
  return s_w[WARPS];
}

// ---------------------------------------------------------------------------
// fastmode1, blockSize L = 8*LPB (8..256): LPB lanes per block, 8 elements
// per lane.  Eight elements fill whole bytes in every section of a block
// (one sign byte, 8*B bytes of byte planes, r bytes of remainder bits), so
// each lane packs its part of a block without talking to other lanes; only
// the block max (LPB-lane reduction) and the byte offsets (a scan over the
// warp's lane groups and rounds, the warps' totals, decoupled look-back) are
// shared.  A warp handles ROUNDS groups of 32/LPB
// consecutive blocks; the 8 compute warps a tile of 8*ROUNDS*32/LPB blocks.
// fastmode2 keeps the layout: a block's L-1 deltas leave its last lane 7.
// ---------------------------------------------------------------------------


// Exact path for |x/eb| >= 2^24 (or NaN/inf), out of line so the common path
// issues no FP64 instructions; returns q in the low word, flags in the high.
__device__ __noinline__ uint64_t quantize_rare(float x, float inv) {
  uint32_t f = 0;
  const int32_t q = quantize_slow(x, inv, f);
  return ((uint64_t)f << 32) | (uint32_t)q;
}

// q = trunc(x/eb) (see quantize()), fast path inline.
__device__ __forceinline__ int32_t quantize_lean(float x, float inv, uint32_t& flags) {
  const float p = __fmul_rz(x, inv);
  int32_t q = __float2int_rz(p);
  if (!(fabsf(p) < 16777216.0f)) {
    const uint64_t r = quantize_rare(x, inv);
    q = (int32_t)(uint32_t)r;
    flags |= (uint32_t)(r >> 32);
  }
  return q;
}


// Tile geometry, computed by the producer.
struct TileGeo {
  uint64_t lo, hi;  // segment element range
  uint64_t e0;      // first element of the tile's first block
  uint32_t seg, nblk, nel;  // blocks, elements of those blocks
  uint32_t first;   // first tile of its segment
  uint32_t d;       // slot float index of element e0-1
  uint32_t has_seg;
};

// ---------------------------------------------------------------------------
// Persistent, warp-specialised pipeline (blockSize L = 8*LPB; fastmode1, and
// fastmode2 with its per-block seeds).
//
// A CTA works through tiles until the tickets run out.  Warp roles:
//   compute  (warps 0-7)  quantize, delta, sign and bit-count analysis, a
//                         scan of each warp's block sizes in registers, one
//                         barrier for the warps' totals, then packing of the
//                         blocks into the tile's slot from offset 0.  They
//                         never wait for the tile's stream offset.
//   control  (kPipeControl warps, tiles round robin)  decoupled look-back for
//                         the stream offset, then a shifted copy of the packed
//                         slot to the stream with 16-byte stores.
//   producer (1 warp)     draws tile tickets and fills free slots with the
//                         tiles' input windows by bulk copy (TMA).
// kPipeSlots shared-memory slots cycle through four mbarriers each: full
// (producer -> compute, control), agg (tile byte count known), packed
// (every compute warp -> control) and empty (control -> producer).  Tickets are drawn in
// order and every wait depends only on lower tickets or earlier stages of the
// same tile, so the pipeline cannot deadlock; every wait is bounded.
// ---------------------------------------------------------------------------
constexpr int kPipeSlots = 3, kPipeControl = 2;
constexpr int kPipeThreads = (8 + kPipeControl + 1) * 32;

// What the compute and control warps need of a slot's tile, written by the
// producer before the slot's full barrier completes.
struct SlotMeta {
  TileGeo g;
  uint32_t tile;       // launch tile (its look-back word); kStopTile: no more tiles
  uint32_t ltile;      // tile within its field
  uint32_t tile_base;  // the field's first launch tile
  uint32_t ntiles;     // tiles of the field
  float eb, inv;       // the field's bound and 1/bound
  Segments seg;        // the field's segments
  uint8_t* out;        // the field's stream
  uint64_t cap;
  uint64_t* out_size;
  uint32_t* err;       // the field's error word
};

// Producer: one thread.  Draws tickets, and for each tile computes its
// geometry and bulk-copies its input window [e0-1, e0+nel) into a free slot
// (element e at slot float e - (e0-1) + d).
template <uint32_t L, uint32_t TB, int NS, bool BATCH, bool FM2>
__device__ __forceinline__ void pipe_producer(const CompressArgs& a, uint8_t* slots, uint32_t slot_bytes,
                                              SlotMeta* meta, uint64_t* full, uint64_t* empty,
                                              uint32_t* s_epoch, volatile uint32_t* s_stop_k, const volatile uint32_t* s_started) {
  *s_epoch = *(volatile uint32_t*)&a.ls->epoch;
  __threadfence();
  CompressField f1;  // the single field of a non-batched launch
  if (!BATCH) {
    f1.x = a.x;
    f1.out = a.out;
    f1.cap = a.cap;
    f1.seg = a.seg;
    f1.nb_reg = a.nb_reg;
    f1.nb_last = a.nb_last;
    f1.tiles_per_seg = a.tiles_per_seg;
    f1.ntiles = a.ntiles;
    f1.tile_base = 0;
    f1.eb = a.eb_dev ? *a.eb_dev : a.eb;
    f1.out_size = a.out_size;
    f1.err = a.err;
  }
  const float inv1 = BATCH ? 0.0f : __fdiv_rn(1.0f, f1.eb);
  for (uint32_t k = 0;; k++) {
    const int s = (int)(k % NS);
    if (k >= (uint32_t)NS) mbar_wait_or_flag(&empty[s], ((k / NS) - 1) & 1, a.err);
    // draw the ticket only once the compute warps have started the previous
    // position: a tile's predecessors are then never more than a tile behind it
    // in their work, which keeps the look-back short
    for (uint32_t i = 0; i < kWaitLimit && *s_started < k; i++) __nanosleep(64);
    const uint32_t tile = draw_ticket_persistent(a.ls, a.ntiles);
    SlotMeta& m = meta[s];
    if (tile >= a.ntiles) {
      drain_copies<NS>(full, k);
      m.tile = kStopTile;
      *s_stop_k = k;
      mbar_arrive(&full[s]);
      return;
    }
    const CompressField& fd = BATCH ? a.fields[a.tile_field[tile]] : f1;
    const Segments sg = fd.seg;
    const uint32_t lt = tile - fd.tile_base;
    m.ltile = lt;
    m.tile_base = fd.tile_base;
    m.ntiles = fd.ntiles;
    m.eb = fd.eb;
    m.inv = BATCH ? __fdiv_rn(1.0f, fd.eb) : inv1;
    m.seg = sg;
    m.out = fd.out;
    m.cap = fd.cap;
    m.out_size = fd.out_size;
    m.err = fd.err;
    float* sx = reinterpret_cast<float*>(slots + (size_t)s * slot_bytes);
    TileGeo g;
    g.has_seg = sg.n > 0;
    uint32_t t = sg.T - 1, ts = lt;
    if (fd.tiles_per_seg) {
      t = lt / fd.tiles_per_seg;
      if (t > sg.T - 1) t = sg.T - 1;
      ts = lt - t * fd.tiles_per_seg;
    }
    g.seg = t;
    g.lo = (uint64_t)t * sg.tsz;
    g.hi = t + 1 == sg.T ? sg.n : g.lo + sg.tsz;
    const uint64_t nb = t + 1 == sg.T ? fd.nb_last : fd.nb_reg;
    const uint64_t blk0 = (uint64_t)ts * TB;
    g.nblk = nb > blk0 ? (uint32_t)min((uint64_t)TB, nb - blk0) : 0u;
    g.first = ts == 0;
    // fastmode1: blocks start after the segment's seed, the window starts one
    // element before block 0; fastmode2: block b starts at lo + bL with its own
    // seed, the window starts at block 0's seed.  Either way the data element j
    // of block b lies at window index 1 + bL + j.
    g.e0 = FM2 ? g.lo + blk0 * L : g.lo + 1 + blk0 * L;
    g.nel = g.nblk ? (uint32_t)min((uint64_t)g.nblk * L, g.hi - g.e0) : 0u;
    g.d = 0;
    uint32_t bytes = 0;
    uintptr_t b0 = 0, a0 = 0;
    if (g.has_seg && (g.nblk || (!FM2 && g.first && g.hi > g.lo))) {  // a lone seed still needs x[lo]
      const uintptr_t xa = (uintptr_t)fd.x;
      const uintptr_t w0 = xa + 4 * (FM2 ? g.e0 : g.e0 - 1), w1 = xa + 4 * (g.e0 + g.nel);
      a0 = w0 & ~(uintptr_t)15;
      g.d = (uint32_t)((w0 - a0) >> 2);
      b0 = max(a0, (xa + 15) & ~(uintptr_t)15);
      const uintptr_t b1 = min((w1 + 15) & ~(uintptr_t)15, (xa + 4 * sg.n) & ~(uintptr_t)15);
      if (b1 > b0) {
        bytes = (uint32_t)(b1 - b0);
        for (uintptr_t p = w0; p < b0; p += 4) sx[(p - a0) >> 2] = __ldg(reinterpret_cast<const float*>(p));
        for (uintptr_t p = max(b1, w0); p < w1; p += 4) sx[(p - a0) >> 2] = __ldg(reinterpret_cast<const float*>(p));
      } else {
        for (uintptr_t p = w0; p < w1; p += 4) sx[(p - a0) >> 2] = __ldg(reinterpret_cast<const float*>(p));
      }
    }
    m.g = g;
    m.tile = tile;
    if (bytes) {
      fence_async_smem();
      mbar_arrive_expect_tx(&full[s], bytes);
      bulk_load(reinterpret_cast<uint8_t*>(sx) + (b0 - a0), reinterpret_cast<const void*>(b0), bytes, &full[s]);
    } else {
      mbar_arrive(&full[s]);
    }
  }
}

// Control warp c: tiles c, c + kPipeControl, ... of this CTA.
template <int NS, int NC, bool QI = false>
__device__ __forceinline__ void pipe_control(int c, const CompressArgs& a, const uint8_t* slots,
                                             uint32_t slot_bytes, const SlotMeta* meta, const uint32_t* s_agg,
                                             uint64_t* full, uint64_t* aggb, uint64_t* packed, uint64_t* empty,
                                             const uint32_t* s_epoch, const volatile uint32_t* s_stop_k) {
  const int lane = threadIdx.x & 31;
  for (uint32_t k = (uint32_t)c;; k += NC) {
    const int s = (int)(k % NS);
    const uint32_t par = (k / NS) & 1;
    if (!control_wait_full(&full[s], par, k, s_stop_k, a.err)) return;
    const SlotMeta& m = meta[s];
    const uint32_t tile = m.tile;
    if (tile >= a.ntiles) return;
    const uint32_t seg = m.g.seg, lt = m.ltile;
    const bool first_of_seg = m.g.has_seg && m.g.first;
    uint8_t* out = m.out;
    const uint64_t cap = m.cap;
    mbar_wait_or_flag(&aggb[s], par, a.err);
    const uint32_t agg = s_agg[s];
    const uint32_t epoch = *s_epoch;
    uint64_t excl = 0;
    const uint32_t HB = QI ? a.qhb : 4;  // eb header bytes: float64 streams carry a double
    if (lt == 0) {
      if (QI && HB == 8) {
        write_header_warp(out, a.ebd_dev ? *a.ebd_dev : a.ebd, m.seg, lane);
      } else {
        write_header_warp(out, m.eb, m.seg, lane);
      }
    } else {
      excl = lookback_sum(a.status, tile, m.tile_base, epoch, a.err);
      if (lane == 0) st_relaxed_u64(a.status + tile, make_status(epoch, kFlagInclusive, excl + agg));
    }
    const uint64_t gpos = HB + 8ull * m.seg.T + excl;
    const bool fits = gpos + agg <= cap;
    if (lane == 0) {
      if (lt == m.ntiles - 1) *m.out_size = gpos + agg;
      if (first_of_seg && fits) write_offset(out, seg, excl, HB);
      if (!fits) atomicOr(m.err, kErrCapacity);
    }
    mbar_wait_or_flag(&packed[s], par, a.err);
    if (fits) warp_store_span(out + gpos, slots + (size_t)s * slot_bytes, agg, lane);
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
}

// QI: the input is int32 codes (four bytes per element like a float): float64
// data already quantized, or summed codes of the homomorphic reduction;
// a.qhb gives the stream's eb header width.
template <int LPB, bool BATCH, int ROUNDS, bool FM2 = false, bool QI = false>
__global__ void __launch_bounds__(kPipeThreads, 2) compress_pipe(const __grid_constant__ CompressArgs a,
                                                                 uint32_t slot_bytes) {
  constexpr int NS = kPipeSlots, NC = kPipeControl;
  // a control warp's next position must never share a slot phase it has not
  // waited for (an mbarrier parity names one of two phases)
  static_assert(NC <= NS, "more control warps than slots");
  constexpr uint32_t L = 8 * LPB;
  constexpr int BPR = 32 / LPB;
  constexpr uint32_t TB = 8 * ROUNDS * BPR;
  extern __shared__ __align__(16) uint8_t s_slots[];
  __shared__ SlotMeta s_meta[NS];
  __shared__ uint32_t s_agg[NS];
  __shared__ uint32_t s_wtot[2][8];  // compute warps' packed bytes, by tile parity
  __shared__ uint32_t s_thr[36];
  __shared__ uint32_t s_epoch;
  __shared__ volatile uint32_t s_stop_k;
  __shared__ volatile uint32_t s_started;
  __shared__ __align__(8) uint64_t s_full[NS], s_aggb[NS], s_packed[NS], s_empty[NS];

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x < 36) s_thr[threadIdx.x] = a.thr.thr[threadIdx.x];
  if (threadIdx.x < NS) s_meta[threadIdx.x].tile = kStopTile;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; s++) {
      mbar_init(&s_full[s], 1);
      mbar_init(&s_aggb[s], 1);
      mbar_init(&s_packed[s], 8);  // one arrival per compute warp
      mbar_init(&s_empty[s], 1);
    }
    s_stop_k = kStopTile;
    s_started = 0;
  }
  __syncthreads();

  if (warp == 8 + NC) {
    if (lane == 0)
      pipe_producer<L, TB, NS, BATCH, FM2>(a, s_slots, slot_bytes, s_meta, s_full, s_empty, &s_epoch, &s_stop_k,
                                           &s_started);
    return;
  }
  if (warp >= 8) {
    pipe_control<NS, NC, QI>(warp - 8, a, s_slots, slot_bytes, s_meta, s_agg, s_full, s_aggb, s_packed, s_empty,
                             &s_epoch, &s_stop_k);
    return;
  }

  // ---- compute warps ----
  const int sub = lane % LPB, grp = lane / LPB;
  for (uint32_t k = 0;; k++) {
    const int s = (int)(k % NS);
    const uint32_t par = (k / NS) & 1;
    mbar_wait_or_flag(&s_full[s], par, a.err);
    const uint32_t tile = s_meta[s].tile;
    if (threadIdx.x == 0) s_started = k + 1;
    if (tile >= a.ntiles) return;
    const TileGeo g = s_meta[s].g;
    const float inv = s_meta[s].inv;
    uint8_t* slot = s_slots + (size_t)s * slot_bytes;
    const float* sx = reinterpret_cast<const float*>(slot);
    const bool seed = !FM2 && g.has_seg && g.first && g.hi > g.lo;  // the segment's seed (fastmode1)
    int32_t seedv = 0;
    uint32_t flags = 0;
    if (seed && threadIdx.x == 0)  // x[lo] = window element 0
      seedv = QI ? __float_as_int(sx[g.d]) : quantize(sx[g.d], inv, flags);

    // ---- analysis: q, deltas, signs, block max, bit count, block size ----
    uint32_t vv[ROUNDS][8];
    uint32_t sgnb[ROUNDS];
    uint32_t rinfo[ROUNDS];  // the lane's block: bit count, then (after the scan) its offset in the warp's run * 64
    int32_t bseed[ROUNDS];  // fastmode2: each block's seed, in its first lane
    const uint32_t sh = 1 + g.d;  // slot index of tile element 0
    const uint32_t ph = sh & 3;   // its 16-byte phase (same for every lane: L % 8 == 0)
    // every lane of every round holds 8 elements (never in fastmode2: a block has L-1 deltas)
    const bool full = !FM2 && g.nblk == TB && g.nel == TB * L;
    // All rounds run on the fast quantization (exact while |x/eb| < 2^24); if
    // any lane met a larger value the whole tile is redone on the exact path,
    // so the common case has no per-round branch.
    auto analyse = [&](auto exact_tag) -> bool {
      constexpr bool EXACT = decltype(exact_tag)::value;
      bool slow = false;
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
      const uint32_t bt = (warp * ROUNDS + r) * BPR + grp;
      const uint32_t k0 = bt * L + 8 * sub;  // tile-relative first element of the lane
      uint32_t ml;                          // elements (deltas) of the lane
      if (FM2) {
        const uint32_t mblk = bt < g.nblk ? min(L, g.nel - bt * L) : 0u;
        const uint32_t md = mblk ? mblk - 1 : 0u;
        ml = md > 8u * sub ? min(8u, md - 8u * sub) : 0u;
      } else {
        ml = (bt < g.nblk && k0 < g.nel) ? min(8u, g.nel - k0) : 0u;
      }
      float xv[8];
      const uint32_t i = sh + k0;
      if (full) {
        const float4* q4 = reinterpret_cast<const float4*>(sx + (i & ~3u));
        const float4 A = q4[0], B = q4[1];
        if (ph == 0) {
          xv[0] = A.x; xv[1] = A.y; xv[2] = A.z; xv[3] = A.w; xv[4] = B.x; xv[5] = B.y; xv[6] = B.z; xv[7] = B.w;
        } else {
          const float4 C = q4[2];
          if (ph == 1) {
            xv[0] = A.y; xv[1] = A.z; xv[2] = A.w; xv[3] = B.x; xv[4] = B.y; xv[5] = B.z; xv[6] = B.w; xv[7] = C.x;
          } else if (ph == 2) {
            xv[0] = A.z; xv[1] = A.w; xv[2] = B.x; xv[3] = B.y; xv[4] = B.z; xv[5] = B.w; xv[6] = C.x; xv[7] = C.y;
          } else {
            xv[0] = A.w; xv[1] = B.x; xv[2] = B.y; xv[3] = B.z; xv[4] = B.w; xv[5] = C.x; xv[6] = C.y; xv[7] = C.z;
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < 8; j++) xv[j] = (uint32_t)j < ml ? sx[i + j] : 0.0f;
      }
      int32_t q[8];
      if (QI) {
#pragma unroll
        for (int j = 0; j < 8; j++) q[j] = __float_as_int(xv[j]);
      } else if (EXACT) {
#pragma unroll
        for (int j = 0; j < 8; j++) q[j] = quantize_lean(xv[j], inv, flags);
      } else {
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const float pj = __fmul_rz(xv[j], inv);
          q[j] = __float2int_rz(pj);
          slow |= !(fabsf(pj) < 16777216.0f);
        }
      }
      int32_t prev = __shfl_up_sync(0xffffffffu, q[7], 1);
      if (FM2 ? sub == 0 : lane == 0) {  // the element before the lane's first: fastmode2 the block's seed
        const float xp = bt < g.nblk ? sx[i - 1] : 0.0f;  // past the tile's blocks the slot holds no input
        if (QI) {
          prev = __float_as_int(xp);
        } else if (EXACT) {
          prev = quantize_lean(xp, inv, flags);
        } else {
          const float pp = __fmul_rz(xp, inv);
          prev = __float2int_rz(pp);
          slow |= !(fabsf(pp) < 16777216.0f);
        }
      }
      bseed[r] = prev;
      uint32_t sb = 0, lmax = 0;
      if (full) {
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int32_t d = (int32_t)((uint32_t)q[j] - (uint32_t)prev);  // wrapping, as the compiled reference
          prev = q[j];
          const uint32_t v = (uint32_t)abs(d);  // |INT_MIN| is 2^31 as in the reference
          sb = (sb << 1) + ((uint32_t)d >> 31);
          lmax = max(lmax, v);
          vv[r][j] = v;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int32_t d = (int32_t)((uint32_t)q[j] - (uint32_t)prev);
          prev = q[j];
          const bool valid = (uint32_t)j < ml;
          const uint32_t v = valid ? (uint32_t)abs(d) : 0u;
          sb = (sb << 1) + (valid ? ((uint32_t)d >> 31) : 0u);
          lmax = max(lmax, v);
          vv[r][j] = v;
        }
      }
      sgnb[r] = sb;
#pragma unroll
      for (int o = 1; o < LPB; o <<= 1) lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
      // every lane of the block holds its bit count and size
      uint32_t bc = 0;
      if (lmax) {
        const int kk = 32 - __clz(lmax);
        bc = kk + (kk >= 21 && lmax >= s_thr[kk + 1] ? 1 : 0);
      }
      rinfo[r] = bc;
    }
      return slow;
    };
    if (__any_sync(0xffffffffu, analyse(std::false_type{}))) analyse(std::true_type{});
    if (__any_sync(0xffffffffu, flags != 0) && lane == 0) atomicOr(s_meta[s].err, kErrQuantRange);

    // ---- block offsets: a scan of the warp's block sizes over its lane
    // groups and rounds, then one barrier for the warps' totals (which also
    // ends every read of the input window) ----
    uint32_t wrun = 0;
    {
      uint32_t incl[ROUNDS], bsz[ROUNDS];
#pragma unroll
      for (int r = 0; r < ROUNDS; r++) {
        const uint32_t bt = (warp * ROUNDS + r) * BPR + grp;
        const uint32_t m = bt < g.nblk ? min(L, g.nel - bt * L) : 0u;
        const uint32_t bc = rinfo[r];
        bsz[r] = m ? (FM2 ? 4 + block_bytes(m - 1, bc) : block_bytes(m, bc)) : 0u;  // fastmode2: seed, L-1 deltas
        incl[r] = bsz[r];
      }
#pragma unroll
      for (int o = LPB; o < 32; o <<= 1) {
#pragma unroll
        for (int r = 0; r < ROUNDS; r++) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, incl[r], o);
          if (lane >= o) incl[r] += y;
        }
      }
#pragma unroll
      for (int r = 0; r < ROUNDS; r++) {
        rinfo[r] |= (wrun + incl[r] - bsz[r]) << 6;
        wrun += __shfl_sync(0xffffffffu, incl[r], 31);
      }
    }
    uint32_t* wtot = s_wtot[k & 1];  // alternate: a fast warp's next tile never meets a slow warp's reads
    if (lane == 0) wtot[warp] = wrun;
    compute_sync();
    const uint32_t front = seed ? 4u : 0u;
    uint32_t wexcl = front, agg = front;
#pragma unroll
    for (int w = 0; w < 8; w++) {
      const uint32_t t = wtot[w];
      wexcl += w < warp ? t : 0u;
      agg += t;
    }
    if (threadIdx.x == 0) {
      s_agg[s] = agg;
      const bool head = s_meta[s].ltile == 0;  // a field's first tile has no predecessor
      st_relaxed_u64(a.status + tile, make_status(s_epoch, head ? kFlagInclusive : kFlagAggregate, agg));
      mbar_arrive(&s_aggb[s]);
    }

    // ---- pack into the slot from offset 0 ----
    uint8_t* s_tile = slot;
    if (seed && threadIdx.x == 0) {
      s_tile[0] = (uint8_t)seedv;
      s_tile[1] = (uint8_t)((uint32_t)seedv >> 8);
      s_tile[2] = (uint8_t)((uint32_t)seedv >> 16);
      s_tile[3] = (uint8_t)((uint32_t)seedv >> 24);
    }
    if (full) {
#pragma unroll
      for (int r = 0; r < ROUNDS; r++) {
        const uint32_t bc = rinfo[r] & 63;
        uint8_t* dst = s_tile + wexcl + (rinfo[r] >> 6);
        if (sub == 0) dst[0] = (uint8_t)bc;
        const uint32_t B = bc >> 3, rr = bc & 7;
        constexpr uint32_t ns = L / 8;
        if (bc) dst[1 + sub] = (uint8_t)sgnb[r];
        if (__all_sync(0xffffffffu, B <= 1)) {
          if (B) {
            uint8_t* q8 = dst + 1 + ns + 8 * sub;
#pragma unroll
            for (int j = 0; j < 8; j++) q8[j] = (uint8_t)(vv[r][j] >> rr);
          }
        } else if (B) {
          uint8_t* q8 = dst + 1 + ns + 8 * B * sub;
#pragma unroll
          for (int j = 0; j < 8; j++) {
            const uint32_t h = vv[r][j] >> rr;
            q8[j * B] = (uint8_t)h;
            if (B > 1) q8[j * B + 1] = (uint8_t)(h >> 8);
            if (B > 2) q8[j * B + 2] = (uint8_t)(h >> 16);
            if (B > 3) q8[j * B + 3] = (uint8_t)(h >> 24);
          }
        }
        if (rr) {
          const uint32_t mask = (1u << rr) - 1u;
          uint32_t hi4 = 0, lo4 = 0;
#pragma unroll
          for (int j = 0; j < 4; j++) hi4 = (hi4 << rr) | (vv[r][j] & mask);
#pragma unroll
          for (int j = 4; j < 8; j++) lo4 = (lo4 << rr) | (vv[r][j] & mask);
          // 8*rr bits, element 0 first, moved to the top of 64 bits
          const uint64_t top = (((uint64_t)hi4 << (4 * rr)) | lo4) << (64 - 8 * rr);
          const uint32_t th = (uint32_t)(top >> 32), tl = (uint32_t)top;
          uint8_t* rp = dst + 1 + ns + B * L + rr * sub;
          rp[0] = (uint8_t)(th >> 24);
          if (rr > 1) rp[1] = (uint8_t)(th >> 16);
          if (rr > 2) rp[2] = (uint8_t)(th >> 8);
          if (rr > 3) rp[3] = (uint8_t)th;
          if (rr > 4) rp[4] = (uint8_t)(tl >> 24);
          if (rr > 5) rp[5] = (uint8_t)(tl >> 16);
          if (rr > 6) rp[6] = (uint8_t)(tl >> 8);
        }
      }
    } else {
#pragma unroll
      for (int r = 0; r < ROUNDS; r++) {
        const uint32_t bt = (warp * ROUNDS + r) * BPR + grp;
        if (bt >= g.nblk) continue;
        const uint32_t mblk = min(L, g.nel - bt * L);
        const uint32_t m = FM2 ? mblk - 1 : mblk;  // values packed in the block
        const uint32_t ml = m > 8u * sub ? min(8u, m - 8u * sub) : 0u;
        const uint32_t bc = rinfo[r] & 63;
        uint8_t* dst = s_tile + wexcl + (rinfo[r] >> 6);
        if (FM2) {
          if (sub == 0) {  // the block's seed, szp_float.cc:812-864
            dst[0] = (uint8_t)bseed[r];
            dst[1] = (uint8_t)((uint32_t)bseed[r] >> 8);
            dst[2] = (uint8_t)((uint32_t)bseed[r] >> 16);
            dst[3] = (uint8_t)((uint32_t)bseed[r] >> 24);
          }
          dst += 4;
        }
        if (sub == 0) dst[0] = (uint8_t)bc;
        if (bc == 0 || ml == 0) continue;
        const uint32_t ns = (m + 7) >> 3, B = bc >> 3, rr = bc & 7;
        dst[1 + sub] = (uint8_t)sgnb[r];  // sign bits, szp_TypeManager.cc:820-844
        if (B) {  // byte planes, szp_TypeManager.cc:36-52
          uint8_t* q8 = dst + 1 + ns + 8 * B * sub;
#pragma unroll
          for (int j = 0; j < 8; j++) {
            if ((uint32_t)j < ml) {
              const uint32_t h = vv[r][j] >> rr;
              q8[j * B] = (uint8_t)h;
              if (B > 1) q8[j * B + 1] = (uint8_t)(h >> 8);
              if (B > 2) q8[j * B + 2] = (uint8_t)(h >> 16);
              if (B > 3) q8[j * B + 3] = (uint8_t)(h >> 24);
            }
          }
        }
        if (rr) {  // remainder bits, MSB first, szp_TypeManager.cc:122-434
          const uint32_t mask = (1u << rr) - 1u;
          uint32_t hi4 = 0, lo4 = 0;  // elements 0-3 and 4-7, 4*rr bits each
#pragma unroll
          for (int j = 0; j < 4; j++) hi4 = (hi4 << rr) | ((uint32_t)j < ml ? (vv[r][j] & mask) : 0u);
#pragma unroll
          for (int j = 4; j < 8; j++) lo4 = (lo4 << rr) | ((uint32_t)j < ml ? (vv[r][j] & mask) : 0u);
          const uint64_t acc = ((uint64_t)hi4 << (4 * rr)) | lo4;  // 8*rr bits, element 0 on top
          uint8_t* rp = dst + 1 + ns + B * m + rr * sub;
          const uint32_t nb = (ml * rr + 7) >> 3;
          const uint32_t top = 8 * rr - 8;
#pragma unroll
          for (uint32_t kk = 0; kk < 7; kk++)
            if (kk < nb) rp[kk] = (uint8_t)(acc >> (top - 8 * kk));
        }
      }
    }
    // fastmode1 tiles measured faster with the compute warps kept in step by
    // an end-of-tile barrier, fastmode2 tiles without it
    if (FM2) {
      __syncwarp();
    } else {
      compute_sync();
    }
    if (lane == 0) mbar_arrive(&s_packed[s]);  // the warp's part of the slot is packed
  }
}

// ---------------------------------------------------------------------------
// Any blockSize: one warp per block, the block walked in 32-element pieces.
// Pieces start on byte boundaries in every section (32 signs = 4 bytes,
// 32*B bytes, 32*r bits = 4r bytes), so each piece packs like a 32-block.
// fastmode2 (FM2) gives every block its own seed and L-1 deltas.
// ---------------------------------------------------------------------------
// V = float, or double for float64 data (szp_double.cc: 8-byte eb header,
// q = (int)(x * (1/eb)) with a double product).
template <int WARPS, bool FM2, typename V = float>
__global__ void __launch_bounds__(WARPS * 32) compress_generic(CompressArgs a) {
  constexpr bool DBL = std::is_same<V, double>::value;
  constexpr uint32_t HB = DBL ? 8 : 4;  // eb header bytes
  extern __shared__ __align__(16) uint8_t s_out[];
  __shared__ uint32_t s_tk[2];
  __shared__ uint32_t s_w[WARPS + 1];
  __shared__ uint64_t s_base;

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t tile, epoch;
  draw_ticket(a.ls, a.ntiles, tile, epoch, s_tk);

  const Segments sg = a.seg;
  const uint32_t L = sg.L;
  uint32_t flags = 0;
  const uint32_t TB = WARPS * a.bpw;
  // float64 values are loaded as their bits (see f64_key)
  using LT = typename std::conditional<DBL, unsigned long long, float>::type;
  const LT* __restrict__ xs = DBL ? reinterpret_cast<const LT*>(a.xd) : reinterpret_cast<const LT*>(a.x);
  V eb, inv;
  if constexpr (DBL) {
    eb = a.ebd_dev ? *a.ebd_dev : a.ebd;
    inv = a.invd_dev ? *a.invd_dev : a.invd;  // 1/eb in double, szp_double.cc:180
  } else {
    eb = a.eb_dev ? *a.eb_dev : a.eb;
    inv = __fdiv_rn(1.0f, eb);
  }
  f64i::Inverse invo{};  // 1/eb's fields for the integer float64 quantizer
  if constexpr (DBL) invo = f64i::prepare_inverse(f64i::bits_of(inv));
  auto qz = [&](LT v) -> int32_t {
    if constexpr (DBL) {
      bool bad = false;
      const int32_t q = f64i::quantize_fast(v, invo, bad);
      if (bad) flags |= kErrQuantRange;
      return q;
    } else {
      return quantize(v, inv, flags);
    }
  };
  const TileInfo ti = tile_info(sg, tile, a.tiles_per_seg, TB, FM2);
  if (tile == 0) write_header_common(a.out, eb, sg);
  const uint64_t lo = sg.lo(ti.seg), hi = sg.hi(ti.seg);

  // block b of the segment: fastmode1 elements [lo+1+bL, ...), previous
  // element lo+bL; fastmode2 seed at lo+bL and deltas after it.
  auto block_start = [&](uint64_t b) -> uint64_t { return FM2 ? lo + b * L + 1 : lo + 1 + b * L; };
  auto block_len = [&](uint64_t b) -> uint32_t {
    uint64_t s = block_start(b);
    uint64_t end = s + L;
    if (FM2) end -= 1;
    if (end > hi) end = hi;
    return end > s ? (uint32_t)(end - s) : 0;
  };
  const uint32_t per_blk_extra = FM2 ? 4u : 0u;  // fastmode2 seed

  // pass 1: bit counts and sizes.  With blockSize <= 32 (one piece per block)
  // and at most KC blocks per warp, the warp loads all its values at once,
  // lane c quantizes the value before block c (its seed in fastmode2), and
  // every lane keeps its quantized value and the blocks' bit counts in
  // registers, so pass 2 loads and quantizes nothing again.
  constexpr int KC = 8;
  const bool cache = L <= 32 && a.bpw <= (uint32_t)KC;
  int32_t cq[KC];
  uint32_t cbc[KC];
  int32_t pq = 0;  // lane c: the quantized value before block c
  uint32_t wbytes = 0;
  const uint32_t wfirst = warp * a.bpw;
#pragma unroll
  for (int k = 0; k < KC; k++) {
    cq[k] = 0;
    cbc[k] = 0;
  }
  if (cache) {
    LT xv[KC];
    LT xp = LT(0);
#pragma unroll
    for (int c = 0; c < KC; c++) {
      xv[c] = LT(0);
      const uint32_t bi = wfirst + c;
      if ((uint32_t)c < a.bpw && bi < ti.nblk && (uint32_t)lane < block_len(ti.blk0 + bi))
        xv[c] = __ldg(xs + block_start(ti.blk0 + bi) + lane);
    }
    if ((uint32_t)lane < a.bpw && wfirst + lane < ti.nblk) xp = __ldg(xs + block_start(ti.blk0 + wfirst + lane) - 1);
    pq = qz(xp);
#pragma unroll
    for (int c = 0; c < KC; c++) {
      const uint32_t bi = wfirst + c;
      if ((uint32_t)c >= a.bpw || bi >= ti.nblk) break;
      const uint32_t m = block_len(ti.blk0 + bi);
      const bool valid = (uint32_t)lane < m;
      const int32_t q = valid ? qz(xv[c]) : 0;
      int32_t qp = __shfl_up_sync(0xffffffffu, q, 1);
      const int32_t p0 = __shfl_sync(0xffffffffu, pq, c);
      if (lane == 0) qp = p0;
      const uint32_t d = (uint32_t)q - (uint32_t)qp;
      const uint32_t v = valid ? (((int32_t)d < 0) ? 0u - d : d) : 0u;
      const uint32_t bc = bitcount_from_table(__reduce_max_sync(0xffffffffu, v), a.thr.thr);
      wbytes += per_blk_extra + (m ? block_bytes(m, bc) : 1u);
      cq[c] = q;
      cbc[c] = bc;
    }
  }
  for (uint32_t k = 0; !cache && k < a.bpw; k++) {
    uint32_t bi = wfirst + k;
    if (bi >= ti.nblk) break;
    uint64_t b = ti.blk0 + bi;
    uint64_t s = block_start(b);
    uint32_t m = block_len(b);
    uint32_t mx = 0;
    int32_t prev = qz(__ldg(xs + s - 1));
    for (uint32_t p0 = 0; p0 < m; p0 += 32) {
      uint32_t j = p0 + lane;
      bool valid = j < m;
      int32_t q = valid ? qz(__ldg(xs + s + j)) : 0;
      int32_t qp = __shfl_up_sync(0xffffffffu, q, 1);
      if (lane == 0) qp = prev;
      prev = __shfl_sync(0xffffffffu, q, 31);
      uint32_t d = (uint32_t)q - (uint32_t)qp;
      uint32_t v = valid ? (((int32_t)d < 0) ? 0u - d : d) : 0u;
      mx = max(mx, __reduce_max_sync(0xffffffffu, v));
    }
    uint32_t bc = bitcount_from_table(mx, a.thr.thr);
    wbytes += per_blk_extra + (m ? block_bytes(m, bc) : 1u);
  }
  if (__any_sync(0xffffffffu, flags != 0) && lane == 0) atomicOr(a.err, kErrQuantRange);

  const bool seed = !FM2 && ti.has_seg && ti.first && hi > lo;
  uint32_t wexcl;
  const uint32_t agg = scan_warps<WARPS>(s_w, wbytes, warp, lane, wexcl, seed ? 4u : 0u);

  if (warp == 0) {
    uint64_t excl = 0;
    if (tile == 0) {
      if (lane == 0) st_relaxed_u64(a.status + tile, make_status(epoch, kFlagInclusive, agg));
    } else {
      if (lane == 0) st_relaxed_u64(a.status + tile, make_status(epoch, kFlagAggregate, agg));
      excl = lookback_sum(a.status, tile, 0, epoch, a.err);
      if (lane == 0) st_relaxed_u64(a.status + tile, make_status(epoch, kFlagInclusive, excl + agg));
    }
    if (lane == 0) s_base = excl;
  }
  __syncthreads();
  const uint64_t base = s_base;
  const uint64_t head = HB + 8ull * sg.T;
  const uint64_t gpos = head + base;
  if (tile == a.ntiles - 1 && threadIdx.x == 0) *a.out_size = gpos + agg;
  if (ti.has_seg && ti.first && threadIdx.x == 0 && gpos + agg <= a.cap) write_offset(a.out, ti.seg, base, HB);
  if (gpos + agg > a.cap) {
    if (threadIdx.x == 0) atomicOr(a.err, kErrCapacity);
    return;
  }

  const uint32_t align = (uint32_t)(((uintptr_t)a.out + gpos) & 15);
  uint8_t* s_tile = s_out + align;
  if (seed && warp == 0) {
    int32_t sq = qz(__ldg(xs + lo));
    if (lane < 4) s_tile[lane] = (uint8_t)((uint32_t)sq >> (8 * lane));
  }

  // pass 2: recompute and pack piece by piece
  uint32_t off = wexcl;
  for (uint32_t k = 0; k < a.bpw; k++) {
    uint32_t bi = wfirst + k;
    if (bi >= ti.nblk) break;
    uint64_t b = ti.blk0 + bi;
    uint64_t s = block_start(b);
    uint32_t m = block_len(b);
    uint8_t* dst = s_tile + off;
    int32_t kq = 0;
    uint32_t kbc = 0;
    const int32_t kprev = __shfl_sync(0xffffffffu, pq, k & 31);
    if (cache) {
#pragma unroll
      for (int c = 0; c < KC; c++)
        if ((uint32_t)c == k) {
          kq = cq[c];
          kbc = cbc[c];
        }
    }
    if (FM2) {
      int32_t sq = cache ? kprev : qz(__ldg(xs + s - 1));
      if (lane < 4) dst[lane] = (uint8_t)((uint32_t)sq >> (8 * lane));
      dst += 4;
    }
    // without the cache: recompute the max (L1-resident) to know the bit count
    uint32_t mx = 0;
    if (!cache) {
      int32_t prev = qz(__ldg(xs + s - 1));
      for (uint32_t p0 = 0; p0 < m; p0 += 32) {
        uint32_t j = p0 + lane;
        bool valid = j < m;
        int32_t q = valid ? qz(__ldg(xs + s + j)) : 0;
        int32_t qp = __shfl_up_sync(0xffffffffu, q, 1);
        if (lane == 0) qp = prev;
        prev = __shfl_sync(0xffffffffu, q, 31);
        uint32_t d = (uint32_t)q - (uint32_t)qp;
        uint32_t v = valid ? (((int32_t)d < 0) ? 0u - d : d) : 0u;
        mx = max(mx, __reduce_max_sync(0xffffffffu, v));
      }
    }
    const uint32_t bc = cache ? kbc : bitcount_from_table(mx, a.thr.thr);
    if (lane == 0) dst[0] = (uint8_t)bc;
    if (m == 0 || bc == 0) {
      off += per_blk_extra + 1;
      continue;
    }
    const uint32_t ns = (m + 7) >> 3, B = bc >> 3, r = bc & 7;
    uint8_t* sgnp = dst + 1;
    uint8_t* bytp = sgnp + ns;
    uint8_t* remp = bytp + B * m;
    int32_t prev = cache ? kprev : qz(__ldg(xs + s - 1));
    for (uint32_t p0 = 0; p0 < m; p0 += 32) {
      uint32_t j = p0 + lane;
      bool valid = j < m;
      uint32_t pm = m - p0 < 32 ? m - p0 : 32;  // elements in this piece
      int32_t q = cache ? kq : (valid ? qz(__ldg(xs + s + j)) : 0);
      int32_t qp = __shfl_up_sync(0xffffffffu, q, 1);
      if (lane == 0) qp = prev;
      prev = __shfl_sync(0xffffffffu, q, 31);
      uint32_t d = (uint32_t)q - (uint32_t)qp;
      bool neg = valid && (int32_t)d < 0;
      uint32_t v = valid ? (neg ? 0u - d : d) : 0u;
      uint32_t sign = __ballot_sync(0xffffffffu, neg);
      uint32_t pns = (pm + 7) >> 3;
      if ((uint32_t)lane < pns) sgnp[(p0 >> 3) + lane] = (uint8_t)(__brev(sign) >> (24 - 8 * lane));
      if (B && valid) {
        uint32_t h = v >> r;
        uint8_t* q8 = bytp + (uint64_t)j * B;
        for (uint32_t t = 0; t < B; t++) q8[t] = (uint8_t)(h >> (8 * t));
      }
      if (r) {
        uint32_t lo_bits = v & ((1u << r) - 1u);
        uint8_t* rp = remp + (p0 >> 3) * r;  // 32 elements * r bits = 4r bytes per piece
        uint32_t nrem = (r * pm + 7) >> 3;
        uint32_t kk = lane;
        uint32_t j0 = (8 * kk) / r;
        uint32_t acc = 0;
        for (int t = 0; t < 8; t++) {  // r == 1 needs 8 contributors
          uint32_t jj = j0 + t;
          uint32_t val = __shfl_sync(0xffffffffu, lo_bits, jj & 31);
          int start = (int)(jj * r) - (int)(8 * kk);
          if (jj < 32 && start < 8) {
            int sh = 8 - start - (int)r;
            acc |= sh >= 0 ? (val << sh) : (val >> (-sh));
          }
        }
        if (kk < nrem) rp[kk] = (uint8_t)acc;
      }
    }
    off += per_blk_extra + block_bytes(m, bc);
  }
  __syncthreads();
  flush_span(a.out + gpos, s_out, align, agg);
}

// ---------------------------------------------------------------------------
// REL bound: min/max over x (szp.cc:33-48) finished by the last CTA, which
// writes eb = range * (float)rel to *eb_out.  Semantics of the reference's
// serial loop: NaNs are skipped unless x[0] is NaN (then range is NaN);
// when max == min the same element is both, so range = x - x.
// ---------------------------------------------------------------------------
// The end of both float range passes: the CTA's min/max go to its partial;
// the last CTA to finish reduces the partials and writes eb.
__device__ __forceinline__ void rel_finish(const RelArgs& a, float mn, float mx) {
  __shared__ float s_mn[8], s_mx[8];
  __shared__ bool s_last;
  const uint64_t n = a.n;
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    s_mn[warp] = mn;
    s_mx[warp] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
      mn = fminf(mn, s_mn[w]);
      mx = fmaxf(mx, s_mx[w]);
    }
    a.partial[2 * blockIdx.x] = mn;
    a.partial[2 * blockIdx.x + 1] = mx;
    __threadfence();
    uint32_t done = atomicAdd(a.counter, 1u);
    s_last = done == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  // the last CTA reduces the per-CTA partials with all its threads
  __threadfence();
  mn = INFINITY;
  mx = -INFINITY;
  for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    mn = fminf(mn, ((volatile float*)a.partial)[2 * b]);
    mx = fmaxf(mx, ((volatile float*)a.partial)[2 * b + 1]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  __syncthreads();  // s_mn / s_mx are free again
  if (lane == 0) {
    s_mn[warp] = mn;
    s_mx[warp] = mx;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
    mn = fminf(mn, s_mn[w]);
    mx = fmaxf(mx, s_mx[w]);
  }
  *a.counter = 0;  // ready for the next launch
  float range;
  if (n == 0) {
    range = 0.0f;
  } else if (isnan(a.x[0])) {
    range = __uint_as_float(__float_as_uint(a.x[0]) | 0x00400000u);
  } else if (mx == mn && isfinite(mx)) {
    range = 0.0f;
  } else {
    range = x86_nan_fix(__fsub_rn(mx, mn), mx, mn);
  }
  *a.eb_out = x86_nan_fix(__fmul_rn(range, a.rel), range, a.rel);
}

__global__ void __launch_bounds__(256) rel_bound_kernel(RelArgs a) {
  float mn = INFINITY, mx = -INFINITY;
  const uint64_t n = a.n;
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  // scalar head up to 16-byte alignment, vector body, scalar tail
  uint64_t mis = ((uintptr_t)a.x & 15) >> 2;
  uint64_t headn = mis ? (4 - mis) : 0;
  if (headn > n) headn = n;
  for (uint64_t i = tid; i < headn; i += stride) {
    float v = a.x[i];
    mn = fminf(mn, v);
    mx = fmaxf(mx, v);
  }
  const float4* x4 = reinterpret_cast<const float4*>(a.x + headn);
  const uint64_t n4 = (n - headn) >> 2;
  uint64_t i = tid;
  // four independent 16-byte loads in flight per thread
  for (; i + 3 * stride < n4; i += 4 * stride) {
    const float4 v0 = __ldg(x4 + i), v1 = __ldg(x4 + i + stride);
    const float4 v2 = __ldg(x4 + i + 2 * stride), v3 = __ldg(x4 + i + 3 * stride);
    mn = fminf(mn, fminf(fminf(fminf(v0.x, v0.y), fminf(v0.z, v0.w)), fminf(fminf(v1.x, v1.y), fminf(v1.z, v1.w))));
    mx = fmaxf(mx, fmaxf(fmaxf(fmaxf(v0.x, v0.y), fmaxf(v0.z, v0.w)), fmaxf(fmaxf(v1.x, v1.y), fmaxf(v1.z, v1.w))));
    mn = fminf(mn, fminf(fminf(fminf(v2.x, v2.y), fminf(v2.z, v2.w)), fminf(fminf(v3.x, v3.y), fminf(v3.z, v3.w))));
    mx = fmaxf(mx, fmaxf(fmaxf(fmaxf(v2.x, v2.y), fmaxf(v2.z, v2.w)), fmaxf(fmaxf(v3.x, v3.y), fmaxf(v3.z, v3.w))));
  }
  for (; i < n4; i += stride) {
    float4 v = __ldg(x4 + i);
    mn = fminf(fminf(mn, v.x), fminf(v.y, fminf(v.z, v.w)));
    mx = fmaxf(fmaxf(mx, v.x), fmaxf(v.y, fmaxf(v.z, v.w)));
  }
  for (uint64_t i = headn + n4 * 4 + tid; i < n; i += stride) {
    float v = a.x[i];
    mn = fminf(mn, v);
    mx = fmaxf(mx, v);
  }
  rel_finish(a, mn, mx);
}

// The range pass over large inputs: persistent CTAs stream 16 KB chunks of
// the 16-byte-aligned body through a 3-stage shared-memory ring by bulk copy
// (CTA c takes chunks c, c + grid, ...); CTA 0 also takes the scalar head and
// tail.  The same fminf/fmaxf reduction as rel_bound_kernel.
constexpr int kRelStages = 3;
constexpr uint32_t kRelChunk = 4096;  // floats per bulk copy

__global__ void __launch_bounds__(256) rel_bound_bulk(RelArgs a, uint64_t body0, uint64_t nbody) {
  extern __shared__ __align__(16) float s_stage[];  // kRelStages * kRelChunk floats
  __shared__ __align__(8) uint64_t s_full[kRelStages];
  float mn = INFINITY, mx = -INFINITY;
  const uint64_t n = a.n;
  if (blockIdx.x == 0) {
    for (uint64_t i = threadIdx.x; i < body0; i += blockDim.x) {
      const float v = a.x[i];
      mn = fminf(mn, v);
      mx = fmaxf(mx, v);
    }
    for (uint64_t i = body0 + nbody + threadIdx.x; i < n; i += blockDim.x) {
      const float v = a.x[i];
      mn = fminf(mn, v);
      mx = fmaxf(mx, v);
    }
  }
  const float* body = a.x + body0;  // 16-byte aligned; nbody is a multiple of 4
  const uint64_t nch = (nbody + kRelChunk - 1) / kRelChunk;
  if (threadIdx.x == 0)
    for (int s = 0; s < kRelStages; s++) mbar_init(&s_full[s], 1);
  __syncthreads();
  auto issue = [&](uint64_t c, int s) {
    const uint32_t cnt = (uint32_t)min((uint64_t)kRelChunk, nbody - c * kRelChunk);
    mbar_arrive_expect_tx(&s_full[s], 4 * cnt);
    bulk_load(s_stage + (size_t)s * kRelChunk, body + c * kRelChunk, 4 * cnt, &s_full[s]);
  };
  if (threadIdx.x == 0)
    for (int s = 0; s < kRelStages; s++) {
      const uint64_t c = blockIdx.x + (uint64_t)s * gridDim.x;
      if (c < nch) issue(c, s);
    }
  bool gave_up = false;
  for (uint32_t k = 0;; k++) {
    const uint64_t c = blockIdx.x + (uint64_t)k * gridDim.x;
    if (c >= nch) break;
    const int s = (int)(k % kRelStages);
    const uint32_t par = (k / kRelStages) & 1;
    if (!mbar_wait_ns(&s_full[s], par, kWaitNs)) {
      gave_up = true;
      mbar_wait_ns(&s_full[s], par, kWaitNs);  // the copy lands before its stage is reused
    }
    const uint32_t cnt = (uint32_t)min((uint64_t)kRelChunk, nbody - c * kRelChunk);
    const float4* s4 = reinterpret_cast<const float4*>(s_stage + (size_t)s * kRelChunk);
#pragma unroll
    for (int u = 0; u < (int)(kRelChunk / 1024); u++) {
      const uint32_t q = threadIdx.x + 256u * u;
      if (4 * q < cnt) {
        const float4 v = s4[q];
        mn = fminf(mn, fminf(fminf(v.x, v.y), fminf(v.z, v.w)));
        mx = fmaxf(mx, fmaxf(fmaxf(v.x, v.y), fmaxf(v.z, v.w)));
      }
    }
    __syncthreads();  // every thread has read stage s
    if (threadIdx.x == 0) {
      const uint64_t cn = c + (uint64_t)kRelStages * gridDim.x;
      if (cn < nch) issue(cn, s);
    }
  }
  if (gave_up && threadIdx.x == 0 && a.err) atomicOr(a.err, kErrLookbackTimeout);
  rel_finish(a, mn, mx);
}

// Order-preserving key of a double's bits (larger value, larger key); NaNs
// get key 0, below every number's (the reduction uses 0 as "nothing seen"
// too).  The float64 passes load their data as 64-bit integers: on bits
// taken from a double the compiler turns these tests back into FP64 compares,
// which run on this GPU's narrow FP64 pipe.
__device__ __forceinline__ uint64_t f64_key(uint64_t u) {
  if ((u & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull) return 0;  // NaN: skipped, as the reference's compares do
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double f64_unkey(uint64_t k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}

// REL bound of float64 data: min/max over x and eb = range * rel in double
// (szp.cc:77-89), with the rules of rel_bound_kernel (NaNs skipped unless x[0]
// is NaN; max == min gives range x - x).  The min/max run on integer keys
// (FP64 min/max would take the GPU's narrow FP64 pipe); the last CTA reduces
// the per-CTA partials (2 keys each) and does the FP64 arithmetic once.
__global__ void __launch_bounds__(256) rel_bound_kernel_f64(RelArgs a) {
  __shared__ uint64_t s_mn[8], s_mx[8];
  __shared__ bool s_last;
  uint64_t mn = ~0ull, mx = 0;  // keys; 0 also stands for "none" (NaN keys never count)
  const double* x = a.xd;
  const unsigned long long* xb = reinterpret_cast<const unsigned long long*>(x);  // the doubles' bits
  const uint64_t n = a.n;
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  auto take = [&](uint64_t u) {
    const uint64_t k = f64_key(u);
    if (k) {
      mn = min(mn, k);
      mx = max(mx, k);
    }
  };
  const uint64_t headn = min(n, (uint64_t)((((uintptr_t)x & 15) >> 3)));  // one double to 16-byte alignment
  for (uint64_t i = tid; i < headn; i += stride) take(xb[i]);
  const ulonglong2* x2 = reinterpret_cast<const ulonglong2*>(xb + headn);
  const uint64_t n2 = (n - headn) >> 1;
  uint64_t i = tid;
  for (; i + 3 * stride < n2; i += 4 * stride) {
    const ulonglong2 v0 = __ldg(x2 + i), v1 = __ldg(x2 + i + stride);
    const ulonglong2 v2 = __ldg(x2 + i + 2 * stride), v3 = __ldg(x2 + i + 3 * stride);
    take(v0.x); take(v0.y); take(v1.x); take(v1.y);
    take(v2.x); take(v2.y); take(v3.x); take(v3.y);
  }
  for (; i < n2; i += stride) {
    const ulonglong2 v = __ldg(x2 + i);
    take(v.x);
    take(v.y);
  }
  for (uint64_t j = headn + 2 * n2 + tid; j < n; j += stride) take(xb[j]);
  for (int o = 16; o > 0; o >>= 1) {
    mn = min(mn, (uint64_t)__shfl_xor_sync(0xffffffffu, (unsigned long long)mn, o));
    mx = max(mx, (uint64_t)__shfl_xor_sync(0xffffffffu, (unsigned long long)mx, o));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    s_mn[warp] = mn;
    s_mx[warp] = mx;
  }
  __syncthreads();
  uint64_t* part = reinterpret_cast<uint64_t*>(a.partial);
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
      mn = min(mn, s_mn[w]);
      mx = max(mx, s_mx[w]);
    }
    part[2 * blockIdx.x] = mn;
    part[2 * blockIdx.x + 1] = mx;
    __threadfence();
    s_last = atomicAdd(a.counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  mn = ~0ull;
  mx = 0;
  for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    mn = min(mn, ((volatile uint64_t*)part)[2 * b]);
    mx = max(mx, ((volatile uint64_t*)part)[2 * b + 1]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = min(mn, (uint64_t)__shfl_xor_sync(0xffffffffu, (unsigned long long)mn, o));
    mx = max(mx, (uint64_t)__shfl_xor_sync(0xffffffffu, (unsigned long long)mx, o));
  }
  __syncthreads();
  if (lane == 0) {
    s_mn[warp] = mn;
    s_mx[warp] = mx;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
    mn = min(mn, s_mn[w]);
    mx = max(mx, s_mx[w]);
  }
  *a.counter = 0;  // ready for the next launch
  double range;
  if (n == 0) {
    range = 0.0;
  } else if (isnan(x[0])) {
    range = __longlong_as_double(__double_as_longlong(x[0]) | 0x0008000000000000ll);
  } else {
    const double fmn = f64_unkey(mn), fmx = f64_unkey(mx);  // x[0] is a number, so both were seen
    range = (fmx == fmn && isfinite(fmx)) ? 0.0 : x86_nan_fix_d(__dsub_rn(fmx, fmn), fmx, fmn);
  }
  const double eb = x86_nan_fix_d(__dmul_rn(range, a.rel_d), range, a.rel_d);
  *a.ebd_out = eb;
  *a.invd_out = x86_nan_fix_d(__ddiv_rn(1.0, eb), 1.0, eb);  // once, for every quantizing thread
}

// ---------------------------------------------------------------------------
// Device self-test of the bit-count rule on arbitrary inputs.
// ---------------------------------------------------------------------------
__global__ void bitcount_probe_kernel(const uint32_t* __restrict__ in, uint8_t* __restrict__ out, uint64_t n,
                                      BitcountTable thr) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (uint8_t)bitcount_from_table(in[i], thr.thr);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
constexpr int kGenWarps = 8;

// lanes per block for the lane-group kernel, 0 if L needs the generic one
static int lanes_per_block(uint32_t L) {
  switch (L) {
    case 8: return 1;
    case 16: return 2;
    case 32: return 4;
    case 64: return 8;
    case 128: return 16;
    case 256: return 32;
    default: return 0;
  }
}
constexpr int kRounds = 4;

uint32_t compress_blocks_per_tile(uint32_t L, uint32_t& bpw) {
  int lpb = lanes_per_block(L);
  if (lpb) {
    bpw = kRounds * (32 / lpb);
    return 8 * bpw;
  }
  // keep the staged tile near 16 KB
  uint32_t mb = max_block_bytes(L) + 4;
  uint32_t b = (16384u / kGenWarps) / mb;
  bpw = b < 1 ? 1 : (b > 8 ? 8 : b);
  return kGenWarps * bpw;
}

size_t compress_smem_bytes(uint32_t L, uint32_t tb) {
  // the staged output, or the input window (tb*L+1 floats, 16-byte aligned) it replaces
  size_t out = 16 + 4 + (size_t)tb * (max_block_bytes(L) + 4) + 32;
  size_t in = 4 * ((size_t)tb * L + 1) + 32;
  return out > in ? out : in;
}

// Bytes of one pipeline slot: the packed tile (read 16 bytes past its end by
// the shifted copy) or the 16-byte-aligned input window it replaces.
static uint32_t pipe_slot_bytes(uint32_t L, uint32_t tb, bool fm2) {
  const size_t out = 4 + (size_t)tb * (max_block_bytes(L) + (fm2 ? 4 : 0)) + 32;  // fastmode2: a seed per block
  const size_t in = 4 * ((size_t)tb * L + 1) + 32;
  return (uint32_t)(((out > in ? out : in) + 15) & ~(size_t)15);
}

template <int LPB, bool BATCH = false, int ROUNDS = kRounds, bool FM2 = false, bool QI = false>
static cudaError_t launch_lanes(const CompressArgs& a, cudaStream_t st) {
  auto k = compress_pipe<LPB, BATCH, ROUNDS, FM2, QI>;
  const uint32_t slot = pipe_slot_bytes(a.seg.L, a.tb, FM2);
  const size_t smem = (size_t)kPipeSlots * slot;
  // resident CTAs of this instance, cached per device as (device + 1) << 32 | CTAs
  static std::atomic<uint64_t> s_cache{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  uint64_t c = s_cache.load(std::memory_order_relaxed);
  if ((c >> 32) != (uint64_t)dev + 1) {
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kPipeThreads, smem);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    c = ((uint64_t)dev + 1) << 32 | (uint32_t)((occ < 1 ? 1 : occ) * sms);
    s_cache.store(c, std::memory_order_relaxed);
  }
  const uint32_t s_grid = (uint32_t)c;
  const uint32_t grid = a.ntiles < s_grid ? a.ntiles : s_grid;
  if (grid == 0) return cudaSuccess;
  k<<<grid, kPipeThreads, smem, st>>>(a, slot);
  return cudaGetLastError();
}

cudaError_t launch_compress(const CompressArgs& a, bool fm2, cudaStream_t st) {
  if (!fm2 && compress32_supported(a)) return launch_compress32(a, st);
  size_t smem = compress_smem_bytes(a.seg.L, a.tb);
  if (fm2) {
    switch (lanes_per_block(a.seg.L)) {
      case 1: return launch_lanes<1, false, kRounds, true>(a, st);
      case 2: return launch_lanes<2, false, kRounds, true>(a, st);
      case 4: return launch_lanes<4, false, kRounds, true>(a, st);
      case 8: return launch_lanes<8, false, kRounds, true>(a, st);
      case 16: return launch_lanes<16, false, kRounds, true>(a, st);
      case 32: return launch_lanes<32, false, kRounds, true>(a, st);
      default: break;
    }
  }
  if (!fm2) {
    switch (lanes_per_block(a.seg.L)) {
      case 1: return launch_lanes<1>(a, st);
      case 2: return launch_lanes<2>(a, st);
      case 4: return launch_lanes<4>(a, st);
      case 8: return launch_lanes<8>(a, st);
      case 16: return launch_lanes<16>(a, st);
      case 32: return launch_lanes<32>(a, st);
      default: break;
    }
    auto k = compress_generic<kGenWarps, false>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<a.ntiles, kGenWarps * 32, smem, st>>>(a);
  } else {
    auto k = compress_generic<kGenWarps, true>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<a.ntiles, kGenWarps * 32, smem, st>>>(a);
  }
  return cudaGetLastError();
}

// Order-preserving encoding of a non-NaN float as an unsigned integer.
__host__ __device__ __forceinline__ uint32_t rel_encode(float v) {
  uint32_t u;
  memcpy(&u, &v, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float rel_decode(uint32_t e) {
  const uint32_t u = (e & 0x80000000u) ? (e & 0x7FFFFFFFu) : ~e;
  return __uint_as_float(u);
}
uint32_t rel_encode_host(float v) { return rel_encode(v); }

// Range pass of a batch: every CTA reduces work items (a chunk of one REL
// field) with the single-field pass's rules (fminf/fmaxf, NaN ignored), and
// the last item of a field turns its range into the bound exactly as
// rel_bound_kernel does (szp.cc:36-51 semantics).
__global__ void __launch_bounds__(256) rel_batch_kernel(const __grid_constant__ RelBatchArgs a) {
  __shared__ float s_mn[8], s_mx[8];
  __shared__ uint32_t s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t it = blockIdx.x; it < a.nitems; it += gridDim.x) {
    const uint32_t f = a.item_field[it];
    CompressField& fd = a.fields[f];
    RelFieldState& st = a.state[f];
    const float* x = fd.x;
    const uint64_t n = fd.seg.n;
    const uint64_t lo = (uint64_t)(it - st.first_item) * a.chunk;
    const uint64_t hi = min(n, lo + a.chunk);
    float mn = INFINITY, mx = -INFINITY;
    // scalar head to a 16-byte boundary, 16-byte body, scalar tail
    uint64_t b0 = lo;
    while (b0 < hi && (((uintptr_t)(x + b0)) & 15)) b0++;
    const uint64_t n4 = (hi - b0) >> 2;
    for (uint64_t i = lo + threadIdx.x; i < b0; i += blockDim.x) {
      mn = fminf(mn, x[i]);
      mx = fmaxf(mx, x[i]);
    }
    const float4* x4 = reinterpret_cast<const float4*>(x + b0);
    const uint32_t bs = blockDim.x;
    uint64_t i = threadIdx.x;
    // four independent 16-byte loads in flight per thread
    for (; i + 3 * bs < n4; i += 4 * bs) {
      const float4 v0 = __ldg(x4 + i), v1 = __ldg(x4 + i + bs);
      const float4 v2 = __ldg(x4 + i + 2 * bs), v3 = __ldg(x4 + i + 3 * bs);
      mn = fminf(mn, fminf(fminf(fminf(v0.x, v0.y), fminf(v0.z, v0.w)), fminf(fminf(v1.x, v1.y), fminf(v1.z, v1.w))));
      mx = fmaxf(mx, fmaxf(fmaxf(fmaxf(v0.x, v0.y), fmaxf(v0.z, v0.w)), fmaxf(fmaxf(v1.x, v1.y), fmaxf(v1.z, v1.w))));
      mn = fminf(mn, fminf(fminf(fminf(v2.x, v2.y), fminf(v2.z, v2.w)), fminf(fminf(v3.x, v3.y), fminf(v3.z, v3.w))));
      mx = fmaxf(mx, fmaxf(fmaxf(fmaxf(v2.x, v2.y), fmaxf(v2.z, v2.w)), fmaxf(fmaxf(v3.x, v3.y), fmaxf(v3.z, v3.w))));
    }
    for (; i < n4; i += bs) {
      const float4 v = __ldg(x4 + i);
      mn = fminf(mn, fminf(fminf(v.x, v.y), fminf(v.z, v.w)));
      mx = fmaxf(mx, fmaxf(fmaxf(v.x, v.y), fmaxf(v.z, v.w)));
    }
    for (uint64_t i = b0 + 4 * n4 + threadIdx.x; i < hi; i += blockDim.x) {
      mn = fminf(mn, x[i]);
      mx = fmaxf(mx, x[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane == 0) {
      s_mn[warp] = mn;
      s_mx[warp] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < 8; w++) {
        mn = fminf(mn, s_mn[w]);
        mx = fmaxf(mx, s_mx[w]);
      }
      // +inf / -inf (an all-NaN chunk) leave the field's state unchanged
      atomicMin(&st.mn, rel_encode(mn));
      atomicMax(&st.mx, rel_encode(mx));
      __threadfence();
      s_last = atomicAdd(&st.done, 1u) == st.nitems - 1;
      if (s_last) {
        __threadfence();
        const float fmn = rel_decode(*(volatile uint32_t*)&st.mn);
        const float fmx = rel_decode(*(volatile uint32_t*)&st.mx);
        float range;
        if (isnan(x[0])) {
          range = __uint_as_float(__float_as_uint(x[0]) | 0x00400000u);
        } else if (fmx == fmn && isfinite(fmx)) {
          range = 0.0f;
        } else {
          range = x86_nan_fix(__fsub_rn(fmx, fmn), fmx, fmn);
        }
        fd.eb = x86_nan_fix(__fmul_rn(range, fd.rel), range, fd.rel);
        st.mn = rel_encode(INFINITY);  // ready for the next run
        st.mx = rel_encode(-INFINITY);
        st.done = 0;
      }
    }
    __syncthreads();
  }
}

cudaError_t launch_rel_batch(const RelBatchArgs& a, uint32_t grid, cudaStream_t st) {
  if (a.nitems == 0) return cudaSuccess;
  rel_batch_kernel<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

// Sets the batched compress kernels' shared-memory limits and caches their
// grids (a no-op launch of zero tiles), so no later launch does that work.
cudaError_t prepare_compress_batch() {
  CompressArgs a;
  memset(&a, 0, sizeof a);
  a.seg.L = 32;
  cudaError_t e = cudaSuccess;
  for (int r : {1, 2, 4}) {
    a.tb = 8u * (uint32_t)r * 8u;
    e = r == 1 ? launch_lanes<4, true, 1>(a, 0) : r == 2 ? launch_lanes<4, true, 2>(a, 0) : launch_lanes<4, true, 4>(a, 0);
    if (e != cudaSuccess) return e;
  }
  return e;
}

// Batched fastmode1 compression, blockSize 32, tiles of 8*rounds*8 blocks.
cudaError_t launch_compress_batch(const CompressArgs& a, uint32_t L, int rounds, cudaStream_t st) {
  if (L != 32) return cudaErrorInvalidValue;
  switch (rounds) {
    case 1: return launch_lanes<4, true, 1>(a, st);
    case 2: return launch_lanes<4, true, 2>(a, st);
    case 4: return launch_lanes<4, true, 4>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_rel_bound_f64(const RelArgs& a, uint32_t grid, cudaStream_t st) {
  rel_bound_kernel_f64<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

// float64 quantization pass (szp_double.cc:180-230's q = (int)(x * inver)):
// q[i] from x[i] in integer arithmetic, four elements per step (two 16-byte
// loads, one 16-byte store; x + h and q + h are 16-byte aligned, h the
// elements before x's first 16-byte boundary).  Range errors set the
// quantization flag, as the compress kernels do.
__global__ void __launch_bounds__(256) quantize_f64_kernel(const double* __restrict__ x, int32_t* __restrict__ q,
                                                           uint64_t n, double invd, const double* invd_dev,
                                                           uint32_t* err) {
  const f64i::Inverse io = f64i::prepare_inverse(f64i::bits_of(invd_dev ? *invd_dev : invd));
  bool bad = false;
  const uint64_t h = min(n, (uint64_t)((((uintptr_t)x & 15) >> 3)));
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const unsigned long long* xb = reinterpret_cast<const unsigned long long*>(x);  // bits, see f64_key
  if (tid < h) q[tid] = f64i::quantize_fast(xb[tid], io, bad);
  const ulonglong2* x2 = reinterpret_cast<const ulonglong2*>(xb + h);
  int4* q4 = reinterpret_cast<int4*>(q + h);
  const uint64_t n4 = (n - h) >> 2;
  for (uint64_t i = tid; i < n4; i += stride) {
    const ulonglong2 u = __ldcs(x2 + 2 * i), v = __ldcs(x2 + 2 * i + 1);
    int4 r;
    r.x = f64i::quantize_fast(u.x, io, bad);
    r.y = f64i::quantize_fast(u.y, io, bad);
    r.z = f64i::quantize_fast(v.x, io, bad);
    r.w = f64i::quantize_fast(v.y, io, bad);
    q4[i] = r;
  }
  for (uint64_t i = h + 4 * n4 + tid; i < n; i += stride) q[i] = f64i::quantize_fast(xb[i], io, bad);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(err, kErrQuantRange);
}

bool f64_pipe_supported(uint32_t L) { return lanes_per_block(L) != 0; }

// qbuf (16-byte aligned) holds n + 4 int32; the view starts 0 or 3 elements
// in so that q + h and x + h are both 16-byte aligned, h being the doubles
// before x's first 16-byte boundary (0 or 1): the quantization pass then
// moves whole vectors.
int32_t* f64_q_view(void* qbuf, const void* x) {
  const uint32_t h = ((uintptr_t)x & 15) ? 1u : 0u;
  return reinterpret_cast<int32_t*>(qbuf) + ((4 - h) & 3);
}

cudaError_t launch_quantize_f64(const double* x, int32_t* q, uint64_t n, double invd, const double* invd_dev,
                                uint32_t* err, uint32_t sm_count, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const uint64_t want = (n / 4 + 255) / 256;
  const uint64_t lim = (uint64_t)(sm_count ? sm_count : 1) * 8;
  const uint32_t grid = (uint32_t)(want < 1 ? 1 : (want > lim ? lim : want));
  quantize_f64_kernel<<<grid, 256, 0, st>>>(x, q, n, invd, invd_dev, err);
  return cudaGetLastError();
}

// The fastmode pipelines over int32 codes (eb header of a.qhb bytes).
cudaError_t launch_compress_q(const CompressArgs& a, bool fm2, cudaStream_t st) {
  if (fm2) {
    switch (lanes_per_block(a.seg.L)) {
      case 1: return launch_lanes<1, false, kRounds, true, true>(a, st);
      case 2: return launch_lanes<2, false, kRounds, true, true>(a, st);
      case 4: return launch_lanes<4, false, kRounds, true, true>(a, st);
      case 8: return launch_lanes<8, false, kRounds, true, true>(a, st);
      case 16: return launch_lanes<16, false, kRounds, true, true>(a, st);
      case 32: return launch_lanes<32, false, kRounds, true, true>(a, st);
      default: return cudaErrorInvalidValue;
    }
  }
  switch (lanes_per_block(a.seg.L)) {
    case 1: return launch_lanes<1, false, kRounds, false, true>(a, st);
    case 2: return launch_lanes<2, false, kRounds, false, true>(a, st);
    case 4: return launch_lanes<4, false, kRounds, false, true>(a, st);
    case 8: return launch_lanes<8, false, kRounds, false, true>(a, st);
    case 16: return launch_lanes<16, false, kRounds, false, true>(a, st);
    case 32: return launch_lanes<32, false, kRounds, false, true>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

// float64 data: the one-warp-per-block kernel for every blockSize, tiles kept
// near 16 KB of stream like the float kernel's.
uint32_t compress_blocks_per_tile_f64(uint32_t L, uint32_t& bpw) {
  const uint32_t mb = max_block_bytes(L) + 4;
  const uint32_t b = (16384u / kGenWarps) / mb;
  bpw = b < 1 ? 1 : (b > 8 ? 8 : b);
  return kGenWarps * bpw;
}

size_t compress_smem_bytes_f64(uint32_t L, uint32_t tb) { return 16 + 8 + (size_t)tb * (max_block_bytes(L) + 4) + 32; }

cudaError_t launch_compress_f64(const CompressArgs& a, bool fm2, cudaStream_t st) {
  const size_t smem = compress_smem_bytes_f64(a.seg.L, a.tb);
  if (fm2) {
    auto k = compress_generic<kGenWarps, true, double>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<a.ntiles, kGenWarps * 32, smem, st>>>(a);
  } else {
    auto k = compress_generic<kGenWarps, false, double>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<a.ntiles, kGenWarps * 32, smem, st>>>(a);
  }
  return cudaGetLastError();
}

// Inputs of at least 64 chunks take the bulk-copy pass, on at most 4 CTAs
// per SM (the partials hold `grid` CTAs).
cudaError_t launch_rel_bound(const RelArgs& a, uint32_t grid, cudaStream_t st) {
  const uintptr_t xa = (uintptr_t)a.x;
  const uint64_t mis = (xa & 15) >> 2;
  const uint64_t body0 = min((uint64_t)(mis ? 4 - mis : 0), a.n);
  const uint64_t nbody = (a.n - body0) & ~3ull;
  if ((xa & 3) == 0 && nbody >= 64ull * kRelChunk) {
    static std::atomic<uint64_t> s_sms{0};  // (device + 1) << 32 | SM count
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    uint64_t c = s_sms.load(std::memory_order_relaxed);
    if ((c >> 32) != (uint64_t)dev + 1) {
      int sms = 0;
      e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      e = cudaFuncSetAttribute(rel_bound_bulk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(kRelStages * kRelChunk * sizeof(float)));
      if (e != cudaSuccess) return e;
      c = ((uint64_t)dev + 1) << 32 | (uint32_t)sms;
      s_sms.store(c, std::memory_order_relaxed);
    }
    const uint64_t nch = (nbody + kRelChunk - 1) / kRelChunk;
    uint32_t g = grid < 4 * (uint32_t)c ? grid : 4 * (uint32_t)c;
    if (g > nch) g = (uint32_t)nch;
    rel_bound_bulk<<<g, 256, kRelStages * kRelChunk * sizeof(float), st>>>(a, body0, nbody);
    return cudaGetLastError();
  }
  rel_bound_kernel<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

// Diagnostics of the bounded waits: one thread waits on an mbarrier that
// nothing arrives at, for at most limit_ns; it records the time it waited and
// flags the launch like a pipeline wait that gives up.
__global__ void wait_probe_kernel(uint64_t limit_ns, uint32_t* err, unsigned long long* waited) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  const uint64_t t0 = globaltimer_ns();
  const bool done = mbar_wait_ns(&bar, 0, limit_ns);
  *waited = globaltimer_ns() - t0;
  if (!done) atomicOr(err, kErrLookbackTimeout);
}

cudaError_t launch_wait_probe(uint64_t limit_ns, uint32_t* err, unsigned long long* waited, cudaStream_t st) {
  wait_probe_kernel<<<1, 32, 0, st>>>(limit_ns, err, waited);
  return cudaGetLastError();
}

cudaError_t launch_bitcount_probe(const uint32_t* in, uint8_t* out, uint64_t n, const BitcountTable& thr,
                                  cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  bitcount_probe_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n, thr);
  return cudaGetLastError();
}

}  // namespace szp
