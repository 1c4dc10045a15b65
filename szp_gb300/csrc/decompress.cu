// decompress.cu -- SZp fastmode1 / fastmode2 float32 decompressors for sm_103a.
//
// The stream keeps no block index: a block's position depends on the bit
// counts of all blocks before it in its segment (szpd_float.cc:76-118).  Three
// launches recover the positions and decode:
//
//  1. dec_setup   one CTA reads eb and the T segment offsets, validates them and
//                 cuts every segment's block region into fixed chunks.
//  2. locate      one CTA per super-chunk (threads x chunk bytes) of a segment:
//                 the bytes (plus an overlap before them) are staged in shared
//                 memory by a bulk copy and every thread walks the chain of
//                 block headers through its chunk.  Only a segment's first
//                 chunk knows where its first header is; the others start early
//                 (in the overlap) at the first position whose chain stays
//                 valid: chains started on payload bytes die within a step or
//                 two (a header byte must be <= 33) or land on a true header and
//                 follow the true chain from then on.  A chunk is right when its
//                 first header is its predecessor's exit; wrong chunks (rare)
//                 are re-walked in order.  Across CTAs a decoupled look-back
//                 sums header counts and checks the same chain property on the
//                 (entry, exit) pairs the predecessors published; a CTA whose
//                 entry proves wrong re-walks from the true one.  Each chunk then
//                 writes the header offset of each of its blocks.
//  3. decode      decode_pipe (blockSize 8..256, a power of two), a persistent,
//                 warp-specialised pipeline: per tile of blocks the stream span
//                 and block offsets are staged in shared memory by TMA; LPB
//                 lanes per block unpack 8 elements each (sign byte, byte
//                 planes and remainder bits are byte-aligned per 8 elements),
//                 prefix-add (fastmode1: warp and tile scans and a look-back
//                 over the tiles of a segment; fastmode2: a scan inside the
//                 block from its seed) and dequantize.  decode_generic covers
//                 the other blockSizes.
#include <atomic>

#include <type_traits>

#include "szp_device.cuh"
#include "szp_f64.h"
#include "szp_kernels.h"
#include "szp_pipe.cuh"
#include "szp_tma.cuh"

namespace szp {

constexpr uint32_t kPosEnd = 0xFFFFFFFEu;   // the walk left the segment region
constexpr uint32_t kPosDead = 0xFFFFFFFFu;  // the walk met an invalid header

// Size of a full block whose bit-count byte is b; 0 if b is not a valid
// header.  fastmode2 blocks carry a 4-byte seed and L-1 deltas.
__host__ __device__ __forceinline__ uint32_t full_block_size(uint32_t b, uint32_t L, bool fm2) {
  if (b > (uint32_t)kMaxBitCount) return 0;
  if (!fm2) return block_bytes(L, b);
  if (L == 1) return b == 0 ? 5u : 0u;
  return 4 + block_bytes(L - 1, b);
}

__host__ __device__ __forceinline__ uint32_t max_walk_block(uint32_t L, bool fm2) {
  return fm2 ? (L == 1 ? 5u : 4 + block_bytes(L - 1, kMaxBitCount)) : block_bytes(L, kMaxBitCount);
}

constexpr int kLocThreads = 128;

// A chunk may hold no header at all (a block larger than the chunk), so the
// chunk size does not depend on the block size; the overlap that lets a
// speculative walk synchronise spans at least 8 of the largest blocks.
uint32_t locate_chunk_bytes(uint32_t) { return 512; }
uint32_t locate_super_bytes(uint32_t maxsz) { return locate_chunk_bytes(maxsz) * kLocThreads; }
uint32_t locate_overlap_bytes(uint32_t maxsz) {
  uint32_t w = 2048;
  while (w < 8 * maxsz && w < 65536) w *= 2;
  return w;
}
size_t locate_smem_bytes(uint32_t super_chunk, uint32_t overlap, uint32_t maxsz) {
  return (size_t)overlap + super_chunk + maxsz + 64;
}

__device__ __forceinline__ uint64_t load_u64le(const uint8_t* p) {
  uint64_t v = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) v |= (uint64_t)p[i] << (8 * i);
  return v;
}

// ---------------------------------------------------------------------------
// 1. header -> plan
// ---------------------------------------------------------------------------
template <bool BATCH>
__global__ void dec_setup_kernel(const __grid_constant__ DecArgs a) {
  const DecField& fd = BATCH ? a.fields[blockIdx.x] : a.f;
  const Segments sg = fd.seg;
  const uint32_t T = sg.T;
  const uint32_t hb = a.hb == 8 ? 8u : 4u;  // eb header: float, or double (szpd_double.cc)
  const uint64_t head = hb + 8ull * T;
  __shared__ uint32_t s_bad;
  uint64_t len = fd.len;
  if (fd.len_dev) {
    uint64_t l2 = *fd.len_dev;
    len = l2 < len ? l2 : len;
  }
  if (threadIdx.x == 0) {
    s_bad = len < head ? 1u : 0u;
    if (!s_bad) {
      uint32_t b = ((uint32_t)fd.in[0] << 24) | ((uint32_t)fd.in[1] << 16) | ((uint32_t)fd.in[2] << 8) | fd.in[3];
      fd.plan->eb = __uint_as_float(b);
      unsigned long long d = 0;
      if (hb == 8)
        for (int i = 0; i < 8; i++) d = (d << 8) | fd.in[i];
      fd.plan->ebd = __longlong_as_double((long long)d);
    } else {
      fd.plan->eb = 0.0f;
      fd.plan->ebd = 0.0;
    }
  }
  __syncthreads();
  const bool hdr_ok = !s_bad;
  for (uint32_t t = threadIdx.x; t < T; t += blockDim.x) {
    uint64_t len_t = sg.len(t);
    uint64_t r0 = 0, r1 = 0;
    uint32_t nch = 0;
    bool bad = false;
    if (len_t > 0 && hdr_ok) {
      uint64_t off = load_u64le(fd.in + hb + 8ull * t);
      uint64_t body = len - head;
      uint64_t end;
      if (off > body) {
        bad = true;
      } else {
        uint64_t start = head + off;
        if (t + 1 < T) {
          uint64_t off2 = load_u64le(fd.in + hb + 8ull * (t + 1));
          if (off2 < off || off2 > body) bad = true;
          end = head + off2;
        } else {
          end = len;
        }
        if (!bad) {
          uint64_t nblk = a.fm2 ? (len_t + sg.L - 1) / sg.L : sg.blocks_fm1(t);
          r0 = a.fm2 ? start : start + 4;
          if (r0 > end) {
            bad = true;
          } else {
            uint64_t bound = r0 + nblk * (uint64_t)a.maxsz;
            r1 = end < bound ? end : bound;
            if (nblk > 0 && r1 <= r0) bad = true;
            if (r1 - r0 >= (1ull << 32)) bad = true;  // block offsets are 32-bit
            nch = (uint32_t)((r1 - r0 + a.super_chunk - 1) / a.super_chunk);
          }
        }
      }
    }
    if (bad) {
      atomicOr(&s_bad, 1u);
      nch = 0;
    }
    fd.reg0[t] = r0;
    fd.reg1[t] = r1;
    fd.chunk_base[t + 1] = nch;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    fd.chunk_base[0] = 0;
    if (s_bad) {
      for (uint32_t t = 0; t < T; t++) fd.chunk_base[t + 1] = 0;
      atomicOr(fd.err, kErrCorrupt);
    } else {
      for (uint32_t t = 0; t < T; t++) {
        acc += fd.chunk_base[t + 1];
        fd.chunk_base[t + 1] = acc;
      }
    }
    fd.plan->nchunks = s_bad ? 0 : acc;
    fd.plan->bad = s_bad;
  }
}

// Global block index of block 0 of segment t (segments 0..T-2 are alike).
__device__ __forceinline__ uint64_t seg_block_base(const Segments& sg, uint32_t t, bool fm2) {
  uint64_t per = fm2 ? (sg.tsz + sg.L - 1) / sg.L : (sg.tsz > 1 ? (sg.tsz - 1 + sg.L - 1) / sg.L : 0);
  return (uint64_t)t * per;
}
__device__ __forceinline__ uint64_t seg_blocks(const Segments& sg, uint32_t t, bool fm2) {
  return fm2 ? (sg.len(t) + sg.L - 1) / sg.L : sg.blocks_fm1(t);
}

// ---------------------------------------------------------------------------
// 2. locate block headers
// ---------------------------------------------------------------------------
constexpr uint64_t kFlagRepair = 3;  // status: the CTA is re-walking; not ready

// CTA (super-chunk) of ticket c: largest t with chunk_base[t] <= c.
__device__ __forceinline__ uint32_t chunk_segment(const uint32_t* __restrict__ cb, uint32_t T, uint32_t c) {
  uint32_t lo_t = 0, hi_t = T - 1;
  while (lo_t < hi_t) {
    uint32_t mid = (lo_t + hi_t + 1) >> 1;
    if (cb[mid] <= c) lo_t = mid; else hi_t = mid - 1;
  }
  return lo_t;
}

// A header chain walked in the shared-memory copy of a segment's region:
// region offset p is at sb[p - base0]; bytes exist below `avail`.
struct SmemChain {
  const uint8_t* sb;
  uint32_t base0, avail, rlen, L;
  uint32_t l8;  // L / 8 for fastmode1 with L % 8 == 0 (block size 1 + l8*(b+1)), else 0
  bool fm2;
  // block size at p, 0 when its bit-count byte is invalid or not staged
  __device__ __forceinline__ uint32_t step(uint32_t p) const {
    uint32_t hp = fm2 ? p + 4 : p;
    if (hp >= avail) return 0;
    const uint32_t b = sb[hp - base0];
    if (l8) return b > (uint32_t)kMaxBitCount ? 0u : (b ? 1 + l8 * (b + 1) : 1u);
    return full_block_size(b, L, fm2);
  }
  // walk from p to cE: header count, exit (kPosEnd past the region, kPosDead)
  __device__ __forceinline__ uint32_t walk(uint32_t p, uint32_t cE, uint32_t* exit) const {
    uint32_t k = 0;
    while (p < cE) {
      uint32_t sz = step(p);
      if (!sz) {
        *exit = kPosDead;
        return k;
      }
      k++;
      p += sz;
    }
    *exit = p >= rlen ? kPosEnd : p;
    return k;
  }
};


// Re-walks, in order, every chunk from `from` on whose first header is not
// the exit of the chunk before it (e = exit before chunk `from`); thread-serial.
__device__ __forceinline__ void rewalk_from(const SmemChain& ch, uint32_t* h, uint32_t* x, uint32_t* k,
                                            uint32_t from, uint32_t e, uint32_t nactive, uint32_t scS,
                                            uint32_t scE, uint32_t C) {
  for (uint32_t i = from; i < nactive; i++) {
    if (e == kPosEnd || e == kPosDead) {
      h[i] = e;
      x[i] = e;
      k[i] = 0;
      continue;
    }
    if (h[i] != e) {
      const uint32_t cE = min(scS + (i + 1) * C, scE);
      h[i] = e;
      uint32_t ex;
      k[i] = ch.walk(e, cE, &ex);
      x[i] = ex;
    }
    e = x[i];
  }
}

// PACK: a super-chunk's look-back word carries its (entry, exit) pair too, so
// one load reads a predecessor (blocks of at most 254 bytes, super-chunks
// below 2^17 - 2 bytes).  An aggregate's 42-bit value holds the header count
// (17 bits), the entry relative to the super-chunk's start (17 bits) and the
// exit relative to its end (8 bits); an inclusive value holds the count
// prefix and the exit.  Otherwise the pair sits in a second word, read between
// two reads of the status word.
constexpr uint32_t kRelDead = 0x1FFFFu, kRelEnd = 0x1FFFEu, kXDead = 0xFFu, kXEnd = 0xFEu;

__device__ __forceinline__ uint64_t loc_word(uint64_t cnt, uint32_t h0, uint32_t xl, uint32_t scS, uint32_t scE,
                                             bool incl) {
  const uint64_t xr = xl == kPosDead ? kXDead : xl == kPosEnd ? kXEnd : (uint64_t)(xl - scE);
  if (incl) return (cnt << 8) | xr;
  const uint64_t hr = h0 == kPosDead ? kRelDead : h0 == kPosEnd ? kRelEnd : (uint64_t)(h0 - scS);
  return (cnt << 25) | (hr << 8) | xr;
}

static bool locate_packs(uint32_t super_chunk, uint32_t maxsz) {
  return maxsz <= 254 && (uint64_t)super_chunk + maxsz < kRelEnd;
}

template <bool FM2, bool BATCH, bool PACK>
__global__ void __launch_bounds__(kLocThreads) locate_kernel(const __grid_constant__ DecArgs a) {
  constexpr int NT = kLocThreads;
  extern __shared__ __align__(16) uint8_t s_bytes[];
  __shared__ uint32_t s_tk[2];
  __shared__ uint32_t s_h[NT], s_x[NT], s_k[NT];
  __shared__ uint64_t s_val[1];
  __shared__ uint32_t s_misc[2 * (NT / 32)];
  __shared__ __align__(8) uint64_t s_bar;
  uint32_t tile, epoch;
  draw_ticket(a.ls, a.nlocate_ctas, tile, epoch, s_tk);
  // status and aux words are indexed by launch ticket, chunks by field-local ticket
  const DecField& fd = BATCH ? a.fields[a.loc_field[tile]] : a.f;
  const uint32_t lt = tile - fd.loc_base;
  const uint32_t nct = fd.plan->bad ? 0 : fd.chunk_base[fd.seg.T];
  if (lt >= nct) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const Segments sg = fd.seg;
  const uint32_t t = chunk_segment(fd.chunk_base, sg.T, lt);
  const uint32_t first = fd.loc_base + fd.chunk_base[t];  // launch ticket of the segment's first chunk
  const uint32_t j = tile - first;
  const uint64_t R0 = fd.reg0[t];
  const uint32_t rlen = (uint32_t)(fd.reg1[t] - R0);
  const uint32_t C = a.chunk, SC = a.super_chunk, W0 = a.overlap;
  const uint32_t scS = j * SC, scE = min(scS + SC, rlen);

  // ---- stage [scS - W0, scE + maxsz) of the region ----
  const uint32_t st0 = scS > W0 ? scS - W0 : 0u;
  const uint32_t st1 = (uint32_t)min((uint64_t)rlen, (uint64_t)scE + a.maxsz + 8);
  const uint8_t* g = fd.in + R0 + st0;
  const uint32_t align = (uint32_t)((uintptr_t)g & 15);
  {
    if (tid == 0) mbar_init(&s_bar, 1);
    __syncthreads();
    const uint32_t end = align + (st1 - st0);
    const uint32_t i0 = (align + 15) & ~15u, i1 = end & ~15u;
    const uint8_t* g0 = g - align;
    const bool bulk = i1 > i0;
    if (tid == 0 && bulk) {
      mbar_arrive_expect_tx(&s_bar, i1 - i0);
      bulk_load(s_bytes + i0, g0 + i0, i1 - i0, &s_bar);
    }
    if (bulk) {
      for (uint32_t b = align + tid; b < i0; b += NT) s_bytes[b] = __ldg(g0 + b);
      for (uint32_t b = i1 + tid; b < end; b += NT) s_bytes[b] = __ldg(g0 + b);
    } else {
      for (uint32_t b = align + tid; b < end; b += NT) s_bytes[b] = __ldg(g0 + b);
    }
    if (bulk && !mbar_wait_ns(&s_bar, 0, kWaitNs)) {
      atomicOr(a.err, kErrLookbackTimeout);
      mbar_wait_ns(&s_bar, 0, kWaitNs);  // the copy lands before the CTA may exit
    }
    __syncthreads();
  }
  SmemChain ch;
  ch.sb = s_bytes + align;
  ch.base0 = st0;
  ch.avail = st1;
  ch.rlen = rlen;
  ch.L = sg.L;
  ch.l8 = (!FM2 && sg.L % 8 == 0) ? sg.L / 8 : 0u;
  ch.fm2 = FM2;

  // ---- speculative walk of each thread's chunk ----
  // A lane's chain starts at `anchor` (a segment's first chunk: at its first
  // header); the first position >= cS on it is the chunk's entry, headers in
  // [cS, cE) are counted, and the first position >= cE is its exit.  A chain
  // that meets an invalid header restarts one byte after its anchor.  Each
  // lane runs its own loop of single header steps: lanes finish at different
  // times, but an iteration is a handful of instructions (a lockstep loop that
  // applied every outcome with selects cost several times as much).
  const uint32_t nactive = (scE - scS + C - 1) / C;
  const uint32_t cS = scS + tid * C, cE = min(cS + C, scE);
  uint32_t h = kPosEnd, x = kPosEnd, k = 0;
  if ((uint32_t)tid < nactive) {
    const bool known = j == 0 && tid == 0;  // a segment's block region starts with a header
    // a wrong guess is caught by the chain checks (inside the CTA, or across
    // CTAs for its first chunk) and re-walked from the true exit
    const uint32_t W = min(W0, max(512u, 4 * a.maxsz));
    uint32_t anchor = known ? 0u : (cS > st0 + W ? cS - W : st0);
    uint32_t pos = anchor, entry = anchor >= cS ? anchor : kPosDead, cnt = 0;
    uint32_t budget = 4 * (W + C);
    bool broken = false;
    h = kPosDead;
    x = kPosDead;
    const uint8_t* sb = ch.sb - ch.base0;  // region offset p at sb[p]
    const bool b32 = !FM2 && ch.l8 == 4;  // blockSize 32: a block of 1 or 4b + 5 bytes
    while (pos < cE && budget != 0) {
      budget--;
      // every position read is below cE, inside the staged bytes
      const uint32_t b = sb[pos];
      const uint32_t sz = b32 ? (b > (uint32_t)kMaxBitCount ? 0u : (b ? 4 * b + 5 : 1u)) : ch.step(pos);
      if (sz) {
        cnt += pos >= cS ? 1u : 0u;
        const uint32_t np = pos + sz;
        if (entry == kPosDead && np >= cS) entry = np;
        pos = np;
      } else if (!known && anchor + 1 < cE) {
        anchor++;
        pos = anchor;
        cnt = 0;
        entry = anchor >= cS ? anchor : kPosDead;
      } else {
        broken = true;
        break;
      }
    }
    if (pos >= cE) {
      h = entry >= rlen ? kPosEnd : entry;
      x = pos >= rlen ? kPosEnd : pos;
      k = cnt;
    } else if (broken && known) {
      h = 0;
      k = cnt;  // x stays kPosDead: the true chain is broken
    }
  }
  s_h[tid] = h;
  s_x[tid] = x;
  s_k[tid] = k;
  __syncthreads();
  // ---- chunk boundaries inside the CTA ----
  bool bad = false;
  if (tid > 0 && (uint32_t)tid < nactive) {
    const uint32_t px = s_x[tid - 1];
    bad = (px == kPosEnd) ? (h != kPosEnd || k != 0) : (px != h);
  }
  const uint32_t repairs = __syncthreads_count(bad);
  if (repairs) {
    if (tid == 0) {
      rewalk_from(ch, s_h, s_x, s_k, 1, s_x[0], nactive, scS, scE, C);
      atomicAdd(&a.counters[0], repairs);
    }
    __syncthreads();
  }

  // ---- look-back over header counts, verifying entries (warp 0; the
  // other warps wait at the barrier after it) ----
  uint32_t K = 0;
  for (int i = 0; i < NT; i++) K += s_k[i];  // shared reads, same in every thread
  uint32_t h0 = s_h[0], xl = s_x[nactive - 1];
  uint64_t prefix = 0;
  if (j == 0) {
    if (tid == 0) {
      if (PACK) {
        st_relaxed_u64(a.status + tile, make_status(epoch, kFlagInclusive, loc_word(K, h0, xl, scS, scE, true)));
      } else {
        a.aux[tile] = make_uint2(h0, xl);
        __threadfence();
        st_release_u64(a.status + tile, make_status(epoch, kFlagInclusive, K));
      }
    }
  } else {
    if (tid == 0) {
      if (PACK) {
        st_relaxed_u64(a.status + tile, make_status(epoch, kFlagAggregate, loc_word(K, h0, xl, scS, scE, false)));
      } else {
        a.aux[tile] = make_uint2(h0, xl);
        __threadfence();
        st_release_u64(a.status + tile, make_status(epoch, kFlagAggregate, K));
      }
    }
    if (warp == 0) {
      // lane l reads tile base - l (seqlock read of status + aux); a window
      // whose entries are not all ready, or whose chain of (entry, exit)
      // pairs is broken (an older tile will repair itself), is read again
      // after a pause
      uint32_t spins = 0;
      int verdict = 0;  // 1 done, 2 retry, 3 repair self
      uint64_t acc = 0;
      uint32_t pred_x = kPosDead;
      while (true) {
        int64_t base = (int64_t)tile - 1;
        uint32_t need_x = h0;  // exit the next-older tile must have
        bool self_ok = true;
        acc = 0;
        while (true) {
          const int64_t idx = base - lane;
          const bool inr = idx >= (int64_t)first;
          uint64_t s1 = 0, cnt = 0;
          uint2 ax = make_uint2(0, 0);
          bool ready = true, incl = false;
          if (inr) {
            if (PACK) {
              s1 = ld_volatile_u64(a.status + idx);
              const uint64_t f = status_flag(s1);
              ready = status_epoch(s1) == (epoch & 0xFFFFF) && (f == kFlagAggregate || f == kFlagInclusive);
              incl = ready && f == kFlagInclusive;
              const uint64_t v = status_value(s1);
              const uint32_t sS = (uint32_t)(idx - (int64_t)first) * SC, sE = min(sS + SC, rlen);
              const uint32_t xr = (uint32_t)v & 0xFFu;
              ax.y = xr == kXDead ? kPosDead : xr == kXEnd ? kPosEnd : sE + xr;
              if (incl) {
                cnt = v >> 8;
              } else {
                const uint32_t hr = (uint32_t)(v >> 8) & 0x1FFFFu;
                ax.x = hr == kRelDead ? kPosDead : hr == kRelEnd ? kPosEnd : sS + hr;
                cnt = v >> 25;
              }
            } else {
              // acquire loads keep the aux read between the two status reads
              s1 = ld_acquire_u64(a.status + idx);
              const uint64_t axw = ld_acquire_u64(reinterpret_cast<const uint64_t*>(a.aux + idx));
              ax = make_uint2((uint32_t)axw, (uint32_t)(axw >> 32));
              const uint64_t s2 = ld_volatile_u64(a.status + idx);
              const uint64_t f = status_flag(s1);
              ready = s1 == s2 && status_epoch(s1) == (epoch & 0xFFFFF) && (f == kFlagAggregate || f == kFlagInclusive);
              incl = ready && f == kFlagInclusive;
              cnt = status_value(s1);
            }
          }
          const uint32_t bi = __ballot_sync(0xffffffffu, incl);
          const int jstar = bi ? __ffs(bi) - 1 : 32;  // nearest inclusive of the window
          const bool relevant = inr && lane <= jstar;
          if (__any_sync(0xffffffffu, relevant && !ready)) {
            verdict = 2;
            break;
          }
          // the entry of lane l's tile must be the exit of the next older
          // tile (lane l + 1); the inclusive tile is already verified
          const uint32_t ox = __shfl_down_sync(0xffffffffu, ax.y, 1);
          bool bad = false;
          if (relevant && lane < jstar && lane < 31 && idx - 1 >= (int64_t)first)
            bad = (ox == kPosEnd) ? (ax.x != kPosEnd) : (ax.x != ox);
          if (__any_sync(0xffffffffu, bad)) {
            verdict = 2;
            break;
          }
          const uint32_t px = __shfl_sync(0xffffffffu, ax.y, 0);
          if (base == (int64_t)tile - 1) {
            // our own entry against the nearest predecessor's exit
            self_ok = (px == kPosEnd) ? (h0 == kPosEnd && K == 0) : (px == h0);
            pred_x = px;
          } else if (!((px == kPosEnd) ? (need_x == kPosEnd) : (px == need_x))) {
            // window boundary: the nearest of this window must exit where the
            // farthest of the previous window entered
            verdict = 2;
            break;
          }
          uint64_t v = relevant ? cnt : 0;
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          acc += v;
          const uint32_t far_h = __shfl_sync(0xffffffffu, ax.x, 31);
          if (jstar < 32 || base - 32 < (int64_t)first) {
            verdict = self_ok ? 1 : 3;
            break;
          }
          need_x = far_h;
          base -= 32;
        }
        if (verdict != 2) break;
        if (++spins > kSpinLimit) {
          if (lane == 0) atomicOr(a.err, kErrLookbackTimeout);
          break;
        }
        __nanosleep(200);
      }
      if (lane == 0) {
        s_misc[0] = (uint32_t)verdict;
        s_misc[1] = pred_x;
        s_val[0] = acc;
      }
    }
    __syncthreads();
    const int verdict = (int)s_misc[0];
    const uint32_t pred_x = s_misc[1];
    const uint64_t acc = s_val[0];
    __syncthreads();  // s_misc and s_val are reused below
    if (verdict == 3) {
      // our speculative entry was wrong: re-walk from the verified exit
      if (tid == 0) {
        if (PACK) {
          st_relaxed_u64(a.status + tile, make_status(epoch, kFlagRepair, 0));
        } else {
          st_release_u64(a.status + tile, make_status(epoch, kFlagRepair, 0));
          __threadfence();
        }
        s_h[0] = pred_x == kPosDead ? kPosEnd : kPosDead;  // differs from the entry: chunk 0 is re-walked
        rewalk_from(ch, s_h, s_x, s_k, 0, pred_x, nactive, scS, scE, C);
        atomicAdd(&a.counters[0], 1u);
      }
      __syncthreads();
      K = 0;
      for (int i = 0; i < NT; i++) K += s_k[i];
      h0 = s_h[0];
      xl = s_x[nactive - 1];
      if (tid == 0 && !PACK) {
        a.aux[tile] = make_uint2(h0, xl);
        __threadfence();
      }
    }
    prefix = acc;
    if (tid == 0) {
      if (PACK) {
        st_relaxed_u64(a.status + tile, make_status(epoch, kFlagInclusive, loc_word(prefix + K, h0, xl, scS, scE, true)));
      } else {
        st_release_u64(a.status + tile, make_status(epoch, kFlagInclusive, prefix + K));
      }
    }
  }
  // ---- header offsets of every block of every chunk ----
  uint32_t kx = s_k[tid];
  uint32_t incl_k = kx;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, incl_k, o);
    if (lane >= o) incl_k += y;
  }
  if (lane == 31) s_misc[warp] = incl_k;
  __syncthreads();
  uint32_t wex = 0;
  for (int w = 0; w < warp; w++) wex += s_misc[w];
  const uint64_t g0 = prefix + wex + (incl_k - kx);
  const uint64_t gb = seg_block_base(sg, t, FM2), nb = seg_blocks(sg, t, FM2);
  uint32_t p = s_h[tid];
  if (kx && p < rlen) {
    for (uint32_t i = 0; i < kx; i++) {
      const uint64_t gi = g0 + i;
      if (gi < nb) fd.blkpos[gb + gi] = p;
      const uint32_t sz = ch.step(p);
      if (!sz) break;
      p += sz;
    }
  }
  // the last CTA of a segment checks the block total
  if (tid == 0 && lt + 1 == fd.chunk_base[t + 1]) {
    const uint64_t total = prefix + K;
    const bool last_seg = t + 1 == sg.T;
    if (total < nb || (!last_seg && total != nb)) atomicOr(fd.err, kErrBlockCount);
  }
}

// ---------------------------------------------------------------------------
// 3. decode
// ---------------------------------------------------------------------------

// Delta of element j of a block whose bit-count byte is at hdr (m elements).
__device__ __forceinline__ uint32_t decode_delta(const uint8_t* __restrict__ hdr, uint32_t m, uint32_t bc,
                                                 uint32_t j) {
  const uint32_t ns = (m + 7) >> 3, B = bc >> 3, r = bc & 7;
  uint32_t neg = (__ldg(hdr + 1 + (j >> 3)) >> (7 - (j & 7))) & 1u;
  const uint8_t* bp = hdr + 1 + ns;
  uint32_t hi = 0;
  if (B) {
    const uint8_t* q = bp + j * B;
    hi = __ldg(q);
    if (B > 1) hi |= (uint32_t)__ldg(q + 1) << 8;
    if (B > 2) hi |= (uint32_t)__ldg(q + 2) << 16;
    if (B > 3) hi |= (uint32_t)__ldg(q + 3) << 24;
  }
  uint32_t lo = 0;
  if (r) {
    const uint8_t* rp = bp + B * m;
    uint32_t bit = j * r;
    uint32_t off = bit & 7;
    uint32_t w = (uint32_t)__ldg(rp + (bit >> 3)) << 8;
    if (off + r > 8) w |= __ldg(rp + (bit >> 3) + 1);
    lo = (w >> (16 - off - r)) & ((1u << r) - 1u);
  }
  uint32_t v = (B ? (hi << r) : 0u) | lo;
  return neg ? 0u - v : v;
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// (float)q * eb (szpd_float.cc:67,86,112).  NaN can only appear when eb is
// not finite; `special` (warp-uniform) selects the x86 NaN rule then.
__device__ __forceinline__ float dequant(uint32_t q, float eb, bool special = false) {
  float f = __int2float_rn((int32_t)q);
  float r = __fmul_rn(f, eb);
  return special ? x86_nan_fix(r, f, eb) : r;
}

// (double)q * eb for float64 streams (szpd_double.cc:67,86,112).
__device__ __forceinline__ double dequant(uint32_t q, double eb, bool special = false) {
  const double f = (double)(int32_t)q;
  const double r = __dmul_rn(f, eb);
  return special ? x86_nan_fix_d(r, f, eb) : r;
}

template <int WARPS>
__device__ __forceinline__ uint32_t scan_warps_u32(uint32_t* s_w, uint32_t mine, int warp, int lane,
                                                   uint32_t& excl) {
  if (lane == 0) s_w[warp] = mine;
  __syncthreads();
  if (warp == 0) {
    uint32_t x = lane < WARPS ? s_w[lane] : 0;
    uint32_t incl = warp_incl_scan(x, lane);
    if (lane < WARPS) s_w[lane] = incl - x;
    if (lane == 31) s_w[WARPS] = incl;
  }
  __syncthreads();
  excl = s_w[warp];
  return s_w[WARPS];
}

struct DecTile {
  uint32_t seg;
  uint64_t blk0;
  uint32_t nblk;
  bool first;
  bool any;
};

__device__ __forceinline__ DecTile dec_tile(const Segments& sg, uint32_t tile, uint32_t tiles_per_seg, uint32_t tb,
                                           bool fm2) {
  DecTile d;
  uint32_t t, ts;
  if (tiles_per_seg) {
    t = tile / tiles_per_seg;
    if (t > sg.T - 1) t = sg.T - 1;
    ts = tile - t * tiles_per_seg;
  } else {
    t = sg.T - 1;
    ts = tile;
  }
  uint64_t nb = seg_blocks(sg, t, fm2);
  d.seg = t;
  d.blk0 = (uint64_t)ts * tb;
  uint64_t rem = nb > d.blk0 ? nb - d.blk0 : 0;
  d.nblk = (uint32_t)(rem < tb ? rem : tb);
  d.first = ts == 0;
  d.any = sg.n > 0 && sg.len(t) > 0;
  return d;
}


constexpr int kDecWarps = 8;
constexpr int kDecRounds = 4;

// ---------------------------------------------------------------------------
// fastmode1 decode, blockSize L = 8*LPB, as a persistent, warp-specialised
// pipeline (the mirror of the compressor's):
//   producer  draws tile tickets; stages the tile's block offsets and its
//             stream span in a slot by bulk copy
//   compute   unpacks the deltas (LPB lanes per block, 8 elements per lane:
//             the byte layout of 8 elements is self-contained), scans them
//             inside the tile and stages the tile-relative prefix sums (int32)
//             in the slot, over the span they came from; then finishes the
//             previous tile: adds its base, dequantizes, 16-byte stores
//   control   looks back for each tile's base (the segment's seed plus the
//             deltas of the tiles before it, szpd_float.cc:76-118) while the
//             compute warps unpack the next tile
// ---------------------------------------------------------------------------
constexpr int kDecControl = 2;
// Slots of a decode pipeline with ROUNDS rounds per warp: a tile is finished
// (dequantized and stored) NS - 2 tiles after it was staged, so that its
// base (the look-back over the tiles before it) has that long to arrive.
// Tiles of 2 rounds (half the shared memory of 4) get 6 slots, 4 tiles of slack.
template <int ROUNDS>
__host__ __device__ constexpr int dec_slots() {
  return ROUNDS >= 4 ? 3 : 6;
}
constexpr int kDecPipeThreads = (8 + kDecControl + 1) * 32;

struct DecSlot {
  uint32_t tile;     // kStopTile: none
  uint32_t seg;
  uint32_t nblk;     // blocks in the tile
  uint32_t nel;      // elements of those blocks
  uint64_t e0;       // first element of the tile (its segment's lo + 1 + blk0*L)
  uint32_t first;    // first tile of its segment
  uint32_t seed;     // q of the segment's element lo (first tile only)
  uint32_t span0;    // region offset of span byte 0
  uint32_t spanlen;  // staged span bytes
  uint32_t sofs;     // slot byte offset of span byte 0
  uint32_t pofs;     // slot word offset of the tile's first block offset
  uint32_t seg_tile0;  // launch tile of its segment's first tile (the look-back stops there)
  float eb;          // the field's bound
  double ebd;        // float64 streams: the bound
  float* y;          // the field's output (float64 streams: its doubles)
  uint32_t* err;     // the field's error word
};

// Bytes of the block-offset area at the front of a slot.
__host__ __device__ constexpr uint32_t dec_pos_bytes(uint32_t tb) { return 4 * tb + 32; }

// Tile order of a decode pipeline launch.  A single field's launch is
// cooperative (a.static_tiles), so all its CTAs are resident and CTA c takes
// tiles c, c + grid, c + 2 grid, ...: the producer may run ahead as far as
// its slots allow, and a tile's predecessors are the tiles the other CTAs hold
// at the same time.  Batched launches, and a single field whose cooperative
// launch was refused, draw tickets (a tile's predecessors have then started
// before it).
template <uint32_t L, uint32_t TB, int NS, bool BATCH, bool FM2>
__device__ __forceinline__ void dec_producer(const DecArgs& a, uint8_t* slots, uint32_t slot_bytes, DecSlot* meta,
                                             uint64_t* full, uint64_t* empty, uint32_t* s_epoch,
                                             volatile uint32_t* s_stop_k, const volatile uint32_t* s_started) {
  constexpr uint32_t PB = dec_pos_bytes(TB);
  *s_epoch = *(volatile uint32_t*)&a.ls->epoch;
  __threadfence();
  // the plan of a single field and the region of the current segment, read once
  uint32_t bad = 0, cseg = 0xFFFFFFFFu;
  float eb = 0.0f;
  double ebd = 0.0;
  if (!BATCH) {
    bad = a.f.plan->bad;
    eb = a.f.plan->eb;
    ebd = a.f.plan->ebd;
  }
  uint64_t R0 = 0;
  uint32_t rlen = 0;
  for (uint32_t k = 0, j = 0;; j++) {
    const int s = (int)(k % NS);
    if (k >= (uint32_t)NS) mbar_wait_or_flag(&empty[s], ((k / NS) - 1) & 1, a.err);
    uint32_t tile;
    if (BATCH || !a.static_tiles) {
      // draw the ticket only once the compute warps have started the previous
      // position: a tile's predecessors are then never more than a tile behind it
      // in their work, which keeps the look-back short
      for (uint32_t i = 0; i < kWaitLimit && *s_started < k; i++) __nanosleep(64);
      tile = draw_ticket_persistent(a.ls, a.ntiles);
    } else {
      tile = blockIdx.x + j * gridDim.x;
      if (tile >= a.ntiles) {
        // the last CTA to stop advances the epoch (every CTA has read it)
        const uint32_t t = atomicAdd(&a.ls->ticket, 1u);
        if (t == gridDim.x - 1) {
          a.ls->ticket = 0;
          __threadfence();
          atomicAdd(&a.ls->epoch, 1u);
        }
      }
    }
    DecSlot& m = meta[s];
    if (tile >= a.ntiles) {
      drain_copies<NS>(full, k);
      m.tile = kStopTile;
      *s_stop_k = k;
      mbar_arrive(&full[s]);
      return;
    }
    const DecField& fd = BATCH ? a.fields[a.tile_field[tile]] : a.f;
    const Segments sg = fd.seg;
    const DecTile dt = dec_tile(sg, tile - fd.tile_base, fd.tiles_per_seg, TB, FM2);
    if (BATCH) bad = fd.plan->bad;
    // nothing to write: a failed plan, an empty segment, a tile past its segment's blocks
    // (fastmode1 keeps a segment's first tile for its seed)
    if (bad || !dt.any || (dt.nblk == 0 && (FM2 || !dt.first))) continue;  // the slot stays free
    const uint64_t lo = sg.lo(dt.seg), hi = sg.hi(dt.seg);
    if (BATCH || dt.seg != cseg) {
      R0 = fd.reg0[dt.seg];
      rlen = (uint32_t)(fd.reg1[dt.seg] - R0);
      cseg = dt.seg;
    }
    uint8_t* slot = slots + (size_t)s * slot_bytes;
    m.seg = dt.seg;
    m.seg_tile0 = fd.tile_base + (fd.tiles_per_seg ? dt.seg * fd.tiles_per_seg : 0u);
    m.eb = BATCH ? fd.plan->eb : eb;
    m.ebd = BATCH ? fd.plan->ebd : ebd;
    m.y = fd.y;
    m.err = fd.err;
    m.nblk = dt.nblk;
    m.first = dt.first;
    m.e0 = FM2 ? lo + dt.blk0 * L : lo + 1 + dt.blk0 * L;  // fastmode2 blocks start with their seed
    m.nel = dt.nblk ? (uint32_t)min((uint64_t)dt.nblk * L, hi - m.e0) : 0u;
    m.seed = 0;
    if (!FM2 && dt.first) {
      const uint8_t* sp = fd.in + R0 - 4;  // the segment's 4-byte seed precedes its blocks
      m.seed = (uint32_t)__ldg(sp) | ((uint32_t)__ldg(sp + 1) << 8) | ((uint32_t)__ldg(sp + 2) << 16) |
               ((uint32_t)__ldg(sp + 3) << 24);
    }
    m.span0 = 0;
    m.spanlen = 0;
    m.sofs = PB;
    m.pofs = 0;
    uint32_t tx = 0;
    uintptr_t p0 = 0, p1 = 0, q0 = 0, q1 = 0;
    if (dt.nblk) {
      const uint32_t* bp = fd.blkpos + seg_block_base(sg, dt.seg, FM2) + dt.blk0;
      const uint32_t s0 = min(__ldg(bp), rlen);
      uint32_t s1 = (uint32_t)min((uint64_t)rlen, (uint64_t)__ldg(bp + dt.nblk - 1) + a.maxsz);
      if (s1 < s0) s1 = s0;
      m.span0 = s0;
      m.spanlen = min(s1 - s0, TB * a.maxsz);  // bounds a corrupt index to the slot
      p0 = (uintptr_t)bp;
      p1 = p0 + 4ull * dt.nblk;
      m.pofs = (uint32_t)((p0 & 15) >> 2);
      tx += stage_range(slot, reinterpret_cast<const uint8_t*>(fd.blkpos), 4 * fd.nblk_total, p0, p1);
      q0 = (uintptr_t)(fd.in + R0 + s0);
      q1 = q0 + m.spanlen;
      m.sofs = PB + (uint32_t)(q0 & 15);
      tx += stage_range(slot + PB, fd.in, fd.len, q0, q1);
    }
    m.tile = tile;
    if (tx) {
      fence_async_smem();
      mbar_arrive_expect_tx(&full[s], tx);
      stage_range_issue(slot, reinterpret_cast<const uint8_t*>(fd.blkpos), 4 * fd.nblk_total, p0, p1, &full[s]);
      stage_range_issue(slot + PB, fd.in, fd.len, q0, q1, &full[s]);
    } else {
      mbar_arrive(&full[s]);
    }
    k++;
  }
}

// All ones when byte k of w has its top bit set, else 0 (prmt's sign
// replication; the __byte_perm intrinsic takes only the selector's low 3 bits).
__device__ __forceinline__ uint32_t prmt_sign(uint32_t w, int k) {
  uint32_t r;
  switch (k) {
    case 0: asm("prmt.b32 %0, %1, 0, 0x8888;" : "=r"(r) : "r"(w)); break;
    case 1: asm("prmt.b32 %0, %1, 0, 0x9999;" : "=r"(r) : "r"(w)); break;
    case 2: asm("prmt.b32 %0, %1, 0, 0xAAAA;" : "=r"(r) : "r"(w)); break;
    default: asm("prmt.b32 %0, %1, 0, 0xBBBB;" : "=r"(r) : "r"(w)); break;
  }
  return r;
}

// Little-endian bytes [o, o+8) of shared array b as (lo, hi), from three
// aligned 32-bit loads and two funnel shifts (reads b[o&~3 .. (o&~3)+12)).
__device__ __forceinline__ void lds_le64(const uint8_t* b, uint32_t o, uint32_t& lo, uint32_t& hi) {
  const uint32_t* w = reinterpret_cast<const uint32_t*>(b + (o & ~3u));
  const uint32_t sh = (o & 3u) * 8u;
  const uint32_t w0 = w[0], w1 = w[1], w2 = w[2];
  lo = __funnelshift_r(w0, w1, sh);
  hi = __funnelshift_r(w1, w2, sh);
}

// The aligned middle of cta_dequant_store, compiled per 16-byte phase PH of
// dst and per SPECIAL (eb not finite: the x86 NaN rule is applied): output
// chunk c (4 floats) takes stage words [4c - PH, 4c - PH + 4), picked from
// two aligned lines by fixed register moves.
template <bool CODES, bool ACC, int PH, bool SPECIAL>
__device__ __forceinline__ void cta_dequant_chunks(float* __restrict__ g0, const uint32_t* __restrict__ stage,
                                                   uint32_t c0, uint32_t c1, uint32_t base, float eb, bool& wrap,
                                                   uint32_t tid) {
  auto dq = [eb](uint32_t q) -> float { return CODES ? __uint_as_float(q) : dequant(q, eb, SPECIAL); };
  auto acc = [&wrap](float old, uint32_t q) -> float {  // old + q as int32 codes
    const int32_t x = (int32_t)__float_as_uint(old), y = (int32_t)q;
    const int32_t z = (int32_t)((uint32_t)x + (uint32_t)y);
    wrap |= ((x ^ z) & (y ^ z)) < 0;
    return __uint_as_float((uint32_t)z);
  };
  const uint4* s4 = reinterpret_cast<const uint4*>(stage);
  // four chunks per thread per pass: their shared-memory loads are in flight together
  constexpr int U = 4;
  for (uint32_t cb = c0; cb < c1; cb += 256 * U) {
    uint4 w[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const uint32_t c = min(cb + tid + 256 * u, c1 - 1);  // clamped: always a readable chunk
      if constexpr (PH == 0) {
        w[u] = s4[c];
      } else {
        const uint4 a = s4[c - 1], b = s4[c];  // stage words [4c-4, 4c+4)
        const uint32_t v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        w[u] = make_uint4(v[4 - PH], v[5 - PH], v[6 - PH], v[7 - PH]);
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const uint32_t c = cb + tid + 256 * u;
      if (c < c1) {
        float4 o;
        if (ACC) {
          const float4 p = reinterpret_cast<const float4*>(g0)[c];
          o.x = acc(p.x, base + w[u].x);
          o.y = acc(p.y, base + w[u].y);
          o.z = acc(p.z, base + w[u].z);
          o.w = acc(p.w, base + w[u].w);
        } else {
          o.x = dq(base + w[u].x);
          o.y = dq(base + w[u].y);
          o.z = dq(base + w[u].z);
          o.w = dq(base + w[u].w);
        }
        reinterpret_cast<float4*>(g0)[c] = o;
      }
    }
  }
}

// The 256 compute threads: y[e] = dequant(base + stage[e - e0]) for the
// tile's nel elements starting at dst = y + e0; 16-byte stores for the aligned
// middle (cta_dequant_chunks), plain stores at the ragged ends.  stage is
// 16-byte aligned and readable for nel + 4 words.
// CODES: the quantization codes themselves are stored (their bits), for the
// homomorphic reduction; with ACC they are added to the codes already in dst
// (wrapping int32; a wrap sets kErrQuantRange in *err).
template <bool CODES = false, bool ACC = false>
__device__ __forceinline__ void cta_dequant_store(float* __restrict__ dst, const uint32_t* __restrict__ stage,
                                                  uint32_t nel, uint32_t base, float eb, bool ebsp,
                                                  uint32_t* err = nullptr) {
  auto dq = [eb, ebsp](uint32_t q) -> float { return CODES ? __uint_as_float(q) : dequant(q, eb, ebsp); };
  bool wrap = false;
  auto acc = [&wrap](float old, uint32_t q) -> float {  // old + q as int32 codes
    const int32_t x = (int32_t)__float_as_uint(old), y = (int32_t)q;
    const int32_t z = (int32_t)((uint32_t)x + (uint32_t)y);
    wrap |= ((x ^ z) & (y ^ z)) < 0;
    return __uint_as_float((uint32_t)z);
  };
  auto put = [&](float* p, uint32_t q) { *p = ACC ? acc(*p, q) : dq(q); };
  const uint32_t tid = threadIdx.x;
  if (nel == 0) return;
  const uint32_t ph = (uint32_t)(((uintptr_t)dst >> 2) & 3);
  float* g0 = dst - ph;  // 16-byte aligned
  const uint32_t end = ph + nel;
  const uint32_t c0 = (ph + 3) >> 2, c1 = end >> 2;  // whole float4 chunks [c0, c1)
  if (c0 >= c1) {
    if (tid < nel) put(g0 + ph + tid, base + stage[tid]);
  } else {
    if (tid < 4 * c0 - ph) put(g0 + ph + tid, base + stage[tid]);
    if (tid >= 32 && tid - 32 < end - 4 * c1) put(g0 + 4 * c1 + tid - 32, base + stage[4 * c1 + tid - 32 - ph]);
    if (!CODES && ebsp) {  // eb not finite
      switch (ph) {
        case 0: cta_dequant_chunks<CODES, ACC, 0, true>(g0, stage, c0, c1, base, eb, wrap, tid); break;
        case 1: cta_dequant_chunks<CODES, ACC, 1, true>(g0, stage, c0, c1, base, eb, wrap, tid); break;
        case 2: cta_dequant_chunks<CODES, ACC, 2, true>(g0, stage, c0, c1, base, eb, wrap, tid); break;
        default: cta_dequant_chunks<CODES, ACC, 3, true>(g0, stage, c0, c1, base, eb, wrap, tid); break;
      }
    } else {
      switch (ph) {
        case 0: cta_dequant_chunks<CODES, ACC, 0, false>(g0, stage, c0, c1, base, eb, wrap, tid); break;
        case 1: cta_dequant_chunks<CODES, ACC, 1, false>(g0, stage, c0, c1, base, eb, wrap, tid); break;
        case 2: cta_dequant_chunks<CODES, ACC, 2, false>(g0, stage, c0, c1, base, eb, wrap, tid); break;
        default: cta_dequant_chunks<CODES, ACC, 3, false>(g0, stage, c0, c1, base, eb, wrap, tid); break;
      }
    }
  }
  if (ACC && wrap) atomicOr(err, kErrQuantRange);
}

// (double)q * eb of float64 data as bits: integer arithmetic for every eb
// whose products stay normal (szp_f64.h), the FP64 multiply otherwise.
struct DequantD {
  uint64_t m, sgn;
  uint32_t ef;
  bool fast, special;
  double eb;
  __device__ __forceinline__ explicit DequantD(double e) : eb(e) {
    const uint64_t u = f64i::bits_of(e);
    fast = f64i::dequant_fast_ok(u);
    special = !isfinite(e);
    m = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    ef = (uint32_t)(u >> 52) & 0x7FFu;
    sgn = u & 0x8000000000000000ull;
  }
  __device__ __forceinline__ unsigned long long operator()(uint32_t q) const {
    return fast ? f64i::dequant_bits((int32_t)q, m, ef, sgn) : f64i::bits_of(dequant(q, eb, special));
  }
};

// cta_dequant_store for float64 data: y[e] = (double)(base + stage[e - e0]) * eb
// for the tile's nel elements from dst = y + e0, 16-byte stores of two
// results (the first result alone when dst is 8 bytes past a 16-byte
// boundary), written as bits.
__device__ __forceinline__ void cta_dequant_store_d(double* __restrict__ dst, const uint32_t* __restrict__ stage,
                                                    uint32_t nel, uint32_t base, double eb) {
  if (nel == 0) return;
  const DequantD dq(eb);
  const uint32_t tid = threadIdx.x;
  unsigned long long* g = reinterpret_cast<unsigned long long*>(dst);
  const uint32_t ph = (uint32_t)(((uintptr_t)dst >> 3) & 1);  // results before the first 16-byte boundary
  if (ph && tid == 0) g[0] = dq(base + stage[0]);
  const uint32_t n2 = (nel - ph) >> 1;
  ulonglong2* g2 = reinterpret_cast<ulonglong2*>(g + ph);
  for (uint32_t c = tid; c < n2; c += 256) {
    const uint32_t e = ph + 2 * c;
    g2[c] = make_ulonglong2(dq(base + stage[e]), dq(base + stage[e + 1]));
  }
  if (((nel - ph) & 1) && tid == 32) g[nel - 1] = dq(base + stage[nel - 1]);
}

// Control warp c: tiles c, c + kDecControl, ... of this CTA.  Finds each
// tile's base q (the segment's seed plus the deltas of the tiles before it) and
// hands it to the compute warps, which finish the tile.
// Output kinds of the decode pipeline: floats, doubles (float64 streams,
// dequantized in integer arithmetic, see DequantD), the int32 codes, or the
// codes added to those already in y (the homomorphic reduction).
enum { kOutFloat = 0, kOutDouble = 1, kOutCodes = 2, kOutCodesAdd = 3 };

template <int NS, int NC, int OUT = kOutFloat>
__device__ __forceinline__ void dec_control(int c, const DecArgs& a, const DecSlot* meta, const uint32_t* s_agg,
                                            uint32_t* s_base, uint64_t* full, uint64_t* aggb, uint64_t* based,
                                            const uint32_t* s_epoch, const volatile uint32_t* s_stop_k) {
  const int lane = threadIdx.x & 31;
  for (uint32_t k = (uint32_t)c;; k += NC) {
    const int s = (int)(k % NS);
    const uint32_t par = (k / NS) & 1;
    if (!control_wait_full(&full[s], par, k, s_stop_k, a.err)) return;
    const uint32_t tile = meta[s].tile;
    if (tile >= a.ntiles) return;
    const bool first = meta[s].first;
    mbar_wait_or_flag(&aggb[s], par, a.err);
    const uint32_t agg = s_agg[s];
    const uint32_t epoch = *s_epoch;
    uint32_t base;
    if (first) {
      base = meta[s].seed;
      if (lane == 0) {
        const float eb = meta[s].eb;
        if (OUT == kOutDouble) {
          reinterpret_cast<unsigned long long*>(meta[s].y)[meta[s].e0 - 1] = DequantD(meta[s].ebd)(base);
        } else if (OUT == kOutCodes) {
          meta[s].y[meta[s].e0 - 1] = __uint_as_float(base);
        } else if (OUT == kOutCodesAdd) {
          float* p = meta[s].y + meta[s].e0 - 1;
          const int32_t x = (int32_t)__float_as_uint(*p), z = (int32_t)((uint32_t)x + base);
          *p = __uint_as_float((uint32_t)z);
          if (((x ^ z) & ((int32_t)base ^ z)) < 0) atomicOr(meta[s].err, kErrQuantRange);
        } else {
          meta[s].y[meta[s].e0 - 1] = dequant(base, eb, !isfinite(eb));
        }
      }
    } else {
      base = (uint32_t)lookback_sum(a.status, tile, meta[s].seg_tile0, epoch, a.err);
      if (lane == 0) st_relaxed_u64(a.status + tile, make_status(epoch, kFlagInclusive, (uint32_t)(base + agg)));
    }
    if (lane == 0) {
      s_base[s] = base;
      mbar_arrive(&based[s]);
    }
    __syncwarp();
  }
}

// OUT: what y holds (kOutFloat, kOutDouble: an array of doubles, kOutCodes:
// int32 codes).
template <int LPB, bool BATCH, int ROUNDS, bool FM2 = false, int OUT = kOutFloat>
__global__ void __launch_bounds__(kDecPipeThreads, 2) decode_pipe(const __grid_constant__ DecArgs a,
                                                                  uint32_t slot_bytes) {
  constexpr int NS = dec_slots<ROUNDS>(), NC = kDecControl, WARPS = 8;
  constexpr uint32_t DEFER = NS - 2;  // fastmode1: tiles between staging a tile and finishing it
  // a control warp's next position must never share a slot phase it has not
  // waited for (an mbarrier parity names one of two phases)
  static_assert(NC <= NS, "more control warps than slots");
  constexpr uint32_t L = 8 * LPB;
  constexpr int BPR = 32 / LPB;
  constexpr uint32_t TB = WARPS * ROUNDS * BPR;
  constexpr uint32_t PB = dec_pos_bytes(TB);
  extern __shared__ __align__(16) uint8_t s_slots[];
  __shared__ DecSlot s_meta[NS];
  __shared__ uint32_t s_agg[NS];
  __shared__ uint32_t s_w[WARPS + 1];
  __shared__ uint32_t s_epoch;
  __shared__ volatile uint32_t s_stop_k;
  __shared__ volatile uint32_t s_started;
  __shared__ uint32_t s_base[NS];
  __shared__ __align__(8) uint64_t s_full[NS], s_aggb[NS], s_based[NS], s_empty[NS];

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x < NS) s_meta[threadIdx.x].tile = kStopTile;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; s++) {
      mbar_init(&s_full[s], 1);
      mbar_init(&s_aggb[s], 1);
      mbar_init(&s_based[s], 1);
      mbar_init(&s_empty[s], 1);
    }
    s_stop_k = kStopTile;
    s_started = 0;
  }
  __syncthreads();
  if (warp == WARPS + NC) {
    if (lane == 0)
      dec_producer<L, TB, NS, BATCH, FM2>(a, s_slots, slot_bytes, s_meta, s_full, s_empty, &s_epoch, &s_stop_k,
                                          &s_started);
    return;
  }
  if (warp >= WARPS) {
    // fastmode2 blocks carry their own seeds: no look-back, nothing to control
    if (!FM2)
      dec_control<NS, NC, OUT>(warp - WARPS, a, s_meta, s_agg, s_base, s_full, s_aggb, s_based, &s_epoch, &s_stop_k);
    return;
  }

  // ---- compute warps ----
  // Tile k is unpacked and staged, then tile k - DEFER (whose base the
  // control warps have looked up meanwhile) is finished: base added,
  // dequantized, stored.
  const int sub = lane % LPB, grp = lane / LPB;
  const uint32_t wfirst = (uint32_t)warp * ROUNDS * BPR;
  auto finish = [&](uint32_t kp) {
    const int sp_ = (int)(kp % NS);
    mbar_wait_or_flag(&s_based[sp_], (kp / NS) & 1, a.err);
    const float ebp = s_meta[sp_].eb;
    const uint32_t* stage = reinterpret_cast<const uint32_t*>(s_slots + (size_t)sp_ * slot_bytes + PB);
    if (OUT == kOutDouble) {
      cta_dequant_store_d(reinterpret_cast<double*>(s_meta[sp_].y) + s_meta[sp_].e0, stage, s_meta[sp_].nel,
                          s_base[sp_], s_meta[sp_].ebd);
    } else {
      cta_dequant_store<OUT >= kOutCodes, OUT == kOutCodesAdd>(s_meta[sp_].y + s_meta[sp_].e0, stage,
                                                               s_meta[sp_].nel, s_base[sp_], ebp, !isfinite(ebp),
                                                               s_meta[sp_].err);
    }
    compute_sync();  // every read of the slot is done
    if (threadIdx.x == 0) mbar_arrive(&s_empty[sp_]);
  };
  for (uint32_t k = 0;; k++) {
    const int s = (int)(k % NS);
    const uint32_t par = (k / NS) & 1;
    mbar_wait_or_flag(&s_full[s], par, a.err);
    const uint32_t tile = s_meta[s].tile;
    if (threadIdx.x == 0) s_started = k + 1;
    if (tile >= a.ntiles) {
      if (!FM2)  // fastmode2 tiles are finished at once
        for (uint32_t j = k > DEFER ? k - DEFER : 0u; j < k; j++) finish(j);
      return;
    }
    const uint32_t nblk = s_meta[s].nblk, nel = s_meta[s].nel, span0 = s_meta[s].span0;
    const uint32_t spanlen = s_meta[s].spanlen;
    uint8_t* slot = s_slots + (size_t)s * slot_bytes;
    const uint8_t* sp = slot + s_meta[s].sofs;  // span byte i at sp[i]
    const uint32_t* bpos = reinterpret_cast<const uint32_t*>(slot) + s_meta[s].pofs;

    // ---- unpack deltas and prefix-add inside each lane ----
    uint32_t pre[ROUNDS][8];
    uint32_t lex[ROUNDS], rbase[ROUNDS];
    uint32_t seedv[ROUNDS];  // fastmode2: each block's seed
    uint32_t wtot = 0;
    bool corrupt = false;
    // FULL: a fastmode1 tile of TB whole blocks (every tile of a segment but
    // its last); its rounds skip the per-block element counts
    auto unpack = [&](auto fullc) {
    constexpr bool FULL = decltype(fullc)::value;
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
      const uint32_t bt = wfirst + r * BPR + grp;
      const uint32_t mblk = FULL ? L : (bt < nblk ? min(L, nel - bt * L) : 0u);
      const uint32_t m = FM2 ? (mblk ? mblk - 1 : 0u) : mblk;  // values packed in the block
      const uint32_t ml = FULL ? 8u : (m > 8u * sub ? min(8u, m - 8u * sub) : 0u);
      uint32_t d[8];
#pragma unroll
      for (int j = 0; j < 8; j++) d[j] = 0;
      uint32_t off = 0, bc = 0;
      seedv[r] = 0;
      if (FULL) {
        // a corrupt offset is kept inside the slot; a block of bit count b
        // takes 1 + (L/8)(b+1) bytes (1 when b = 0)
        off = min(bpos[bt] - span0, spanlen);
        bc = sp[off];
        if (bc > 33 || off + (bc ? 1 + (L / 8) * (bc + 1) : 1u) > spanlen) {
          corrupt = true;
          bc = 0;
        }
      } else if (FM2 && mblk) {
        // fastmode2: the block's 4-byte seed, then its header (a one-element
        // block has no header on the decode side, szpd_float.cc:483)
        const uint32_t b0 = bpos[bt] - span0;
        if (b0 + 4 > spanlen) {
          corrupt = true;
        } else {
          seedv[r] = (uint32_t)sp[b0] | ((uint32_t)sp[b0 + 1] << 8) | ((uint32_t)sp[b0 + 2] << 16) |
                     ((uint32_t)sp[b0 + 3] << 24);
        }
        off = b0 + 4;
        if (m) {
          bc = off < spanlen ? sp[off] : 255u;
          if (bc > 33 || off + block_bytes(m, bc) > spanlen) {
            corrupt = true;
            bc = 0;
          }
        }
      } else if (!FM2 && m) {
        off = bpos[bt] - span0;
        bc = off < spanlen ? sp[off] : 255u;
        if (bc > 33 || off + block_bytes(m, bc) > spanlen) {
          corrupt = true;
          bc = 0;
        }
      }
      constexpr uint32_t MF = FM2 ? L - 1 : L;  // values of a full block
      if (__all_sync(0xffffffffu, (FULL || m == MF || m == 0) && bc <= 15)) {
        // every block of the round is full and has at most one byte plane:
        // the lane's plane and remainder bytes come from aligned word loads
        // (fastmode2: L-1 values, the last lane's eighth is not one of them)
        if (bc) {
          constexpr uint32_t NSB = L / 8;  // sign bytes, ceil(MF / 8) either way
          const uint32_t B = bc >> 3, rr = bc & 7;
          const uint32_t ob = (uint32_t)(sp - s_slots) + off;  // the block in s_slots
          const uint32_t sb = s_slots[ob + 1 + sub];             // sign bits, szp_TypeManager.cc:820-844
          uint32_t lo, hi, plo = 0, phi = 0;
          lds_le64(s_slots, ob + 1 + NSB + B * MF + rr * sub, lo, hi);  // remainder, szp_TypeManager.cc:122-434
          if (B) lds_le64(s_slots, ob + 1 + NSB + 8 * sub, plo, phi);  // byte plane, szp_TypeManager.cc:36-52
          const uint32_t t = __byte_perm(lo, 0, 0x0123);  // remainder bits 0..31, MSB first
          const uint32_t t2 = __funnelshift_l(__byte_perm(hi, 0, 0x0123), t, 4 * rr);  // bits 4rr..
          // byte k of sw0 (sw1) has the sign bit of value k (4 + k) as its top bit
          const uint32_t sw0 = sb * 0x08040201u, sw1 = (sb << 4) * 0x08040201u;
#pragma unroll
          for (int j = 0; j < 8; j++) {
            // value j: its plane byte above its rr remainder bits, in one funnel shift
            const uint32_t h = __byte_perm(j < 4 ? plo : phi, 0, 0x4440 + (j & 3));
            const uint32_t v = __funnelshift_l((j < 4 ? t : t2) << (rr * (j & 3)), h, rr);
            const uint32_t sg = prmt_sign(j < 4 ? sw0 : sw1, j & 3);  // 0 or all ones
            d[j] = (FM2 && j == 7 && sub == LPB - 1) ? 0u : (v ^ sg) - sg;
          }
        }
      } else if (m) {
        if (bc && ml) {
          const uint32_t ns = (m + 7) >> 3, B = bc >> 3, rr = bc & 7;
          const uint32_t sb = sp[off + 1 + sub];  // sign bits, szp_TypeManager.cc:820-844
          uint32_t hv[8];
#pragma unroll
          for (int j = 0; j < 8; j++) hv[j] = 0;
          if (B) {  // byte planes, szp_TypeManager.cc:36-52
            const uint8_t* q8 = sp + off + 1 + ns + 8 * B * sub;
#pragma unroll
            for (int j = 0; j < 8; j++) {
              if ((uint32_t)j < ml) {
                uint32_t h = q8[j * B];
                if (B > 1) h |= (uint32_t)q8[j * B + 1] << 8;
                if (B > 2) h |= (uint32_t)q8[j * B + 2] << 16;
                if (B > 3) h |= (uint32_t)q8[j * B + 3] << 24;
                hv[j] = h << rr;
              }
            }
          }
          if (rr) {  // remainder bits, MSB first, szp_TypeManager.cc:122-434
            const uint8_t* rp = sp + off + 1 + ns + B * m + rr * sub;
            const uint32_t nb = (ml * rr + 7) >> 3;
            uint64_t acc = 0;
#pragma unroll
            for (uint32_t kk = 0; kk < 7; kk++) acc = (acc << 8) | (uint64_t)(kk < nb ? rp[kk] : 0u);
            // 56-bit window: field j occupies bits [56 - rr*(j+1), 56 - rr*j)
            const uint32_t mask = (1u << rr) - 1u;
#pragma unroll
            for (int j = 0; j < 8; j++) hv[j] |= (uint32_t)(acc >> (56 - rr * (j + 1))) & mask;
          }
#pragma unroll
          for (int j = 0; j < 8; j++) {
            const uint32_t v = (uint32_t)j < ml ? hv[j] : 0u;
            d[j] = ((sb >> (7 - j)) & 1u) ? 0u - v : v;
          }
        }
      }
      uint32_t run = 0;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        run += d[j];
        pre[r][j] = run;
      }
      lex[r] = run;
    }
    };
    if (!FM2 && nblk == TB && nel == TB * L) {
      unpack(std::true_type{});
    } else {
      unpack(std::false_type{});
    }
    if constexpr (FM2) {
      // every block restarts from its seed: a scan over the block's LPB lanes,
      // the values staged, then the tile finished at once
#pragma unroll
      for (int r = 0; r < ROUNDS; r++) {
        uint32_t incl = lex[r];
#pragma unroll
        for (int o = 1; o < LPB; o <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o, LPB);
          if (sub >= o) incl += y;
        }
        lex[r] = incl - lex[r];
      }
      if (__any_sync(0xffffffffu, corrupt) && lane == 0) atomicOr(s_meta[s].err, kErrCorrupt);
      compute_sync();  // every read of the span is done
      uint32_t* stage = reinterpret_cast<uint32_t*>(slot + PB);
#pragma unroll
      for (int r = 0; r < ROUNDS; r++) {
        const uint32_t bt = wfirst + r * BPR + grp;
        const uint32_t mblk = bt < nblk ? min(L, nel - bt * L) : 0u;
        const uint32_t m = mblk ? mblk - 1 : 0u;
        const uint32_t ml = m > 8u * sub ? min(8u, m - 8u * sub) : 0u;
        if (mblk && sub == 0) stage[bt * L] = seedv[r];
        const uint32_t q0 = seedv[r] + lex[r];
        const uint32_t k1 = bt * L + 1 + 8 * sub;
#pragma unroll
        for (int j = 0; j < 8; j++)
          if ((uint32_t)j < ml) stage[k1 + j] = q0 + pre[r][j];
      }
      compute_sync();
      const float ebp = s_meta[s].eb;
      if (OUT == kOutDouble) {
        cta_dequant_store_d(reinterpret_cast<double*>(s_meta[s].y) + s_meta[s].e0, stage, nel, 0u, s_meta[s].ebd);
      } else {
        cta_dequant_store<OUT >= kOutCodes, OUT == kOutCodesAdd>(s_meta[s].y + s_meta[s].e0, stage, nel, 0u, ebp,
                                                                 !isfinite(ebp), s_meta[s].err);
      }
      compute_sync();  // every read of the slot is done
      if (threadIdx.x == 0) mbar_arrive(&s_empty[s]);
      continue;
    }
    // the rounds' warp scans, interleaved: four independent shuffle chains
    {
      uint32_t incl[ROUNDS];
#pragma unroll
      for (int r = 0; r < ROUNDS; r++) incl[r] = lex[r];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int r = 0; r < ROUNDS; r++) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, incl[r], o);
          if (lane >= o) incl[r] += y;
        }
      }
#pragma unroll
      for (int r = 0; r < ROUNDS; r++) {
        lex[r] = incl[r] - lex[r];
        rbase[r] = wtot;
        wtot += __shfl_sync(0xffffffffu, incl[r], 31);
      }
    }
    if (__any_sync(0xffffffffu, corrupt) && lane == 0) atomicOr(s_meta[s].err, kErrCorrupt);

    // ---- tile scan over the warps (its first barrier ends every read of the span) ----
    if (lane == 0) s_w[warp] = wtot;
    compute_sync();
    uint32_t wexcl = 0, agg = 0;
#pragma unroll
    for (int w = 0; w < WARPS; w++) {
      const uint32_t t = s_w[w];
      wexcl += w < warp ? t : 0u;
      agg += t;
    }
    if (threadIdx.x == 0) {
      s_agg[s] = agg;
      const bool first = s_meta[s].first;
      const uint32_t v = first ? s_meta[s].seed + agg : agg;
      st_relaxed_u64(a.status + tile, make_status(s_epoch, first ? kFlagInclusive : kFlagAggregate, v));
      mbar_arrive(&s_aggb[s]);
    }

    // ---- stage the tile-relative prefix sums over the span ----
    uint32_t* stage = reinterpret_cast<uint32_t*>(slot + PB);
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
      const uint32_t bt = wfirst + r * BPR + grp;
      const uint32_t k0 = bt * L + 8 * sub;
      const uint32_t ml = (bt < nblk && k0 < nel) ? min(8u, nel - k0) : 0u;
      const uint32_t q0 = wexcl + rbase[r] + lex[r];
      if (ml == 8) {
        uint4* d4 = reinterpret_cast<uint4*>(stage + k0);
        d4[0] = make_uint4(q0 + pre[r][0], q0 + pre[r][1], q0 + pre[r][2], q0 + pre[r][3]);
        d4[1] = make_uint4(q0 + pre[r][4], q0 + pre[r][5], q0 + pre[r][6], q0 + pre[r][7]);
      } else {
#pragma unroll
        for (int j = 0; j < 8; j++)
          if ((uint32_t)j < ml) stage[k0 + j] = q0 + pre[r][j];
      }
    }
    compute_sync();  // staged; s_w is free for the next tile
    if (k >= DEFER) finish(k - DEFER);
  }
}

// Any blockSize, fastmode1 or fastmode2: one warp per block in 32-element
// pieces.  fastmode1 decodes twice (totals, then values after the look-back).
// V = float, or double for float64 streams (x' = (double)q * eb).
template <int WARPS, bool FM2, typename V = float>
__global__ void __launch_bounds__(WARPS * 32) decode_generic(const __grid_constant__ DecArgs a) {
  constexpr bool DBL = std::is_same<V, double>::value;
  const DecField& fd = a.f;
  __shared__ uint32_t s_tk[2];
  __shared__ uint32_t s_w[WARPS + 1];
  __shared__ uint32_t s_base;
  uint32_t tile, epoch;
  draw_ticket(a.ls, a.ntiles, tile, epoch, s_tk);
  if (fd.plan->bad) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Segments sg = fd.seg;
  const uint32_t L = sg.L;
  const uint32_t TB = WARPS * a.bpw;
  const DecTile dt = dec_tile(sg, tile, fd.tiles_per_seg, TB, FM2);
  if (!dt.any) return;
  V eb;
  if constexpr (DBL) eb = fd.plan->ebd;
  else eb = fd.plan->eb;
  const bool ebsp = !isfinite(eb);
  // float64: (double)q * eb in integer arithmetic for every eb whose
  // products stay normal (FP64 instructions are slow on this GPU)
  bool fastdq = false;
  uint64_t ebm = 0, ebs = 0;
  uint32_t ebe = 0;
  if constexpr (DBL) {
    const uint64_t u = f64i::bits_of(eb);
    fastdq = f64i::dequant_fast_ok(u);
    ebm = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    ebe = (uint32_t)(u >> 52) & 0x7FFu;
    ebs = u & 0x8000000000000000ull;
  }
  auto dq = [&](uint32_t q) -> V {
    if constexpr (DBL) {
      if (fastdq) return f64i::double_of(f64i::dequant_bits((int32_t)q, ebm, ebe, ebs));
    }
    return dequant(q, eb, ebsp);
  };
  V* __restrict__ yv = DBL ? reinterpret_cast<V*>(fd.yd) : reinterpret_cast<V*>(fd.y);
  const uint64_t lo = sg.lo(dt.seg), hi = sg.hi(dt.seg);
  const uint64_t R0 = fd.reg0[dt.seg], R1 = fd.reg1[dt.seg];
  const uint8_t* __restrict__ in = fd.in;
  const uint64_t gb = seg_block_base(sg, dt.seg, FM2);
  const uint32_t wfirst = warp * a.bpw;
  bool corrupt = false;

  // elements of block b: fastmode1 [lo+1+bL, +L), fastmode2 seed at lo+bL then L-1
  auto blk_start = [&](uint64_t b) -> uint64_t { return FM2 ? lo + b * L + 1 : lo + 1 + b * L; };
  auto blk_len = [&](uint64_t b) -> uint32_t {
    uint64_t s = blk_start(b);
    uint64_t e = s + (FM2 ? L - 1 : L);
    if (e > hi) e = hi;
    return e > s ? (uint32_t)(e - s) : 0u;
  };
  // block header pointer and validation; returns bc or 255 when corrupt
  auto blk_hdr = [&](uint64_t b, uint32_t m, uint64_t& hp) -> uint32_t {
    hp = R0 + __ldg(fd.blkpos + gb + b) + (FM2 ? 4 : 0);
    if (FM2 && m == 0) return 0;  // one-element block: no header is read (szpd_float.cc:483)
    if (hp >= R1) return 255u;
    uint32_t bc = __ldg(in + hp);
    if (bc > 33 || hp + block_bytes(m, bc) > R1) return 255u;
    return bc;
  };

  // fastmode1 decodes every delta twice (the warp's total, then the values
  // once its base is known); with blockSize <= 32 (one piece per block) and
  // at most KC blocks per warp, lane c fetches block c's position and header
  // byte, the deltas of all the warp's blocks are decoded with their loads
  // in flight together, and each lane keeps its deltas in registers
  constexpr int KC = 8;
  const bool cache = !FM2 && L <= 32 && a.bpw <= (uint32_t)KC;
  uint32_t cd[KC];
#pragma unroll
  for (int c = 0; c < KC; c++) cd[c] = 0;
  uint32_t q0 = 0;
  if (!FM2) {
    uint32_t wtot = 0;
    if (cache) {
      uint64_t hpl = 0;
      uint32_t bcl = 0, ml = 0;
      if ((uint32_t)lane < a.bpw && wfirst + lane < dt.nblk) {
        ml = blk_len(dt.blk0 + wfirst + lane);
        bcl = blk_hdr(dt.blk0 + wfirst + lane, ml, hpl);
        if (bcl == 255u) {
          corrupt = true;
          bcl = 0;
        }
      }
      uint32_t lsum = 0;
#pragma unroll
      for (int c = 0; c < KC; c++) {
        if ((uint32_t)c >= a.bpw || wfirst + c >= dt.nblk) break;
        const uint32_t bc = __shfl_sync(0xffffffffu, bcl, c), m = __shfl_sync(0xffffffffu, ml, c);
        const uint64_t hp = __shfl_sync(0xffffffffu, (unsigned long long)hpl, c);
        cd[c] = (bc && (uint32_t)lane < m) ? decode_delta(in + hp, m, bc, lane) : 0u;
        lsum += cd[c];
      }
      for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
      wtot = lsum;
    }
    for (uint32_t k = 0; !cache && k < a.bpw; k++) {
      uint32_t bi = wfirst + k;
      if (bi >= dt.nblk) break;
      uint64_t b = dt.blk0 + bi, hp;
      uint32_t m = blk_len(b);
      uint32_t bc = blk_hdr(b, m, hp);
      if (bc == 255u) {
        corrupt = true;
        continue;
      }
      if (!bc) continue;
      for (uint32_t p0 = 0; p0 < m; p0 += 32) {
        uint32_t j = p0 + lane;
        uint32_t d = j < m ? decode_delta(in + hp, m, bc, j) : 0u;
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        wtot += d;
      }
    }
    uint32_t wexcl;
    const uint32_t agg = scan_warps_u32<WARPS>(s_w, wtot, warp, lane, wexcl);
    const uint32_t first_tile = fd.tiles_per_seg ? dt.seg * fd.tiles_per_seg : 0;
    if (warp == 0) {
      uint32_t excl;
      if (dt.first) {
        const uint8_t* sp = in + R0 - 4;
        excl = (uint32_t)sp[0] | ((uint32_t)sp[1] << 8) | ((uint32_t)sp[2] << 16) | ((uint32_t)sp[3] << 24);
        if (lane == 0) {
          st_relaxed_u64(a.status + tile, make_status(epoch, kFlagInclusive, (uint32_t)(excl + agg)));
          yv[lo] = dq(excl);
        }
      } else {
        if (lane == 0) st_relaxed_u64(a.status + tile, make_status(epoch, kFlagAggregate, agg));
        excl = (uint32_t)lookback_sum(a.status, tile, first_tile, epoch, a.err);
        if (lane == 0) st_relaxed_u64(a.status + tile, make_status(epoch, kFlagInclusive, (uint32_t)(excl + agg)));
      }
      if (lane == 0) s_base = excl;
    }
    __syncthreads();
    q0 = s_base + wexcl;
  }

  for (uint32_t k = 0; k < a.bpw; k++) {
    uint32_t bi = wfirst + k;
    if (bi >= dt.nblk) break;
    uint64_t b = dt.blk0 + bi, hp;
    uint64_t s = blk_start(b);
    uint32_t m = blk_len(b);
    hp = 0;
    uint32_t bc = cache ? 0u : blk_hdr(b, m, hp);  // the cache holds the deltas
    if (bc == 255u) {
      corrupt = true;
      bc = 0;
    }
    if (FM2) {
      // blockSize 1: the reference's decoder reads no header byte for a
      // one-value block and so steps 4 bytes per block where its encoder
      // wrote 5 (szpd_float.cc:483, szpd_double.cc:487); results follow it
      const uint64_t so = L == 1 ? R0 + 4 * b : hp - 4;
      if (so + 4 > R1) {
        corrupt = true;
        q0 = 0;
      } else {
        const uint8_t* sp = in + so;
        q0 = (uint32_t)__ldg(sp) | ((uint32_t)__ldg(sp + 1) << 8) | ((uint32_t)__ldg(sp + 2) << 16) |
             ((uint32_t)__ldg(sp + 3) << 24);
      }
      if (lane == 0) yv[s - 1] = dq(q0);
    }
    uint32_t dk = 0;
    if (cache) {
#pragma unroll
      for (int c = 0; c < KC; c++)
        if ((uint32_t)c == k) dk = cd[c];
    }
    for (uint32_t p0 = 0; p0 < m; p0 += 32) {
      uint32_t j = p0 + lane;
      uint32_t d = cache ? dk : ((bc && j < m) ? decode_delta(in + hp, m, bc, j) : 0u);
      uint32_t sc = warp_incl_scan(d, lane);
      if (j < m) yv[s + j] = dq(q0 + sc);
      q0 += __shfl_sync(0xffffffffu, sc, 31);
    }
  }
  if (__any_sync(0xffffffffu, corrupt) && lane == 0) atomicOr(fd.err, kErrCorrupt);
}

static int dec_lanes_per_block(uint32_t L) {
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

uint32_t decode_blocks_per_tile(uint32_t L, uint32_t& bpw) {
  int lpb = dec_lanes_per_block(L);
  if (lpb) {
    bpw = kDecRounds * (32 / lpb);
    return kDecWarps * bpw;
  }
  uint32_t b = 2048u / (L < 32 ? 32u : L);
  bpw = b < 1 ? 1 : (b > 8 ? 8 : b);
  return kDecWarps * bpw;
}

size_t decode_smem_bytes(uint32_t L, uint32_t tb, bool fm2) {
  if (fm2 || !dec_lanes_per_block(L)) return 0;
  return (size_t)tb * max_block_bytes(L) + 64;
}

cudaError_t launch_dec_setup(const DecArgs& a, cudaStream_t st) {
  dec_setup_kernel<false><<<1, 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_dec_setup_batch(const DecArgs& a, uint32_t nfields, cudaStream_t st) {
  if (nfields == 0) return cudaSuccess;
  dec_setup_kernel<true><<<nfields, 256, 0, st>>>(a);
  return cudaGetLastError();
}

template <bool FM2, bool BATCH>
static cudaError_t launch_locate_t(const DecArgs& a, cudaStream_t st) {
  const size_t smem = locate_smem_bytes(a.super_chunk, a.overlap, a.maxsz);
  auto k = locate_packs(a.super_chunk, a.maxsz) ? locate_kernel<FM2, BATCH, true> : locate_kernel<FM2, BATCH, false>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<a.nlocate_ctas, kLocThreads, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_locate(const DecArgs& a, cudaStream_t st) {
  if (a.nlocate_ctas == 0) return cudaSuccess;
  return a.fm2 ? launch_locate_t<true, false>(a, st) : launch_locate_t<false, false>(a, st);
}

cudaError_t launch_locate_batch(const DecArgs& a, cudaStream_t st) {
  if (a.nlocate_ctas == 0) return cudaSuccess;
  return launch_locate_t<false, true>(a, st);
}

// Bytes of one decode slot: the block offsets, then the stream span or the
// staged prefix sums that replace it (read 16 bytes past their end).
static uint32_t dec_slot_bytes(uint32_t L, uint32_t tb, uint32_t maxsz) {
  const size_t span = (size_t)tb * maxsz + 32, stage = 4 * (size_t)tb * L + 32;
  return (uint32_t)((dec_pos_bytes(tb) + (span > stage ? span : stage) + 15) & ~(size_t)15);
}

template <int LPB, bool BATCH = false, int ROUNDS = kDecRounds, bool FM2 = false, int OUT = kOutFloat>
static cudaError_t launch_dec_lanes(const DecArgs& a, cudaStream_t st) {
  auto k = decode_pipe<LPB, BATCH, ROUNDS, FM2, OUT>;
  const uint32_t slot = dec_slot_bytes(8 * LPB, a.tb, a.maxsz);
  const size_t smem = (size_t)dec_slots<ROUNDS>() * slot;
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
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kDecPipeThreads, smem);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    c = ((uint64_t)dev + 1) << 32 | (uint32_t)((occ < 1 ? 1 : occ) * sms);
    s_cache.store(c, std::memory_order_relaxed);
  }
  const uint32_t cap = (uint32_t)c;
  const uint32_t grid = a.ntiles < cap ? a.ntiles : cap;
  if (grid == 0) return cudaSuccess;
  if (!BATCH && a.static_tiles) {
    // a single field's tiles are scheduled statically: its CTAs must all be
    // resident, which a cooperative launch guarantees or refuses
    DecArgs args = a;
    uint32_t slot_arg = slot;
    void* params[] = {&args, &slot_arg};
    e = cudaLaunchCooperativeKernel((const void*)k, dim3(grid), dim3(kDecPipeThreads), params, smem, st);
    if (e != cudaErrorCooperativeLaunchTooLarge && e != cudaErrorNotSupported) return e;
    (void)cudaGetLastError();  // refused (a partitioned GPU): draw tickets instead
  }
  DecArgs args = a;
  args.static_tiles = 0;
  k<<<grid, kDecPipeThreads, smem, st>>>(args, slot);
  return cudaGetLastError();
}

uint32_t decode_blocks_per_tile_f64(uint32_t L, uint32_t& bpw) {
  const uint32_t b = 2048u / (L < 32 ? 32u : L);
  bpw = b < 1 ? 1 : (b > 8 ? 8 : b);
  return kDecWarps * bpw;
}

cudaError_t launch_decode_f64(const DecArgs& a, cudaStream_t st) {
  if (a.fm2) {
    decode_generic<kDecWarps, true, double><<<a.ntiles, kDecWarps * 32, 0, st>>>(a);
  } else {
    decode_generic<kDecWarps, false, double><<<a.ntiles, kDecWarps * 32, 0, st>>>(a);
  }
  return cudaGetLastError();
}

// The fastmode pipelines for float64 streams (blockSize 8..256): a.f.y is the
// output array of doubles.
cudaError_t launch_decode_q(const DecArgs& a, cudaStream_t st) {
  if (a.fm2) {
    switch (dec_lanes_per_block(a.f.seg.L)) {
      case 1: return launch_dec_lanes<1, false, kDecRounds, true, kOutDouble>(a, st);
      case 2: return launch_dec_lanes<2, false, kDecRounds, true, kOutDouble>(a, st);
      case 4: return launch_dec_lanes<4, false, kDecRounds, true, kOutDouble>(a, st);
      case 8: return launch_dec_lanes<8, false, kDecRounds, true, kOutDouble>(a, st);
      case 16: return launch_dec_lanes<16, false, kDecRounds, true, kOutDouble>(a, st);
      case 32: return launch_dec_lanes<32, false, kDecRounds, true, kOutDouble>(a, st);
      default: return cudaErrorInvalidValue;
    }
  }
  switch (dec_lanes_per_block(a.f.seg.L)) {
    case 1: return launch_dec_lanes<1, false, kDecRounds, false, kOutDouble>(a, st);
    case 2: return launch_dec_lanes<2, false, kDecRounds, false, kOutDouble>(a, st);
    case 4: return launch_dec_lanes<4, false, kDecRounds, false, kOutDouble>(a, st);
    case 8: return launch_dec_lanes<8, false, kDecRounds, false, kOutDouble>(a, st);
    case 16: return launch_dec_lanes<16, false, kDecRounds, false, kOutDouble>(a, st);
    case 32: return launch_dec_lanes<32, false, kDecRounds, false, kOutDouble>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

// The fastmode pipelines writing the int32 codes to a.f.y, or adding them to
// the codes there (accumulate); blockSize 8..256.
template <int OUT>
static cudaError_t launch_decode_codes_t(const DecArgs& a, cudaStream_t st) {
  if (a.fm2) {
    switch (dec_lanes_per_block(a.f.seg.L)) {
      case 1: return launch_dec_lanes<1, false, kDecRounds, true, OUT>(a, st);
      case 2: return launch_dec_lanes<2, false, kDecRounds, true, OUT>(a, st);
      case 4: return launch_dec_lanes<4, false, kDecRounds, true, OUT>(a, st);
      case 8: return launch_dec_lanes<8, false, kDecRounds, true, OUT>(a, st);
      case 16: return launch_dec_lanes<16, false, kDecRounds, true, OUT>(a, st);
      case 32: return launch_dec_lanes<32, false, kDecRounds, true, OUT>(a, st);
      default: return cudaErrorInvalidValue;
    }
  }
  switch (dec_lanes_per_block(a.f.seg.L)) {
    case 1: return launch_dec_lanes<1, false, kDecRounds, false, OUT>(a, st);
    case 2: return launch_dec_lanes<2, false, kDecRounds, false, OUT>(a, st);
    case 4: return launch_dec_lanes<4, false, kDecRounds, false, OUT>(a, st);
    case 8: return launch_dec_lanes<8, false, kDecRounds, false, OUT>(a, st);
    case 16: return launch_dec_lanes<16, false, kDecRounds, false, OUT>(a, st);
    case 32: return launch_dec_lanes<32, false, kDecRounds, false, OUT>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_decode_codes(const DecArgs& a, bool accumulate, cudaStream_t st) {
  return accumulate ? launch_decode_codes_t<kOutCodesAdd>(a, st) : launch_decode_codes_t<kOutCodes>(a, st);
}

cudaError_t launch_decode(const DecArgs& a, cudaStream_t st) {
  if (a.fm2) {
    switch (dec_lanes_per_block(a.f.seg.L)) {
      case 1: return launch_dec_lanes<1, false, kDecRounds, true>(a, st);
      case 2: return launch_dec_lanes<2, false, kDecRounds, true>(a, st);
      case 4: return launch_dec_lanes<4, false, kDecRounds, true>(a, st);
      case 8: return launch_dec_lanes<8, false, kDecRounds, true>(a, st);
      case 16: return launch_dec_lanes<16, false, kDecRounds, true>(a, st);
      case 32: return launch_dec_lanes<32, false, kDecRounds, true>(a, st);
      default: break;
    }
    decode_generic<kDecWarps, true><<<a.ntiles, kDecWarps * 32, 0, st>>>(a);
    return cudaGetLastError();
  }
  switch (dec_lanes_per_block(a.f.seg.L)) {
    case 1: return launch_dec_lanes<1>(a, st);
    case 2: return launch_dec_lanes<2>(a, st);
    case 4: return launch_dec_lanes<4>(a, st);
    case 8: return launch_dec_lanes<8>(a, st);
    case 16: return launch_dec_lanes<16>(a, st);
    case 32: return launch_dec_lanes<32>(a, st);
    default: break;
  }
  decode_generic<kDecWarps, false><<<a.ntiles, kDecWarps * 32, 0, st>>>(a);
  return cudaGetLastError();
}

// Sets the batched decompression kernels' shared-memory limits and caches
// their grids without launching anything.
cudaError_t prepare_decompress_batch() {
  DecArgs a;
  memset(&a, 0, sizeof a);
  a.maxsz = max_block_bytes(32);
  a.super_chunk = locate_super_bytes(a.maxsz);
  a.overlap = locate_overlap_bytes(a.maxsz);
  const size_t smem = locate_smem_bytes(a.super_chunk, a.overlap, a.maxsz);
  cudaError_t e = cudaFuncSetAttribute(locate_kernel<false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(locate_kernel<false, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  for (int r : {1, 2, 4}) {
    if (e != cudaSuccess) return e;
    a.tb = 8u * (uint32_t)r * 8u;
    e = r == 1 ? launch_dec_lanes<4, true, 1>(a, 0) : r == 2 ? launch_dec_lanes<4, true, 2>(a, 0) : launch_dec_lanes<4, true, 4>(a, 0);
  }
  return e;
}

// Batched fastmode1 decode, blockSize 32, tiles of 8*rounds*8 blocks.
cudaError_t launch_decode_batch(const DecArgs& a, uint32_t L, int rounds, cudaStream_t st) {
  if (L != 32) return cudaErrorInvalidValue;
  switch (rounds) {
    case 1: return launch_dec_lanes<4, true, 1>(a, st);
    case 2: return launch_dec_lanes<4, true, 2>(a, st);
    case 4: return launch_dec_lanes<4, true, 4>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace szp
