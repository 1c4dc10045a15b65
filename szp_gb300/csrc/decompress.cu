// decompress.cu -- SZp fastmode1 / fastmode2 float32 decompressors for sm_103a.
//
// The stream keeps no block index: a block's position depends on the bit
// counts of all blocks before it in its segment (szpd_float.cc:76-118).  Three
// launches recover it in parallel:
//
//  1. dec_setup   one CTA reads eb and the T segment offsets, validates them
//                 and cuts every segment's block region into fixed chunks.
//  2. locate      one warp per chunk.  It walks the chunk from every entry
//                 offset a block could start at (0 .. largest block - 1),
//                 merging walks that meet (claims in shared memory) so the
//                 work is roughly one walk.  The result is the chunk's exit
//                 function entry -> first position past the chunk.  When all
//                 live entries agree (the usual case, walks re-synchronise),
//                 the chunk's exit is known at once; otherwise successors
//                 compose functions in a look-back.  With its entry known the
//                 chunk counts its blocks, a second look-back turns counts
//                 into block indices, and every block's header offset is
//                 written to blkpos.
//  3. decode      one CTA per run of blocks: unpack sign bits and fixed-length
//                 fields, prefix-add deltas (fastmode1: decoupled look-back
//                 over the tiles of a segment), dequantize (float)q*eb.
#include "szp_device.cuh"
#include "szp_kernels.h"

namespace szp {

constexpr uint16_t kExEnd = 0xFFFE;    // walk left the segment
constexpr uint16_t kExDead = 0xFFFF;   // walk met an invalid header
constexpr uint16_t kExMerged = 0xFFFD;
constexpr uint16_t kExLive = 0xFFFC;
constexpr uint16_t kFree = 0xFFFF;
constexpr int kLocWarps = 4;
constexpr uint32_t kPreMax = 64;

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

uint32_t locate_chunk_bytes(uint32_t maxsz) {
  uint32_t c = 2048;
  while (c < 2 * maxsz) c *= 2;
  return c;
}

// per-warp shared memory layout of the locate kernel
struct LocLayout {
  uint32_t bytes_off, claim_off, pos_off, res_off, tgt_off, l0_off, l1_off, lead_off, pre_off, per_warp;
  __host__ __device__ LocLayout(uint32_t C, uint32_t maxsz) {
    uint32_t o = 0;
    bytes_off = o;
    o += (C + maxsz + 32 + 15) & ~15u;
    claim_off = o;
    o += 2 * C;
    pos_off = o;
    o += 2 * maxsz;
    res_off = o;
    o += 2 * maxsz;
    tgt_off = o;
    o += 2 * maxsz;
    l0_off = o;
    o += 2 * maxsz;
    l1_off = o;
    o += 2 * maxsz;
    lead_off = o;
    o += 2 * C;
    pre_off = o;
    o += 2 * kPreMax;
    per_warp = (o + 15) & ~15u;
  }
};

size_t locate_smem_bytes(uint32_t chunk, uint32_t maxsz) {
  return (size_t)LocLayout(chunk, maxsz).per_warp * kLocWarps;
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
__global__ void dec_setup_kernel(DecArgs a) {
  const Segments sg = a.seg;
  const uint32_t T = sg.T;
  const uint64_t head = 4 + 8ull * T;
  __shared__ uint32_t s_bad;
  uint64_t len = a.len;
  if (a.len_dev) {
    uint64_t l2 = *a.len_dev;
    len = l2 < len ? l2 : len;
  }
  if (threadIdx.x == 0) {
    s_bad = len < head ? 1u : 0u;
    if (!s_bad) {
      uint32_t b = ((uint32_t)a.in[0] << 24) | ((uint32_t)a.in[1] << 16) | ((uint32_t)a.in[2] << 8) | a.in[3];
      a.plan->eb = __uint_as_float(b);
    } else {
      a.plan->eb = 0.0f;
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
      uint64_t off = load_u64le(a.in + 4 + 8ull * t);
      uint64_t body = len - head;
      uint64_t end;
      if (off > body) {
        bad = true;
      } else {
        uint64_t start = head + off;
        if (t + 1 < T) {
          uint64_t off2 = load_u64le(a.in + 4 + 8ull * (t + 1));
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
            nch = (uint32_t)((r1 - r0 + a.chunk - 1) / a.chunk);
          }
        }
      }
    }
    if (bad) {
      atomicOr(&s_bad, 1u);
      nch = 0;
    }
    a.reg0[t] = r0;
    a.reg1[t] = r1;
    a.chunk_base[t + 1] = nch;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    a.chunk_base[0] = 0;
    if (s_bad) {
      for (uint32_t t = 0; t < T; t++) a.chunk_base[t + 1] = 0;
      atomicOr(a.err, kErrCorrupt);
    } else {
      for (uint32_t t = 0; t < T; t++) {
        acc += a.chunk_base[t + 1];
        a.chunk_base[t + 1] = acc;
      }
    }
    a.plan->nchunks = s_bad ? 0 : acc;
    a.plan->bad = s_bad;
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
template <bool FM2>
__global__ void __launch_bounds__(kLocWarps * 32) locate_kernel(DecArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ uint32_t s_tk[2];
  uint32_t tk, epoch;
  draw_ticket(a.ls, a.nlocate_ctas, tk, epoch, s_tk);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Segments sg = a.seg;
  const uint32_t T = sg.T, L = sg.L, C = a.chunk, maxsz = a.maxsz;
  const uint32_t c = tk * kLocWarps + warp;
  const uint32_t nch = a.chunk_base[T];
  if (c >= nch) return;  // no CTA-wide barrier below this point

  // segment of chunk c: largest t with chunk_base[t] <= c
  uint32_t lo_t = 0, hi_t = T - 1;
  while (lo_t < hi_t) {
    uint32_t mid = (lo_t + hi_t + 1) >> 1;
    if (a.chunk_base[mid] <= c) lo_t = mid; else hi_t = mid - 1;
  }
  const uint32_t t = lo_t;
  const uint32_t first = a.chunk_base[t];
  const uint32_t ci = c - first;
  const uint64_t R0 = a.reg0[t], R1 = a.reg1[t];
  const uint64_t c0 = R0 + (uint64_t)ci * C;
  const uint64_t rest = R1 - c0;
  const uint32_t clen = (uint32_t)(rest < C ? rest : C);
  const uint32_t end_rel = (uint32_t)(rest < (uint64_t)clen + maxsz + 8 ? rest : (uint64_t)clen + maxsz + 8);
  const uint32_t nload = end_rel;  // never read past the segment region

  const LocLayout lay(C, maxsz);
  uint8_t* base = smem + warp * lay.per_warp;
  uint8_t* sb = base + lay.bytes_off;
  uint16_t* claim = reinterpret_cast<uint16_t*>(base + lay.claim_off);
  uint16_t* pos_s = reinterpret_cast<uint16_t*>(base + lay.pos_off);
  uint16_t* res_s = reinterpret_cast<uint16_t*>(base + lay.res_off);
  uint16_t* tgt_s = reinterpret_cast<uint16_t*>(base + lay.tgt_off);
  uint16_t* list0 = reinterpret_cast<uint16_t*>(base + lay.l0_off);
  uint16_t* list1 = reinterpret_cast<uint16_t*>(base + lay.l1_off);
  uint16_t* lead = reinterpret_cast<uint16_t*>(base + lay.lead_off);
  uint16_t* pre = reinterpret_cast<uint16_t*>(base + lay.pre_off);

  // stage the chunk (and the longest block that may start in it)
  {
    const uint8_t* src = a.in + c0;
    uint32_t mis = (uint32_t)((uintptr_t)src & 15);
    uint32_t headb = mis ? 16 - mis : 0;
    if (headb > nload) headb = nload;
    for (uint32_t i = lane; i < headb; i += 32) sb[i] = src[i];
    uint32_t nvec = (nload - headb) >> 4;
    const uint4* s4 = reinterpret_cast<const uint4*>(src + headb);
    for (uint32_t i = lane; i < nvec; i += 32) {
      uint4 v = __ldg(s4 + i);
      uint8_t* d = sb + headb + 16 * i;
      const uint8_t* vb = reinterpret_cast<const uint8_t*>(&v);
#pragma unroll
      for (int k = 0; k < 16; k++) d[k] = vb[k];
    }
    for (uint32_t i = headb + 16 * nvec + lane; i < nload; i += 32) sb[i] = src[i];
    for (uint32_t i = lane; i < clen; i += 32) claim[i] = kFree;
  }
  __syncwarp();

  // header byte of a block at p (p < clen); 0 size means invalid
  auto step = [&](uint32_t p) -> uint32_t {
    uint32_t hp = FM2 ? p + 4 : p;
    if (hp >= nload) return 0;
    return full_block_size(sb[hp], L, FM2);
  };

  // ---- walks from every entry, merged through claims ----
  const uint32_t E = maxsz;
  uint32_t cnt = 0;
  for (uint32_t e = lane; e < E; e += 32) {
    if (e >= clen) {
      res_s[e] = kExEnd;  // only the short last chunk: past its end is past the segment
    } else {
      res_s[e] = kExLive;
      pos_s[e] = (uint16_t)e;
    }
  }
  {
    uint32_t live = E < clen ? E : clen;
    for (uint32_t e = lane; e < live; e += 32) list0[e] = (uint16_t)e;
    cnt = live;
  }
  __syncwarp();
  uint16_t* cur = list0;
  uint16_t* nxt = list1;
  int leader = -1;
  while (cnt > 0) {
    if (cnt == 1) {
      leader = cur[0];
      break;
    }
    uint32_t newcnt = 0;
    for (uint32_t b0 = 0; b0 < cnt; b0 += 32) {
      uint32_t i = b0 + lane;
      bool live = false;
      uint16_t id = 0;
      if (i < cnt) {
        id = cur[i];
        uint32_t p = pos_s[id];
        uint16_t old = atomicCAS(claim + p, kFree, id);
        if (old != kFree) {
          res_s[id] = kExMerged;
          tgt_s[id] = old;
        } else {
          uint32_t sz = step(p);
          if (!sz) {
            res_s[id] = kExDead;
          } else {
            uint32_t np = p + sz;
            if (np >= end_rel) res_s[id] = kExEnd;
            else if (np >= clen) res_s[id] = (uint16_t)(np - clen);
            else {
              pos_s[id] = (uint16_t)np;
              live = true;
            }
          }
        }
      }
      uint32_t bal = __ballot_sync(0xffffffffu, live);
      if (live) nxt[newcnt + __popc(bal & ((1u << lane) - 1u))] = id;
      newcnt += __popc(bal);
    }
    __syncwarp();
    uint16_t* tmp = cur;
    cur = nxt;
    nxt = tmp;
    cnt = newcnt;
  }
  // one walk left: follow it without atomics, recording its headers.  Its
  // recorded headers can be spliced onto the true path unless it ended by
  // merging into an earlier walk (whose later headers are not recorded).
  uint32_t nlead = 0;
  bool can_splice = false;
  if (leader >= 0) {
    uint32_t ok = 0;
    if (lane == 0) {
      uint32_t p = pos_s[leader];
      uint32_t k = 0;
      uint16_t r = kExDead;
      while (true) {
        uint16_t cl = claim[p];
        if (cl != kFree) {
          r = kExMerged;
          tgt_s[leader] = cl;
          break;
        }
        uint32_t sz = step(p);
        if (!sz) {
          r = kExDead;
          break;
        }
        claim[p] = (uint16_t)(0x8000u | k);
        lead[k++] = (uint16_t)p;
        uint32_t np = p + sz;
        if (np >= end_rel) {
          r = kExEnd;
          break;
        }
        if (np >= clen) {
          r = (uint16_t)(np - clen);
          break;
        }
        p = np;
      }
      res_s[leader] = r;
      nlead = k;
      ok = r != kExMerged;
    }
    nlead = __shfl_sync(0xffffffffu, nlead, 0);
    can_splice = __shfl_sync(0xffffffffu, ok, 0) != 0;
  }
  __syncwarp();
  // resolve merged walks to their final exits (claims only point backwards)
  uint32_t fmin = 0xFFFFu, fmax = 0;
  for (uint32_t e = lane; e < E; e += 32) {
    uint32_t j = e;
    uint16_t r = res_s[j];
    for (uint32_t guard = 0; r == kExMerged && guard < E + 1; guard++) {
      uint16_t tg = tgt_s[j];
      j = tg & 0x7FFFu;  // list-phase claims hold walk ids
      if (j >= E) {
        r = kExDead;
        break;
      }
      r = res_s[j];
    }
    if (r == kExMerged || r == kExLive) r = kExDead;
    // other lanes following a chain through e read either the merged marker
    // (and then the unchanged target) or this final value: both agree
    res_s[e] = r;
    if (r != kExDead) {
      fmin = min(fmin, (uint32_t)r);
      fmax = max(fmax, (uint32_t)r);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    fmin = min(fmin, __shfl_xor_sync(0xffffffffu, fmin, o));
    fmax = max(fmax, __shfl_xor_sync(0xffffffffu, fmax, o));
  }
  __syncwarp();
  const bool constant = fmin == fmax;  // all live entries leave at one place
  const uint16_t cexit = constant ? (uint16_t)fmin : kExDead;

  uint64_t* st_entry = a.status;
  uint64_t* st_count = a.status + a.status_stride;

  // ---- publish exit function, find own entry ----
  if (!constant) {
    for (uint32_t e = lane; e < E; e += 32) a.fn[(uint64_t)c * maxsz + e] = res_s[e];
    __threadfence();
    __syncwarp();
  }
  uint32_t entry;
  if (ci == 0) {
    entry = 0;
    if (lane == 0) st_release_u64(st_entry + c, make_status(epoch, kFlagInclusive, res_s[0]));
  } else {
    if (lane == 0) {
      if (constant) st_release_u64(st_entry + c, make_status(epoch, kFlagInclusive, cexit));
      else st_release_u64(st_entry + c, make_status(epoch, kFlagAggregate, 0));
    }
    // nearest predecessor whose exit is known
    int64_t k = (int64_t)c - 1;
    int64_t found = -1;
    uint32_t fval = 0, spins = 0;
    bool timeout = false;
    while (found < 0) {
      int64_t idx = k - lane;
      bool inrange = idx >= (int64_t)first;
      uint64_t s = inrange ? ld_volatile_u64(st_entry + idx) : 0;
      bool ready = !inrange || (status_epoch(s) == (epoch & 0xFFFFF) && status_flag(s) != 0);
      uint32_t incl = __ballot_sync(0xffffffffu, inrange && ready && status_flag(s) == kFlagInclusive);
      uint32_t notready = __ballot_sync(0xffffffffu, !ready);
      uint32_t upto = incl & (0u - incl);
      uint32_t relevant = upto ? (upto | (upto - 1)) : 0xffffffffu;
      if (notready & relevant) {
        if (++spins > kSpinLimit) {
          timeout = true;
          break;
        }
        continue;
      }
      if (upto) {
        int fl = __ffs(upto) - 1;
        found = k - fl;
        fval = (uint32_t)__shfl_sync(0xffffffffu, (uint32_t)status_value(s), fl);
      } else {
        k -= 32;  // the segment's first chunk is always inclusive, so this ends
        if (k < (int64_t)first) {
          timeout = true;  // unreachable unless the status words are corrupt
          break;
        }
      }
    }
    if (timeout) {
      if (lane == 0) atomicOr(a.err, kErrLookbackTimeout);
      entry = kExDead;
    } else {
      if (found + 1 < (int64_t)c) __threadfence();  // order the fn-row reads after the status reads
      uint32_t e = fval;
      for (int64_t m = found + 1; m < (int64_t)c; m++) {
        if (e >= maxsz) break;  // END / DEAD propagate
        e = a.fn[(uint64_t)m * maxsz + e];
      }
      entry = e;
    }
    if (!constant && lane == 0) {
      uint16_t ex = entry < maxsz ? res_s[entry] : (uint16_t)entry;
      st_release_u64(st_entry + c, make_status(epoch, kFlagInclusive, ex));
    }
  }

  // ---- headers on the true path through this chunk ----
  uint32_t npre = 0, splice = 0xFFFFFFFFu, count = 0;
  bool overflow = false;
  if (lane == 0 && entry < clen) {
    uint32_t p = entry;
    while (p < clen) {
      uint16_t cl = claim[p];
      if (can_splice && (cl & 0x8000u) && cl != kFree) {
        splice = cl & 0x7FFFu;
        break;
      }
      uint32_t sz = step(p);
      if (!sz) break;
      if (npre < kPreMax) pre[npre] = (uint16_t)p;
      else overflow = true;
      npre++;
      p += sz;
    }
    count = npre + (splice != 0xFFFFFFFFu ? nlead - splice : 0);
  }
  count = __shfl_sync(0xffffffffu, count, 0);
  npre = __shfl_sync(0xffffffffu, npre, 0);
  splice = __shfl_sync(0xffffffffu, splice, 0);
  overflow = __shfl_sync(0xffffffffu, overflow ? 1 : 0, 0) != 0;

  // ---- block index of the first header: look-back over counts ----
  uint64_t g0 = 0;
  if (ci == 0) {
    if (lane == 0) st_release_u64(st_count + c, make_status(epoch, kFlagInclusive, count));
  } else {
    if (lane == 0) st_release_u64(st_count + c, make_status(epoch, kFlagAggregate, count));
    g0 = lookback_sum(st_count, c, first, epoch, a.err);
    if (lane == 0) st_release_u64(st_count + c, make_status(epoch, kFlagInclusive, g0 + count));
  }
  const uint64_t nb = seg_blocks(sg, t, FM2);
  const uint64_t gb = seg_block_base(sg, t, FM2);
  const uint32_t rel0 = (uint32_t)(c0 - R0);
  if (!overflow) {
    for (uint32_t i = lane; i < count; i += 32) {
      uint64_t g = g0 + i;
      if (g >= nb) break;
      uint32_t p = i < npre ? pre[i] : lead[splice + (i - npre)];
      a.blkpos[gb + g] = rel0 + p;
    }
  } else if (lane == 0) {
    // long unmerged prefix (rare): walk again, writing as we go
    uint32_t p = entry;
    uint64_t g = g0;
    while (p < clen && g < g0 + npre) {
      uint16_t cl = claim[p];
      if (can_splice && (cl & 0x8000u) && cl != kFree) break;
      uint32_t sz = step(p);
      if (!sz) break;
      if (g < nb) a.blkpos[gb + g] = rel0 + p;
      g++;
      p += sz;
    }
    for (uint32_t i = npre; i < count; i++) {
      uint64_t gg = g0 + i;
      if (gg < nb) a.blkpos[gb + gg] = rel0 + lead[splice + (i - npre)];
    }
  }
  // the last chunk of a segment checks the block total
  if (lane == 0 && c + 1 == a.chunk_base[t + 1]) {
    uint64_t total = g0 + count;
    bool last_seg = t + 1 == T;
    if (total < nb || (!last_seg && total != nb)) atomicOr(a.err, kErrBlockCount);
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

// fastmode1, blockSize 32: one warp per block, one element per lane.
template <int WARPS, int BPW>
__global__ void __launch_bounds__(WARPS * 32) decode_fm1_l32(DecArgs a) {
  __shared__ uint32_t s_tk[2];
  __shared__ uint32_t s_w[WARPS + 1];
  __shared__ uint32_t s_base;
  constexpr uint32_t TB = WARPS * BPW;
  uint32_t tile, epoch;
  draw_ticket(a.ls, a.ntiles, tile, epoch, s_tk);
  if (a.plan->bad) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Segments sg = a.seg;
  const DecTile dt = dec_tile(sg, tile, a.tiles_per_seg, TB, false);
  if (!dt.any) return;
  const float eb = a.plan->eb;
  const bool ebsp = !isfinite(eb);
  const uint64_t lo = sg.lo(dt.seg), hi = sg.hi(dt.seg);
  const uint64_t R0 = a.reg0[dt.seg], R1 = a.reg1[dt.seg];
  const uint8_t* __restrict__ in = a.in;
  const uint64_t gb = seg_block_base(sg, dt.seg, false);

  const uint32_t wfirst = warp * BPW;
  const uint32_t wn = dt.nblk > wfirst ? min((uint32_t)BPW, dt.nblk - wfirst) : 0;
  uint32_t mypos = 0;
  if ((uint32_t)lane < wn) mypos = __ldg(a.blkpos + gb + dt.blk0 + wfirst + lane);
  uint32_t sc[BPW], tot = 0, wtot = 0;
  bool corrupt = false;
#pragma unroll
  for (int k = 0; k < BPW; k++) {
    sc[k] = 0;
    if ((uint32_t)k < wn) {
      uint64_t b = dt.blk0 + wfirst + k;
      uint64_t s = lo + 1 + b * 32;
      uint32_t m = hi - s < 32 ? (uint32_t)(hi - s) : 32u;
      uint64_t hp = R0 + __shfl_sync(0xffffffffu, mypos, k);
      uint32_t bc = hp < R1 ? __ldg(in + hp) : 255u;
      uint32_t d = 0;
      if (bc > 33 || hp + block_bytes(m, bc) > R1) {
        corrupt = true;
      } else if (bc) {
        if ((uint32_t)lane < m) d = decode_delta(in + hp, m, bc, lane);
      }
      sc[k] = warp_incl_scan(d, lane);
      wtot += __shfl_sync(0xffffffffu, sc[k], 31);
    }
  }
  if (corrupt && lane == 0) atomicOr(a.err, kErrCorrupt);
  (void)tot;

  uint32_t wexcl;
  const uint32_t agg = scan_warps_u32<WARPS>(s_w, wtot, warp, lane, wexcl);
  // q chain of the segment: first tile starts from the seed
  const uint32_t first_tile = a.tiles_per_seg ? dt.seg * a.tiles_per_seg : 0;
  if (warp == 0) {
    uint32_t excl;
    if (dt.first) {
      const uint8_t* sp = in + R0 - 4;
      excl = (uint32_t)sp[0] | ((uint32_t)sp[1] << 8) | ((uint32_t)sp[2] << 16) | ((uint32_t)sp[3] << 24);
      if (lane == 0) {
        st_release_u64(a.status + tile, make_status(epoch, kFlagInclusive, (uint32_t)(excl + agg)));
        a.y[lo] = dequant(excl, eb, ebsp);
      }
    } else {
      if (lane == 0) st_release_u64(a.status + tile, make_status(epoch, kFlagAggregate, agg));
      excl = (uint32_t)lookback_sum(a.status, tile, first_tile, epoch, a.err);
      if (lane == 0) st_release_u64(a.status + tile, make_status(epoch, kFlagInclusive, (uint32_t)(excl + agg)));
    }
    if (lane == 0) s_base = excl;
  }
  __syncthreads();
  uint32_t q0 = s_base + wexcl;
#pragma unroll
  for (int k = 0; k < BPW; k++) {
    if ((uint32_t)k < wn) {
      uint64_t b = dt.blk0 + wfirst + k;
      uint64_t s = lo + 1 + b * 32;
      uint32_t m = hi - s < 32 ? (uint32_t)(hi - s) : 32u;
      if ((uint32_t)lane < m) a.y[s + lane] = dequant(q0 + sc[k], eb, ebsp);
      q0 += __shfl_sync(0xffffffffu, sc[k], 31);
    }
  }
}

// Any blockSize, fastmode1 or fastmode2: one warp per block in 32-element
// pieces.  fastmode1 decodes twice (totals, then values after the look-back).
template <int WARPS, bool FM2>
__global__ void __launch_bounds__(WARPS * 32) decode_generic(DecArgs a) {
  __shared__ uint32_t s_tk[2];
  __shared__ uint32_t s_w[WARPS + 1];
  __shared__ uint32_t s_base;
  uint32_t tile, epoch;
  draw_ticket(a.ls, a.ntiles, tile, epoch, s_tk);
  if (a.plan->bad) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Segments sg = a.seg;
  const uint32_t L = sg.L;
  const uint32_t TB = WARPS * a.bpw;
  const DecTile dt = dec_tile(sg, tile, a.tiles_per_seg, TB, FM2);
  if (!dt.any) return;
  const float eb = a.plan->eb;
  const bool ebsp = !isfinite(eb);
  const uint64_t lo = sg.lo(dt.seg), hi = sg.hi(dt.seg);
  const uint64_t R0 = a.reg0[dt.seg], R1 = a.reg1[dt.seg];
  const uint8_t* __restrict__ in = a.in;
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
    hp = R0 + __ldg(a.blkpos + gb + b) + (FM2 ? 4 : 0);
    if (FM2 && m == 0) return 0;  // one-element block: no header is read (szpd_float.cc:481)
    if (hp >= R1) return 255u;
    uint32_t bc = __ldg(in + hp);
    if (bc > 33 || hp + block_bytes(m, bc) > R1) return 255u;
    return bc;
  };

  uint32_t q0 = 0;
  if (!FM2) {
    uint32_t wtot = 0;
    for (uint32_t k = 0; k < a.bpw; k++) {
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
    const uint32_t first_tile = a.tiles_per_seg ? dt.seg * a.tiles_per_seg : 0;
    if (warp == 0) {
      uint32_t excl;
      if (dt.first) {
        const uint8_t* sp = in + R0 - 4;
        excl = (uint32_t)sp[0] | ((uint32_t)sp[1] << 8) | ((uint32_t)sp[2] << 16) | ((uint32_t)sp[3] << 24);
        if (lane == 0) {
          st_release_u64(a.status + tile, make_status(epoch, kFlagInclusive, (uint32_t)(excl + agg)));
          a.y[lo] = dequant(excl, eb, ebsp);
        }
      } else {
        if (lane == 0) st_release_u64(a.status + tile, make_status(epoch, kFlagAggregate, agg));
        excl = (uint32_t)lookback_sum(a.status, tile, first_tile, epoch, a.err);
        if (lane == 0) st_release_u64(a.status + tile, make_status(epoch, kFlagInclusive, (uint32_t)(excl + agg)));
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
    uint32_t bc = blk_hdr(b, m, hp);
    if (bc == 255u) {
      corrupt = true;
      bc = 0;
    }
    if (FM2) {
      const uint8_t* sp = in + hp - 4;
      q0 = (uint32_t)__ldg(sp) | ((uint32_t)__ldg(sp + 1) << 8) | ((uint32_t)__ldg(sp + 2) << 16) |
           ((uint32_t)__ldg(sp + 3) << 24);
      if (lane == 0) a.y[s - 1] = dequant(q0, eb, ebsp);
    }
    for (uint32_t p0 = 0; p0 < m; p0 += 32) {
      uint32_t j = p0 + lane;
      uint32_t d = (bc && j < m) ? decode_delta(in + hp, m, bc, j) : 0u;
      uint32_t sc = warp_incl_scan(d, lane);
      if (j < m) a.y[s + j] = dequant(q0 + sc, eb, ebsp);
      q0 += __shfl_sync(0xffffffffu, sc, 31);
    }
  }
  if (__any_sync(0xffffffffu, corrupt) && lane == 0) atomicOr(a.err, kErrCorrupt);
}

constexpr int kDecWarps = 8, kDecBpw = 8;

uint32_t decode_blocks_per_tile(uint32_t L, uint32_t& bpw) {
  if (L == 32) {
    bpw = kDecBpw;
    return kDecWarps * kDecBpw;
  }
  uint32_t b = 2048u / (L < 32 ? 32u : L);
  bpw = b < 1 ? 1 : (b > 8 ? 8 : b);
  return kDecWarps * bpw;
}

cudaError_t launch_dec_setup(const DecArgs& a, cudaStream_t st) {
  dec_setup_kernel<<<1, 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_locate(const DecArgs& a, cudaStream_t st) {
  size_t smem = locate_smem_bytes(a.chunk, a.maxsz);
  if (a.fm2) {
    auto k = locate_kernel<true>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<a.nlocate_ctas, kLocWarps * 32, smem, st>>>(a);
  } else {
    auto k = locate_kernel<false>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<a.nlocate_ctas, kLocWarps * 32, smem, st>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_decode(const DecArgs& a, cudaStream_t st) {
  if (a.fm2) {
    decode_generic<kDecWarps, true><<<a.ntiles, kDecWarps * 32, 0, st>>>(a);
  } else if (a.seg.L == 32) {
    decode_fm1_l32<kDecWarps, kDecBpw><<<a.ntiles, kDecWarps * 32, 0, st>>>(a);
  } else {
    decode_generic<kDecWarps, false><<<a.ntiles, kDecWarps * 32, 0, st>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace szp
