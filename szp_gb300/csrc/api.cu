// api.cu -- host runtime and C ABI of libszp_gb300.so.
//
// Every calling host thread gets a Workspace per device: a CUDA stream, device
// buffers that grow on demand and stay resident (input staging, stream
// staging, look-back words, block index), and small pinned host scalars.
// The reference entry points stage host buffers through it; the *_dev
// extensions work on caller device memory.  No entry point falls back to the
// CPU: without a usable GPU they fail with an error.
#include <omp.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <memory>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "szp_gb300.h"
#include "szp_kernels.h"

using namespace szp;

namespace {

// ---------------------------------------------------------------- errors --
thread_local std::string t_err;
thread_local int t_status = SZP_GB300_OK;
thread_local int t_notices = 0;

int fail(int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_err = buf;
  t_status = status;
  return status;
}
void clear_error() {
  t_err.clear();
  t_status = SZP_GB300_OK;
}

#define CU(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return fail(SZP_GB300_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// ------------------------------------------------------- bit-count table --
// thr[k] = smallest m >= 1 with (int)log2f((float)m)+1 >= k (k = 1..33), from
// this host's libm, the same function the reference calls
// (SZp/src/szp_float.cc:261).  Bisection is valid because the rule is
// non-decreasing in m (the test suite checks all 2^32 values).
int host_bitcount(uint32_t m) { return m ? (int)log2f((float)m) + 1 : 0; }

BitcountTable make_table() {
  BitcountTable t;
  memset(&t, 0, sizeof t);
  for (int k = 1; k <= kMaxBitCount; k++) {
    uint64_t a = 1, b = 0xFFFFFFFFull;
    if (host_bitcount((uint32_t)b) < k) {
      t.thr[k] = 0xFFFFFFFFu;
      continue;
    }
    while (a < b) {
      uint64_t mid = (a + b) / 2;
      if (host_bitcount((uint32_t)mid) >= k) b = mid; else a = mid + 1;
    }
    t.thr[k] = (uint32_t)a;
  }
  for (int k = kMaxBitCount + 1; k < 36; k++) t.thr[k] = 0xFFFFFFFFu;
  return t;
}

const BitcountTable& table() {
  static BitcountTable t = make_table();
  return t;
}

// ------------------------------------------------------------- settings --
std::mutex g_mu;
int g_segments = 0;
int g_timing = 0;
int g_overlap = -1;  // locate overlap override (tests of the repair paths)
int g_decode_tickets = 0;  // single-field decode draws tickets (tests of that path)
unsigned long long g_launches = 0;

int resolve_segments(int requested) {
  if (requested > 0) return requested;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_segments > 0) return g_segments;
  }
  int t = omp_get_max_threads();
  return t > 0 ? t : 1;
}

void count_launches(int k) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_launches += (unsigned long long)k;
}

// ------------------------------------------------------------ workspace --
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t n) {
    if (n <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = n < 256 ? 256 : n;
    want += want / 8;  // grow with headroom
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  template <class T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

// Device scalars of one workspace.
struct DevMisc {
  LaunchState ls;
  uint32_t err;
  uint32_t rel_counter;
  uint64_t out_size;
  float eb;
  float pad;
  uint32_t verify[4];  // [0] locate repairs of the last launch
  double ebd;          // REL bound of float64 data
  double invd;         // and its inverse
};
constexpr int kRelMaxGrid = 1024;

enum { kSlotRel = 0, kSlotCompress, kSlotSetup, kSlotLocate, kSlotDecode, kSlotLorenzo, kSlotLorenzoInv, kNumSlots };

struct Workspace {
  int device = -1;
  cudaStream_t own = nullptr;
  cudaStream_t last = nullptr;
  cudaEvent_t done = nullptr;
  DevBuf misc, rel_partial, status, in, stream, out, plan, walks, blkpos;
  DevBuf qbuf;  // int32 q of float64 data between a pipeline and its pass
  uint8_t* h_small = nullptr;  // pinned: out_size (8) + err (4)
  size_t last_stream = 0;      // size of this thread's last host-API stream
  // ring of event pairs per kernel slot: every launch is timed when timing
  // is on, and szp_gb300_kernel_time() sums the launches not yet read
  static constexpr int kRing = 1024;
  cudaEvent_t ev[kNumSlots][kRing][2];
  int ev_head[kNumSlots];     // next pair to record
  int ev_pending[kNumSlots];  // recorded and not yet read
  int ev_last[kNumSlots];     // most recent completed pair
  int sm_count = 0;

  int init(int dev) {
    device = dev;
    CU(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
    CU(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    CU(misc.ensure(sizeof(DevMisc)));
    CU(cudaMemset(misc.p, 0, sizeof(DevMisc)));
    CU(rel_partial.ensure(2 * sizeof(double) * kRelMaxGrid));
    CU(cudaMallocHost((void**)&h_small, 64));
    for (int s = 0; s < kNumSlots; s++) {
      for (int i = 0; i < kRing; i++) {
        CU(cudaEventCreate(&ev[s][i][0]));
        CU(cudaEventCreate(&ev[s][i][1]));
      }
      ev_head[s] = 0;
      ev_pending[s] = 0;
      ev_last[s] = -1;
    }
    CU(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev));
    return SZP_GB300_OK;
  }
  DevMisc* dm() const { return misc.as<DevMisc>(); }

  // Calls of one thread may use different streams: order them on the
  // workspace's look-back words and buffers.  Host-buffer entry points run on
  // the workspace's own stream; device entry points on the caller's stream
  // (NULL = the legacy default stream, as everywhere in CUDA).
  cudaStream_t begin_own() { return begin_on(own); }
  cudaStream_t begin(void* user) { return begin_on((cudaStream_t)user); }
  cudaStream_t begin_on(cudaStream_t st) {
    if (last && last != st) cudaStreamWaitEvent(st, done, 0);
    last = st;
    return st;
  }
  void end(cudaStream_t st) { cudaEventRecord(done, st); }

  void mark(int slot, int which, cudaStream_t st) {
    if (!g_timing) return;
    int h = ev_head[slot];
    cudaEventRecord(ev[slot][h][which], st);
    if (which == 1) {
      ev_last[slot] = h;
      ev_head[slot] = (h + 1) % kRing;
      if (ev_pending[slot] < kRing) ev_pending[slot]++;
    }
  }
};

thread_local std::vector<Workspace*> t_ws;

int get_ws(Workspace** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(SZP_GB300_ECUDA, "no CUDA device: %s", cudaGetErrorString(e));
  if ((int)t_ws.size() <= dev) t_ws.resize(dev + 1, nullptr);
  if (!t_ws[dev]) {
    Workspace* w = new Workspace();
    int rc = w->init(dev);
    if (rc != SZP_GB300_OK) {
      delete w;
      return rc;
    }
    t_ws[dev] = w;
  }
  *out = t_ws[dev];
  return SZP_GB300_OK;
}

int status_from_err(uint32_t err) {
  if (err & kErrCapacity) return fail(SZP_GB300_ECAPACITY, "stream does not fit the output buffer");
  if (err & kErrLookbackTimeout) return fail(SZP_GB300_ETIMEOUT, "a device look-back wait gave up");
  if (err & (kErrCorrupt | kErrBlockCount)) return fail(SZP_GB300_ECORRUPT, "malformed stream (flags 0x%x)", err);
  return SZP_GB300_OK;
}

Segments make_segments(size_t n, int T, int L) {
  Segments s;
  s.n = n;
  s.T = (uint32_t)T;
  s.L = (uint32_t)L;
  s.tsz = n / (uint64_t)T;
  return s;
}

uint64_t seg_blocks_host(const Segments& s, uint32_t t, bool fm2) {
  uint64_t len = s.len(t);
  if (fm2) return (len + s.L - 1) / s.L;
  return len > 1 ? (len - 1 + s.L - 1) / s.L : 0;
}

// tiles of segments 0..T-2 and in total, for tb blocks per tile
void tile_counts(const Segments& s, bool fm2, uint32_t tb, uint64_t& per_seg, uint64_t& total) {
  per_seg = 0;
  if (s.tsz > 0) {
    uint64_t nb = seg_blocks_host(s, 0, fm2);
    per_seg = nb ? (nb + tb - 1) / tb : 1;
  }
  uint64_t last = 0;
  if (s.n > 0) {
    uint64_t nb = seg_blocks_host(s, s.T - 1, fm2);
    last = nb ? (nb + tb - 1) / tb : 1;
  }
  total = (uint64_t)(s.T - 1) * per_seg + last;
  if (total == 0) total = 1;
}

// hb: bytes of the eb header, 4 (float) or 8 (double)
size_t max_stream_bytes(size_t n, int L, int T, int fm, int hb = 4) {
  if (L <= 0 || T <= 0) return 0;
  Segments s = make_segments(n, T, L);
  bool fm2 = fm == 2;
  uint64_t per = fm2 ? (L == 1 ? 5 : 4 + block_bytes((uint32_t)L - 1, kMaxBitCount)) : max_block_bytes((uint32_t)L);
  uint64_t total = (uint64_t)hb + 8ull * (uint64_t)T;
  for (uint32_t t = 0; t < (uint32_t)T; t++) {
    uint64_t len = s.len(t);
    if (!len) continue;
    uint64_t nb = seg_blocks_host(s, t, fm2);
    total += (fm2 ? 0 : 4) + nb * per;
    if (t + 1 < (uint32_t)T && s.tsz > 0) {  // segments 0..T-2 are alike
      total += (uint64_t)(T - 2 - t) * ((fm2 ? 0 : 4) + nb * per);
      t = T - 2;
    }
  }
  return (size_t)total;
}

// ----------------------------------------------------------- compression --
struct CompressJob {
  const float* d_x;
  size_t n;
  int eb_mode;
  float eb_abs;
  double rel;
  int L, T, fm;
  uint8_t* d_out;
  size_t cap;
  unsigned long long* d_size;  // optional: size copied here too
  bool dbl = false;               // float64 data: d_xd and eb_abs_d, 8-byte eb header
  const double* d_xd = nullptr;
  double eb_abs_d = 0.0;
  // int32 codes to pack as they are (the homomorphic reduction): ABS with
  // eb_abs (float stream) or eb_abs_d (dbl: float64 stream), no quantization
  const int32_t* d_codes = nullptr;
  const float* d_eb = nullptr;  // codes: the float header's eb on the device instead of eb_abs
  bool keep_err = false;        // the caller cleared the error word (earlier passes report into it)
};

// The REL range pass over float data: eb = range * (float)rel into dm->eb.
static int launch_rel_float(Workspace& w, const float* d_x, size_t n, double rel, cudaStream_t st) {
  DevMisc* dm = w.dm();
  RelArgs r;
  memset(&r, 0, sizeof r);
  r.x = d_x;
  r.n = n;
  r.rel = (float)rel;
  r.partial = w.rel_partial.as<float>();
  r.counter = &dm->rel_counter;
  r.eb_out = &dm->eb;
  r.err = &dm->err;
  uint64_t want = (n / 4 + 255) / 256;
  uint32_t grid = (uint32_t)(want < 1 ? 1 : want);
  uint32_t lim = (uint32_t)(w.sm_count * 4 < kRelMaxGrid ? w.sm_count * 4 : kRelMaxGrid);
  if (grid > lim) grid = lim;
  w.mark(kSlotRel, 0, st);
  CU(launch_rel_bound(r, grid, st));
  w.mark(kSlotRel, 1, st);
  return SZP_GB300_OK;
}

int compress_launch(Workspace& w, const CompressJob& j, cudaStream_t st) {
  if (j.L <= 0) return fail(SZP_GB300_EINVAL, "blockSize must be positive (got %d)", j.L);
  if (j.T <= 0) return fail(SZP_GB300_EINVAL, "segment count must be positive");
  if (j.fm != 1 && j.fm != 2) return fail(SZP_GB300_EINVAL, "fastMode must be 1 or 2 (got %d)", j.fm);
  const bool dbl = j.dbl;
  const bool codes = j.d_codes != nullptr;
  const void* xin = codes ? (const void*)j.d_codes : dbl ? (const void*)j.d_xd : (const void*)j.d_x;
  if (j.n && !xin) return fail(SZP_GB300_EINVAL, "null input");
  if ((uintptr_t)xin & (dbl && !codes ? 7 : 3)) return fail(SZP_GB300_EINVAL, "input not aligned to its element size");
  if (codes && (j.eb_mode != ABS || !f64_pipe_supported((uint32_t)j.L)))
    return fail(SZP_GB300_EINVAL, "code streams take blockSize 8..256 (got %d)", j.L);
  const uint64_t head = (dbl ? 8 : 4) + 8ull * j.T;
  if (j.cap < head) return fail(SZP_GB300_ECAPACITY, "output buffer smaller than the stream header");
  const bool fm2 = j.fm == 2;
  // float64 data on blockSizes the pipelines take: a quantization pass, then
  // the pipeline over int32 q
  const bool qpipe = codes || (dbl && f64_pipe_supported((uint32_t)j.L));
  Segments sg = make_segments(j.n, j.T, j.L);
  uint32_t bpw = 1;
  uint32_t tb = dbl && !qpipe ? compress_blocks_per_tile_f64((uint32_t)j.L, bpw)
                              : compress_blocks_per_tile((uint32_t)j.L, bpw);
  uint64_t per_seg, ntiles;
  tile_counts(sg, fm2, tb, per_seg, ntiles);
  if (ntiles >= (1ull << 31) || per_seg >= (1ull << 31))
    return fail(SZP_GB300_EINVAL, "input too large for one launch");
  CU(w.status.ensure(ntiles * sizeof(uint64_t)));
  DevMisc* dm = w.dm();
  if (!j.keep_err) CU(cudaMemsetAsync(&dm->err, 0, sizeof(uint32_t), st));

  CompressArgs a;
  memset(&a, 0, sizeof a);
  a.x = j.d_x;
  a.out = j.d_out;
  a.cap = j.cap;
  a.seg = sg;
  a.eb = j.eb_abs;
  a.eb_dev = codes ? j.d_eb : nullptr;
  a.status = w.status.as<uint64_t>();
  a.ls = &dm->ls;
  a.err = &dm->err;
  a.out_size = &dm->out_size;
  a.ntiles = (uint32_t)ntiles;
  a.tiles_per_seg = (uint32_t)per_seg;
  a.tb = tb;
  a.bpw = bpw;
  a.nb_reg = sg.tsz ? seg_blocks_host(sg, 0, fm2) : 0;
  a.nb_last = seg_blocks_host(sg, sg.T - 1, fm2);
  a.thr = table();
  a.xd = j.d_xd;
  a.ebd = j.eb_abs_d;
  a.invd = dbl ? 1.0 / j.eb_abs_d : 0.0;  // binary64 division, as the reference's inverse
  a.qhb = dbl ? 8 : 4;

  int launches = 0;
  if (j.eb_mode == REL && dbl) {
    RelArgs r;
    memset(&r, 0, sizeof r);
    r.xd = j.d_xd;
    r.n = j.n;
    r.rel_d = j.rel;
    r.partial = w.rel_partial.as<float>();  // 2 doubles per CTA
    r.counter = &dm->rel_counter;
    r.ebd_out = &dm->ebd;
    r.invd_out = &dm->invd;
    uint64_t want = (j.n / 4 + 255) / 256;
    uint32_t grid = (uint32_t)(want < 1 ? 1 : want);
    uint32_t lim = (uint32_t)(w.sm_count * 4 < kRelMaxGrid ? w.sm_count * 4 : kRelMaxGrid);
    if (grid > lim) grid = lim;
    w.mark(kSlotRel, 0, st);
    CU(launch_rel_bound_f64(r, grid, st));
    w.mark(kSlotRel, 1, st);
    a.ebd_dev = &dm->ebd;
    a.invd_dev = &dm->invd;
    launches++;
  } else if (j.eb_mode == REL) {
    const int rc = launch_rel_float(w, j.d_x, j.n, j.rel, st);
    if (rc) return rc;
    a.eb_dev = &dm->eb;
    launches++;
  }
  size_t smem = dbl && !qpipe ? compress_smem_bytes_f64((uint32_t)j.L, tb) : compress_smem_bytes((uint32_t)j.L, tb);
  if (smem > 200 * 1024) return fail(SZP_GB300_EINVAL, "blockSize %d too large", j.L);
  int32_t* q = nullptr;
  if (qpipe && !codes) {
    CU(w.qbuf.ensure((j.n + 4) * sizeof(int32_t)));
    q = f64_q_view(w.qbuf.p, j.d_xd);
  }
  w.mark(kSlotCompress, 0, st);
  if (codes) {
    a.x = reinterpret_cast<const float*>(j.d_codes);
    CU(launch_compress_q(a, fm2, st));
  } else if (qpipe) {
    CU(launch_quantize_f64(j.d_xd, q, j.n, a.invd, a.invd_dev, a.err, (uint32_t)w.sm_count, st));
    a.x = reinterpret_cast<const float*>(q);
    CU(launch_compress_q(a, fm2, st));
    launches++;
  } else {
    CU(dbl ? launch_compress_f64(a, fm2, st) : launch_compress(a, fm2, st));
  }
  w.mark(kSlotCompress, 1, st);
  launches++;
  if (j.d_size) CU(cudaMemcpyAsync(j.d_size, &dm->out_size, 8, cudaMemcpyDeviceToDevice, st));
  count_launches(launches);
  return SZP_GB300_OK;
}

// Copies the stream size and error word to pinned memory and waits.
int finish_sync(Workspace& w, cudaStream_t st, size_t* out_size) {
  DevMisc* dm = w.dm();
  CU(cudaMemcpyAsync(w.h_small, &dm->out_size, 8, cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(w.h_small + 8, &dm->err, 4, cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  uint64_t sz;
  uint32_t err;
  memcpy(&sz, w.h_small, 8);
  memcpy(&err, w.h_small + 8, 4);
  t_notices = (err & kErrQuantRange) ? 1 : 0;
  if (out_size) *out_size = (size_t)sz;
  return status_from_err(err);
}

// --------------------------------------------------------- decompression --
struct DecompressJob {
  const uint8_t* d_in;
  size_t len;
  const uint64_t* d_len;
  size_t n;
  int L, T, fm;
  float* d_y;
  bool dbl = false;        // float64 stream: output of doubles in d_yd (8-byte eb header)
  double* d_yd = nullptr;
  int32_t* d_codes = nullptr;  // output of the int32 codes instead (the homomorphic reduction)
  bool accumulate = false;     // ... added to the codes already in d_codes
};

int decompress_launch(Workspace& w, const DecompressJob& j, cudaStream_t st) {
  if (j.L <= 0) return fail(SZP_GB300_EINVAL, "blockSize must be positive (got %d)", j.L);
  if (j.T <= 0) return fail(SZP_GB300_EINVAL, "segment count must be positive");
  if (j.fm != 1 && j.fm != 2) return fail(SZP_GB300_EINVAL, "fastMode must be 1 or 2 (got %d)", j.fm);
  const bool dbl = j.dbl;
  const uint64_t head = (dbl ? 8 : 4) + 8ull * j.T;
  if (j.len < head) return fail(SZP_GB300_ECORRUPT, "stream shorter than its header");
  const bool codes = j.d_codes != nullptr;
  void* yout = codes ? (void*)j.d_codes : dbl ? (void*)j.d_yd : (void*)j.d_y;
  if (j.n && !yout) return fail(SZP_GB300_EINVAL, "null output");
  if ((uintptr_t)yout & (dbl && !codes ? 7 : 3)) return fail(SZP_GB300_EINVAL, "output not aligned to its element size");
  if (codes && !f64_pipe_supported((uint32_t)j.L))
    return fail(SZP_GB300_EINVAL, "code streams take blockSize 8..256 (got %d)", j.L);
  const bool fm2 = j.fm == 2;
  const bool qpipe = codes || (dbl && f64_pipe_supported((uint32_t)j.L));  // a pipeline writing doubles or codes
  Segments sg = make_segments(j.n, j.T, j.L);
  const uint32_t maxsz = fm2 ? (j.L == 1 ? 5u : 4 + block_bytes((uint32_t)j.L - 1, kMaxBitCount))
                             : max_block_bytes((uint32_t)j.L);
  if (maxsz > 16384) return fail(SZP_GB300_EINVAL, "blockSize %d too large", j.L);
  const uint32_t C = locate_chunk_bytes(maxsz);
  const uint32_t SC = locate_super_bytes(maxsz);
  const uint64_t nlocate = (j.len + SC - 1) / SC + (uint64_t)j.T + 1;
  uint32_t bpw = 1;
  uint32_t tb = dbl && !qpipe ? decode_blocks_per_tile_f64((uint32_t)j.L, bpw)
                              : decode_blocks_per_tile((uint32_t)j.L, bpw);
  uint64_t per_seg, ntiles;
  tile_counts(sg, fm2, tb, per_seg, ntiles);
  uint64_t nblk_total = 0;
  if (sg.n) {
    nblk_total = (uint64_t)(sg.T - 1) * (sg.tsz ? seg_blocks_host(sg, 0, fm2) : 0) + seg_blocks_host(sg, sg.T - 1, fm2);
  }
  if (ntiles >= (1ull << 31) || nlocate >= (1ull << 31)) return fail(SZP_GB300_EINVAL, "input too large");
  const uint64_t nstatus = ntiles > nlocate ? ntiles : nlocate;
  CU(w.status.ensure(nstatus * sizeof(uint64_t)));
  CU(w.walks.ensure(nlocate * sizeof(uint2)));
  CU(w.blkpos.ensure((nblk_total + 1) * sizeof(uint32_t)));
  const size_t plan_bytes = 64 + 4ull * (j.T + 1) + 16ull * j.T + 64;
  CU(w.plan.ensure(plan_bytes));
  DevMisc* dm = w.dm();
  CU(cudaMemsetAsync(&dm->err, 0, sizeof(uint32_t), st));

  DecArgs a;
  memset(&a, 0, sizeof a);
  DecField& f = a.f;
  f.in = j.d_in;
  f.len = j.len;
  f.len_dev = j.d_len;
  f.seg = sg;
  a.fm2 = fm2;
  a.hb = dbl ? 8 : 4;
  uint8_t* pb = w.plan.as<uint8_t>();
  f.plan = reinterpret_cast<DecPlan*>(pb);
  f.reg0 = reinterpret_cast<uint64_t*>(pb + 64);
  f.reg1 = f.reg0 + j.T;
  f.chunk_base = reinterpret_cast<uint32_t*>(f.reg1 + j.T);
  a.chunk = C;
  a.super_chunk = SC;
  a.overlap = g_overlap >= 0 ? (uint32_t)g_overlap : locate_overlap_bytes(maxsz);
  a.maxsz = maxsz;
  a.aux = w.walks.as<uint2>();
  a.counters = dm->verify;
  a.status = w.status.as<uint64_t>();
  a.ls = &dm->ls;
  a.err = &dm->err;
  f.err = &dm->err;
  f.blkpos = w.blkpos.as<uint32_t>();
  f.nblk_total = nblk_total;
  f.y = j.d_y;
  f.yd = j.d_yd;
  f.ntiles = (uint32_t)ntiles;
  f.tiles_per_seg = (uint32_t)per_seg;
  f.tile_base = 0;
  f.loc_base = 0;
  f.loc_ctas = (uint32_t)nlocate;
  a.ntiles = (uint32_t)ntiles;
  a.tb = tb;
  a.bpw = bpw;
  a.nlocate_ctas = (uint32_t)nlocate;
  a.static_tiles = g_decode_tickets ? 0u : 1u;
  if (((!dbl || qpipe) && decode_smem_bytes((uint32_t)j.L, tb, fm2) > 200 * 1024) ||
      locate_smem_bytes(SC, a.overlap, maxsz) > 200 * 1024)
    return fail(SZP_GB300_EINVAL, "blockSize too large");
  if (qpipe) f.y = reinterpret_cast<float*>(codes ? (void*)j.d_codes : (void*)j.d_yd);  // it writes doubles or codes
  CU(cudaMemsetAsync(dm->verify, 0, sizeof(uint32_t), st));

  w.mark(kSlotSetup, 0, st);
  CU(launch_dec_setup(a, st));
  w.mark(kSlotSetup, 1, st);
  w.mark(kSlotLocate, 0, st);
  CU(launch_locate(a, st));
  w.mark(kSlotLocate, 1, st);
  w.mark(kSlotDecode, 0, st);
  CU(codes ? launch_decode_codes(a, j.accumulate, st)
            : qpipe ? launch_decode_q(a, st) : dbl ? launch_decode_f64(a, st) : launch_decode(a, st));
  w.mark(kSlotDecode, 1, st);
  count_launches(3);
  return SZP_GB300_OK;
}

// Host-side stream length: segment offsets give every segment's start; the
// last one is walked block by block (the stream does not record its end).
int host_stream_length(const uint8_t* stream, size_t n, int L, int T, int fm, size_t* len, int hb = 4) {
  if (L <= 0 || T <= 0) return fail(SZP_GB300_EINVAL, "bad blockSize/segments");
  Segments s = make_segments(n, T, L);
  const bool fm2 = fm == 2;
  const uint64_t head = (uint64_t)hb + 8ull * T;
  uint64_t off = 0;
  memcpy(&off, stream + hb + 8ull * (T - 1), 8);
  const uint8_t* p = stream + head + off;
  uint64_t seglen = s.len(T - 1);
  if (seglen == 0) {
    *len = (size_t)(head + off);
    return SZP_GB300_OK;
  }
  uint64_t nb = seg_blocks_host(s, T - 1, fm2);
  if (!fm2) p += 4;
  uint64_t lo = s.lo(T - 1), hi = s.hi(T - 1);
  for (uint64_t b = 0; b < nb; b++) {
    uint64_t start = fm2 ? lo + b * L + 1 : lo + 1 + b * L;
    uint64_t end = start + (fm2 ? L - 1 : L);
    if (end > hi) end = hi;
    uint32_t m = end > start ? (uint32_t)(end - start) : 0;
    if (fm2) {
      p += 4;
      // the encoder writes a header byte even for a one-element block
    }
    uint32_t bc = *p;
    if (bc > (uint32_t)kMaxBitCount) return fail(SZP_GB300_ECORRUPT, "invalid bit count %u in last segment", bc);
    p += (m == 0) ? 1 : block_bytes(m, bc);
  }
  *len = (size_t)(p - stream);
  return SZP_GB300_OK;
}

// The reference's single-thread _record entry points return
// `total_memaccess`, their own tally of the bytes each statement touches
// (szp_float.cc:607-750, szpd_float.cc:216-318, szp_double.cc:613-756,
// szpd_double.cc:219-321).  In closed form over the T = 1 fastmode1 stream
// those functions write and read, with q the value size (4 float, 8 double),
// S the segment's bytes (seed and blocks), E0 the elements of zero blocks and
// E1 the elements of the other blocks:
//   compress    64 + [n>0](q + 4) + (q + 5)(n - 1) + 3S + 5 E1
//   decompress  8 + [n>0](8 + 2q) + (S - 4[n>0]) + 2q E0 + (10 + 2q) E1
// The blocks' bit counts come from one host walk of the segment.
struct RecordTally {
  uint64_t seg_bytes = 0, e0 = 0, e1 = 0;
};

static int host_record_tally(const uint8_t* stream, size_t len, size_t n, int L, int hb, RecordTally* t) {
  *t = RecordTally();
  if (L <= 0) return fail(SZP_GB300_EINVAL, "bad blockSize");
  const uint64_t head = (uint64_t)hb + 8;
  if (len < head) return fail(SZP_GB300_ECORRUPT, "stream shorter than its header");
  uint64_t off = 0;
  memcpy(&off, stream + hb, 8);
  if (n == 0) return SZP_GB300_OK;
  uint64_t p = head + off + 4;  // the seed
  for (uint64_t i = 1; i < n; i += (uint64_t)L) {
    const uint32_t m = (uint32_t)std::min<uint64_t>((uint64_t)L, n - i);
    if (p >= len) return fail(SZP_GB300_ECORRUPT, "stream ends inside its blocks");
    const uint32_t bc = stream[p];
    if (bc > (uint32_t)kMaxBitCount) return fail(SZP_GB300_ECORRUPT, "invalid bit count %u", bc);
    (bc ? t->e1 : t->e0) += m;
    p += block_bytes(m, bc);
  }
  if (p > len) return fail(SZP_GB300_ECORRUPT, "stream ends inside its blocks");
  t->seg_bytes = p - head - off;
  return SZP_GB300_OK;
}

static size_t record_compress_tally(const RecordTally& t, size_t n, uint64_t q) {
  const uint64_t nz = n > 0, e = n > 0 ? n - 1 : 0;
  return (size_t)(64 + nz * (q + 4) + (q + 5) * e + 3 * t.seg_bytes + 5 * t.e1);
}

static size_t record_decompress_tally(const RecordTally& t, size_t n, uint64_t q) {
  const uint64_t nz = n > 0;
  return (size_t)(8 + nz * (8 + 2 * q) + (t.seg_bytes - 4 * nz) + 2 * q * t.e0 + (10 + 2 * q) * t.e1);
}

// ------------------------------------------------- host-buffer pipelines --
size_t host_page_bytes() {
  static const size_t page = [] {
    long v = sysconf(_SC_PAGESIZE);
    return v > 0 ? (size_t)v : (size_t)4096;
  }();
  return page;
}

// Maps the pages of host range [p, p + bytes): one write per page, inside the
// range, so a neighbouring range being copied into is never touched.  (One
// madvise(MADV_POPULATE_WRITE) per range measured slower when threads do it
// side by side: 537 MB took 9.4 ms against 5.1 ms by touching.)
void touch_pages(uint8_t* p, size_t bytes) {
  const size_t page = host_page_bytes();
  volatile uint8_t* b = p;
  for (size_t o = 0; o < bytes;) {
    b[o] = 0;
    o = (((uintptr_t)(p + o) / page) + 1) * page - (uintptr_t)p;
  }
}

// Maps [p, p + bytes) with all OpenMP threads (1 MiB per task).
void map_pages(uint8_t* p, size_t bytes) {
  constexpr size_t kBatch = (size_t)1 << 20;
  if (bytes < 8 * kBatch) {
    touch_pages(p, bytes);
    return;
  }
  const int64_t nb = (int64_t)((bytes + kBatch - 1) / kBatch);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t b = 0; b < nb; b++) touch_pages(p + b * kBatch, std::min(kBatch, bytes - (size_t)b * kBatch));
}

// Copies a device result into host memory that may be fresh (a malloc'd
// result): worker threads map its pages ahead in address order while one
// thread issues 16 MiB copies behind them, so the page faults overlap the
// transfer instead of landing inside it (a copy into unmapped pages takes its
// faults one at a time).  The copies are ordered on `st` after earlier work;
// returns once they have landed.
cudaError_t copy_to_host(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return cudaSuccess;
  uint8_t* d = static_cast<uint8_t*>(dst);
  const uint8_t* s = static_cast<const uint8_t*>(src);
  constexpr size_t kBatch = (size_t)1 << 20, kChunk = 16 * kBatch;
  if (bytes < 2 * kChunk || omp_get_max_threads() < 2) {
    touch_pages(d, bytes);
    cudaError_t e = cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToHost, st);
    return e == cudaSuccess ? cudaStreamSynchronize(st) : e;
  }
  const size_t nbatch = (bytes + kBatch - 1) / kBatch, nchunk = (bytes + kChunk - 1) / kChunk;
  std::unique_ptr<std::atomic<uint32_t>[]> left(new std::atomic<uint32_t>[nchunk]);
  for (size_t c = 0; c < nchunk; c++) left[c].store((uint32_t)std::min<size_t>(16, nbatch - 16 * c));
  std::atomic<size_t> next{0};
  auto map_one = [&]() -> bool {  // maps the next batch; false when none is left
    const size_t b = next.fetch_add(1, std::memory_order_relaxed);
    if (b >= nbatch) return false;
    touch_pages(d + b * kBatch, std::min(kBatch, bytes - b * kBatch));
    left[b / 16].fetch_sub(1, std::memory_order_release);
    return true;
  };
  cudaError_t err = cudaSuccess;
#pragma omp parallel
  {
    if (omp_get_thread_num() == 0) {
      for (size_t c = 0; c < nchunk; c++) {
        while (left[c].load(std::memory_order_acquire) != 0)
          if (!map_one()) std::this_thread::yield();  // help, or wait for the batch in flight
        const size_t o = c * kChunk;
        if (err == cudaSuccess) err = cudaMemcpyAsync(d + o, s + o, std::min(kChunk, bytes - o), cudaMemcpyDeviceToHost, st);
      }
    } else {
      while (map_one()) {
      }
    }
  }
  return err == cudaSuccess ? cudaStreamSynchronize(st) : err;
}

// Host-buffer compressor: float data (dbl false, eb_abs is the float bound)
// or double data (dbl true, 8-byte eb header, szp_double.cc).
int compress_host(const void* data, bool dbl, size_t n, int eb_mode, double eb_abs, double rel, int L, int T,
                  int fm, uint8_t** out_malloc, uint8_t* out_user, size_t user_cap, size_t* out_size) {
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  cudaStream_t st = w->begin_own();
  if (n && !data) return fail(SZP_GB300_EINVAL, "null input");
  const size_t elem = dbl ? sizeof(double) : sizeof(float);
  const size_t cap = max_stream_bytes(n, L, T, fm, (int)elem);
  if (!cap) return fail(SZP_GB300_EINVAL, "bad blockSize/segments");
  CU(w->in.ensure(n * elem + 16));
  CU(w->stream.ensure(cap));
  if (n) CU(cudaMemcpyAsync(w->in.p, data, n * elem, cudaMemcpyHostToDevice, st));
  CompressJob j{dbl ? nullptr : w->in.as<float>(), n, eb_mode, (float)eb_abs, rel, L, T, fm,
                w->stream.as<uint8_t>(), cap, nullptr};
  if (dbl) {
    j.dbl = true;
    j.d_xd = w->in.as<double>();
    j.eb_abs_d = eb_abs;
  }
  rc = compress_launch(*w, j, st);
  if (rc) return rc;
  // a malloc'd result is allocated while the GPU works, and as many of its
  // pages as the previous stream of this thread had are mapped meanwhile (the
  // stream's size is known only at the end)
  uint8_t* dst = out_user;
  if (!dst) {
    const size_t alloc = std::max(cap, elem + elem * n);  // the reference hands out sizeof(T) * (1 + n)
    dst = (uint8_t*)malloc(alloc);
    if (!dst) {
      finish_sync(*w, st, nullptr);
      w->end(st);
      return fail(SZP_GB300_ENOMEM, "malloc(%zu) failed", alloc);
    }
    map_pages(dst, std::min(w->last_stream, alloc));
  }
  size_t sz = 0;
  rc = finish_sync(*w, st, &sz);
  w->end(st);
  if (rc) {
    if (!out_user) free(dst);
    return rc;
  }
  w->last_stream = sz;
  if (out_user && sz > user_cap) {
    return fail(SZP_GB300_ECAPACITY, "stream of %zu bytes exceeds the %zu-byte output", sz, user_cap);
  }
  cudaError_t e = copy_to_host(dst, w->stream.p, sz, st);
  if (e != cudaSuccess) {
    if (!out_user) free(dst);
    return fail(SZP_GB300_ECUDA, "copy of the stream failed: %s", cudaGetErrorString(e));
  }
  if (out_malloc) *out_malloc = dst;
  *out_size = sz;
  return SZP_GB300_OK;
}

// stream: whole stream (eb first) unless after_eb; then the bytes after eb
// (the per-type entries) and eb is eb_value.  dbl: a float64 stream (8-byte
// eb header, double output).
int decompress_host(const uint8_t* bytes, size_t len, bool len_known, size_t n, int L, int T, int fm,
                    bool after_eb, double eb_value, void** out_malloc, void* out_user, bool dbl = false) {
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  if (!bytes) return fail(SZP_GB300_EINVAL, "null stream");
  if (L <= 0 || T <= 0) return fail(SZP_GB300_EINVAL, "bad blockSize/segments");
  const int hb = dbl ? 8 : 4;
  const size_t elem = dbl ? sizeof(double) : sizeof(float);
  const uint64_t head = (uint64_t)hb + 8ull * T;
  // stream as seen from its eb header
  const uint8_t* full = after_eb ? bytes - hb : bytes;
  size_t total = len;
  if (!len_known || total < head) {
    // host_stream_length never reads the eb bytes, so `full` may point
    // before the caller's buffer when only the bytes after eb were given
    rc = host_stream_length(full, n, L, T, fm, &total, hb);
    if (rc) return rc;
  } else {
    size_t bound = max_stream_bytes(n, L, T, fm, hb);
    if (total > bound) total = bound;
  }
  cudaStream_t st = w->begin_own();
  CU(w->stream.ensure(total + 16));
  CU(w->out.ensure(n * elem + 16));
  uint8_t* d_stream = w->stream.as<uint8_t>();
  if (after_eb) {
    uint8_t be[8];
    if (dbl) {
      uint64_t b;
      memcpy(&b, &eb_value, 8);
      for (int i = 0; i < 8; i++) be[i] = (uint8_t)(b >> (56 - 8 * i));
    } else {
      const float f = (float)eb_value;
      uint32_t b;
      memcpy(&b, &f, 4);
      for (int i = 0; i < 4; i++) be[i] = (uint8_t)(b >> (24 - 8 * i));
    }
    memcpy(w->h_small + 16, be, hb);
    CU(cudaMemcpyAsync(d_stream, w->h_small + 16, hb, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(d_stream + hb, bytes, total - hb, cudaMemcpyHostToDevice, st));
  } else {
    CU(cudaMemcpyAsync(d_stream, bytes, total, cudaMemcpyHostToDevice, st));
  }
  DecompressJob j{d_stream, total, nullptr, n, L, T, fm, dbl ? nullptr : w->out.as<float>()};
  if (dbl) {
    j.dbl = true;
    j.d_yd = w->out.as<double>();
  }
  rc = decompress_launch(*w, j, st);
  if (rc) return rc;
  void* dst = out_user;
  if (!dst) {
    dst = malloc(n ? n * elem : 1);
    if (!dst) {
      finish_sync(*w, st, nullptr);
      w->end(st);
      return fail(SZP_GB300_ENOMEM, "malloc failed");
    }
  }
  // the status words, then the values (their pages mapped while the kernels
  // and the first copies run); the status decides whether they are returned
  DevMisc* dm = w->dm();
  CU(cudaMemcpyAsync(w->h_small + 8, &dm->err, 4, cudaMemcpyDeviceToHost, st));
  cudaError_t e = copy_to_host(dst, w->out.p, n * elem, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  w->end(st);
  if (e != cudaSuccess) {
    if (!out_user) free(dst);
    return fail(SZP_GB300_ECUDA, "copy of the data failed: %s", cudaGetErrorString(e));
  }
  uint32_t err;
  memcpy(&err, w->h_small + 8, 4);
  t_notices = (err & kErrQuantRange) ? 1 : 0;
  rc = status_from_err(err);
  if (rc) {
    if (!out_user) free(dst);
    return rc;
  }
  if (out_malloc) *out_malloc = dst;
  return SZP_GB300_OK;
}

}  // namespace

// Host helpers shared with noalloc.cu (no allocation in any of them).
namespace szp {
const BitcountTable& host_bitcount_table() { return table(); }
int host_resolve_segments(int requested) { return resolve_segments(requested); }
void host_compress_tiles(size_t n, int T, int L, uint64_t& tiles_per_seg, uint64_t& ntiles, uint32_t& tb,
                         uint32_t& bpw) {
  tb = compress_blocks_per_tile((uint32_t)L, bpw);
  Segments sg = make_segments(n, T, L);
  tile_counts(sg, false, tb, tiles_per_seg, ntiles);
}
void host_tile_counts(size_t n, int T, int L, uint32_t tb, uint64_t& tiles_per_seg, uint64_t& ntiles) {
  Segments sg = make_segments(n, T, L);
  tile_counts(sg, false, tb, tiles_per_seg, ntiles);
}
uint64_t host_block_count(size_t n, int T, int L) {
  Segments sg = make_segments(n, T, L);
  if (!sg.n) return 0;
  return (uint64_t)(sg.T - 1) * (sg.tsz ? seg_blocks_host(sg, 0, false) : 0) + seg_blocks_host(sg, sg.T - 1, false);
}
size_t host_max_stream_bytes(size_t n, int L, int T) { return max_stream_bytes(n, L, T, 1); }
int host_status_from_err(uint32_t err) { return status_from_err(err); }
void host_segment_blocks(size_t n, int T, int L, uint64_t& nb_reg, uint64_t& nb_last) {
  Segments sg = make_segments(n, T, L);
  nb_reg = sg.tsz ? seg_blocks_host(sg, 0, false) : 0;
  nb_last = seg_blocks_host(sg, sg.T - 1, false);
}
int host_fail(int status, const char* msg) { return fail(status, "%s", msg); }
void host_set_notices(uint32_t err) { t_notices = (err & kErrQuantRange) ? 1 : 0; }
void host_clear_error() { clear_error(); }
void host_count_launches(int k) { count_launches(k); }
}  // namespace szp

// =============================================================== C ABI ====
// Per-type entry points (float or double), shared by the C ABI below.
template <typename V>
static unsigned char* fm_compress_alloc(V* x, size_t* outSize, V eb, size_t n, int L, int T, int fm) {
  clear_error();
  if (outSize) *outSize = 0;
  if (!outSize) {
    fail(SZP_GB300_EINVAL, "null outSize");
    return nullptr;
  }
  uint8_t* out = nullptr;
  int rc = compress_host(x, sizeof(V) == 8, n, ABS, (double)eb, 0.0, L, T, fm, &out, nullptr, 0, outSize);
  return rc ? nullptr : out;
}

// The reference's callers size `output` as sizeof(V) * (1 + n) bytes (szp.cc:53).
template <typename V>
static void fm_compress_arg(unsigned char* output, V* x, size_t* outSize, V eb, size_t n, int L, int T, int fm) {
  clear_error();
  if (!outSize) {
    fail(SZP_GB300_EINVAL, "null outSize");
    return;
  }
  *outSize = 0;
  if (!output) {
    fail(SZP_GB300_EINVAL, "null output");
    return;
  }
  size_t sz = 0;
  int rc = compress_host(x, sizeof(V) == 8, n, ABS, (double)eb, 0.0, L, T, fm, nullptr, output,
                         sizeof(V) + sizeof(V) * n, &sz);
  if (!rc) *outSize = sz;
}

template <typename V>
static V* fm_decompress_alloc(size_t n, V eb, int L, unsigned char* cmp, int T, int fm) {
  clear_error();
  void* y = nullptr;
  int rc = decompress_host(cmp, 0, false, n, L, T, fm, true, (double)eb, &y, nullptr, sizeof(V) == 8);
  return rc ? nullptr : static_cast<V*>(y);
}

template <typename V>
static void fm_decompress_arg(V* out, size_t n, V eb, int L, unsigned char* cmp, int T, int fm) {
  clear_error();
  if (!out && n) {
    fail(SZP_GB300_EINVAL, "null output");
    return;
  }
  decompress_host(cmp, 0, false, n, L, T, fm, true, (double)eb, nullptr, out, sizeof(V) == 8);
}

extern "C" {

unsigned char* szp_compress(int fastMode, int dataType, void* data, size_t* outSize, int errBoundMode,
                            double absErrBound, double relBoundRatio, size_t nbEle, int blockSize) {
  clear_error();
  if (outSize) *outSize = 0;
  if (fastMode != SZP_NONRANDOMACCESS && fastMode != SZP_RANDOMACCESS) {
    fail(SZP_GB300_EINVAL, "fastMode must be 1 or 2");
    return nullptr;
  }
  if (!outSize) {
    fail(SZP_GB300_EINVAL, "null outSize");
    return nullptr;
  }
  uint8_t* out = nullptr;
  int T = resolve_segments(0);
  // any dataType but SZ_FLOAT is double data (szp.cc:71); the float bound is
  // (float)absErrBound (szp.cc:31), the double one absErrBound itself (szp.cc:74)
  const bool dbl = dataType != SZ_FLOAT;
  int rc = compress_host(data, dbl, nbEle, errBoundMode == REL ? REL : ABS,
                         dbl ? absErrBound : (double)(float)absErrBound, relBoundRatio, blockSize, T, fastMode,
                         &out, nullptr, 0, outSize);
  return rc ? nullptr : out;
}

void* szp_decompress(int fastMode, int dataType, unsigned char* bytes, size_t byteLength, size_t nbEle,
                     int blockSize) {
  clear_error();
  int fm = fastMode == SZP_NONRANDOMACCESS ? 1 : 2;  // the reference treats any other mode as 2
  int T = resolve_segments(0);
  void* y = nullptr;
  int rc = decompress_host(bytes, byteLength, true, nbEle, blockSize, T, fm, false, 0.0, &y, nullptr,
                           dataType != SZ_FLOAT);
  return rc ? nullptr : y;
}



unsigned char* szp_float_openmp_threadblock(float* oriData, size_t* outSize, float absErrBound, size_t nbEle,
                                            int blockSize) {
  return fm_compress_alloc(oriData, outSize, absErrBound, nbEle, blockSize, resolve_segments(0), 1);
}

void szp_float_openmp_threadblock_arg(unsigned char* output, float* oriData, size_t* outSize, float absErrBound,
                                      size_t nbEle, int blockSize) {
  fm_compress_arg(output, oriData, outSize, absErrBound, nbEle, blockSize, resolve_segments(0), 1);
}

void szp_float_single_thread_arg(unsigned char* output, float* oriData, size_t* outSize, float absErrBound,
                                 size_t nbEle, int blockSize) {
  fm_compress_arg(output, oriData, outSize, absErrBound, nbEle, blockSize, 1, 1);
}

size_t szp_float_single_thread_arg_record(unsigned char* output, float* oriData, size_t* outSize,
                                          float absErrBound, size_t nbEle, int blockSize) {
  fm_compress_arg(output, oriData, outSize, absErrBound, nbEle, blockSize, 1, 1);
  if (t_status || !outSize || !*outSize) return 0;
  RecordTally t;
  if (host_record_tally(output, *outSize, nbEle, blockSize, 4, &t)) return 0;
  return record_compress_tally(t, nbEle, 4);
}

unsigned char* szp_float_openmp_threadblock_randomaccess(float* oriData, size_t* outSize, float absErrBound,
                                                         size_t nbEle, int blockSize) {
  return fm_compress_alloc(oriData, outSize, absErrBound, nbEle, blockSize, resolve_segments(0), 2);
}

void szp_float_openmp_threadblock_randomaccess_arg(unsigned char* output, float* oriData, size_t* outSize,
                                                   float absErrBound, size_t nbEle, int blockSize) {
  fm_compress_arg(output, oriData, outSize, absErrBound, nbEle, blockSize, resolve_segments(0), 2);
}

// float64 compressors, SZp/include/szp_double.h (szp_double.cc:149-1090)
unsigned char* szp_double_openmp_threadblock(double* oriData, size_t* outSize, double absErrBound, size_t nbEle,
                                             int blockSize) {
  return fm_compress_alloc(oriData, outSize, absErrBound, nbEle, blockSize, resolve_segments(0), 1);
}

void szp_double_openmp_threadblock_arg(unsigned char* output, double* oriData, size_t* outSize,
                                       double absErrBound, size_t nbEle, int blockSize) {
  fm_compress_arg(output, oriData, outSize, absErrBound, nbEle, blockSize, resolve_segments(0), 1);
}

void szp_double_single_thread_arg(unsigned char* output, double* oriData, size_t* outSize, double absErrBound,
                                  size_t nbEle, int blockSize) {
  fm_compress_arg(output, oriData, outSize, absErrBound, nbEle, blockSize, 1, 1);
}

size_t szp_double_single_thread_arg_record(unsigned char* output, double* oriData, size_t* outSize,
                                           double absErrBound, size_t nbEle, int blockSize) {
  fm_compress_arg(output, oriData, outSize, absErrBound, nbEle, blockSize, 1, 1);
  if (t_status || !outSize || !*outSize) return 0;
  RecordTally t;
  if (host_record_tally(output, *outSize, nbEle, blockSize, 8, &t)) return 0;
  return record_compress_tally(t, nbEle, 8);
}

unsigned char* szp_double_openmp_threadblock_randomaccess(double* oriData, size_t* outSize, double absErrBound,
                                                          size_t nbEle, int blockSize) {
  return fm_compress_alloc(oriData, outSize, absErrBound, nbEle, blockSize, resolve_segments(0), 2);
}

void szp_double_openmp_threadblock_randomaccess_arg(unsigned char* output, double* oriData, size_t* outSize,
                                                    double absErrBound, size_t nbEle, int blockSize) {
  fm_compress_arg(output, oriData, outSize, absErrBound, nbEle, blockSize, resolve_segments(0), 2);
}



float* szp_float_decompress_openmp_threadblock(size_t nbEle, float absErrBound, int blockSize,
                                               unsigned char* cmpBytes) {
  return fm_decompress_alloc(nbEle, absErrBound, blockSize, cmpBytes, resolve_segments(0), 1);
}

void szp_float_decompress_openmp_threadblock_arg(float* newData, size_t nbEle, float absErrBound, int blockSize,
                                                 unsigned char* cmpBytes) {
  fm_decompress_arg(newData, nbEle, absErrBound, blockSize, cmpBytes, resolve_segments(0), 1);
}

void szp_float_decompress_single_thread_arg(float* newData, size_t nbEle, float absErrBound, int blockSize,
                                            unsigned char* cmpBytes) {
  fm_decompress_arg(newData, nbEle, absErrBound, blockSize, cmpBytes, 1, 1);
}

size_t szp_float_decompress_single_thread_arg_record(float* newData, size_t nbEle, float absErrBound,
                                                     int blockSize, unsigned char* cmpBytes) {
  fm_decompress_arg(newData, nbEle, absErrBound, blockSize, cmpBytes, 1, 1);
  if (t_status) return 0;
  size_t len = 0;
  if (host_stream_length(cmpBytes - 4, nbEle, blockSize, 1, 1, &len)) return 0;
  RecordTally t;
  if (host_record_tally(cmpBytes - 4, len, nbEle, blockSize, 4, &t)) return 0;
  return record_decompress_tally(t, nbEle, 4);
}

float* szp_float_decompress_openmp_threadblock_randomaccess(size_t nbEle, float absErrBound, int blockSize,
                                                            unsigned char* cmpBytes) {
  return fm_decompress_alloc(nbEle, absErrBound, blockSize, cmpBytes, resolve_segments(0), 2);
}

void szp_float_decompress_openmp_threadblock_randomaccess_arg(float* newData, size_t nbEle, float absErrBound,
                                                              int blockSize, unsigned char* cmpBytes) {
  fm_decompress_arg(newData, nbEle, absErrBound, blockSize, cmpBytes, resolve_segments(0), 2);
}

// float64 decompressors, SZp/include/szpd_double.h (szpd_double.cc:23-645);
// cmpBytes points after the 8-byte eb
double* szp_double_decompress_openmp_threadblock(size_t nbEle, double absErrBound, int blockSize,
                                                 unsigned char* cmpBytes) {
  return fm_decompress_alloc(nbEle, absErrBound, blockSize, cmpBytes, resolve_segments(0), 1);
}

void szp_double_decompress_openmp_threadblock_arg(double* newData, size_t nbEle, double absErrBound,
                                                  int blockSize, unsigned char* cmpBytes) {
  fm_decompress_arg(newData, nbEle, absErrBound, blockSize, cmpBytes, resolve_segments(0), 1);
}

void szp_double_decompress_single_thread_arg(double* newData, size_t nbEle, double absErrBound, int blockSize,
                                             unsigned char* cmpBytes) {
  fm_decompress_arg(newData, nbEle, absErrBound, blockSize, cmpBytes, 1, 1);
}

size_t szp_double_decompress_single_thread_arg_record(double* newData, size_t nbEle, double absErrBound,
                                                      int blockSize, unsigned char* cmpBytes) {
  fm_decompress_arg(newData, nbEle, absErrBound, blockSize, cmpBytes, 1, 1);
  if (t_status) return 0;
  size_t len = 0;
  if (host_stream_length(cmpBytes - 8, nbEle, blockSize, 1, 1, &len, 8)) return 0;
  RecordTally t;
  if (host_record_tally(cmpBytes - 8, len, nbEle, blockSize, 8, &t)) return 0;
  return record_decompress_tally(t, nbEle, 8);
}

double* szp_double_decompress_openmp_threadblock_randomaccess(size_t nbEle, double absErrBound, int blockSize,
                                                              unsigned char* cmpBytes) {
  return fm_decompress_alloc(nbEle, absErrBound, blockSize, cmpBytes, resolve_segments(0), 2);
}

void szp_double_decompress_openmp_threadblock_randomaccess_arg(double* newData, size_t nbEle, double absErrBound,
                                                               int blockSize, unsigned char* cmpBytes) {
  fm_decompress_arg(newData, nbEle, absErrBound, blockSize, cmpBytes, resolve_segments(0), 2);
}

// ---------------------------------------------------------- extensions --
void szp_gb300_set_segments(int segments) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_segments = segments > 0 ? segments : 0;
}

int szp_gb300_get_segments(void) { return resolve_segments(0); }

const char* szp_gb300_last_error(void) { return t_err.c_str(); }
int szp_gb300_last_status(void) { return t_status; }
int szp_gb300_last_notices(void) { return t_notices; }

size_t szp_gb300_max_stream_bytes(size_t nbEle, int blockSize, int segments, int fastMode) {
  return max_stream_bytes(nbEle, blockSize, resolve_segments(segments), fastMode == 2 ? 2 : 1);
}

int szp_gb300_compress_dev_async(int fastMode, const float* d_data, size_t nbEle, int errBoundMode,
                                 double absErrBound, double relBoundRatio, int blockSize, int segments,
                                 unsigned char* d_out, size_t out_capacity, unsigned long long* d_outSize,
                                 void* stream) {
  clear_error();
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  if (!d_out) return fail(SZP_GB300_EINVAL, "null output");
  cudaStream_t st = w->begin(stream);
  CompressJob j{d_data, nbEle, errBoundMode == REL ? REL : ABS, (float)absErrBound, relBoundRatio, blockSize,
                resolve_segments(segments), fastMode, d_out, out_capacity, d_outSize};
  rc = compress_launch(*w, j, st);
  w->end(st);
  return rc;
}

int szp_gb300_compress_dev(int fastMode, const float* d_data, size_t nbEle, int errBoundMode, double absErrBound,
                           double relBoundRatio, int blockSize, int segments, unsigned char* d_out,
                           size_t out_capacity, size_t* outSize, void* stream) {
  clear_error();
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  if (!d_out) return fail(SZP_GB300_EINVAL, "null output");
  cudaStream_t st = w->begin(stream);
  CompressJob j{d_data, nbEle, errBoundMode == REL ? REL : ABS, (float)absErrBound, relBoundRatio, blockSize,
                resolve_segments(segments), fastMode, d_out, out_capacity, nullptr};
  rc = compress_launch(*w, j, st);
  if (rc) return rc;
  size_t sz = 0;
  rc = finish_sync(*w, st, &sz);
  w->end(st);
  if (outSize) *outSize = sz;
  return rc;
}

size_t szp_gb300_max_stream_bytes_f64(size_t nbEle, int blockSize, int segments, int fastMode) {
  return max_stream_bytes(nbEle, blockSize, resolve_segments(segments), fastMode == 2 ? 2 : 1, 8);
}

int szp_gb300_compress_dev_f64(int fastMode, const double* d_data, size_t nbEle, int errBoundMode,
                               double absErrBound, double relBoundRatio, int blockSize, int segments,
                               unsigned char* d_out, size_t out_capacity, size_t* outSize, void* stream) {
  clear_error();
  if (outSize) *outSize = 0;
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  if (!d_out) return fail(SZP_GB300_EINVAL, "null output");
  if (nbEle && !d_data) return fail(SZP_GB300_EINVAL, "null input");
  cudaStream_t st = w->begin(stream);
  CompressJob j{nullptr, nbEle, errBoundMode == REL ? REL : ABS, 0.0f, relBoundRatio, blockSize,
                resolve_segments(segments), fastMode, d_out, out_capacity, nullptr};
  j.dbl = true;
  j.d_xd = d_data;
  j.eb_abs_d = absErrBound;
  rc = compress_launch(*w, j, st);
  if (rc == SZP_GB300_OK) {
    size_t sz = 0;
    rc = finish_sync(*w, st, &sz);
    if (outSize) *outSize = sz;
  }
  w->end(st);
  return rc;
}

int szp_gb300_decompress_dev_f64(int fastMode, const unsigned char* d_bytes, size_t byteLength, size_t nbEle,
                                 int blockSize, int segments, double* d_out, void* stream) {
  clear_error();
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  if (!d_bytes) return fail(SZP_GB300_EINVAL, "null stream");
  if (nbEle && !d_out) return fail(SZP_GB300_EINVAL, "null output");
  cudaStream_t st = w->begin(stream);
  DecompressJob j{d_bytes, byteLength, nullptr, nbEle, blockSize, resolve_segments(segments), fastMode, nullptr};
  j.dbl = true;
  j.d_yd = d_out;
  rc = decompress_launch(*w, j, st);
  if (rc == SZP_GB300_OK) rc = finish_sync(*w, st, nullptr);
  w->end(st);
  return rc;
}

int szp_gb300_reduce_sum_dev(int fastMode, int dataType, const unsigned char* d_a, size_t lenA,
                             const unsigned char* d_b, size_t lenB, size_t nbEle, int blockSize, int segments,
                             unsigned char* d_out, size_t out_capacity, size_t* outSize, void* stream) {
  clear_error();
  if (outSize) *outSize = 0;
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  if (!d_a || !d_b || !d_out) return fail(SZP_GB300_EINVAL, "null stream");
  if (dataType != SZ_FLOAT && dataType != SZ_DOUBLE) return fail(SZP_GB300_EINVAL, "unknown dataType %d", dataType);
  const bool dbl = dataType == SZ_DOUBLE;
  const size_t hb = dbl ? 8 : 4;
  if (lenA < hb || lenB < hb) return fail(SZP_GB300_ECORRUPT, "stream shorter than its header");
  const int T = resolve_segments(segments);
  cudaStream_t st = w->begin(stream);
  // both error bounds, from the headers: they must be the same bytes
  uint8_t* h = w->h_small + 16;
  rc = SZP_GB300_OK;
  if (cudaMemcpyAsync(h, d_a, hb, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(h + 8, d_b, hb, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    rc = fail(SZP_GB300_ECUDA, "reading the stream headers failed");
  } else if (memcmp(h, h + 8, hb) != 0) {
    rc = fail(SZP_GB300_EINVAL, "the streams were compressed with different error bounds");
  }
  // the codes, in the workspace: a's, then b's added to them by its decode
  if (rc == SZP_GB300_OK && w->qbuf.ensure((nbEle + 4) * sizeof(int32_t)) != cudaSuccess)
    rc = fail(SZP_GB300_ENOMEM, "no device memory for the codes");
  int32_t* q = rc == SZP_GB300_OK ? w->qbuf.as<int32_t>() : nullptr;
  for (int k = 0; k < 2 && rc == SZP_GB300_OK; k++) {
    DecompressJob d{k ? d_b : d_a, k ? lenB : lenA, nullptr, nbEle, blockSize, T, fastMode, nullptr};
    d.dbl = dbl;
    d.d_codes = q;
    d.accumulate = k == 1;
    rc = decompress_launch(*w, d, st);
    if (rc == SZP_GB300_OK) rc = finish_sync(*w, st, nullptr);  // each decode reports its own errors
  }
  const bool wrapped = t_notices != 0;  // a sum that wrapped (b's decode added the codes)
  if (rc == SZP_GB300_OK) {
    CompressJob c{nullptr, nbEle, ABS, 0.0f, 0.0, blockSize, T, fastMode, d_out, out_capacity, nullptr};
    c.dbl = dbl;
    c.d_codes = q;
    if (dbl) {
      uint64_t u = 0;
      for (int i = 0; i < 8; i++) u = (u << 8) | h[i];
      memcpy(&c.eb_abs_d, &u, 8);
    } else {
      const uint32_t u = ((uint32_t)h[0] << 24) | ((uint32_t)h[1] << 16) | ((uint32_t)h[2] << 8) | h[3];
      memcpy(&c.eb_abs, &u, 4);
    }
    rc = compress_launch(*w, c, st);
    if (rc == SZP_GB300_OK) {
      size_t sz = 0;
      rc = finish_sync(*w, st, &sz);
      if (outSize) *outSize = sz;
      if (wrapped) t_notices = 1;
    }
  }
  w->end(st);
  return rc;
}

// The multidimensional Lorenzo variant (lorenzo.cu): the fastmode1 stream
// (blockSize 32) of the codes r after a 12-byte [nx][ny][nz] header.
static constexpr size_t kLorenzoHead = 12;

static int lorenzo_dims(size_t nx, size_t ny, size_t nz, size_t* n) {
  if (nx > 0xFFFFFFFFull || ny > 0xFFFFFFFFull || nz > 0xFFFFFFFFull)
    return fail(SZP_GB300_EINVAL, "a dimension above 2^32 - 1");
  if ((nx && ny > ~(size_t)0 / nx) || (nx * ny && nz > ~(size_t)0 / (nx * ny)))
    return fail(SZP_GB300_EINVAL, "nx * ny * nz overflows");
  *n = nx * ny * nz;
  return SZP_GB300_OK;
}

size_t szp_gb300_lorenzo_max_stream_bytes(size_t nx, size_t ny, size_t nz, int segments) {
  size_t n = 0;
  if (lorenzo_dims(nx, ny, nz, &n)) return 0;
  const size_t b = max_stream_bytes(n, 32, resolve_segments(segments), 1);
  return b ? kLorenzoHead + b : 0;
}

int szp_gb300_lorenzo_compress_dev(const float* d_data, size_t nx, size_t ny, size_t nz, int errBoundMode,
                                   double absErrBound, double relBoundRatio, int segments, unsigned char* d_out,
                                   size_t out_capacity, size_t* outSize, void* stream) {
  clear_error();
  if (outSize) *outSize = 0;
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  size_t n = 0;
  rc = lorenzo_dims(nx, ny, nz, &n);
  if (rc) return rc;
  if (!d_out) return fail(SZP_GB300_EINVAL, "null output");
  if (n && !d_data) return fail(SZP_GB300_EINVAL, "null input");
  if ((uintptr_t)d_data & 3) return fail(SZP_GB300_EINVAL, "input not aligned to its element size");
  if (errBoundMode != ABS && errBoundMode != REL) return fail(SZP_GB300_EINVAL, "unknown errBoundMode %d", errBoundMode);
  const int T = resolve_segments(segments);
  if (out_capacity < kLorenzoHead + 4 + 8ull * T) return fail(SZP_GB300_ECAPACITY, "output buffer smaller than the stream header");
  cudaStream_t st = w->begin(stream);
  DevMisc* dm = w->dm();
  rc = SZP_GB300_OK;
  if (cudaMemsetAsync(&dm->err, 0, sizeof(uint32_t), st) != cudaSuccess) rc = fail(SZP_GB300_ECUDA, "memset failed");
  if (rc == SZP_GB300_OK && errBoundMode == REL) rc = launch_rel_float(*w, d_data, n, relBoundRatio, st);
  if (rc == SZP_GB300_OK && w->qbuf.ensure((n + 4) * sizeof(int32_t)) != cudaSuccess)
    rc = fail(SZP_GB300_ENOMEM, "no device memory for the codes");
  if (rc == SZP_GB300_OK) {
    LorenzoArgs a;
    memset(&a, 0, sizeof a);
    a.x = d_data;
    a.r = w->qbuf.as<int32_t>();
    a.head = d_out;
    a.nx = (uint32_t)nx;
    a.ny = (uint32_t)ny;
    a.nz = (uint32_t)nz;
    a.eb = (float)absErrBound;
    a.eb_dev = errBoundMode == REL ? &dm->eb : nullptr;
    a.err = &dm->err;
    w->mark(kSlotLorenzo, 0, st);
    cudaError_t e = launch_lorenzo_codes(a, (uint32_t)w->sm_count, st);
    w->mark(kSlotLorenzo, 1, st);
    if (e != cudaSuccess) rc = fail(SZP_GB300_ECUDA, "Lorenzo codes pass: %s", cudaGetErrorString(e));
    count_launches(1);
  }
  if (rc == SZP_GB300_OK) {
    CompressJob c{nullptr, n, ABS, (float)absErrBound, 0.0, 32, T, 1, d_out + kLorenzoHead,
                  out_capacity - kLorenzoHead, nullptr};
    c.d_codes = w->qbuf.as<int32_t>();
    c.d_eb = errBoundMode == REL ? &dm->eb : nullptr;
    c.keep_err = true;
    rc = compress_launch(*w, c, st);
  }
  if (rc == SZP_GB300_OK) {
    size_t sz = 0;
    rc = finish_sync(*w, st, &sz);
    if (rc == SZP_GB300_OK && outSize) *outSize = sz + kLorenzoHead;
  }
  w->end(st);
  return rc;
}

int szp_gb300_lorenzo_decompress_dev(const unsigned char* d_bytes, size_t byteLength, size_t nx, size_t ny, size_t nz,
                                     int segments, float* d_out, void* stream) {
  clear_error();
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  size_t n = 0;
  rc = lorenzo_dims(nx, ny, nz, &n);
  if (rc) return rc;
  if (!d_bytes) return fail(SZP_GB300_EINVAL, "null stream");
  if (n && !d_out) return fail(SZP_GB300_EINVAL, "null output");
  if (byteLength < kLorenzoHead + 4) return fail(SZP_GB300_ECORRUPT, "stream shorter than its header");
  const int T = resolve_segments(segments);
  cudaStream_t st = w->begin(stream);
  // the dims the stream was written with must be the caller's
  uint8_t* h = w->h_small + 16;
  rc = SZP_GB300_OK;
  if (cudaMemcpyAsync(h, d_bytes, kLorenzoHead, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    rc = fail(SZP_GB300_ECUDA, "reading the stream header failed");
  } else {
    uint32_t d[3];
    for (int i = 0; i < 3; i++)
      d[i] = (uint32_t)h[4 * i] | ((uint32_t)h[4 * i + 1] << 8) | ((uint32_t)h[4 * i + 2] << 16) |
             ((uint32_t)h[4 * i + 3] << 24);
    if (d[0] != nx || d[1] != ny || d[2] != nz)
      rc = fail(SZP_GB300_EINVAL, "the stream holds a %ux%ux%u field", d[0], d[1], d[2]);
  }
  if (rc == SZP_GB300_OK) {
    DecompressJob j{d_bytes + kLorenzoHead, byteLength - kLorenzoHead, nullptr, n, 32, T, 1, nullptr};
    j.d_codes = reinterpret_cast<int32_t*>(d_out);
    rc = decompress_launch(*w, j, st);
  }
  if (rc == SZP_GB300_OK) {
    LorenzoArgs a;
    memset(&a, 0, sizeof a);
    a.q = reinterpret_cast<int32_t*>(d_out);
    a.nx = (uint32_t)nx;
    a.ny = (uint32_t)ny;
    a.nz = (uint32_t)nz;
    a.eb_dev = &w->plan.as<DecPlan>()->eb;  // the decoded stream's bound
    a.err = &w->dm()->err;
    w->mark(kSlotLorenzoInv, 0, st);
    cudaError_t e = launch_lorenzo_inverse(a, (uint32_t)w->sm_count, st);
    w->mark(kSlotLorenzoInv, 1, st);
    if (e != cudaSuccess) rc = fail(SZP_GB300_ECUDA, "Lorenzo inverse passes: %s", cudaGetErrorString(e));
    count_launches(2);
  }
  if (rc == SZP_GB300_OK) rc = finish_sync(*w, st, nullptr);
  w->end(st);
  return rc;
}

int szp_gb300_decompress_dev(int fastMode, const unsigned char* d_bytes, size_t byteLength, size_t nbEle,
                             int blockSize, int segments, float* d_out, void* stream) {
  clear_error();
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  if (!d_bytes) return fail(SZP_GB300_EINVAL, "null stream");
  cudaStream_t st = w->begin(stream);
  DecompressJob j{d_bytes, byteLength, nullptr, nbEle, blockSize, resolve_segments(segments), fastMode, d_out};
  rc = decompress_launch(*w, j, st);
  w->end(st);
  return rc;
}

int szp_gb300_decompress_dev_async(int fastMode, const unsigned char* d_bytes, size_t capacity,
                                   const unsigned long long* d_byteLength, size_t nbEle, int blockSize,
                                   int segments, float* d_out, void* stream) {
  clear_error();
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  if (!d_bytes) return fail(SZP_GB300_EINVAL, "null stream");
  cudaStream_t st = w->begin(stream);
  DecompressJob j{d_bytes, capacity, reinterpret_cast<const uint64_t*>(d_byteLength), nbEle, blockSize,
                  resolve_segments(segments), fastMode, d_out};
  rc = decompress_launch(*w, j, st);
  w->end(st);
  return rc;
}

int szp_gb300_sync_status(void* stream) {
  clear_error();
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  return finish_sync(*w, (cudaStream_t)stream, nullptr);
}

void szp_gb300_bitcount_thresholds(uint32_t* thr34) {
  const BitcountTable& t = table();
  for (int k = 0; k < 34; k++) thr34[k] = t.thr[k];
}

int szp_gb300_bitcount_probe(const uint32_t* d_max, uint8_t* d_bc, size_t n, void* stream) {
  clear_error();
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  cudaStream_t st = w->begin(stream);
  CU(launch_bitcount_probe(d_max, d_bc, n, table(), st));
  count_launches(n ? 1 : 0);
  w->end(st);
  return SZP_GB300_OK;
}

int szp_gb300_wait_probe(unsigned long long limit_ns, unsigned long long* waited_ns) {
  clear_error();
  Workspace* w;
  int rc = get_ws(&w);
  if (rc) return rc;
  cudaStream_t st = w->begin_own();
  DevMisc* dm = w->dm();
  CU(cudaMemsetAsync(&dm->err, 0, sizeof(uint32_t), st));
  CU(launch_wait_probe(limit_ns, &dm->err, reinterpret_cast<unsigned long long*>(&dm->out_size), st));
  count_launches(1);
  size_t waited = 0;
  rc = finish_sync(*w, st, &waited);
  w->end(st);
  if (waited_ns) *waited_ns = waited;
  return rc;
}

void szp_gb300_set_timing(int enable) { g_timing = enable ? 1 : 0; }

void szp_gb300_set_locate_overlap(int bytes) { g_overlap = bytes; }
void szp_gb300_set_decode_tickets(int on) { g_decode_tickets = on ? 1 : 0; }

double szp_gb300_kernel_ms(int slot) {
  Workspace* w;
  if (get_ws(&w) || slot < 0 || slot >= kNumSlots || w->ev_last[slot] < 0) return -1.0;
  int h = w->ev_last[slot];
  float ms = -1.0f;
  if (cudaEventSynchronize(w->ev[slot][h][1]) != cudaSuccess) return -1.0;
  if (cudaEventElapsedTime(&ms, w->ev[slot][h][0], w->ev[slot][h][1]) != cudaSuccess) return -1.0;
  return ms;
}

double szp_gb300_kernel_time(int slot, int* launches) {
  if (launches) *launches = 0;
  Workspace* w;
  if (get_ws(&w) || slot < 0 || slot >= kNumSlots) return -1.0;
  int n = w->ev_pending[slot];
  double total = 0.0;
  for (int i = 0; i < n; i++) {
    int h = ((w->ev_head[slot] - n + i) % Workspace::kRing + Workspace::kRing) % Workspace::kRing;
    float ms = 0.0f;
    if (cudaEventSynchronize(w->ev[slot][h][1]) != cudaSuccess) return -1.0;
    if (cudaEventElapsedTime(&ms, w->ev[slot][h][0], w->ev[slot][h][1]) != cudaSuccess) return -1.0;
    total += ms;
  }
  w->ev_pending[slot] = 0;
  if (launches) *launches = n;
  return total;
}

int szp_gb300_last_repairs(void) {
  Workspace* w;
  if (get_ws(&w)) return -1;
  uint32_t v = 0;
  if (cudaMemcpy(&v, &w->dm()->verify[0], 4, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return (int)v;
}

unsigned long long szp_gb300_kernel_launches(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_launches;
}

}  // extern "C"
