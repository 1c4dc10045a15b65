// serve.cu -- a request server over the batched kernels.
//
// Clients submit compress and decompress requests on device-resident data as
// they arrive.  A worker thread runs continuous batching: it admits queued
// requests in arrival order while their results fit the HBM budget (one device
// arena carved by a host-side allocator), launches each admitted group as one
// compress batch and one decompress batch on a free lane (stream), and keeps
// admitting while earlier lanes run, so the work of successive groups overlaps
// on the device.  A finished request keeps its result in the arena until the
// client releases it; a compressed result is shrunk to its stream size first.
// Every result is byte-identical to the single-field calls on the same input.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "szp_batch.h"
#include "szp_gb300.h"
#include "szp_kernels.h"

using namespace szp;

namespace {

#define SCU(call)                                                                             \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return host_fail(SZP_GB300_ECUDA, cudaGetErrorString(e_));          \
  } while (0)

constexpr size_t kArenaAlign = 256;

// First-fit allocator over [0, size) with coalescing free ranges.
class Arena {
 public:
  void init(size_t size) {
    free_.clear();
    if (size) free_[0] = size;
    used_ = peak_ = 0;
  }
  bool alloc(size_t bytes, size_t* off) {
    bytes = round(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes, at = it->first + bytes;
        free_.erase(it);
        if (rest) free_[at] = rest;
        used_ += bytes;
        peak_ = std::max(peak_, used_);
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = round(bytes);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  // Gives back the tail of a block beyond `keep` bytes.
  size_t shrink(size_t off, size_t bytes, size_t keep) {
    bytes = round(bytes);
    keep = round(keep);
    if (keep < bytes) release(off + keep, bytes - keep);
    return keep;
  }
  size_t used() const { return used_; }
  size_t peak() const { return peak_; }

 private:
  static size_t round(size_t b) { return ((b ? b : 1) + kArenaAlign - 1) & ~(kArenaAlign - 1); }
  std::map<size_t, size_t> free_;
  size_t used_ = 0, peak_ = 0;
};

struct Req {
  szp_gb300_request r;
  unsigned long long id = 0;
  double admitted = 0, done = 0;
  int status = SZP_GB300_OK;
  size_t off = 0, alloc = 0;  // arena block of the result
  size_t result_bytes = 0;
  bool finished = false;
};

// A buffer that grows on demand (only ever in the worker thread).  Device
// buffers grow in stream order on their lane (no device-wide synchronisation);
// they start large enough for typical groups.
struct Grow {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t n, bool pinned = false, cudaStream_t st = nullptr) {
    if (n <= cap) return cudaSuccess;
    size_t want = std::max(n + n / 2, (size_t)4096);
    if (p) {
      if (pinned) cudaFreeHost(p); else cudaFreeAsync(p, st);
    }
    p = nullptr;
    cap = 0;
    cudaError_t e = pinned ? cudaMallocHost(&p, want) : cudaMallocAsync(&p, want, st);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void free_it(bool pinned) {
    if (p) {
      if (pinned) cudaFreeHost(p); else cudaFree(p);
    }
    p = nullptr;
    cap = 0;
  }
};

// Launch state, launch error word and locate counters of a lane.
struct LaneScalars {
  LaunchState ls;
  uint32_t err;
  uint32_t counters[4];
};

// One stream with its own look-back words and tables: a batch in flight.
struct Lane {
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  bool busy = false;
  std::vector<Req*> reqs;           // the group in flight
  std::vector<int> cidx, didx;      // their positions in the compress / decompress batch
  LaneScalars* misc = nullptr;      // device
  Grow status, tables, htables, hresults, plans, blkpos, aux, sizes, errs;
};

}  // namespace

struct szp_gb300_server_s {
  szp_gb300_server_config cfg{};
  int T = 1;
  int device = 0;
  int sms = 0;
  uint8_t* arena_base = nullptr;
  Arena arena;
  std::vector<Lane> lanes;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Req*> queue;
  std::unordered_map<unsigned long long, Req*> reqs;
  std::deque<unsigned long long> completions;
  unsigned long long next_id = 1;
  int in_flight = 0;
  bool stop = false;
  int worker_status = SZP_GB300_OK;
  std::thread worker;
  std::chrono::steady_clock::time_point t0;
  // statistics
  unsigned long long batches = 0, served = 0, bytes = 0;
  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

int pick_rounds(const szp_gb300_server_s& s, const std::vector<Req*>& g) {
  if (s.cfg.tile_rounds == 1 || s.cfg.tile_rounds == 2 || s.cfg.tile_rounds == 4) return s.cfg.tile_rounds;
  // small requests leave large tiles mostly empty (every field has T segments)
  double el = 0;
  for (Req* r : g) el += (double)r->r.nbEle;
  const double per_seg = g.empty() ? 0.0 : el / g.size() / s.T;
  return per_seg < 4096 ? 1 : per_seg < 16384 ? 2 : 4;
}

// Packs host vectors into one staging area; returns each one's byte offset.
struct Packer {
  std::vector<uint8_t> buf;
  template <class T>
  size_t add(const std::vector<T>& v) {
    const size_t at = (buf.size() + 15) & ~(size_t)15;
    buf.resize(at + v.size() * sizeof(T) + 16);
    if (!v.empty()) memcpy(buf.data() + at, v.data(), v.size() * sizeof(T));
    return at;
  }
};

// Launches one group on a lane.
int launch_group(szp_gb300_server_s& s, Lane& ln) {
  const int L = (int)kBatchL, T = s.T;
  std::vector<szp_gb300_field> cf, df;
  ln.cidx.assign(ln.reqs.size(), -1);
  ln.didx.assign(ln.reqs.size(), -1);
  for (size_t i = 0; i < ln.reqs.size(); i++) {
    Req* q = ln.reqs[i];
    szp_gb300_field f;
    memset(&f, 0, sizeof f);
    f.input = q->r.input;
    f.input_bytes = q->r.input_bytes;
    f.output = s.arena_base + q->off;
    f.output_bytes = q->alloc;
    f.nbEle = q->r.nbEle;
    f.errBoundMode = q->r.errBoundMode;
    f.absErrBound = q->r.absErrBound;
    f.relBoundRatio = q->r.relBoundRatio;
    if (q->r.op == SZP_GB300_BATCH_COMPRESS) {
      ln.cidx[i] = (int)cf.size();
      cf.push_back(f);
    } else {
      ln.didx[i] = (int)df.size();
      df.push_back(f);
    }
  }
  const int rounds = pick_rounds(s, ln.reqs);
  const uint32_t tb = batch_tile_blocks(rounds);
  CompressPlan cp;
  DecompressPlan dp;
  int rc = plan_compress(cf.data(), (int)cf.size(), L, T, tb, cp);
  if (!rc) rc = plan_decompress(df.data(), (int)df.size(), L, T, tb, dp);
  if (rc) return rc;
  const size_t nc = cf.size(), nd = df.size();
  // per-lane device buffers for this group
  SCU(ln.sizes.ensure(8 * (nc + 1), false, ln.st));
  SCU(ln.errs.ensure(4 * (nc + nd + 2), false, ln.st));
  SCU(ln.plans.ensure(dp.plan_stride * (nd + 1), false, ln.st));
  SCU(ln.blkpos.ensure(4 * (dp.blocks + 1), false, ln.st));
  SCU(ln.aux.ensure(sizeof(uint2) * (dp.locs + 1), false, ln.st));
  const size_t words = std::max<uint64_t>(std::max(cp.tiles, dp.tiles), std::max<uint64_t>(dp.locs, 1));
  if (words * 8 > ln.status.cap) {
    SCU(ln.status.ensure(words * 8, false, ln.st));
    SCU(cudaMemsetAsync(ln.status.p, 0, ln.status.cap, ln.st));  // fresh words must not look ready
  }
  unsigned long long* d_sizes = static_cast<unsigned long long*>(ln.sizes.p);
  uint32_t* d_cerr = static_cast<uint32_t*>(ln.errs.p);
  uint32_t* d_derr = d_cerr + nc;
  place_compress(cp, d_sizes, d_cerr);
  place_decompress(dp, static_cast<uint8_t*>(ln.plans.p), static_cast<uint32_t*>(ln.blkpos.p), d_derr);
  Packer pk;
  const size_t o_cf = pk.add(cp.fields), o_ctf = pk.add(cp.tile_field), o_it = pk.add(cp.item_field);
  const size_t o_rs = pk.add(cp.rel), o_df = pk.add(dp.fields), o_dtf = pk.add(dp.tile_field);
  const size_t o_lf = pk.add(dp.loc_field);
  SCU(ln.tables.ensure(pk.buf.size(), false, ln.st));
  SCU(ln.htables.ensure(pk.buf.size(), true));
  memcpy(ln.htables.p, pk.buf.data(), pk.buf.size());  // the lane's previous group has finished with it
  uint8_t* tb_d = static_cast<uint8_t*>(ln.tables.p);
  SCU(cudaMemcpyAsync(tb_d, ln.htables.p, pk.buf.size(), cudaMemcpyHostToDevice, ln.st));
  SCU(cudaMemsetAsync(d_cerr, 0, 4 * (nc + nd), ln.st));
  SCU(cudaMemsetAsync(&ln.misc->err, 0, sizeof(uint32_t) * 5, ln.st));
  const int sms = s.sms;
  if (nc) {
    CompressArgs a;
    RelBatchArgs r;
    args_compress(a, r, cp, reinterpret_cast<CompressField*>(tb_d + o_cf), reinterpret_cast<uint32_t*>(tb_d + o_ctf),
                  reinterpret_cast<uint32_t*>(tb_d + o_it), reinterpret_cast<RelFieldState*>(tb_d + o_rs),
                  static_cast<uint64_t*>(ln.status.p), &ln.misc->ls, &ln.misc->err, tb);
    rc = issue_compress(a, r, (uint32_t)std::min<uint64_t>(r.nitems, (uint64_t)sms * 8), rounds, ln.st);
    if (rc) return rc;
  }
  if (nd) {
    DecArgs a;
    args_decompress(a, dp, reinterpret_cast<DecField*>(tb_d + o_df), reinterpret_cast<uint32_t*>(tb_d + o_dtf),
                    reinterpret_cast<uint32_t*>(tb_d + o_lf), static_cast<uint2*>(ln.aux.p), ln.misc->counters,
                    static_cast<uint64_t*>(ln.status.p), &ln.misc->ls, &ln.misc->err, tb);
    rc = issue_decompress(a, (uint32_t)nd, rounds, ln.st);
    if (rc) return rc;
  }
  // results: compressed sizes, per-field errors, the lane's error word
  SCU(ln.hresults.ensure(8 * (nc + 1) + 4 * (nc + nd + 2), true));
  uint8_t* hr = static_cast<uint8_t*>(ln.hresults.p);
  if (nc) SCU(cudaMemcpyAsync(hr, d_sizes, 8 * nc, cudaMemcpyDeviceToHost, ln.st));
  SCU(cudaMemcpyAsync(hr + 8 * (nc + 1), d_cerr, 4 * (nc + nd), cudaMemcpyDeviceToHost, ln.st));
  SCU(cudaMemcpyAsync(hr + 8 * (nc + 1) + 4 * (nc + nd), &ln.misc->err, 4, cudaMemcpyDeviceToHost, ln.st));
  SCU(cudaEventRecord(ln.ev, ln.st));
  host_count_launches((nc ? (cp.item_field.empty() ? 1 : 2) : 0) + (nd ? 3 : 0));
  return SZP_GB300_OK;
}

// Marks a lane's group done (under the server lock).
void complete_group(szp_gb300_server_s& s, Lane& ln) {
  const size_t nc = std::count_if(ln.cidx.begin(), ln.cidx.end(), [](int v) { return v >= 0; });
  const size_t nd = ln.reqs.size() - nc;
  const uint8_t* hr = static_cast<const uint8_t*>(ln.hresults.p);
  const unsigned long long* sizes = reinterpret_cast<const unsigned long long*>(hr);
  const uint32_t* errs = reinterpret_cast<const uint32_t*>(hr + 8 * (nc + 1));
  const uint32_t lerr = errs[nc + nd];
  const double t = s.now();
  for (size_t i = 0; i < ln.reqs.size(); i++) {
    Req* q = ln.reqs[i];
    const bool comp = ln.cidx[i] >= 0;
    const uint32_t e = (comp ? errs[ln.cidx[i]] : errs[nc + ln.didx[i]]) | lerr;
    q->status = host_status_from_err(e);
    if (comp) {
      q->result_bytes = q->status == SZP_GB300_OK ? sizes[ln.cidx[i]] : 0;
      q->alloc = s.arena.shrink(q->off, q->alloc, q->result_bytes);
    } else {
      q->result_bytes = 4 * q->r.nbEle;
    }
    q->done = t;
    q->finished = true;
    s.served++;
    s.bytes += 4 * q->r.nbEle;
    s.completions.push_back(q->id);
  }
  host_clear_error();
  ln.reqs.clear();
  ln.busy = false;
  s.in_flight--;
}

void worker_main(szp_gb300_server_s* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    // retire finished lanes
    for (Lane& ln : s->lanes)
      if (ln.busy && cudaEventQuery(ln.ev) == cudaSuccess) complete_group(*s, ln);
    s->cv_done.notify_all();
    if (s->stop && s->queue.empty() && s->in_flight == 0) break;
    Lane* free_lane = nullptr;
    for (Lane& ln : s->lanes)
      if (!ln.busy) {
        free_lane = &ln;
        break;
      }
    // admit in arrival order while the results fit
    std::vector<Req*> group;
    if (free_lane) {
      while (!s->queue.empty() && (int)group.size() < s->cfg.max_batch) {
        Req* q = s->queue.front();
        const size_t need = q->r.op == SZP_GB300_BATCH_COMPRESS ? host_max_stream_bytes(q->r.nbEle, kBatchL, s->T)
                                                               : 4 * std::max<size_t>(q->r.nbEle, 1);
        size_t off;
        if (!s->arena.alloc(need, &off)) break;
        q->off = off;
        q->alloc = need;
        q->admitted = s->now();
        group.push_back(q);
        s->queue.pop_front();
      }
    }
    if (!group.empty()) {
      free_lane->reqs = group;
      free_lane->busy = true;
      s->in_flight++;
      lk.unlock();
      int rc = launch_group(*s, *free_lane);
      lk.lock();
      if (rc) {
        s->worker_status = rc;
        for (Req* q : group) {
          q->status = rc;
          q->done = s->now();
          q->finished = true;
          s->completions.push_back(q->id);
        }
        free_lane->reqs.clear();
        free_lane->busy = false;
        s->in_flight--;
        s->cv_done.notify_all();
      }
      continue;
    }
    if (s->in_flight > 0) {
      // lanes are running: poll them without blocking new arrivals for long
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(20));
      lk.lock();
    } else {
      s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
    }
  }
}

}  // namespace

extern "C" {

int szp_gb300_server_create(szp_gb300_server* out, const szp_gb300_server_config* cfg) {
  host_clear_error();
  if (!out || !cfg) return host_fail(SZP_GB300_EINVAL, "null argument");
  *out = nullptr;
  if (cfg->hbm_budget < (1u << 20)) return host_fail(SZP_GB300_EINVAL, "HBM budget below 1 MiB");
  if (cfg->max_batch < 1 || cfg->lanes < 1 || cfg->lanes > 16)
    return host_fail(SZP_GB300_EINVAL, "max_batch >= 1 and 1 <= lanes <= 16");
  szp_gb300_server_s* s = new szp_gb300_server_s();
  s->cfg = *cfg;
  s->T = host_resolve_segments(cfg->segments);
  s->t0 = std::chrono::steady_clock::now();
  auto bad = [&](cudaError_t e) {
    delete s;
    return host_fail(SZP_GB300_ENOMEM, cudaGetErrorString(e));
  };
  cudaError_t e = cudaGetDevice(&s->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->arena_base, cfg->hbm_budget);
  if (e != cudaSuccess) return bad(e);
  s->arena.init(cfg->hbm_budget);
  s->lanes.resize(cfg->lanes);
  for (Lane& ln : s->lanes) {
    e = cudaStreamCreateWithFlags(&ln.st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ln.ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc((void**)&ln.misc, sizeof(LaneScalars));
    if (e == cudaSuccess) e = cudaMemset(ln.misc, 0, sizeof(LaneScalars));
    // room for groups of typical size, so steady state allocates nothing
    const size_t mb = (size_t)cfg->max_batch + 1;
    if (e == cudaSuccess) e = ln.status.ensure(8u << 16, false, ln.st);
    if (e == cudaSuccess) e = cudaMemsetAsync(ln.status.p, 0, ln.status.cap, ln.st);
    if (e == cudaSuccess) e = ln.tables.ensure(1u << 20, false, ln.st);
    if (e == cudaSuccess) e = ln.htables.ensure(1u << 20, true);
    if (e == cudaSuccess) e = ln.hresults.ensure(12 * mb + 64, true);
    if (e == cudaSuccess) e = ln.sizes.ensure(8 * mb, false, ln.st);
    if (e == cudaSuccess) e = ln.errs.ensure(8 * mb, false, ln.st);
    if (e == cudaSuccess) e = ln.plans.ensure(512 * mb, false, ln.st);
    if (e == cudaSuccess) e = ln.blkpos.ensure(16u << 20, false, ln.st);
    if (e == cudaSuccess) e = ln.aux.ensure(1u << 20, false, ln.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ln.st);
    if (e != cudaSuccess) return bad(e);
  }
  e = prepare_compress_batch();
  if (e == cudaSuccess) e = prepare_decompress_batch();
  if (e != cudaSuccess) return bad(e);
  s->worker = std::thread(worker_main, s);
  *out = s;
  return SZP_GB300_OK;
}

double szp_gb300_server_clock(szp_gb300_server s) { return s ? s->now() : 0.0; }

int szp_gb300_server_submit(szp_gb300_server s, const szp_gb300_request* reqs, int n, unsigned long long* ids) {
  host_clear_error();
  if (!s || n < 0 || (n && !reqs)) return host_fail(SZP_GB300_EINVAL, "bad submission");
  for (int i = 0; i < n; i++) {
    const szp_gb300_request& r = reqs[i];
    if (r.op != SZP_GB300_BATCH_COMPRESS && r.op != SZP_GB300_BATCH_DECOMPRESS)
      return host_fail(SZP_GB300_EINVAL, "request op must be SZP_GB300_BATCH_COMPRESS or _DECOMPRESS");
    if (r.nbEle && !r.input) return host_fail(SZP_GB300_EINVAL, "null request input");
    const size_t need = r.op == SZP_GB300_BATCH_COMPRESS ? host_max_stream_bytes(r.nbEle, kBatchL, s->T)
                                                          : 4 * std::max<size_t>(r.nbEle, 1);
    if (need + kArenaAlign > s->cfg.hbm_budget) return host_fail(SZP_GB300_ENOMEM, "request larger than the budget");
  }
  const double t = s->now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return host_fail(SZP_GB300_EINVAL, "server is stopping");
    for (int i = 0; i < n; i++) {
      Req* q = new Req();
      q->r = reqs[i];
      if (q->r.arrival < 0) q->r.arrival = t;
      q->id = s->next_id++;
      s->reqs[q->id] = q;
      s->queue.push_back(q);
      if (ids) ids[i] = q->id;
    }
  }
  s->cv_work.notify_one();
  return SZP_GB300_OK;
}

static void fill_result(const Req* q, szp_gb300_server_s* s, szp_gb300_result* res) {
  res->id = q->id;
  res->status = q->status;
  res->output = s->arena_base + q->off;
  res->output_bytes = q->result_bytes;
  res->arrival = q->r.arrival;
  res->admitted = q->admitted;
  res->done = q->done;
}

int szp_gb300_server_completed(szp_gb300_server s, szp_gb300_result* res, int max) {
  if (!s || !res || max < 0) return host_fail(SZP_GB300_EINVAL, "bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  int k = 0;
  while (k < max && !s->completions.empty()) {
    auto it = s->reqs.find(s->completions.front());
    s->completions.pop_front();
    if (it == s->reqs.end()) continue;
    fill_result(it->second, s, &res[k++]);
  }
  return k;
}

int szp_gb300_server_wait(szp_gb300_server s, unsigned long long id, szp_gb300_result* res) {
  host_clear_error();
  if (!s) return host_fail(SZP_GB300_EINVAL, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return host_fail(SZP_GB300_EINVAL, "unknown request");
  Req* q = it->second;
  s->cv_done.wait(lk, [&] { return q->finished; });
  if (res) fill_result(q, s, res);
  return q->status;
}

int szp_gb300_server_release(szp_gb300_server s, unsigned long long id) {
  host_clear_error();
  if (!s) return host_fail(SZP_GB300_EINVAL, "null server");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || !it->second->finished) return host_fail(SZP_GB300_EINVAL, "request not finished");
    Req* q = it->second;
    if (q->alloc) s->arena.release(q->off, q->alloc);
    s->reqs.erase(it);
    delete q;
  }
  s->cv_work.notify_one();  // memory came free: queued requests may fit now
  return SZP_GB300_OK;
}

int szp_gb300_server_drain(szp_gb300_server s) {
  if (!s) return host_fail(SZP_GB300_EINVAL, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [&] { return s->queue.empty() && s->in_flight == 0; });
  return s->worker_status;
}

int szp_gb300_server_get_stats(szp_gb300_server s, szp_gb300_server_stats* st) {
  if (!s || !st) return host_fail(SZP_GB300_EINVAL, "bad argument");
  std::lock_guard<std::mutex> lk(s->mu);
  st->requests = s->served;
  st->bytes = s->bytes;
  st->queued = s->queue.size();
  st->in_flight = (unsigned long long)s->in_flight;
  st->memory_used = s->arena.used();
  st->memory_peak = s->arena.peak();
  return SZP_GB300_OK;
}

void szp_gb300_server_destroy(szp_gb300_server s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (Lane& ln : s->lanes) {
    if (ln.st) cudaStreamSynchronize(ln.st);
    for (Grow* g : {&ln.status, &ln.tables, &ln.plans, &ln.blkpos, &ln.aux, &ln.sizes, &ln.errs})
      g->free_it(false);
    ln.htables.free_it(true);
    ln.hresults.free_it(true);
    if (ln.misc) cudaFree(ln.misc);
    if (ln.ev) cudaEventDestroy(ln.ev);
    if (ln.st) cudaStreamDestroy(ln.st);
  }
  for (auto& kv : s->reqs) delete kv.second;
  if (s->arena_base) cudaFree(s->arena_base);
  delete s;
}

}  // extern "C"
