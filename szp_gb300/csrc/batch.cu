// batch.cu -- batched fastmode1 compression and decompression.
//
// Many fields of uneven sizes and bounds go through one persistent launch per
// stage instead of one launch sequence per field: the tiles (and, when
// decompressing, the locate chunks) of all fields share one ticket space, a
// small device table maps each ticket to its field, and each field keeps its
// own look-back range, stream, sizes and error word.  A batch object owns
// those tables and replays its stage sequence as one CUDA graph.  Each field's
// stream is byte-identical to a single-field call with the same arguments.
//
// Stages per run:
//   compress    clear errors | range pass (REL fields) | compress tiles
//   decompress  clear errors | header setup (one CTA per field) | locate | decode
//
// The tile size (8*rounds*8 blocks of 32, rounds 1/2/4) is chosen per batch by
// timing each candidate on the batch itself (SZP_GB300_BATCH_AUTOTUNE).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "szp_batch.h"
#include "szp_gb300.h"
#include "szp_kernels.h"

using namespace szp;

namespace {

#define BCU(call)                                                                             \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return host_fail(SZP_GB300_ECUDA, cudaGetErrorString(e_));          \
  } while (0)

// x86 result of 0 * rel (the bound of an empty REL field, szp.cc:36-51).
float empty_rel_bound(float rel) {
  if (std::isnan(rel)) {
    uint32_t u;
    memcpy(&u, &rel, 4);
    u |= 0x00400000u;
    memcpy(&rel, &u, 4);
    return rel;
  }
  if (std::isinf(rel)) {
    uint32_t u = 0xFFC00000u;  // invalid operation: the x86 default NaN
    float r;
    memcpy(&r, &u, 4);
    return r;
  }
  return 0.0f * rel;
}

// Device allocations of a batch, freed together.
struct Allocs {
  std::vector<void*> ptrs;
  ~Allocs() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t get(T** out, size_t count) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T) + 16);
    if (e == cudaSuccess) ptrs.push_back(p);
    *out = static_cast<T*>(p);
    return e;
  }
};

template <class T>
cudaError_t upload(Allocs& al, T** out, const std::vector<T>& v) {
  cudaError_t e = al.get(out, v.size() ? v.size() : 1);
  if (e == cudaSuccess && !v.empty()) e = cudaMemcpy(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

// Launch state, launch-level error word and locate counters of a batch.
struct DevScalars {
  LaunchState ls;
  uint32_t err;
  uint32_t counters[4];
};

// One tile-size choice of a batch: its launch arguments and tables.
struct Config {
  int rounds = 4;
  Allocs al;
  // compression
  CompressArgs ca{};
  RelBatchArgs ra{};
  uint32_t rel_grid = 0;
  // decompression
  DecArgs da{};
  uint32_t nfields = 0;
};

}  // namespace

struct szp_gb300_batch_s {
  int dir = 0;
  int device = 0;
  int nfields = 0, L = 32, T = 1;
  bool graph = true;
  std::vector<szp_gb300_field> fields;
  Allocs al;                       // per-batch buffers shared by the configs
  unsigned long long* d_sizes = nullptr;
  uint32_t* d_err = nullptr;       // per field
  DevScalars* d_misc = nullptr;    // launch state, launch error, locate counters
  uint64_t* d_status = nullptr;
  size_t status_words = 0;
  Config* cfg = nullptr;           // in use
  cudaGraphExec_t exec = nullptr;
  cudaStream_t own = nullptr;      // capture and tuning stream
  cudaEvent_t done = nullptr;
  unsigned long long* h_sizes = nullptr;  // pinned
  uint32_t* h_err = nullptr;              // pinned, nfields + 1
  std::vector<Config*> tuned;
  ~szp_gb300_batch_s() {
    if (exec) cudaGraphExecDestroy(exec);
    for (Config* c : tuned) delete c;
    if (own) cudaStreamDestroy(own);
    if (done) cudaEventDestroy(done);
    if (h_sizes) cudaFreeHost(h_sizes);
    if (h_err) cudaFreeHost(h_err);
  }
};

namespace {

int build_compress(szp_gb300_batch_s& b, Config& c) {
  const uint32_t tb = batch_tile_blocks(c.rounds);
  CompressPlan p;
  int rc = plan_compress(b.fields.data(), b.nfields, b.L, b.T, tb, p);
  if (rc) return rc;
  place_compress(p, b.d_sizes, b.d_err);
  if (p.tiles > b.status_words) return host_fail(SZP_GB300_EINVAL, "look-back words too few for the batch");
  CompressField* d_fields;
  uint32_t *d_tile_field, *d_items;
  RelFieldState* d_state;
  BCU(upload(c.al, &d_fields, p.fields));
  BCU(upload(c.al, &d_tile_field, p.tile_field));
  BCU(upload(c.al, &d_items, p.item_field));
  BCU(upload(c.al, &d_state, p.rel));
  args_compress(c.ca, c.ra, p, d_fields, d_tile_field, d_items, d_state, b.d_status, &b.d_misc->ls,
                &b.d_misc->err, tb);
  int sms = 0;
  BCU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b.device));
  c.rel_grid = (uint32_t)std::min<uint64_t>(c.ra.nitems, (uint64_t)sms * 8);
  return SZP_GB300_OK;
}

int build_decompress(szp_gb300_batch_s& b, Config& c) {
  const uint32_t tb = batch_tile_blocks(c.rounds);
  DecompressPlan p;
  int rc = plan_decompress(b.fields.data(), b.nfields, b.L, b.T, tb, p);
  if (rc) return rc;
  if (p.tiles > b.status_words || p.locs > b.status_words)
    return host_fail(SZP_GB300_EINVAL, "look-back words too few for the batch");
  uint8_t* d_plans;
  uint32_t* d_blkpos;
  uint2* d_aux;
  BCU(c.al.get(&d_plans, p.plan_stride * (size_t)b.nfields + 16));
  BCU(c.al.get(&d_blkpos, p.blocks + 1));
  BCU(c.al.get(&d_aux, p.locs + 1));
  place_decompress(p, d_plans, d_blkpos, b.d_err);
  DecField* d_fields;
  uint32_t *d_tile_field, *d_loc_field;
  BCU(upload(c.al, &d_fields, p.fields));
  BCU(upload(c.al, &d_tile_field, p.tile_field));
  BCU(upload(c.al, &d_loc_field, p.loc_field));
  args_decompress(c.da, p, d_fields, d_tile_field, d_loc_field, d_aux, b.d_misc->counters, b.d_status,
                  &b.d_misc->ls, &b.d_misc->err, tb);
  c.nfields = (uint32_t)b.nfields;
  return SZP_GB300_OK;
}

// The stage sequence of one run on stream st.
int issue(szp_gb300_batch_s& b, const Config& c, cudaStream_t st) {
  BCU(cudaMemsetAsync(b.d_err, 0, sizeof(uint32_t) * (size_t)b.nfields, st));
  BCU(cudaMemsetAsync(&b.d_misc->err, 0, sizeof(uint32_t) * 5, st));  // launch error + counters
  if (b.dir == SZP_GB300_BATCH_COMPRESS) return issue_compress(c.ca, c.ra, c.rel_grid, c.rounds, st);
  return issue_decompress(c.da, c.nfields, c.rounds, st);
}

int make_config(szp_gb300_batch_s& b, int rounds, Config** out) {
  Config* c = new Config();
  c->rounds = rounds;
  int rc = b.dir == SZP_GB300_BATCH_COMPRESS ? build_compress(b, *c) : build_decompress(b, *c);
  if (rc) {
    delete c;
    return rc;
  }
  *out = c;
  return SZP_GB300_OK;
}

// Runs config c once un-captured (first launches set kernel attributes) and
// returns its time on the batch's own stream.
int time_config(szp_gb300_batch_s& b, const Config& c, float* ms) {
  cudaEvent_t e0, e1;
  BCU(cudaEventCreate(&e0));
  BCU(cudaEventCreate(&e1));
  int rc = issue(b, c, b.own);  // warm-up
  if (!rc) {
    cudaEventRecord(e0, b.own);
    rc = issue(b, c, b.own);
    cudaEventRecord(e1, b.own);
  }
  cudaError_t e = cudaStreamSynchronize(b.own);
  if (!rc && e == cudaSuccess) cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  BCU(e);
  return SZP_GB300_OK;
}

// Captures the stage sequence of the chosen config as a CUDA graph.  If the
// capture fails the batch launches its stages directly instead.
void capture(szp_gb300_batch_s& b) {
  if (b.exec) {
    cudaGraphExecDestroy(b.exec);
    b.exec = nullptr;
  }
  if (!b.graph) return;
  cudaGraph_t g = nullptr;
  bool ok = cudaStreamBeginCapture(b.own, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  if (ok) {
    const int rc = issue(b, *b.cfg, b.own);
    ok = cudaStreamEndCapture(b.own, &g) == cudaSuccess && rc == SZP_GB300_OK;
  }
  if (ok) ok = cudaGraphInstantiate(&b.exec, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    b.exec = nullptr;
    b.graph = false;
    cudaGetLastError();
  }
}

}  // namespace

namespace szp {

int plan_compress(const szp_gb300_field* fl, int nf, int L, int T, uint32_t tb, CompressPlan& p) {
  p.fields.assign(nf, CompressField{});
  p.rel.assign(nf, RelFieldState{});
  p.tile_field.clear();
  p.item_field.clear();
  p.tiles = 0;
  for (int f = 0; f < nf; f++) {
    const szp_gb300_field& in = fl[f];
    CompressField& cf = p.fields[f];
    memset(&cf, 0, sizeof cf);
    cf.x = static_cast<const float*>(in.input);
    cf.out = static_cast<uint8_t*>(in.output);
    cf.cap = in.output_bytes;
    cf.seg.n = in.nbEle;
    cf.seg.T = (uint32_t)T;
    cf.seg.L = (uint32_t)L;
    cf.seg.tsz = in.nbEle / (uint64_t)T;
    host_segment_blocks(in.nbEle, T, L, cf.nb_reg, cf.nb_last);
    uint64_t per_seg = 0, nt = 0;
    host_tile_counts(in.nbEle, T, L, tb, per_seg, nt);
    cf.tiles_per_seg = (uint32_t)per_seg;
    cf.ntiles = (uint32_t)nt;
    cf.tile_base = (uint32_t)p.tiles;
    cf.out_size = reinterpret_cast<uint64_t*>((uintptr_t)f);
    cf.err = reinterpret_cast<uint32_t*>((uintptr_t)f);
    RelFieldState& st = p.rel[f];
    memset(&st, 0, sizeof st);
    st.mn = rel_encode_host(INFINITY);
    st.mx = rel_encode_host(-INFINITY);
    if (in.errBoundMode == REL) {
      cf.rel = (float)in.relBoundRatio;
      if (in.nbEle == 0) {
        cf.eb = empty_rel_bound(cf.rel);
      } else {
        st.first_item = (uint32_t)p.item_field.size();
        st.nitems = (uint32_t)((in.nbEle + kRelChunk - 1) / kRelChunk);
        for (uint32_t i = 0; i < st.nitems; i++) p.item_field.push_back((uint32_t)f);
      }
    } else {
      cf.eb = (float)in.absErrBound;
    }
    p.tile_field.insert(p.tile_field.end(), nt, (uint32_t)f);
    p.tiles += nt;
    if (p.tiles >= (1ull << 31)) return host_fail(SZP_GB300_EINVAL, "batch too large for one launch");
  }
  return SZP_GB300_OK;
}

void place_compress(CompressPlan& p, unsigned long long* d_sizes, uint32_t* d_err) {
  for (auto& cf : p.fields) {
    const uintptr_t f = reinterpret_cast<uintptr_t>(cf.err);
    cf.out_size = reinterpret_cast<uint64_t*>(d_sizes + f);
    cf.err = d_err + f;
  }
}

int plan_decompress(const szp_gb300_field* fl, int nf, int L, int T, uint32_t tb, DecompressPlan& p) {
  const uint32_t maxsz = max_block_bytes((uint32_t)L);
  const uint32_t SC = locate_super_bytes(maxsz);
  p.fields.assign(nf, DecField{});
  p.tile_field.clear();
  p.loc_field.clear();
  p.tiles = p.locs = p.blocks = 0;
  p.plan_stride = ((sizeof(DecPlan) + 16ull * T + 4ull * (T + 1)) + 15) & ~(size_t)15;
  for (int f = 0; f < nf; f++) {
    const szp_gb300_field& in = fl[f];
    DecField& df = p.fields[f];
    memset(&df, 0, sizeof df);
    df.in = static_cast<const uint8_t*>(in.input);
    df.len = in.input_bytes;
    df.len_dev = reinterpret_cast<const uint64_t*>(in.input_len_dev);
    df.seg.n = in.nbEle;
    df.seg.T = (uint32_t)T;
    df.seg.L = (uint32_t)L;
    df.seg.tsz = in.nbEle / (uint64_t)T;
    df.plan = reinterpret_cast<DecPlan*>((uintptr_t)(p.plan_stride * (size_t)f));
    df.nblk_total = host_block_count(in.nbEle, T, L);
    df.blkpos = reinterpret_cast<uint32_t*>((uintptr_t)p.blocks);
    df.err = reinterpret_cast<uint32_t*>((uintptr_t)f);
    df.y = static_cast<float*>(in.output);
    uint64_t per_seg = 0, nt = 0;
    host_tile_counts(in.nbEle, T, L, tb, per_seg, nt);
    df.ntiles = (uint32_t)nt;
    df.tiles_per_seg = (uint32_t)per_seg;
    df.tile_base = (uint32_t)p.tiles;
    const uint64_t nloc = in.input_bytes / SC + (uint64_t)T + 1;
    df.loc_base = (uint32_t)p.locs;
    df.loc_ctas = (uint32_t)nloc;
    p.tile_field.insert(p.tile_field.end(), nt, (uint32_t)f);
    p.loc_field.insert(p.loc_field.end(), nloc, (uint32_t)f);
    p.tiles += nt;
    p.locs += nloc;
    p.blocks += df.nblk_total;
    if (p.tiles >= (1ull << 31) || p.locs >= (1ull << 31)) return host_fail(SZP_GB300_EINVAL, "batch too large");
  }
  return SZP_GB300_OK;
}

void place_decompress(DecompressPlan& p, uint8_t* d_plans, uint32_t* d_blkpos, uint32_t* d_err) {
  const int T = p.fields.empty() ? 1 : (int)p.fields[0].seg.T;
  for (auto& df : p.fields) {
    uint8_t* pb = d_plans + reinterpret_cast<uintptr_t>(df.plan);
    df.plan = reinterpret_cast<DecPlan*>(pb);
    df.reg0 = reinterpret_cast<uint64_t*>(pb + sizeof(DecPlan));
    df.reg1 = df.reg0 + T;
    df.chunk_base = reinterpret_cast<uint32_t*>(df.reg1 + T);
    df.blkpos = d_blkpos + reinterpret_cast<uintptr_t>(df.blkpos);
    df.err = d_err + reinterpret_cast<uintptr_t>(df.err);
  }
}

void args_compress(CompressArgs& a, RelBatchArgs& r, const CompressPlan& p, CompressField* d_fields,
                   const uint32_t* d_tile_field, const uint32_t* d_items, RelFieldState* d_state, uint64_t* status,
                   LaunchState* ls, uint32_t* err, uint32_t tb) {
  memset(&a, 0, sizeof a);
  a.seg.L = kBatchL;
  a.status = status;
  a.ls = ls;
  a.err = err;
  a.ntiles = (uint32_t)p.tiles;
  a.tb = tb;
  a.thr = host_bitcount_table();
  a.fields = d_fields;
  a.tile_field = d_tile_field;
  memset(&r, 0, sizeof r);
  r.fields = d_fields;
  r.state = d_state;
  r.item_field = d_items;
  r.nitems = (uint32_t)p.item_field.size();
  r.chunk = kRelChunk;
}

void args_decompress(DecArgs& a, const DecompressPlan& p, const DecField* d_fields, const uint32_t* d_tile_field,
                     const uint32_t* d_loc_field, uint2* aux, uint32_t* counters, uint64_t* status, LaunchState* ls,
                     uint32_t* err, uint32_t tb) {
  const uint32_t maxsz = max_block_bytes(kBatchL);
  memset(&a, 0, sizeof a);
  a.fm2 = false;
  a.chunk = locate_chunk_bytes(maxsz);
  a.super_chunk = locate_super_bytes(maxsz);
  a.overlap = locate_overlap_bytes(maxsz);
  a.maxsz = maxsz;
  a.aux = aux;
  a.counters = counters;
  a.status = status;
  a.ls = ls;
  a.err = err;
  a.ntiles = (uint32_t)p.tiles;
  a.tb = tb;
  a.bpw = tb / 8;
  a.nlocate_ctas = (uint32_t)p.locs;
  a.fields = d_fields;
  a.tile_field = d_tile_field;
  a.loc_field = d_loc_field;
}

int issue_compress(const CompressArgs& a, const RelBatchArgs& r, uint32_t rel_grid, int rounds, cudaStream_t st) {
  if (r.nitems) BCU(launch_rel_batch(r, rel_grid, st));
  if (a.ntiles) BCU(launch_compress_batch(a, kBatchL, rounds, st));
  return SZP_GB300_OK;
}

int issue_decompress(const DecArgs& a, uint32_t nfields, int rounds, cudaStream_t st) {
  BCU(launch_dec_setup_batch(a, nfields, st));
  BCU(launch_locate_batch(a, st));
  if (a.ntiles) BCU(launch_decode_batch(a, kBatchL, rounds, st));
  return SZP_GB300_OK;
}

}  // namespace szp

extern "C" {

int szp_gb300_batch_create(szp_gb300_batch* out, int direction, const szp_gb300_field* fields, int nfields,
                           int blockSize, int segments, int flags) {
  host_clear_error();
  if (!out) return host_fail(SZP_GB300_EINVAL, "null batch handle");
  *out = nullptr;
  if (direction != SZP_GB300_BATCH_COMPRESS && direction != SZP_GB300_BATCH_DECOMPRESS)
    return host_fail(SZP_GB300_EINVAL, "direction must be SZP_GB300_BATCH_COMPRESS or _DECOMPRESS");
  if (nfields < 0 || (nfields > 0 && !fields)) return host_fail(SZP_GB300_EINVAL, "bad field list");
  if ((uint32_t)blockSize != kBatchL) return host_fail(SZP_GB300_EINVAL, "batched path supports blockSize 32");
  const int T = host_resolve_segments(segments);
  for (int f = 0; f < nfields; f++) {
    const szp_gb300_field& fd = fields[f];
    if (fd.nbEle && (!fd.input || !fd.output)) return host_fail(SZP_GB300_EINVAL, "null field buffer");
    if (direction == SZP_GB300_BATCH_COMPRESS) {
      if (fd.output_bytes < 4 + 8ull * (uint64_t)T)
        return host_fail(SZP_GB300_ECAPACITY, "a field's output is smaller than the stream header");
    } else {
      if (fd.output_bytes < 4ull * fd.nbEle) return host_fail(SZP_GB300_ECAPACITY, "a field's output is too small");
      if (!fd.input) return host_fail(SZP_GB300_EINVAL, "null stream");
    }
  }
  szp_gb300_batch_s* b = new szp_gb300_batch_s();
  b->dir = direction;
  b->nfields = nfields;
  b->L = blockSize;
  b->T = T;
  b->graph = (flags & SZP_GB300_BATCH_NO_GRAPH) == 0;
  b->fields.assign(fields, fields + nfields);
  auto fail_out = [&](int rc) {
    delete b;
    return rc;
  };
  if (cudaGetDevice(&b->device) != cudaSuccess) return fail_out(host_fail(SZP_GB300_ECUDA, "no CUDA device"));
  {
    // kernel attributes are set before any capture
    cudaError_t pe = direction == SZP_GB300_BATCH_COMPRESS ? prepare_compress_batch() : prepare_decompress_batch();
    if (pe != cudaSuccess) return fail_out(host_fail(SZP_GB300_ECUDA, cudaGetErrorString(pe)));
  }
  // look-back words: the most tiles / locate tickets any tile size needs
  const uint32_t maxsz = max_block_bytes((uint32_t)blockSize);
  const uint32_t SC = locate_super_bytes(maxsz);
  uint64_t words = 1;
  {
    uint64_t tiles = 0, locs = 0;
    for (int f = 0; f < nfields; f++) {
      uint64_t ps, nt;
      host_tile_counts(fields[f].nbEle, T, blockSize, 64, ps, nt);  // the smallest tile (rounds 1)
      tiles += nt;
      if (direction == SZP_GB300_BATCH_DECOMPRESS) locs += fields[f].input_bytes / SC + (uint64_t)T + 1;
    }
    words = std::max<uint64_t>(words, std::max(tiles, locs));
  }
  b->status_words = words;
  cudaError_t e = b->al.get(&b->d_sizes, (size_t)nfields + 1);
  if (e == cudaSuccess) e = b->al.get(&b->d_err, (size_t)nfields + 1);
  if (e == cudaSuccess) e = b->al.get(&b->d_misc, 1);
  if (e == cudaSuccess) e = b->al.get(&b->d_status, words);
  if (e == cudaSuccess) e = cudaMemset(b->d_misc, 0, sizeof(DevScalars));
  if (e == cudaSuccess) e = cudaMemset(b->d_status, 0, words * sizeof(uint64_t));
  if (e == cudaSuccess) e = cudaMemset(b->d_sizes, 0, sizeof(unsigned long long) * ((size_t)nfields + 1));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&b->h_sizes, sizeof(unsigned long long) * ((size_t)nfields + 1));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&b->h_err, sizeof(uint32_t) * ((size_t)nfields + 2));
  if (e != cudaSuccess) return fail_out(host_fail(SZP_GB300_ENOMEM, cudaGetErrorString(e)));

  // tile size: fixed (the single-field choice) or tuned on this batch
  const int forced = (flags >> 8) & 0xF;
  if (forced && forced != 1 && forced != 2 && forced != 4)
    return fail_out(host_fail(SZP_GB300_EINVAL, "tile rounds must be 1, 2 or 4"));
  std::vector<int> cand = forced ? std::vector<int>{forced}
                         : (flags & SZP_GB300_BATCH_AUTOTUNE) ? std::vector<int>{4, 2, 1}
                                                             : std::vector<int>{4};
  float best = 0.0f;
  for (int r : cand) {
    Config* c = nullptr;
    int rc = make_config(*b, r, &c);
    if (rc) return fail_out(rc);
    b->tuned.push_back(c);
    float ms = 0.0f;
    if (cand.size() > 1) {  // tuning runs the batch on its current inputs
      rc = time_config(*b, *c, &ms);
      if (rc) return fail_out(rc);
    }
    if (!b->cfg || ms < best) {
      b->cfg = c;
      best = ms;
    }
  }
  capture(*b);
  *out = b;
  return SZP_GB300_OK;
}

int szp_gb300_batch_run(szp_gb300_batch b, void* stream) {
  host_clear_error();
  if (!b) return host_fail(SZP_GB300_EINVAL, "null batch");
  cudaStream_t st = (cudaStream_t)stream;
  if (b->exec) {
    BCU(cudaGraphLaunch(b->exec, st));
  } else {
    int rc = issue(*b, *b->cfg, st);
    if (rc) return rc;
  }
  BCU(cudaEventRecord(b->done, st));
  host_count_launches(b->dir == SZP_GB300_BATCH_COMPRESS ? (b->cfg->ra.nitems ? 2 : 1) : 3);
  return SZP_GB300_OK;
}

int szp_gb300_batch_sync(szp_gb300_batch b, unsigned long long* sizes, int* status) {
  host_clear_error();
  if (!b) return host_fail(SZP_GB300_EINVAL, "null batch");
  BCU(cudaEventSynchronize(b->done));
  const size_t nf = (size_t)b->nfields;
  BCU(cudaMemcpy(b->h_err, b->d_err, sizeof(uint32_t) * nf, cudaMemcpyDeviceToHost));
  BCU(cudaMemcpy(b->h_err + nf, &b->d_misc->err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  if (b->dir == SZP_GB300_BATCH_COMPRESS) {
    BCU(cudaMemcpy(b->h_sizes, b->d_sizes, sizeof(unsigned long long) * nf, cudaMemcpyDeviceToHost));
    if (sizes) memcpy(sizes, b->h_sizes, sizeof(unsigned long long) * nf);
  }
  const uint32_t launch_err = b->h_err[nf];
  int worst = SZP_GB300_OK;
  for (size_t f = 0; f < nf; f++) {
    const int st = host_status_from_err(b->h_err[f] | launch_err);
    if (status) status[f] = st;
    if (st != SZP_GB300_OK && worst == SZP_GB300_OK) worst = st;
  }
  if (worst != SZP_GB300_OK) return host_fail(worst, "a field of the batch failed (see its status)");
  host_clear_error();
  return SZP_GB300_OK;
}

const unsigned long long* szp_gb300_batch_sizes_dev(szp_gb300_batch b) { return b ? b->d_sizes : nullptr; }

int szp_gb300_batch_tile_rounds(szp_gb300_batch b) { return b && b->cfg ? b->cfg->rounds : 0; }

void szp_gb300_batch_destroy(szp_gb300_batch b) {
  if (!b) return;
  cudaEventSynchronize(b->done);
  delete b;
}

}  // extern "C"
