// noalloc.cu -- a fastmode1 compressor entry point that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they compress: a
// process that hands all GPU memory to its own pool or allocator up front, a
// real-time or serving loop where the implicit device synchronisation of
// cudaMalloc/cudaFree would stall every other stream, or code running where
// the CUDA allocator may not be entered.  szp_gb300_compress_dev_noalloc()
// serves them: the caller passes the input and output device buffers, and the
// kernel's working memory (look-back status words, launch counters, the REL
// range partials) lives in one statically sized __device__ array of this file,
// which every GPU that loads the library holds until the process exits.
//
// The array is shared by all calls: calls that overlap on the GPU (different
// streams, or host threads without ordering between them) race on it.  Each
// call clears the parts that must start at zero before launching.
#include <cstring>
#include <mutex>

#include "szp_gb300.h"
#include "szp_kernels.h"

namespace szp {
namespace {

constexpr uint64_t kNoAllocMaxTiles = 16384;  // 134,217,728 floats at blockSize 32
constexpr int kNoAllocRelGrid = 1024;
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
  LaunchState ls;
  uint32_t err;
  uint32_t rel_counter;
  uint64_t out_size;
  float eb;
  float pad;
  float rel_partial[2 * kNoAllocRelGrid];
  uint64_t status[kNoAllocMaxTiles];
};

// The working memory.  In host code this name is only a stand-in for the
// device symbol: its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

std::mutex g_setup_mu;
NoAllocScratch* g_scratch_dev[kMaxDevices];  // device address per device, set once

// Once per device, with that device current: the device address of the array.
int scratch_for_current_device(NoAllocScratch** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return host_fail(SZP_GB300_ECUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return host_fail(SZP_GB300_EINVAL, "device index out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return host_fail(SZP_GB300_ECUDA, cudaGetErrorString(e));
    g_scratch_dev[dev] = static_cast<NoAllocScratch*>(p);
  }
  *out = g_scratch_dev[dev];
  return SZP_GB300_OK;
}

}  // namespace
}  // namespace szp

using namespace szp;

extern "C" int szp_gb300_compress_dev_noalloc(const float* d_data, size_t nbEle, int errBoundMode,
                                              double absErrBound, double relBoundRatio, int blockSize,
                                              int segments, unsigned char* d_out, size_t out_capacity,
                                              size_t* outSize, void* stream) {
  host_clear_error();
  if (outSize) *outSize = 0;
  if (blockSize <= 0) return host_fail(SZP_GB300_EINVAL, "blockSize must be positive");
  if (!d_out || (nbEle && !d_data)) return host_fail(SZP_GB300_EINVAL, "null device buffer");
  if ((uintptr_t)d_data & 3) return host_fail(SZP_GB300_EINVAL, "input not aligned to its element size");
  const int T = host_resolve_segments(segments);
  const uint64_t head = 4 + 8ull * (uint64_t)T;
  if (out_capacity < head) return host_fail(SZP_GB300_ECAPACITY, "output buffer smaller than the stream header");
  uint64_t per_seg = 0, ntiles = 0;
  uint32_t tb = 0, bpw = 0;
  host_compress_tiles(nbEle, T, blockSize, per_seg, ntiles, tb, bpw);
  if (ntiles > kNoAllocMaxTiles)
    return host_fail(SZP_GB300_EINVAL,
                     "input too large for the allocation-free compressor (at most 16384 tiles of "
                     "256 blocks, 134217728 floats at blockSize 32)");
  if (compress_smem_bytes((uint32_t)blockSize, tb) > 200 * 1024)
    return host_fail(SZP_GB300_EINVAL, "blockSize too large");
  NoAllocScratch* sc = nullptr;
  int rc = scratch_for_current_device(&sc);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;

  // clear what must start at zero: ticket, error word, REL counter, and the
  // status words this launch will use (older contents would look ready)
  cudaError_t e = cudaMemsetAsync(sc, 0, offsetof(NoAllocScratch, out_size), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(sc->status, 0, ntiles * sizeof(uint64_t), st);
  if (e != cudaSuccess) return host_fail(SZP_GB300_ECUDA, cudaGetErrorString(e));

  CompressArgs a;
  memset(&a, 0, sizeof a);
  a.x = d_data;
  a.out = d_out;
  a.cap = out_capacity;
  a.seg.n = nbEle;
  a.seg.T = (uint32_t)T;
  a.seg.L = (uint32_t)blockSize;
  a.seg.tsz = nbEle / (uint64_t)T;
  a.eb = (float)absErrBound;
  a.eb_dev = nullptr;
  a.status = sc->status;
  a.ls = &sc->ls;
  a.err = &sc->err;
  a.out_size = &sc->out_size;
  a.ntiles = (uint32_t)ntiles;
  a.tiles_per_seg = (uint32_t)per_seg;
  a.tb = tb;
  a.bpw = bpw;
  host_segment_blocks(nbEle, T, blockSize, a.nb_reg, a.nb_last);
  a.thr = host_bitcount_table();
  int launches = 1;
  if (errBoundMode == REL) {
    RelArgs r;
    memset(&r, 0, sizeof r);
    r.x = d_data;
    r.n = nbEle;
    r.rel = (float)relBoundRatio;
    r.partial = sc->rel_partial;
    r.counter = &sc->rel_counter;
    r.eb_out = &sc->eb;
    r.err = &sc->err;
    uint64_t want = (nbEle / 4 + 255) / 256;
    uint32_t grid = (uint32_t)(want < 1 ? 1 : (want > kNoAllocRelGrid ? kNoAllocRelGrid : want));
    e = launch_rel_bound(r, grid, st);
    if (e != cudaSuccess) return host_fail(SZP_GB300_ECUDA, cudaGetErrorString(e));
    a.eb_dev = &sc->eb;
    launches++;
  }
  e = launch_compress(a, false, st);
  if (e != cudaSuccess) return host_fail(SZP_GB300_ECUDA, cudaGetErrorString(e));
  host_count_launches(launches);

  // the stream size and the error word, copied to host variables
  uint64_t size = 0;
  uint32_t err = 0;
  e = cudaMemcpyAsync(&size, &sc->out_size, sizeof size, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, &sc->err, sizeof err, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return host_fail(SZP_GB300_ECUDA, cudaGetErrorString(e));
  if (outSize) *outSize = (size_t)size;
  host_set_notices(err);  // NaN or |x/eb| >= 2^31 met, as szp_gb300_compress_dev reports it
  return host_status_from_err(err);
}
