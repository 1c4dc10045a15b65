// szp_kernels.h -- kernel argument blocks and launchers (host + device view).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "szp_device.cuh"

namespace szp {

// One field of a batched compression (a device array, one entry per field).
struct CompressField {
  const float* x;
  uint8_t* out;
  uint64_t cap;          // bytes available at out
  Segments seg;
  uint64_t nb_reg;       // blocks of segments 0..T-2
  uint64_t nb_last;      // blocks of segment T-1
  uint32_t tiles_per_seg;
  uint32_t ntiles;       // tiles of this field
  uint32_t tile_base;    // its first tile in the launch
  float eb;              // the bound (REL: written by the range pass)
  float rel;             // (float)relBoundRatio, or 0 for ABS
  uint32_t pad;
  uint64_t* out_size;    // stream bytes of this field
  uint32_t* err;         // this field's error word
};

struct CompressArgs {
  const float* x;
  uint8_t* out;
  uint64_t cap;          // bytes available at out
  Segments seg;
  float eb;              // used when eb_dev == nullptr
  const float* eb_dev;   // device eb (REL mode)
  uint64_t* status;      // one look-back word per tile
  LaunchState* ls;
  uint32_t* err;
  uint64_t* out_size;    // stream bytes, written by the last tile
  uint32_t ntiles;
  uint32_t tiles_per_seg;  // tiles of segments 0..T-2
  uint32_t tb;           // blocks per tile
  uint32_t bpw;          // blocks per warp (generic kernel)
  uint64_t nb_reg;       // blocks of segments 0..T-2
  uint64_t nb_last;      // blocks of segment T-1
  BitcountTable thr;
  // batched launches: tiles of all fields, field of each tile
  const CompressField* fields;
  const uint32_t* tile_field;
  // float64 data (compress_generic<.., double>): input, bound and where a REL
  // range pass left it; the stream's eb header is then 8 bytes
  const double* xd;
  double ebd;
  const double* ebd_dev;
  // 1/eb of float64 data, rounded as binary64 (the reference's inverse), and
  // where a REL range pass left it
  double invd;
  const double* invd_dev;
  // compress_pipe<…, QI>: eb header bytes, 8 (float64 stream, eb from
  // ebd/ebd_dev) or 4 (float stream of codes, eb from eb/eb_dev)
  uint32_t qhb;
};

// Per-field state of the batched range pass: order-preserving encodings of
// the running min and max, chunks done, and the field's chunk count.  The
// last chunk of a field computes its bound and resets the state.
struct RelFieldState {
  uint32_t mn, mx, done, nitems;
  uint32_t first_item;  // the field's first work item
  uint32_t pad[3];
};

struct RelBatchArgs {
  CompressField* fields;        // eb written for REL fields
  RelFieldState* state;         // per field
  const uint32_t* item_field;   // work item -> field
  uint32_t nitems;
  uint32_t chunk;               // elements per work item
};

struct RelArgs {
  const float* x;
  uint64_t n;
  float rel;        // (float)relBoundRatio
  float* partial;   // 2 floats per CTA (2 doubles for float64 data)
  uint32_t* counter;
  float* eb_out;
  // float64 data: (max - min) * rel in double (szp.cc:77-89)
  const double* xd;
  double rel_d;
  double* ebd_out;
  double* invd_out;  // 1/eb, rounded as binary64
  uint32_t* err;     // optional: a bulk copy that never landed sets kErrLookbackTimeout
};

// Decompression plan, filled on the device from the stream header.
struct DecPlan {
  float eb;
  uint32_t nchunks;      // total chunks over all segments
  uint32_t bad;          // header failed validation
  uint32_t pad;
  double ebd;            // float64 streams: the 8-byte eb
  // followed in memory by: uint32 chunk_base[T+1]; uint64 reg0[T]; uint64 reg1[T]
};

// One field of a decompression: its stream, geometry, plan and output.
struct DecField {
  const uint8_t* in;        // stream (device)
  uint64_t len;             // stream bytes available
  const uint64_t* len_dev;  // optional device-side stream length (min with len)
  Segments seg;
  DecPlan* plan;
  uint32_t* chunk_base;     // [T+1] locate chunks before each segment
  uint64_t* reg0;           // [T] absolute start of each segment's block region
  uint64_t* reg1;           // [T] absolute end of it (exclusive)
  uint32_t* blkpos;         // per block: header offset relative to its segment's region start
  uint64_t nblk_total;
  float* y;                 // output
  double* yd;               // output of a float64 stream (decode_generic<.., double>)
  uint32_t ntiles;          // decode tiles of this field
  uint32_t tiles_per_seg;
  uint32_t tile_base;       // its first decode tile in the launch
  uint32_t loc_base;        // its first locate ticket in the launch
  uint32_t loc_ctas;        // locate tickets it may use
  uint32_t* err;            // this field's error word
};

struct DecArgs {
  DecField f;            // the field of a single-field launch
  bool fm2;
  uint32_t hb;           // bytes of the stream's eb header: 4 (float) or 8 (double)
  uint32_t chunk;        // bytes per locate thread
  uint32_t super_chunk;  // bytes per locate CTA (chunk * threads)
  uint32_t overlap;      // bytes walked before a CTA's region to find the header chain
  uint32_t maxsz;        // largest block (including a fastmode2 seed)
  uint2* aux;            // per locate ticket: (entry, exit) of its header chain
  uint32_t* counters;    // [0] repairs of the last launch
  uint64_t* status;      // look-back words
  LaunchState* ls;
  uint32_t* err;         // launch error word (waits that gave up)
  uint32_t ntiles;       // decode tiles of the launch
  uint32_t tb;
  uint32_t bpw;
  uint32_t nlocate_ctas; // locate tickets of the launch (upper bound)
  uint32_t static_tiles; // decode pipeline: CTA c takes tiles c, c + grid, ... (a cooperative launch)
  // batched launches
  const DecField* fields;
  const uint32_t* tile_field;  // decode tile -> field
  const uint32_t* loc_field;   // locate ticket -> field
};

uint32_t compress_blocks_per_tile(uint32_t L, uint32_t& bpw);
size_t compress_smem_bytes(uint32_t L, uint32_t tb);
cudaError_t launch_compress(const CompressArgs& a, bool fm2, cudaStream_t st);
// fastmode1, blockSize 32, one field (fm1_pipes.cu); launch_compress takes it
// whenever it applies
bool compress32_supported(const CompressArgs& a);
cudaError_t launch_compress32(const CompressArgs& a, cudaStream_t st);
// float64 data: every blockSize on the one-warp-per-block kernels
uint32_t compress_blocks_per_tile_f64(uint32_t L, uint32_t& bpw);
size_t compress_smem_bytes_f64(uint32_t L, uint32_t tb);
cudaError_t launch_compress_f64(const CompressArgs& a, bool fm2, cudaStream_t st);
cudaError_t launch_rel_bound_f64(const RelArgs& a, uint32_t grid, cudaStream_t st);
// float64 data on the fastmode pipelines (blockSize 8..256): a pass turns x
// into int32 q, the pipeline packs q into a stream with an 8-byte eb header
// (a.x = q, a.ebd/a.ebd_dev the header's eb).  The decode pipeline writes the
// doubles itself.
bool f64_pipe_supported(uint32_t L);
int32_t* f64_q_view(void* qbuf, const void* x);  // q array whose 16-byte boundaries match x's
cudaError_t launch_quantize_f64(const double* x, int32_t* q, uint64_t n, double invd, const double* invd_dev,
                                uint32_t* err, uint32_t sm_count, cudaStream_t st);
cudaError_t launch_compress_q(const CompressArgs& a, bool fm2, cudaStream_t st);

cudaError_t launch_rel_bound(const RelArgs& a, uint32_t grid, cudaStream_t st);
cudaError_t launch_compress_batch(const CompressArgs& a, uint32_t L, int rounds, cudaStream_t st);
cudaError_t prepare_compress_batch();
cudaError_t launch_rel_batch(const RelBatchArgs& a, uint32_t grid, cudaStream_t st);
uint32_t rel_encode_host(float v);
cudaError_t launch_wait_probe(uint64_t limit_ns, uint32_t* err, unsigned long long* waited, cudaStream_t st);
cudaError_t launch_bitcount_probe(const uint32_t* in, uint8_t* out, uint64_t n, const BitcountTable& thr,
                                  cudaStream_t st);

// decompression
uint32_t decode_blocks_per_tile(uint32_t L, uint32_t& bpw);
uint32_t locate_chunk_bytes(uint32_t maxsz);
uint32_t locate_super_bytes(uint32_t maxsz);
uint32_t locate_overlap_bytes(uint32_t maxsz);
size_t locate_smem_bytes(uint32_t super_chunk, uint32_t overlap, uint32_t maxsz);
size_t decode_smem_bytes(uint32_t L, uint32_t tb, bool fm2);
cudaError_t launch_dec_setup(const DecArgs& a, cudaStream_t st);
cudaError_t launch_locate(const DecArgs& a, cudaStream_t st);
cudaError_t launch_decode(const DecArgs& a, cudaStream_t st);
uint32_t decode_blocks_per_tile_f64(uint32_t L, uint32_t& bpw);
cudaError_t launch_decode_f64(const DecArgs& a, cudaStream_t st);
cudaError_t launch_decode_q(const DecArgs& a, cudaStream_t st);      // a.f.y: the output doubles
// a.f.y: the int32 codes (accumulate: added to the codes already there)
cudaError_t launch_decode_codes(const DecArgs& a, bool accumulate, cudaStream_t st);
// batched decompression (fastmode1, blockSize 32)
cudaError_t launch_dec_setup_batch(const DecArgs& a, uint32_t nfields, cudaStream_t st);
cudaError_t launch_locate_batch(const DecArgs& a, cudaStream_t st);
cudaError_t launch_decode_batch(const DecArgs& a, uint32_t L, int rounds, cudaStream_t st);
cudaError_t prepare_decompress_batch();

// the multidimensional Lorenzo variant (lorenzo.cu)
struct LorenzoArgs {
  const float* x;       // field, x fastest (compression)
  int32_t* r;           // its codes r (compression)
  int32_t* q;           // decoded codes, summed and dequantized in place (decompression)
  uint8_t* head;        // the stream's 12-byte dims header (compression)
  uint32_t nx, ny, nz;
  float eb;             // bound, when eb_dev is null
  const float* eb_dev;  // device bound: the range pass's, or the decoded stream's
  uint32_t* err;
};
cudaError_t launch_lorenzo_codes(const LorenzoArgs& a, uint32_t sm_count, cudaStream_t st);
cudaError_t launch_lorenzo_inverse(const LorenzoArgs& a, uint32_t sm_count, cudaStream_t st);
// host helpers (api.cu)
const BitcountTable& host_bitcount_table();
int host_resolve_segments(int requested);
void host_compress_tiles(size_t n, int T, int L, uint64_t& tiles_per_seg, uint64_t& ntiles, uint32_t& tb,
                         uint32_t& bpw);
void host_segment_blocks(size_t n, int T, int L, uint64_t& nb_reg, uint64_t& nb_last);
void host_tile_counts(size_t n, int T, int L, uint32_t tb, uint64_t& tiles_per_seg, uint64_t& ntiles);
uint64_t host_block_count(size_t n, int T, int L);
size_t host_max_stream_bytes(size_t n, int L, int T);
int host_status_from_err(uint32_t err);
int host_fail(int status, const char* msg);
// Records the non-fatal notices of a finished launch's error word (what
// szp_gb300_last_notices() returns).
void host_set_notices(uint32_t err);
void host_clear_error();
void host_count_launches(int k);

}  // namespace szp
