// szp_kernels.h -- kernel argument blocks and launchers (host + device view).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "szp_device.cuh"

namespace szp {

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
};

struct RelArgs {
  const float* x;
  uint64_t n;
  float rel;        // (float)relBoundRatio
  float* partial;   // 2 floats per CTA
  uint32_t* counter;
  float* eb_out;
};

// Decompression plan, filled on the device from the stream header.
struct DecPlan {
  float eb;
  uint32_t nchunks;      // total chunks over all segments
  uint32_t bad;          // header failed validation
  uint32_t pad;
  // followed in memory by: uint32 chunk_base[T+1]; uint64 reg0[T]; uint64 reg1[T]
};

struct DecArgs {
  const uint8_t* in;     // stream (device)
  uint64_t len;          // stream bytes available
  const uint64_t* len_dev;  // optional device-side stream length (min with len)
  Segments seg;
  bool fm2;
  DecPlan* plan;
  uint32_t* chunk_base;  // [T+1]
  uint64_t* reg0;        // [T] absolute start of each segment's block region
  uint64_t* reg1;        // [T] absolute end of it (exclusive)
  uint32_t chunk;        // bytes per locate thread
  uint32_t super_chunk;  // bytes per locate CTA (chunk * threads)
  uint32_t overlap;      // bytes walked before a CTA's region to find the header chain
  uint32_t maxsz;        // largest block (including a fastmode2 seed)
  uint2* aux;            // per locate CTA: (entry, exit) of its header chain
  uint32_t* counters;    // [0] repairs of the last launch
  uint64_t* status;      // look-back words
  LaunchState* ls;
  uint32_t* err;
  uint32_t* blkpos;      // per block: header offset relative to its segment's region start
  uint64_t nblk_total;
  float* y;              // output
  uint32_t ntiles;
  uint32_t tiles_per_seg;
  uint32_t tb;
  uint32_t bpw;
  uint32_t nlocate_ctas; // CTAs of the locate kernel (upper bound)
};

uint32_t compress_blocks_per_tile(uint32_t L, uint32_t& bpw);
size_t compress_smem_bytes(uint32_t L, uint32_t tb);
cudaError_t launch_compress(const CompressArgs& a, bool fm2, cudaStream_t st);
cudaError_t launch_rel_bound(const RelArgs& a, uint32_t grid, cudaStream_t st);
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

// host helpers (api.cu)
const BitcountTable& host_bitcount_table();
int host_resolve_segments(int requested);
void host_compress_tiles(size_t n, int T, int L, uint64_t& tiles_per_seg, uint64_t& ntiles, uint32_t& tb,
                         uint32_t& bpw);
void host_segment_blocks(size_t n, int T, int L, uint64_t& nb_reg, uint64_t& nb_last);
int host_fail(int status, const char* msg);
void host_clear_error();
void host_count_launches(int k);

}  // namespace szp
