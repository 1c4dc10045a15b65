// szp_batch.h -- host-side tables of one batched launch, shared by the batch
// objects (batch.cu) and the request server (serve.cu).
//
// plan_*() turns a field list into the per-field descriptors and the ticket ->
// field tables the batched kernels read; device addresses inside the
// descriptors are left as offsets until place_*() adds the bases of the
// buffers the caller placed the tables in.
#pragma once
#include <cstdint>
#include <vector>

#include "szp_gb300.h"
#include "szp_kernels.h"

namespace szp {

constexpr uint32_t kBatchL = 32;          // blockSize of the batched path
constexpr uint32_t kRelChunk = 1u << 15;  // floats per range-pass work item (128 KiB: 32 loads per thread)

inline uint32_t batch_tile_blocks(int rounds) { return 8u * (uint32_t)rounds * 8u; }

struct CompressPlan {
  std::vector<CompressField> fields;  // out_size / err: field index until placed
  std::vector<uint32_t> tile_field, item_field;
  std::vector<RelFieldState> rel;
  uint64_t tiles = 0;
};

struct DecompressPlan {
  std::vector<DecField> fields;  // plan/reg0/reg1/chunk_base, blkpos, err: offsets until placed
  std::vector<uint32_t> tile_field, loc_field;
  uint64_t tiles = 0, locs = 0, blocks = 0;
  size_t plan_stride = 0;  // bytes of DecPlan + reg0[T] + reg1[T] + chunk_base[T+1] per field
};

int plan_compress(const szp_gb300_field* fl, int nf, int L, int T, uint32_t tb, CompressPlan& p);
void place_compress(CompressPlan& p, unsigned long long* d_sizes, uint32_t* d_err);
int plan_decompress(const szp_gb300_field* fl, int nf, int L, int T, uint32_t tb, DecompressPlan& p);
void place_decompress(DecompressPlan& p, uint8_t* d_plans, uint32_t* d_blkpos, uint32_t* d_err);

// Launch arguments over placed tables.
void args_compress(CompressArgs& a, RelBatchArgs& r, const CompressPlan& p, CompressField* d_fields,
                   const uint32_t* d_tile_field, const uint32_t* d_items, RelFieldState* d_state, uint64_t* status,
                   LaunchState* ls, uint32_t* err, uint32_t tb);
void args_decompress(DecArgs& a, const DecompressPlan& p, const DecField* d_fields, const uint32_t* d_tile_field,
                     const uint32_t* d_loc_field, uint2* aux, uint32_t* counters, uint64_t* status, LaunchState* ls,
                     uint32_t* err, uint32_t tb);

// The stages of one run.
int issue_compress(const CompressArgs& a, const RelBatchArgs& r, uint32_t rel_grid, int rounds,
                   cudaStream_t st);
int issue_decompress(const DecArgs& a, uint32_t nfields, int rounds, cudaStream_t st);

}  // namespace szp
