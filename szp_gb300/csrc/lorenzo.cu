// lorenzo.cu -- the multidimensional Lorenzo variant's own passes for sm_103a.
//
// A field of nx*ny*nz floats (x fastest) is stored as the fastmode1 stream
// (blockSize 32) of the int32 codes
//     r = q - q[j-1] - q[k-1] + q[j-1][k-1]      (neighbours outside are 0)
// where q are fastmode1's quantization codes; the 1-D delta fastmode1 takes
// along x makes the packed values the 3-D Lorenzo residual.  The stream starts
// with [nx][ny][nz] as u32 little-endian.  This file holds the passes around
// the fastmode1 pipelines (which pack and unpack r as codes):
//   lorenzo_codes_kernel  x -> r, and the 12-byte dims header (lorenzo_codes4_kernel:
//                         the same by float4s)
//   lorenzo_ysum_kernel   r -> r summed along y, in place
//   lorenzo_zsum_kernel   ... summed along z and dequantized, in place
// The reference predicts along the flattened array only; this variant has no
// reference code and is checked against the oracle's restatement.
#include "szp_device.cuh"
#include "szp_kernels.h"

namespace szp {

// (float)q * eb with the x86 NaN rule when eb is not finite (szpd_float.cc:67,86,112);
// the same arithmetic as the decode pipelines'.
__device__ __forceinline__ float x86_dequant(uint32_t q, float eb, bool special) {
  const float f = __int2float_rn((int32_t)q);
  const float r = __fmul_rn(f, eb);
  return special ? x86_nan_fix(r, f, eb) : r;
}

// x -> r: one CTA per row (j, k) at a time, rows blockIdx.x, + grid, ...
// ((j, k) stepped without a division per row); each element quantizes itself
// and its three neighbours in y and z (those rows were read moments before,
// by this or a neighbouring CTA, and come from L2).
__global__ void __launch_bounds__(256) lorenzo_codes_kernel(const LorenzoArgs a) {
  const float eb = a.eb_dev ? *a.eb_dev : a.eb;
  const float inv = __fdiv_rn(1.0f, eb);  // fastmode1's float inverse (szp_float.cc:185)
  uint32_t flags = 0;
  const uint32_t nx = a.nx, ny = a.ny;
  const uint64_t plane = (uint64_t)nx * ny, rows = (uint64_t)ny * a.nz;
  const uint64_t G = gridDim.x;
  const uint64_t gk = G / ny;
  const uint32_t gj = (uint32_t)(G % ny);
  uint64_t k = blockIdx.x / ny;
  uint32_t j = (uint32_t)(blockIdx.x % ny);
  for (uint64_t row = blockIdx.x; row < rows; row += G) {
    const float* __restrict__ x0 = a.x + row * nx;
    int32_t* __restrict__ r0 = a.r + row * nx;
    for (uint32_t i = threadIdx.x; i < nx; i += blockDim.x) {
      uint32_t v = (uint32_t)quantize(__ldg(x0 + i), inv, flags);
      if (j) v -= (uint32_t)quantize(__ldg(x0 + i - nx), inv, flags);
      if (k) v -= (uint32_t)quantize(__ldg(x0 + i - plane), inv, flags);
      if (j && k) v += (uint32_t)quantize(__ldg(x0 + i - plane - nx), inv, flags);
      r0[i] = (int32_t)v;
    }
    j += gj;
    k += gk;
    if (j >= ny) {
      j -= ny;
      k++;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < 12) {
    const uint32_t d[3] = {a.nx, a.ny, a.nz};
    a.head[threadIdx.x] = (uint8_t)(d[threadIdx.x >> 2] >> (8 * (threadIdx.x & 3)));
  }
  if (__any_sync(0xffffffffu, flags != 0) && (threadIdx.x & 31) == 0) atomicOr(a.err, kErrQuantRange);
}

// The same codes, 4 elements per thread: rows of nx = 4 * nx4 values, x and r
// 16-byte aligned, n / 4 below 2^32.  A flat grid-stride over the float4s of
// the field; each takes its row's (j, k) by two 32-bit divisions and loads its
// three neighbours as float4s (from L2: the grid covers several planes at once).
__global__ void __launch_bounds__(256) lorenzo_codes4_kernel(const LorenzoArgs a) {
  const float eb = a.eb_dev ? *a.eb_dev : a.eb;
  const float inv = __fdiv_rn(1.0f, eb);
  uint32_t flags = 0;
  const uint32_t nx4 = a.nx >> 2, ny = a.ny;
  const uint32_t plane4 = nx4 * ny;
  const uint32_t total = plane4 * a.nz;
  const float4* __restrict__ x4 = reinterpret_cast<const float4*>(a.x);
  int4* __restrict__ r4 = reinterpret_cast<int4*>(a.r);
  auto q4 = [&](float4 v) {
    return make_int4(quantize(v.x, inv, flags), quantize(v.y, inv, flags), quantize(v.z, inv, flags),
                     quantize(v.w, inv, flags));
  };
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i64 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i64 < total; i64 += stride) {
    const uint32_t it = (uint32_t)i64;
    const uint32_t row = it / nx4, j = row % ny, k = row / ny;
    const int4 c = q4(__ldg(x4 + it));
    uint32_t v0 = (uint32_t)c.x, v1 = (uint32_t)c.y, v2 = (uint32_t)c.z, v3 = (uint32_t)c.w;
    if (j) {
      const int4 p = q4(__ldg(x4 + it - nx4));
      v0 -= (uint32_t)p.x; v1 -= (uint32_t)p.y; v2 -= (uint32_t)p.z; v3 -= (uint32_t)p.w;
    }
    if (k) {
      const int4 p = q4(__ldg(x4 + it - plane4));
      v0 -= (uint32_t)p.x; v1 -= (uint32_t)p.y; v2 -= (uint32_t)p.z; v3 -= (uint32_t)p.w;
    }
    if (j && k) {
      const int4 p = q4(__ldg(x4 + it - plane4 - nx4));
      v0 += (uint32_t)p.x; v1 += (uint32_t)p.y; v2 += (uint32_t)p.z; v3 += (uint32_t)p.w;
    }
    r4[it] = make_int4((int32_t)v0, (int32_t)v1, (int32_t)v2, (int32_t)v3);
  }
  if (blockIdx.x == 0 && threadIdx.x < 12) {
    const uint32_t d[3] = {a.nx, a.ny, a.nz};
    a.head[threadIdx.x] = (uint8_t)(d[threadIdx.x >> 2] >> (8 * (threadIdx.x & 3)));
  }
  if (__any_sync(0xffffffffu, flags != 0) && (threadIdx.x & 31) == 0) atomicOr(a.err, kErrQuantRange);
}

// In-place running sums of q along a line of `len` elements `stride` apart,
// starting at p; eight loads in flight before their sums are stored.
// DEQ: the sums are dequantized ((float)q * eb, szpd_float.cc:67,86,112) and
// stored as floats.
template <bool DEQ>
__device__ __forceinline__ void lorenzo_line(int32_t* __restrict__ p, uint64_t stride, uint32_t len, float eb,
                                             bool special) {
  uint32_t run = 0;
  uint32_t j = 0;
  for (; j + 8 <= len; j += 8) {
    uint32_t v[8];
#pragma unroll
    for (int u = 0; u < 8; u++) v[u] = (uint32_t)p[(j + u) * stride];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      run += v[u];
      if (DEQ) {
        reinterpret_cast<float*>(p)[(j + u) * stride] = x86_dequant(run, eb, special);
      } else {
        p[(j + u) * stride] = (int32_t)run;
      }
    }
  }
  for (; j < len; j++) {
    run += (uint32_t)p[j * stride];
    if (DEQ) {
      reinterpret_cast<float*>(p)[j * stride] = x86_dequant(run, eb, special);
    } else {
      p[j * stride] = (int32_t)run;
    }
  }
}

// One thread per (k, i): sums along y.
__global__ void __launch_bounds__(256) lorenzo_ysum_kernel(const LorenzoArgs a) {
  const uint64_t cols = (uint64_t)a.nx * a.nz, plane = (uint64_t)a.nx * a.ny;
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = c % a.nx, k = c / a.nx;
    lorenzo_line<false>(a.q + k * plane + i, a.nx, a.ny, 0.0f, false);
  }
}

// One thread per (j, i): sums along z, then dequantizes in place.
__global__ void __launch_bounds__(256) lorenzo_zsum_kernel(const LorenzoArgs a) {
  const float eb = *a.eb_dev;
  const bool special = !isfinite(eb);
  const uint64_t cols = (uint64_t)a.nx * a.ny;
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += (uint64_t)gridDim.x * blockDim.x)
    lorenzo_line<true>(a.q + c, cols, a.nz, eb, special);
}

static uint32_t lorenzo_grid(uint64_t items, uint32_t per_cta, uint32_t cap) {
  const uint64_t g = (items + per_cta - 1) / per_cta;
  return (uint32_t)(g < 1 ? 1 : (g > cap ? cap : g));
}

cudaError_t launch_lorenzo_codes(const LorenzoArgs& a, uint32_t sm_count, cudaStream_t st) {
  const uint64_t n4 = (uint64_t)a.nx * a.ny * a.nz / 4;
  if ((a.nx & 3) == 0 && n4 > 0 && n4 < (1ull << 32) && ((uintptr_t)a.x & 15) == 0 && ((uintptr_t)a.r & 15) == 0) {
    lorenzo_codes4_kernel<<<lorenzo_grid(n4, 256, 8 * sm_count), 256, 0, st>>>(a);
  } else {
    lorenzo_codes_kernel<<<lorenzo_grid((uint64_t)a.ny * a.nz, 1, 8 * sm_count), 256, 0, st>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_lorenzo_inverse(const LorenzoArgs& a, uint32_t sm_count, cudaStream_t st) {
  if ((uint64_t)a.nx * a.ny * a.nz == 0) return cudaSuccess;
  lorenzo_ysum_kernel<<<lorenzo_grid((uint64_t)a.nx * a.nz, 256, 16 * sm_count), 256, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  lorenzo_zsum_kernel<<<lorenzo_grid((uint64_t)a.nx * a.ny, 256, 16 * sm_count), 256, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace szp
