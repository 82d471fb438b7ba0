// convert.cu — packs the dense operand B for the tensor-core SpMM.
//
// B arrives as FP32, FP16 or BF16, row-major (k*ld + n) or column-major
// (k + n*ld, the reference's layout, src/cuda_hgemm/src/mma/mmaOBT.cu:75).
// The SpMM's B producer moves one 16-row slab of a 128-column tile with a
// single 4 KB bulk copy, so B is first packed into caller-provided scratch:
// tile (kb, t) holds rows k = 16*kb .. 16*kb+15 and columns
// n = 128*t .. 128*t+127 as 128 rows (one per n) of 16 16-bit k-values
// (32 bytes each), in the 32-byte-swizzled shared-memory layout the MMA reads
// (inside every 8-row group the two 16-byte halves of rows 4..7 are swapped).
// Tiles are ordered [t][kb] (column tile, then k-block: tile t*KB + kb);
// K is zero-padded to 16 and N to 128 (to 256
// when there is more than one tile, so that 256-column tiles stay in range).
// The split form writes hi = bf16(b) and lo = bf16(b - hi) as one 8 KB
// [hi tile | lo tile] pair per tile, so a tile is still one copy.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "convert.h"

namespace smat {
namespace dev {

enum : int { OUT_F16 = 0, OUT_BF16 = 1, OUT_SPLIT = 2 };

template <typename T>
__device__ __forceinline__ float load_f(const T* p);
template <>
__device__ __forceinline__ float load_f<float>(const float* p) {
  return __ldg(p);
}
template <>
__device__ __forceinline__ float load_f<__half>(const __half* p) {
  return __half2float(__ldg(p));
}
template <>
__device__ __forceinline__ float load_f<__nv_bfloat16>(const __nv_bfloat16* p) {
  return __bfloat162float(__ldg(p));
}

__device__ __forceinline__ uint4 pack8(const uint16_t* h) {
  return make_uint4(h[0] | ((uint32_t)h[1] << 16), h[2] | ((uint32_t)h[3] << 16), h[4] | ((uint32_t)h[5] << 16),
                    h[6] | ((uint32_t)h[7] << 16));
}

// Element i of a 16-byte vector of T, as float.
template <typename T>
__device__ __forceinline__ float vec_elem(const uint4* v, int i);
template <>
__device__ __forceinline__ float vec_elem<float>(const uint4* v, int i) {
  return __uint_as_float(reinterpret_cast<const uint32_t*>(v)[i]);
}
template <>
__device__ __forceinline__ float vec_elem<__half>(const uint4* v, int i) {
  return __half2float(__ushort_as_half(reinterpret_cast<const uint16_t*>(v)[i]));
}
template <>
__device__ __forceinline__ float vec_elem<__nv_bfloat16>(const uint4* v, int i) {
  return __bfloat162float(__ushort_as_bfloat16(reinterpret_cast<const uint16_t*>(v)[i]));
}

// One thread per (tile row n, k-block); 128 threads per tile. In the
// column-major layout the 16 k-values of a thread are contiguous and are
// read as 16-byte vectors where they are aligned and inside K.
template <typename T, int OUT>
__device__ __forceinline__ void pack_tile(const T* __restrict__ in, int layout, int64_t ldi, uint8_t* __restrict__ out,
                                          int64_t K, int64_t N, int ntiles, int64_t kb, int t, int r,
                                          const int32_t* __restrict__ kperm) {
  const int64_t n = (int64_t)t * 128 + r;
  constexpr int VEC = 16 / sizeof(T);  // elements per 16-byte vector
  float xv[16];
  const T* colp = in + kb * 16 + n * ldi;
  if (!kperm && layout == 1 && n < N && kb * 16 + 16 <= K && (reinterpret_cast<uintptr_t>(colp) & 15) == 0) {
    uint4 v[16 / VEC];
#pragma unroll
    for (int q = 0; q < 16 / VEC; q++) v[q] = __ldg(reinterpret_cast<const uint4*>(colp) + q);
#pragma unroll
    for (int i = 0; i < 16; i++) xv[i] = vec_elem<T>(&v[i / VEC], i % VEC);
  } else {
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const int64_t k = kb * 16 + i;
      const int64_t ks = (k < K && kperm) ? (int64_t)kperm[k] : k;  // row of B feeding permuted column k
      xv[i] = (k < K && n < N) ? load_f<T>(layout == 1 ? in + ks + n * ldi : in + ks * ldi + n) : 0.0f;
    }
  }
  uint16_t h[16], l[16];
#pragma unroll
  for (int i = 0; i < 16; i++) {
    const float x = xv[i];
    if (OUT == OUT_F16) {
      h[i] = __half_as_ushort(__float2half_rn(x));
    } else {
      const __nv_bfloat16 b = __float2bfloat16_rn(x);
      h[i] = __bfloat16_as_ushort(b);
      if (OUT == OUT_SPLIT) l[i] = __bfloat16_as_ushort(__float2bfloat16_rn(x - __bfloat162float(b)));
    }
  }
  const int64_t tile = (int64_t)t * ((K + 15) / 16) + kb;  // [column tile][k-block]
  const int sw = (r >> 2) & 1;
  constexpr int64_t kTileBytes = OUT == OUT_SPLIT ? 8192 : 4096;
  uint4* dst = reinterpret_cast<uint4*>(out + tile * kTileBytes + r * 32);
  dst[sw] = pack8(h);
  dst[sw ^ 1] = pack8(h + 8);
  if (OUT == OUT_SPLIT) {
    uint4* d2 = reinterpret_cast<uint4*>(out + tile * kTileBytes + 4096 + r * 32);
    d2[sw] = pack8(l);
    d2[sw ^ 1] = pack8(l + 8);
  }
}

template <typename T, int OUT>
__global__ void pack_b_tiles(const T* __restrict__ in, int layout, int64_t ldi, uint8_t* __restrict__ out,
                             int64_t K, int64_t N, int ntiles, const int32_t* __restrict__ kperm) {
  pack_tile<T, OUT>(in, layout, ldi, out, K, N, ntiles, blockIdx.y, blockIdx.x, threadIdx.x, kperm);
}

// Many B operands in one launch: block g packs tile (kb, t) of the job whose
// block range holds g (jobs sorted by their first block).
__global__ void pack_b_grouped_kernel(const PackJob* __restrict__ jobs, int njobs, int64_t total) {
  for (int64_t g = blockIdx.x; g < total; g += gridDim.x) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].begin <= g) lo = mid; else hi = mid - 1;
    }
    const PackJob& j = jobs[lo];
    const int64_t local = g - j.begin;
    const int64_t kb = local / j.ntiles;
    const int t = (int)(local % j.ntiles);
#define SMAT_GPACK(T)                                                                                        \
  switch (j.out_mode) {                                                                                      \
    case OUT_F16: pack_tile<T, OUT_F16>((const T*)j.in, j.layout, j.ldi, j.out, j.K, j.N, j.ntiles, kb, t, threadIdx.x, j.kperm); break; \
    case OUT_BF16: pack_tile<T, OUT_BF16>((const T*)j.in, j.layout, j.ldi, j.out, j.K, j.N, j.ntiles, kb, t, threadIdx.x, j.kperm); break; \
    default: pack_tile<T, OUT_SPLIT>((const T*)j.in, j.layout, j.ldi, j.out, j.K, j.N, j.ntiles, kb, t, threadIdx.x, j.kperm); break; \
  }
    switch (j.in_dtype) {
      case 0: SMAT_GPACK(float) break;
      case 1: SMAT_GPACK(__half) break;
      default: SMAT_GPACK(__nv_bfloat16) break;
    }
#undef SMAT_GPACK
  }
}

// Column-major B with 16-byte aligned columns: warp w of a block packs
// column n = blockIdx.y * 8 + w for 32 consecutive k-blocks (lane = k-block),
// so a warp reads 32 consecutive 32-byte pieces of one column (1 KB,
// contiguous) -- the access shape that also suits B in host memory read over
// the CPU-GPU link -- and each lane writes its 32-byte row of one tile.
template <typename T, int OUT>
__global__ void pack_b_colmajor(const T* __restrict__ in, int64_t ldi, uint8_t* __restrict__ out, int64_t K,
                                int64_t N, int ntiles, int64_t kbs) {
  const int64_t kb = (int64_t)blockIdx.x * 32 + (threadIdx.x & 31);
  const int64_t n = (int64_t)blockIdx.y * 8 + (threadIdx.x >> 5);
  if (kb >= kbs || n >= (int64_t)ntiles * 128) return;
  pack_tile<T, OUT>(in, 1, ldi, out, K, N, ntiles, kb, (int)(n >> 7), (int)(n & 127), nullptr);
}

template <typename T, int OUT>
static cudaError_t run_pack(const void* in, int layout, int64_t ldi, uint8_t* out, int64_t K, int64_t N,
                            const int32_t* kperm, cudaStream_t s) {
  const int ntiles = (int)packed_b_tiles(N);
  const int64_t kbs = (K + 15) / 16;
  if (kbs == 0 || ntiles == 0) return cudaSuccess;
  if (!kperm && layout == 1 && ((reinterpret_cast<uintptr_t>(in) | (uint64_t)ldi * sizeof(T)) & 15) == 0) {
    dim3 grid((unsigned)((kbs + 31) / 32), (unsigned)((int64_t)ntiles * 128 / 8));
    pack_b_colmajor<T, OUT><<<grid, 256, 0, s>>>((const T*)in, ldi, out, K, N, ntiles, kbs);
    return cudaGetLastError();
  }
  dim3 grid((unsigned)ntiles, (unsigned)kbs);
  pack_b_tiles<T, OUT><<<grid, 128, 0, s>>>((const T*)in, layout, ldi, out, K, N, ntiles, kperm);
  return cudaGetLastError();
}

// The 2:4 path's B operand from the packed tiles: tile (t, w) holds k-blocks
// 2w and 2w+1 of column tile t side by side, 128 rows (n) of 64 bytes (32
// k-values) in the 64-byte swizzle (inside every 8-row group, 16-byte chunk
// c of row n sits at chunk c ^ ((n >> 1) & 3)). One thread per row.
__global__ void pack_b_sw64_kernel(const uint8_t* __restrict__ p32, uint8_t* __restrict__ out, int64_t kbs,
                                   int64_t kw) {
  const int64_t w = blockIdx.x;
  const int64_t t = blockIdx.y;
  const int n = threadIdx.x;
  uint4 c[4];
#pragma unroll
  for (int hb = 0; hb < 2; ++hb) {
    const int64_t kb = 2 * w + hb;
    if (kb < kbs) {
      const uint4* src = reinterpret_cast<const uint4*>(p32 + (t * kbs + kb) * 4096 + n * 32);
      const int sw = (n >> 2) & 1;
      c[2 * hb] = src[sw];
      c[2 * hb + 1] = src[sw ^ 1];
    } else {
      c[2 * hb] = c[2 * hb + 1] = make_uint4(0, 0, 0, 0);
    }
  }
  uint4* dst = reinterpret_cast<uint4*>(out + (t * kw + w) * 8192 + n * 64);
  const int sw = (n >> 1) & 3;
#pragma unroll
  for (int q = 0; q < 4; ++q) dst[q ^ sw] = c[q];
}

}  // namespace dev

size_t packed_b64_bytes(int64_t K, int64_t N) {
  const int64_t kw = ((K + 15) / 16 + 1) / 2;
  return (size_t)kw * (size_t)packed_b_tiles(N) * 8192;
}

cudaError_t pack_b_sw64(const uint8_t* packed32, int64_t K, int64_t N, uint8_t* out, cudaStream_t s) {
  const int64_t kbs = (K + 15) / 16, kw = (kbs + 1) / 2, nt = packed_b_tiles(N);
  if (kw == 0 || nt == 0) return cudaSuccess;
  dim3 grid((unsigned)kw, (unsigned)nt);
  dev::pack_b_sw64_kernel<<<grid, 128, 0, s>>>(packed32, out, kbs, kw);
  return cudaGetLastError();
}

int64_t packed_b_tiles(int64_t N) {
  const int64_t t = (N + 127) / 128;
  return t > 1 ? (t + 1) / 2 * 2 : t;
}

size_t packed_b_bytes(int64_t K, int64_t N) {
  return (size_t)((K + 15) / 16) * (size_t)packed_b_tiles(N) * 4096;
}

cudaError_t pack_b(const void* in, int in_dtype, int layout, int64_t ldi, int out_mode, uint8_t* out,
                   int64_t K, int64_t N, const int32_t* kperm, cudaStream_t s) {
  using namespace dev;
#define SMAT_PACK(T)                                                                  \
  switch (out_mode) {                                                                 \
    case OUT_F16: return run_pack<T, OUT_F16>(in, layout, ldi, out, K, N, kperm, s);     \
    case OUT_BF16: return run_pack<T, OUT_BF16>(in, layout, ldi, out, K, N, kperm, s);   \
    case OUT_SPLIT: return run_pack<T, OUT_SPLIT>(in, layout, ldi, out, K, N, kperm, s); \
    default: return cudaErrorInvalidValue;                                            \
  }
  switch (in_dtype) {
    case 0: SMAT_PACK(float)
    case 1: SMAT_PACK(__half)
    case 2: SMAT_PACK(__nv_bfloat16)
    default: return cudaErrorInvalidValue;
  }
#undef SMAT_PACK
}

}  // namespace smat

namespace smat {

cudaError_t pack_b_grouped(const PackJob* d_jobs, int njobs, int64_t total_blocks, int num_sms, cudaStream_t s) {
  if (njobs == 0 || total_blocks == 0) return cudaSuccess;
  const int64_t want = (int64_t)num_sms * 16;
  const int grid = (int)(total_blocks < want ? total_blocks : want);
  dev::pack_b_grouped_kernel<<<grid, 128, 0, s>>>(d_jobs, njobs, total_blocks);
  return cudaGetLastError();
}

}  // namespace smat
