// spmm_24ref.cu — the reference's 2:4 compression, in the reference's own
// output format, behind its launcher names (preprocessing_mmaSTKernel,
// src/cuda_hgemm/src/mma/mmaST.cu:22-140 and :316-326, and
// preprocessing_mmaSTKernel_large, mmaST_large.cu:22-152 and :324-335), for
// callers that feed the result to other reference code.
//
// 16 x 16 blocks, per block whose blockInfo entry is 1 (relative index rel):
// each of the 32 lanes of a block owns row lane / 2, columns
// 8 * (lane % 2) .. +7, as two groups of four. In each group the nonzero
// values (FP16 compare with zero: -0 counts as zero, NaN as nonzero) are
// kept in order, the first two of them into the group's two output slots
// (unused slots 0), and the column of the n-th kept value (n = 0, 1, ...) is
// ORed into the lane's metadata byte at bit 4 - 4g + 2n for group g (bits
// that fall past bit 7 are lost). So for a true 2:4 row the byte holds
// group 0's indices in bits 4-5 and 6-7 and group 1's in bits 0-1 and 2-3;
// a group with more than two nonzeros keeps its first two values and, in
// group 1, ORs the extra indices over group 0's bits, as the reference does.
// metadata[rel * 32 + lane] = that byte; the lane's four kept values go to
// sparseMatrixA[rel * 128 + lane * 4 .. +3].
//
// 16 x 32 blocks ("large"): lane owns row lane / 2, columns
// 16 * (lane % 2) .. +15, as two parts of eight columns, each compressed
// like a 16-wide lane above into one byte m0 / m1 and four values; the
// eight values go to sparseMatrixA[rel * 256 + lane * 8 .. +7]. The
// reference stores the bytes as metadata[rel * 64 + lane] = m0 and then
// metadata[rel * 64 + lane + 1] = m1, so each lane's m1 lands on the byte
// the next lane's m0 went to, one instruction later: the block's metadata
// ends up as m0 of lane 0 at byte 0 and m1 of lane l at byte l + 1
// (bytes 0..32 of the block's 64; bytes 33..63 are not written).
//
// Blocks marked 0 or 2 are not written. Nothing is written when M or N is
// 0 (the reference's grid is then empty).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "smat_internal.h"
#include "smat_ref_shims.h"

namespace smat {
namespace dev {

// One warp per block-grid cell, grid-stride over the cells.
__global__ void compress24_ref_kernel(const uint16_t* __restrict__ vals, uint8_t* __restrict__ meta,
                                      uint16_t* __restrict__ packed, const int* __restrict__ block_info,
                                      const int* __restrict__ rel_map, int64_t n_cells) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t cell = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); cell < n_cells;
       cell += warps) {
    if (block_info[cell] != 1) continue;  // warp-uniform
    const int64_t rel = rel_map[cell];
    const uint16_t* src = vals + rel * 256 + (lane >> 1) * 16 + (lane & 1) * 8;
    uint32_t m = 0;
    uint16_t out[4] = {0, 0, 0, 0};
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      int n = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint16_t v = src[4 * g + i];
        if ((v & 0x7fffu) != 0) {
          if (n < 2) out[2 * g + n] = v;
          m |= (uint32_t)i << (4 - 4 * g + 2 * n);
          ++n;
        }
      }
    }
    meta[rel * 32 + lane] = (uint8_t)(m & 0xffu);
    uint2 w;
    w.x = (uint32_t)out[0] | ((uint32_t)out[1] << 16);
    w.y = (uint32_t)out[2] | ((uint32_t)out[3] << 16);
    reinterpret_cast<uint2*>(packed)[rel * 32 + lane] = w;
  }
}

// One byte of metadata and four values from the eight 16-bit values of two
// groups of four (the rule described at the top of the file).
__device__ __forceinline__ uint32_t compress_two_groups(const uint16_t* src, uint16_t out[4]) {
  uint32_t m = 0;
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    int n = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const uint16_t v = src[4 * g + i];
      if ((v & 0x7fffu) != 0) {
        if (n < 2) out[2 * g + n] = v;
        m |= (uint32_t)i << (4 - 4 * g + 2 * n);
        ++n;
      }
    }
  }
  return m & 0xffu;
}

// 16 x 32 blocks: one warp per block-grid cell, grid-stride over the cells.
__global__ void compress24_ref_large_kernel(const uint16_t* __restrict__ vals, uint8_t* __restrict__ meta,
                                            uint16_t* __restrict__ packed, const int* __restrict__ block_info,
                                            const int* __restrict__ rel_map, int64_t n_cells) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t cell = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); cell < n_cells;
       cell += warps) {
    if (block_info[cell] != 1) continue;  // warp-uniform
    const int64_t rel = rel_map[cell];
    const uint16_t* src = vals + rel * 512 + (lane >> 1) * 32 + (lane & 1) * 16;
    uint16_t out[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const uint32_t m0 = compress_two_groups(src, out);
    const uint32_t m1 = compress_two_groups(src + 8, out + 4);
    // the bytes as they stand after the reference's two stores (see above)
    if (lane == 0) meta[rel * 64] = (uint8_t)m0;
    meta[rel * 64 + lane + 1] = (uint8_t)m1;
    uint4 w;
    w.x = (uint32_t)out[0] | ((uint32_t)out[1] << 16);
    w.y = (uint32_t)out[2] | ((uint32_t)out[3] << 16);
    w.z = (uint32_t)out[4] | ((uint32_t)out[5] << 16);
    w.w = (uint32_t)out[6] | ((uint32_t)out[7] << 16);
    reinterpret_cast<uint4*>(packed)[rel * 32 + lane] = w;
  }
}

}  // namespace dev
}  // namespace smat

void preprocessing_mmaSTKernel(half* bcsrValuesA, char* metadata, half* sparseMatrixA, size_t M, size_t N, size_t K,
                               size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping) {
  (void)nonzeroBlocks;
  if (M == 0 || N == 0 || K == 0) return;
  const int64_t cells = (int64_t)((M + 15) / 16) * (int64_t)((K + 15) / 16);
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = (cells + 7) / 8;
  const int grid = (int)(want < (int64_t)sms * 16 ? want : (int64_t)sms * 16);
  smat::dev::compress24_ref_kernel<<<grid, 256>>>(reinterpret_cast<const uint16_t*>(bcsrValuesA),
                                                  reinterpret_cast<uint8_t*>(metadata),
                                                  reinterpret_cast<uint16_t*>(sparseMatrixA), blockInfo,
                                                  relativeBlockIndexMapping, cells);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) smat::set_error(std::string("preprocessing_mmaSTKernel: ") + cudaGetErrorString(e));
}

void preprocessing_mmaSTKernel_large(half* bcsrValuesA, char* metadata, half* sparseMatrixA, size_t M, size_t N,
                                     size_t K, size_t nonzeroBlocks, int* blockInfo,
                                     int* relativeBlockIndexMapping) {
  (void)nonzeroBlocks;
  if (M == 0 || N == 0 || K == 0) return;
  const int64_t cells = (int64_t)((M + 15) / 16) * (int64_t)((K + 31) / 32);
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = (cells + 7) / 8;
  const int grid = (int)(want < (int64_t)sms * 16 ? want : (int64_t)sms * 16);
  smat::dev::compress24_ref_large_kernel<<<grid, 256>>>(reinterpret_cast<const uint16_t*>(bcsrValuesA),
                                                        reinterpret_cast<uint8_t*>(metadata),
                                                        reinterpret_cast<uint16_t*>(sparseMatrixA), blockInfo,
                                                        relativeBlockIndexMapping, cells);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) smat::set_error(std::string("preprocessing_mmaSTKernel_large: ") + cudaGetErrorString(e));
}
