// convert.h — B operand packing (convert.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace smat {

// 128-column tiles per k-block of the packed layout (padded to an even count
// when there is more than one).
int64_t packed_b_tiles(int64_t N);

// Bytes of one packed copy of a K x N operand.
size_t packed_b_bytes(int64_t K, int64_t N);

// Packs B into 4 KB swizzled tiles ordered [128-column tile][k-block], so
// that the tiles of consecutive k-blocks of one column tile are contiguous.
// in_dtype: 0 F32, 1 F16, 2 BF16; layout: 0 row-major (k*ldi + n), 1
// column-major (k + n*ldi); out_mode: 0 FP16, 1 BF16, 2 hi+lo BF16 (8 KB
// [hi | lo] per tile, twice packed_b_bytes).
// kperm (device, optional): row kperm[k] of `in` feeds packed row k (a
// column permutation of A; gathered with scalar loads).
cudaError_t pack_b(const void* in, int in_dtype, int layout, int64_t ldi, int out_mode, uint8_t* out,
                   int64_t K, int64_t N, const int32_t* kperm, cudaStream_t s);

// The 2:4 path's copy of B: 8 KB tiles ordered [128-column tile][window],
// window w = k-blocks 2w and 2w+1 (32 k-values; the second half zero past
// K), 128 rows of 64 bytes in the 64-byte swizzle, made from the packed
// FP16/BF16 tiles of pack_b.
size_t packed_b64_bytes(int64_t K, int64_t N);
cudaError_t pack_b_sw64(const uint8_t* packed32, int64_t K, int64_t N, uint8_t* out, cudaStream_t s);

// One B operand of a grouped pack: tiles of `in` (in_dtype, layout, ldi,
// K x N) into `out` (out_mode as pack_b), covering global blocks
// [begin, begin + ntiles * ceil(K / 16)).
struct PackJob {
  const void* in;
  uint8_t* out;
  const int32_t* kperm;  // column permutation of A (device), or null
  int64_t ldi, K, N, begin;
  int32_t in_dtype, layout, out_mode, ntiles;
};

// Packs every job in one launch (jobs sorted by begin, in device memory).
cudaError_t pack_b_grouped(const PackJob* d_jobs, int njobs, int64_t total_blocks, int num_sms, cudaStream_t s);

}  // namespace smat
