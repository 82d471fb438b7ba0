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

// Packs B into 4 KB swizzled tiles ordered [k-block][128-column tile].
// in_dtype: 0 F32, 1 F16, 2 BF16; layout: 0 row-major (k*ldi + n), 1
// column-major (k + n*ldi); out_mode: 0 FP16, 1 BF16, 2 hi+lo BF16 (8 KB
// [hi | lo] per tile, twice packed_b_bytes).
cudaError_t pack_b(const void* in, int in_dtype, int layout, int64_t ldi, int out_mode, uint8_t* out,
                   int64_t K, int64_t N, cudaStream_t s);

}  // namespace smat
