// features.cu — the 64-value matrix description the tau / block-shape
// predictor reads, computed on the GPU from the CSR.
//
//   [0, 16)   row-length histogram: fraction of rows with length 0, 1, 2-3,
//             4-7, ..., >= 2^14 (bin 1 + floor(log2 len), capped at 15)
//   [16, 32)  bandwidth profile: fraction of nonzeros with |col - row| /
//             max(rows, cols) in each of 16 equal bins
//   [32, 48)  fill of the nonzero 16 x 16 tiles: fraction of tiles whose
//             nonzero count c has floor(2 log2 c) in each bin (capped at 15)
//   [48, 64)  scalars: log2(rows + 1) / 20, log2(cols + 1) / 20,
//             log2(nnz + 1) / 30, min(1, 100 * density), mean row length / 64,
//             row-length std / mean, max / mean row length / 100, fraction of
//             nonzeros on the diagonal, fraction of empty rows, nonzero tiles
//             per 16-row block row / 64, mean tile fill (nnz / tiles / 256),
//             log2(tiles + 1) / 25, fraction of nonzeros with |col - row| < 64,
//             then three zeros.
//
// Tiles are counted with an open-addressing hash table in device memory
// (twice as many slots as nonzeros, bounded probing).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "smat_internal.h"

namespace smat {
namespace dev {

constexpr unsigned long long kEmpty = ~0ull;

struct FeatAcc {
  unsigned long long row_hist[16];
  unsigned long long band_hist[16];
  unsigned long long tile_hist[16];
  unsigned long long sum_len, sum_len2, max_len, diag, empty_rows, near, tiles, tile_nnz;
};

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

__global__ void feat_rows_kernel(const int64_t* __restrict__ rp, const int32_t* __restrict__ ci, int64_t rows,
                                 int64_t cols, int64_t nbc, unsigned long long* __restrict__ keys,
                                 unsigned int* __restrict__ counts, unsigned long long mask, FeatAcc* acc,
                                 int* overflow) {
  __shared__ unsigned long long s_row[16], s_band[16];
  for (int i = threadIdx.x; i < 16; i += blockDim.x) s_row[i] = s_band[i] = 0;
  __syncthreads();
  const double span = (double)(rows > cols ? rows : cols);
  unsigned long long sl = 0, sl2 = 0, ml = 0, dg = 0, er = 0, nr = 0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = rp[r], e = rp[r + 1];
    const unsigned long long len = (unsigned long long)(e - b);
    const int bin = len == 0 ? 0 : min(15, 1 + (63 - __clzll((long long)len)));
    atomicAdd(&s_row[bin], 1ull);
    sl += len;
    sl2 += len * len;
    ml = len > ml ? len : ml;
    er += len == 0;
    for (int64_t k = b; k < e; k++) {
      const int64_t c = ci[k];
      const int64_t d = c > r ? c - r : r - c;
      dg += d == 0;
      nr += d < 64;
      atomicAdd(&s_band[min(15, (int)((double)d / span * 16.0))], 1ull);
      const unsigned long long key = (unsigned long long)(r >> 4) * (unsigned long long)nbc + (unsigned long long)(c >> 4);
      unsigned long long h = mix64(key) & mask;
      bool placed = false;
      for (unsigned long long probe = 0; probe <= mask; probe++) {
        const unsigned long long prev = atomicCAS(&keys[h], kEmpty, key);
        if (prev == kEmpty || prev == key) {
          atomicAdd(&counts[h], 1u);
          placed = true;
          break;
        }
        h = (h + 1) & mask;
      }
      if (!placed) atomicExch(overflow, 1);
    }
  }
  atomicAdd(&acc->sum_len, sl);
  atomicAdd(&acc->sum_len2, sl2);
  atomicMax(&acc->max_len, ml);
  atomicAdd(&acc->diag, dg);
  atomicAdd(&acc->empty_rows, er);
  atomicAdd(&acc->near, nr);
  __syncthreads();
  for (int i = threadIdx.x; i < 16; i += blockDim.x) {
    atomicAdd(&acc->row_hist[i], s_row[i]);
    atomicAdd(&acc->band_hist[i], s_band[i]);
  }
}

__global__ void feat_tiles_kernel(const unsigned long long* __restrict__ keys, const unsigned int* __restrict__ counts,
                                  unsigned long long slots, FeatAcc* acc) {
  __shared__ unsigned long long s_hist[16];
  for (int i = threadIdx.x; i < 16; i += blockDim.x) s_hist[i] = 0;
  __syncthreads();
  unsigned long long nt = 0, nz = 0;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < slots;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    if (keys[i] == kEmpty) continue;
    const unsigned int c = counts[i];
    nt++;
    nz += c;
    const int bin = min(15, (int)floorf(2.0f * log2f((float)c)));
    atomicAdd(&s_hist[bin], 1ull);
  }
  atomicAdd(&acc->tiles, nt);
  atomicAdd(&acc->tile_nnz, nz);
  __syncthreads();
  for (int i = threadIdx.x; i < 16; i += blockDim.x) atomicAdd(&acc->tile_hist[i], s_hist[i]);
}

}  // namespace dev
}  // namespace smat

using namespace smat;

extern "C" smat_status smat_features(const smat_csr* A, int32_t device, float* out) {
  if (!A || !out || !A->row_ptr || (A->nnz > 0 && !A->col_idx)) return fail(SMAT_ERR_INVALID, "null argument");
  if (A->rows < 0 || A->cols < 0 || A->row_ptr[0] != 0 || A->row_ptr[A->rows] != A->nnz)
    return fail(SMAT_ERR_INVALID, "malformed CSR");
  for (int64_t k = 0; k < A->nnz; k++)
    if (A->col_idx[k] < 0 || A->col_idx[k] >= A->cols) return fail(SMAT_ERR_INVALID, "column index out of range");
  int prev = -1;
  cudaGetDevice(&prev);
  if (cudaSetDevice(device) != cudaSuccess) return fail(SMAT_ERR_CUDA, "cudaSetDevice failed");
  const int64_t rows = A->rows, nnz = A->nnz;
  unsigned long long slots = 1024;
  while (slots < 2ull * (unsigned long long)nnz) slots <<= 1;
  int64_t* d_rp = nullptr;
  int32_t* d_ci = nullptr;
  unsigned long long* d_keys = nullptr;
  unsigned int* d_counts = nullptr;
  dev::FeatAcc* d_acc = nullptr;
  int* d_over = nullptr;
  std::string err;
  auto ck = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && err.empty()) err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaSuccess;
  };
  if (ck(cudaMalloc(&d_rp, (rows + 1) * sizeof(int64_t)), "cudaMalloc") &&
      ck(cudaMalloc(&d_ci, std::max<int64_t>(nnz, 1) * sizeof(int32_t)), "cudaMalloc") &&
      ck(cudaMalloc(&d_keys, slots * sizeof(unsigned long long)), "cudaMalloc") &&
      ck(cudaMalloc(&d_counts, slots * sizeof(unsigned int)), "cudaMalloc") &&
      ck(cudaMalloc(&d_acc, sizeof(dev::FeatAcc)), "cudaMalloc") && ck(cudaMalloc(&d_over, sizeof(int)), "cudaMalloc") &&
      ck(cudaMemcpy(d_rp, A->row_ptr, (rows + 1) * sizeof(int64_t), cudaMemcpyHostToDevice), "cudaMemcpy") &&
      (nnz == 0 || ck(cudaMemcpy(d_ci, A->col_idx, nnz * sizeof(int32_t), cudaMemcpyHostToDevice), "cudaMemcpy")) &&
      ck(cudaMemset(d_keys, 0xff, slots * sizeof(unsigned long long)), "cudaMemset") &&
      ck(cudaMemset(d_counts, 0, slots * sizeof(unsigned int)), "cudaMemset") &&
      ck(cudaMemset(d_acc, 0, sizeof(dev::FeatAcc)), "cudaMemset") && ck(cudaMemset(d_over, 0, sizeof(int)), "cudaMemset")) {
    int sms = 148;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int64_t nbc = (A->cols + 15) / 16;
    const int gr = (int)std::max<int64_t>(1, std::min<int64_t>((rows + 255) / 256, (int64_t)sms * 8));
    dev::feat_rows_kernel<<<gr, 256>>>(d_rp, d_ci, rows, A->cols, nbc, d_keys, d_counts, slots - 1, d_acc, d_over);
    ck(cudaGetLastError(), "feature kernel launch");
    const int gt = (int)std::min<unsigned long long>((slots + 255) / 256, (unsigned long long)sms * 8);
    dev::feat_tiles_kernel<<<gt, 256>>>(d_keys, d_counts, slots, d_acc);
    ck(cudaGetLastError(), "feature kernel launch");
    dev::FeatAcc acc;
    int over = 0;
    if (ck(cudaMemcpy(&acc, d_acc, sizeof(acc), cudaMemcpyDeviceToHost), "cudaMemcpy") &&
        ck(cudaMemcpy(&over, d_over, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy")) {
      if (over) err = "tile hash table overflow";
      const double R = std::max<double>(1.0, (double)rows), Z = std::max<double>(1.0, (double)nnz);
      const double T = std::max<double>(1.0, (double)acc.tiles);
      for (int i = 0; i < 16; i++) {
        out[i] = (float)(acc.row_hist[i] / R);
        out[16 + i] = (float)(acc.band_hist[i] / Z);
        out[32 + i] = (float)(acc.tile_hist[i] / T);
      }
      const double mean = acc.sum_len / R;
      const double var = std::max(0.0, acc.sum_len2 / R - mean * mean);
      const double density = (double)nnz / std::max(1.0, (double)rows * (double)std::max<int64_t>(1, A->cols));
      float* s = out + 48;
      s[0] = (float)(std::log2((double)rows + 1) / 20);
      s[1] = (float)(std::log2((double)A->cols + 1) / 20);
      s[2] = (float)(std::log2((double)nnz + 1) / 30);
      s[3] = (float)std::min(1.0, 100.0 * density);
      s[4] = (float)(mean / 64);
      s[5] = (float)(mean > 0 ? std::sqrt(var) / mean : 0.0);
      s[6] = (float)(mean > 0 ? acc.max_len / mean / 100 : 0.0);
      s[7] = (float)(acc.diag / Z);
      s[8] = (float)(acc.empty_rows / R);
      s[9] = (float)(acc.tiles / std::max(1.0, std::ceil(rows / 16.0)) / 64);
      s[10] = (float)(acc.tile_nnz / T / 256);
      s[11] = (float)(std::log2((double)acc.tiles + 1) / 25);
      s[12] = (float)(acc.near / Z);
      s[13] = s[14] = s[15] = 0.0f;
    }
  }
  cudaFree(d_rp);
  cudaFree(d_ci);
  cudaFree(d_keys);
  cudaFree(d_counts);
  cudaFree(d_acc);
  cudaFree(d_over);
  if (prev >= 0) cudaSetDevice(prev);
  if (!err.empty()) return fail(SMAT_ERR_CUDA, err);
  return SMAT_OK;
}
