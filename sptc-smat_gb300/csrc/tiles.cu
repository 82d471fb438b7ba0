// tiles.cu — the reference's merged 4 x 4-block tiles (SparseMatrix::
// bcsrBlocking, src/cuda_hgemm/src/common/matrix.h:794-1137), built on the
// GPU from a device BCSR, bit-identical to the reference's output.
//
// The reference builds the tiles on the host with a linear search over the
// tiles made so far for every block. Here each step is data-parallel over
// blocks, tiles or tile-grid cells (tiles_core.h gives the reasoning):
//   1. check the row pointers, then every block finds the block that made
//      its tile (binary searches in at most three block rows above it);
//   2. tile numbers = exclusive scan of the "maker" flags;
//   3. makers write their tile's column start, tile row and grid cell; every
//      block copies its values into its tile (one warp per block, 16-byte
//      vectors) and, from the values in its registers, ORs its share of the
//      tile's position labels in (warp ballots, one atomic per position);
//   4. tile-row starts and their ranks (scan) give the tile row pointer; a
//      scan over the tile grid gives the relative index map; the label
//      flags become labels.
// Scans are a three-launch exclusive scan (chunk sums, one CTA over the sums,
// chunk scans). The build reads the tile and row counts back twice, so it
// synchronises the stream it runs on; it allocates its outputs and scratch
// with cudaMalloc. Memory: the tile values take 256 k FP16 per tile, the
// grid two int32 per 64 x 4k cell.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "smat_internal.h"
#include "tiles_core.h"

struct smat_tiles {
  int device = 0;
  smat::tiles::Geom g{};
  int64_t n_tiles = 0;
  int64_t n_rowptr = 1;
  uint16_t* val = nullptr;
  int32_t* rowptr = nullptr;
  int32_t* colidx = nullptr;
  int32_t* block_info = nullptr;
  int32_t* rel_map = nullptr;
  int32_t* tile_info = nullptr;
};

namespace smat {
namespace dev {

using tiles::Geom;

constexpr int kScanThreads = 256;
constexpr int kScanPer = 8;
constexpr int kScanChunk = kScanThreads * kScanPer;

// Exclusive scan of one value per thread over a 256-thread CTA; *total gets
// the CTA's sum. Every thread of the CTA must call it.
__device__ __forceinline__ int cta_exclusive_scan(int v, int* total) {
  __shared__ int warp_sum[kScanThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int s = lane < kScanThreads / 32 ? warp_sum[lane] : 0;
#pragma unroll
    for (int o = 1; o < kScanThreads / 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kScanThreads / 32) warp_sum[lane] = s;
  }
  __syncthreads();
  const int base = wid ? warp_sum[wid - 1] : 0;
  *total = warp_sum[kScanThreads / 32 - 1];
  __syncthreads();  // warp_sum is reused by the next call
  return base + x - v;
}

// Scan phase 1: the sum of each chunk of kScanChunk inputs.
__global__ void __launch_bounds__(kScanThreads) scan_chunk_sums(const int32_t* in, int64_t n, int32_t* sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * kScanPer;
  int s = 0;
#pragma unroll
  for (int j = 0; j < kScanPer; ++j)
    if (base + j < n) s += in[base + j];
  int tot = 0;
  cta_exclusive_scan(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// Scan phase 2 (one CTA): chunk sums -> chunk offsets, in place; *total = all.
__global__ void __launch_bounds__(kScanThreads) scan_chunk_offsets(int32_t* sums, int64_t nchunks, int32_t* total) {
  int carry = 0;
  for (int64_t b0 = 0; b0 < nchunks; b0 += kScanThreads) {
    const int64_t i = b0 + threadIdx.x;
    const int v = i < nchunks ? sums[i] : 0;
    int tot = 0;
    const int e = cta_exclusive_scan(v, &tot);
    if (i < nchunks) sums[i] = carry + e;
    carry += tot;
  }
  if (threadIdx.x == 0) *total = carry;
}

// Scan phase 3: out[i] = offset of i's chunk + sum of the chunk's inputs
// before i (out may alias in: a thread reads its own inputs before writing).
__global__ void __launch_bounds__(kScanThreads) scan_chunks(const int32_t* in, int64_t n, const int32_t* offsets,
                                                            int32_t* out) {
  const int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * kScanPer;
  int v[kScanPer];
  int s = 0;
#pragma unroll
  for (int j = 0; j < kScanPer; ++j) {
    v[j] = base + j < n ? in[base + j] : 0;
    s += v[j];
  }
  int tot = 0;
  int run = offsets[blockIdx.x] + cta_exclusive_scan(s, &tot);
#pragma unroll
  for (int j = 0; j < kScanPer; ++j) {
    if (base + j < n) out[base + j] = run;
    run += v[j];
  }
}

__global__ void tiles_check_rows(Geom g, const int32_t* rowptr, int32_t* bad) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < g.nbr; r += (int64_t)gridDim.x * blockDim.x) {
    const int b = tiles::check_row(g, rowptr, r);
    if (b) atomicOr(bad, b);
  }
}

// Step 1. Runs only when the row pointers passed their check (they index the
// column array). Also keeps every block's block row for the later steps.
__global__ void tiles_mark(Geom g, const int32_t* rowptr, const int32_t* colidx, const int32_t* bad,
                           int32_t* maker, int32_t* is_maker, int32_t* brow, int32_t* bad_out) {
  if (*bad & tiles::BAD_ROWPTR) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.nnzb; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = tiles::block_row_of(rowptr, g.nbr, i);
    int b = 0;
    int64_t m = tiles::tile_maker(g, rowptr, colidx, i, r, &b);
    if (b) {
      atomicOr(bad_out, b);
      m = i;
    }
    maker[i] = (int32_t)m;
    is_maker[i] = m == i ? 1 : 0;
    brow[i] = (int32_t)r;
  }
}

// Step 3a: tile of every block; makers describe their tile.
__global__ void tiles_place(Geom g, const int32_t* brow, const int32_t* colidx, const int32_t* maker,
                            const int32_t* tile_no, int32_t* tile_of_block, int32_t* tile_col, int32_t* tile_row,
                            int32_t* block_info) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.nnzb; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = maker[i];
    const int32_t t = tile_no[m];
    tile_of_block[i] = t;
    if (m == i) {
      const int64_t x = colidx[i] / g.tw, y = brow[i] / 4;
      tile_col[t] = (int32_t)(x * g.tw);
      tile_row[t] = (int32_t)y;
      block_info[y * g.tile_cols + x] = 1;
    }
  }
}

// Step 3b: one warp per block copies its 16 x k values (32k bytes) into its
// tile with 16-byte vectors, and ORs the label flags of its rows into
// positions (block row in tile, rho % 4) of the tile (tiles_core.h). A
// lane's vectors all lie in rows with the same rho % 4.
__global__ void tiles_scatter(Geom g, const int32_t* brow, const int32_t* colidx, const uint16_t* bval,
                              const int32_t* tile_of_block, uint16_t* tval, int32_t* label_flags) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int vpr = g.k / 8;   // 16-byte vectors per block row
  const int nvec = 16 * vpr;  // 16-byte vectors per block
  // lanes whose rows fall on position column sc = lane (lanes 0..3 use it)
  uint32_t lanes_of_sc = 0;
  for (int l = 0; l < 32; ++l) lanes_of_sc |= (((l / vpr) & 3) == (lane & 3) ? 1u : 0u) << l;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < g.nnzb; i += warps) {
    const int64_t r = brow[i];
    const int32_t t = tile_of_block[i];
    const int64_t off = (int64_t)t * g.tsz + tiles::block_offset_in_tile(g, r, colidx[i]);
    const uint4* src = reinterpret_cast<const uint4*>(bval + i * 16 * g.k);
    uint4* dst = reinterpret_cast<uint4*>(tval + off);
    int fl = 0;
    for (int j = lane; j < nvec; j += 32) {
      const uint4 v = src[j];
      dst[j] = v;
      fl |= tiles::group_flags(v.x, v.y) | tiles::group_flags(v.z, v.w);
    }
    const uint32_t any = __ballot_sync(0xffffffffu, fl & 1);
    const uint32_t two = __ballot_sync(0xffffffffu, fl & 2);
    if (lane < 4 && (any & lanes_of_sc))
      atomicOr(&label_flags[(int64_t)t * 16 + 4 * (r % 4) + lane], (two & lanes_of_sc) ? 3 : 1);
  }
}

// Step 4a: 1 where tile t starts a tile row.
__global__ void tiles_row_starts(int64_t nt, const int32_t* tile_row, int32_t* start) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x)
    start[t] = (t == 0 || tile_row[t - 1] != tile_row[t]) ? 1 : 0;
}

// Step 4b: the tile row pointer (one entry per tile row with a tile, then
// the tile count).
__global__ void tiles_rowptr(int64_t nt, const int32_t* start, const int32_t* rank, const int32_t* n_used,
                             int32_t* rowptr) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x)
    if (start[t]) rowptr[rank[t]] = (int32_t)t;
  if (blockIdx.x == 0 && threadIdx.x == 0) rowptr[*n_used] = (int32_t)nt;
}

// Step 4c: grid cells without a tile get -1 in the relative index map.
__global__ void tiles_rel_fix(int64_t cells, const int32_t* block_info, int32_t* rel_map) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += (int64_t)gridDim.x * blockDim.x)
    if (!block_info[c]) rel_map[c] = -1;
}

// Step 4d: label flags -> the 16 labels of every tile, in place.
__global__ void tiles_labels(int64_t nt, int32_t* tile_info) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nt * 16; e += (int64_t)gridDim.x * blockDim.x)
    tile_info[e] = tiles::label_of_flags(tile_info[e]);
}

}  // namespace dev
}  // namespace smat

namespace {

using smat::fail;

// Device scratch released on every exit path.
struct DevBuf {
  void* p = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes ? bytes : 16); }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
  void* release() {
    void* q = p;
    p = nullptr;
    return q;
  }
};

int grid_for(int64_t n, int sms, int threads = 256) {
  const int64_t want = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)sms * 16;
  return (int)(want < 1 ? 1 : (want > cap ? cap : want));
}

// Exclusive scan of n int32 (0/1) on the stream; *total (device) = sum.
cudaError_t exclusive_scan(const int32_t* in, int64_t n, int32_t* out, int32_t* chunk_buf, int32_t* total,
                           cudaStream_t s) {
  if (n == 0) return cudaMemsetAsync(total, 0, sizeof(int32_t), s);
  const int64_t nchunks = (n + smat::dev::kScanChunk - 1) / smat::dev::kScanChunk;
  smat::dev::scan_chunk_sums<<<(unsigned)nchunks, smat::dev::kScanThreads, 0, s>>>(in, n, chunk_buf);
  smat::dev::scan_chunk_offsets<<<1, smat::dev::kScanThreads, 0, s>>>(chunk_buf, nchunks, total);
  smat::dev::scan_chunks<<<(unsigned)nchunks, smat::dev::kScanThreads, 0, s>>>(in, n, chunk_buf, out);
  return cudaGetLastError();
}

std::string bad_text(int bad) {
  std::string m;
  if (bad & smat::tiles::BAD_ROWPTR) m += " block row pointers must start at 0, not decrease and end at nnzb;";
  if (bad & smat::tiles::BAD_COLIDX) m += " a block column start is out of range or not a multiple of block_cols;";
  if (bad & smat::tiles::BAD_ORDER) m += " block column starts must ascend within a block row;";
  return m;
}

void free_tiles(smat_tiles* t) {
  if (!t) return;
  cudaFree(t->val);
  cudaFree(t->rowptr);
  cudaFree(t->colidx);
  cudaFree(t->block_info);
  cudaFree(t->rel_map);
  cudaFree(t->tile_info);
  delete t;
}

#define TILES_CUDA(call, what)                                                                        \
  do {                                                                                                \
    const cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) {                                                                          \
      cudaGetLastError();                                                                             \
      free_tiles(res);                                                                                \
      return fail(e_ == cudaErrorMemoryAllocation ? SMAT_ERR_NOMEM : SMAT_ERR_CUDA,                   \
                  std::string("smat_tiles_create: ") + (what) + ": " + cudaGetErrorString(e_));       \
    }                                                                                                 \
  } while (0)

}  // namespace

extern "C" smat_status smat_tiles_create(int64_t rows, int64_t cols, int32_t block_cols, int64_t nnzb,
                                         const int32_t* row_ptr, const int32_t* col_idx, const void* values,
                                         void* stream, smat_tiles** out) {
  using namespace smat;
  if (!out) return fail(SMAT_ERR_INVALID, "smat_tiles_create: null output");
  *out = nullptr;
  if (block_cols != 16 && block_cols != 32)
    return fail(SMAT_ERR_UNSUPPORTED, "smat_tiles_create: block_cols must be 16 or 32");
  if (rows < 0 || cols < 0 || rows % 16 || cols % block_cols)
    return fail(SMAT_ERR_INVALID, "smat_tiles_create: rows must be a multiple of 16 and cols of block_cols");
  if (nnzb < 0 || nnzb > INT32_MAX) return fail(SMAT_ERR_INVALID, "smat_tiles_create: nnzb out of range");
  if (rows > 0 && !row_ptr) return fail(SMAT_ERR_INVALID, "smat_tiles_create: null row_ptr");
  if (nnzb > 0 && (!col_idx || !values)) return fail(SMAT_ERR_INVALID, "smat_tiles_create: null col_idx or values");
  if (nnzb > 0 && rows == 0) return fail(SMAT_ERR_INVALID, "smat_tiles_create: blocks in a matrix without rows");
  if ((uintptr_t)values % 16) return fail(SMAT_ERR_INVALID, "smat_tiles_create: values must be 16-byte aligned");
  const tiles::Geom g = tiles::make_geom(rows, cols, block_cols, nnzb);
  const int64_t cells = g.tile_rows * g.tile_cols;
  if (cells > INT32_MAX) return fail(SMAT_ERR_UNSUPPORTED, "smat_tiles_create: tile grid too large");
  const cudaStream_t s = static_cast<cudaStream_t>(stream);

  smat_tiles* res = new smat_tiles;
  res->g = g;
  TILES_CUDA(cudaGetDevice(&res->device), "cudaGetDevice");
  // the kernels dereference the three arrays: they must be device (or
  // managed) memory of the current device
  for (const void* p : {static_cast<const void*>(row_ptr), static_cast<const void*>(col_idx), values}) {
    if (!p) continue;
    cudaPointerAttributes pa{};
    const cudaError_t e = cudaPointerGetAttributes(&pa, p);
    if (e != cudaSuccess || !(pa.type == cudaMemoryTypeManaged ||
                              (pa.type == cudaMemoryTypeDevice && pa.device == res->device))) {
      cudaGetLastError();
      free_tiles(res);
      return fail(SMAT_ERR_INVALID, "smat_tiles_create: row_ptr, col_idx and values must be device memory of "
                                    "the current device");
    }
  }
  int sms = 0;
  TILES_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, res->device), "device attribute");

  // counters: [0] input faults, [1] tiles, [2] tile rows with a tile, [3] grid total
  DevBuf cnt, maker, is_maker, tile_no, brow, chunks;
  TILES_CUDA(cnt.alloc(4 * sizeof(int32_t)), "scratch");
  TILES_CUDA(cudaMemsetAsync(cnt.p, 0, 4 * sizeof(int32_t), s), "memset");
  const int64_t scan_max = nnzb > cells ? nnzb : cells;
  TILES_CUDA(chunks.alloc(sizeof(int32_t) * (size_t)((scan_max + dev::kScanChunk - 1) / dev::kScanChunk + 1)),
             "scratch");
  TILES_CUDA(maker.alloc(sizeof(int32_t) * (size_t)nnzb), "scratch");
  TILES_CUDA(is_maker.alloc(sizeof(int32_t) * (size_t)nnzb), "scratch");
  TILES_CUDA(tile_no.alloc(sizeof(int32_t) * (size_t)nnzb), "scratch");
  TILES_CUDA(brow.alloc(sizeof(int32_t) * (size_t)nnzb), "scratch");
  int32_t* c = cnt.as<int32_t>();

  // steps 1-2
  if (g.nbr > 0) {
    dev::tiles_check_rows<<<grid_for(g.nbr, sms), 256, 0, s>>>(g, row_ptr, c);
    TILES_CUDA(cudaGetLastError(), "launch");
  }
  if (nnzb > 0) {
    dev::tiles_mark<<<grid_for(nnzb, sms), 256, 0, s>>>(g, row_ptr, col_idx, c, maker.as<int32_t>(),
                                                         is_maker.as<int32_t>(), brow.as<int32_t>(), c);
    TILES_CUDA(cudaGetLastError(), "launch");
  }
  TILES_CUDA(exclusive_scan(is_maker.as<int32_t>(), nnzb, tile_no.as<int32_t>(), chunks.as<int32_t>(), c + 1, s),
             "scan");
  int32_t hc[4] = {0, 0, 0, 0};
  TILES_CUDA(cudaMemcpyAsync(hc, c, sizeof(hc), cudaMemcpyDeviceToHost, s), "copy");
  TILES_CUDA(cudaStreamSynchronize(s), "synchronize");
  if (hc[0]) {
    free_tiles(res);
    return fail(SMAT_ERR_INVALID, "smat_tiles_create:" + bad_text(hc[0]));
  }
  const int64_t nt = hc[1];
  res->n_tiles = nt;

  // outputs
  const int64_t max_rows_used = (nt < g.tile_rows ? nt : g.tile_rows);
  TILES_CUDA(cudaMalloc(&res->val, sizeof(uint16_t) * (size_t)(nt * g.tsz > 0 ? nt * g.tsz : 8)), "tile values");
  TILES_CUDA(cudaMalloc(&res->rowptr, sizeof(int32_t) * (size_t)(max_rows_used + 1)), "tile row pointer");
  TILES_CUDA(cudaMalloc(&res->colidx, sizeof(int32_t) * (size_t)(nt > 0 ? nt : 1)), "tile columns");
  TILES_CUDA(cudaMalloc(&res->block_info, sizeof(int32_t) * (size_t)(cells > 0 ? cells : 1)), "tile grid");
  TILES_CUDA(cudaMalloc(&res->rel_map, sizeof(int32_t) * (size_t)(cells > 0 ? cells : 1)), "tile map");
  TILES_CUDA(cudaMalloc(&res->tile_info, sizeof(int32_t) * (size_t)(nt > 0 ? nt * 16 : 1)), "tile labels");
  TILES_CUDA(cudaMemsetAsync(res->val, 0, sizeof(uint16_t) * (size_t)(nt * g.tsz), s), "memset");
  TILES_CUDA(cudaMemsetAsync(res->rowptr, 0, sizeof(int32_t) * (size_t)(max_rows_used + 1), s), "memset");
  TILES_CUDA(cudaMemsetAsync(res->block_info, 0, sizeof(int32_t) * (size_t)cells, s), "memset");
  TILES_CUDA(cudaMemsetAsync(res->tile_info, 0, sizeof(int32_t) * (size_t)(nt * 16), s), "memset");

  // steps 3-4
  DevBuf tile_of_block, tile_row, start, rank;
  TILES_CUDA(tile_of_block.alloc(sizeof(int32_t) * (size_t)nnzb), "scratch");
  TILES_CUDA(tile_row.alloc(sizeof(int32_t) * (size_t)nt), "scratch");
  TILES_CUDA(start.alloc(sizeof(int32_t) * (size_t)nt), "scratch");
  TILES_CUDA(rank.alloc(sizeof(int32_t) * (size_t)nt), "scratch");
  if (nnzb > 0) {
    dev::tiles_place<<<grid_for(nnzb, sms), 256, 0, s>>>(g, brow.as<int32_t>(), col_idx, maker.as<int32_t>(),
                                                          tile_no.as<int32_t>(), tile_of_block.as<int32_t>(),
                                                          res->colidx, tile_row.as<int32_t>(), res->block_info);
    dev::tiles_scatter<<<grid_for(nnzb * 32, sms), 256, 0, s>>>(g, brow.as<int32_t>(), col_idx,
                                                                 static_cast<const uint16_t*>(values),
                                                                 tile_of_block.as<int32_t>(), res->val,
                                                                 res->tile_info);
    dev::tiles_row_starts<<<grid_for(nt, sms), 256, 0, s>>>(nt, tile_row.as<int32_t>(), start.as<int32_t>());
    TILES_CUDA(cudaGetLastError(), "launch");
  }
  TILES_CUDA(exclusive_scan(start.as<int32_t>(), nt, rank.as<int32_t>(), chunks.as<int32_t>(), c + 2, s), "scan");
  if (nt > 0) {
    dev::tiles_rowptr<<<grid_for(nt, sms), 256, 0, s>>>(nt, start.as<int32_t>(), rank.as<int32_t>(), c + 2,
                                                         res->rowptr);
    TILES_CUDA(cudaGetLastError(), "launch");
  }
  TILES_CUDA(exclusive_scan(res->block_info, cells, res->rel_map, chunks.as<int32_t>(), c + 3, s), "scan");
  if (cells > 0) {
    dev::tiles_rel_fix<<<grid_for(cells, sms), 256, 0, s>>>(cells, res->block_info, res->rel_map);
    TILES_CUDA(cudaGetLastError(), "launch");
  }
  if (nt > 0) {
    dev::tiles_labels<<<grid_for(nt * 16, sms), 256, 0, s>>>(nt, res->tile_info);
    TILES_CUDA(cudaGetLastError(), "launch");
  }
  TILES_CUDA(cudaMemcpyAsync(hc, c, sizeof(hc), cudaMemcpyDeviceToHost, s), "copy");
  TILES_CUDA(cudaStreamSynchronize(s), "synchronize");
  if (hc[3] != hc[1] || hc[2] > max_rows_used) {
    free_tiles(res);
    return fail(SMAT_ERR_CUDA, "smat_tiles_create: inconsistent tile counts");
  }
  res->n_rowptr = (int64_t)hc[2] + 1;
  *out = res;
  return SMAT_OK;
}

extern "C" smat_status smat_tiles_describe(const smat_tiles* t, smat_tiles_desc* d) {
  if (!t || !d) return smat::fail(SMAT_ERR_INVALID, "smat_tiles_describe: null argument");
  d->rows = t->g.m_row;
  d->cols = t->g.m_col;
  d->block_cols = t->g.k;
  d->device = t->device;
  d->n_tiles = t->n_tiles;
  d->n_rowptr = t->n_rowptr;
  d->tile_rows = t->g.tile_rows;
  d->tile_cols = t->g.tile_cols;
  d->values = t->val;
  d->row_ptr = t->rowptr;
  d->col_idx = t->colidx;
  d->block_info = t->block_info;
  d->rel_map = t->rel_map;
  d->tile_info = t->tile_info;
  return SMAT_OK;
}

extern "C" smat_status smat_tiles_copy_to_host(const smat_tiles* t, int32_t* row_ptr, int32_t* col_idx,
                                               uint16_t* values, int32_t* block_info, int32_t* rel_map,
                                               int32_t* tile_info) {
  if (!t) return smat::fail(SMAT_ERR_INVALID, "smat_tiles_copy_to_host: null handle");
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != t->device) cudaSetDevice(t->device);
  const int64_t cells = t->g.tile_rows * t->g.tile_cols;
  struct Part {
    void* dst;
    const void* src;
    size_t bytes;
  } parts[] = {{row_ptr, t->rowptr, sizeof(int32_t) * (size_t)t->n_rowptr},
               {col_idx, t->colidx, sizeof(int32_t) * (size_t)t->n_tiles},
               {values, t->val, sizeof(uint16_t) * (size_t)(t->n_tiles * t->g.tsz)},
               {block_info, t->block_info, sizeof(int32_t) * (size_t)cells},
               {rel_map, t->rel_map, sizeof(int32_t) * (size_t)cells},
               {tile_info, t->tile_info, sizeof(int32_t) * (size_t)(t->n_tiles * 16)}};
  smat_status st = SMAT_OK;
  for (const Part& p : parts) {
    if (!p.dst || !p.bytes) continue;
    const cudaError_t e = cudaMemcpy(p.dst, p.src, p.bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      st = smat::fail(SMAT_ERR_CUDA, std::string("smat_tiles_copy_to_host: ") + cudaGetErrorString(e));
      break;
    }
  }
  if (prev >= 0 && prev != t->device) cudaSetDevice(prev);
  return st;
}

extern "C" smat_status smat_tiles_destroy(smat_tiles* t) {
  free_tiles(t);
  return SMAT_OK;
}
