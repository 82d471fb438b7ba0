// ref_shims.cu — the reference's kernel launchers, by their own names and
// signatures (C++ linkage, src/cuda_hgemm/src/main.cu:10-75), backed by
// libsmat, so that the reference harness (main.cu + tester.h) links against
// this library unchanged.
//
// The launchers receive device pointers to a BCSR matrix (values FP16
// row-major per block, row pointers, column starts), B (K x N, column-major
// FP16) and C (M x N, row-major FP16) and return nothing. The first call for
// a given matrix copies the BCSR to the host and builds a libsmat handle;
// later calls reuse it. The cache is keyed on the device, M, K, the block
// count and, for every array, its address and the allocation's buffer ID
// (CU_POINTER_ATTRIBUTE_BUFFER_ID, unique within the process): a matrix
// freed and allocated again, even at the same addresses, is a new entry.
// Contents changed in place are not detected, so the arrays must not be
// rewritten while cached (the reference's SparseMatrix never rewrites
// them); smat_ref_shims_release() drops every cached handle. Every call
// then runs the SpMM on the legacy default stream, like the reference
// launchers: through smat_spmm_static_scratch when the packed B fits its
// fixed array (nothing allocated), else with a workspace kept beside the
// cached handle, allocated on the first call that needs it (the stencil
// shape, K = 262144 at N = 256, needs 128 MiB).
//
// The `_tiled` launchers take the merged 4 x 4-block tiles of bcsrBlocking
// (see entry_for_tiled) and compute from their values in the same way.
//
// The 2:4 variants take the reference's compressed values and metadata, but
// compute from the uncompressed block values (which hold every block), so the
// result does not depend on how the reference's blockInfo heuristic labelled
// a block. The preprocessing launchers write the reference's compressed
// format (see spmm_24ref.cu).
//
// Errors cannot be returned through these signatures: the status of the last
// shim call is kept (smat_ref_shims_last_status) and the message in
// smat_last_error().
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "smat_internal.h"
#include "smat_ref_shims.h"

namespace {

// (device, M, K, block count, block width, then address and buffer ID of
// each array: values, row pointers, column starts, and the same three of the
// dense part and the relative block index map for the separate variant)
using Key = std::tuple<int, size_t, size_t, size_t, int, std::array<uint64_t, 14>>;

struct Entry {
  smat_bcsr* h = nullptr;
  void* ws = nullptr;  // workspace for packed B beyond the static scratch (device)
  size_t ws_bytes = 0;
};

std::mutex g_mu;
std::map<Key, Entry> g_cache;
smat_status g_last = SMAT_OK;

// Unique ID of the allocation holding p (0 when the driver knows none).
uint64_t buffer_id(const void* p) {
  using PointerGetAttribute = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);
  static const auto get_attr = reinterpret_cast<PointerGetAttribute>(smat::driver_fn("cuPointerGetAttribute"));
  unsigned long long id = 0;
  if (!p || !get_attr || get_attr(&id, CU_POINTER_ATTRIBUTE_BUFFER_ID, (CUdeviceptr)(uintptr_t)p) != CUDA_SUCCESS)
    return 0;
  return (uint64_t)id;
}

Key make_key(int dev, size_t M, size_t K, size_t nnzb, int bw, std::initializer_list<const void*> arrays) {
  std::array<uint64_t, 14> a{};
  size_t i = 0;
  for (const void* p : arrays) {
    a[i++] = (uint64_t)(uintptr_t)p;
    a[i++] = buffer_id(p);
  }
  return Key{dev, M, K, nnzb, bw, a};
}

// The SpMM of a cached entry on the legacy default stream: the static
// scratch when it is large enough, else the entry's own workspace.
smat_status spmm_entry(Entry& e, const half* B, half* C, size_t N, size_t K) {
  size_t need = 0;
  smat_status st = smat_spmm_workspace_size(e.h, SMAT_FORM_F16, SMAT_F16, (int64_t)N, &need);
  if (st != SMAT_OK) return st;
  if (need <= (size_t)SMAT_SPMM_STATIC_SCRATCH_BYTES)
    return smat_spmm_static_scratch(e.h, SMAT_FORM_F16, B, SMAT_F16, SMAT_COL_MAJOR, (int64_t)K, C, SMAT_F16,
                                    (int64_t)N, (int64_t)N, nullptr);
  if (need > e.ws_bytes) {
    if (e.ws) cudaFree(e.ws);
    e.ws = nullptr;
    e.ws_bytes = 0;
    if (cudaMalloc(&e.ws, need) != cudaSuccess) {
      cudaGetLastError();
      return smat::fail(SMAT_ERR_NOMEM, "workspace for the packed B: cudaMalloc failed");
    }
    e.ws_bytes = need;
  }
  return smat_spmm(e.h, SMAT_FORM_F16, B, SMAT_F16, SMAT_COL_MAJOR, (int64_t)K, C, SMAT_F16, (int64_t)N, (int64_t)N,
                   e.ws, e.ws_bytes, nullptr);
}

// Cache entry for a device BCSR (16 x bw blocks), built on first sight.
smat_status entry_for(const half* vals, const int* rowptr, const int* colidx, size_t M, size_t K, size_t nnzb,
                      int bw, Entry** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return smat::fail(SMAT_ERR_CUDA, "cudaGetDevice failed");
  const Key key = make_key(dev, M, K, nnzb, bw, {vals, rowptr, colidx});
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_cache.find(key);
  if (it != g_cache.end()) {
    *out = &it->second;
    return SMAT_OK;
  }
  if (M % 16 || K % bw) return smat::fail(SMAT_ERR_INVALID, "M and K must be multiples of the block shape");
  const size_t nbr = M / 16;
  std::vector<int32_t> rp(nbr + 1), ci(nnzb);
  std::vector<uint16_t> v(nnzb * 16 * bw);
  if (cudaMemcpy(rp.data(), rowptr, rp.size() * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
      (nnzb && cudaMemcpy(ci.data(), colidx, ci.size() * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) ||
      (nnzb && cudaMemcpy(v.data(), vals, v.size() * sizeof(uint16_t), cudaMemcpyDeviceToHost) != cudaSuccess))
    return smat::fail(SMAT_ERR_CUDA, "copying the BCSR arrays to the host failed");
  smat_bcsr_opts o{};
  o.device = dev;
  smat_bcsr* h = nullptr;
  smat_status st = smat_bcsr_create_from_bcsr((int64_t)M, (int64_t)K, 16, bw, (int64_t)nnzb, rp.data(), ci.data(),
                                              v.data(), &o, &h);
  if (st != SMAT_OK) return st;
  Entry& e = g_cache[key];
  e.h = h;
  *out = &e;
  return SMAT_OK;
}

void run(const half* vals, const int* rowptr, const int* colidx, const half* B, half* C, size_t M, size_t N, size_t K,
         size_t nnzb, int bw) {
  Entry* e = nullptr;
  smat_status st = entry_for(vals, rowptr, colidx, M, K, nnzb, bw, &e);
  if (st == SMAT_OK) {
    std::lock_guard<std::mutex> lock(g_mu);
    st = spmm_entry(*e, B, C, N, K);
  }
  std::lock_guard<std::mutex> lock(g_mu);
  g_last = st;
}

// Merges two BCSRs with the same block shape (the 2:4 part and the dense part
// of filterBcsrBlocks, matrix.h:1140-1288) into one, per block row in column
// order, and runs it. Where a block's values are: with a relative block
// index map (the reference harness, tester.h:554-590, passes the full BCSR's
// values for both parts and its map), block (r, c) is at
// vs[rel[r * K/bw + c/bw]], as the reference kernel reads it
// (mmaOBTS_large_separate.cu:156-186); without one (rel == nullptr), each
// part's k-th block is at its own values array's k-th block.
void run_separate(const half* vs, const int* rps, const int* cis, const half* vd, const int* rpd, const int* cid,
                  const half* B, half* C, size_t M, size_t N, size_t K, size_t nnzb_full, const int* rel, int bw) {
  smat_status st = SMAT_OK;
  int dev = 0;
  cudaGetDevice(&dev);
  // the merged matrix is keyed on both parts' arrays and the map (block
  // count: the full BCSR's with a map, else 0: the parts' counts are in
  // their row pointers)
  const Key key = make_key(dev, M, K, rel ? nnzb_full : 0, bw, {vs, rps, cis, vd, rpd, cid, rel});
  Entry* e = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) e = &it->second;
  }
  if (!e) {
    const size_t nbr = M / 16, bsz = 16 * (size_t)bw;
    std::vector<int32_t> rp[2] = {std::vector<int32_t>(nbr + 1), std::vector<int32_t>(nbr + 1)};
    const int* rpp[2] = {rps, rpd};
    const int* cip[2] = {cis, cid};
    const half* vp[2] = {vs, vd};
    std::vector<int32_t> ci[2];
    std::vector<uint16_t> v[2];
    std::vector<int32_t> relh;  // the relative block index map, when given
    const size_t ncb = bw > 0 ? K / (size_t)bw : 0;
    if (M % 16 || K % bw) st = smat::fail(SMAT_ERR_INVALID, "M and K must be multiples of the block shape");
    if (st == SMAT_OK && rel) {
      // with a map both parts read the first values array (the full BCSR)
      relh.resize(nbr * ncb);
      v[0].resize(nnzb_full * bsz);
      if ((!relh.empty() &&
           cudaMemcpy(relh.data(), rel, relh.size() * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) ||
          (nnzb_full &&
           cudaMemcpy(v[0].data(), vs, v[0].size() * sizeof(uint16_t), cudaMemcpyDeviceToHost) != cudaSuccess))
        st = smat::fail(SMAT_ERR_CUDA, "copying the block map or values failed");
    }
    for (int p = 0; p < 2 && st == SMAT_OK; p++) {
      if (cudaMemcpy(rp[p].data(), rpp[p], (nbr + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) {
        st = smat::fail(SMAT_ERR_CUDA, "copying row pointers failed");
        break;
      }
      const size_t nb = (size_t)rp[p][nbr];
      ci[p].resize(nb);
      if (nb && cudaMemcpy(ci[p].data(), cip[p], nb * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) {
        st = smat::fail(SMAT_ERR_CUDA, "copying BCSR arrays failed");
        break;
      }
      if (rel) continue;
      v[p].resize(nb * bsz);
      if (nb && cudaMemcpy(v[p].data(), vp[p], nb * bsz * sizeof(uint16_t), cudaMemcpyDeviceToHost) != cudaSuccess)
        st = smat::fail(SMAT_ERR_CUDA, "copying BCSR arrays failed");
    }
    if (st == SMAT_OK) {
      std::vector<int32_t> mrp(nbr + 1, 0), mci;
      std::vector<uint16_t> mv;
      for (size_t r = 0; r < nbr; r++) {
        int32_t a = rp[0][r], b = rp[1][r];
        while (a < rp[0][r + 1] || b < rp[1][r + 1]) {
          const bool take_a = b >= rp[1][r + 1] || (a < rp[0][r + 1] && ci[0][a] < ci[1][b]);
          const int p = take_a ? 0 : 1;
          const int32_t k = take_a ? a++ : b++;
          if (!mci.empty() && (int64_t)mci.size() > mrp[r] && mci.back() == ci[p][k]) {
            st = smat::fail(SMAT_ERR_INVALID, "a block appears in both parts");
            break;
          }
          mci.push_back(ci[p][k]);
          size_t src = (size_t)k;  // block index in the values array it comes from
          const std::vector<uint16_t>* vv = &v[p];
          if (rel) {
            const int64_t col = ci[p][k];
            const int64_t ri = col >= 0 && (size_t)col < K ? relh[r * ncb + (size_t)col / bw] : -1;
            if (ri < 0 || (size_t)ri >= nnzb_full) {
              st = smat::fail(SMAT_ERR_INVALID, "a block of a part is not in the relative block index map");
              break;
            }
            src = (size_t)ri;
            vv = &v[0];
          }
          mv.insert(mv.end(), vv->begin() + src * bsz, vv->begin() + (src + 1) * bsz);
        }
        mrp[r + 1] = (int32_t)mci.size();
        if (st != SMAT_OK) break;
      }
      if (st == SMAT_OK) {
        smat_bcsr_opts o{};
        o.device = dev;
        smat_bcsr* h = nullptr;
        st = smat_bcsr_create_from_bcsr((int64_t)M, (int64_t)K, 16, bw, (int64_t)mci.size(), mrp.data(), mci.data(),
                                        mv.data(), &o, &h);
        if (st == SMAT_OK) {
          std::lock_guard<std::mutex> lock(g_mu);
          e = &g_cache[key];
          e->h = h;
        }
      }
    }
  }
  if (st == SMAT_OK) {
    std::lock_guard<std::mutex> lock(g_mu);
    st = spmm_entry(*e, B, C, N, K);
  }
  std::lock_guard<std::mutex> lock(g_mu);
  g_last = st;
}

// Cache entry for a matrix given as the reference's merged 4 x 4-block tiles
// (SparseMatrix::bcsrBlocking, matrix.h:794-1137; built here by
// smat_tiles_create): the tiles are taken apart into their 16 x bw blocks on
// the host and the blocks holding any nonzero bit become a BCSR handle. The
// tile grid (the launchers' blockInfo argument, mergedBlockInfo) gives the
// array sizes and which tile rows the row pointer's entries belong to (it has
// entries only for tile rows holding a tile). Each tile's values are read at
// its own position in the arrays, so the product is the one the arrays
// describe; the reference's kernels read a tile's values at its rank in grid
// order (rel_map), which is the same place whenever a tile row's tiles were
// first met in column order and no tile row is empty.
smat_status entry_for_tiled(const half* vals, const int* rowptr, const int* colidx, const int* grid, size_t M,
                            size_t K, size_t nnzb, int bw, Entry** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return smat::fail(SMAT_ERR_CUDA, "cudaGetDevice failed");
  if (!grid) return smat::fail(SMAT_ERR_INVALID, "the tiled launchers need the merged tile grid (blockInfo)");
  if (M % 16 || K % bw) return smat::fail(SMAT_ERR_INVALID, "M and K must be multiples of the block shape");
  // the block width's bit 8 keeps these entries apart from plain BCSRs at the same addresses
  const Key key = make_key(dev, M, K, nnzb, bw | 0x100, {vals, rowptr, colidx, grid});
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_cache.find(key);
  if (it != g_cache.end()) {
    *out = &it->second;
    return SMAT_OK;
  }
  const size_t tw = 4 * (size_t)bw, tsz = 256 * (size_t)bw, nbr = M / 16;
  const size_t nrr = (M + 63) / 64, ncr = (K + tw - 1) / tw;
  std::vector<int32_t> g(nrr * ncr);
  if (!g.empty() && cudaMemcpy(g.data(), grid, g.size() * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
    return smat::fail(SMAT_ERR_CUDA, "copying the tile grid failed");
  std::vector<size_t> used;  // tile rows holding a tile, ascending
  size_t nt = 0;
  for (size_t y = 0; y < nrr; y++) {
    size_t n = 0;
    for (size_t x = 0; x < ncr; x++) n += g[y * ncr + x] != 0;
    if (n) used.push_back(y);
    nt += n;
  }
  std::vector<int32_t> rp(used.size() + 1), ci(nt);
  std::vector<uint16_t> v(nt * tsz);
  if (cudaMemcpy(rp.data(), rowptr, rp.size() * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
      (nt && cudaMemcpy(ci.data(), colidx, ci.size() * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) ||
      (nt && cudaMemcpy(v.data(), vals, v.size() * sizeof(uint16_t), cudaMemcpyDeviceToHost) != cudaSuccess))
    return smat::fail(SMAT_ERR_CUDA, "copying the merged tile arrays to the host failed");
  if (rp[0] != 0 || (size_t)rp.back() != nt)
    return smat::fail(SMAT_ERR_INVALID, "merged tile row pointer does not match the tile grid");
  std::vector<std::vector<std::pair<int32_t, size_t>>> rows(nbr);  // per block row: (column, source offset)
  for (size_t j = 0; j < used.size(); j++) {
    if (rp[j] > rp[j + 1]) return smat::fail(SMAT_ERR_INVALID, "merged tile row pointer decreases");
    for (int32_t t = rp[j]; t < rp[j + 1]; t++) {
      const int64_t x0 = ci[t];
      if (x0 < 0 || x0 % (int64_t)tw || (size_t)(x0 / tw) >= ncr || !g[used[j] * ncr + (size_t)(x0 / tw)])
        return smat::fail(SMAT_ERR_INVALID, "a merged tile's column is not in the tile grid");
      for (size_t by = 0; by < 4; by++)
        for (size_t bx = 0; bx < 4; bx++) {
          const size_t off = (size_t)t * tsz + 16 * (size_t)bw * (4 * by + bx);
          bool any = false;
          for (size_t e = 0; e < 16 * (size_t)bw && !any; e++) any = v[off + e] != 0;
          if (!any) continue;
          const size_t br = 4 * used[j] + by;
          if (br >= nbr || (size_t)x0 + bx * bw >= K)
            return smat::fail(SMAT_ERR_INVALID, "a merged tile holds values outside the matrix");
          rows[br].push_back({(int32_t)(x0 + bx * bw), off});
        }
    }
  }
  std::vector<int32_t> brp(nbr + 1, 0), bci;
  std::vector<uint16_t> bv;
  for (size_t r = 0; r < nbr; r++) {
    std::sort(rows[r].begin(), rows[r].end());
    for (const auto& b : rows[r]) {
      bci.push_back(b.first);
      bv.insert(bv.end(), v.begin() + b.second, v.begin() + b.second + 16 * (size_t)bw);
    }
    brp[r + 1] = (int32_t)bci.size();
  }
  smat_bcsr_opts o{};
  o.device = dev;
  smat_bcsr* h = nullptr;
  smat_status st = smat_bcsr_create_from_bcsr((int64_t)M, (int64_t)K, 16, bw, (int64_t)bci.size(), brp.data(),
                                              bci.data(), bv.data(), &o, &h);
  if (st != SMAT_OK) return st;
  Entry& e = g_cache[key];
  e.h = h;
  *out = &e;
  return SMAT_OK;
}

void run_tiled(const half* vals, const int* rowptr, const int* colidx, const int* grid, const half* B, half* C,
               size_t M, size_t N, size_t K, size_t nnzb, int bw) {
  Entry* e = nullptr;
  smat_status st = entry_for_tiled(vals, rowptr, colidx, grid, M, K, nnzb, bw, &e);
  if (st == SMAT_OK) {
    std::lock_guard<std::mutex> lock(g_mu);
    st = spmm_entry(*e, B, C, N, K);
  }
  std::lock_guard<std::mutex> lock(g_mu);
  g_last = st;
}

}  // namespace

// ---------------------------------------------------------------- launchers

void mmaOBTKernel(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, half* B, half* C, size_t M, size_t N,
                  size_t K, size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping) {
  (void)blockInfo;
  (void)relativeBlockIndexMapping;
  run(bcsrValuesA, bcsrRowPtrA, bcsrColIdxA, B, C, M, N, K, nonzeroBlocks, 16);
}

void mmaOBTKernel_large(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, half* B, half* C, size_t M,
                        size_t N, size_t K, size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping) {
  (void)blockInfo;
  (void)relativeBlockIndexMapping;
  run(bcsrValuesA, bcsrRowPtrA, bcsrColIdxA, B, C, M, N, K, nonzeroBlocks, 32);
}

void mmaOBTSKernel(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, char* metadata, half* sparseMatrixA,
                   half* B, half* C, size_t M, size_t N, size_t K, size_t nonzeroBlocks, int* blockInfo,
                   int* relativeBlockIndexMapping) {
  (void)metadata;
  (void)sparseMatrixA;
  (void)blockInfo;
  (void)relativeBlockIndexMapping;
  run(bcsrValuesA, bcsrRowPtrA, bcsrColIdxA, B, C, M, N, K, nonzeroBlocks, 16);
}

void mmaOBTSKernel_large(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, char* metadata, half* sparseMatrixA,
                         half* B, half* C, size_t M, size_t N, size_t K, size_t nonzeroBlocks, int* blockInfo,
                         int* relativeBlockIndexMapping) {
  (void)metadata;
  (void)sparseMatrixA;
  (void)blockInfo;
  (void)relativeBlockIndexMapping;
  run(bcsrValuesA, bcsrRowPtrA, bcsrColIdxA, B, C, M, N, K, nonzeroBlocks, 32);
}

void mmaOBTSKernel_large_separate(half* bcsrValuesA_sparse, int* bcsrRowPtrA_sparse, int* bcsrColIdxA_sparse,
                                  half* bcsrValuesA_dense, int* bcsrRowPtrA_dense, int* bcsrColIdxA_dense,
                                  char* metadata, half* sparseMatrixA, half* B, half* C, size_t M, size_t N, size_t K,
                                  size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping) {
  (void)metadata;
  (void)sparseMatrixA;
  (void)blockInfo;
  run_separate(bcsrValuesA_sparse, bcsrRowPtrA_sparse, bcsrColIdxA_sparse, bcsrValuesA_dense, bcsrRowPtrA_dense,
               bcsrColIdxA_dense, B, C, M, N, K, nonzeroBlocks, relativeBlockIndexMapping, 32);
}

void mmaOBTKernel_tiled(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, half* B, half* C, size_t M, size_t N,
                        size_t K, size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping) {
  (void)relativeBlockIndexMapping;
  run_tiled(bcsrValuesA, bcsrRowPtrA, bcsrColIdxA, blockInfo, B, C, M, N, K, nonzeroBlocks, 16);
}

void mmaOBTSKernel_tiled_large(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, char* metadata,
                               half* sparseMatrixA, half* B, half* C, size_t M, size_t N, size_t K,
                               size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping, int* tileInfo) {
  (void)metadata;
  (void)sparseMatrixA;
  (void)relativeBlockIndexMapping;
  (void)tileInfo;
  run_tiled(bcsrValuesA, bcsrRowPtrA, bcsrColIdxA, blockInfo, B, C, M, N, K, nonzeroBlocks, 32);
}

// ---------------------------------------------------------------- C helpers

extern "C" smat_status smat_ref_shims_last_status(void) {
  std::lock_guard<std::mutex> lock(g_mu);
  return g_last;
}

extern "C" smat_status smat_ref_shims_release(void) {
  std::lock_guard<std::mutex> lock(g_mu);
  for (auto& kv : g_cache) {
    if (kv.second.ws) cudaFree(kv.second.ws);
    smat_bcsr_destroy(kv.second.h);
  }
  g_cache.clear();
  return SMAT_OK;
}
