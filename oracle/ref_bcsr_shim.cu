// ref_bcsr_shim.cu — TEST INFRASTRUCTURE ONLY.
//
// A C-ABI wrapper that runs the reference's own CSR->BCSR conversion,
// SparseMatrix::csrToBcsr (src/cuda_hgemm/src/common/matrix.h:666-792), and
// its MatrixMarket reader mmio_allinone (mmio_highlevel.h:523-680), and its
// 4 x 4-block tile merge, SparseMatrix::bcsrBlocking (matrix.h:794-1137), on
// the CPU. Compiled by oracle/Makefile straight from the reference headers into
// oracle/_ref/libsmat_ref_bcsr.so. The SparseMatrix constructor allocates
// device memory, so the object is laid out by hand and only csrToBcsr() and
// bcsrBlocking() are called; private members are opened for that purpose.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

// SparseMatrix::bcsrBlocking() (matrix.h:794-1137) ends by copying its
// results to the device. To run it on the CPU, this translation unit points
// those two calls at host memory; the *_dev arrays it makes are then host
// copies, released by ref_tiles_free.
template <class T>
static cudaError_t ref_host_malloc(T** p, size_t n) {
  *p = static_cast<T*>(std::malloc(n ? n : 1));
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
static cudaError_t ref_host_memcpy(void* dst, const void* src, size_t n, cudaMemcpyKind) {
  std::memcpy(dst, src, n);
  return cudaSuccess;
}
#define cudaMalloc ref_host_malloc
#define cudaMemcpy ref_host_memcpy

#define private public
#include "matrix.h"
#undef private
#undef cudaMalloc
#undef cudaMemcpy

extern "C" {

struct ref_bcsr {
  int64_t nnzb;
  int64_t grid;
  int32_t* rowptr;
  int32_t* colidx;
  uint16_t* val;
  int32_t* block_info;
  int32_t* rel_map;
};

// Inputs: padded m_row (multiple of 16) x m_col (multiple of k) CSR with fp16
// values given as bit patterns.
ref_bcsr* ref_csr_to_bcsr(int64_t m_row, int64_t m_col, int k, int64_t nnz, const int32_t* rowptr,
                          const int32_t* colidx, const uint16_t* val) {
  void* mem = std::calloc(1, sizeof(SparseMatrix));
  SparseMatrix* sm = reinterpret_cast<SparseMatrix*>(mem);
  sm->m_row = m_row;
  sm->m_col = m_col;
  sm->nnz = nnz;
  sm->mMMA_K = k;
  sm->csrRowPtr_host = const_cast<int*>(rowptr);
  sm->csrColIdx_host = const_cast<int*>(colidx);
  sm->csrVal_host = reinterpret_cast<half*>(const_cast<uint16_t*>(val));
  sm->csrToBcsr();
  ref_bcsr* out = new ref_bcsr;
  out->nnzb = sm->nonzeroBlocks;
  out->grid = sm->numberOfBlocks;
  out->rowptr = sm->bcsrRowPtr_host;
  out->colidx = sm->bcsrColIdx_host;
  out->val = reinterpret_cast<uint16_t*>(sm->bcsrVal_host);
  out->block_info = sm->blockInfo_host;
  out->rel_map = sm->relativeBlockIndexMapping_host;
  std::free(mem);
  return out;
}

void ref_bcsr_free(ref_bcsr* b) {
  std::free(b->rowptr);
  std::free(b->colidx);
  std::free(b->val);
  std::free(b->block_info);
  std::free(b->rel_map);
  delete b;
}

// mmio_allinone on a .mtx file: padded sizes, CSR in file order, fp16 values.
// Returns 0 on success; the arrays are malloc'ed and released by ref_free.
int ref_read_mtx(const char* path, int k, int64_t* m, int64_t* n, int64_t* nnz, int* symmetric,
                 int32_t** rowptr, int32_t** colidx, uint16_t** val) {
  size_t mm = 0, nn = 0, zz = 0;
  int sym = 0;
  int* rp = nullptr;
  int* ci = nullptr;
  half* v = nullptr;
  int rc = mmio_allinone(&mm, &nn, &zz, &sym, &rp, &ci, &v, const_cast<char*>(path), k);
  if (rc != 0) return rc;
  *m = (int64_t)mm;
  *n = (int64_t)nn;
  *nnz = (int64_t)zz;
  *symmetric = sym;
  *rowptr = rp;
  *colidx = ci;
  *val = reinterpret_cast<uint16_t*>(v);
  return 0;
}

void ref_free(void* p) { std::free(p); }

struct ref_tiles {
  int64_t ntiles;
  int64_t n_rowptr;
  int64_t grid;
  int32_t* rowptr;
  int32_t* colidx;
  uint16_t* val;
  int32_t* block_info;
  int32_t* rel_map;
  int32_t* tile_info;
};

// SparseMatrix::bcsrBlocking on a BCSR as csrToBcsr leaves it (16 x k
// blocks, column starts, values row-major per block). The merged row
// pointer's length is not kept by the reference; it is the number of tile
// rows holding a tile, plus one (matrix.h:932-958).
ref_tiles* ref_bcsr_blocking(int64_t m_row, int64_t m_col, int k, int64_t nnzb, const int32_t* brp,
                             const int32_t* bci, const uint16_t* bval) {
  void* mem = std::calloc(1, sizeof(SparseMatrix));
  SparseMatrix* sm = reinterpret_cast<SparseMatrix*>(mem);
  sm->m_row = m_row;
  sm->m_col = m_col;
  sm->mMMA_K = k;
  sm->nonzeroBlocks = nnzb;
  sm->bcsrRowPtr_host = const_cast<int*>(brp);
  sm->bcsrColIdx_host = const_cast<int*>(bci);
  sm->bcsrVal_host = reinterpret_cast<half*>(const_cast<uint16_t*>(bval));
  sm->bcsrBlocking();
  const int64_t ncr = (m_col + 4 * k - 1) / (4 * k), nrr = (m_row + 63) / 64;
  ref_tiles* out = new ref_tiles;
  out->ntiles = sm->mergedNonzeroBlocks;
  out->grid = ncr * nrr;
  int64_t rows_used = 0;
  for (int64_t y = 0; y < nrr; y++) {
    bool any = false;
    for (int64_t x = 0; x < ncr; x++) any = any || sm->mergedBlockInfo_host[y * ncr + x] != 0;
    rows_used += any;
  }
  out->n_rowptr = rows_used + 1;
  out->rowptr = sm->mergedBcsrRowPtr_host;
  out->colidx = sm->mergedBcsrColIdx_host;
  out->val = reinterpret_cast<uint16_t*>(sm->mergedBcsrVal_host);
  out->block_info = sm->mergedBlockInfo_host;
  out->rel_map = sm->mergedRelativeBlockIndexMapping_host;
  out->tile_info = sm->mergedTileInfo_host;
  std::free(sm->mergedBcsrVal_dev);
  std::free(sm->mergedBcsrRowPtr_dev);
  std::free(sm->mergedBcsrColIdx_dev);
  std::free(sm->mergedBlockInfo_dev);
  std::free(sm->mergedRelativeBlockIndexMapping_dev);
  std::free(sm->mergedTileInfo_dev);
  std::free(mem);
  return out;
}

void ref_tiles_free(ref_tiles* t) {
  std::free(t->rowptr);
  std::free(t->colidx);
  std::free(t->val);
  std::free(t->block_info);
  std::free(t->rel_map);
  std::free(t->tile_info);
  delete t;
}

}  // extern "C"
