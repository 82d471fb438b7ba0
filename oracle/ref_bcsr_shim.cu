// ref_bcsr_shim.cu — TEST INFRASTRUCTURE ONLY.
//
// A C-ABI wrapper that runs the reference's own CSR->BCSR conversion,
// SparseMatrix::csrToBcsr (src/cuda_hgemm/src/common/matrix.h:666-792), and
// its MatrixMarket reader mmio_allinone (mmio_highlevel.h:523-680), on the
// CPU. Compiled by oracle/Makefile straight from the reference headers into
// oracle/_ref/libsmat_ref_bcsr.so. The SparseMatrix constructor allocates
// device memory, so the object is laid out by hand and only the host-only
// member csrToBcsr() is called; private members are opened for that purpose.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>

#define private public
#include "matrix.h"
#undef private

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

}  // extern "C"
