/*
 * smat_ref_shims.h — the reference's kernel launchers, with the reference's
 * own names and C++ signatures (src/cuda_hgemm/src/main.cu:10-75), exported
 * by libsmat so that the reference harness (main.cu + tester.h) links
 * against it unchanged. Each one replaces the reference definition named
 * beside it. All pointers are device pointers; B is K x N column-major
 * FP16, C is M x N row-major FP16 (the reference's layouts).
 *
 * The first call for a matrix copies its BCSR arrays to the host and builds
 * a libsmat handle, cached on the device, M, K, the block count and each
 * array's address and allocation (buffer ID): arrays freed and allocated
 * again are a new matrix, even at the same addresses, but contents rewritten
 * in place are not noticed, so do not rewrite a cached matrix's arrays
 * (smat_ref_shims_release() drops the cache). Calls run on the legacy
 * default stream and return nothing; smat_ref_shims_last_status() reports
 * the last call's status. The packed B goes to the library's static scratch
 * when it fits (SMAT_SPMM_STATIC_SCRATCH_BYTES), else to a workspace kept
 * with the cached handle and allocated by the first call that needs it.
 */
#ifndef SMAT_REF_SHIMS_H_
#define SMAT_REF_SHIMS_H_

#include <cuda_fp16.h>
#include <stddef.h>

#include "smat.h"

#ifdef __cplusplus
/* mmaOBT.cu:160-169 (HGEMM_FUNC_SPARSE2): 16 x 16 blocks. */
void mmaOBTKernel(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, half* B, half* C, size_t M, size_t N,
                  size_t K, size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping);
/* mmaOBT_large.cu (HGEMM_FUNC_SPARSE2): 16 x 32 blocks. */
void mmaOBTKernel_large(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, half* B, half* C, size_t M,
                        size_t N, size_t K, size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping);
/* mmaOBTS.cu (HGEMM_FUNC_SPARSE24_2): mixed dense / 2:4, 16 x 16 blocks; the
 * product is computed from bcsrValuesA, metadata and sparseMatrixA are not read. */
void mmaOBTSKernel(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, char* metadata, half* sparseMatrixA,
                   half* B, half* C, size_t M, size_t N, size_t K, size_t nonzeroBlocks, int* blockInfo,
                   int* relativeBlockIndexMapping);
/* mmaOBTS_large.cu:256-266 (HGEMM_FUNC_SPARSE24_2): the same with 16 x 32 blocks. */
void mmaOBTSKernel_large(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, char* metadata, half* sparseMatrixA,
                         half* B, half* C, size_t M, size_t N, size_t K, size_t nonzeroBlocks, int* blockInfo,
                         int* relativeBlockIndexMapping);
/* mmaOBTS_large_separate.cu:262-280 (HGEMM_FUNC_SPLIT): the 2:4 and dense
 * parts of filterBcsrBlocks (matrix.h:1140-1288) as two 16 x 32 BCSRs. */
void mmaOBTSKernel_large_separate(half* bcsrValuesA_sparse, int* bcsrRowPtrA_sparse, int* bcsrColIdxA_sparse,
                                  half* bcsrValuesA_dense, int* bcsrRowPtrA_dense, int* bcsrColIdxA_dense,
                                  char* metadata, half* sparseMatrixA, half* B, half* C, size_t M, size_t N, size_t K,
                                  size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping);
/* mmaOBT_tiled.cu:208-217 (HGEMM_FUNC_SPARSE2, main.cu:55): the matrix as
 * the merged 4 x 4-block tiles of SparseMatrix::bcsrBlocking (matrix.h:
 * 794-1137; built on the GPU by smat_tiles_create), 16 x 16 blocks:
 * bcsrValuesA / bcsrRowPtrA / bcsrColIdxA are the merged values, tile row
 * pointer and tile column starts, blockInfo the merged tile grid
 * (required: it sizes the arrays); nonzeroBlocks only keys the cache. Each
 * tile's values are read at its own position in the arrays. */
void mmaOBTKernel_tiled(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, half* B, half* C, size_t M, size_t N,
                        size_t K, size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping);
/* mmaOBTS_tiled_large.cu:431-451 (HGEMM_FUNC_SPARSE24_2_tiled, main.cu:58):
 * the same for tiles of 16 x 32 blocks; metadata, sparseMatrixA and
 * tileInfo are not read (the product comes from the merged values). */
void mmaOBTSKernel_tiled_large(half* bcsrValuesA, int* bcsrRowPtrA, int* bcsrColIdxA, char* metadata,
                               half* sparseMatrixA, half* B, half* C, size_t M, size_t N, size_t K,
                               size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping, int* tileInfo);
/* mmaST.cu:22-140 launcher (main.cu:60-63): the reference's 2:4 compression
 * of the blocks blockInfo marks 1, into its own metadata / value layout. */
void preprocessing_mmaSTKernel(half* bcsrValuesA, char* metadata, half* sparseMatrixA, size_t M, size_t N, size_t K,
                               size_t nonzeroBlocks, int* blockInfo, int* relativeBlockIndexMapping);
/* mmaST_large.cu:22-152 launcher :324-335 (main.cu:64-68): the same for 16 x 32
 * blocks (two metadata bytes and eight values per lane); the launcher that
 * main.cu:306-311 hands to evaluateSparse24_2 and evaluateSplit. */
void preprocessing_mmaSTKernel_large(half* bcsrValuesA, char* metadata, half* sparseMatrixA, size_t M, size_t N,
                                     size_t K, size_t nonzeroBlocks, int* blockInfo,
                                     int* relativeBlockIndexMapping);
#endif

#ifdef __cplusplus
extern "C" {
#endif
/* Status of the last shim call (SMAT_OK if none failed). No counterpart in
 * the reference, whose launchers report nothing. */
smat_status smat_ref_shims_last_status(void);
/* Destroys the handles the shims cached. No counterpart in the reference. */
smat_status smat_ref_shims_release(void);
#ifdef __cplusplus
}
#endif
#endif /* SMAT_REF_SHIMS_H_ */
