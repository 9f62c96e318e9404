// Force-included into the reference's translation units by
// oracle/ref_cuda/Makefile (test infrastructure, never part of the product).
//
// The reference's BE and CN solvers (solve_bem.cu:45, solve_cnm.cu:72, 692,
// 695) multiply by their CSR matrix with cusparseCsrmvEx and
// CUSPARSE_ALG_MERGE_PATH, which cuSPARSE 12 removed.  This restates that
// call -- y = alpha * op(A) x + beta * y for a CSR matrix with 32-bit
// indices -- over the generic SpMV API that replaced it, so the reference
// sources compile unmodified with the CUDA 13 toolkit.  The merge-path
// algorithm choice has no generic counterpart; the default CSR algorithm is
// used.  The caller's work buffer (the reference passes one of ngc doubles)
// is used when large enough, else one grown on demand and kept.
#pragma once
#include <cuda_runtime.h>
#include <cusparse.h>

#ifndef CUSPARSE_ALG_MERGE_PATH
#define CUSPARSE_ALG_MERGE_PATH 1
#endif

static inline cusparseStatus_t cusparseCsrmvEx(cusparseHandle_t handle, int alg, cusparseOperation_t op, int m,
                                               int n, int nnz, const void *alpha, cudaDataType alpha_type,
                                               const cusparseMatDescr_t descr, const void *val,
                                               cudaDataType val_type, const int *row, const int *col,
                                               const void *x, cudaDataType x_type, const void *beta,
                                               cudaDataType beta_type, void *y, cudaDataType y_type,
                                               cudaDataType exec_type, void *buffer) {
  (void)alg;
  (void)alpha_type;
  (void)beta_type;
  static void *own = nullptr;
  static size_t own_bytes = 0;
  cusparseSpMatDescr_t A;
  cusparseDnVecDescr_t X, Y;
  cusparseStatus_t s =
      cusparseCreateCsr(&A, m, n, nnz, (void *)row, (void *)col, (void *)val, CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I,
                        cusparseGetMatIndexBase(descr), val_type);
  if (s != CUSPARSE_STATUS_SUCCESS) return s;
  cusparseCreateDnVec(&X, n, (void *)x, x_type);
  cusparseCreateDnVec(&Y, m, y, y_type);
  size_t bytes = 0;
  s = cusparseSpMV_bufferSize(handle, op, alpha, A, X, beta, Y, exec_type, CUSPARSE_SPMV_ALG_DEFAULT, &bytes);
  void *work = buffer;
  if (s == CUSPARSE_STATUS_SUCCESS && bytes > (size_t)m * sizeof(double)) {
    if (bytes > own_bytes) {
      if (own) cudaFree(own);
      own = nullptr;
      own_bytes = 0;
      if (cudaMalloc(&own, bytes) == cudaSuccess) own_bytes = bytes;
    }
    work = own;
  }
  if (s == CUSPARSE_STATUS_SUCCESS) s = cusparseSpMV(handle, op, alpha, A, X, beta, Y, exec_type,
                                                     CUSPARSE_SPMV_ALG_DEFAULT, work);
  cusparseDestroyDnVec(Y);
  cusparseDestroyDnVec(X);
  cusparseDestroySpMat(A);
  return s;
}
