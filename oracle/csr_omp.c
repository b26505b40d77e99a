/*
 * ORACLE (test infrastructure only): y = A x for a CSR matrix on all host threads (OpenMP).
 *
 * The CPU baseline times the oracle's MG-PCG / Patera solve with its sparse products here; the
 * reference's own product (mgpcg_solver_p.m:728-733 -> MUTILS spmv) is multi-threaded the same way.
 * Each row is summed in index order with separate multiply and add (built with
 * -ffp-contract=off): the same sums as scipy's serial CSR product, bit-identical to it where the
 * host compiler does not fuse scipy's multiply-adds (x86-64) and equal to rounding elsewhere.
 */
#include <stdint.h>

void csr_matvec(int64_t nrows, const int64_t *ptr, const int32_t *col, const double *val, const double *x,
                double *y, int nthreads) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int64_t i = 0; i < nrows; ++i) {
    double s = 0.0;
    for (int64_t k = ptr[i]; k < ptr[i + 1]; ++k) s += val[k] * x[col[k]];
    y[i] = s;
  }
}
