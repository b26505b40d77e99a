/*
 * ORACLE (test infrastructure only): y = A x for a CSR matrix on all host threads (OpenMP).
 *
 * The CPU baseline times the oracle's MG-PCG / Patera solve with its sparse products here; the
 * reference's own product (mgpcg_solver_p.m:728-733 -> MUTILS spmv) is multi-threaded the same way.
 * Each row is summed in index order with separate multiply and add (built with
 * -ffp-contract=off), so the result is bit-identical to scipy's serial CSR product.
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

/*
 * y = A x for a symmetric A stored as its lower triangle L (diagonal included), A = L + L^T - D,
 * as the reference stores and multiplies its stiffness matrices (flow3d_patera_mg_sph_p.m:311-318
 * converts K1 to the symmetric format of MUTILS spmv; mgpcg_solver_p.m:728-740 forms
 * K*x + K'*x - diag(K).*x for lower-triangle levels). Rows are split over the threads; the
 * transposed contributions of a thread's rows go to its own buffer in work (nthreads x nrows),
 * summed at the end, so there are no races.
 */
#include <omp.h>
#include <string.h>

void sym_csr_matvec(int64_t nrows, const int64_t *ptr, const int32_t *col, const double *val, const double *x,
                    double *y, double *work, int nthreads) {
#pragma omp parallel num_threads(nthreads)
  {
    const int t = omp_get_thread_num();
    double *yt = work + (size_t)t * (size_t)nrows;
    memset(yt, 0, sizeof(double) * (size_t)nrows);
#pragma omp for schedule(static)
    for (int64_t i = 0; i < nrows; ++i) {
      const double xi = x[i];
      double s = 0.0;
      for (int64_t k = ptr[i]; k < ptr[i + 1]; ++k) {
        const int32_t j = col[k];
        const double v = val[k];
        s += v * x[j];
        if (j != i) yt[j] += v * xi;
      }
      y[i] = s;
    }
#pragma omp for schedule(static)
    for (int64_t i = 0; i < nrows; ++i) {
      double s = y[i];
      for (int u = 0; u < nthreads; ++u) s += work[(size_t)u * (size_t)nrows + i];
      y[i] = s;
    }
  }
}
