// Vector kernels (warp-shuffle FP64 reductions, fused CG updates), multigrid transfer
// (intermesh_transfer_matrix / Ic2f' restriction), Jacobi smoothing and the dense coarse
// solve that stands in for cholesky_factorization / cholesky_solve.
#include "common.cuh"

namespace m3sph {

constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 608;      // 4 CTAs per SM on 152 SMs

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int NV>
__device__ __forceinline__ void block_sums(double (&v)[NV], double *partials) {
  __shared__ double sh[NV][RED_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double s = warp_sum(v[k]);
    if (lane == 0) sh[k][wid] = s;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = lane < RED_THREADS / 32 ? sh[k][lane] : 0.0;
      s = warp_sum(s);
      if (lane == 0) partials[k * gridDim.x + blockIdx.x] = s;
    }
  }
}

// final pass: out[k] = sum of partials[k][0..nb)
template <int NV>
__global__ void k_finish(const double *partials, int nb, double *out) {
  double v[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partials[k * nb + i];
    v[k] = s;
  }
  __shared__ double sh[NV][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double s = warp_sum(v[k]);
    if (lane == 0) sh[k][wid] = s;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = lane < (int)(blockDim.x / 32) ? sh[k][lane] : 0.0;
      s = warp_sum(s);
      if (lane == 0) out[k] = s;
    }
  }
}

// out[0] = a.b
__global__ void k_dot(const double *__restrict__ a, const double *__restrict__ b, size_t n, double *partials) {
  double v[1] = {0.0};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    v[0] += a[i] * b[i];
  block_sums<1>(v, partials);
}
// out[0] = a.b, out[1] = c.b
__global__ void k_dot2(const double *__restrict__ a, const double *__restrict__ c, const double *__restrict__ b,
                       size_t n, double *partials) {
  double v[2] = {0.0, 0.0};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    v[0] += a[i] * b[i];
    v[1] += c[i] * b[i];
  }
  block_sums<2>(v, partials);
}
// out[0] = sum(a)
__global__ void k_sum(const double *__restrict__ a, size_t n, double *partials) {
  double v[1] = {0.0};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) v[0] += a[i];
  block_sums<1>(v, partials);
}

int dot(const double *a, const double *b, size_t n, double *partials, double *out, cudaStream_t s) {
  k_dot<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, b, n, partials); count_launch();
  k_finish<1><<<1, 1024, 0, s>>>(partials, RED_BLOCKS, out); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
int dot2(const double *a, const double *c, const double *b, size_t n, double *partials, double *out, cudaStream_t s) {
  k_dot2<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, c, b, n, partials); count_launch();
  k_finish<2><<<1, 1024, 0, s>>>(partials, RED_BLOCKS, out); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
int vsum(const double *a, size_t n, double *partials, double *out, cudaStream_t s) {
  k_sum<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, n, partials); count_launch();
  k_finish<1><<<1, 1024, 0, s>>>(partials, RED_BLOCKS, out); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// ---------------------------------------------------------------------------------------
// flexible PCG updates with device-resident scalars
// scal layout used by the CG: [0] rd, [1] Kqprev.d, [2] qKq, [3] rr, [4] rdlast, [5] alpha_prev
// ---------------------------------------------------------------------------------------
// q = d + beta q, beta = -alpha_prev * (Kq_prev . d) / rdlast (Polak-Ribiere: (r - rlast).d / rdlast)
__global__ void k_cg_dir(const double *__restrict__ d, double *__restrict__ q, size_t n, const double *scal, int first) {
  if (first < 0) first = scal[6] != 0.0;   // flag kept on the device (graph replay)
  double beta = 0.0;
  if (!first) beta = -scal[5] * scal[1] / scal[4];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    q[i] = first ? d[i] : d[i] + beta * q[i];
}
// alpha = rd / qKq ; x += alpha q ; r -= alpha Kq ; partial r.r
__global__ void k_cg_update(double *__restrict__ x, double *__restrict__ r, const double *__restrict__ q,
                            const double *__restrict__ Kq, size_t n, const double *scal, double *partials) {
  const double alpha = scal[0] / scal[2];
  double v[1] = {0.0};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    x[i] += alpha * q[i];
    const double ri = r[i] - alpha * Kq[i];
    r[i] = ri;
    v[0] += ri * ri;
  }
  block_sums<1>(v, partials);
}
// scal[4] = scal[0] (rdlast = rd); scal[5] = alpha
__global__ void k_cg_roll(double *scal) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    scal[5] = scal[0] / scal[2];
    scal[4] = scal[0];
  }
}

int cg_dir(const double *d, double *q, size_t n, const double *scal, int first, cudaStream_t s) {
  k_cg_dir<<<RED_BLOCKS, RED_THREADS, 0, s>>>(d, q, n, scal, first); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
int cg_update(double *x, double *r, const double *q, const double *Kq, size_t n, double *scal, double *partials,
              cudaStream_t s) {
  k_cg_update<<<RED_BLOCKS, RED_THREADS, 0, s>>>(x, r, q, Kq, n, scal, partials); count_launch();
  k_finish<1><<<1, 1024, 0, s>>>(partials, RED_BLOCKS, scal + 3); count_launch();
  k_cg_roll<<<1, 1, 0, s>>>(scal); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// ---------------------------------------------------------------------------------------
// generic elementwise kernels
// ---------------------------------------------------------------------------------------
__global__ void k_axpby(double a, const double *__restrict__ x, double b, double *__restrict__ y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}
int axpby(double a, const double *x, double b, double *y, size_t n, cudaStream_t s) {
  k_axpby<<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, x, b, y, n); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
// y = (x - y) masked: residual r = b - Kx on free dofs
__global__ void k_sub_mask(const double *__restrict__ b, double *__restrict__ y, const uint8_t *__restrict__ mask,
                           size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = mask[i] ? b[i] - y[i] : 0.0;
}
int sub_mask(const double *b, double *y, const uint8_t *mask, size_t n, cudaStream_t s) {
  k_sub_mask<<<RED_BLOCKS, RED_THREADS, 0, s>>>(b, y, mask, n); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
__global__ void k_mask(double *__restrict__ y, const uint8_t *__restrict__ mask, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (!mask[i]) y[i] = 0.0;
}
int apply_mask(double *y, const uint8_t *mask, size_t n, cudaStream_t s) {
  k_mask<<<RED_BLOCKS, RED_THREADS, 0, s>>>(y, mask, n); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template <typename A, typename B>
__global__ void k_convert(const A *__restrict__ a, B *__restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (B)a[i];
}
int d2f(const double *a, float *b, size_t n, cudaStream_t s) {
  k_convert<double, float><<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, b, n); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
int f2d(const float *a, double *b, size_t n, cudaStream_t s) {
  k_convert<float, double><<<RED_BLOCKS, RED_THREADS, 0, s>>>(a, b, n); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// ---------------------------------------------------------------------------------------
// Jacobi smoothing pieces (MG_V_cycle_v2, mgpcg_solver_p.m:397-437, 525-550)
// ---------------------------------------------------------------------------------------
// first down sweep: d = w * r0 * Dinv
template <typename T>
__global__ void k_jac_first(T w, const T *__restrict__ r0, const T *__restrict__ Di, T *__restrict__ d, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    d[i] = w * r0[i] * Di[i];
}
// d += w * (r0 - Kd) * Dinv
template <typename T>
__global__ void k_jac(T w, const T *__restrict__ r0, const T *__restrict__ Kd, const T *__restrict__ Di,
                      T *__restrict__ d, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    d[i] += w * (r0[i] - Kd[i]) * Di[i];
}
template <typename T>
int jac_first(T w, const T *r0, const T *Di, T *d, size_t n, cudaStream_t s) {
  k_jac_first<T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(w, r0, Di, d, n); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template <typename T>
int jac(T w, const T *r0, const T *Kd, const T *Di, T *d, size_t n, cudaStream_t s) {
  k_jac<T><<<RED_BLOCKS, RED_THREADS, 0, s>>>(w, r0, Kd, Di, d, n); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template int jac_first<double>(double, const double *, const double *, double *, size_t, cudaStream_t);
template int jac_first<float>(float, const float *, const float *, float *, size_t, cudaStream_t);
template int jac<double>(double, const double *, const double *, const double *, double *, size_t, cudaStream_t);
template int jac<float>(float, const float *, const float *, const float *, float *, size_t, cudaStream_t);

// ---------------------------------------------------------------------------------------
// transfer: restriction rc = Ic2f' (r0 - Kd) (gather over coarse rows), prolongation
// d_f += Ic2f d_c (gather over fine rows); both masked to free dofs
// ---------------------------------------------------------------------------------------
// one warp per coarse row: lane l takes fine entries ptr[i] + l, + 32, ... (coarse rows gather ~40
// fine nodes), then a shuffle sum
template <typename T>
__global__ void __launch_bounds__(256) k_restrict(const int *__restrict__ ptr, const int *__restrict__ col,
                                                  const float *__restrict__ w, int nrow, const T *__restrict__ a,
                                                  const T *__restrict__ b, const uint8_t *__restrict__ mask,
                                                  T *__restrict__ out) {
  const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= nrow) return;
  T s0 = 0, s1 = 0, s2 = 0;
  for (int k = ptr[i] + lane; k < ptr[i + 1]; k += 32) {
    const int j = col[k];
    const T wk = (T)w[k];
    if (b) {
      s0 += wk * (a[3 * j] - b[3 * j]);
      s1 += wk * (a[3 * j + 1] - b[3 * j + 1]);
      s2 += wk * (a[3 * j + 2] - b[3 * j + 2]);
    } else {
      s0 += wk * a[3 * j];
      s1 += wk * a[3 * j + 1];
      s2 += wk * a[3 * j + 2];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if (lane < 3) {
    const T v = lane == 0 ? s0 : lane == 1 ? s1 : s2;
    out[3 * (size_t)i + lane] = mask[3 * (size_t)i + lane] ? v : T(0);
  }
}
// out = add + P xc (masked); add may alias out
template <typename T>
__global__ void k_prolong(const int *__restrict__ ptr, const int *__restrict__ col, const float *__restrict__ w,
                          int nrow, const T *__restrict__ xc, const T *add, const uint8_t *__restrict__ mask, T *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrow) return;
  T s0 = 0, s1 = 0, s2 = 0;
  for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
    const int j = col[k];
    const T wk = (T)w[k];
    s0 += wk * xc[3 * j];
    s1 += wk * xc[3 * j + 1];
    s2 += wk * xc[3 * j + 2];
  }
  for (int c = 0; c < 3; ++c) {
    const T s = c == 0 ? s0 : (c == 1 ? s1 : s2);
    const T base = add ? add[3 * i + c] : T(0);
    out[3 * i + c] = mask[3 * i + c] ? base + s : T(0);
  }
}
template <typename T>
int restrict_(const Level &F, const Level &C, const T *a, const T *b, T *out, cudaStream_t s) {
  k_restrict<T><<<(unsigned)(((size_t)C.nnod * 32 + 255) / 256), 256, 0, s>>>(F.R_ptr, F.R_col, F.R_w, C.nnod, a, b,
                                                                             C.freemask, out);
  count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template <typename T>
int prolong(const Level &F, const Level &C, const T *xc, const T *add, T *out, cudaStream_t s) {
  k_prolong<T><<<(F.nnod + 255) / 256, 256, 0, s>>>(F.P_ptr, F.P_col, F.P_w, F.nnod, xc, add, F.freemask, out); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template int restrict_<double>(const Level &, const Level &, const double *, const double *, double *, cudaStream_t);
template int restrict_<float>(const Level &, const Level &, const float *, const float *, float *, cudaStream_t);
template int prolong<double>(const Level &, const Level &, const double *, const double *, double *, cudaStream_t);
template int prolong<float>(const Level &, const Level &, const float *, const float *, float *, cudaStream_t);

// ---------------------------------------------------------------------------------------
// coarsest level: dense assembly, in-place Gauss-Jordan inverse (SPD, no pivoting), GEMV
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void k_dense_assemble(const T *__restrict__ K, const int *__restrict__ el2nod, int nel, int n,
                                 T *__restrict__ A) {
  const int e = blockIdx.x;
  for (int q = threadIdx.x; q < NPACK; q += blockDim.x) {
    int cc = 0, rem = q;
    while (rem >= 30 - cc) { rem -= 30 - cc; ++cc; }
    const int rr = cc + rem;
    const int gr = 3 * el2nod[(size_t)(rr / 3) * nel + e] + rr % 3;
    const int gc = 3 * el2nod[(size_t)(cc / 3) * nel + e] + cc % 3;
    const T v = K[kidx<T>(q, e, nel)];
    if (v == T(0)) continue;
    atomicAdd(&A[(size_t)gr * n + gc], v);
    if (gr != gc) atomicAdd(&A[(size_t)gc * n + gr], v);
  }
}
// dense matrix from the level's 3x3-block rows (blocks [9][nnzb]): every entry is written once, so
// the result does not depend on the order in which threads run
template <typename T>
__global__ void k_dense_from_bsr(const int *__restrict__ ptr, const int *__restrict__ col, const T *__restrict__ B,
                                 int nrow, size_t nnzb, int n, T *__restrict__ A) {
  const int i = blockIdx.x;
  if (i >= nrow) return;
  for (int k = ptr[i] + threadIdx.x; k < ptr[i + 1]; k += blockDim.x) {
    const int j = col[k];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = 0; q < 3; ++q) A[(size_t)(3 * i + p) * n + 3 * j + q] = B[(size_t)(p * 3 + q) * nnzb + k];
  }
}
template <typename T>
__global__ void k_dense_fix_diag(T *A, const uint8_t *mask, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !mask[i]) A[(size_t)i * n + i] = T(1);
}
template <typename T>
__global__ void k_gj_save(const T *A, int n, int k, T *colk, T *rowk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T piv = A[(size_t)k * n + k];
  colk[i] = A[(size_t)i * n + k];
  rowk[i] = A[(size_t)k * n + i] / piv;
}
template <typename T>
__global__ void k_gj_update(T *A, int n, int k, const T *colk, const T *rowk) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= n) return;
  const T piv = colk[k];
  T v;
  if (i == k)
    v = (j == k) ? T(1) / piv : rowk[j];
  else if (j == k)
    v = -colk[i] / piv;
  else
    v = A[(size_t)i * n + j] - colk[i] * rowk[j];
  A[(size_t)i * n + j] = v;
}
template <typename T>
int dense_inverse(const Level &L, const T *K, const T *B, T *A, T *work, cudaStream_t s) {
  const int n = L.ndof;
  M3_CUDA(cudaMemsetAsync(A, 0, sizeof(T) * (size_t)n * n, s));
  if (B)
    k_dense_from_bsr<T><<<L.nnod, 64, 0, s>>>(L.bsr_ptr, L.bsr_col, B, L.nnod, (size_t)L.nnzb, n, A);
  else
    k_dense_assemble<T><<<L.nel, 128, 0, s>>>(K, L.el2nod, L.nel, n, A);
  count_launch();
  k_dense_fix_diag<T><<<(n + 255) / 256, 256, 0, s>>>(A, L.freemask, n); count_launch();
  T *colk = work, *rowk = work + n;
  dim3 g((n + 255) / 256, n);
  for (int k = 0; k < n; ++k) {
    k_gj_save<T><<<(n + 255) / 256, 256, 0, s>>>(A, n, k, colk, rowk); count_launch();
    k_gj_update<T><<<g, 256, 0, s>>>(A, n, k, colk, rowk); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template int dense_inverse<double>(const Level &, const double *, const double *, double *, double *, cudaStream_t);
template int dense_inverse<float>(const Level &, const float *, const float *, float *, float *, cudaStream_t);

// y = A x masked (one warp per row)
template <typename T>
__global__ void k_dense_gemv(const T *__restrict__ A, int n, const T *__restrict__ x, const uint8_t *__restrict__ mask,
                             T *__restrict__ y) {
  const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  T s = 0;
  for (int j = lane; j < n; j += 32) s += A[(size_t)row * n + j] * x[j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[row] = mask[row] ? s : T(0);
}
template <typename T>
int dense_gemv(const T *A, int n, const T *x, const uint8_t *mask, T *y, cudaStream_t s) {
  k_dense_gemv<T><<<(n + 7) / 8, 256, 0, s>>>(A, n, x, mask, y); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template int dense_gemv<double>(const double *, int, const double *, const uint8_t *, double *, cudaStream_t);
template int dense_gemv<float>(const float *, int, const float *, const uint8_t *, float *, cudaStream_t);

}  // namespace m3sph
