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
// dense matrix from the level's 3x3-block rows (blocks [9][nnzb]): every entry is written once, so
// the result does not depend on the order in which threads run
// rows and columns of fixed dofs are left out: the matrix is the free-dof block, nf x nf, through
// the compact map cmap (-1 for a fixed dof)
template <typename T>
__global__ void k_dense_from_bsr(const int *__restrict__ ptr, const int *__restrict__ col, const T *__restrict__ B,
                                 int nrow, size_t nnzb, const int *__restrict__ cmap, int nf, T *__restrict__ A) {
  const int i = blockIdx.x;
  if (i >= nrow) return;
  for (int k = ptr[i] + threadIdx.x; k < ptr[i + 1]; k += blockDim.x) {
    const int j = col[k];
#pragma unroll
    for (int p = 0; p < 3; ++p) {
      const int a = cmap[3 * i + p];
      if (a < 0) continue;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int b = cmap[3 * j + q];
        if (b >= 0) A[(size_t)a * nf + b] = B[(size_t)(p * 3 + q) * nnzb + k];
      }
    }
  }
}
// ---------------------------------------------------------------------------------------
// blocked Gauss-Jordan inverse of the SPD coarsest matrix, 128-wide panels (no pivoting):
// per panel k, with D = A_kk, C = A_:k (saved) and R = D^-1 A_k: :
//   A_ij -= C_i R_j (i, j outside panel k), A_kj = R_j, A_ik = -C_i D^-1, A_kk = D^-1.
// Three launches per panel; the rank-128 update is a 128x128-tile GEMM in shared memory with an
// 8x8 register block per thread (16-byte shared loads, K chunks copied with cp.async one chunk
// ahead of the FMAs). The inner dimension runs in chunks of GJK(T) (32 FP32, 16 FP64)
// so that the two staged tiles stay near 33 KB.
// ---------------------------------------------------------------------------------------
constexpr int GJB = 128;
template <typename T> struct GjChunk { static constexpr int K = sizeof(T) == 4 ? 32 : 16; };

// D^-1 of the nb x nb diagonal block (one CTA, unblocked Gauss-Jordan in dynamic shared memory:
// GJB x (GJB+1) values + two pivot vectors)
template <typename T>
__global__ void __launch_bounds__(256) k_gjb_diag(const T *__restrict__ A, int n, int kb, int nb, T *__restrict__ Dinv) {
  extern __shared__ __align__(16) unsigned char gj_smem[];
  T(*a)[GJB + 1] = reinterpret_cast<T(*)[GJB + 1]>(gj_smem);
  T *colp = reinterpret_cast<T *>(gj_smem) + GJB * (GJB + 1), *rowp = colp + GJB;
  for (int t = threadIdx.x; t < GJB * GJB; t += blockDim.x) {
    const int r = t / GJB, c = t % GJB;
    a[r][c] = (r < nb && c < nb) ? A[(size_t)(kb + r) * n + kb + c] : (r == c ? T(1) : T(0));
  }
  __syncthreads();
  for (int p = 0; p < GJB; ++p) {
    if (threadIdx.x < GJB) {
      colp[threadIdx.x] = a[threadIdx.x][p];
      rowp[threadIdx.x] = a[p][threadIdx.x] / a[p][p];
    }
    __syncthreads();
    const T piv = colp[p];
    for (int t = threadIdx.x; t < GJB * GJB; t += blockDim.x) {
      const int r = t / GJB, c = t % GJB;
      T v;
      if (r == p) v = (c == p) ? T(1) / piv : rowp[c];
      else if (c == p) v = -colp[r] / piv;
      else v = a[r][c] - colp[r] * rowp[c];
      a[r][c] = v;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < GJB * GJB; t += blockDim.x) Dinv[t] = a[t / GJB][t % GJB];
}

// 128x128 tile product acc = X (rows i0.., inner dimension 0..127) * Y (inner, cols j0..), X and Y
// read through the loaders (row / column index fastest across threads, so global reads coalesce
// and shared stores do not conflict). 256 threads; thread (ty, tx) owns rows 4ty..4ty+3 and
// 64+4ty..64+4ty+3 and the same columns with tx, read from shared memory as 16-byte vectors
// (a quarter-warp's vectors are consecutive: no bank conflicts).
template <typename T> struct GjVec;
template <> struct GjVec<float> {
  static __device__ __forceinline__ void ld4(const float *p, float *v) {
    const float4 q = *reinterpret_cast<const float4 *>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  }
};
template <> struct GjVec<double> {
  static __device__ __forceinline__ void ld4(const double *p, double *v) {
    const double2 a = *reinterpret_cast<const double2 *>(p), b = *reinterpret_cast<const double2 *>(p + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
};
constexpr int GJ_LD = GJB + 4;       // shared row stride (16-byte aligned rows)
__device__ __forceinline__ int gj_row(int t, int a) { return (a < 4 ? 0 : 64) + 4 * t + (a & 3); }

// asynchronous 4- or 8-byte global -> shared copies (cp.async), grouped per K chunk
template <typename T>
__device__ __forceinline__ void gj_cp(T *dst, const T *src) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void gj_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void gj_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// dynamic shared memory of the tile product: two buffers of X and Y chunks
template <typename T> constexpr size_t gj_tile_smem() { return sizeof(T) * 2 * 2 * GjChunk<T>::K * GJ_LD; }

// the loaders return the source address of an operand element, or nullptr for a zero; chunks of
// the inner dimension are copied asynchronously one chunk ahead of the FMAs (double buffer)
template <typename T, typename LX, typename LY>
__device__ __forceinline__ void gj_tile_mma(T (&acc)[8][8], LX srcx, LY srcy) {
  constexpr int KC = GjChunk<T>::K, NCH = GJB / KC;
  extern __shared__ __align__(16) unsigned char gj_tile_raw[];
  T(*xs)[KC][GJ_LD] = reinterpret_cast<T(*)[KC][GJ_LD]>(gj_tile_raw);               // [2][KC][GJ_LD]
  T(*ys)[KC][GJ_LD] = reinterpret_cast<T(*)[KC][GJ_LD]>(gj_tile_raw + sizeof(T) * 2 * KC * GJ_LD);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) acc[a][b] = T(0);
  auto issue = [&](int ch) {
    const int buf = ch & 1, k0 = ch * KC;
    for (int q = threadIdx.x; q < GJB * KC; q += blockDim.x) {
      const int r = q % GJB, m = q / GJB;
      const T *px = srcx(r, k0 + m), *py = srcy(k0 + m, r);
      if (px) gj_cp(&xs[buf][m][r], px); else xs[buf][m][r] = T(0);
      if (py) gj_cp(&ys[buf][m][r], py); else ys[buf][m][r] = T(0);
    }
    gj_commit();
  };
  issue(0);
  for (int ch = 0; ch < NCH; ++ch) {
    if (ch + 1 < NCH) {
      issue(ch + 1);
      gj_wait<1>();
    } else {
      gj_wait<0>();
    }
    __syncthreads();
    const int buf = ch & 1;
#pragma unroll 4
    for (int m = 0; m < KC; ++m) {
      T xv[8], yv[8];
      GjVec<T>::ld4(&xs[buf][m][4 * ty], xv);
      GjVec<T>::ld4(&xs[buf][m][64 + 4 * ty], xv + 4);
      GjVec<T>::ld4(&ys[buf][m][4 * tx], yv);
      GjVec<T>::ld4(&ys[buf][m][64 + 4 * tx], yv + 4);
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] += xv[a] * yv[b];
    }
    __syncthreads();                     // buffer `buf` is refilled by the next issue
  }
}

// column panel C (n x 128, saved transposed as Ct [128][n] before the update overwrites it) and
// row panel R = D^-1 A_k: (128 x n); block x handles columns [128x, 128x+128) of R and rows
// [128x, 128x+128) of C
template <typename T>
__global__ void __launch_bounds__(256) k_gjb_panels(const T *__restrict__ A, int n, int kb, int nb,
                                                    const T *__restrict__ Dinv, T *__restrict__ R, T *__restrict__ Cc) {
  const int j0 = blockIdx.x * GJB;
  for (int q = threadIdx.x; q < GJB * GJB; q += blockDim.x) {
    const int r = q % GJB, c = q / GJB;
    const int i = j0 + r;
    if (i < n) Cc[(size_t)c * n + i] = c < nb ? A[(size_t)i * n + kb + c] : T(0);
  }
  T acc[8][8];
  gj_tile_mma<T>(
      acc, [&](int r, int m) -> const T * { return Dinv + r * GJB + m; },
      [&](int m, int c) -> const T * { return (m < nb && j0 + c < n) ? A + (size_t)(kb + m) * n + j0 + c : nullptr; });
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int j = j0 + gj_row(tx, b);
      if (j < n) R[(size_t)gj_row(ty, a) * n + j] = acc[a][b];
    }
}

// the update of one 128x128 tile (by, bx): outside panel k A -= C R; row panel R; column panel
// -C D^-1; diagonal block D^-1
template <typename T>
__global__ void __launch_bounds__(256) k_gjb_update(T *__restrict__ A, int n, int kblk, int nb,
                                                    const T *__restrict__ Dinv, const T *__restrict__ R,
                                                    const T *__restrict__ Cc) {
  const int bi = blockIdx.y, bj = blockIdx.x;
  const int i0 = bi * GJB, j0 = bj * GJB, kb = kblk * GJB;
  const bool rowk = bi == kblk, colk = bj == kblk;
  if (rowk && colk) {
    for (int q = threadIdx.x; q < GJB * GJB; q += blockDim.x) {
      const int r = q / GJB, c = q % GJB;
      if (r < nb && c < nb) A[(size_t)(kb + r) * n + kb + c] = Dinv[q];
    }
    return;
  }
  if (rowk) {
    for (int q = threadIdx.x; q < GJB * GJB; q += blockDim.x) {
      const int r = q / GJB, c = q % GJB;
      if (r < nb && j0 + c < n) A[(size_t)(kb + r) * n + j0 + c] = R[(size_t)r * n + j0 + c];
    }
    return;
  }
  T acc[8][8];
  gj_tile_mma<T>(
      acc, [&](int r, int m) -> const T * { return (i0 + r < n) ? Cc + (size_t)m * n + i0 + r : nullptr; },
      [&](int m, int c) -> const T * {
        return colk ? Dinv + m * GJB + c : ((j0 + c < n) ? R + (size_t)m * n + j0 + c : nullptr);
      });
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int i = i0 + gj_row(ty, a);
    if (i >= n) continue;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int j = j0 + gj_row(tx, b);
      if (j >= n) continue;
      if (colk) {
        if (j - kb < nb) A[(size_t)i * n + j] = -acc[a][b];           // -C D^-1
      } else {
        A[(size_t)i * n + j] -= acc[a][b];                           // A - C R
      }
    }
  }
}

// in-place inverse of the n x n SPD matrix A; work holds GJB*GJB + 2*GJB*n values
template <typename T>
int gj_blocked_inverse(T *A, int n, T *work, cudaStream_t s) {
  T *Dinv = work, *R = work + GJB * GJB, *Cc = R + (size_t)GJB * n;
  const int nbk = (n + GJB - 1) / GJB;
  const size_t dsmem = sizeof(T) * ((size_t)GJB * (GJB + 1) + 2 * GJB);
  M3_CUDA(cudaFuncSetAttribute(k_gjb_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem));
  M3_CUDA(cudaFuncSetAttribute(k_gjb_panels<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gj_tile_smem<T>()));
  M3_CUDA(cudaFuncSetAttribute(k_gjb_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gj_tile_smem<T>()));
  for (int k = 0; k < nbk; ++k) {
    const int kb = k * GJB, nb = std::min(GJB, n - kb);
    k_gjb_diag<T><<<1, 256, dsmem, s>>>(A, n, kb, nb, Dinv); count_launch();
    k_gjb_panels<T><<<nbk, 256, gj_tile_smem<T>(), s>>>(A, n, kb, nb, Dinv, R, Cc); count_launch();
    k_gjb_update<T><<<dim3(nbk, nbk), 256, gj_tile_smem<T>(), s>>>(A, n, k, nb, Dinv, R, Cc); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// dense coarse matrix (from the level's block rows) and its blocked Gauss-Jordan inverse; with a
// `lowp` target the FP64 matrix is rounded to FP32 first and A receives nothing
// free-dof inverse of the level matrix: A (nf x nf) = (K restricted to the free dofs)^-1
template <typename T>
int dense_inverse_blocked(const Level &L, const T *B, T *A, T *work, const int *cmap, int nf, cudaStream_t s) {
  M3_CUDA(cudaMemsetAsync(A, 0, sizeof(T) * (size_t)nf * nf, s));
  k_dense_from_bsr<T><<<L.nnod, 64, 0, s>>>(L.bsr_ptr, L.bsr_col, B, L.nnod, (size_t)L.nnzb, cmap, nf, A); count_launch();
  return gj_blocked_inverse<T>(A, nf, work, s);
}
template int dense_inverse_blocked<double>(const Level &, const double *, double *, double *, const int *, int,
                                           cudaStream_t);
template int dense_inverse_blocked<float>(const Level &, const float *, float *, float *, const int *, int,
                                          cudaStream_t);

// y[fidx[row]] = sum_j A[row][j] x[fidx[j]] over the nf free dofs (one warp per row); the fixed
// entries of y are zeroed beforehand
template <typename T>
__global__ void k_dense_gemv(const T *__restrict__ A, int nf, const int *__restrict__ fidx, const T *__restrict__ x,
                             T *__restrict__ y) {
  const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= nf) return;
  T s = 0;
  for (int j = lane; j < nf; j += 32) s += A[(size_t)row * nf + j] * x[fidx[j]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[fidx[row]] = s;
}
// the same with A in FP32 and x, y in FP64 (FP64 accumulation): the refined FP64 coarse solve
__global__ void k_dense_gemv_mixed(const float *__restrict__ A, int nf, const int *__restrict__ fidx,
                                   const double *__restrict__ x, double *__restrict__ y, int accumulate) {
  const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= nf) return;
  double s = 0.0;
  for (int j = lane; j < nf; j += 32) s += (double)A[(size_t)row * nf + j] * x[fidx[j]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[fidx[row]] = accumulate ? y[fidx[row]] + s : s;
}
__global__ void k_sub_masked(const double *a, const double *b, const uint8_t *mask, double *out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = mask[i] ? a[i] - b[i] : 0.0;
}
template <typename T> int bsr_apply(const Level &L, const T *B, const T *x, T *y, cudaStream_t s);

// FP64 coarse solve d = A^-1 r from the FP32 inverse A32 and the FP64 operator B64 of the coarsest
// level: d = A32 r, then `sweeps` steps of iterative refinement d += A32 (r - A d)
int coarse_refined(const Level &L, const float *A32, const double *B64, const double *r, double *d, double *t,
                   int sweeps, const int *fidx, int nf, cudaStream_t s) {
  const int n = L.ndof;
  const unsigned g = (unsigned)((nf + 7) / 8);
  M3_CUDA(cudaMemsetAsync(d, 0, sizeof(double) * n, s));
  k_dense_gemv_mixed<<<g, 256, 0, s>>>(A32, nf, fidx, r, d, 0); count_launch();
  for (int k = 0; k < sweeps; ++k) {
    M3_TRY(bsr_apply<double>(L, B64, d, t, s));
    k_sub_masked<<<(n + 255) / 256, 256, 0, s>>>(r, t, L.freemask, t, n); count_launch();
    k_dense_gemv_mixed<<<g, 256, 0, s>>>(A32, nf, fidx, t, d, 1); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

__global__ void k_d2f_n(const double *a, float *b, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}
// FP32 inverse of the FP64 coarsest operator (its blocks rounded to FP32)
int dense_inverse_from64(const Level &L, const double *B64, float *B32tmp, float *A, float *work, const int *cmap,
                         int nf, cudaStream_t s) {
  const size_t nb = 9 * (size_t)L.nnzb;
  k_d2f_n<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(B64, B32tmp, nb); count_launch();
  return dense_inverse_blocked<float>(L, B32tmp, A, work, cmap, nf, s);
}

// d = A^-1 r on the free dofs, 0 on the fixed ones
template <typename T>
int dense_gemv(const T *A, int n, int nf, const int *fidx, const T *x, T *y, cudaStream_t s) {
  M3_CUDA(cudaMemsetAsync(y, 0, sizeof(T) * n, s));
  if (nf > 0) {
    k_dense_gemv<T><<<(nf + 7) / 8, 256, 0, s>>>(A, nf, fidx, x, y);
    count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template int dense_gemv<double>(const double *, int, int, const int *, const double *, double *, cudaStream_t);
template int dense_gemv<float>(const float *, int, int, const int *, const float *, float *, cudaStream_t);

}  // namespace m3sph
