// Partially assembled FP32 operator of the finest level (the V-cycle operator).
//
// The stored form streams the 465 packed entries of every element matrix (1,860 B per element in
// FP32). This form stores, per element and integration point, only the 3x3 factor
//   A_q = sqrt(w_q eta_q) R_cls^T J_dbl,q      (A[c][j] = d xi_j / d x_c, global Cartesian)
// (J_dbl and w = detJ_CS detJ_SL w_ip as in assembly_stokes_els_*_opt.m:134-164, eta the
// vertex-interpolated viscosity of calc_element_visc.m:5-7, R_cls the element's frame rotation
// undone), 14 x 9 FP32 = 504 B per element, and forms the product on the fly: with u the element's
// velocities in global Cartesian components (node dofs rotated by RR, make_rotation_matrix.m),
//   L = grad u (scaled by sqrt(w eta)),  S = L + L^T - 2/3 tr(L) I,
//   y_n += S grad N_n (scaled)
// which is K = sum_q w eta B^T D B with the deviatoric "23rd" D (C1 = 4/3, C2 = -2/3) of
// assembly_stokes_els_*_opt.m:201-317, written in the rotation-invariant tensor form. Reference
// gradients use the barycentric structure of the P2 basis (vertices L(2L-1), edges 4 La Lb), so a
// node contributes to one or two barycentric directions: 48 + 48 FMA per point instead of 90 + 90.
// Fixed dofs are masked on input and output, as in the stored matrices. Outputs go to the element
// output array Ye[e][30] of the streamed apply, whose node gather (phase 2) sums them per node in
// element order, so the result does not depend on scheduling.
//
// A CTA takes 128 consecutive elements; one thread issues a single 2D TMA load of their factors
// (126 rows x 512 B = 63 KB, L2 evict-first) into shared memory at the start, the threads gather and
// rotate their velocities while it is in flight, and the loop over integration points then reads
// shared memory only. The wait on the load is bounded in time; a wait that gives up sets a bit of
// the level's error word.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"

namespace m3sph {

__constant__ float c_pa_lam[NIP][4];      // barycentric coordinates of the integration points

constexpr int PA_T = 128;
constexpr int PA_SY = 31;                 // staging stride (floats) of the Ye stores: odd, no conflicts
// end vertices of the edge nodes 4..9 (edges 1-2, 2-3, 3-4, 4-1, 1-3, 2-4 of the P2 numbering)
__device__ __forceinline__ constexpr int pa_ea(int k) { return k == 1 ? 1 : k == 2 ? 2 : k == 5 ? 1 : 0; }
__device__ __forceinline__ constexpr int pa_eb(int k) { return k == 0 ? 1 : k == 1 ? 2 : k == 4 ? 2 : 3; }

int pa_upload_tables() {
  ShapeTables t;
  build_shape_tables(t);
  float lam[NIP][4];
  for (int q = 0; q < NIP; ++q)
    for (int v = 0; v < 4; ++v) lam[q][v] = (float)t.NP[q][v];
  M3_CUDA(cudaMemcpyToSymbol(c_pa_lam, lam, sizeof(lam)));
  return M3SPH_OK;
}

// per node (cos theta, sin theta, cos phi, sin phi) from the rotation blocks RR (row-major
// 3x3, [9][nnod]): RR = [cp ct, -sp, cp st; sp ct, cp, sp st; -st, 0, ct]
__global__ void k_pa_trig(const double *__restrict__ RR, int nnod, float4 *__restrict__ trig) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnod) return;
  const double ct = RR[8 * (size_t)nnod + n], st = -RR[6 * (size_t)nnod + n];
  const double cp = RR[4 * (size_t)nnod + n], sp = -RR[1 * (size_t)nnod + n];
  trig[n] = make_float4((float)ct, (float)st, (float)cp, (float)sp);
}

int pa_build_trig(const double *RR, int nnod, float4 *trig, cudaStream_t s) {
  k_pa_trig<<<(nnod + 255) / 256, 256, 0, s>>>(RR, nnod, trig);
  count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

constexpr int PA_ROWS = NIP * 9;                    // factor rows per element block
constexpr int PA_ABYTES = PA_ROWS * PA_T * 4;        // 64,512 B per CTA
constexpr int PA_SMEM = PA_ABYTES + 128 + 16;        // + alignment slack + mbarrier
constexpr unsigned long long PA_TIMEOUT_NS = 1000000000ull;

__device__ __forceinline__ uint32_t pa_smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long pa_gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool pa_mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool pa_mbar_wait(uint32_t bar, uint32_t parity) {
  if (pa_mbar_test(bar, parity)) return true;
  const unsigned long long t0 = pa_gtime();
  for (;;) {
    for (int i = 0; i < 32; ++i)
      if (pa_mbar_test(bar, parity)) return true;
    if (pa_gtime() - t0 > PA_TIMEOUT_NS) return false;
  }
}

__global__ void __launch_bounds__(PA_T, 3)
k_pa_elem_f32(const __grid_constant__ CUtensorMap tmA, const int *__restrict__ el2nod,
              const uint32_t *__restrict__ emask, const float4 *__restrict__ trig, int nel,
              const float *__restrict__ x, float *__restrict__ ye, int *__restrict__ err) {
  extern __shared__ unsigned char pa_raw[];
  float *sA = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(pa_raw) + 127) & ~uintptr_t(127));
  const uint32_t bar = pa_smem_u32(sA + PA_ROWS * PA_T);
  const int e0 = blockIdx.x * PA_T;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(bar),
                 "r"((uint32_t)PA_ABYTES)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
        " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(pa_smem_u32(sA)),
        "l"(reinterpret_cast<uint64_t>(&tmA)), "r"(e0), "r"(0), "r"(bar), "l"(pol)
        : "memory");
  }
  const int e = e0 + threadIdx.x;
  const bool live = e < nel;
  const int ec = live ? e : nel - 1;
  const uint32_t m = live ? emask[ec] : 0u;
  // gather the element's velocities and rotate them to global Cartesian components
  float u[10][3];
#pragma unroll
  for (int n = 0; n < 10; ++n) {
    const int nod = el2nod[(size_t)n * nel + ec];
    const float4 tr = trig[nod];
    const float x0 = (m >> (3 * n)) & 1u ? x[3 * (size_t)nod] : 0.f;
    const float x1 = (m >> (3 * n + 1)) & 1u ? x[3 * (size_t)nod + 1] : 0.f;
    const float x2 = (m >> (3 * n + 2)) & 1u ? x[3 * (size_t)nod + 2] : 0.f;
    const float a = tr.x * x0 + tr.y * x2;          // ct x0 + st x2
    u[n][0] = tr.z * a - tr.w * x1;
    u[n][1] = tr.w * a + tr.z * x1;
    u[n][2] = tr.x * x2 - tr.y * x0;
  }
  __syncthreads();                                   // barrier initialised before anyone waits
  const bool landed = pa_mbar_wait(bar, 0);
  if (!__syncthreads_and(landed)) {                  // the whole CTA leaves together
    if (threadIdx.x == 0) atomicOr(err, 32);
    if (!landed) pa_mbar_wait(bar, 0);               // a second bounded chance for the copy to land
    return;
  }
  float y[10][3];
#pragma unroll
  for (int n = 0; n < 10; ++n) y[n][0] = y[n][1] = y[n][2] = 0.f;
  const float *myA = sA + threadIdx.x;
#pragma unroll 1
  for (int q = 0; q < NIP; ++q) {
    float a[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) a[k] = myA[(q * 9 + k) * PA_T];
    float cv[4], ce[4];                              // 4 L_v - 1 (vertices), 4 L_v (edges)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      ce[v] = 4.f * c_pa_lam[q][v];
      cv[v] = ce[v] - 1.f;
    }
    // derivatives along the four barycentric directions
    float D[3][4];
#pragma unroll
    for (int p = 0; p < 3; ++p) {
#pragma unroll
      for (int v = 0; v < 4; ++v) D[p][v] = u[v][p] * cv[v];
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const int ia = pa_ea(k), ib = pa_eb(k);
        D[p][ia] = fmaf(u[4 + k][p], ce[ib], D[p][ia]);
        D[p][ib] = fmaf(u[4 + k][p], ce[ia], D[p][ib]);
      }
    }
    // L[p][c] = sum_j (D[p][j] - D[p][3]) A[c][j]
    float L[3][3];
#pragma unroll
    for (int p = 0; p < 3; ++p) {
      const float g0 = D[p][0] - D[p][3], g1 = D[p][1] - D[p][3], g2 = D[p][2] - D[p][3];
#pragma unroll
      for (int c = 0; c < 3; ++c) L[p][c] = g0 * a[3 * c] + g1 * a[3 * c + 1] + g2 * a[3 * c + 2];
    }
    const float tr3 = (2.f / 3.f) * (L[0][0] + L[1][1] + L[2][2]);
    float S[3][3];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int c = 0; c < 3; ++c) S[p][c] = L[p][c] + L[c][p];
    S[0][0] -= tr3;
    S[1][1] -= tr3;
    S[2][2] -= tr3;
    // back to the barycentric directions: T[p][j] = sum_c S[p][c] A[c][j], T[p][3] = -sum_j T[p][j]
#pragma unroll
    for (int p = 0; p < 3; ++p) {
      float T[4];
#pragma unroll
      for (int j = 0; j < 3; ++j) T[j] = S[p][0] * a[j] + S[p][1] * a[3 + j] + S[p][2] * a[6 + j];
      T[3] = -(T[0] + T[1] + T[2]);
#pragma unroll
      for (int v = 0; v < 4; ++v) y[v][p] = fmaf(T[v], cv[v], y[v][p]);
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const int ia = pa_ea(k), ib = pa_eb(k);
        y[4 + k][p] = fmaf(T[ia], ce[ib], fmaf(T[ib], ce[ia], y[4 + k][p]));
      }
    }
  }
  __syncthreads();                                   // every thread done with the factors
  // rotate back to the node frames, mask fixed dofs, stage (over the factors) for coalesced stores
  float *my = sA + threadIdx.x * PA_SY;
#pragma unroll
  for (int n = 0; n < 10; ++n) {
    const int nod = el2nod[(size_t)n * nel + ec];
    const float4 tr = trig[nod];
    const float b = tr.z * y[n][0] + tr.w * y[n][1];  // cp yx + sp yy
    const float l0 = tr.x * b - tr.y * y[n][2];
    const float l1 = tr.z * y[n][1] - tr.w * y[n][0];
    const float l2 = tr.y * b + tr.x * y[n][2];
    my[3 * n] = (m >> (3 * n)) & 1u ? l0 : 0.f;
    my[3 * n + 1] = (m >> (3 * n + 1)) & 1u ? l1 : 0.f;
    my[3 * n + 2] = (m >> (3 * n + 2)) & 1u ? l2 : 0.f;
  }
  __syncthreads();
  const int nv = min(PA_T, nel - e0) * 30;
  float *out = ye + (size_t)e0 * 30;
  for (int i = threadIdx.x; i < nv; i += PA_T) out[i] = sA[(i / 30) * PA_SY + i % 30];
}

__global__ void k_node_gather_f32(const int *ptr, const int *idx, int nnod, const float *ye, float *y);
__global__ void k_node_gather_jac_f32(const int *ptr, const int *idx, int nnod, const float *ye, float w,
                                      const float *r, const float *Di, float *d);

static PFN_cuTensorMapEncodeTiled_v12000 g_pa_encode = nullptr;
static std::once_flag g_pa_encode_once;
static cudaError_t g_pa_encode_status = cudaSuccess;

// row stride (floats) of the factor array: a multiple of 4 so TMA rows start on 16-byte boundaries
int pa_row_stride(int nel) { return (nel + 3) & ~3; }

static int pa_phase1(const Level &L, const float *x, cudaStream_t s) {
  std::call_once(g_pa_encode_once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    g_pa_encode_status = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (g_pa_encode_status == cudaSuccess && q != cudaDriverEntryPointSuccess) g_pa_encode_status = cudaErrorNotSupported;
    g_pa_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    if (g_pa_encode_status == cudaSuccess)
      g_pa_encode_status = cudaFuncSetAttribute(k_pa_elem_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, PA_SMEM);
  });
  if (g_pa_encode_status != cudaSuccess || !g_pa_encode) return cuda_fail(g_pa_encode_status, "partially assembled apply set-up");
  CUtensorMap map;
  const cuuint64_t dims[2] = {(cuuint64_t)L.pa_ld, (cuuint64_t)PA_ROWS};
  const cuuint64_t strides[1] = {(cuuint64_t)L.pa_ld * 4};
  const cuuint32_t box[2] = {(cuuint32_t)PA_T, (cuuint32_t)PA_ROWS};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = g_pa_encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(L.pa32), dims, strides,
                                 box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return M3SPH_ERR_CUDA;
  }
  k_pa_elem_f32<<<(L.nel + PA_T - 1) / PA_T, PA_T, PA_SMEM, s>>>(map, L.el2nod, L.pa_emask, L.pa_trig, L.nel, x,
                                                                  L.ye32, L.sa_err);
  count_launch();
  return M3SPH_OK;
}

int pa_apply_f32(const Level &L, const float *x, float *y, cudaStream_t s) {
  M3_TRY(pa_phase1(L, x, s));
  k_node_gather_f32<<<(L.nnod + 255) / 256, 256, 0, s>>>(L.g_ptr, L.g_idx, L.nnod, L.ye32, y);
  count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// d += w (r - K d) / diag with K d from the partially assembled apply (one weighted Jacobi sweep)
int pa_apply_jac_f32(const Level &L, float w, const float *r, const float *Di, float *d, cudaStream_t s) {
  M3_TRY(pa_phase1(L, d, s));
  k_node_gather_jac_f32<<<(L.nnod + 255) / 256, 256, 0, s>>>(L.g_ptr, L.g_idx, L.nnod, L.ye32, w, r, Di, d);
  count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

}  // namespace m3sph
