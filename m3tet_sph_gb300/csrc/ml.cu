// Learned per-element multigrid smoother (no counterpart in the reference): a 52-128-30 MLP
// with GELU, BF16 weights and activations on the tensor cores with FP32 accumulation.
//
// Per element the input is the Jacobi-scaled local residual (30 dofs, divided by its 2-norm s),
// the 10 nodal log-viscosities and 12 geometry factors; the output, times s, is a local
// correction that is gathered to the nodes with partition-of-unity weights 1/multiplicity
// (atomic-free). The network replaces Jacobi sweeps on the two finest levels of the V-cycle; the
// FP64 outer CG judges its effect, so it changes iteration counts but not the converged answer.
// Training pairs (local residual, local error) are (K e, e) for white-noise errors e on the
// project's own operators; training runs here with these forward / backward kernels and Adam.
// Inference runs either as the fused tcgen05 sweep (default) or as the WMMA tile kernel.
#include <mma.h>

#include "common.cuh"

namespace m3sph {

using namespace nvcuda;

constexpr int IN = 52, INP = 64, HID = 128, OUT = 30, OUTP = 32;
constexpr int LDX = INP + 8;     // bf16 leading dimensions (multiples of 8)
constexpr int LDH = HID + 8;
constexpr int LDY = OUTP + 4;    // f32
constexpr int INF_ROWS = 128;    // inference rows per CTA (8 warps x 16)
constexpr int TR_ROWS = 64;      // training rows per CTA (4 warps x 16)
constexpr int NPARAM = HID * INP + HID + OUTP * HID + OUTP;   // flat FP32 parameters (with pads)
constexpr int OFF_W1 = 0, OFF_B1 = HID * INP, OFF_W2 = OFF_B1 + HID, OFF_B2 = OFF_W2 + OUTP * HID;

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
// GELU with erf from Abramowitz & Stegun, Handbook of Mathematical Functions, 7.1.26:
// erf(z) = 1 - (a1 t + a2 t^2 + a3 t^3 + a4 t^4 + a5 t^5) exp(-z^2), t = 1/(1 + p z), z >= 0,
// |error| <= 1.5e-7. With z = |x|/sqrt(2) and q = x/2 * poly(t) * exp(-x^2/2):
// GELU(x) = x - q for x >= 0 and q for x < 0. The fused inference sweep uses it (its hidden
// activations are rounded to BF16, 2^-8 relative, right after); training keeps erff.
__device__ __forceinline__ float gelu_as(float x) {
  const float z = fabsf(x) * 0.70710678118654752f;
  const float t = __fdividef(1.0f, fmaf(0.3275911f, z, 1.0f));
  float p = fmaf(1.061405429f, t, -1.453152027f);
  p = fmaf(p, t, 1.421413741f);
  p = fmaf(p, t, -0.284496736f);
  p = fmaf(p, t, 0.254829592f);
  p = p * t;
  const float q = 0.5f * x * p * __expf(-0.5f * x * x);
  return x >= 0.0f ? x - q : q;
}
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

struct MlpDev {
  const __nv_bfloat16 *W1;   // [HID][INP]
  const __nv_bfloat16 *W2;   // [OUTP][HID]
  const float *b1;           // [HID]
  const float *b2;           // [OUTP]
};

// load weights into shared memory (bf16 with padded leading dimensions)
__device__ __forceinline__ void load_weights(const MlpDev &w, __nv_bfloat16 *sW1, __nv_bfloat16 *sW2, float *sb1,
                                             float *sb2) {
  for (int i = threadIdx.x; i < HID * INP; i += blockDim.x) sW1[(i / INP) * LDX + i % INP] = w.W1[i];
  for (int i = threadIdx.x; i < OUTP * HID; i += blockDim.x) sW2[(i / HID) * LDH + i % HID] = w.W2[i];
  for (int i = threadIdx.x; i < HID; i += blockDim.x) sb1[i] = w.b1[i];
  for (int i = threadIdx.x; i < OUTP; i += blockDim.x) sb2[i] = w.b2[i];
}

// forward of one 16-row strip owned by this warp: H = X W1^T + b1 (f32, pre-activation),
// G = gelu(H) (bf16), Y = G W2^T + b2 (f32)
__device__ __forceinline__ void forward_strip(int row0, const __nv_bfloat16 *sX, const __nv_bfloat16 *sW1,
                                              const __nv_bfloat16 *sW2, const float *sb1, const float *sb2,
                                              float *sH, __nv_bfloat16 *sG, float *sY) {
  const int lane = threadIdx.x & 31;
  for (int j = 0; j < HID / 16; ++j) {
    wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc;
    wmma::fill_fragment(acc, 0.0f);
#pragma unroll
    for (int kk = 0; kk < INP / 16; ++kk) {
      wmma::fragment<wmma::matrix_a, 16, 16, 16, __nv_bfloat16, wmma::row_major> a;
      wmma::fragment<wmma::matrix_b, 16, 16, 16, __nv_bfloat16, wmma::col_major> b;
      wmma::load_matrix_sync(a, sX + row0 * LDX + kk * 16, LDX);
      wmma::load_matrix_sync(b, sW1 + (j * 16) * LDX + kk * 16, LDX);
      wmma::mma_sync(acc, a, b, acc);
    }
    wmma::store_matrix_sync(sH + row0 * LDH + j * 16, acc, LDH, wmma::mem_row_major);
  }
  __syncwarp();
  for (int i = lane; i < 16 * HID; i += 32) {
    const int r = row0 + i / HID, c = i % HID;
    const float h = sH[r * LDH + c] + sb1[c];
    sH[r * LDH + c] = h;
    sG[r * LDH + c] = __float2bfloat16(gelu(h));
  }
  __syncwarp();
  for (int j = 0; j < OUTP / 16; ++j) {
    wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc;
    wmma::fill_fragment(acc, 0.0f);
#pragma unroll
    for (int kk = 0; kk < HID / 16; ++kk) {
      wmma::fragment<wmma::matrix_a, 16, 16, 16, __nv_bfloat16, wmma::row_major> a;
      wmma::fragment<wmma::matrix_b, 16, 16, 16, __nv_bfloat16, wmma::col_major> b;
      wmma::load_matrix_sync(a, sG + row0 * LDH + kk * 16, LDH);
      wmma::load_matrix_sync(b, sW2 + (j * 16) * LDH + kk * 16, LDH);
      wmma::mma_sync(acc, a, b, acc);
    }
    wmma::store_matrix_sync(sY + row0 * LDY + j * 16, acc, LDY, wmma::mem_row_major);
  }
  __syncwarp();
  for (int i = lane; i < 16 * OUTP; i += 32) {
    const int r = row0 + i / OUTP, c = i % OUTP;
    sY[r * LDY + c] += sb2[c];
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------------------
// features of one element from a residual vector (level operator in stored order)
// ---------------------------------------------------------------------------------------
struct FeatLevel {
  int nel;
  const int *el2nod;     // [10][nel] stored order
  const float *lvisc;    // [10][nel] standardised log-viscosity
  const float *geo;      // [12][nel]
};

template <typename T>
__device__ __forceinline__ float element_features(const FeatLevel &L, int e, const T *r, const T *Dinv,
                                                  __nv_bfloat16 *xrow) {
  float rt[30];
  float s2 = 0.f;
#pragma unroll
  for (int n = 0; n < 10; ++n) {
    const int nod = L.el2nod[(size_t)n * L.nel + e];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v = (float)(r[3 * nod + c] * Dinv[3 * nod + c]);
      rt[3 * n + c] = v;
      s2 += v * v;
    }
  }
  const float s = sqrtf(s2);
  const float is = s > 0.f ? 1.0f / s : 0.f;
#pragma unroll
  for (int q = 0; q < 30; ++q) xrow[q] = __float2bfloat16(rt[q] * is);
#pragma unroll
  for (int q = 0; q < 10; ++q) xrow[30 + q] = __float2bfloat16(L.lvisc[(size_t)q * L.nel + e]);
#pragma unroll
  for (int q = 0; q < 12; ++q) xrow[40 + q] = __float2bfloat16(L.geo[(size_t)q * L.nel + e]);
#pragma unroll
  for (int q = IN; q < INP; ++q) xrow[q] = __float2bfloat16(0.f);
  return s;
}

constexpr size_t INF_SMEM = sizeof(__nv_bfloat16) * (INF_ROWS * LDX + HID * LDX + INF_ROWS * LDH + OUTP * LDH) +
                            sizeof(float) * (INF_ROWS * LDH + INF_ROWS * LDY + HID + OUTP + INF_ROWS);

// inference: corrections C[30][nel] (f32) for every element of a level
template <typename T>
__global__ void __launch_bounds__(256) k_ml_infer(FeatLevel L, MlpDev w, const T *__restrict__ r,
                                                  const T *__restrict__ Dinv, float *__restrict__ C) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __nv_bfloat16 *sX = reinterpret_cast<__nv_bfloat16 *>(smraw);
  __nv_bfloat16 *sW1 = sX + INF_ROWS * LDX;
  __nv_bfloat16 *sG = sW1 + HID * LDX;
  __nv_bfloat16 *sW2 = sG + INF_ROWS * LDH;
  float *sH = reinterpret_cast<float *>(sW2 + OUTP * LDH);
  float *sY = sH + INF_ROWS * LDH;
  float *sb1 = sY + INF_ROWS * LDY;
  float *sb2 = sb1 + HID;
  float *sS = sb2 + OUTP;
  load_weights(w, sW1, sW2, sb1, sb2);
  const int e0 = blockIdx.x * INF_ROWS;
  for (int i = threadIdx.x; i < INF_ROWS; i += blockDim.x) {
    const int e = e0 + i;
    if (e < L.nel) {
      sS[i] = element_features<T>(L, e, r, Dinv, sX + i * LDX);
    } else {
      sS[i] = 0.f;
      for (int q = 0; q < INP; ++q) sX[i * LDX + q] = __float2bfloat16(0.f);
    }
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  forward_strip(warp * 16, sX, sW1, sW2, sb1, sb2, sH, sG, sY);
  __syncthreads();
  for (int i = threadIdx.x; i < INF_ROWS * OUT; i += blockDim.x) {
    const int q = i / INF_ROWS, row = i % INF_ROWS, e = e0 + row;
    if (e < L.nel) C[(size_t)q * L.nel + e] = sS[row] * sY[row * LDY + q];
  }
}

// d[3n+c] += omega * sum over (element, local node) of node n of C[3a+c][e] / multiplicity(n)
template <typename T>
__global__ void k_ml_gather(int nnod, int nel, const int *__restrict__ ptr, const int *__restrict__ code,
                            const float *__restrict__ C, const uint8_t *__restrict__ mask, float omega,
                            T *__restrict__ d) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnod) return;
  const int b = ptr[n], e = ptr[n + 1];
  if (e <= b) return;
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  for (int k = b; k < e; ++k) {
    const int el = code[k] / 10, a = code[k] % 10;
    s0 += C[(size_t)(3 * a) * nel + el];
    s1 += C[(size_t)(3 * a + 1) * nel + el];
    s2 += C[(size_t)(3 * a + 2) * nel + el];
  }
  // a non-finite correction (an unusable network) is dropped; the outer CG's rate check then
  // switches the smoother off
  const float w = omega / (float)(e - b);
  if (mask[3 * n] && isfinite(s0)) d[3 * n] += (T)(w * s0);
  if (mask[3 * n + 1] && isfinite(s1)) d[3 * n + 1] += (T)(w * s1);
  if (mask[3 * n + 2] && isfinite(s2)) d[3 * n + 2] += (T)(w * s2);
}

// ---------------------------------------------------------------------------------------
// Fused sweep on the 5th-generation tensor cores (the default inference path).
//
// Persistent CTAs of 8 warps take tiles of 128 consecutive stored elements (tile = MMA M = TMEM
// lanes). Warps 4-7 gather: thread g computes the 52 features of element g of a tile (the local
// residual r0 - kd is formed here) and writes them, BF16, as row g of a K-major 128-byte-swizzled
// A tile; two A tiles alternate, so the gather of the next tile overlaps the MMAs and the GELU of
// this one. Warps 0-3 compute: one thread issues H = A W1^T (M 128, N 128, K 64) into TMEM, thread
// t reads row t of H (tcgen05.ld), adds b1, applies GELU and writes G (BF16, swizzled), one thread
// issues Y = G W2^T (M 128, N 32, K 128) into the same TMEM columns, and thread t stores
// s (Y + b2) as the element's 30 corrections C[e][30]. The weights stay in shared memory for the
// CTA's lifetime. Every mbarrier wait is bounded; a wait that gives up sets the error word and the
// CTA still frees its TMEM before it returns.
// ---------------------------------------------------------------------------------------
namespace tc {
constexpr int ROWS = 128;                       // elements per tile = MMA M = TMEM lanes
constexpr int THREADS = 256;                    // 4 compute warps + 4 gather warps
constexpr int OFF_W1 = 0;                       // W1: [128 hidden][64 in] BF16, K-major, 128 B swizzle
constexpr int OFF_W2 = OFF_W1 + HID * 128;      // W2: 2 atoms (hidden 0-63, 64-127) of [32 out][64]
constexpr int W2_ATOM = OUTP * 128;
constexpr int ATOM = ROWS * 128;                // one [128][64] BF16 operand atom
constexpr int OFF_F = OFF_W2 + 2 * W2_ATOM;     // two feature tiles
constexpr int OFF_G = OFF_F + 2 * ATOM;         // G: 2 atoms (hidden 0-63, 64-127)
constexpr int OFF_B1 = OFF_G + 2 * ATOM;
constexpr int OFF_B2 = OFF_B1 + HID * 4;
constexpr int OFF_S = OFF_B2 + OUTP * 4;        // residual norms of the two feature tiles
constexpr int OFF_BAR = OFF_S + 2 * ROWS * 4;   // f_full[2], f_empty[2], mma_done
constexpr int OFF_TM = OFF_BAR + 5 * 8;
constexpr int SMEM = OFF_TM + 8;
constexpr int SMEM_ALLOC = SMEM + 1024;         // room to align the base to 1024 B
constexpr int TMEM_COLS = 128;                  // H uses 128 columns, Y reuses the first 32
constexpr unsigned long long TIMEOUT_NS = 1000000000ull;
static_assert(OFF_W2 % 1024 == 0 && W2_ATOM % 1024 == 0 && OFF_F % 1024 == 0 && OFF_G % 1024 == 0,
              "swizzle atoms start on 1024 B");
static_assert(OFF_BAR % 8 == 0 && 2 * (SMEM_ALLOC + 1024) <= 233472, "two CTAs per SM");
// instruction descriptor of tcgen05.mma kind::f16: D f32 (bits 4-5 = 1), A and B BF16 (bits 7-9,
// 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28
constexpr uint32_t idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
}  // namespace tc

__device__ __forceinline__ uint32_t tc_smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// byte offset of 16-byte chunk c of row r in a 128-byte-swizzled K-major atom
__device__ __forceinline__ uint32_t tc_sw(int r, int c) { return (uint32_t)(r * 128 + ((c ^ (r & 7)) << 4)); }
__device__ __forceinline__ void tc_st16(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}
__device__ __forceinline__ uint32_t tc_pack(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(id), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ bool tc_bar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool tc_bar_wait(uint32_t bar, uint32_t parity) {
  if (tc_bar_test(bar, parity)) return true;
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (;;) {
    for (int i = 0; i < 32; ++i)
      if (tc_bar_test(bar, parity)) return true;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > tc::TIMEOUT_NS) return false;
  }
}

// the 52 FP32 features of element e from the Jacobi-scaled residual z = (r0 - kd) Dinv: the 30
// local values divided by their norm s, the 10 standardised log-viscosities, the 12 geometry
// factors; returns s (same arithmetic and order as element_features)
__device__ __forceinline__ float element_features_f32(const FeatLevel &L, int e, const float *__restrict__ z,
                                                      float (&x)[IN]) {
  float s2 = 0.f;
#pragma unroll
  for (int n = 0; n < 10; ++n) {
    const int nod = L.el2nod[(size_t)n * L.nel + e];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v = z[3 * nod + c];
      x[3 * n + c] = v;
      s2 += v * v;
    }
  }
  const float s = sqrtf(s2);
  const float is = s > 0.f ? 1.0f / s : 0.f;
#pragma unroll
  for (int q = 0; q < 30; ++q) x[q] *= is;
#pragma unroll
  for (int q = 0; q < 10; ++q) x[30 + q] = L.lvisc[(size_t)q * L.nel + e];
#pragma unroll
  for (int q = 0; q < 12; ++q) x[40 + q] = L.geo[(size_t)q * L.nel + e];
  return s;
}

// the same as 32 BF16 pairs (the sweep's A-operand row)
__device__ __forceinline__ float element_features_packed(const FeatLevel &L, int e, const float *__restrict__ z,
                                                         uint32_t (&xp)[32]) {
  float x[IN];
  const float s = element_features_f32(L, e, z, x);
#pragma unroll
  for (int q = 0; q < IN / 2; ++q) xp[q] = tc_pack(x[2 * q], x[2 * q + 1]);
#pragma unroll
  for (int q = IN / 2; q < 32; ++q) xp[q] = 0u;
  return s;
}

// features of every element of a level in original element order (rows of IN values) and the
// residual norms s, for checks against a CPU restatement
__global__ void k_ml_feature_rows(FeatLevel L, const int *__restrict__ perm, const float *__restrict__ z,
                                  float *__restrict__ X, float *__restrict__ S) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= L.nel) return;
  float x[IN];
  const float s = element_features_f32(L, e, z, x);
  const int o = perm[e];
#pragma unroll
  for (int q = 0; q < IN; ++q) X[(size_t)o * IN + q] = x[q];
  S[o] = s;
}

// z = (r0 - kd) Dinv in FP32 (kd may be null), the per-dof input of the features
template <typename T>
__global__ void k_ml_scale(const T *__restrict__ r0, const T *__restrict__ kd, const T *__restrict__ Dinv,
                           float *__restrict__ z, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T rv = kd ? (T)(r0[i] - kd[i]) : r0[i];
  z[i] = (float)(rv * Dinv[i]);
}

__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
// barrier of the 128 compute threads (named barrier 1) that ANDs a predicate over them
__device__ __forceinline__ bool tc_group_and(bool v) {
  uint32_t out;
  __syncwarp();
  asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, 1, 128, p;\n selp.u32 %0, 1, 0, q;\n}"
               : "=r"(out)
               : "r"((uint32_t)v)
               : "memory");
  return out != 0;
}
__device__ __forceinline__ void tc_arrive(uint32_t bar) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(bar) : "memory");
}

__global__ void __launch_bounds__(tc::THREADS, 2) k_ml_sweep_tc(FeatLevel L, MlpDev w, const float *__restrict__ z,
                                                                float *__restrict__ C, int *__restrict__ err) {
  using namespace tc;
  extern __shared__ unsigned char smraw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sbase = tc_smem_u32(sm);
  const uint32_t f_full = sbase + OFF_BAR, f_empty = f_full + 16, mma_done = f_full + 32;
  float *sb1 = reinterpret_cast<float *>(sm + tc::OFF_B1);
  float *sb2 = reinterpret_cast<float *>(sm + tc::OFF_B2);
  float *sS = reinterpret_cast<float *>(sm + OFF_S);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + OFF_TM);
  // weights into the swizzled layouts: W1 row n (64 inputs = 8 chunks); W2 row n, hidden chunk k
  {
    const uint4 *g1 = reinterpret_cast<const uint4 *>(w.W1);
    for (int i = tid; i < HID * 8; i += THREADS) {
      const uint4 v = g1[i];
      tc_st16(sbase + tc::OFF_W1 + tc_sw(i >> 3, i & 7), v.x, v.y, v.z, v.w);
    }
    const uint4 *g2 = reinterpret_cast<const uint4 *>(w.W2);
    for (int i = tid; i < OUTP * 16; i += THREADS) {
      const int n = i >> 4, k = i & 15;
      const uint4 v = g2[i];
      tc_st16(sbase + tc::OFF_W2 + (k >> 3) * W2_ATOM + tc_sw(n, k & 7), v.x, v.y, v.z, v.w);
    }
    if (tid < HID) sb1[tid] = w.b1[tid];
    if (tid < OUTP) sb2[tid] = w.b2[tid];
  }
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(f_full + 8 * b) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(f_empty + 8 * b) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mma_done) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem_u32(tslot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const int ntile = (L.nel + ROWS - 1) / ROWS;

  if (warp >= 4) {
    // ---------------- gather warps: features of tile i into feature buffer i & 1 ----------------
    const int g = tid - 128;
    int i = 0;
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x, ++i) {
      const int b = i & 1;
      if (i >= 2 && !__all_sync(0xffffffffu, tc_bar_wait(f_empty + 8 * b, ((i >> 1) - 1) & 1))) {
        if (lane == 0) atomicOr(err, 2);
        break;
      }
      const int e = tile * ROWS + g;
      uint32_t xp[32];
      float s = 0.f;
      if (e < L.nel) {
        s = element_features_packed(L, e, z, xp);
      } else {
#pragma unroll
        for (int q = 0; q < 32; ++q) xp[q] = 0u;
      }
      const uint32_t fb = sbase + OFF_F + b * ATOM;
#pragma unroll
      for (int c = 0; c < 8; ++c) tc_st16(fb + tc_sw(g, c), xp[4 * c], xp[4 * c + 1], xp[4 * c + 2], xp[4 * c + 3]);
      sS[b * ROWS + g] = s;
      tc_fence_async_smem();
      __syncwarp();
      if (lane == 0) tc_arrive(f_full + 8 * b);
    }
  } else {
    // ---------------- compute warps: thread t owns row t (TMEM lane t) ----------------
    const int t = tid;
    const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
    uint32_t phase = 0;
    bool ok = true, pending = false;
    int i = 0;
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x, ++i) {
      const int b = i & 1;
      ok = tc_bar_wait(f_full + 8 * b, (i >> 1) & 1);
      const float s = sS[b * ROWS + t];
      // every thread has read its norm and its row of the previous Y: the MMAs may start
      tc_fence_before();
      if (!tc_group_and(ok)) break;
      if (t == 0) {
        tc_fence_after();
#pragma unroll
        for (int k = 0; k < 4; ++k)
          tc_mma(tmem, tc_sdesc(sbase + OFF_F + b * ATOM + 32 * k), tc_sdesc(sbase + tc::OFF_W1 + 32 * k),
                 idesc(ROWS, HID), k > 0);
        tc_commit(f_empty + 8 * b);      // the feature buffer is free once these MMAs are done
        tc_commit(mma_done);
      }
      pending = true;
      ok = tc_bar_wait(mma_done, phase);
      if (!tc_group_and(ok)) break;
      phase ^= 1;
      pending = false;
      tc_fence_after();
      // G = gelu(H + b1): hidden 64a..64a+63 in atom a, 16-column chunk c in swizzle chunks 2c, 2c+1
#pragma unroll 1
      for (int c2 = 0; c2 < HID / 32; ++c2) {
        float h[32];
        tc_ld32(trow + 32 * c2, h);
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          const int c = 2 * c2 + half;
          uint32_t gv[8];
#pragma unroll
          for (int q = 0; q < 8; ++q)
            gv[q] = tc_pack(gelu_as(h[16 * half + 2 * q] + sb1[16 * c + 2 * q]),
                            gelu_as(h[16 * half + 2 * q + 1] + sb1[16 * c + 2 * q + 1]));
          const uint32_t atom = sbase + OFF_G + (c >> 2) * ATOM;
          tc_st16(atom + tc_sw(t, 2 * (c & 3)), gv[0], gv[1], gv[2], gv[3]);
          tc_st16(atom + tc_sw(t, 2 * (c & 3) + 1), gv[4], gv[5], gv[6], gv[7]);
        }
      }
      tc_fence_async_smem();
      tc_fence_before();
      tc_group_and(true);
      if (t == 0) {
        tc_fence_after();
#pragma unroll
        for (int k = 0; k < 8; ++k)
          tc_mma(tmem, tc_sdesc(sbase + OFF_G + (k >> 2) * ATOM + 32 * (k & 3)),
                 tc_sdesc(sbase + tc::OFF_W2 + (k >> 2) * W2_ATOM + 32 * (k & 3)), idesc(ROWS, OUTP), k > 0);
        tc_commit(mma_done);
      }
      pending = true;
      ok = tc_bar_wait(mma_done, phase);
      if (!tc_group_and(ok)) break;
      phase ^= 1;
      pending = false;
      tc_fence_after();
      float y[32];
      tc_ld32(trow, y);
      const int e = tile * ROWS + t;
      if (e < L.nel) {
        float2 *out = reinterpret_cast<float2 *>(C + (size_t)e * OUT);
#pragma unroll
        for (int q = 0; q < OUT / 2; ++q)
          out[q] = make_float2(s * (y[2 * q] + sb2[2 * q]), s * (y[2 * q + 1] + sb2[2 * q + 1]));
      }
    }
    if (!ok) {
      if (t == 0) atomicOr(err, 1);
      if (pending) tc_bar_wait(mma_done, phase);    // MMAs of the abandoned wait, if they still run
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// gather of row-layout corrections C[e][30]: code entries e * 10 + a, element order (same sums as
// k_ml_gather); each (element, node) triple is read with one 8-byte and one 4-byte load
template <typename T>
__global__ void k_ml_gather_rows(int nnod, const int *__restrict__ ptr, const int *__restrict__ code,
                                 const float *__restrict__ C, const uint8_t *__restrict__ mask, float omega,
                                 T *__restrict__ d) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnod) return;
  const int b = ptr[n], e = ptr[n + 1];
  if (e <= b) return;
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  for (int k = b; k < e; ++k) {
    const int el = code[k] / 10, a = code[k] - 10 * el;
    const float *c = C + (size_t)el * OUT + 3 * a;
    if ((a & 1) == 0) {
      const float2 v = *reinterpret_cast<const float2 *>(c);
      s0 += v.x;
      s1 += v.y;
      s2 += c[2];
    } else {
      const float2 v = *reinterpret_cast<const float2 *>(c + 1);
      s0 += c[0];
      s1 += v.x;
      s2 += v.y;
    }
  }
  const float w = omega / (float)(e - b);
  if (mask[3 * n] && isfinite(s0)) d[3 * n] += (T)(w * s0);
  if (mask[3 * n + 1] && isfinite(s1)) d[3 * n + 1] += (T)(w * s1);
  if (mask[3 * n + 2] && isfinite(s2)) d[3 * n + 2] += (T)(w * s2);
}

// ---------------------------------------------------------------------------------------
// training: fused forward + backward on TR_ROWS samples per CTA, gradients atomically summed
// ---------------------------------------------------------------------------------------
constexpr size_t TR_SMEM = sizeof(__nv_bfloat16) * (TR_ROWS * LDX + HID * LDX + TR_ROWS * LDH + OUTP * LDH +
                                                    TR_ROWS * (OUTP + 8)) +
                           sizeof(float) * (2 * TR_ROWS * LDH + TR_ROWS * LDY + HID + OUTP);

__global__ void __launch_bounds__(128) k_ml_train(MlpDev w, const __nv_bfloat16 *__restrict__ X,
                                                  const float *__restrict__ Tg, int n0, int nrows, float scale,
                                                  float *__restrict__ grad, float *__restrict__ loss) {
  extern __shared__ __align__(128) unsigned char smraw[];
  constexpr int LDD = OUTP + 8;
  __nv_bfloat16 *sX = reinterpret_cast<__nv_bfloat16 *>(smraw);
  __nv_bfloat16 *sW1 = sX + TR_ROWS * LDX;
  __nv_bfloat16 *sG = sW1 + HID * LDX;        // G, later dH
  __nv_bfloat16 *sW2 = sG + TR_ROWS * LDH;
  __nv_bfloat16 *sdY = sW2 + OUTP * LDH;      // [rows][LDD]
  float *sH = reinterpret_cast<float *>(sdY + TR_ROWS * LDD);
  float *sF = sH + TR_ROWS * LDH;              // f32 scratch: dG, then weight-gradient tiles
  float *sY = sF + TR_ROWS * LDH;
  float *sb1 = sY + TR_ROWS * LDY;
  float *sb2 = sb1 + HID;
  load_weights(w, sW1, sW2, sb1, sb2);
  const int r0 = blockIdx.x * TR_ROWS;
  for (int i = threadIdx.x; i < TR_ROWS * INP; i += blockDim.x) {
    const int row = i / INP, q = i % INP, g = n0 + r0 + row;
    sX[row * LDX + q] = (r0 + row < nrows) ? X[(size_t)g * INP + q] : __float2bfloat16(0.f);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  forward_strip(warp * 16, sX, sW1, sW2, sb1, sb2, sH, sG, sY);
  __syncthreads();
  // dY = scale * (Y - T) (MSE); loss
  float lsum = 0.f;
  for (int i = threadIdx.x; i < TR_ROWS * OUTP; i += blockDim.x) {
    const int row = i / OUTP, q = i % OUTP, g = n0 + r0 + row;
    float dy = 0.f;
    if (r0 + row < nrows && q < OUT) {
      const float diff = sY[row * LDY + q] - Tg[(size_t)g * OUTP + q];
      lsum += diff * diff;
      dy = scale * diff;
    }
    sY[row * LDY + q] = dy;
    sdY[row * LDD + q] = __float2bfloat16(dy);
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) atomicAdd(loss, lsum);
  __syncthreads();
  // db2 = sum_rows dY
  for (int q = threadIdx.x; q < OUTP; q += blockDim.x) {
    float s = 0.f;
    for (int row = 0; row < TR_ROWS; ++row) s += sY[row * LDY + q];
    if (q < OUT) atomicAdd(&grad[OFF_B2 + q], s);
  }
  // dW2 (OUTP x HID) += dY^T G : 2 x 8 output tiles, k over rows
  for (int t = warp; t < 2 * (HID / 16); t += 4) {
    const int mi = t / (HID / 16), nj = t % (HID / 16);
    wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc;
    wmma::fill_fragment(acc, 0.0f);
    for (int kk = 0; kk < TR_ROWS / 16; ++kk) {
      wmma::fragment<wmma::matrix_a, 16, 16, 16, __nv_bfloat16, wmma::col_major> a;
      wmma::fragment<wmma::matrix_b, 16, 16, 16, __nv_bfloat16, wmma::row_major> b;
      wmma::load_matrix_sync(a, sdY + (kk * 16) * LDD + mi * 16, LDD);
      wmma::load_matrix_sync(b, sG + (kk * 16) * LDH + nj * 16, LDH);
      wmma::mma_sync(acc, a, b, acc);
    }
    float *tile = sF + warp * 256;
    wmma::store_matrix_sync(tile, acc, 16, wmma::mem_row_major);
    __syncwarp();
    for (int i = lane; i < 256; i += 32) {
      const int o = mi * 16 + i / 16, h = nj * 16 + i % 16;
      if (o < OUT) atomicAdd(&grad[OFF_W2 + o * HID + h], tile[i]);
    }
    __syncwarp();
  }
  __syncthreads();
  // dG (rows x HID) = dY W2 ; dH = dG * gelu'(H) (bf16 into sG, f32 sum for db1)
  {
    const int row0 = warp * 16;
    for (int j = 0; j < HID / 16; ++j) {
      wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc;
      wmma::fill_fragment(acc, 0.0f);
#pragma unroll
      for (int kk = 0; kk < OUTP / 16; ++kk) {
        wmma::fragment<wmma::matrix_a, 16, 16, 16, __nv_bfloat16, wmma::row_major> a;
        wmma::fragment<wmma::matrix_b, 16, 16, 16, __nv_bfloat16, wmma::row_major> b;
        wmma::load_matrix_sync(a, sdY + row0 * LDD + kk * 16, LDD);
        wmma::load_matrix_sync(b, sW2 + (kk * 16) * LDH + j * 16, LDH);
        wmma::mma_sync(acc, a, b, acc);
      }
      wmma::store_matrix_sync(sF + row0 * LDH + j * 16, acc, LDH, wmma::mem_row_major);
    }
    __syncwarp();
    for (int i = lane; i < 16 * HID; i += 32) {
      const int r = row0 + i / HID, c = i % HID;
      const float dh = sF[r * LDH + c] * gelu_grad(sH[r * LDH + c]);
      sF[r * LDH + c] = dh;
      sG[r * LDH + c] = __float2bfloat16(dh);
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < HID; c += blockDim.x) {
    float s = 0.f;
    for (int row = 0; row < TR_ROWS; ++row) s += sF[row * LDH + c];
    atomicAdd(&grad[OFF_B1 + c], s);
  }
  __syncthreads();
  // dW1 (HID x INP) += dH^T X : 8 x 4 output tiles
  for (int t = warp; t < (HID / 16) * (INP / 16); t += 4) {
    const int mi = t / (INP / 16), nj = t % (INP / 16);
    wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc;
    wmma::fill_fragment(acc, 0.0f);
    for (int kk = 0; kk < TR_ROWS / 16; ++kk) {
      wmma::fragment<wmma::matrix_a, 16, 16, 16, __nv_bfloat16, wmma::col_major> a;
      wmma::fragment<wmma::matrix_b, 16, 16, 16, __nv_bfloat16, wmma::row_major> b;
      wmma::load_matrix_sync(a, sG + (kk * 16) * LDH + mi * 16, LDH);
      wmma::load_matrix_sync(b, sX + (kk * 16) * LDX + nj * 16, LDX);
      wmma::mma_sync(acc, a, b, acc);
    }
    float *tile = sF + warp * 256;
    __syncwarp();
    wmma::store_matrix_sync(tile, acc, 16, wmma::mem_row_major);
    __syncwarp();
    for (int i = lane; i < 256; i += 32) {
      const int h = mi * 16 + i / 16, q = nj * 16 + i % 16;
      if (q < IN) atomicAdd(&grad[OFF_W1 + h * INP + q], tile[i]);
    }
    __syncwarp();
  }
}

// Adam step on the flat FP32 parameters, then refresh the bf16 / f32 device copies
__global__ void k_ml_adam(float *p, float *m, float *v, float *g, int n, float lr, float b1, float b2, float eps,
                          float bc1, float bc2, __nv_bfloat16 *W1, __nv_bfloat16 *W2, float *bias1, float *bias2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  // pads stay zero: W1 columns >= IN, W2 rows >= OUT, b2 entries >= OUT
  if (i < OFF_B1 && (i % INP) >= IN) pi = 0.f;
  if (i >= OFF_W2 && i < OFF_B2 && (i - OFF_W2) / HID >= OUT) pi = 0.f;
  if (i >= OFF_B2 && i - OFF_B2 >= OUT) pi = 0.f;
  p[i] = pi;
  g[i] = 0.f;
  if (i < OFF_B1) W1[i] = __float2bfloat16(pi);
  else if (i < OFF_W2) bias1[i - OFF_B1] = pi;
  else if (i < OFF_B2) W2[i - OFF_W2] = __float2bfloat16(pi);
  else bias2[i - OFF_B2] = pi;
}

// refresh device copies from FP32 parameters (after upload)
__global__ void k_ml_publish(const float *p, int n, __nv_bfloat16 *W1, __nv_bfloat16 *W2, float *bias1, float *bias2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float pi = p[i];
  if (i < OFF_B1) W1[i] = __float2bfloat16(pi);
  else if (i < OFF_W2) bias1[i - OFF_B1] = pi;
  else if (i < OFF_B2) W2[i - OFF_W2] = __float2bfloat16(pi);
  else bias2[i - OFF_B2] = pi;
}

}  // namespace m3sph

// ======================================================================================
// host side
// ======================================================================================
namespace m3sph {

struct MlLevel {
  int *n2e_ptr = nullptr, *n2e_code = nullptr;   // node -> (stored element * 10 + local node)
  float *lvisc = nullptr, *geo = nullptr;         // [10][nel], [12][nel]
  float *C = nullptr;                             // 30 corrections per element ([30][nel] or [nel][30])
  float *z = nullptr;                             // [3 nnod] Jacobi-scaled residual (fused sweep)
};

struct MlState {
  MlLevel lev[2];
  int nlev = 0;
  float *params = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *loss = nullptr;
  __nv_bfloat16 *W1 = nullptr, *W2 = nullptr;
  float *b1 = nullptr, *b2 = nullptr;
  bool trained = false;
  long adam_t = 0;
  int *err = nullptr;          // bounded waits of the fused sweep that gave up
  // dataset
  __nv_bfloat16 *X = nullptr, *X2 = nullptr;
  float *T = nullptr, *T2 = nullptr;
  long cap = 0, count = 0;
};

static MlState *mls(m3sph_mesh *M) { return reinterpret_cast<MlState *>(M->ml); }

template <typename T>
static int ml_alloc(T **p, size_t n) {
  *p = nullptr;
  M3_CUDA(cudaMalloc((void **)p, sizeof(T) * (n ? n : 1)));
  return M3SPH_OK;
}

// geometry and viscosity features of a level (vertex coordinates from the finest GCOORD: the
// nodes of a coarse level are the leading nodes of the finest level)
__global__ void k_ml_features(int nel, const int *__restrict__ el2nod, const double *__restrict__ X, int nnod0,
                              const double *__restrict__ visc, float lmu, float lsig, float lh_ref, float r0,
                              float r1, float level, float *__restrict__ lv, float *__restrict__ geo) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  double x[4][3];
  for (int i = 0; i < 4; ++i) {
    const int v = el2nod[(size_t)i * nel + e];
    for (int k = 0; k < 3; ++k) x[i][k] = X[(size_t)k * nnod0 + v];
  }
  double ed[3][3];
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) ed[i][k] = x[i][k] - x[3][k];
  const double det = ed[0][0] * (ed[1][1] * ed[2][2] - ed[1][2] * ed[2][1]) - ed[0][1] * (ed[1][0] * ed[2][2] - ed[1][2] * ed[2][0]) +
                     ed[0][2] * (ed[1][0] * ed[2][1] - ed[1][1] * ed[2][0]);
  const double h = cbrt(fabs(det));
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) geo[(size_t)(3 * i + k) * nel + e] = (float)(ed[i][k] / h);
  geo[(size_t)9 * nel + e] = (float)log(h) - lh_ref;
  double rc = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double c = 0.25 * (x[0][k] + x[1][k] + x[2][k] + x[3][k]);
    rc += c * c;
  }
  geo[(size_t)10 * nel + e] = ((float)sqrt(rc) - r0) / (r1 - r0);
  geo[(size_t)11 * nel + e] = level;
  for (int n = 0; n < 10; ++n) {
    const int nod = el2nod[(size_t)n * nel + e];
    lv[(size_t)n * nel + e] = ((float)log(visc[nod]) - lmu) / lsig;
  }
}

int ml_build(m3sph_mesh *M) {
  if (M->ml) return M3SPH_OK;
  MlState *S = new MlState();
  M->ml = S;
  M->ml_free = [](void *p) {
    MlState *S = reinterpret_cast<MlState *>(p);
    for (int i = 0; i < 2; ++i)
      for (void *q : {(void *)S->lev[i].n2e_ptr, (void *)S->lev[i].n2e_code, (void *)S->lev[i].lvisc,
                      (void *)S->lev[i].geo, (void *)S->lev[i].C, (void *)S->lev[i].z})
        if (q) cudaFree(q);
    for (void *q : {(void *)S->params, (void *)S->m, (void *)S->v, (void *)S->grad, (void *)S->loss, (void *)S->W1,
                    (void *)S->W2, (void *)S->b1, (void *)S->b2, (void *)S->X, (void *)S->X2, (void *)S->T,
                    (void *)S->T2, (void *)S->err})
      if (q) cudaFree(q);
    delete S;
  };
  cudaStream_t s = M->stream;
  S->nlev = std::min(2, M->nmg);
  for (int j = 0; j < S->nlev; ++j) {
    Level &L = M->lev[j];
    std::vector<int> perm(L.nel), invp(L.nel);
    M3_CUDA(cudaMemcpy(perm.data(), L.perm, sizeof(int) * L.nel, cudaMemcpyDeviceToHost));
    for (int p = 0; p < L.nel; ++p) invp[perm[p]] = p;
    std::vector<int> ptr(L.nnod + 1, 0), code((size_t)L.nel * 10);
    for (size_t i = 0; i < (size_t)L.nel * 10; ++i) ptr[L.h_el2nod_orig[i] + 1]++;
    for (int n = 0; n < L.nnod; ++n) ptr[n + 1] += ptr[n];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int e = 0; e < L.nel; ++e)
      for (int a = 0; a < 10; ++a) code[fill[L.h_el2nod_orig[(size_t)e * 10 + a]]++] = invp[e] * 10 + a;
    MlLevel &ml = S->lev[j];
    M3_TRY(ml_alloc(&ml.n2e_ptr, ptr.size()));
    M3_TRY(ml_alloc(&ml.n2e_code, code.size()));
    M3_CUDA(cudaMemcpyAsync(ml.n2e_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice, s));
    M3_CUDA(cudaMemcpyAsync(ml.n2e_code, code.data(), sizeof(int) * code.size(), cudaMemcpyHostToDevice, s));
    M3_TRY(ml_alloc(&ml.lvisc, 10 * (size_t)L.nel));
    M3_TRY(ml_alloc(&ml.geo, 12 * (size_t)L.nel));
    M3_TRY(ml_alloc(&ml.C, 30 * (size_t)L.nel));
    M3_TRY(ml_alloc(&ml.z, (size_t)L.ndof));
  }
  M3_TRY(ml_alloc(&S->err, 1));
  M3_CUDA(cudaMemsetAsync(S->err, 0, sizeof(int), s));
  M3_TRY(ml_alloc(&S->params, NPARAM));
  M3_TRY(ml_alloc(&S->m, NPARAM));
  M3_TRY(ml_alloc(&S->v, NPARAM));
  M3_TRY(ml_alloc(&S->grad, NPARAM));
  M3_TRY(ml_alloc(&S->loss, 4));
  M3_TRY(ml_alloc(&S->W1, HID * INP));
  M3_TRY(ml_alloc(&S->W2, OUTP * HID));
  M3_TRY(ml_alloc(&S->b1, HID));
  M3_TRY(ml_alloc(&S->b2, OUTP));
  M3_CUDA(cudaMemsetAsync(S->m, 0, sizeof(float) * NPARAM, s));
  M3_CUDA(cudaMemsetAsync(S->v, 0, sizeof(float) * NPARAM, s));
  M3_CUDA(cudaMemsetAsync(S->grad, 0, sizeof(float) * NPARAM, s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

// recompute the per-element features from the current viscosity (called by the operator set-up)
// sums of log(visc) and log(visc)^2 in a fixed order: per-block partial sums, then one block
constexpr int LOGSTAT_BLOCKS = 512;
__global__ void k_logstats_partial(const double *v, int n, double *part) {
  __shared__ double s1[256], s2[256];
  double a = 0.0, b = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double l = log(v[i]);
    a += l;
    b += l * l;
  }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s1[threadIdx.x] += s1[threadIdx.x + o];
      s2[threadIdx.x] += s2[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s1[0];
    part[2 * blockIdx.x + 1] = s2[0];
  }
}
__global__ void k_logstats_final(const double *part, int nb, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double a = 0.0, b = 0.0;
  for (int k = 0; k < nb; ++k) {
    a += part[2 * k];
    b += part[2 * k + 1];
  }
  out[0] = a;
  out[1] = b;
}

// features of the learned smoother; h_visc (nnod, host) or nullptr: the statistics of log(visc)
// are then reduced on the device from the resident viscosity
int ml_features(m3sph_mesh *M, const double *h_visc) {
  MlState *S = mls(M);
  if (!S) return M3SPH_OK;
  Level &L0 = M->lev[0];
  double mu = 0.0, m2 = 0.0, rmin = 1e300, rmax = 0.0;
  if (h_visc) {
    for (int n = 0; n < L0.nnod; ++n) {
      const double l = std::log(h_visc[n]);
      mu += l;
      m2 += l * l;
    }
  } else {
    // M->red holds 4096 doubles of reduction partials; scal[16..17] the two sums
    k_logstats_partial<<<LOGSTAT_BLOCKS, 256, 0, M->stream>>>(M->fin.visc, L0.nnod, M->red); count_launch();
    k_logstats_final<<<1, 32, 0, M->stream>>>(M->red, LOGSTAT_BLOCKS, M->scal + 16); count_launch();
    M3_CUDA(cudaMemcpyAsync(M->h_scal + 16, M->scal + 16, 2 * sizeof(double), cudaMemcpyDeviceToHost, M->stream));
    M3_CUDA(cudaStreamSynchronize(M->stream));
    mu = M->h_scal[16];
    m2 = M->h_scal[17];
  }
  mu /= L0.nnod;
  const double sig = std::sqrt(std::max(m2 / L0.nnod - mu * mu, 1e-12)) + 1e-3;
  rmin = M->r_min;
  rmax = M->r_max;
  cudaStream_t s = M->stream;
  for (int j = 0; j < S->nlev; ++j) {
    Level &L = M->lev[j];
    const double vol = 4.0 / 3.0 * M_PI * (rmax * rmax * rmax - rmin * rmin * rmin);
    const double lh_ref = std::log(std::cbrt(6.0 * vol / L.nel));
    k_ml_features<<<(L.nel + 127) / 128, 128, 0, s>>>(L.nel, L.el2nod, M->fin.gcoord, L0.nnod, M->fin.visc, (float)mu,
                                                      (float)sig, (float)lh_ref, (float)rmin, (float)rmax, (float)j,
                                                      S->lev[j].lvisc, S->lev[j].geo); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

template <typename T>
__global__ void k_sub(const T *a, const T *b, T *out, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}

// inference kernels: 1 fused tcgen05 sweep (default), 0 the WMMA tile kernel with column-layout
// corrections and a separate residual pass (kept as the reference form for tests)
static int g_ml_infer = 1;
static int g_nsm = 152;
int ml_set_infer(int v) {
  if (v != 0 && v != 1) {
    set_error("ml_infer must be 0 or 1");
    return M3SPH_ERR_BAD_INPUT;
  }
  g_ml_infer = v;
  return M3SPH_OK;
}

int ml_check(m3sph_mesh *M) {
  MlState *S = mls(M);
  if (!S || !S->err) return M3SPH_OK;
  int h = 0;
  M3_CUDA(cudaMemcpyAsync(&h, S->err, sizeof(int), cudaMemcpyDeviceToHost, M->stream));
  M3_CUDA(cudaStreamSynchronize(M->stream));
  if (h) {
    M3_CUDA(cudaMemsetAsync(S->err, 0, sizeof(int), M->stream));
    set_error("learned smoother sweep: a bounded wait gave up");
    return M3SPH_ERR_CUDA;
  }
  return M3SPH_OK;
}

// d += PoU(MLP(features(r0 - kd))) on level j (kd may be null: residual r0)
template <typename T>
int ml_sweep(m3sph_mesh *M, int j, const T *r0, const T *kd, const T *Dinv, T *tmp, T *d) {
  MlState *S = mls(M);
  Level &L = M->lev[j];
  cudaStream_t s = M->stream;
  FeatLevel f{L.nel, L.el2nod, S->lev[j].lvisc, S->lev[j].geo};
  MlpDev w{S->W1, S->W2, S->b1, S->b2};
  if (g_ml_infer == 1) {
    const int ntile = (L.nel + tc::ROWS - 1) / tc::ROWS;
    const int grid = std::min(ntile, 2 * g_nsm);
    k_ml_scale<T><<<(unsigned)((L.ndof + 255) / 256), 256, 0, s>>>(r0, kd, Dinv, S->lev[j].z, L.ndof); count_launch();
    k_ml_sweep_tc<<<grid, tc::THREADS, tc::SMEM_ALLOC, s>>>(f, w, S->lev[j].z, S->lev[j].C, S->err); count_launch();
    k_ml_gather_rows<T><<<(L.nnod + 127) / 128, 128, 0, s>>>(L.nnod, S->lev[j].n2e_ptr, S->lev[j].n2e_code,
                                                              S->lev[j].C, L.freemask, M->ml_omega, d); count_launch();
    M3_CUDA(cudaGetLastError());
    return M3SPH_OK;
  }
  const T *r = r0;
  if (kd) {
    k_sub<T><<<(unsigned)((L.ndof + 255) / 256), 256, 0, s>>>(r0, kd, tmp, L.ndof); count_launch();
    r = tmp;
  }
  k_ml_infer<T><<<(L.nel + INF_ROWS - 1) / INF_ROWS, 256, INF_SMEM, s>>>(f, w, r, Dinv, S->lev[j].C); count_launch();
  k_ml_gather<T><<<(L.nnod + 127) / 128, 128, 0, s>>>(L.nnod, L.nel, S->lev[j].n2e_ptr, S->lev[j].n2e_code,
                                                       S->lev[j].C, L.freemask, M->ml_omega, d); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template int ml_sweep<float>(m3sph_mesh *, int, const float *, const float *, const float *, float *, float *);
template int ml_sweep<double>(m3sph_mesh *, int, const double *, const double *, const double *, double *, double *);

int ml_init_kernels() {
  M3_CUDA(cudaFuncSetAttribute(k_ml_infer<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)INF_SMEM));
  M3_CUDA(cudaFuncSetAttribute(k_ml_infer<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)INF_SMEM));
  M3_CUDA(cudaFuncSetAttribute(k_ml_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TR_SMEM));
  M3_CUDA(cudaFuncSetAttribute(k_ml_sweep_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_ALLOC));
  int dev = 0;
  M3_CUDA(cudaGetDevice(&dev));
  M3_CUDA(cudaDeviceGetAttribute(&g_nsm, cudaDevAttrMultiProcessorCount, dev));
  return M3SPH_OK;
}

bool ml_ready(m3sph_mesh *M) { return M->ml && mls(M)->trained; }

// ---- training data: features of r and targets e_loc / s for every element of level 0 ----
// Training pair of element e: features of the residual, and as target the element's error values scaled
// like the network output (1 / local residual norm), zero on fixed dofs and clamped against outliers.
constexpr float TARGET_CLIP = 20.f;
__global__ void k_ml_samples(FeatLevel L, const double *__restrict__ r, const double *__restrict__ Dinv,
                             const double *__restrict__ err, const uint8_t *__restrict__ mask, int stride, int offset,
                             long base, long cap, __nv_bfloat16 *__restrict__ Xo, float *__restrict__ Tg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int e = offset + i * stride;
  if (e >= L.nel) return;
  const long row = base + i;
  if (row >= cap) return;
  __nv_bfloat16 xr[INP];
  const float s = element_features<double>(L, e, r, Dinv, xr);
  for (int q = 0; q < INP; ++q) Xo[row * INP + q] = xr[q];
  const float is = s > 0.f ? 1.0f / s : 0.f;
  for (int n = 0; n < 10; ++n) {
    const int nod = L.el2nod[(size_t)n * L.nel + e];
    for (int c = 0; c < 3; ++c) {
      const float t = mask[3 * (size_t)nod + c] ? (float)err[3 * (size_t)nod + c] * is : 0.f;
      Tg[row * OUTP + 3 * n + c] = fminf(fmaxf(t, -TARGET_CLIP), TARGET_CLIP);
    }
  }
  Tg[row * OUTP + 30] = 0.f;
  Tg[row * OUTP + 31] = 0.f;
}

int ml_add_samples(m3sph_mesh *M, const double *r, const double *err, int stride, int offset) {
  MlState *S = mls(M);
  Level &L0 = M->lev[0];
  const int n = (L0.nel - offset + stride - 1) / stride;
  const long room = S->cap - S->count;
  if (room <= 0) return M3SPH_OK;
  FeatLevel f{L0.nel, L0.el2nod, S->lev[0].lvisc, S->lev[0].geo};
  k_ml_samples<<<(n + 127) / 128, 128, 0, M->stream>>>(f, r, L0.Dinv64, err, L0.freemask, stride, offset, S->count,
                                                        S->cap, S->X, S->T);
  count_launch();
  M3_CUDA(cudaGetLastError());
  S->count = std::min<long>(S->cap, S->count + n);
  return M3SPH_OK;
}

// features of level j (z: Jacobi-scaled residual, device, 3 nnod) into X [nel][IN] and S [nel]
int ml_feature_rows(m3sph_mesh *M, int j, const float *z, float *X, float *Sn) {
  MlState *S = mls(M);
  Level &L = M->lev[j];
  FeatLevel f{L.nel, L.el2nod, S->lev[j].lvisc, S->lev[j].geo};
  k_ml_feature_rows<<<(L.nel + 127) / 128, 128, 0, M->stream>>>(f, L.perm, z, X, Sn);
  count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

int ml_reserve(m3sph_mesh *M, long cap) {
  MlState *S = mls(M);
  if (S->cap >= cap) return M3SPH_OK;
  for (void *q : {(void *)S->X, (void *)S->X2, (void *)S->T, (void *)S->T2})
    if (q) cudaFree(q);
  M3_TRY(ml_alloc(&S->X, (size_t)cap * INP));
  M3_TRY(ml_alloc(&S->X2, (size_t)cap * INP));
  M3_TRY(ml_alloc(&S->T, (size_t)cap * OUTP));
  M3_TRY(ml_alloc(&S->T2, (size_t)cap * OUTP));
  S->cap = cap;
  S->count = 0;
  return M3SPH_OK;
}

__global__ void k_ml_permute(const __nv_bfloat16 *X, const float *T, const int *perm, long n, __nv_bfloat16 *X2,
                             float *T2) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long j = perm[i];
  for (int q = 0; q < INP; ++q) X2[i * INP + q] = X[j * INP + q];
  for (int q = 0; q < OUTP; ++q) T2[i * OUTP + q] = T[j * OUTP + q];
}

int ml_set_params(m3sph_mesh *M, const float *h) {
  MlState *S = mls(M);
  M3_CUDA(cudaMemcpyAsync(S->params, h, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, M->stream));
  k_ml_publish<<<(NPARAM + 255) / 256, 256, 0, M->stream>>>(S->params, NPARAM, S->W1, S->W2, S->b1, S->b2); count_launch();
  M3_CUDA(cudaMemsetAsync(S->m, 0, sizeof(float) * NPARAM, M->stream));
  M3_CUDA(cudaMemsetAsync(S->v, 0, sizeof(float) * NPARAM, M->stream));
  M3_CUDA(cudaMemsetAsync(S->grad, 0, sizeof(float) * NPARAM, M->stream));
  M3_CUDA(cudaStreamSynchronize(M->stream));
  S->adam_t = 0;
  return M3SPH_OK;
}

// one epoch over the shuffled dataset; returns the mean squared error per output
int ml_epoch(m3sph_mesh *M, int batch, float lr, unsigned long long seed, double *mse) {
  MlState *S = mls(M);
  cudaStream_t s = M->stream;
  const long n = S->count;
  if (n < batch) {
    set_error("not enough training samples for one batch");
    return M3SPH_ERR_BAD_INPUT;
  }
  std::vector<int> perm(n);
  for (long i = 0; i < n; ++i) perm[i] = (int)i;
  unsigned long long st = seed * 6364136223846793005ull + 1442695040888963407ull;
  for (long i = n - 1; i > 0; --i) {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    const long j = (long)((st >> 33) % (unsigned long long)(i + 1));
    std::swap(perm[i], perm[j]);
  }
  int *dperm = nullptr;
  M3_TRY(ml_alloc(&dperm, n));
  M3_CUDA(cudaMemcpyAsync(dperm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  k_ml_permute<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(S->X, S->T, dperm, n, S->X2, S->T2); count_launch();
  M3_CUDA(cudaMemsetAsync(S->loss, 0, sizeof(float), s));
  MlpDev w{S->W1, S->W2, S->b1, S->b2};
  const long nb = n / batch;
  for (long b = 0; b < nb; ++b) {
    const float scale = 2.0f / (float)(batch * OUT);
    k_ml_train<<<(batch + TR_ROWS - 1) / TR_ROWS, 128, TR_SMEM, s>>>(w, S->X2, S->T2, (int)(b * batch), batch, scale,
                                                                     S->grad, S->loss); count_launch();
    ++S->adam_t;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.0f - std::pow(b1, (float)S->adam_t), bc2 = 1.0f - std::pow(b2, (float)S->adam_t);
    k_ml_adam<<<(NPARAM + 255) / 256, 256, 0, s>>>(S->params, S->m, S->v, S->grad, NPARAM, lr, b1, b2, 1e-8f, bc1, bc2,
                                                   S->W1, S->W2, S->b1, S->b2); count_launch();
  }
  float loss = 0.f;
  M3_CUDA(cudaMemcpyAsync(&loss, S->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  cudaFree(dperm);
  M3_CUDA(cudaGetLastError());
  *mse = loss / ((double)nb * batch * OUT);
  S->trained = true;
  return M3SPH_OK;
}

// gradients of the MSE loss on caller data (no parameter update), for gradient checks
int ml_gradients(m3sph_mesh *M, const float *hX, const float *hT, int n, float *hgrad, double *loss_out) {
  MlState *S = mls(M);
  cudaStream_t s = M->stream;
  std::vector<__nv_bfloat16> xb((size_t)n * INP);
  for (size_t i = 0; i < xb.size(); ++i) xb[i] = __float2bfloat16(hX[i]);
  __nv_bfloat16 *dX = nullptr;
  float *dT = nullptr;
  M3_TRY(ml_alloc(&dX, xb.size()));
  M3_TRY(ml_alloc(&dT, (size_t)n * OUTP));
  M3_CUDA(cudaMemcpyAsync(dX, xb.data(), sizeof(__nv_bfloat16) * xb.size(), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(dT, hT, sizeof(float) * n * OUTP, cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemsetAsync(S->grad, 0, sizeof(float) * NPARAM, s));
  M3_CUDA(cudaMemsetAsync(S->loss, 0, sizeof(float), s));
  MlpDev w{S->W1, S->W2, S->b1, S->b2};
  k_ml_train<<<(n + TR_ROWS - 1) / TR_ROWS, 128, TR_SMEM, s>>>(w, dX, dT, 0, n, 2.0f / (float)(n * OUT), S->grad,
                                                               S->loss); count_launch();
  float loss = 0.f;
  M3_CUDA(cudaMemcpyAsync(hgrad, S->grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaMemcpyAsync(&loss, S->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaMemsetAsync(S->grad, 0, sizeof(float) * NPARAM, s));
  M3_CUDA(cudaStreamSynchronize(s));
  cudaFree(dX);
  cudaFree(dT);
  *loss_out = loss;
  return M3SPH_OK;
}

// forward only on caller data (inference path of the training kernel's forward)
__global__ void __launch_bounds__(256) k_ml_forward_rows(MlpDev w, const __nv_bfloat16 *__restrict__ X, int n,
                                                         float *__restrict__ Y) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __nv_bfloat16 *sX = reinterpret_cast<__nv_bfloat16 *>(smraw);
  __nv_bfloat16 *sW1 = sX + INF_ROWS * LDX;
  __nv_bfloat16 *sG = sW1 + HID * LDX;
  __nv_bfloat16 *sW2 = sG + INF_ROWS * LDH;
  float *sH = reinterpret_cast<float *>(sW2 + OUTP * LDH);
  float *sY = sH + INF_ROWS * LDH;
  float *sb1 = sY + INF_ROWS * LDY;
  float *sb2 = sb1 + HID;
  load_weights(w, sW1, sW2, sb1, sb2);
  const int r0 = blockIdx.x * INF_ROWS;
  for (int i = threadIdx.x; i < INF_ROWS * INP; i += blockDim.x) {
    const int row = i / INP, q = i % INP;
    sX[row * LDX + q] = (r0 + row < n) ? X[(size_t)(r0 + row) * INP + q] : __float2bfloat16(0.f);
  }
  __syncthreads();
  forward_strip((threadIdx.x >> 5) * 16, sX, sW1, sW2, sb1, sb2, sH, sG, sY);
  __syncthreads();
  for (int i = threadIdx.x; i < INF_ROWS * OUT; i += blockDim.x) {
    const int row = i / OUT, q = i % OUT;
    if (r0 + row < n) Y[(size_t)(r0 + row) * OUT + q] = sY[row * LDY + q];
  }
}

int ml_forward(m3sph_mesh *M, const float *hX, int n, float *hY) {
  MlState *S = mls(M);
  cudaStream_t s = M->stream;
  std::vector<__nv_bfloat16> xb((size_t)n * INP);
  for (size_t i = 0; i < xb.size(); ++i) xb[i] = __float2bfloat16(hX[i]);
  __nv_bfloat16 *dX = nullptr;
  float *dY = nullptr;
  M3_TRY(ml_alloc(&dX, xb.size()));
  M3_TRY(ml_alloc(&dY, (size_t)n * OUT));
  M3_CUDA(cudaMemcpyAsync(dX, xb.data(), sizeof(__nv_bfloat16) * xb.size(), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaFuncSetAttribute(k_ml_forward_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)INF_SMEM));
  MlpDev w{S->W1, S->W2, S->b1, S->b2};
  k_ml_forward_rows<<<(n + INF_ROWS - 1) / INF_ROWS, 256, INF_SMEM, s>>>(w, dX, n, dY); count_launch();
  M3_CUDA(cudaMemcpyAsync(hY, dY, sizeof(float) * n * OUT, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  cudaFree(dX);
  cudaFree(dY);
  return M3SPH_OK;
}

int ml_get_params(m3sph_mesh *M, float *h) {
  MlState *S = mls(M);
  M3_CUDA(cudaMemcpy(h, S->params, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return M3SPH_OK;
}

int ml_nparam() { return NPARAM; }
long ml_count(m3sph_mesh *M) { return M->ml ? mls(M)->count : 0; }
void ml_mark_trained(m3sph_mesh *M, bool t) {
  if (M->ml) mls(M)->trained = t;
}

}  // namespace m3sph
