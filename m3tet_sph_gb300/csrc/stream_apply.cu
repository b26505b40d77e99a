// Streamed element-by-element apply of the finest-level FP32 operator, y = sum_e K_e x_e
// (the matrix-free product of mgpcg_solver_p.m:388-596 with the stored element matrices).
//
// Phase 1, one persistent launch: CTAs take chunks of 32 consecutive stored elements by ticket.
//   * a producer warp streams a chunk's packed matrices into a 3-stage shared-memory ring with one
//     2D TMA tensor load (117 rows x 512 B, L2 evict-first) and the chunk's connectivity with one
//     bulk copy, both completing on mbarriers;
//   * two consumer groups of 4 warps take alternate chunks: gather x while the matrices are in
//     flight, form the products from shared memory (warp w does rows [117w/4, 117(w+1)/4)), sum the
//     four partial results and store the element outputs Ye[e][30] (coalesced).
// Phase 2: y at every node is the sum of its incident element outputs, taken in element order from
// a node -> (element, local node) table. No atomics and no waits between CTAs: the result does not
// depend on scheduling. Every wait is bounded in time; a wait that gives up sets a bit of the
// level's error word instead of hanging.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>
#include <type_traits>

#include "common.cuh"

namespace m3sph {
namespace sa {
constexpr int E = 32;                         // elements per chunk
constexpr int NST = 3;                        // matrix stages
constexpr int NGRP = 2;                       // consumer groups of 4 warps
constexpr int ROWS = 117;                     // float4 rows of a packed FP32 element matrix
constexpr int KBYTES = ROWS * E * 16;         // 59,904 B per stage
constexpr int KSTRIDE = 60416;                // stage stride (multiple of 1024)
constexpr int CBYTES = 10 * E * 4;            // connectivity of a chunk
constexpr int XBYTES = 30 * E * 4;            // gathered x of a chunk
constexpr int SY_LD = 33;
constexpr int OFF_K = 0;
constexpr int OFF_CX = OFF_K + NST * KSTRIDE;              // slot: connectivity, then x
constexpr unsigned long long TIMEOUT_NS = 1000000000ull;
static_assert(KBYTES <= KSTRIDE && KSTRIDE % 1024 == 0, "stage layout");
static_assert(4 * 30 * SY_LD * 4 <= KBYTES, "partial sums fit in a matrix stage");
// layout for NCX connectivity + gathered-x slots and NGW gather warps
template <int NCX, int NGW> struct Lay {
  static constexpr int THREADS = NGRP * 128 + NGW * 32 + 32;   // + one producer warp
  static constexpr int OFF_HDR = OFF_CX + NCX * (CBYTES + XBYTES);
  static constexpr int HDR_BYTES = ((16 * NCX + 63) / 64) * 64;   // one int4 header per slot
  static constexpr int OFF_KTAG = OFF_HDR + HDR_BYTES;            // use tags of the matrix stages
  static constexpr int OFF_BAR = OFF_KTAG + 64;   // (the partial sums of a chunk reuse its matrix stage)
  static constexpr int NBAR = 2 * NST + 3 * NCX;
  static constexpr int SMEM = OFF_BAR + NBAR * 8;
  static constexpr int SMEM_ALLOC = SMEM + 1024;    // room to align the base to 1024 B
  static_assert(SMEM_ALLOC <= 232448, "shared memory budget");
  static_assert(16 * NCX <= HDR_BYTES && 4 * NST <= 64, "header and tag areas");
};
}  // namespace sa

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// wait for the phase with this parity to complete; false after TIMEOUT_NS
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = gtime();
  for (;;) {
    for (int i = 0; i < 32; ++i)
      if (mbar_test(bar, parity)) return true;
    if (gtime() - t0 > sa::TIMEOUT_NS) return false;
  }
}
__device__ __forceinline__ uint64_t evict_first_policy() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
// Wait for use u of a ring barrier when several waiters take turns on the ring: a waiter may run
// a full ring ahead, and then the phase parity alone cannot tell use u from the still-pending use
// u - depth. The producer writes the tag u before arming the barrier for use u, which it only does
// after use u - depth has completed; so the tag is read first and the parity trusted after.
__device__ __forceinline__ bool ring_wait(uint32_t bar, uint32_t parity, const volatile int *tag, int u) {
  if (*tag == u && mbar_test(bar, parity)) return true;
  const unsigned long long t0 = gtime();
  for (;;) {
    for (int i = 0; i < 32; ++i)
      if (*tag == u && mbar_test(bar, parity)) return true;
    if (gtime() - t0 > sa::TIMEOUT_NS) return false;
  }
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar,
                                            uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar), "l"(policy)
      : "memory");
}
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
// barrier of one consumer group (128 threads) that also ANDs a predicate over the group
__device__ __forceinline__ bool group_and(int g, bool v) {
  uint32_t out;
  __syncwarp();
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, %2, 128, p;\n selp.u32 %0, 1, 0, q;\n}"
      : "=r"(out)
      : "r"((uint32_t)v), "r"(g + 1)
      : "memory");
  return out != 0;
}
__device__ __forceinline__ void group_sync(int g) {
  __syncwarp();
  asm volatile("bar.sync %0, 128;" ::"r"(g + 1) : "memory");
}

template <int k>
__device__ __forceinline__ void packed_mac(float v, const float (&x)[30], float (&y)[30]) {
  if constexpr (k < NPACK) {
    constexpr int c = unpack_c(k), r = unpack_r(k);
    y[r] += v * x[c];
    if constexpr (r != c) y[c] += v * x[r];
  }
}
template <int Q0, int... Is>
__device__ __forceinline__ void rows_mac(const float4 *rows, const float (&x)[30], float (&y)[30],
                                         std::integer_sequence<int, Is...>) {
  auto one = [&](auto qc) {
    constexpr int Q = decltype(qc)::value;
    const float4 v = rows[Q * sa::E];
    packed_mac<4 * Q + 0>(v.x, x, y);
    packed_mac<4 * Q + 1>(v.y, x, y);
    packed_mac<4 * Q + 2>(v.z, x, y);
    packed_mac<4 * Q + 3>(v.w, x, y);
  };
  (one(std::integral_constant<int, Q0 + Is>{}), ...);
}
template <int P>
__device__ __forceinline__ void part_mac(const float4 *rows, const float (&x)[30], float (&y)[30]) {
  constexpr int b = (sa::ROWS * P) / 4, e = (sa::ROWS * (P + 1)) / 4;
  rows_mac<b>(rows, x, y, std::make_integer_sequence<int, e - b>{});
}

}  // namespace

template <int NCX, int NGW>
__global__ void __launch_bounds__(sa::Lay<NCX, NGW>::THREADS, 1)
    k_stream_elem_f32(const __grid_constant__ CUtensorMap tmK, const int *__restrict__ conn, int nchunk, int nel,
                      int *__restrict__ ticket, int *__restrict__ err, const float *__restrict__ x,
                      float *__restrict__ ye) {
  using namespace sa;
  using Ly = Lay<NCX, NGW>;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t bar0 = smem_u32(sm + Ly::OFF_BAR);
  // matrix ring: full_k / empty_k; slot ring: conn landed / x gathered / slot free
  auto full_k = [&](int s) { return bar0 + 8u * s; };
  auto empty_k = [&](int s) { return bar0 + 8u * (NST + s); };
  auto cx_conn = [&](int j) { return bar0 + 8u * (2 * NST + j); };
  auto cx_x = [&](int j) { return bar0 + 8u * (2 * NST + NCX + j); };
  auto cx_empty = [&](int j) { return bar0 + 8u * (2 * NST + 2 * NCX + j); };
  auto slot_conn = [&](int j) { return reinterpret_cast<int *>(sm + OFF_CX + j * (CBYTES + XBYTES)); };
  auto slot_x = [&](int j) { return reinterpret_cast<float *>(sm + OFF_CX + j * (CBYTES + XBYTES) + CBYTES); };
  int4 *hdr = reinterpret_cast<int4 *>(sm + Ly::OFF_HDR);   // {first element, count, ticket, use tag}
  int *ktag = reinterpret_cast<int *>(sm + Ly::OFF_KTAG);
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(full_k(s), 1);
      mbar_init(empty_k(s), 1);
      ktag[s] = -1;
    }
    for (int j = 0; j < NCX; ++j) {
      hdr[j] = make_int4(0, 0, 0, -1);
      mbar_init(cx_conn(j), 1);
      mbar_init(cx_x(j), 1);
      mbar_init(cx_empty(j), 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  const int gw0 = NGRP * 4;          // first gather warp
  const int pw = gw0 + NGW;          // producer warp
  if (warp == pw) {
    // ---------------- producer: connectivity one chunk ahead of the matrices ----------------
    if (lane != 0) return;
    const uint64_t pol = evict_first_policy();
    bool ok = true;
    auto issue_k = [&](int m) -> bool {
      const int s = m % NST;
      if (m >= NST && !mbar_wait(empty_k(s), ((m / NST) & 1) ^ 1)) return false;
      reinterpret_cast<volatile int *>(ktag)[s] = m;
      mbar_arrive_tx(full_k(s), KBYTES);
      tma_load_2d(smem_u32(sm + OFF_K + s * KSTRIDE), &tmK, 4 * hdr[m % NCX].x, 0, full_k(s), pol);
      return true;
    };
    int i = 0;
    for (;; ++i) {
      const int j = i % NCX;
      if (i >= NCX && !mbar_wait(cx_empty(j), ((i / NCX) & 1) ^ 1)) {
        ok = false;
        break;
      }
      const int t = atomicAdd(ticket, 1);
      if (t >= nchunk) break;
      const int e0 = t * E;
      hdr[j] = make_int4(e0, min(E, nel - e0), t, i);
      mbar_arrive_tx(cx_conn(j), CBYTES);
      bulk_load(smem_u32(slot_conn(j)), conn + (size_t)t * (10 * E), CBYTES, cx_conn(j));
      if (i >= 1 && !issue_k(i - 1)) {
        ok = false;
        break;
      }
    }
    if (ok && i >= 1 && !issue_k(i - 1)) ok = false;
    // end markers at chunk indices i .. i + max(NGRP, NGW) - 1: consecutive indices reach every
    // gather warp and every consumer group
    constexpr int NEND = NGRP > NGW ? NGRP : NGW;
    for (int m = i; ok && m < i + NEND; ++m) {
      const int j = m % NCX;
      if (m >= NCX && !mbar_wait(cx_empty(j), ((m / NCX) & 1) ^ 1)) {
        ok = false;
        break;
      }
      hdr[j] = make_int4(0, -1, 0, m);
      mbar_arrive(cx_conn(j));
    }
    if (!ok) {
      atomicOr(err, 1);
      // let the copies already issued land before the block can exit
      for (int m = i - 1; m >= 0 && m >= i - NST; --m) mbar_wait(full_k(m % NST), (m / NST) & 1);
      for (int m = i - 1; m >= 0 && m >= i - NCX; --m) mbar_wait(cx_conn(m % NCX), (m / NCX) & 1);
    }
    return;
  }

  if (warp >= gw0) {
    // ---------------- gather warps: x of the chunk's 30 dofs per element ----------------
    for (int m = warp - gw0;; m += NGW) {
      const int j = m % NCX;
      if (!__all_sync(0xffffffffu, ring_wait(cx_conn(j), (m / NCX) & 1, &hdr[j].w, m))) {
        if (lane == 0) atomicOr(err, 16);
        break;
      }
      const int4 c = hdr[j];
      if (c.y >= 0) {
        const int *cs = slot_conn(j);
        float *xs = slot_x(j);
        float v[30];
#pragma unroll
        for (int q = 0; q < 30; ++q) v[q] = lane < c.y ? x[3 * cs[(q / 3) * E + lane] + q % 3] : 0.f;
#pragma unroll
        for (int q = 0; q < 30; ++q) xs[q * E + lane] = v[q];
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(cx_x(j));
      if (c.y < 0) break;
    }
    return;
  }

  // ---------------- consumers ----------------
  const int g = warp >> 2, w = warp & 3, t = tid & 127;
  for (int m = g;; m += NGRP) {
    const int j = m % NCX, s = m % NST;
    if (!group_and(g, ring_wait(cx_x(j), (m / NCX) & 1, &hdr[j].w, m))) {
      if (t == 0) atomicOr(err, 2);
      break;
    }
    const int4 c = hdr[j];
    if (c.y < 0) break;
    const float *xs = slot_x(j);
    float xh[30], yv[30];
#pragma unroll
    for (int q = 0; q < 30; ++q) {
      xh[q] = xs[q * E + lane];
      yv[q] = 0.f;
    }
    const bool kok = ring_wait(full_k(s), (m / NST) & 1, &ktag[s], m);
    unsigned char *stage = sm + OFF_K + s * KSTRIDE;
    const float4 *rows = reinterpret_cast<const float4 *>(stage) + lane;
    switch (w) {
      case 0: part_mac<0>(rows, xh, yv); break;
      case 1: part_mac<1>(rows, xh, yv); break;
      case 2: part_mac<2>(rows, xh, yv); break;
      default: part_mac<3>(rows, xh, yv); break;
    }
    // every warp has its x in registers and is done with the matrix rows
    if (!group_and(g, kok)) {
      if (t == 0) atomicOr(err, 4);
      break;
    }
    if (t == 0) mbar_arrive(cx_empty(j));
    // the four partial sums go into the consumed stage; it is released after the outputs are written
    float *sY = reinterpret_cast<float *>(stage);
#pragma unroll
    for (int q = 0; q < 30; ++q) sY[(w * 30 + q) * SY_LD + lane] = yv[q];
    group_sync(g);
    // element outputs, 30 consecutive values per element (contiguous over the chunk)
    float *yo = ye + (size_t)c.x * 30;
    for (int i = t; i < 30 * c.y; i += 128) {
      const int el = i / 30, q = i - 30 * el;
      yo[i] = sY[q * SY_LD + el] + sY[(30 + q) * SY_LD + el] + sY[(60 + q) * SY_LD + el] + sY[(90 + q) * SY_LD + el];
    }
    // order this thread's generic writes to the stage before the next TMA write into it
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    group_sync(g);
    if (t == 0) mbar_arrive(empty_k(s));
  }
}

// phase 2: y at node n = sum over the node's (element, local node) entries in element order
__global__ void k_node_gather_f32(const int *__restrict__ ptr, const int *__restrict__ idx, int nnod,
                                  const float *__restrict__ ye, float *__restrict__ y) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnod) return;
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  const int b = ptr[n], e = ptr[n + 1];
  for (int j = b; j < e; ++j) {
    // the triple starts at 30 e + 3 n: 8-byte aligned for even n; one 8-byte and one 4-byte load
    // at per-thread offsets (no branch)
    const int o = idx[j], odd = o & 1;
    const float2 v2 = *reinterpret_cast<const float2 *>(ye + o + odd);
    const float v1 = ye[o + 2 * (1 - odd)];
    s0 += odd ? v1 : v2.x;
    s1 += odd ? v2.x : v2.y;
    s2 += odd ? v2.y : v1;
  }
  y[3 * (size_t)n] = s0;
  y[3 * (size_t)n + 1] = s1;
  y[3 * (size_t)n + 2] = s2;
}

// ---------------------------------------------------------------------------------------
// FP64-accurate operators, row-per-lane form: a stage holds 8 elements (one 128-byte TMA row per
// packed row, 128-byte swizzle so the 16-byte piece of element e in row q sits at e ^ (q & 7)).
// Each consumer warp owns whole stages; lane r < 30 forms output row r of each element,
// y_r = sum_c K_rc x_c, reading K_rc from the packed lower triangle (k = pack(max, min)), with
// x_c broadcast from shared memory. The code per element is 30 unrolled multiply-adds, so it stays
// in the instruction cache; two elements are interleaved for instruction-level parallelism.
// ---------------------------------------------------------------------------------------
namespace sr {
constexpr int E = 8;
constexpr int NST = 7;
constexpr int ARR = 15360;                    // array stride inside a stage (multiple of 1024)
constexpr int KSTRIDE = 30720;                // stage stride
constexpr int CBYTES = 10 * E * 4;
template <int NCW> struct Map {
  static constexpr int THREADS = 32 * (NCW + 1);
  static constexpr int OFF_K = 0;
  static constexpr int OFF_CONN = OFF_K + NST * KSTRIDE;
  static constexpr int OFF_HDR = OFF_CONN + NST * CBYTES;
  static constexpr int OFF_XS = OFF_HDR + 128;
  static constexpr int OFF_BAR = OFF_XS + NCW * E * 30 * 8;
  static constexpr int SMEM = OFF_BAR + 2 * NST * 8;
  static constexpr int SMEM_ALLOC = SMEM + 1024;
  static_assert(SMEM_ALLOC <= 232448, "shared memory budget");
};
}  // namespace sr

struct RlDF {   // double-float: K_hi, K_lo as FP32 (117 float4 rows), x split into FP32 hi + lo
  static constexpr int NARR = 2, ROWS = 117, V = 4;
  static constexpr int ARR_BYTES = ROWS * 128;
  struct Acc {
    float h, l;
  };
  __device__ __forceinline__ static int base(int k) {
    const int q = k >> 2;
    return (q * 32 + (k & 3)) ^ ((q & 7) << 2);
  }
  __device__ __forceinline__ static int eshift(int e) { return e << 2; }
  __device__ __forceinline__ static void mac(const unsigned char *st, int off, float2 xv, Acc &a) {
    const float vh = reinterpret_cast<const float *>(st)[off];
    const float vl = reinterpret_cast<const float *>(st + sr::ARR)[off];
    df_mac(vh, vl, xv.x, xv.y, a.h, a.l);
  }
  __device__ __forceinline__ static float2 xsplit(double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
  }
  __device__ __forceinline__ static double finish(const Acc &a) { return (double)a.h + (double)a.l; }
};
struct RlF64 {  // FP64: K as 233 double2 rows
  static constexpr int NARR = 1, ROWS = 233, V = 2;
  static constexpr int ARR_BYTES = ROWS * 128;
  struct Acc {
    double h;
  };
  __device__ __forceinline__ static int base(int k) {
    const int q = k >> 1;
    return (q * 16 + (k & 1)) ^ ((q & 7) << 1);
  }
  __device__ __forceinline__ static int eshift(int e) { return e << 1; }
  __device__ __forceinline__ static void mac(const unsigned char *st, int off, double xv, Acc &a) {
    a.h = fma(reinterpret_cast<const double *>(st)[off], xv, a.h);
  }
  __device__ __forceinline__ static double xsplit(double v) { return v; }
  __device__ __forceinline__ static double finish(const Acc &a) { return a.h; }
};
static_assert(RlDF::ARR_BYTES <= sr::ARR && RlF64::ARR_BYTES <= sr::KSTRIDE, "row-lane stage layout");
static_assert(sizeof(decltype(RlDF::xsplit(0.0))) == 8 && sizeof(decltype(RlF64::xsplit(0.0))) == 8,
              "x entries are 8 bytes in the per-warp buffer");

template <class Op, int NCW, int EG, int SPLIT>
__global__ void __launch_bounds__(32 * (NCW * SPLIT + 1), 1)
    k_stream_rowlane(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const int *__restrict__ conn, int nchunk, int nel, int *__restrict__ ticket,
                     int *__restrict__ err, const double *__restrict__ x, double *__restrict__ ye) {
  using namespace sr;
  using Mp = Map<NCW>;
  using XV = decltype(Op::xsplit(0.0));
  extern __shared__ unsigned char smem_raw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t bar0 = smem_u32(sm + Mp::OFF_BAR);
  auto full = [&](int s) { return bar0 + 8u * s; };
  auto empty = [&](int s) { return bar0 + 8u * (NST + s); };
  int4 *hdr = reinterpret_cast<int4 *>(sm + Mp::OFF_HDR);   // {first element, count, ticket, use tag}
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), SPLIT);
      hdr[s] = make_int4(0, 0, 0, -1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  if (warp == NCW * SPLIT) {
    // ---------------- producer ----------------
    if (lane != 0) return;
    const uint64_t pol = evict_first_policy();
    int it = 0;
    bool ok = true;
    for (;; ++it) {
      const int s = it % NST;
      if (it >= NST && !mbar_wait(empty(s), ((it / NST) & 1) ^ 1)) {
        ok = false;
        break;
      }
      const int t = atomicAdd(ticket, 1);
      if (t >= nchunk) break;
      const int e0 = t * E;
      hdr[s] = make_int4(e0, min(E, nel - e0), t, it);
      mbar_arrive_tx(full(s), CBYTES + Op::NARR * Op::ARR_BYTES);
      bulk_load(smem_u32(sm + Mp::OFF_CONN + s * CBYTES), conn + (size_t)t * (10 * E), CBYTES, full(s));
      const uint32_t dst = smem_u32(sm + Mp::OFF_K + s * KSTRIDE);
      tma_load_2d(dst, &tmA, Op::V * e0, 0, full(s), pol);
      if (Op::NARR == 2) tma_load_2d(dst + ARR, &tmB, Op::V * e0, 0, full(s), pol);
    }
    for (int j = 0; ok && j < NCW; ++j, ++it) {
      const int s = it % NST;
      if (it >= NST && !mbar_wait(empty(s), ((it / NST) & 1) ^ 1)) {
        ok = false;
        break;
      }
      hdr[s] = make_int4(0, -1, 0, it);
      mbar_arrive(full(s));
    }
    if (!ok) {
      atomicOr(err, 1);
      for (int j = 1; j <= NST && it - j >= 0; ++j) {
        const int i2 = it - j;
        mbar_wait(full(i2 % NST), (i2 / NST) & 1);
      }
    }
    return;
  }

  // ---------------- consumers: SPLIT warps per stage, each with E / SPLIT elements ----------------
  constexpr int EW = E / SPLIT;
  constexpr int EGI = EG < EW ? EG : EW;   // elements interleaved per pass
  const int owner = warp / SPLIT, part = warp % SPLIT, eb = part * EW;
  const int r = lane < 30 ? lane : 29;
  int base[30];
#pragma unroll
  for (int c = 0; c < 30; ++c) base[c] = Op::base(r >= c ? pack_idx(r, c) : pack_idx(c, r));
  XV *xs = reinterpret_cast<XV *>(sm + Mp::OFF_XS + warp * EW * 30 * 8);
  for (int it = owner;; it += NCW) {
    const int s = it % NST;
    const uint32_t par = (it / NST) & 1;
    if (!__all_sync(0xffffffffu, ring_wait(full(s), par, &hdr[s].w, it))) {
      if (lane == 0) atomicOr(err, 2);
      break;
    }
    const int4 h = hdr[s];
    if (h.y < 0) break;
    const int ne = min(EW, h.y - eb);   // elements of this warp (may be <= 0 in the last chunk)
    const int *cs = reinterpret_cast<const int *>(sm + Mp::OFF_CONN + s * CBYTES);
    if (lane < 30) {
      double xv[EW];
#pragma unroll
      for (int e = 0; e < EW; ++e) xv[e] = e < ne ? x[3 * cs[(lane / 3) * E + eb + e] + lane % 3] : 0.0;
#pragma unroll
      for (int e = 0; e < EW; ++e) xs[e * 30 + lane] = Op::xsplit(xv[e]);
    }
    __syncwarp();
    const unsigned char *st = sm + Mp::OFF_K + s * KSTRIDE;
    double *yo = ye + (size_t)(h.x + eb) * 30;
    for (int e = 0; e < ne; e += EGI) {
      typename Op::Acc a[EGI];
#pragma unroll
      for (int g = 0; g < EGI; ++g) a[g] = typename Op::Acc{};
      const XV *xe = xs + e * 30;
#pragma unroll
      for (int c = 0; c < 30; ++c) {
#pragma unroll
        for (int g = 0; g < EGI; ++g) Op::mac(st, base[c] ^ Op::eshift(eb + e + g), xe[g * 30 + c], a[g]);
      }
      if (lane < 30) {
#pragma unroll
        for (int g = 0; g < EGI; ++g)
          if (e + g < ne) yo[(e + g) * 30 + lane] = Op::finish(a[g]);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty(s));
  }
}

// phase 2 fused with a weighted Jacobi sweep: (K d)_n is complete once gathered, so
// d_n += w (r_n - (K d)_n) / diag_n follows in the same pass (d_n is read only by its own node)
__global__ void k_node_gather_jac_f32(const int *__restrict__ ptr, const int *__restrict__ idx, int nnod,
                                      const float *__restrict__ ye, float w, const float *__restrict__ r,
                                      const float *__restrict__ Di, float *__restrict__ d) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnod) return;
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  const int b = ptr[n], e = ptr[n + 1];
  for (int j = b; j < e; ++j) {
    // the triple starts at 30 e + 3 n: 8-byte aligned for even n; one 8-byte and one 4-byte load
    // at per-thread offsets (no branch)
    const int o = idx[j], odd = o & 1;
    const float2 v2 = *reinterpret_cast<const float2 *>(ye + o + odd);
    const float v1 = ye[o + 2 * (1 - odd)];
    s0 += odd ? v1 : v2.x;
    s1 += odd ? v2.x : v2.y;
    s2 += odd ? v2.y : v1;
  }
  const size_t i = 3 * (size_t)n;
  d[i] += w * (r[i] - s0) * Di[i];
  d[i + 1] += w * (r[i + 1] - s1) * Di[i + 1];
  d[i + 2] += w * (r[i + 2] - s2) * Di[i + 2];
}

__global__ void k_node_gather_f64(const int *__restrict__ ptr, const int *__restrict__ idx, int nnod,
                                  const double *__restrict__ ye, double *__restrict__ y) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnod) return;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  const int b = ptr[n], e = ptr[n + 1];
  for (int j = b; j < e; ++j) {
    const int o = idx[j], odd = o & 1;   // 16-byte aligned pair for even n, as in the FP32 gather
    const double2 v2 = *reinterpret_cast<const double2 *>(ye + o + odd);
    const double v1 = ye[o + 2 * (1 - odd)];
    s0 += odd ? v1 : v2.x;
    s1 += odd ? v2.x : v2.y;
    s2 += odd ? v2.y : v1;
  }
  y[3 * (size_t)n] = s0;
  y[3 * (size_t)n + 1] = s1;
  y[3 * (size_t)n + 2] = s2;
}

// ---------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------
__global__ void k_chunk_conn(const int *__restrict__ el2nod, int nel, int nchunk, int E, int *__restrict__ conn) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)nchunk * 10 * E) return;
  const int ch = (int)(i / (10 * E)), r = (int)(i % (10 * E)), n = r / E, el = r % E;
  const int e = ch * E + el;
  conn[i] = e < nel ? el2nod[(size_t)n * nel + e] : 0;
}

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;
static cudaError_t g_encode_status = cudaSuccess;

template <class Op> static int rowlane_attrs();
static int f32_attrs();

int stream_build(Level &L, const std::vector<int> &perm, cudaStream_t s) {
  std::call_once(g_encode_once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    g_encode_status = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (g_encode_status == cudaSuccess && q != cudaDriverEntryPointSuccess) g_encode_status = cudaErrorNotSupported;
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  if (g_encode_status != cudaSuccess || !g_encode) return cuda_fail(g_encode_status, "cuTensorMapEncodeTiled lookup");
  const int nel = L.nel, nnod = L.nnod;
  L.nchunk = (nel + sa::E - 1) / sa::E;
  L.nchunk8 = (nel + sr::E - 1) / sr::E;
  // node -> (element, local node) table in stored element order
  std::vector<int> ptr(nnod + 1, 0), idx((size_t)nel * 10);
  for (int p = 0; p < nel; ++p)
    for (int n = 0; n < 10; ++n) ptr[L.h_el2nod_orig[(size_t)perm[p] * 10 + n] + 1]++;
  for (int i = 0; i < nnod; ++i) ptr[i + 1] += ptr[i];
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int p = 0; p < nel; ++p)
    for (int n = 0; n < 10; ++n) idx[fill[L.h_el2nod_orig[(size_t)perm[p] * 10 + n]]++] = p * 30 + 3 * n;
  M3_CUDA(cudaMalloc(&L.chunk_conn, sizeof(int) * (size_t)L.nchunk * 10 * sa::E));
  M3_CUDA(cudaMalloc(&L.ye32, sizeof(float) * (size_t)nel * 30));
  M3_CUDA(cudaMalloc(&L.chunk_conn8, sizeof(int) * (size_t)L.nchunk8 * 10 * sr::E));
  M3_CUDA(cudaMalloc(&L.ye64, sizeof(double) * (size_t)nel * 30));
  M3_CUDA(cudaMalloc(&L.g_ptr, sizeof(int) * ptr.size()));
  M3_CUDA(cudaMalloc(&L.g_idx, sizeof(int) * idx.size()));
  M3_CUDA(cudaMalloc(&L.sa_err, sizeof(int) * 2));   // [0] error bits, [1] chunk ticket
  M3_CUDA(cudaMemcpyAsync(L.g_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(L.g_idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemsetAsync(L.sa_err, 0, sizeof(int) * 2, s));
  const size_t n = (size_t)L.nchunk * 10 * sa::E, n8 = (size_t)L.nchunk8 * 10 * sr::E;
  k_chunk_conn<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(L.el2nod, nel, L.nchunk, sa::E, L.chunk_conn);
  count_launch();
  k_chunk_conn<<<(unsigned)((n8 + 255) / 256), 256, 0, s>>>(L.el2nod, nel, L.nchunk8, sr::E, L.chunk_conn8);
  count_launch();
  M3_CUDA(cudaGetLastError());
  M3_TRY(f32_attrs());
  M3_TRY(rowlane_attrs<RlDF>());
  M3_TRY(rowlane_attrs<RlF64>());
  int dev = 0, nsm = 0;
  M3_CUDA(cudaGetDevice(&dev));
  M3_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  L.sa_grid = std::max(1, std::min(nsm, L.nchunk));
  // the host copies above read stack vectors: finish them before they go out of scope
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

// 2D view of a packed operator [rows][V nel] of FP32 (V = 4) or FP64 (V = 2) values; a box covers
// E elements x all rows
static int encode_k(const Level &L, const void *K, bool f64, int rows, int E, CUtensorMap *map, bool swz = false) {
  const int V = f64 ? 2 : 4;
  const cuuint64_t dims[2] = {(cuuint64_t)L.nel * V, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)L.nel * 16};
  const cuuint32_t box[2] = {(cuuint32_t)(V * E), (cuuint32_t)rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = g_encode(map, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                              const_cast<void *>(K), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              swz ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return M3SPH_ERR_CUDA;
  }
  return M3SPH_OK;
}
static int encode_k32(const Level &L, const float *K, CUtensorMap *map) { return encode_k(L, K, false, sa::ROWS, sa::E, map); }

static int stream_ready(const Level &L, const void *K) {
  if (!L.nchunk || !g_encode) {
    set_error("streamed apply not built for this level");
    return M3SPH_ERR_BAD_INPUT;
  }
  if (!K || (reinterpret_cast<uintptr_t>(K) & 15) != 0) {
    set_error("streamed apply: element matrices missing or not 16-byte aligned");
    return M3SPH_ERR_BAD_INPUT;
  }
  return M3SPH_OK;
}

// FP32 streamed kernel variants: (connectivity/x slots, gather warps)
static int g_f32_variant = 0;
template <int NCX, int NGW>
static int f32_attr() {
  M3_CUDA(cudaFuncSetAttribute(k_stream_elem_f32<NCX, NGW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               sa::Lay<NCX, NGW>::SMEM_ALLOC));
  return M3SPH_OK;
}
static int f32_attrs() {
  M3_TRY((f32_attr<6, 2>()));
  M3_TRY((f32_attr<8, 2>()));
  M3_TRY((f32_attr<6, 3>()));
  M3_TRY((f32_attr<8, 3>()));
  return M3SPH_OK;
}
int stream_set_f32_variant(int v) {
  if (v < 0 || v > 3) {
    set_error("stream_f32_variant must be 0..3");
    return M3SPH_ERR_BAD_INPUT;
  }
  g_f32_variant = v;
  return M3SPH_OK;
}
template <int NCX, int NGW>
static void f32_launch(const Level &L, const CUtensorMap &map, const float *x, cudaStream_t s) {
  k_stream_elem_f32<NCX, NGW><<<L.sa_grid, sa::Lay<NCX, NGW>::THREADS, sa::Lay<NCX, NGW>::SMEM_ALLOC, s>>>(
      map, L.chunk_conn, L.nchunk, L.nel, L.sa_err + 1, L.sa_err, x, L.ye32);
}
static void f32_phase1(const Level &L, const CUtensorMap &map, const float *x, cudaStream_t s) {
  switch (g_f32_variant) {
    case 1: f32_launch<8, 2>(L, map, x, s); break;
    case 2: f32_launch<6, 3>(L, map, x, s); break;
    case 3: f32_launch<8, 3>(L, map, x, s); break;
    default: f32_launch<6, 2>(L, map, x, s); break;
  }
}

int stream_apply_f32(const Level &L, const float *K, const float *x, float *y, cudaStream_t s) {
  M3_TRY(stream_ready(L, K));
  CUtensorMap map;
  M3_TRY(encode_k32(L, K, &map));
  M3_CUDA(cudaMemsetAsync(L.sa_err + 1, 0, sizeof(int), s));
  f32_phase1(L, map, x, s);
  count_launch();
  k_node_gather_f32<<<(L.nnod + 255) / 256, 256, 0, s>>>(L.g_ptr, L.g_idx, L.nnod, L.ye32, y);
  count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// row-per-lane kernels. Double-float: `owners` warps-groups own stages in turn, SPLIT warps share a
// stage (E / SPLIT elements each), 2 elements interleaved; FP64: 6 owners, one warp per stage.
struct RlShape {
  int owners, split;
};
static const RlShape RL_DF_SHAPES[] = {{6, 1}, {6, 2}, {5, 2}, {4, 2}, {4, 4}, {5, 4}, {6, 4}, {3, 8}};
static int g_rowlane_variant = 4;
int stream_set_outer_warps(int n) {
  if (n < 0 || n >= (int)(sizeof(RL_DF_SHAPES) / sizeof(RL_DF_SHAPES[0]))) {
    set_error("stream_outer_variant out of range");
    return M3SPH_ERR_BAD_INPUT;
  }
  g_rowlane_variant = n;
  return M3SPH_OK;
}

template <class Op, int NCW, int SPLIT>
static int rowlane_attr() {
  M3_CUDA(cudaFuncSetAttribute(k_stream_rowlane<Op, NCW, 2, SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               sr::Map<NCW>::SMEM_ALLOC));
  return M3SPH_OK;
}
template <class Op>
static int rowlane_attrs() {
  if constexpr (std::is_same<Op, RlF64>::value) {
    return rowlane_attr<Op, 6, 1>();
  } else {
    M3_TRY((rowlane_attr<Op, 6, 1>()));
    M3_TRY((rowlane_attr<Op, 6, 2>()));
    M3_TRY((rowlane_attr<Op, 5, 2>()));
    M3_TRY((rowlane_attr<Op, 4, 2>()));
    M3_TRY((rowlane_attr<Op, 4, 4>()));
    M3_TRY((rowlane_attr<Op, 5, 4>()));
    M3_TRY((rowlane_attr<Op, 6, 4>()));
    M3_TRY((rowlane_attr<Op, 3, 8>()));
    return M3SPH_OK;
  }
}

template <class Op, int NCW, int SPLIT>
static void rowlane_launch(const Level &L, const CUtensorMap &ma, const CUtensorMap &mb, const double *x, cudaStream_t s) {
  k_stream_rowlane<Op, NCW, 2, SPLIT><<<L.sa_grid, 32 * (NCW * SPLIT + 1), sr::Map<NCW>::SMEM_ALLOC, s>>>(
      ma, mb, L.chunk_conn8, L.nchunk8, L.nel, L.sa_err + 1, L.sa_err, x, L.ye64);
}

template <class Op>
static int rowlane_apply(const Level &L, const CUtensorMap &ma, const CUtensorMap &mb, const double *x, double *y,
                         cudaStream_t s) {
  M3_CUDA(cudaMemsetAsync(L.sa_err + 1, 0, sizeof(int), s));
  if constexpr (std::is_same<Op, RlF64>::value) {
    rowlane_launch<RlF64, 6, 1>(L, ma, mb, x, s);
  } else {
    switch (g_rowlane_variant) {
      case 0: rowlane_launch<Op, 6, 1>(L, ma, mb, x, s); break;
      case 2: rowlane_launch<Op, 5, 2>(L, ma, mb, x, s); break;
      case 3: rowlane_launch<Op, 4, 2>(L, ma, mb, x, s); break;
      case 4: rowlane_launch<Op, 4, 4>(L, ma, mb, x, s); break;
      case 5: rowlane_launch<Op, 5, 4>(L, ma, mb, x, s); break;
      case 6: rowlane_launch<Op, 6, 4>(L, ma, mb, x, s); break;
      case 7: rowlane_launch<Op, 3, 8>(L, ma, mb, x, s); break;
      case 1: rowlane_launch<Op, 6, 2>(L, ma, mb, x, s); break;
      default: rowlane_launch<Op, 4, 4>(L, ma, mb, x, s); break;
    }
  }
  count_launch();
  k_node_gather_f64<<<(L.nnod + 255) / 256, 256, 0, s>>>(L.g_ptr, L.g_idx, L.nnod, L.ye64, y);
  count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// d += w (r - K d) / diag with K d from the streamed apply (one weighted Jacobi sweep)
int stream_apply_jac_f32(const Level &L, const float *K, float w, const float *r, const float *Di, float *d,
                         cudaStream_t s) {
  M3_TRY(stream_ready(L, K));
  CUtensorMap map;
  M3_TRY(encode_k32(L, K, &map));
  M3_CUDA(cudaMemsetAsync(L.sa_err + 1, 0, sizeof(int), s));
  f32_phase1(L, map, d, s);
  count_launch();
  k_node_gather_jac_f32<<<(L.nnod + 255) / 256, 256, 0, s>>>(L.g_ptr, L.g_idx, L.nnod, L.ye32, w, r, Di, d);
  count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// y = (K_hi + K_lo) x with FP64 accuracy (double-float arithmetic)
int stream_apply_df(const Level &L, const float *Kh, const float *Kl, const double *x, double *y, cudaStream_t s) {
  M3_TRY(stream_ready(L, Kh));
  M3_TRY(stream_ready(L, Kl));
  CUtensorMap ma, mb;
  M3_TRY(encode_k(L, Kh, false, RlDF::ROWS, sr::E, &ma, true));
  M3_TRY(encode_k(L, Kl, false, RlDF::ROWS, sr::E, &mb, true));
  return rowlane_apply<RlDF>(L, ma, mb, x, y, s);
}

// y = K x in FP64 from the FP64 element matrices
int stream_apply_f64(const Level &L, const double *K, const double *x, double *y, cudaStream_t s) {
  M3_TRY(stream_ready(L, K));
  CUtensorMap ma;
  M3_TRY(encode_k(L, K, true, RlF64::ROWS, sr::E, &ma, true));
  return rowlane_apply<RlF64>(L, ma, ma, x, y, s);
}

// reads (and clears) the error word of the streamed apply
int stream_check(const Level &L, cudaStream_t s) {
  if (!L.sa_err) return M3SPH_OK;
  int h = 0;
  M3_CUDA(cudaMemcpyAsync(&h, L.sa_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  if (h) {
    M3_CUDA(cudaMemsetAsync(L.sa_err, 0, sizeof(int), s));
    set_error("streamed element apply: a bounded wait gave up (code " + std::to_string(h) + ")");
    return M3SPH_ERR_CUDA;
  }
  return M3SPH_OK;
}

}  // namespace m3sph
