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

#include "common.cuh"

namespace m3sph {
namespace sa {
constexpr int E = 32;                         // elements per chunk
constexpr int NST = 3;                        // pipeline stages
constexpr int NGRP = 2;                       // consumer groups of 4 warps
constexpr int THREADS = NGRP * 128 + 32;      // + one producer warp
constexpr int ROWS = 117;                     // float4 rows of a packed FP32 element matrix
constexpr int KBYTES = ROWS * E * 16;         // 59,904 B per stage
constexpr int KSTRIDE = 60416;                // stage stride (multiple of 1024)
constexpr int CBYTES = 10 * E * 4;            // connectivity of a chunk
constexpr int SY_LD = 33;
constexpr int OFF_K = 0;
constexpr int OFF_CONN = OFF_K + NST * KSTRIDE;
constexpr int OFF_HDR = OFF_CONN + NST * CBYTES;
constexpr int OFF_XS = OFF_HDR + 64;
constexpr int OFF_SY = OFF_XS + NGRP * 30 * E * 4;
constexpr int OFF_BAR = OFF_SY + NGRP * 4 * 30 * SY_LD * 4;
constexpr int SMEM = OFF_BAR + 3 * NST * 8;
constexpr int SMEM_ALLOC = SMEM + 1024;       // room to align the base to 1024 B
constexpr unsigned long long TIMEOUT_NS = 1000000000ull;
static_assert(SMEM_ALLOC <= 232448, "shared memory budget");
static_assert(KBYTES <= KSTRIDE && KSTRIDE % 1024 == 0, "stage layout");
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

__global__ void __launch_bounds__(sa::THREADS, 1)
    k_stream_elem_f32(const __grid_constant__ CUtensorMap tmK, const int *__restrict__ conn, int nchunk, int nel,
                      int *__restrict__ ticket, int *__restrict__ err, const float *__restrict__ x,
                      float *__restrict__ ye) {
  using namespace sa;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t bar0 = smem_u32(sm + OFF_BAR);
  auto full_conn = [&](int s) { return bar0 + 8u * s; };
  auto full_k = [&](int s) { return bar0 + 8u * (NST + s); };
  auto empty = [&](int s) { return bar0 + 8u * (2 * NST + s); };
  int4 *hdr = reinterpret_cast<int4 *>(sm + OFF_HDR);
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(full_conn(s), 1);
      mbar_init(full_k(s), 1);
      mbar_init(empty(s), 4);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  if (warp == NGRP * 4) {
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
      hdr[s] = make_int4(e0, min(E, nel - e0), t, 0);
      mbar_arrive_tx(full_conn(s), CBYTES);
      bulk_load(smem_u32(sm + OFF_CONN + s * CBYTES), conn + (size_t)t * (10 * E), CBYTES, full_conn(s));
      mbar_arrive_tx(full_k(s), KBYTES);
      tma_load_2d(smem_u32(sm + OFF_K + s * KSTRIDE), &tmK, 4 * e0, 0, full_k(s), pol);
    }
    // one end marker per consumer group
    for (int j = 0; ok && j < NGRP; ++j, ++it) {
      const int s = it % NST;
      if (it >= NST && !mbar_wait(empty(s), ((it / NST) & 1) ^ 1)) {
        ok = false;
        break;
      }
      hdr[s] = make_int4(0, -1, 0, 0);
      mbar_arrive(full_conn(s));
    }
    if (!ok) {
      atomicOr(err, 1);
      // let the copies already issued land before the block can exit
      for (int j = 1; j <= NST && it - j >= 0; ++j) {
        const int i2 = it - j, s = i2 % NST;
        mbar_wait(full_conn(s), (i2 / NST) & 1);
        mbar_wait(full_k(s), (i2 / NST) & 1);
      }
    }
    return;
  }

  // ---------------- consumers ----------------
  const int g = warp >> 2, w = warp & 3, t = tid & 127;
  float *xs = reinterpret_cast<float *>(sm + OFF_XS) + g * 30 * E;
  float *sY = reinterpret_cast<float *>(sm + OFF_SY) + g * 4 * 30 * SY_LD;
  for (int it = g;; it += NGRP) {
    const int s = it % NST;
    const uint32_t par = (it / NST) & 1;
    // (also the barrier after the previous chunk's reads of xs and sY)
    if (!group_and(g, mbar_wait(full_conn(s), par))) {
      if (t == 0) atomicOr(err, 2);
      break;
    }
    const int4 c = hdr[s];
    if (c.y < 0) break;
    const int *cs = reinterpret_cast<const int *>(sm + OFF_CONN + s * CBYTES);
    for (int i = t; i < 30 * E; i += 128) {
      const int q = i >> 5, el = i & 31;
      xs[i] = el < c.y ? x[3 * cs[(q / 3) * E + el] + q % 3] : 0.f;
    }
    group_sync(g);
    float xh[30], yv[30];
#pragma unroll
    for (int q = 0; q < 30; ++q) {
      xh[q] = xs[q * E + lane];
      yv[q] = 0.f;
    }
    const bool kok = mbar_wait(full_k(s), par);
    const float4 *rows = reinterpret_cast<const float4 *>(sm + OFF_K + s * KSTRIDE) + lane;
    switch (w) {
      case 0: part_mac<0>(rows, xh, yv); break;
      case 1: part_mac<1>(rows, xh, yv); break;
      case 2: part_mac<2>(rows, xh, yv); break;
      default: part_mac<3>(rows, xh, yv); break;
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(empty(s));
#pragma unroll
    for (int q = 0; q < 30; ++q) sY[(w * 30 + q) * SY_LD + lane] = yv[q];
    if (!group_and(g, kok)) {
      if (t == 0) atomicOr(err, 4);
      break;
    }
    // element outputs, 30 consecutive values per element (contiguous over the chunk)
    float *yo = ye + (size_t)c.x * 30;
    for (int i = t; i < 30 * c.y; i += 128) {
      const int el = i / 30, q = i - 30 * el;
      yo[i] = sY[q * SY_LD + el] + sY[(30 + q) * SY_LD + el] + sY[(60 + q) * SY_LD + el] + sY[(90 + q) * SY_LD + el];
    }
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
    const float *p = ye + idx[j];
    s0 += p[0];
    s1 += p[1];
    s2 += p[2];
  }
  y[3 * (size_t)n] = s0;
  y[3 * (size_t)n + 1] = s1;
  y[3 * (size_t)n + 2] = s2;
}

// ---------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------
__global__ void k_chunk_conn(const int *__restrict__ el2nod, int nel, int nchunk, int *__restrict__ conn) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)nchunk * 10 * sa::E) return;
  const int ch = (int)(i / (10 * sa::E)), r = (int)(i % (10 * sa::E)), n = r / sa::E, el = r % sa::E;
  const int e = ch * sa::E + el;
  conn[i] = e < nel ? el2nod[(size_t)n * nel + e] : 0;
}

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;
static cudaError_t g_encode_status = cudaSuccess;

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
  M3_CUDA(cudaMalloc(&L.g_ptr, sizeof(int) * ptr.size()));
  M3_CUDA(cudaMalloc(&L.g_idx, sizeof(int) * idx.size()));
  M3_CUDA(cudaMalloc(&L.sa_err, sizeof(int) * 2));   // [0] error bits, [1] chunk ticket
  M3_CUDA(cudaMemcpyAsync(L.g_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(L.g_idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemsetAsync(L.sa_err, 0, sizeof(int) * 2, s));
  const size_t n = (size_t)L.nchunk * 10 * sa::E;
  k_chunk_conn<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(L.el2nod, nel, L.nchunk, L.chunk_conn);
  count_launch();
  M3_CUDA(cudaGetLastError());
  M3_CUDA(cudaFuncSetAttribute(k_stream_elem_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, sa::SMEM_ALLOC));
  int dev = 0, nsm = 0;
  M3_CUDA(cudaGetDevice(&dev));
  M3_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  L.sa_grid = std::max(1, std::min(nsm, L.nchunk));
  // the host copies above read stack vectors: finish them before they go out of scope
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

// 2D view of a packed FP32 operator [117 rows][4 nel floats]; box = 32 elements x 117 rows
static int encode_k32(const Level &L, const float *K, CUtensorMap *map) {
  const cuuint64_t dims[2] = {(cuuint64_t)L.nel * 4, (cuuint64_t)sa::ROWS};
  const cuuint64_t strides[1] = {(cuuint64_t)L.nel * 16};
  const cuuint32_t box[2] = {4 * sa::E, sa::ROWS};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(K), dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return M3SPH_ERR_CUDA;
  }
  return M3SPH_OK;
}

int stream_apply_f32(const Level &L, const float *K, const float *x, float *y, cudaStream_t s) {
  if (!L.nchunk || !g_encode) {
    set_error("streamed apply not built for this level");
    return M3SPH_ERR_BAD_INPUT;
  }
  if ((reinterpret_cast<uintptr_t>(K) & 15) != 0) {
    set_error("streamed apply: element matrices not 16-byte aligned");
    return M3SPH_ERR_BAD_INPUT;
  }
  CUtensorMap map;
  M3_TRY(encode_k32(L, K, &map));
  M3_CUDA(cudaMemsetAsync(L.sa_err + 1, 0, sizeof(int), s));
  k_stream_elem_f32<<<L.sa_grid, sa::THREADS, sa::SMEM_ALLOC, s>>>(map, L.chunk_conn, L.nchunk, L.nel, L.sa_err + 1,
                                                                    L.sa_err, x, L.ye32);
  count_launch();
  k_node_gather_f32<<<(L.nnod + 255) / 256, 256, 0, s>>>(L.g_ptr, L.g_idx, L.nnod, L.ye32, y);
  count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
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
