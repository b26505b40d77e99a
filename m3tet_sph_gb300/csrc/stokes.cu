// Host orchestration and C ABI of the Stokes hot path: device-resident MESH and multigrid
// hierarchy, operator set-up, V-cycle, flexible MG-PCG and the Patera pressure CG.
//
// Reference behaviour restated (paths inside the reference project):
//   mfiles_M3TET/flow3d_patera_mg_sph_p.m:70-129 (constants), :225-298 (rotation, BCs),
//       :374-384,709-727 (pressure preconditioner), :386-632 (Patera loop), :767-778 (rm0space)
//   mfiles_M3TET/mgpcg_solver_p.m:70-199 (flexible PCG), :388-596 (MG_V_cycle_v2),
//       :676-687 (Jacobi weights), :728-743 (mat_x_vec)
//   mfiles_M3TET/restrict_stiffmat.m:79-142, intermesh_transfer_matrix.m:1-62
//   mfiles_SPH/make_rotation_matrix.m:69-112, mfiles_M3TET/ip_tetrahedron.m:100-123
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <type_traits>

#include "common.cuh"

namespace m3sph {

// ---- declarations of kernels in the other translation units ----

int launch_element_setup(const SetupArgs &a, cudaStream_t s);
template <typename T> int ebe_apply(const Level &L, const T *K, const T *x, T *y, cudaStream_t s);
int ebe_apply_df(const Level &L, const float *Kh, const float *Kl, const double *x, double *y, cudaStream_t s);
int ebe_apply_split_f32(const Level &L, const float *K, const float *x, float *y, cudaStream_t s);
int ebe_apply_split_f64(const Level &L, const double *K, const double *x, double *y, cudaStream_t s);
int ebe_apply_split_df(const Level &L, const float *Kh, const float *Kl, const double *x, double *y, cudaStream_t s);
int stream_build(Level &L, const std::vector<int> &perm, cudaStream_t s);
int stream_apply_f32(const Level &L, const float *K, const float *x, float *y, cudaStream_t s);
int stream_apply_jac_f32(const Level &L, const float *K, float w, const float *r, const float *Di, float *d,
                         cudaStream_t s);
int stream_apply_df(const Level &L, const float *Kh, const float *Kl, const double *x, double *y, cudaStream_t s);
int stream_apply_f64(const Level &L, const double *K, const double *x, double *y, cudaStream_t s);
int stream_check(const Level &L, cudaStream_t s);
int pa_upload_tables();
int ml_feature_rows(m3sph_mesh *M, int j, const float *z, float *X, float *Sn);
int pa_row_stride(int nel);
int pa_build_trig(const double *RR, int nnod, float4 *trig, cudaStream_t s);
int pa_apply_f32(const Level &L, const float *x, float *y, cudaStream_t s);
int pa_apply_jac_f32(const Level &L, float w, const float *r, const float *Di, float *d, cudaStream_t s);
int stream_set_outer_warps(int n);
int stream_set_f32_variant(int v);
int scatter_elvec(const Level &L, const double *V, int nq, int per_node, double *out, size_t nout, cudaStream_t s);
template <typename T> int level_inverse_diag(Level &L, const T *K, double *work, cudaStream_t s);
int grad_apply(const Level &L, const double *G, const double *q, double *y, cudaStream_t s);
int div_apply(const Level &L, const double *G, const double *z, double *out, cudaStream_t s);
int mass_apply(const Level &L, const double *M, const double *d, double *out, cudaStream_t s);
template <typename T> int galerkin(const Level &F, const T *Kf, Level &C, T *Kc, cudaStream_t s);
template <typename T> int bsr_assemble(const Level &L, const T *K, T *B, cudaStream_t s);
template <typename T> int bsr_apply(const Level &L, const T *B, const T *x, T *y, cudaStream_t s);
int dot(const double *a, const double *b, size_t n, double *partials, double *out, cudaStream_t s);
int dot2(const double *a, const double *c, const double *b, size_t n, double *partials, double *out, cudaStream_t s);
int vsum(const double *a, size_t n, double *partials, double *out, cudaStream_t s);
int cg_dir(const double *d, double *q, size_t n, const double *scal, int first, cudaStream_t s);
int cg_update(double *x, double *r, const double *q, const double *Kq, size_t n, double *scal, double *partials,
              cudaStream_t s);
int axpby(double a, const double *x, double b, double *y, size_t n, cudaStream_t s);
int sub_mask(const double *b, double *y, const uint8_t *mask, size_t n, cudaStream_t s);
int apply_mask(double *y, const uint8_t *mask, size_t n, cudaStream_t s);
int d2f(const double *a, float *b, size_t n, cudaStream_t s);
int f2d(const float *a, double *b, size_t n, cudaStream_t s);
template <typename T> int jac_first(T w, const T *r0, const T *Di, T *d, size_t n, cudaStream_t s);
template <typename T> int jac(T w, const T *r0, const T *Kd, const T *Di, T *d, size_t n, cudaStream_t s);
template <typename T> int restrict_(const Level &F, const Level &C, const T *a, const T *b, T *out, cudaStream_t s);
template <typename T> int prolong(const Level &F, const Level &C, const T *xc, const T *add, T *out, cudaStream_t s);
template <typename T>
int dense_inverse_blocked(const Level &L, const T *B, T *A, T *work, const int *cmap, int nf, cudaStream_t s);
int dense_inverse_from64(const Level &L, const double *B64, float *B32tmp, float *A, float *work, const int *cmap,
                         int nf, cudaStream_t s);
int coarse_refined(const Level &L, const float *A32, const double *B64, const double *r, double *d, double *t,
                   int sweeps, const int *fidx, int nf, cudaStream_t s);
template <typename T> int dense_gemv(const T *A, int n, int nf, const int *fidx, const T *x, T *y, cudaStream_t s);
size_t element_setup_smem();

// ---- errors and counters ----
static thread_local std::string g_err;
static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
static void add_launches(unsigned long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
void set_error(const std::string &msg) { g_err = msg; }
int cuda_fail(cudaError_t e, const char *what) {
  g_err = std::string("CUDA error ") + cudaGetErrorString(e) + " in " + what;
  return M3SPH_ERR_CUDA;
}

// ---- quadrature and shape functions (host) ----
void build_shape_tables(ShapeTables &t) {
  // 14-point Gellert-Harbord rule, ip_tetrahedron.m:100-123; weights / 6 (:193)
  const double g = 1.0 / (46.0 * std::sqrt(46.0));
  const double h = std::acos(g) + (2.0 / 3.0) * std::asin(g);
  const double k = (104.0 + 8.0 * std::sqrt(46.0) * std::cos(h)) / 3.0;
  const double s = std::sqrt(49.0 - k);
  const double b = (7.0 + s) / k, a = 1.0 - 3.0 * b;
  const double d = (7.0 - s) / k, c = 1.0 - 3.0 * d;
  const double p = (98.0 - k - 14.0 * s) / (1680.0 * s * std::pow(b - a, 3));
  const double q = (98.0 - k + 14.0 * s) / (1680.0 * s * std::pow(c - d, 3));
  const double r = (1.0 - 4.0 * (p + q)) / 6.0;
  const double e = (1.0 + std::pow(2.0 / (105.0 * r), 0.25)) / 4.0;
  const double f = (1.0 - 2.0 * e) / 2.0;
  const double X[3][NIP] = {{a, b, b, b, c, d, d, d, e, e, e, f, f, f},
                            {b, a, b, b, d, c, d, d, e, f, f, e, e, f},
                            {b, b, a, b, d, d, c, d, f, e, f, e, f, e}};
  const double W[NIP] = {p, p, p, p, q, q, q, q, r, r, r, r, r, r};
  for (int ip = 0; ip < NIP; ++ip) {
    const double R = X[0][ip], S = X[1][ip], T = X[2][ip], U = 1.0 - R - S - T;
    t.ipw[ip] = W[ip] / 6.0;
    const double L[4] = {R, S, T, U};
    const double gL[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, -1, -1}};
    for (int v = 0; v < 4; ++v) t.NP[ip][v] = L[v];
    // P2 (sf_dsf_tet10): vertices L(2L-1), edges 4 La Lb on edges 1-2,2-3,3-4,4-1,1-3,2-4
    const int E10[6][2] = {{0, 1}, {1, 2}, {2, 3}, {0, 3}, {0, 2}, {1, 3}};
    for (int v = 0; v < 4; ++v) {
      t.NU[ip][v] = L[v] * (2 * L[v] - 1);
      for (int j = 0; j < 3; ++j) t.dNU[ip][v][j] = (4 * L[v] - 1) * gL[v][j];
    }
    for (int m = 0; m < 6; ++m) {
      const int ia = E10[m][0], ib = E10[m][1];
      t.NU[ip][4 + m] = 4 * L[ia] * L[ib];
      for (int j = 0; j < 3; ++j) t.dNU[ip][4 + m][j] = 4 * (L[ib] * gL[ia][j] + L[ia] * gL[ib][j]);
    }
    // cubic 20-node tetrahedron (sf_dsf_tet20 node order)
    for (int v = 0; v < 4; ++v) {
      t.N20[ip][v] = 0.5 * L[v] * (3 * L[v] - 1) * (3 * L[v] - 2);
      for (int j = 0; j < 3; ++j) t.dN20[ip][v][j] = 0.5 * (27 * L[v] * L[v] - 18 * L[v] + 2) * gL[v][j];
    }
    const int EP[12][2] = {{0, 1}, {1, 0}, {1, 2}, {2, 1}, {2, 3}, {3, 2}, {3, 0}, {0, 3}, {0, 2}, {2, 0}, {3, 1}, {1, 3}};
    for (int m = 0; m < 12; ++m) {
      const int ia = EP[m][0], ib = EP[m][1];
      t.N20[ip][4 + m] = 4.5 * L[ia] * L[ib] * (3 * L[ia] - 1);
      for (int j = 0; j < 3; ++j)
        t.dN20[ip][4 + m][j] = 4.5 * (L[ib] * (6 * L[ia] - 1) * gL[ia][j] + L[ia] * (3 * L[ia] - 1) * gL[ib][j]);
    }
    const int FC[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
    for (int m = 0; m < 4; ++m) {
      const int i0 = FC[m][0], i1 = FC[m][1], i2 = FC[m][2];
      t.N20[ip][16 + m] = 27 * L[i0] * L[i1] * L[i2];
      for (int j = 0; j < 3; ++j)
        t.dN20[ip][16 + m][j] =
            27 * (L[i1] * L[i2] * gL[i0][j] + L[i0] * L[i2] * gL[i1][j] + L[i0] * L[i1] * gL[i2][j]);
    }
  }
}

// ---- device allocation helpers ----
template <typename T>
static int dalloc(T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  M3_CUDA(cudaMalloc((void **)p, sizeof(T) * n));
  return M3SPH_OK;
}
template <typename T>
static int upload(T **p, const T *h, size_t n, cudaStream_t s) {
  M3_TRY(dalloc(p, n));
  M3_CUDA(cudaMemcpyAsync(*p, h, sizeof(T) * n, cudaMemcpyHostToDevice, s));
  return M3SPH_OK;
}
static void dfree(void *p) {
  if (p) cudaFree(p);
}

// ---- greedy element colouring: elements sharing a vertex get different colours ----
static int color_elements(const std::vector<int> &el, int nel, int nvert_ids, std::vector<int> &color, int &ncolor) {
  std::vector<uint64_t> used(2 * (size_t)nvert_ids, 0);
  color.assign(nel, -1);
  ncolor = 0;
  for (int e = 0; e < nel; ++e) {
    uint64_t m0 = 0, m1 = 0;
    for (int v = 0; v < 4; ++v) {
      const int n = el[(size_t)e * 10 + v];
      m0 |= used[2 * (size_t)n];
      m1 |= used[2 * (size_t)n + 1];
    }
    int c = -1;
    if (~m0) c = __builtin_ctzll(~m0);
    else if (~m1) c = 64 + __builtin_ctzll(~m1);
    if (c < 0) {
      set_error("element colouring needs more than 128 colours");
      return M3SPH_ERR_BAD_INPUT;
    }
    color[e] = c;
    ncolor = std::max(ncolor, c + 1);
    for (int v = 0; v < 4; ++v) {
      const int n = el[(size_t)e * 10 + v];
      used[2 * (size_t)n + (c >> 6)] |= 1ull << (c & 63);
    }
  }
  return M3SPH_OK;
}

static const double P2LC[10][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0},   {.5, .5, 0},
                                   {0, .5, .5}, {0, 0, .5}, {.5, 0, 0}, {.5, 0, .5}, {0, .5, 0}};
static const int EDG[6][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 2}, {3, 1}};

static void sf10h(const double *lc, double *N) {
  const double r = lc[0], s = lc[1], t = lc[2], u = 1 - r - s - t;
  N[0] = r * (2 * r - 1); N[1] = s * (2 * s - 1); N[2] = t * (2 * t - 1); N[3] = u * (2 * u - 1);
  N[4] = 4 * r * s; N[5] = 4 * s * t; N[6] = 4 * t * u; N[7] = 4 * r * u; N[8] = 4 * r * t; N[9] = 4 * s * u;
}

}  // namespace m3sph

using namespace m3sph;

// ======================================================================================
// C ABI
// ======================================================================================
extern "C" const char *m3sph_last_error(void) { return g_err.c_str(); }

extern "C" int m3sph_device_count(int *count) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) {
    *count = 0;
    return cuda_fail(e, "cudaGetDeviceCount");
  }
  *count = n;
  return M3SPH_OK;
}

// block sparsity pattern of a level and the element contributions of every block
static int build_bsr(m3sph_mesh *M, Level &L, const std::vector<int> &perm) {
  const int nel = L.nel, nnod = L.nnod;
  std::vector<int> invp(nel);
  for (int p = 0; p < nel; ++p) invp[perm[p]] = p;
  // node -> (stored element, local index)
  std::vector<int> nptr(nnod + 1, 0);
  for (size_t i = 0; i < (size_t)nel * 10; ++i) nptr[L.h_el2nod_orig[i] + 1]++;
  for (int n = 0; n < nnod; ++n) nptr[n + 1] += nptr[n];
  std::vector<int> nfill(nptr.begin(), nptr.end() - 1), nel_of((size_t)nel * 10), nloc((size_t)nel * 10);
  for (int e = 0; e < nel; ++e)
    for (int a = 0; a < 10; ++a) {
      const int n = L.h_el2nod_orig[(size_t)e * 10 + a];
      const int pos = nfill[n]++;
      nel_of[pos] = invp[e];
      nloc[pos] = a;
    }
  std::vector<int> ptr(nnod + 1, 0), col, cptr(1, 0), contrib;
  col.reserve((size_t)nnod * 32);
  contrib.reserve((size_t)nel * 100);
  std::vector<std::pair<int, int>> row;   // (col node, contribution code)
  for (int i = 0; i < nnod; ++i) {
    row.clear();
    for (int k = nptr[i]; k < nptr[i + 1]; ++k) {
      const int p = nel_of[k], a = nloc[k];
      const int e = perm[p];
      for (int b = 0; b < 10; ++b) row.push_back({L.h_el2nod_orig[(size_t)e * 10 + b], p * 100 + a * 10 + b});
    }
    std::sort(row.begin(), row.end());
    for (size_t k = 0; k < row.size(); ++k) {
      if (k == 0 || row[k].first != row[k - 1].first) {
        col.push_back(row[k].first);
        if (k) cptr.push_back((int)contrib.size());
      }
      contrib.push_back(row[k].second);
    }
    if (!row.empty()) cptr.push_back((int)contrib.size());
    ptr[i + 1] = (int)col.size();
  }
  if ((size_t)nel * 100 > 2147483647ull / 2) {
    set_error("level too large for the block operator contribution list");
    return M3SPH_ERR_BAD_INPUT;
  }
  L.nnzb = (int)col.size();
  cudaStream_t s = M->stream;
  M3_TRY(upload(&L.bsr_ptr, ptr.data(), ptr.size(), s));
  M3_TRY(upload(&L.bsr_col, col.data(), col.size(), s));
  M3_TRY(upload(&L.bsr_cptr, cptr.data(), cptr.size(), s));
  M3_TRY(upload(&L.bsr_contrib, contrib.data(), contrib.size(), s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

static int build_level(m3sph_mesh *M, int img, const m3sph_level &in, Level &L) {
  cudaStream_t s = M->stream;
  L.nel = in.nel;
  L.nnod = in.nnod;
  L.nvnod = in.nvnod;
  L.ndof = 3 * in.nnod;
  if (in.nel <= 0 || in.nnod <= 0 || !in.EL2NOD) {
    set_error("level " + std::to_string(img) + ": empty or missing EL2NOD");
    return M3SPH_ERR_BAD_INPUT;
  }
  L.h_el2nod_orig.resize((size_t)in.nel * 10);
  for (size_t i = 0; i < (size_t)in.nel * 10; ++i) {
    const uint32_t v = in.EL2NOD[i];
    if (v < 1 || v > (uint32_t)in.nnod) {
      set_error("level " + std::to_string(img) + ": EL2NOD entry out of range");
      return M3SPH_ERR_BAD_INPUT;
    }
    L.h_el2nod_orig[i] = (int)v - 1;
  }
  std::vector<int> color;
  int ncolor = 0;
  M3_TRY(color_elements(L.h_el2nod_orig, in.nel, in.nnod, color, ncolor));
  std::vector<int> cnt(ncolor + 1, 0);
  for (int e = 0; e < in.nel; ++e) cnt[color[e] + 1]++;
  for (int c = 0; c < ncolor; ++c) cnt[c + 1] += cnt[c];
  L.cstart = cnt;
  std::vector<int> perm(in.nel), invperm(in.nel), fill(cnt.begin(), cnt.end() - 1);
  for (int e = 0; e < in.nel; ++e) {
    const int pos = fill[color[e]]++;
    perm[pos] = e;
    invperm[e] = pos;
  }
  std::vector<int> el_soa((size_t)in.nel * 10);
  for (int p = 0; p < in.nel; ++p)
    for (int n = 0; n < 10; ++n) el_soa[(size_t)n * in.nel + p] = L.h_el2nod_orig[(size_t)perm[p] * 10 + n];
  M3_TRY(upload(&L.el2nod, el_soa.data(), el_soa.size(), s));
  M3_TRY(upload(&L.perm, perm.data(), perm.size(), s));
  M3_TRY(upload(&L.invperm, invperm.data(), invperm.size(), s));
  M3_TRY(dalloc(&L.freemask, L.ndof));
  M3_CUDA(cudaMemsetAsync(L.freemask, 1, L.ndof, s));
  M3_TRY(dalloc(&L.Dinv64, L.ndof));
  M3_TRY(dalloc(&L.Dinv32, L.ndof));
  if (img > 0) M3_TRY(build_bsr(M, L, perm));
  if (img == 0) M3_TRY(stream_build(L, perm, s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

// children of coarse level C (level img+1) in fine level F (level img), and the transfer rows
static int build_transfer(m3sph_mesh *M, Level &F, Level &C, const uint8_t *isplit_c) {
  cudaStream_t s = M->stream;
  (void)isplit_c;
  if ((size_t)F.nel != 8 * (size_t)C.nel) {
    set_error("fine level must have 8 children per coarse element");
    return M3SPH_ERR_BAD_INPUT;
  }
  std::vector<int> hperm_c(C.nel), hinv_f(F.nel);
  M3_CUDA(cudaMemcpy(hperm_c.data(), C.perm, sizeof(int) * C.nel, cudaMemcpyDeviceToHost));
  M3_CUDA(cudaMemcpy(hinv_f.data(), F.invperm, sizeof(int) * F.nel, cudaMemcpyDeviceToHost));
  std::vector<int> child((size_t)8 * C.nel);
  std::vector<uint32_t> vloc((size_t)8 * C.nel);
  // parent-local index of each child vertex
  std::vector<uint32_t> vloc_orig((size_t)F.nel);
  for (int p = 0; p < C.nel; ++p) {
    const int *pn = &C.h_el2nod_orig[(size_t)p * 10];
    for (int k = 0; k < 8; ++k) {
      const int fe = 8 * p + k;
      uint32_t code = 0;
      for (int v = 0; v < 4; ++v) {
        const int node = F.h_el2nod_orig[(size_t)fe * 10 + v];
        int loc = -1;
        for (int j = 0; j < 10; ++j)
          if (pn[j] == node) loc = j;
        if (loc < 0) {
          set_error("child vertex is not a node of its parent");
          return M3SPH_ERR_BAD_INPUT;
        }
        code |= (uint32_t)loc << (4 * v);
      }
      vloc_orig[fe] = code;
    }
  }
  for (int pc = 0; pc < C.nel; ++pc) {
    const int p = hperm_c[pc];
    for (int k = 0; k < 8; ++k) {
      child[(size_t)k * C.nel + pc] = hinv_f[8 * p + k];
      vloc[(size_t)k * C.nel + pc] = vloc_orig[8 * p + k];
    }
  }
  M3_TRY(upload(&C.child, child.data(), child.size(), s));
  M3_TRY(upload(&C.child_vloc, vloc.data(), vloc.size(), s));
  // transfer rows: parent of the first element listing the node (intermesh_transfer_matrix.m:19-23)
  std::vector<int> first(F.nnod, -1);
  for (size_t i = 0; i < (size_t)F.nel * 10; ++i) {
    const int n = F.h_el2nod_orig[i];
    if (first[n] < 0) first[n] = (int)i;
  }
  std::vector<int> ptr(F.nnod + 1, 0), col;
  std::vector<float> w;
  col.reserve((size_t)F.nnod * 4);
  w.reserve((size_t)F.nnod * 4);
  for (int n = 0; n < F.nnod; ++n) {
    if (first[n] < 0) {
      set_error("fine node not referenced by any element");
      return M3SPH_ERR_BAD_INPUT;
    }
    const int fe = first[n] / 10, ln = first[n] % 10, p = fe / 8;
    const uint32_t code = vloc_orig[fe];
    double lc[3];
    if (ln < 4) {
      const int pl = (code >> (4 * ln)) & 15;
      for (int d = 0; d < 3; ++d) lc[d] = P2LC[pl][d];
    } else {
      const int a0 = (code >> (4 * EDG[ln - 4][0])) & 15, a1 = (code >> (4 * EDG[ln - 4][1])) & 15;
      for (int d = 0; d < 3; ++d) lc[d] = 0.5 * (P2LC[a0][d] + P2LC[a1][d]);
    }
    double N[10];
    sf10h(lc, N);
    for (int j = 0; j < 10; ++j)
      if (std::fabs(N[j]) > 1e-14) {
        col.push_back(C.h_el2nod_orig[(size_t)p * 10 + j]);
        w.push_back((float)N[j]);
      }
    ptr[n + 1] = (int)col.size();
  }
  // transpose (coarse rows)
  std::vector<int> rptr(C.nnod + 1, 0), rcol(col.size());
  std::vector<float> rw(col.size());
  for (int c : col) rptr[c + 1]++;
  for (int i = 0; i < C.nnod; ++i) rptr[i + 1] += rptr[i];
  std::vector<int> fill(rptr.begin(), rptr.end() - 1);
  for (int n = 0; n < F.nnod; ++n)
    for (int k = ptr[n]; k < ptr[n + 1]; ++k) {
      const int pos = fill[col[k]]++;
      rcol[pos] = n;
      rw[pos] = w[k];
    }
  M3_TRY(upload(&F.P_ptr, ptr.data(), ptr.size(), s));
  M3_TRY(upload(&F.P_col, col.data(), col.size(), s));
  M3_TRY(upload(&F.P_w, w.data(), w.size(), s));
  M3_TRY(upload(&F.R_ptr, rptr.data(), rptr.size(), s));
  M3_TRY(upload(&F.R_col, rcol.data(), rcol.size(), s));
  M3_TRY(upload(&F.R_w, rw.data(), rw.size(), s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

static void clear_graphs(m3sph_mesh *M);

static void free_level(Level &L) {
  for (void *p : {(void *)L.el2nod, (void *)L.perm, (void *)L.invperm, (void *)L.freemask, (void *)L.K64,
                  (void *)L.K32, (void *)L.KL32, (void *)L.Dinv64, (void *)L.Dinv32, (void *)L.child, (void *)L.child_vloc,
                  (void *)L.P_ptr, (void *)L.P_col, (void *)L.P_w, (void *)L.R_ptr, (void *)L.R_col, (void *)L.R_w,
                  (void *)L.bsr_ptr, (void *)L.bsr_col, (void *)L.bsr_cptr, (void *)L.bsr_contrib, (void *)L.B64,
                  (void *)L.B32, (void *)L.chunk_conn, (void *)L.ye32, (void *)L.g_ptr, (void *)L.g_idx, (void *)L.sa_err,
                  (void *)L.chunk_conn8, (void *)L.ye64, (void *)L.pa32, (void *)L.pa_emask, (void *)L.pa_trig})
    dfree(p);
  L = Level();
}

extern "C" int m3sph_mesh_destroy(m3sph_mesh *M) {
  if (!M) return M3SPH_OK;
  cudaSetDevice(M->device);
  if (M->stream) cudaStreamSynchronize(M->stream);
  for (auto &L : M->lev) free_level(L);
  Finest &f = M->fin;
  for (void *p : {(void *)f.gcoord, (void *)f.gcoord_sph, (void *)f.RR, (void *)f.cls, (void *)f.iso_slot,
                  (void *)f.cubic, (void *)f.visc, (void *)f.dens, (void *)f.G64, (void *)f.M64, (void *)f.Fbe,
                  (void *)f.BCe, (void *)f.Fb, (void *)f.LiMM, (void *)f.err})
    dfree(p);
  dfree(M->coarse.A64);
  dfree(M->coarse.A32);
  dfree(M->coarse.cmap);
  dfree(M->coarse.fidx);
  dfree(M->coarse.B32tmp);
  dfree(M->coarse.t64);
  dfree(M->Ufix);
  dfree(M->bc_rhs);
  dfree(M->red);
  dfree(M->scal);
  dfree(M->T);
  dfree(M->Usoa);
  for (void *p : M->work) dfree(p);
  if (M->h_scal) cudaFreeHost(M->h_scal);
  clear_graphs(M);
  if (M->wk && M->wk_free) M->wk_free(M->wk);
  if (M->slm && M->slm_free) M->slm_free(M->slm);
  if (M->diff && M->diff_free) M->diff_free(M->diff);
  if (M->ml && M->ml_free) M->ml_free(M->ml);
  if (M->stream) cudaStreamDestroy(M->stream);
  delete M;
  return M3SPH_OK;
}

extern "C" int m3sph_mesh_create(int32_t nmg, const m3sph_level *levels, int32_t device, m3sph_mesh **out) {
  if (!out || !levels || nmg < 1) {
    set_error("m3sph_mesh_create: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_error("no CUDA device available: the m3sph library has no CPU path");
    return M3SPH_ERR_NO_DEVICE;
  }
  M3_CUDA(cudaSetDevice(device));
  m3sph_mesh *M = new m3sph_mesh();
  M->device = device;
  M->nmg = nmg;
  int st = M3SPH_OK;
  auto fail = [&](int code) {
    m3sph_mesh_destroy(M);
    return code;
  };
  if (cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(M3SPH_ERR_CUDA);
  st = upload_shape_tables();
  if (st) return fail(st);
  st = pa_upload_tables();
  if (st) return fail(st);
  M->lev.resize(nmg);
  for (int i = 0; i < nmg; ++i) {
    st = build_level(M, i, levels[i], M->lev[i]);
    if (st) return fail(st);
    if (i > 0 && levels[i].nnod > levels[i - 1].nnod) {
      set_error("coarse level has more nodes than the finer level");
      return fail(M3SPH_ERR_BAD_INPUT);
    }
  }
  for (int i = 0; i + 1 < nmg; ++i) {
    st = build_transfer(M, M->lev[i], M->lev[i + 1], levels[i + 1].isplit);
    if (st) return fail(st);
  }
  // finest-level geometry
  const m3sph_level &f0 = levels[0];
  Level &L0 = M->lev[0];
  if (!f0.GCOORD || !f0.GCOORD_SPH || !f0.elclass) {
    set_error("level 0 needs GCOORD, GCOORD_SPH and elclass");
    return fail(M3SPH_ERR_BAD_INPUT);
  }
  Finest &F = M->fin;
  cudaStream_t s = M->stream;
  const int nnod = f0.nnod, nel = f0.nel;
  std::vector<double> gc(3 * (size_t)nnod), gs(3 * (size_t)nnod), RR(9 * (size_t)nnod);
  for (int n = 0; n < nnod; ++n)
    for (int k = 0; k < 3; ++k) {
      gc[(size_t)k * nnod + n] = f0.GCOORD[3 * (size_t)n + k];
      gs[(size_t)k * nnod + n] = f0.GCOORD_SPH[3 * (size_t)n + k];
    }
  for (int n = 0; n < nnod; ++n) {   // make_rotation_matrix.m:69-112 from cartesian2spherical(GCOORD)
    const double x = f0.GCOORD[3 * (size_t)n], y = f0.GCOORD[3 * (size_t)n + 1], z = f0.GCOORD[3 * (size_t)n + 2];
    const double th = std::atan2(std::sqrt(x * x + y * y), z);
    double ph = std::atan2(y, x);
    if (ph < 0) ph += 2 * M_PI;
    const double st_ = std::sin(th), ct = std::cos(th), sp = std::sin(ph), cp = std::cos(ph);
    const double Rm[9] = {cp * ct, -sp, cp * st_, sp * ct, cp, sp * st_, -st_, 0.0, ct};
    for (int q = 0; q < 9; ++q) RR[(size_t)q * nnod + n] = Rm[q];
  }
  std::vector<int> hperm(nel);
  M3_CUDA(cudaMemcpy(hperm.data(), L0.perm, sizeof(int) * nel, cudaMemcpyDeviceToHost));
  std::vector<uint8_t> cls(nel);
  std::vector<int> iso_slot(nel, -1), iso_of_orig(nel, -1);
  for (int i = 0; i < f0.niso; ++i) {
    const uint32_t e = f0.els_iso[i];
    if (e < 1 || e > (uint32_t)nel) {
      set_error("els_iso entry out of range");
      return fail(M3SPH_ERR_BAD_INPUT);
    }
    iso_of_orig[e - 1] = i;
  }
  for (int p = 0; p < nel; ++p) {
    const int e = hperm[p];
    cls[p] = f0.elclass[e];
    if (cls[p] > 3) {
      set_error("element class out of range");
      return fail(M3SPH_ERR_BAD_INPUT);
    }
    if (cls[p] == M3SPH_IN_CONE_ISO) {
      if (iso_of_orig[e] < 0) {
        set_error("in-cone isoparametric element without cubic geometry");
        return fail(M3SPH_ERR_BAD_INPUT);
      }
      iso_slot[p] = iso_of_orig[e];
    }
  }
  F.niso = f0.niso;
  std::vector<double> cub(60 * (size_t)std::max(1, f0.niso), 0.0);
  for (int i = 0; i < f0.niso; ++i)
    for (int q = 0; q < 60; ++q) cub[(size_t)q * f0.niso + i] = f0.cubic_sph_rot[(size_t)i * 60 + q];
  if ((st = upload(&F.gcoord, gc.data(), gc.size(), s)) || (st = upload(&F.gcoord_sph, gs.data(), gs.size(), s)) ||
      (st = upload(&F.RR, RR.data(), RR.size(), s)) || (st = upload(&F.cls, cls.data(), cls.size(), s)) ||
      (st = upload(&F.iso_slot, iso_slot.data(), iso_slot.size(), s)) ||
      (st = upload(&F.cubic, cub.data(), cub.size(), s)) || (st = dalloc(&F.visc, nnod)) ||
      (st = dalloc(&F.dens, nnod)) || (st = dalloc(&F.G64, 120 * (size_t)nel)) ||
      (st = dalloc(&F.M64, 10 * (size_t)nel)) || (st = dalloc(&F.Fbe, 30 * (size_t)nel)) ||
      (st = dalloc(&F.BCe, 30 * (size_t)nel)) ||
      (st = dalloc(&F.Fb, L0.ndof)) || (st = dalloc(&F.LiMM, L0.nvnod)) || (st = dalloc(&F.err, 4)) ||
      (st = dalloc(&L0.K64, (size_t)kpad<double>() * nel)) || (st = dalloc(&L0.K32, (size_t)kpad<float>() * nel)) ||
      (st = dalloc(&L0.KL32, (size_t)kpad<float>() * nel)) ||
      (st = dalloc(&M->Ufix, L0.ndof)) || (st = dalloc(&M->bc_rhs, L0.ndof)) || (st = dalloc(&M->red, 4096)) ||
      (st = dalloc(&M->scal, 64)))
    return fail(st);
  if (cudaMallocHost((void **)&M->h_scal, 64 * sizeof(double)) != cudaSuccess) return fail(M3SPH_ERR_CUDA);
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(cuda_fail(cudaGetLastError(), "mesh upload"));
  st = slm_build(M, f0);
  if (st) return fail(st);
  {
    double rmin = 1e300, rmax = 0.0;
    for (int n = 0; n < nnod; ++n) {
      const double r = f0.GCOORD_SPH[3 * (size_t)n + 2];
      rmin = std::min(rmin, r);
      rmax = std::max(rmax, r);
    }
    M->r_min = rmin;
    M->r_max = rmax;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int n = 0; n < nnod; ++n)
      for (int c = 0; c < 3; ++c) {
        lo[c] = std::min(lo[c], f0.GCOORD[3 * (size_t)n + c]);
        hi[c] = std::max(hi[c], f0.GCOORD[3 * (size_t)n + c]);
      }
    M->Lx = hi[0] - lo[0];
    M->Ly = hi[1] - lo[1];
    M->Lz = hi[2] - lo[2];
    double r2max = 0.0;
    for (int n = 0; n < nnod; ++n) {
      const double *x = f0.GCOORD + 3 * (size_t)n;
      r2max = std::max(r2max, std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]));
    }
    M->rad_max = r2max;
  }
  if ((st = ml_build(M)) || (st = ml_init_kernels())) return fail(st);
  *out = M;
  return M3SPH_OK;
}

extern "C" int m3sph_mesh_ncolors(const m3sph_mesh *M, int32_t img, int32_t *nc) {
  if (!M || img < 0 || img >= M->nmg || !nc) {
    set_error("bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  *nc = (int)M->lev[img].cstart.size() - 1;
  return M3SPH_OK;
}

// ---- work vectors ----
namespace {
struct Work {
  // per level T vectors for the V-cycle
  std::vector<double *> r64, d64, kd64, t64;
  std::vector<float *> r32, d32, kd32, t32;
  double *cwork64 = nullptr;
  float *cwork32 = nullptr;
  // outer vectors (level 0, fp64)
  double *r = nullptr, *d = nullptr, *q = nullptr, *Kq = nullptr, *tmp = nullptr;
  double *U = nullptr, *z = nullptr, *y = nullptr, *Rhs = nullptr;
  double *pr = nullptr, *pd = nullptr, *pq = nullptr, *pSq = nullptr, *pt = nullptr, *pP = nullptr, *prl = nullptr;
};
}  // namespace


static Work *get_work(m3sph_mesh *M) { return reinterpret_cast<Work *>(M->wk); }

static int alloc_work(m3sph_mesh *M) {
  if (M->wk) return M3SPH_OK;
  Work *W = new Work();
  M->wk = W;
  M->wk_free = [](void *p) { delete reinterpret_cast<Work *>(p); };
  const int nmg = M->nmg;
  W->r64.resize(nmg); W->d64.resize(nmg); W->kd64.resize(nmg); W->t64.resize(nmg);
  W->r32.resize(nmg); W->d32.resize(nmg); W->kd32.resize(nmg); W->t32.resize(nmg);
  for (int i = 0; i < nmg; ++i) {
    const size_t n = M->lev[i].ndof;
    M3_TRY(dalloc(&W->r64[i], n)); M3_TRY(dalloc(&W->d64[i], n)); M3_TRY(dalloc(&W->kd64[i], n));
    M3_TRY(dalloc(&W->r32[i], n)); M3_TRY(dalloc(&W->d32[i], n)); M3_TRY(dalloc(&W->kd32[i], n));
    M3_TRY(dalloc(&W->t64[i], n)); M3_TRY(dalloc(&W->t32[i], n));
  }
  const size_t nc = M->lev[nmg - 1].ndof;
  // blocked Gauss-Jordan: the 128x128 diagonal inverse and the 128-wide row and column panels
  M3_TRY(dalloc(&W->cwork64, 128 * 128 + 2 * 128 * nc));
  M3_TRY(dalloc(&W->cwork32, 128 * 128 + 2 * 128 * nc));
  const size_t n0 = M->lev[0].ndof, np = M->lev[0].nvnod;
  M3_TRY(dalloc(&W->r, n0)); M3_TRY(dalloc(&W->d, n0)); M3_TRY(dalloc(&W->q, n0));
  M3_TRY(dalloc(&W->Kq, n0)); M3_TRY(dalloc(&W->tmp, n0));
  M3_TRY(dalloc(&W->U, n0)); M3_TRY(dalloc(&W->z, n0)); M3_TRY(dalloc(&W->y, n0)); M3_TRY(dalloc(&W->Rhs, n0));
  M3_TRY(dalloc(&W->pr, np)); M3_TRY(dalloc(&W->pd, np)); M3_TRY(dalloc(&W->pq, np));
  M3_TRY(dalloc(&W->pSq, np)); M3_TRY(dalloc(&W->pt, np)); M3_TRY(dalloc(&W->pP, np)); M3_TRY(dalloc(&W->prl, np));
  // register device buffers for freeing
  auto reg = [&](void *p) { M->work.push_back(p); };
  for (int i = 0; i < nmg; ++i) {
    reg(W->r64[i]); reg(W->d64[i]); reg(W->kd64[i]); reg(W->r32[i]); reg(W->d32[i]); reg(W->kd32[i]);
    reg(W->t64[i]); reg(W->t32[i]);
  }
  for (void *p : {(void *)W->cwork64, (void *)W->cwork32, (void *)W->r, (void *)W->d, (void *)W->q, (void *)W->Kq,
                  (void *)W->tmp, (void *)W->U, (void *)W->z, (void *)W->y, (void *)W->Rhs, (void *)W->pr,
                  (void *)W->pd, (void *)W->pq, (void *)W->pSq, (void *)W->pt, (void *)W->pP, (void *)W->prl})
    reg(p);
  return M3SPH_OK;
}

// ======================================================================================
// operator set-up
// ======================================================================================
__global__ void k_set_masks(uint8_t *mask, const int *ifix, int nfix, int ndof) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nfix && ifix[i] >= 0 && ifix[i] < ndof) mask[ifix[i]] = 0;
}
__global__ void k_scatter_vals(double *v, const int *ifix, const double *vals, int nfix) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nfix) v[ifix[i]] = vals[i];
}
__global__ void k_recip(const double *a, double *b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = 1.0 / a[i];
}

// FP64 coarsest levels up to this many dofs are inverted in FP64; larger ones are refined
// FP32 V-cycle operator of the finest level: false = streamed stored matrices (K32), true =
// partially assembled (per-point geometric factors, product formed on the fly)
static bool g_pa_apply = true;
static int g_coarse_f64_direct_max = 6000;
static int g_coarse_refine_sweeps = 3;

// element operator, force vector, Galerkin hierarchy and coarse inverse from the device-resident
// viscosity, density and boundary conditions (assembly_stokes_sph_3d_double_jacobian +
// restrict_stiffmat + cholesky_factorization of the reference)
static int rebuild_operator(m3sph_mesh *M) {
  cudaStream_t s = M->stream;
  Level &L0 = M->lev[0];
  Work *W = get_work(M);
  M->bc_stale = false;
  M3_CUDA(cudaMemsetAsync(M->fin.err, 0, sizeof(int) * 4, s));
  SetupArgs a{};
  a.nel = L0.nel; a.nnod = L0.nnod; a.el2nod = L0.el2nod; a.cls = M->fin.cls; a.iso_slot = M->fin.iso_slot;
  a.cubic = M->fin.cubic; a.niso = M->fin.niso; a.gcoord = M->fin.gcoord; a.gcoord_sph = M->fin.gcoord_sph;
  a.RR = M->fin.RR; a.visc = M->fin.visc; a.dens = M->fin.dens; a.freemask = L0.freemask;
  a.g = M->phys.g; a.Bscale = M->phys.Bscale; a.Dens0 = M->phys.Dens0; a.minVisc = M->phys.minVisc; a.maxVisc = M->phys.maxVisc;
  a.K64 = L0.K64; a.K32 = L0.K32; a.G64 = M->fin.G64; a.M64 = M->fin.M64; a.Fbe = M->fin.Fbe; a.err = M->fin.err;
  a.ufix = nullptr;
  a.BCe = nullptr;
  a.KL32 = L0.KL32;
  a.PA32 = nullptr;
  a.emask = nullptr;
  L0.pa_ready = false;
  if (M->precision == 1 && g_pa_apply) {
    if (!L0.pa32) {
      L0.pa_ld = pa_row_stride(L0.nel);
      M3_TRY(dalloc(&L0.pa32, (size_t)NIP * 9 * L0.pa_ld));
    }
    if (!L0.pa_emask) M3_TRY(dalloc(&L0.pa_emask, (size_t)L0.nel));
    if (!L0.pa_trig) {
      M3_TRY(dalloc(&L0.pa_trig, (size_t)L0.nnod));
      M3_TRY(pa_build_trig(M->fin.RR, L0.nnod, L0.pa_trig, s));
    }
    a.PA32 = L0.pa32;
    a.pa_ld = L0.pa_ld;
    a.emask = L0.pa_emask;
  }
  if (M->has_nonzero_fix) {
    a.ufix = M->Ufix;
    a.BCe = M->fin.BCe;
  }
  M3_TRY(launch_element_setup(a, s));
  L0.pa_ready = a.PA32 != nullptr;
  int herr[4];
  M3_CUDA(cudaMemcpyAsync(herr, M->fin.err, sizeof(herr), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  if (herr[0] & 1) {
    set_error("negative Jacobi");
    return M3SPH_ERR_NEGATIVE_JACOBIAN;
  }
  if (herr[0] & 2) {
    set_error("integration point with theta = 0 (det(J_CS) = Inf)");
    return M3SPH_ERR_BAD_INPUT;
  }
  if (herr[0] & 4) {
    set_error(" Calculated a zero or negative viscosity. STOPPING.");
    return M3SPH_ERR_BAD_INPUT;
  }
  // assembled force vector, lumped pressure mass, boundary-condition rhs
  M3_TRY(scatter_elvec(L0, M->fin.Fbe, 30, 3, M->fin.Fb, L0.ndof, s));
  M3_TRY(mass_apply(L0, M->fin.M64, nullptr, W->pt, s));
  k_recip<<<(L0.nvnod + 255) / 256, 256, 0, s>>>(W->pt, M->fin.LiMM, L0.nvnod); count_launch();
  if (M->has_nonzero_fix) {
    M3_TRY(scatter_elvec(L0, M->fin.BCe, 30, 3, M->bc_rhs, L0.ndof, s));
  } else {
    M3_CUDA(cudaMemsetAsync(M->bc_rhs, 0, sizeof(double) * L0.ndof, s));
  }
  // level diagonals and Galerkin coarse operators
  M3_TRY(level_inverse_diag<double>(L0, L0.K64, W->tmp, s));
  for (int i = 1; i < M->nmg; ++i) {
    Level &F = M->lev[i - 1], &C = M->lev[i];
    if (M->precision == 0) {
      if (!C.K64) M3_TRY(dalloc(&C.K64, (size_t)kpad<double>() * C.nel));
      M3_TRY(galerkin<double>(F, F.K64, C, C.K64, s));
      M3_TRY(level_inverse_diag<double>(C, C.K64, W->tmp, s));
      if (!C.B64) M3_TRY(dalloc(&C.B64, 9 * (size_t)C.nnzb));
      M3_TRY(bsr_assemble<double>(C, C.K64, C.B64, s));
    } else {
      if (!C.K32) M3_TRY(dalloc(&C.K32, (size_t)kpad<float>() * C.nel));
      M3_TRY(galerkin<float>(F, F.K32, C, C.K32, s));
      M3_TRY(level_inverse_diag<float>(C, C.K32, W->tmp, s));
      if (!C.B32) M3_TRY(dalloc(&C.B32, 9 * (size_t)C.nnzb));
      M3_TRY(bsr_assemble<float>(C, C.K32, C.B32, s));
    }
  }
  // coarsest-level solve (stands in for cholesky_factorization / cholesky_solve): the dense
  // inverse by blocked Gauss-Jordan (128-wide panels), applied as one GEMV per V-cycle. FP32 V-cycle: FP32 inverse.
  // Plain FP64 path: the FP64 inverse up to g_coarse_f64_direct_max dofs; above, the FP32 inverse
  // of the FP64 operator refined against it to FP64 rounding in every coarse solve (an FP64 dense
  // inverse costs 2 n^3 FP64 flops, ~10 s at n = 17,334 on this part's FP64 rate).
  Level &Lc = M->lev[M->nmg - 1];
  const int nc = Lc.ndof;
  if (nc > 40000) {
    set_error("coarsest level too large for the dense coarse solve (more than 40,000 dofs); add a multigrid level");
    return M3SPH_ERR_BAD_INPUT;
  }
  M->coarse.n = nc;
  M->coarse.refine64 = false;
  {
    // free dofs of the coarsest level: the dense inverse covers only them
    std::vector<uint8_t> fm(nc);
    M3_CUDA(cudaMemcpyAsync(fm.data(), Lc.freemask, nc, cudaMemcpyDeviceToHost, s));
    M3_CUDA(cudaStreamSynchronize(s));
    std::vector<int> cmap(nc, -1), fidx;
    fidx.reserve(nc);
    for (int i = 0; i < nc; ++i)
      if (fm[i]) {
        cmap[i] = (int)fidx.size();
        fidx.push_back(i);
      }
    if (!M->coarse.cmap) M3_TRY(dalloc(&M->coarse.cmap, (size_t)nc));
    if (!M->coarse.fidx) M3_TRY(dalloc(&M->coarse.fidx, (size_t)nc));
    M->coarse.nf = (int)fidx.size();
    M3_CUDA(cudaMemcpyAsync(M->coarse.cmap, cmap.data(), sizeof(int) * nc, cudaMemcpyHostToDevice, s));
    if (!fidx.empty())
      M3_CUDA(cudaMemcpyAsync(M->coarse.fidx, fidx.data(), sizeof(int) * fidx.size(), cudaMemcpyHostToDevice, s));
    M3_CUDA(cudaStreamSynchronize(s));
  }
  const int nf = M->coarse.nf;
  if (M->nmg > 1) {
    if (M->precision == 0 && nc <= g_coarse_f64_direct_max) {
      if (!M->coarse.A64) M3_TRY(dalloc(&M->coarse.A64, (size_t)nc * nc));
      M3_TRY(dense_inverse_blocked<double>(Lc, Lc.B64, M->coarse.A64, W->cwork64, M->coarse.cmap, nf, s));
    } else if (M->precision == 0) {
      M->coarse.refine64 = true;
      if (!M->coarse.A32) M3_TRY(dalloc(&M->coarse.A32, (size_t)nc * nc));
      if (!M->coarse.B32tmp) M3_TRY(dalloc(&M->coarse.B32tmp, 9 * (size_t)Lc.nnzb));
      if (!M->coarse.t64) M3_TRY(dalloc(&M->coarse.t64, (size_t)nc));
      M3_TRY(dense_inverse_from64(Lc, Lc.B64, M->coarse.B32tmp, M->coarse.A32, W->cwork32, M->coarse.cmap, nf, s));
    } else {
      if (!M->coarse.A32) M3_TRY(dalloc(&M->coarse.A32, (size_t)nc * nc));
      M3_TRY(dense_inverse_blocked<float>(Lc, Lc.B32, M->coarse.A32, W->cwork32, M->coarse.cmap, nf, s));
    }
  }
  return M3SPH_OK;
}

extern "C" int m3sph_stokes_setup(m3sph_mesh *M, const double *Visc, const double *Dens, const int32_t *ifix,
                                  const double *vfix, int32_t nfix, const m3sph_physics *phys, int32_t precision) {
  if (!M || !Visc || !Dens || (nfix > 0 && (!ifix || !vfix)) || !phys) {
    set_error("m3sph_stokes_setup: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  cudaStream_t s = M->stream;
  auto t0 = std::chrono::steady_clock::now();
  Level &L0 = M->lev[0];
  M->precision = precision ? 1 : 0;
  clear_graphs(M);
  M3_TRY(alloc_work(M));
  Work *W = get_work(M);
  // masks
  std::vector<int> fx(nfix);
  for (int i = 0; i < nfix; ++i) {
    if (ifix[i] < 1 || ifix[i] > L0.ndof) {
      set_error("ifix entry out of range");
      return M3SPH_ERR_BAD_INPUT;
    }
    fx[i] = ifix[i] - 1;
  }
  M->h_ifix = fx;
  M->h_vfix.assign(vfix, vfix + nfix);
  M->has_nonzero_fix = false;
  for (int i = 0; i < nfix; ++i) M->has_nonzero_fix |= vfix[i] != 0.0;
  int *d_fix = nullptr;
  double *d_vals = nullptr;
  M3_TRY(upload(&d_fix, fx.data(), std::max<size_t>(1, fx.size()), s));
  M3_TRY(upload(&d_vals, M->h_vfix.data(), std::max<size_t>(1, fx.size()), s));
  for (int i = 0; i < M->nmg; ++i) {
    Level &L = M->lev[i];
    M3_CUDA(cudaMemsetAsync(L.freemask, 1, L.ndof, s));
    if (nfix) k_set_masks<<<(nfix + 255) / 256, 256, 0, s>>>(L.freemask, d_fix, nfix, L.ndof); count_launch();
  }
  M3_CUDA(cudaMemsetAsync(M->Ufix, 0, sizeof(double) * L0.ndof, s));
  if (nfix) k_scatter_vals<<<(nfix + 255) / 256, 256, 0, s>>>(M->Ufix, d_fix, d_vals, nfix); count_launch();
  M3_CUDA(cudaMemcpyAsync(M->fin.visc, Visc, sizeof(double) * L0.nnod, cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(M->fin.dens, Dens, sizeof(double) * L0.nnod, cudaMemcpyHostToDevice, s));
  {
    // free-dof counts per level
    std::vector<uint8_t> fm(L0.ndof, 1);
    for (int i : fx) fm[i] = 0;
    for (int i = 0; i < M->nmg; ++i) {
      int c = 0;
      for (int d = 0; d < M->lev[i].ndof; ++d) c += fm[d];
      M->lev[i].nfree = c;
    }
  }
  M->phys = *phys;
  M3_TRY(ml_features(M, Visc));
  M3_CUDA(cudaStreamSynchronize(s));
  dfree(d_fix);
  dfree(d_vals);
  cudaEvent_t e0, e1;
  M3_CUDA(cudaEventCreate(&e0));
  M3_CUDA(cudaEventCreate(&e1));
  M3_CUDA(cudaEventRecord(e0, s));
  M3_TRY(rebuild_operator(M));
  M3_CUDA(cudaEventRecord(e1, s));
  M3_CUDA(cudaEventSynchronize(e1));
  float fms = 0.f;
  M3_CUDA(cudaEventElapsedTime(&fms, e0, e1));
  M->last_setup_ms = fms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  M->have_operator = true;
  (void)t0;
  return M3SPH_OK;
}

// update_vel_bc between time steps (update_vel_bc.m:84-150): new prescribed values on the fixed
// dofs of the last set-up. The dof set is unchanged (same masks, colours and coarse free-dof maps),
// so only the resident Ufix is rewritten; the next operator rebuild (every time step, or the next
// m3sph_stokes_solve) folds it into the boundary-condition right-hand side.
extern "C" int m3sph_stokes_set_vel_bc(m3sph_mesh *M, const int32_t *ifix, const double *vfix, int32_t nfix) {
  if (!M || nfix < 0 || (nfix > 0 && (!ifix || !vfix))) {
    set_error("m3sph_stokes_set_vel_bc: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  if (!M->have_operator) {
    set_error("m3sph_stokes_set_vel_bc: call m3sph_stokes_setup first");
    return M3SPH_ERR_BAD_INPUT;
  }
  Level &L0 = M->lev[0];
  std::vector<int> fx(nfix);
  for (int i = 0; i < nfix; ++i) {
    if (ifix[i] < 1 || ifix[i] > L0.ndof) {
      set_error("m3sph_stokes_set_vel_bc: ifix entry out of range");
      return M3SPH_ERR_BAD_INPUT;
    }
    fx[i] = ifix[i] - 1;
  }
  {
    std::vector<int> a(fx), b(M->h_ifix);
    std::sort(a.begin(), a.end());
    std::sort(b.begin(), b.end());
    if (a != b) {
      set_error("m3sph_stokes_set_vel_bc: the fixed dofs differ from the set-up's (a new dof set needs "
                "m3sph_stokes_setup)");
      return M3SPH_ERR_BAD_INPUT;
    }
  }
  M3_CUDA(cudaSetDevice(M->device));
  cudaStream_t s = M->stream;
  M->h_ifix = fx;
  M->h_vfix.assign(vfix, vfix + nfix);
  M->has_nonzero_fix = false;
  for (int i = 0; i < nfix; ++i) M->has_nonzero_fix |= vfix[i] != 0.0;
  int *d_fix = nullptr;
  double *d_vals = nullptr;
  M3_TRY(upload(&d_fix, fx.data(), std::max<size_t>(1, fx.size()), s));
  M3_TRY(upload(&d_vals, M->h_vfix.data(), std::max<size_t>(1, fx.size()), s));
  M3_CUDA(cudaMemsetAsync(M->Ufix, 0, sizeof(double) * L0.ndof, s));
  if (nfix) k_scatter_vals<<<(nfix + 255) / 256, 256, 0, s>>>(M->Ufix, d_fix, d_vals, nfix); count_launch();
  M3_CUDA(cudaGetLastError());
  M3_CUDA(cudaStreamSynchronize(s));
  dfree(d_fix);
  dfree(d_vals);
  M->bc_stale = true;
  return M3SPH_OK;
}

// FP64-accurate finest-level operator for the outer iterations: native FP64 on the plain path,
// double-float FP32 arithmetic on the mixed path
// streamed finest-level operators (TMA ring + fixed-order node sums) for the FP32 V-cycle operator
// and, optionally, for the FP64-accurate outer operators; off: per-colour kernels
static bool g_stream_apply = true;
static bool g_stream_outer = true;

static int outer_apply(m3sph_mesh *M, const double *x, double *y) {
  Level &L0 = M->lev[0];
  if (M->precision == 1 && M->df_outer) {
    if (g_stream_outer && L0.nchunk) return stream_apply_df(L0, L0.K32, L0.KL32, x, y, M->stream);
    return M->split_apply ? ebe_apply_split_df(L0, L0.K32, L0.KL32, x, y, M->stream)
                          : ebe_apply_df(L0, L0.K32, L0.KL32, x, y, M->stream);
  }
  if (g_stream_outer && L0.nchunk) return stream_apply_f64(L0, L0.K64, x, y, M->stream);
  return M->split_apply ? ebe_apply_split_f64(L0, L0.K64, x, y, M->stream)
                        : ebe_apply<double>(L0, L0.K64, x, y, M->stream);
}

// ======================================================================================
// V-cycle (MG_V_cycle_v2) in precision T; level-0 residual r0 given in T, d0 out in T
// ======================================================================================
static const double WD0[3] = {0.9, 0.4, 0.25}, WU0[3] = {0.25, 0.4, 0.9};
static const double WDc[3] = {0.25, 0.4, 0.9}, WUc[3] = {0.9, 0.4, 0.25};

template <typename T> static const T *levK(const Level &L);
template <> const double *levK<double>(const Level &L) { return L.K64; }
template <> const float *levK<float>(const Level &L) { return L.K32; }
template <typename T> static const T *levB(const Level &L);
template <> const double *levB<double>(const Level &L) { return L.B64; }
template <> const float *levB<float>(const Level &L) { return L.B32; }

// level operator: element-by-element on the finest level, assembled blocks on coarse levels
static bool g_split_apply = true;
static int split_apply_T(const Level &L, const float *K, const float *x, float *y, cudaStream_t s) {
  return ebe_apply_split_f32(L, K, x, y, s);
}
static int split_apply_T(const Level &L, const double *K, const double *x, double *y, cudaStream_t s) {
  return ebe_apply_split_f64(L, K, x, y, s);
}
static int stream_apply_T(const Level &L, const float *K, const float *x, float *y, cudaStream_t s) {
  return stream_apply_f32(L, K, x, y, s);
}
static int stream_apply_T(const Level &L, const double *K, const double *x, double *y, cudaStream_t s) {
  return stream_apply_f64(L, K, x, y, s);
}
template <typename T>
static int level_op(const Level &L, int img, const T *x, T *y, cudaStream_t s) {
  if (img > 0 && levB<T>(L)) return bsr_apply<T>(L, levB<T>(L), x, y, s);
  if constexpr (std::is_same<T, float>::value) {
    if (img == 0 && g_pa_apply && L.pa_ready) return pa_apply_f32(L, x, y, s);
  }
  if ((std::is_same<T, float>::value ? g_stream_apply : g_stream_outer) && L.nchunk && levK<T>(L))
    return stream_apply_T(L, levK<T>(L), x, y, s);
  if (g_split_apply) return split_apply_T(L, levK<T>(L), x, y, s);
  return ebe_apply<T>(L, levK<T>(L), x, y, s);
}

template <typename T> static const T *levDi(const Level &L);
template <> const double *levDi<double>(const Level &L) { return L.Dinv64; }
template <> const float *levDi<float>(const Level &L) { return L.Dinv32; }

// kd = K d, then d += w (r - kd) / diag; fused into one pass on the streamed finest level (kd is
// then not written)
template <typename T>
static int level_op_jac(const Level &L, int img, T w, const T *r, T *d, T *kd, cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value) {
    if (img == 0 && g_pa_apply && L.pa_ready) return pa_apply_jac_f32(L, w, r, L.Dinv32, d, s);
    if (img == 0 && g_stream_apply && L.nchunk && L.K32) return stream_apply_jac_f32(L, L.K32, w, r, L.Dinv32, d, s);
  }
  M3_TRY(level_op<T>(L, img, d, kd, s));
  return jac<T>(w, r, kd, levDi<T>(L), d, L.ndof, s);
}

// the coarsest-level solve of the V-cycle: one GEMV with the dense inverse, or on the plain FP64
// path with a large coarsest level the FP32 inverse refined against the FP64 operator
template <typename T>
static int coarse_solve(m3sph_mesh *M, const T *Ainv, const T *r, T *d) {
  const Level &Lc = M->lev[M->nmg - 1];
  if constexpr (std::is_same<T, double>::value) {
    if (M->coarse.refine64)
      return coarse_refined(Lc, M->coarse.A32, Lc.B64, r, d, M->coarse.t64, g_coarse_refine_sweeps, M->coarse.fidx,
                            M->coarse.nf, M->stream);
  }
  return dense_gemv<T>(Ainv, M->coarse.n, M->coarse.nf, M->coarse.fidx, r, d, M->stream);
}

template <typename T>
static int vcycle_T(m3sph_mesh *M, std::vector<T *> &r, std::vector<T *> &d, std::vector<T *> &kd,
                    std::vector<T *> &tmp, const T *Ainv) {
  cudaStream_t s = M->stream;
  const int nm = M->nmg;
  if (nm == 1) {
    M3_TRY(dense_gemv<T>(Ainv, M->coarse.n, M->coarse.nf, M->coarse.fidx, r[0], d[0], s));
    return M3SPH_OK;
  }
  const bool ml = M->smoother_active;
  // learned levels: the two finest (schedules 0, 1, 3) or the finest only (schedule 2)
  const int nml = M->ml_schedule == 2 ? 1 : 2;
  const bool one = M->ml_schedule == 1 || M->ml_schedule == 2;
  for (int j = 0; j < nm - 1; ++j) {
    const Level &L = M->lev[j];
    const double *w = j == 0 ? WD0 : WDc;
    const size_t n = L.ndof;
    if (ml && j < nml && one) {
      // one learned sweep from zero, then the residual for the restriction
      M3_CUDA(cudaMemsetAsync(d[j], 0, sizeof(T) * n, s));
      M3_TRY(ml_sweep<T>(M, j, r[j], nullptr, levDi<T>(L), tmp[j], d[j]));
      M3_TRY(level_op<T>(L, j, d[j], kd[j], s));
    } else if (ml && j < nml && M->ml_schedule == 3) {
      // learned sweep from zero, one weighted Jacobi sweep, residual
      M3_CUDA(cudaMemsetAsync(d[j], 0, sizeof(T) * n, s));
      M3_TRY(ml_sweep<T>(M, j, r[j], nullptr, levDi<T>(L), tmp[j], d[j]));
      M3_TRY(level_op_jac<T>(L, j, (T)w[2], r[j], d[j], kd[j], s));
      M3_TRY(level_op<T>(L, j, d[j], kd[j], s));
    } else if (ml && j < nml) {
      // learned sweep, weighted Jacobi sweep, learned sweep
      M3_CUDA(cudaMemsetAsync(d[j], 0, sizeof(T) * n, s));
      M3_TRY(ml_sweep<T>(M, j, r[j], nullptr, levDi<T>(L), tmp[j], d[j]));
      M3_TRY(level_op<T>(L, j, d[j], kd[j], s));
      M3_TRY(jac<T>((T)w[1], r[j], kd[j], levDi<T>(L), d[j], n, s));
      M3_TRY(level_op<T>(L, j, d[j], kd[j], s));
      M3_TRY(ml_sweep<T>(M, j, r[j], kd[j], levDi<T>(L), tmp[j], d[j]));
      M3_TRY(level_op<T>(L, j, d[j], kd[j], s));
    } else {
      M3_TRY(jac_first<T>((T)w[0], r[j], levDi<T>(L), d[j], n, s));
      for (int k = 1; k < 3; ++k) M3_TRY(level_op_jac<T>(L, j, (T)w[k], r[j], d[j], kd[j], s));
      M3_TRY(level_op<T>(L, j, d[j], kd[j], s));
    }
    M3_TRY(restrict_<T>(L, M->lev[j + 1], r[j], kd[j], r[j + 1], s));
  }
  M3_TRY(coarse_solve<T>(M, Ainv, r[nm - 1], d[nm - 1]));
  for (int j = nm - 2; j >= 0; --j) {
    const Level &L = M->lev[j];
    const double *w = j == 0 ? WU0 : WUc;
    const size_t n = L.ndof;
    M3_TRY(prolong<T>(L, M->lev[j + 1], d[j + 1], d[j], d[j], s));
    if (ml && j < nml && one) {
      M3_TRY(level_op<T>(L, j, d[j], kd[j], s));
      M3_TRY(ml_sweep<T>(M, j, r[j], kd[j], levDi<T>(L), tmp[j], d[j]));
    } else if (ml && j < nml && M->ml_schedule == 3) {
      M3_TRY(level_op_jac<T>(L, j, (T)w[0], r[j], d[j], kd[j], s));
      M3_TRY(level_op<T>(L, j, d[j], kd[j], s));
      M3_TRY(ml_sweep<T>(M, j, r[j], kd[j], levDi<T>(L), tmp[j], d[j]));
    } else if (ml && j < nml) {
      M3_TRY(level_op<T>(L, j, d[j], kd[j], s));
      M3_TRY(ml_sweep<T>(M, j, r[j], kd[j], levDi<T>(L), tmp[j], d[j]));
      M3_TRY(level_op<T>(L, j, d[j], kd[j], s));
      M3_TRY(jac<T>((T)w[1], r[j], kd[j], levDi<T>(L), d[j], n, s));
      M3_TRY(level_op<T>(L, j, d[j], kd[j], s));
      M3_TRY(ml_sweep<T>(M, j, r[j], kd[j], levDi<T>(L), tmp[j], d[j]));
    } else {
      for (int k = 0; k < 3; ++k) M3_TRY(level_op_jac<T>(L, j, (T)w[k], r[j], d[j], kd[j], s));
    }
  }
  return M3SPH_OK;
}

// d (fp64) = B r (fp64) in the set-up precision
static int vcycle(m3sph_mesh *M, const double *r, double *dout) {
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  const size_t n0 = M->lev[0].ndof;
  if (M->precision == 0) {
    std::vector<double *> rr = W->r64, dd = W->d64;
    rr[0] = const_cast<double *>(r);
    dd[0] = dout;
    return vcycle_T<double>(M, rr, dd, W->kd64, W->t64, M->coarse.A64);
  }
  M3_TRY(d2f(r, W->r32[0], n0, s));
  M3_TRY(vcycle_T<float>(M, W->r32, W->d32, W->kd32, W->t32, M->coarse.A32));
  M3_TRY(f2d(W->d32[0], dout, n0, s));
  return M3SPH_OK;
}

// ======================================================================================
// flexible MG-PCG (mgpcg_solver_p.m:117-199), FP64 outer iteration
// ======================================================================================
struct CGStats {
  int it = 0;
  double rrms = 0.0;
  int nvc = 0;
};

static int read_scal(m3sph_mesh *M, int idx, double &v) {
  M3_CUDA(cudaMemcpyAsync(M->h_scal + idx, M->scal + idx, sizeof(double), cudaMemcpyDeviceToHost, M->stream));
  M3_CUDA(cudaStreamSynchronize(M->stream));
  v = M->h_scal[idx];
  return M3SPH_OK;
}

__global__ void k_set_scal(double *scal, int idx, double v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) scal[idx] = v;
}
static int set_first_flag(m3sph_mesh *M, double v) {
  k_set_scal<<<1, 1, 0, M->stream>>>(M->scal, 6, v); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// one flexible-PCG iteration on device-resident data (no host synchronisation): V-cycle,
// Polak-Ribiere direction, K q, step and residual norm into scal[3]
static int cg_iteration(m3sph_mesh *M, double *x) {
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  Level &L0 = M->lev[0];
  const size_t n = L0.ndof;
  M3_TRY(vcycle(M, W->r, W->d));
  M3_TRY(dot2(W->r, W->Kq, W->d, n, M->red, M->scal + 0, s));   // scal[0]=r.d, scal[1]=Kq_prev.d
  M3_TRY(cg_dir(W->d, W->q, n, M->scal, -1, s));                // first-iteration flag in scal[6]
  M3_TRY(outer_apply(M, W->q, W->Kq));
  M3_TRY(dot(W->q, W->Kq, n, M->red, M->scal + 2, s));
  M3_TRY(cg_update(x, W->r, W->q, W->Kq, n, M->scal, M->red, s));
  M3_TRY(set_first_flag(M, 0.0));
  return M3SPH_OK;
}

// the iteration captured once per solution-vector pointer as a CUDA graph and replayed
static int iteration_graph(m3sph_mesh *M, double *x, cudaGraphExec_t *out) {
  double *key = M->smoother_active ? x + 1 : x;   // separate graphs with / without the learned smoother
  for (auto &g : M->graphs)
    if (g.first == key) {
      *out = g.second;
      return M3SPH_OK;
    }
  cudaStream_t s = M->stream;
  cudaGraph_t graph;
  const unsigned long long n0 = g_launches.load();
  M3_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  const int st = cg_iteration(M, x);
  // kernels in the graph are counted at each replay, not at capture
  const unsigned long long nk = g_launches.load() - n0;
  g_launches.fetch_sub(nk);
  M->graph_kernels = nk;
  cudaError_t ce = cudaStreamEndCapture(s, &graph);
  if (st) return st;
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
  cudaGraphExec_t exec;
  ce = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaGraphInstantiate");
  M->graphs.push_back({key, exec});
  *out = exec;
  return M3SPH_OK;
}

static void clear_graphs(m3sph_mesh *M) {
  for (auto &g : M->graphs) cudaGraphExecDestroy(g.second);
  M->graphs.clear();
}

// b masked to free dofs on entry; x holds the initial guess (fixed entries are left unchanged)
static int mgpcg(m3sph_mesh *M, const double *b, double *x, double tol, bool abs_tol, int itmax, CGStats &st) {
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  Level &L0 = M->lev[0];
  const size_t n = L0.ndof;
  const double sq = std::sqrt((double)std::max(1, L0.nfree));
  M3_TRY(outer_apply(M, x, W->r));
  M3_TRY(sub_mask(b, W->r, L0.freemask, n, s));
  M3_TRY(dot(W->r, W->r, n, M->red, M->scal + 3, s));
  double rr;
  M3_TRY(read_scal(M, 3, rr));
  if (std::isnan(rr)) {
    set_error("RHS vector contains NaNs");
    return M3SPH_ERR_NAN;
  }
  double rrms = std::sqrt(rr) / sq;
  if (!abs_tol) tol = tol * rrms;
  st.it = 0;
  int it = 0;
  M3_TRY(set_first_flag(M, 1.0));
  cudaGraphExec_t exec = nullptr;
  if (M->use_graphs) M3_TRY(iteration_graph(M, x, &exec));
  int itlim = itmax;
  for (it = 1; it <= itlim; ++it) {
    if (exec) {
      M3_CUDA(cudaGraphLaunch(exec, s));
      add_launches(M->graph_kernels);
    } else {
      M3_TRY(cg_iteration(M, x));
    }
    st.nvc++;
    M3_TRY(read_scal(M, 3, rr));
    const double rrms_prev = rrms;
    rrms = std::sqrt(rr) / sq;
    if (std::isnan(rrms)) {
      set_error("NaN in MG-PCG residual");
      return M3SPH_ERR_NAN;
    }
    if (rrms < tol) break;
    // learned-smoother fallback: a contraction factor above 0.95 (or growth) switches the rest of
    // the solve to the Jacobi smoother
    // the same when the learned smoother runs out of iterations above the tolerance: the solve
    // goes on with Jacobi smoothing for another itmax iterations (flexible CG accepts the change
    // of preconditioner) rather than handing a less accurate K^-1 to the Patera iteration
    const bool stalled = it > 1 && rrms > 0.95 * rrms_prev;
    const bool exhausted = it == itlim;
    if (M->smoother_active && (stalled || exhausted)) {
      M->smoother_active = false;
      M->smoother_fallbacks++;
      if (exhausted) itlim += itmax;
      exec = nullptr;
      if (M->use_graphs) M3_TRY(iteration_graph(M, x, &exec));
    }
  }
  st.it = std::min(it, itlim);
  st.rrms = rrms;
  return M3SPH_OK;
}

// ======================================================================================
// Patera pressure CG (flow3d_patera_mg_sph_p.m:386-632)
// ======================================================================================
static int pdot(m3sph_mesh *M, const double *a, const double *b, double &v) {
  M3_TRY(dot(a, b, M->lev[0].nvnod, M->red, M->scal + 8, M->stream));
  return read_scal(M, 8, v);
}
__global__ void k_shift(double *a, double c, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] += c;
}
__global__ void k_precond_p1(const double *r, const double *LiMM, double *d, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = r[i] * LiMM[i];
}
__global__ void k_precond_p2(const double *r, const double *Md, const double *LiMM, double *d, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] += LiMM[i] * (r[i] - Md[i]);
}
__global__ void k_rhs(const double *Fb, const double *GP, const double *bc, const uint8_t *mask, double *out, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = mask[i] ? Fb[i] + GP[i] - bc[i] : 0.0;
}
__global__ void k_scale(double *a, double c, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] *= c;
}
// Cartesian component r of node n's velocity from its rotated-frame dofs (U_xyz = RR U)
__device__ __forceinline__ double rotate_back_comp(const double *U, const double *RR, int nnod, int n, int r) {
  double v = 0.0;
  for (int c = 0; c < 3; ++c) v += RR[(size_t)(r * 3 + c) * nnod + n] * U[3 * n + c];
  return v;
}
__global__ void k_rotate_back(const double *U, const double *RR, int nnod, double *Uxyz) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnod) return;
  for (int r = 0; r < 3; ++r) Uxyz[3 * n + r] = rotate_back_comp(U, RR, nnod, n, r);
}

// max |Ux|, |Uy|, |Uz| of the resident solution (calculate_dt.m:40-42): warp-shuffle maxima, one
// atomicMax per warp on the bit patterns (non-negative doubles order like their uint64 bits)
__global__ void k_absmax_xyz(const double *U, const double *RR, int nnod, unsigned long long *out) {
  double m[3] = {0.0, 0.0, 0.0};
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnod; n += gridDim.x * blockDim.x)
    for (int r = 0; r < 3; ++r) m[r] = fmax(m[r], fabs(rotate_back_comp(U, RR, nnod, n, r)));
  for (int r = 0; r < 3; ++r) {
    double v = m[r];
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out + r, (unsigned long long)__double_as_longlong(v));
  }
}

static int remove_mean(m3sph_mesh *M, double *a) {
  const int np = M->lev[0].nvnod;
  M3_TRY(vsum(a, np, M->red, M->scal + 9, M->stream));
  double sm;
  M3_TRY(read_scal(M, 9, sm));
  k_shift<<<(np + 255) / 256, 256, 0, M->stream>>>(a, -sm / np, np); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

static int build_rhs(m3sph_mesh *M, const double *P, double *Rhs) {
  Work *W = get_work(M);
  Level &L0 = M->lev[0];
  M3_TRY(grad_apply(L0, M->fin.G64, P, W->y, M->stream));
  k_rhs<<<(unsigned)((L0.ndof + 255) / 256), 256, 0, M->stream>>>(M->fin.Fb, W->y, M->bc_rhs, L0.freemask, Rhs,
                                                                  L0.ndof);
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// coupled FP64 relative residual
static int coupled_residual(m3sph_mesh *M, const double *U, const double *P, double &rel) {
  Work *W = get_work(M);
  Level &L0 = M->lev[0];
  cudaStream_t s = M->stream;
  const size_t n = L0.ndof;
  const int np = L0.nvnod;
  // f = mask(Fb - bc_rhs)
  M3_CUDA(cudaMemsetAsync(W->tmp, 0, sizeof(double) * n, s));
  k_rhs<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(M->fin.Fb, W->tmp, M->bc_rhs, L0.freemask, W->Rhs, n); count_launch();
  double ff;
  M3_TRY(dot(W->Rhs, W->Rhs, n, M->red, M->scal + 10, s));
  M3_TRY(read_scal(M, 10, ff));
  // ru = mask(Fb + G P - bc - K U)
  M3_TRY(build_rhs(M, P, W->Rhs));
  M3_TRY(outer_apply(M, U, W->tmp));
  M3_TRY(sub_mask(W->Rhs, W->tmp, L0.freemask, n, s));
  double ru;
  M3_TRY(dot(W->tmp, W->tmp, n, M->red, M->scal + 10, s));
  M3_TRY(read_scal(M, 10, ru));
  // rp = -G' U, mean removed
  M3_TRY(div_apply(L0, M->fin.G64, U, W->pt, s));
  M3_TRY(remove_mean(M, W->pt));
  double rp;
  M3_TRY(dot(W->pt, W->pt, np, M->red, M->scal + 10, s));
  M3_TRY(read_scal(M, 10, rp));
  rel = std::sqrt(ru + rp) / std::sqrt(std::max(ff, 1e-300));
  return M3SPH_OK;
}

static int precondition_P(m3sph_mesh *M, const double *r, double *d) {
  Work *W = get_work(M);
  const int np = M->lev[0].nvnod;
  k_precond_p1<<<(np + 255) / 256, 256, 0, M->stream>>>(r, M->fin.LiMM, d, np); count_launch();
  M3_TRY(mass_apply(M->lev[0], M->fin.M64, d, W->pSq, M->stream));   // pSq used as temp (Md)
  k_precond_p2<<<(np + 255) / 256, 256, 0, M->stream>>>(r, W->pSq, M->fin.LiMM, d, np); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// Patera solve on device-resident data: the initial pressure must be in the workspace pressure
// vector; U and P stay on the device (workspace U is the rotated-frame velocity).
static int solve_core(m3sph_mesh *M, const m3sph_opts *opts, m3sph_info &inf) {
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  Level &L0 = M->lev[0];
  const size_t n = L0.ndof;
  const int np = L0.nvnod;
  M->smoother_active = opts->smoother == 1 && ml_ready(M);
  M->smoother_fallbacks = 0;
  double rtol_Pat = opts->rtol_Pat > 0 ? opts->rtol_Pat : 1e-4;
  double rtol_U = opts->rtol_U > 0 ? opts->rtol_U : 5e-3;
  const int itmax_Pat = opts->itmax_Pat > 0 ? opts->itmax_Pat : 120;
  const int itmin_Pat = opts->itmin_Pat > 0 ? opts->itmin_Pat : 3;
  const int itmax_U = opts->itmax_U > 0 ? opts->itmax_U : 20;
  const double rtol_restart = 0.8 * rtol_Pat;
  const double sqp = std::sqrt((double)np);
  double *U = W->U, *Pd = W->pP, *r = W->pr, *d = W->pd, *q = W->pq, *Sq = W->pSq, *z = W->z, *y = W->y;
  M3_CUDA(cudaMemcpyAsync(U, M->Ufix, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  CGStats cs;
  // initial velocity
  M3_TRY(build_rhs(M, Pd, W->Rhs));
  M3_TRY(mgpcg(M, W->Rhs, U, rtol_U * rtol_restart, false, itmax_U, cs));
  inf.nitU += cs.it;
  // initial pressure residual r = -G'U
  M3_TRY(div_apply(L0, M->fin.G64, U, r, s));
  k_scale<<<(np + 255) / 256, 256, 0, s>>>(r, -1.0, np); count_launch();
  M3_TRY(remove_mean(M, r));
  double rr;
  M3_TRY(pdot(M, r, r, rr));
  double norm_rP = std::sqrt(rr) / sqp;
  double tol_Pat = rtol_Pat * norm_rP;
  M3_TRY(mgpcg(M, W->Rhs, U, rtol_U * rtol_restart * norm_rP, true, itmax_U, cs));
  inf.nitU += cs.it;
  double tol_U_restart = rtol_U * tol_Pat;
  bool restart = true, conv_problem = false;
  double norm_rP0 = norm_rP, rd = 0.0, rdlast = 0.0, tol_Z = 0.0;
  int itPat = 0;
  const double target = opts->target_rel_residual;
  bool converged = false;
  for (itPat = 1; itPat <= itmax_Pat; ++itPat) {
    M3_TRY(precondition_P(M, r, d));
    if (restart) {
      M3_CUDA(cudaMemcpyAsync(q, d, sizeof(double) * np, cudaMemcpyDeviceToDevice, s));
      restart = false;
      norm_rP0 = norm_rP;
      tol_Z = rtol_U * std::max(rtol_restart * norm_rP0, tol_Pat);
    } else {
      // beta = (r - rlast).d / rdlast
      double rd_new, rld;
      M3_TRY(pdot(M, r, d, rd_new));
      M3_TRY(pdot(M, W->prl, d, rld));
      const double beta = (rd_new - rld) / rdlast;
      M3_TRY(axpby(1.0, d, beta, q, np, s));
    }
    M3_TRY(remove_mean(M, q));
    M3_TRY(pdot(M, r, d, rd));
    rdlast = rd;
    M3_TRY(grad_apply(L0, M->fin.G64, q, y, s));
    M3_TRY(apply_mask(y, L0.freemask, n, s));
    M3_CUDA(cudaMemsetAsync(z, 0, sizeof(double) * n, s));
    M3_TRY(mgpcg(M, y, z, tol_Z, true, itmax_U, cs));
    inf.nitZ += cs.it;
    M3_TRY(div_apply(L0, M->fin.G64, z, Sq, s));
    double qSq;
    M3_TRY(pdot(M, q, Sq, qSq));
    M3_CUDA(cudaMemcpyAsync(W->prl, r, sizeof(double) * np, cudaMemcpyDeviceToDevice, s));
    const double alpha = rd / qSq;
    M3_TRY(axpby(alpha, q, 1.0, Pd, np, s));
    M3_TRY(axpby(alpha, z, 1.0, U, n, s));
    M3_TRY(axpby(-alpha, Sq, 1.0, r, np, s));
    M3_TRY(remove_mean(M, r));
    const double norm_rP_last = norm_rP;
    M3_TRY(pdot(M, r, r, rr));
    norm_rP = std::sqrt(rr) / sqp;
    if (std::isnan(norm_rP)) {
      set_error("Solution containes NaNs !!!!");
      return M3SPH_ERR_NAN;
    }
    const double norm_rP_min = std::min(norm_rP_last, norm_rP);
    bool done = norm_rP < tol_Pat && itPat >= itmin_Pat;
    if (done && target > 0) {
      double rel;
      M3_TRY(coupled_residual(M, U, Pd, rel));
      if (rel > target) {
        // the coupled residual is not yet at the target: tighten both tolerances, replace the
        // recursively updated pressure residual (it drifts from -G'U over many iterations) by the
        // true one of a velocity solved for the current pressure, and restart the CG direction
        tol_Pat *= 0.1;
        rtol_U *= 0.1;
        tol_U_restart = rtol_U * tol_Pat;
        M3_TRY(build_rhs(M, Pd, W->Rhs));
        M3_TRY(mgpcg(M, W->Rhs, U, tol_U_restart, true, itmax_U, cs));
        inf.nitU += cs.it;
        M3_TRY(div_apply(L0, M->fin.G64, U, r, s));
        k_scale<<<(np + 255) / 256, 256, 0, s>>>(r, -1.0, np); count_launch();
        M3_TRY(remove_mean(M, r));
        M3_TRY(pdot(M, r, r, rr));
        norm_rP = std::sqrt(rr) / sqp;
        restart = true;
        continue;
      }
    }
    if (done) {
      converged = true;
      break;
    }
    if (norm_rP < rtol_restart * norm_rP0 || norm_rP > 10 * norm_rP0) {
      M3_TRY(build_rhs(M, Pd, W->Rhs));
      M3_TRY(mgpcg(M, W->Rhs, U, tol_U_restart, true, itmax_U, cs));
      inf.nitU += cs.it;
      M3_TRY(div_apply(L0, M->fin.G64, U, r, s));
      k_scale<<<(np + 255) / 256, 256, 0, s>>>(r, -1.0, np); count_launch();
      double rt;
      M3_TRY(pdot(M, r, r, rt));
      const double norm_rP_true = std::sqrt(rt) / sqp;
      if (norm_rP_true > 1.1 * norm_rP) {
        rtol_U = rtol_U * 0.75 * (norm_rP / norm_rP_true);
        tol_U_restart = rtol_U * tol_Pat;
      }
      if (norm_rP > 10 * norm_rP0 || norm_rP > 1.2 * norm_rP_min) {
        if (conv_problem) break;
        rtol_U = 0.1 * rtol_U;
        tol_U_restart = rtol_U * tol_Pat;
        conv_problem = true;
      }
      restart = true;
    }
  }
  M3_TRY(build_rhs(M, Pd, W->Rhs));
  M3_TRY(mgpcg(M, W->Rhs, U, tol_U_restart, true, itmax_U, cs));
  inf.nitU += cs.it;
  inf.itPat = std::min(itPat, itmax_Pat);
  inf.norm_rP = norm_rP;
  inf.smoother_fallbacks = M->smoother_fallbacks;
  M->smoother_active = false;
  inf.nvcycle = cs.nvc;
  double rel = 0.0;
  M3_TRY(coupled_residual(M, U, Pd, rel));
  inf.rel_residual = rel;
  M3_TRY(stream_check(L0, s));
  M3_TRY(ml_check(M));
  // The reference returns its last iterate silently when itmax_Pat runs out or after the second
  // convergence problem (flow3d_patera_mg_sph_p.m:580-606); here the iterate is still returned, but
  // with M3SPH_ERR_NOT_CONVERGED. With a target the final coupled residual decides.
  if (target > 0) converged = rel <= target;
  if (!converged) {
    char msg[200];
    snprintf(msg, sizeof msg, "Patera iteration not converged: %d iterations (itmax_Pat %d), norm_rP %.3e, "
             "coupled residual %.3e (target %.1e)", inf.itPat, itmax_Pat, norm_rP, rel, target);
    set_error(msg);
    inf.status = M3SPH_ERR_NOT_CONVERGED;
    return M3SPH_ERR_NOT_CONVERGED;
  }
  return M3SPH_OK;
}

static int need_op_fwd(m3sph_mesh *M) {
  if (!M || !M->have_operator) {
    set_error("operator not set up (call m3sph_stokes_setup)");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  return M3SPH_OK;
}

static int time_since(cudaEvent_t a, cudaEvent_t b, double &ms) {
  float f = 0.f;
  M3_CUDA(cudaEventElapsedTime(&f, a, b));
  ms = f;
  return M3SPH_OK;
}

extern "C" int m3sph_stokes_solve(m3sph_mesh *M, double *U_xyz, double *P, const m3sph_opts *opts,
                                  m3sph_info *info) {
  if (!M || !U_xyz || !P || !opts) {
    set_error("m3sph_stokes_solve: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  if (!M->have_operator) {
    set_error("m3sph_stokes_solve: call m3sph_stokes_setup first");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  Level &L0 = M->lev[0];
  // prescribed values replaced by m3sph_stokes_set_vel_bc since the last rebuild
  if (M->bc_stale) M3_TRY(rebuild_operator(M));
  M3_CUDA(cudaMemcpyAsync(W->pP, P, sizeof(double) * L0.nvnod, cudaMemcpyHostToDevice, s));
  cudaEvent_t e0, e1;
  M3_CUDA(cudaEventCreate(&e0));
  M3_CUDA(cudaEventCreate(&e1));
  M3_CUDA(cudaEventRecord(e0, s));
  m3sph_info inf{};
  // M3SPH_ERR_NOT_CONVERGED still delivers the last iterate (and the info) to the caller
  const int st = solve_core(M, opts, inf);
  if (st && st != M3SPH_ERR_NOT_CONVERGED) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
  }
  M3_CUDA(cudaEventRecord(e1, s));
  // back-rotation U_xyz = RR U
  k_rotate_back<<<(L0.nnod + 255) / 256, 256, 0, s>>>(W->U, M->fin.RR, L0.nnod, W->tmp); count_launch();
  M3_CUDA(cudaMemcpyAsync(U_xyz, W->tmp, sizeof(double) * L0.ndof, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaMemcpyAsync(P, W->pP, sizeof(double) * L0.nvnod, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  M3_TRY(time_since(e0, e1, inf.t_iter_ms));
  inf.t_setup_ms = M->last_setup_ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  inf.status = st;
  if (info) *info = inf;
  return st;
}

extern "C" int m3sph_stokes_step_device(m3sph_mesh *M, const m3sph_opts *opts, m3sph_info *info) {
  if (!M || !opts || !M->have_operator) {
    set_error("m3sph_stokes_step_device: call m3sph_stokes_setup first");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  cudaEvent_t e0, e1, e2;
  M3_CUDA(cudaEventCreate(&e0));
  M3_CUDA(cudaEventCreate(&e1));
  M3_CUDA(cudaEventCreate(&e2));
  M3_CUDA(cudaEventRecord(e0, s));
  M3_TRY(rebuild_operator(M));
  M3_CUDA(cudaEventRecord(e1, s));
  M3_CUDA(cudaMemsetAsync(W->pP, 0, sizeof(double) * M->lev[0].nvnod, s));
  m3sph_info inf{};
  const int st = solve_core(M, opts, inf);
  if (st && st != M3SPH_ERR_NOT_CONVERGED) return st;
  M3_CUDA(cudaEventRecord(e2, s));
  M3_CUDA(cudaEventSynchronize(e2));
  M3_TRY(time_since(e0, e1, inf.t_setup_ms));
  M3_TRY(time_since(e1, e2, inf.t_iter_ms));
  for (cudaEvent_t e : {e0, e1, e2}) cudaEventDestroy(e);
  inf.status = st;
  if (info) *info = inf;
  return st;
}

extern "C" int m3sph_stream(m3sph_mesh *M, void **stream) {
  if (!M || !stream) {
    set_error("bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  *stream = (void *)M->stream;
  return M3SPH_OK;
}

extern "C" int m3sph_solution(m3sph_mesh *M, double *U_xyz, double *P) {
  M3_TRY(need_op_fwd(M));
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  Level &L0 = M->lev[0];
  k_rotate_back<<<(L0.nnod + 255) / 256, 256, 0, s>>>(W->U, M->fin.RR, L0.nnod, W->tmp); count_launch();
  if (U_xyz) M3_CUDA(cudaMemcpyAsync(U_xyz, W->tmp, sizeof(double) * L0.ndof, cudaMemcpyDeviceToHost, s));
  if (P) M3_CUDA(cudaMemcpyAsync(P, W->pP, sizeof(double) * L0.nvnod, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

__global__ void k_velocity_soa(const double *U, const double *RR, int nnod, double *out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnod) return;
  for (int r = 0; r < 3; ++r) out[(size_t)r * nnod + n] = rotate_back_comp(U, RR, nnod, n, r);
}

namespace m3sph {
// hooks for the device-resident time step (timestep.cu)
int stokes_velocity_soa(m3sph_mesh *M, double *dst) {
  Work *W = get_work(M);
  const int n = M->lev[0].nnod;
  k_velocity_soa<<<(n + 255) / 256, 256, 0, M->stream>>>(W->U, M->fin.RR, n, dst); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
int stokes_resident_solve(m3sph_mesh *M, const m3sph_opts *opts, bool zero_p, m3sph_info &inf) {
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  cudaEvent_t e0, e1, e2;
  M3_CUDA(cudaEventCreate(&e0));
  M3_CUDA(cudaEventCreate(&e1));
  M3_CUDA(cudaEventCreate(&e2));
  M3_CUDA(cudaEventRecord(e0, s));
  M3_TRY(rebuild_operator(M));
  M3_CUDA(cudaEventRecord(e1, s));
  if (zero_p) M3_CUDA(cudaMemsetAsync(W->pP, 0, sizeof(double) * M->lev[0].nvnod, s));
  inf = m3sph_info{};
  const int st = solve_core(M, opts, inf);
  if (st && st != M3SPH_ERR_NOT_CONVERGED) return st;
  M3_CUDA(cudaEventRecord(e2, s));
  M3_CUDA(cudaEventSynchronize(e2));
  M3_TRY(time_since(e0, e1, inf.t_setup_ms));
  M3_TRY(time_since(e1, e2, inf.t_iter_ms));
  for (cudaEvent_t e : {e0, e1, e2}) cudaEventDestroy(e);
  inf.status = st;
  return st;
}
int stokes_calc_dt(m3sph_mesh *M, double dt_adv_limit, double dtmax, double *dt, double *dt_adv);
int stokes_set_pressure(m3sph_mesh *M, const double *P) {
  Work *W = get_work(M);
  M3_CUDA(cudaMemcpyAsync(W->pP, P, sizeof(double) * M->lev[0].nvnod, cudaMemcpyHostToDevice, M->stream));
  M3_CUDA(cudaStreamSynchronize(M->stream));
  return M3SPH_OK;
}
}  // namespace m3sph

extern "C" int m3sph_calculate_dt(m3sph_mesh *M, double dt_adv_limit, double dtmax, double *dt, double *dt_adv) {
  M3_TRY(need_op_fwd(M));
  if (!dt) {
    set_error("m3sph_calculate_dt: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  return m3sph::stokes_calc_dt(M, dt_adv_limit, dtmax, dt, dt_adv);
}

int m3sph::stokes_calc_dt(m3sph_mesh *M, double dt_adv_limit, double dtmax, double *dt, double *dt_adv) {
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  Level &L0 = M->lev[0];
  unsigned long long *mx = reinterpret_cast<unsigned long long *>(M->scal + 12);
  M3_CUDA(cudaMemsetAsync(mx, 0, 3 * sizeof(double), s));
  k_absmax_xyz<<<152 * 4, 256, 0, s>>>(W->U, M->fin.RR, L0.nnod, mx); count_launch();
  M3_CUDA(cudaGetLastError());
  M3_CUDA(cudaMemcpyAsync(M->h_scal + 12, M->scal + 12, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  const double mux = M->h_scal[12], muy = M->h_scal[13], muz = M->h_scal[14];
  if (std::isnan(mux) || std::isnan(muy) || std::isnan(muz)) {
    set_error("m3sph_calculate_dt: velocity contains NaNs");
    return M3SPH_ERR_NAN;
  }
  // calculate_dt.m:43-52; Lx/0 is +Inf and drops out of the min as in MATLAB
  double adv = 0.0, out = dtmax;
  if (!(mux == 0.0 && muy == 0.0 && muz == 0.0)) {
    adv = dt_adv_limit * std::min(std::min(M->Lx / mux, M->Ly / muy), M->Lz / muz);
    out = std::min(dtmax, adv);
  }
  *dt = out;
  if (dt_adv) *dt_adv = adv;
  return M3SPH_OK;
}

// ======================================================================================
// operator-level entry points (tests, benchmarks)
// ======================================================================================
static int need_op(m3sph_mesh *M) {
  if (!M || !M->have_operator) {
    set_error("operator not set up (call m3sph_stokes_setup)");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  return M3SPH_OK;
}

extern "C" int m3sph_stokes_apply(m3sph_mesh *M, const double *x, double *y) {
  M3_TRY(need_op(M));
  Work *W = get_work(M);
  Level &L0 = M->lev[0];
  cudaStream_t s = M->stream;
  M3_CUDA(cudaMemcpyAsync(W->tmp, x, sizeof(double) * L0.ndof, cudaMemcpyHostToDevice, s));
  M3_TRY(outer_apply(M, W->tmp, W->y));
  M3_CUDA(cudaMemcpyAsync(y, W->y, sizeof(double) * L0.ndof, cudaMemcpyDeviceToHost, s));
  M3_TRY(stream_check(L0, s));
  return M3SPH_OK;
}

extern "C" int m3sph_grad_apply(m3sph_mesh *M, const double *q, double *y) {
  M3_TRY(need_op(M));
  Work *W = get_work(M);
  Level &L0 = M->lev[0];
  cudaStream_t s = M->stream;
  M3_CUDA(cudaMemcpyAsync(W->pt, q, sizeof(double) * L0.nvnod, cudaMemcpyHostToDevice, s));
  M3_TRY(grad_apply(L0, M->fin.G64, W->pt, W->y, s));
  M3_CUDA(cudaMemcpyAsync(y, W->y, sizeof(double) * L0.ndof, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

extern "C" int m3sph_div_apply(m3sph_mesh *M, const double *z, double *out) {
  M3_TRY(need_op(M));
  Work *W = get_work(M);
  Level &L0 = M->lev[0];
  cudaStream_t s = M->stream;
  M3_CUDA(cudaMemcpyAsync(W->tmp, z, sizeof(double) * L0.ndof, cudaMemcpyHostToDevice, s));
  M3_TRY(div_apply(L0, M->fin.G64, W->tmp, W->pt, s));
  M3_CUDA(cudaMemcpyAsync(out, W->pt, sizeof(double) * L0.nvnod, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

extern "C" int m3sph_force_vector(m3sph_mesh *M, double *Fb) {
  M3_TRY(need_op(M));
  M3_CUDA(cudaMemcpyAsync(Fb, M->fin.Fb, sizeof(double) * M->lev[0].ndof, cudaMemcpyDeviceToHost, M->stream));
  M3_CUDA(cudaStreamSynchronize(M->stream));
  return M3SPH_OK;
}

extern "C" int m3sph_element_matrices(m3sph_mesh *M, double *K, double *G, double *Mm) {
  M3_TRY(need_op(M));
  Level &L0 = M->lev[0];
  const int nel = L0.nel;
  std::vector<double> hk((size_t)kpad<double>() * nel), hg(120 * (size_t)nel), hm(10 * (size_t)nel);
  std::vector<int> perm(nel);
  M3_CUDA(cudaMemcpy(hk.data(), L0.K64, sizeof(double) * hk.size(), cudaMemcpyDeviceToHost));
  M3_CUDA(cudaMemcpy(hg.data(), M->fin.G64, sizeof(double) * hg.size(), cudaMemcpyDeviceToHost));
  M3_CUDA(cudaMemcpy(hm.data(), M->fin.M64, sizeof(double) * hm.size(), cudaMemcpyDeviceToHost));
  M3_CUDA(cudaMemcpy(perm.data(), L0.perm, sizeof(int) * nel, cudaMemcpyDeviceToHost));
  for (int p = 0; p < nel; ++p) {
    const int e = perm[p];
    if (K)
      for (int c = 0; c < 30; ++c)
        for (int r = c; r < 30; ++r) {
          const double v = hk[kidx<double>(pack_idx(r, c), p, nel)];
          K[(size_t)e * 900 + r * 30 + c] = v;
          K[(size_t)e * 900 + c * 30 + r] = v;
        }
    if (G)
      for (int pp = 0; pp < 4; ++pp)
        for (int q = 0; q < 30; ++q) G[(size_t)e * 120 + q * 4 + pp] = hg[(size_t)(pp * 30 + q) * nel + p];
    if (Mm) {
      int k = 0;
      for (int c = 0; c < 4; ++c)
        for (int r = c; r < 4; ++r) {
          const double v = hm[(size_t)k * nel + p];
          ++k;
          Mm[(size_t)e * 16 + r * 4 + c] = v;
          Mm[(size_t)e * 16 + c * 4 + r] = v;
        }
    }
  }
  return M3SPH_OK;
}

extern "C" int m3sph_level_apply(m3sph_mesh *M, int32_t img, const double *x, double *y) {
  M3_TRY(need_op(M));
  if (img < 0 || img >= M->nmg) {
    set_error("level out of range");
    return M3SPH_ERR_BAD_INPUT;
  }
  Work *W = get_work(M);
  Level &L = M->lev[img];
  cudaStream_t s = M->stream;
  const size_t n = L.ndof;
  if (img == 0 || M->precision == 0) {
    M3_CUDA(cudaMemcpyAsync(W->r64[img], x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    M3_TRY(level_op<double>(L, img, W->r64[img], W->kd64[img], s));
    M3_CUDA(cudaMemcpyAsync(y, W->kd64[img], sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  } else {
    M3_CUDA(cudaMemcpyAsync(W->r64[img], x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    M3_TRY(d2f(W->r64[img], W->r32[img], n, s));
    M3_TRY(level_op<float>(L, img, W->r32[img], W->kd32[img], s));
    M3_TRY(f2d(W->kd32[img], W->kd64[img], n, s));
    M3_CUDA(cudaMemcpyAsync(y, W->kd64[img], sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  }
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

extern "C" int m3sph_level_apply32(m3sph_mesh *M, int32_t img, const float *x, float *y) {
  M3_TRY(need_op(M));
  if (img < 0 || img >= M->nmg) {
    set_error("level out of range");
    return M3SPH_ERR_BAD_INPUT;
  }
  Level &L = M->lev[img];
  if (!L.K32 && !L.B32) {
    set_error("no FP32 operator on this level (set up with precision 1)");
    return M3SPH_ERR_BAD_INPUT;
  }
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  const size_t n = L.ndof;
  M3_CUDA(cudaMemcpyAsync(W->r32[img], x, sizeof(float) * n, cudaMemcpyHostToDevice, s));
  M3_TRY(level_op<float>(L, img, W->r32[img], W->kd32[img], s));
  M3_CUDA(cudaMemcpyAsync(y, W->kd32[img], sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  M3_TRY(stream_check(L, s));
  return M3SPH_OK;
}

extern "C" int m3sph_ml_sweep32(m3sph_mesh *M, int32_t img, const float *r, const float *kd, float *d) {
  M3_TRY(need_op(M));
  if (!M->ml || img < 0 || img >= std::min(2, M->nmg)) {
    set_error("m3sph_ml_sweep32: no learned smoother on this level");
    return M3SPH_ERR_BAD_INPUT;
  }
  Level &L = M->lev[img];
  if (!L.Dinv32) {
    set_error("no FP32 operator on this level (set up with precision 1)");
    return M3SPH_ERR_BAD_INPUT;
  }
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  const size_t n = L.ndof;
  M3_CUDA(cudaMemcpyAsync(W->r32[img], r, sizeof(float) * n, cudaMemcpyHostToDevice, s));
  if (kd) M3_CUDA(cudaMemcpyAsync(W->kd32[img], kd, sizeof(float) * n, cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(W->d32[img], d, sizeof(float) * n, cudaMemcpyHostToDevice, s));
  M3_TRY(ml_sweep<float>(M, img, W->r32[img], kd ? W->kd32[img] : nullptr, L.Dinv32, W->t32[img], W->d32[img]));
  M3_CUDA(cudaMemcpyAsync(d, W->d32[img], sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  return ml_check(M);
}

extern "C" int m3sph_level_inverse_diag32(m3sph_mesh *M, int32_t img, float *dinv) {
  M3_TRY(need_op(M));
  if (img < 0 || img >= M->nmg || !dinv || !M->lev[img].Dinv32) {
    set_error("m3sph_level_inverse_diag32: level out of range or no FP32 operator (set up with precision 1)");
    return M3SPH_ERR_BAD_INPUT;
  }
  const Level &L = M->lev[img];
  M3_CUDA(cudaMemcpyAsync(dinv, L.Dinv32, sizeof(float) * L.ndof, cudaMemcpyDeviceToHost, M->stream));
  M3_CUDA(cudaStreamSynchronize(M->stream));
  return M3SPH_OK;
}

extern "C" int m3sph_ml_features(m3sph_mesh *M, int32_t img, const float *z, float *X, float *s_norm) {
  M3_TRY(need_op(M));
  if (!M->ml || img < 0 || img >= std::min(2, M->nmg) || !z || !X || !s_norm) {
    set_error("m3sph_ml_features: no learned smoother on this level or bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  Level &L = M->lev[img];
  cudaStream_t s = M->stream;
  float *dz = nullptr, *dX = nullptr, *dS = nullptr;
  const size_t n = L.ndof;
  auto release = [&]() {
    if (dz) cudaFree(dz);
    if (dX) cudaFree(dX);
    if (dS) cudaFree(dS);
  };
  if (cudaMalloc((void **)&dz, sizeof(float) * n) != cudaSuccess ||
      cudaMalloc((void **)&dX, sizeof(float) * 52 * (size_t)L.nel) != cudaSuccess ||
      cudaMalloc((void **)&dS, sizeof(float) * (size_t)L.nel) != cudaSuccess) {
    release();
    return cuda_fail(cudaGetLastError(), "m3sph_ml_features allocation");
  }
  int st = M3SPH_OK;
  if (cudaMemcpyAsync(dz, z, sizeof(float) * n, cudaMemcpyHostToDevice, s) != cudaSuccess) st = M3SPH_ERR_CUDA;
  if (!st) st = ml_feature_rows(M, img, dz, dX, dS);
  if (!st && (cudaMemcpyAsync(X, dX, sizeof(float) * 52 * (size_t)L.nel, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
              cudaMemcpyAsync(s_norm, dS, sizeof(float) * (size_t)L.nel, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
              cudaStreamSynchronize(s) != cudaSuccess))
    st = cuda_fail(cudaGetLastError(), "m3sph_ml_features copy");
  release();
  return st;
}

extern "C" int m3sph_transfer_matrix(const m3sph_mesh *M, int32_t img, int64_t *nnz, int32_t *rows, int32_t *cols,
                                     double *vals) {
  if (!M || !nnz || img < 0 || img + 1 >= M->nmg) {
    set_error("m3sph_transfer_matrix: bad arguments or level out of range");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  const Level &F = M->lev[img];
  std::vector<int> ptr(F.nnod + 1);
  M3_CUDA(cudaMemcpy(ptr.data(), F.P_ptr, sizeof(int) * ptr.size(), cudaMemcpyDeviceToHost));
  const int64_t n = ptr[F.nnod];
  if (!rows || !cols || !vals) {   // first call: the number of entries
    *nnz = n;
    return M3SPH_OK;
  }
  if (*nnz < n) {
    set_error("m3sph_transfer_matrix: arrays hold fewer entries than the matrix has");
    return M3SPH_ERR_BAD_INPUT;
  }
  std::vector<int> col(n);
  std::vector<float> w(n);
  M3_CUDA(cudaMemcpy(col.data(), F.P_col, sizeof(int) * n, cudaMemcpyDeviceToHost));
  M3_CUDA(cudaMemcpy(w.data(), F.P_w, sizeof(float) * n, cudaMemcpyDeviceToHost));
  for (int i = 0; i < F.nnod; ++i)
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      rows[k] = i + 1;
      cols[k] = col[k] + 1;
      vals[k] = (double)w[k];   // multiples of 1/8: exact in FP32
    }
  *nnz = n;
  return M3SPH_OK;
}

extern "C" int m3sph_prolong(m3sph_mesh *M, int32_t img, const double *xc, double *xf) {
  M3_TRY(need_op(M));
  if (img < 0 || img + 1 >= M->nmg) {
    set_error("level out of range");
    return M3SPH_ERR_BAD_INPUT;
  }
  Work *W = get_work(M);
  Level &F = M->lev[img], &C = M->lev[img + 1];
  cudaStream_t s = M->stream;
  M3_CUDA(cudaMemcpyAsync(W->r64[img + 1], xc, sizeof(double) * C.ndof, cudaMemcpyHostToDevice, s));
  M3_TRY(prolong<double>(F, C, W->r64[img + 1], nullptr, W->d64[img], s));
  M3_CUDA(cudaMemcpyAsync(xf, W->d64[img], sizeof(double) * F.ndof, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

extern "C" int m3sph_restrict(m3sph_mesh *M, int32_t img, const double *rf, double *rc) {
  M3_TRY(need_op(M));
  if (img < 0 || img + 1 >= M->nmg) {
    set_error("level out of range");
    return M3SPH_ERR_BAD_INPUT;
  }
  Work *W = get_work(M);
  Level &F = M->lev[img], &C = M->lev[img + 1];
  cudaStream_t s = M->stream;
  M3_CUDA(cudaMemcpyAsync(W->r64[img], rf, sizeof(double) * F.ndof, cudaMemcpyHostToDevice, s));
  M3_TRY(restrict_<double>(F, C, W->r64[img], nullptr, W->d64[img + 1], s));
  M3_CUDA(cudaMemcpyAsync(rc, W->d64[img + 1], sizeof(double) * C.ndof, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

extern "C" int m3sph_vcycle(m3sph_mesh *M, const double *r, double *d) {
  M3_TRY(need_op(M));
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  const size_t n = M->lev[0].ndof;
  M3_CUDA(cudaMemcpyAsync(W->tmp, r, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  M3_TRY(vcycle(M, W->tmp, W->d));
  M3_CUDA(cudaMemcpyAsync(d, W->d, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

extern "C" int m3sph_mgpcg(m3sph_mesh *M, const double *b, double *x, double tol, int32_t is_abs_tol, int32_t itmax,
                           int32_t *itCG, double *rrms_final) {
  M3_TRY(need_op(M));
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  Level &L0 = M->lev[0];
  const size_t n = L0.ndof;
  M3_CUDA(cudaMemcpyAsync(W->Rhs, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  M3_TRY(apply_mask(W->Rhs, L0.freemask, n, s));
  M3_CUDA(cudaMemcpyAsync(W->U, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CGStats cs;
  M3_TRY(mgpcg(M, W->Rhs, W->U, tol, is_abs_tol != 0, itmax, cs));
  M3_CUDA(cudaMemcpyAsync(x, W->U, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  if (itCG) *itCG = cs.it;
  if (rrms_final) *rrms_final = cs.rrms;
  return M3SPH_OK;
}

extern "C" int m3sph_launch_count(unsigned long long *count) {
  if (!count) {
    set_error("bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  *count = g_launches.load();
  return M3SPH_OK;
}

extern "C" int m3sph_apply_timing(m3sph_mesh *M, int32_t img, int32_t precision, int32_t nrep, double *ms_per_apply) {
  M3_TRY(need_op(M));
  if (img < 0 || img >= M->nmg || nrep < 1 || !ms_per_apply) {
    set_error("bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  Level &L = M->lev[img];
  Work *W = get_work(M);
  cudaStream_t s = M->stream;
  const bool f32 = precision == 1;
  if ((f32 && !L.K32 && !L.B32) || (!f32 && !L.K64 && !L.B64)) {
    set_error("no element matrices of that precision on this level");
    return M3SPH_ERR_BAD_INPUT;
  }
  cudaEvent_t e0, e1;
  M3_CUDA(cudaEventCreate(&e0));
  M3_CUDA(cudaEventCreate(&e1));
  // precision 0: FP64 operator, 1: FP32 operator, 2: double-float outer operator (finest level)
  auto run = [&]() -> int {
    if (precision == 2 && img == 0) {
      const bool old = M->df_outer;
      const int oldp = M->precision;
      M->df_outer = true;
      M->precision = 1;
      const int st = outer_apply(M, W->r64[0], W->kd64[0]);
      M->df_outer = old;
      M->precision = oldp;
      return st;
    }
    if (f32) return level_op<float>(L, img, W->r32[img], W->kd32[img], s);
    return level_op<double>(L, img, W->r64[img], W->kd64[img], s);
  };
  M3_TRY(run());
  M3_CUDA(cudaEventRecord(e0, s));
  for (int i = 0; i < nrep; ++i) M3_TRY(run());
  M3_CUDA(cudaEventRecord(e1, s));
  M3_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  M3_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  *ms_per_apply = ms / nrep;
  M3_TRY(stream_check(L, s));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return M3SPH_OK;
}

extern "C" int m3sph_set_option(m3sph_mesh *M, const char *name, int32_t value) {
  if (!M || !name) {
    set_error("bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  const std::string n(name);
  if (n == "stream_apply") {
    g_stream_apply = value != 0;
  } else if (n == "fp32_operator") {
    if (value < 0 || value > 1) {
      set_error("fp32_operator must be 0 (stored element matrices) or 1 (partially assembled)");
      return M3SPH_ERR_BAD_INPUT;
    }
    g_pa_apply = value == 1;
  } else if (n == "ml_schedule") {
    if (value < 0 || value > 3) {
      set_error("ml_schedule must be 0..3");
      return M3SPH_ERR_BAD_INPUT;
    }
    M->ml_schedule = value;
  } else if (n == "ml_omega_pct") {
    if (value < 10 || value > 300) {
      set_error("ml_omega_pct must be in 10..300");
      return M3SPH_ERR_BAD_INPUT;
    }
    M->ml_omega = value / 100.0f;
  } else if (n == "ml_infer") {
    M3_TRY(ml_set_infer(value));
  } else if (n == "stream_f32_variant") {
    M3_TRY(stream_set_f32_variant(value));
  } else if (n == "stream_outer") {
    g_stream_outer = value != 0;
  } else if (n == "stream_outer_variant") {
    M3_TRY(stream_set_outer_warps(value));
  } else if (n == "split_apply") {
    M->split_apply = value != 0;
    g_split_apply = value != 0;
  } else if (n == "graphs") {
    M->use_graphs = value != 0;
  } else if (n == "df_outer") {
    M->df_outer = value != 0;
  } else if (n == "coarse_f64_direct_max") {
    if (value < 0) {
      set_error("coarse_f64_direct_max must be >= 0");
      return M3SPH_ERR_BAD_INPUT;
    }
    g_coarse_f64_direct_max = value;
  } else if (n == "coarse_refine_sweeps") {
    if (value < 0 || value > 20) {
      set_error("coarse_refine_sweeps must be in 0..20");
      return M3SPH_ERR_BAD_INPUT;
    }
    g_coarse_refine_sweeps = value;
  } else {
    set_error("unknown option " + n);
    return M3SPH_ERR_BAD_INPUT;
  }
  clear_graphs(M);
  return M3SPH_OK;
}

// ======================================================================================
// learned smoother: data collection, training, weights
// ======================================================================================
__global__ void k_rand_rhs(double *b, const uint8_t *mask, size_t n, unsigned long long seed) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
  b[i] = mask[i] ? 2.0 * u - 1.0 : 0.0;
}
__global__ void k_diff(const double *a, const double *b, double *out, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}

extern "C" int m3sph_ml_reserve(m3sph_mesh *M, int64_t capacity) {
  M3_TRY(need_op(M));
  return ml_reserve(M, capacity);
}

extern "C" int m3sph_ml_collect(m3sph_mesh *M, uint64_t seed, int32_t n_iterates, int32_t stride, int64_t *count) {
  M3_TRY(need_op(M));
  if (n_iterates < 1 || stride < 1) {
    set_error("m3sph_ml_collect: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  Work *W = get_work(M);
  Level &L0 = M->lev[0];
  cudaStream_t s = M->stream;
  const size_t n = L0.ndof;
  const bool act = M->smoother_active;
  M->smoother_active = false;
  // pairs (r = K e, e) for white-noise errors e on the free dofs: the energy of such an error is spread
  // over all modes, so most of it is determined by the local residual -- the network learns a local
  // approximate inverse of the operator, which is what a smoother applies
  for (int k = 0; k < n_iterates; ++k) {
    k_rand_rhs<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(W->tmp, L0.freemask, n, seed * 1000003ull + k);
    count_launch();
    M3_TRY(outer_apply(M, W->tmp, W->r));
    M3_TRY(apply_mask(W->r, L0.freemask, n, s));
    M3_TRY(ml_add_samples(M, W->r, W->tmp, stride, (int)((seed + k) % (uint64_t)stride)));
  }
  M3_CUDA(cudaStreamSynchronize(s));
  M->smoother_active = act;
  if (count) *count = ml_count(M);
  return M3SPH_OK;
}

extern "C" int m3sph_ml_add_pairs(m3sph_mesh *M, const double *r, const double *e, int32_t stride, int32_t offset,
                                  int64_t *count) {
  M3_TRY(need_op(M));
  if (!r || !e || stride < 1 || offset < 0) {
    set_error("m3sph_ml_add_pairs: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  Work *W = get_work(M);
  Level &L0 = M->lev[0];
  cudaStream_t s = M->stream;
  const size_t n = L0.ndof;
  M3_CUDA(cudaMemcpyAsync(W->r, r, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(W->tmp, e, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  M3_TRY(apply_mask(W->r, L0.freemask, n, s));
  M3_TRY(apply_mask(W->tmp, L0.freemask, n, s));
  M3_TRY(ml_add_samples(M, W->r, W->tmp, stride, offset % stride));
  M3_CUDA(cudaStreamSynchronize(s));
  if (count) *count = ml_count(M);
  return M3SPH_OK;
}

extern "C" int m3sph_ml_train_epoch(m3sph_mesh *M, int32_t batch, float lr, uint64_t seed, double *mse) {
  M3_TRY(need_op(M));
  if (batch < 64 || batch % 64) {
    set_error("m3sph_ml_train_epoch: batch must be a positive multiple of 64");
    return M3SPH_ERR_BAD_INPUT;
  }
  double m = 0.0;
  M3_TRY(ml_epoch(M, batch, lr, seed, &m));
  clear_graphs(M);
  if (mse) *mse = m;
  return M3SPH_OK;
}

extern "C" int m3sph_ml_nparam(int32_t *n) {
  if (!n) return M3SPH_ERR_BAD_INPUT;
  *n = ml_nparam();
  return M3SPH_OK;
}

extern "C" int m3sph_ml_set_params(m3sph_mesh *M, const float *params, int32_t trained) {
  if (!M || !params) {
    set_error("bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  M3_TRY(ml_set_params(M, params));
  ml_mark_trained(M, trained != 0);
  clear_graphs(M);
  return M3SPH_OK;
}

extern "C" int m3sph_ml_get_params(m3sph_mesh *M, float *params) {
  if (!M || !params) {
    set_error("bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  return ml_get_params(M, params);
}

extern "C" int m3sph_ml_gradients(m3sph_mesh *M, const float *X, const float *T, int32_t n, float *grad, double *loss) {
  if (!M || !X || !T || !grad || n < 1) {
    set_error("bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  return ml_gradients(M, X, T, n, grad, loss);
}

extern "C" int m3sph_ml_forward(m3sph_mesh *M, const float *X, int32_t n, float *Y) {
  if (!M || !X || !Y || n < 1) {
    set_error("bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  return ml_forward(M, X, n, Y);
}
