// Shared device/host declarations of the m3sph CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "../../include/m3sph.h"

struct m3sph_mesh;

namespace m3sph {

constexpr int NNODEL = 10;        // P2 velocity nodes per element
constexpr int NUDOF = 30;         // velocity dofs per element
constexpr int NPACK = 465;        // packed lower triangle of a 30x30 symmetric matrix
constexpr int NIP = 14;           // quadrature points (ip_tetrahedron.m:100-123)
constexpr int MAX_COLORS = 128;

// packed lower-triangle index of (r, c), r >= c, column-major (MUTILS sparse_create layout)
__host__ __device__ constexpr int pack_idx(int r, int c) { return c * (2 * NUDOF - c + 1) / 2 + (r - c); }

// Element matrices are stored as vectorised SoA: packed entry k of element e of a level with nel
// elements lives at ((k / V) * nel + e) * V + k % V with V = 4 (float) or 2 (double), so one
// thread loads 16 bytes at a time and a warp's loads stay contiguous (512 B per load).
template <typename T> struct KVec;
template <> struct KVec<float> { static constexpr int V = 4; };
template <> struct KVec<double> { static constexpr int V = 2; };
template <typename T>
__host__ __device__ __forceinline__ size_t kidx(int k, size_t e, size_t nel) {
  constexpr int V = KVec<T>::V;
  return ((size_t)(k / V) * nel + e) * V + (k % V);
}
// packed entry k -> (row r, column c) of the lower triangle, column-major (k = 0: (0,0), 1: (1,0), ...)
__host__ __device__ constexpr int unpack_c(int k) {
  int c = 0;
  while (k >= 30 - c) { k -= 30 - c; ++c; }
  return c;
}
__host__ __device__ constexpr int unpack_r(int k) {
  int c = 0;
  while (k >= 30 - c) { k -= 30 - c; ++c; }
  return c + k;
}
// y_hi + y_lo += (v_hi + v_lo)(x_hi + x_lo) in double-float: the product's rounding error by FMA,
// the sum's by Knuth's two-sum (used by the FP64-accurate outer operator built from FP32 parts)
__device__ __forceinline__ void df_mac(float vh, float vl, float xh, float xl, float &sh, float &sl) {
  const float p = vh * xh;
  float e = fmaf(vh, xh, -p);
  e = fmaf(vh, xl, e);
  e = fmaf(vl, xh, e);
  const float s = sh + p;
  const float bb = s - sh;
  const float err = (sh - (s - bb)) + (p - bb);
  sh = s;
  sl += err + e;
}

template <typename T> constexpr int kpad() { return ((NPACK + KVec<T>::V - 1) / KVec<T>::V) * KVec<T>::V; }

void set_error(const std::string &msg);
// host-side count of kernel launches issued by this library (reported by m3sph_launch_count)
void count_launch();
int cuda_fail(cudaError_t e, const char *what);

#define M3_TRY(call)                 \
  do {                               \
    int _s = (call);                 \
    if (_s != M3SPH_OK) return _s;   \
  } while (0)

#define M3_CUDA(call)                                  \
  do {                                                 \
    cudaError_t _e = (call);                           \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)

// quadrature / shape-function tables (computed on the host, copied to constant memory)
struct ShapeTables {
  double ipw[NIP];
  double NP[NIP][4];
  double NU[NIP][10];
  double dNU[NIP][10][3];
  double N20[NIP][20];
  double dN20[NIP][20][3];
};
void build_shape_tables(ShapeTables &t);
int upload_shape_tables();

// device buffers of one multigrid level
struct Level {
  int nel = 0, nnod = 0, nvnod = 0, ndof = 0;
  int nfree = 0;
  std::vector<int> cstart;            // colour ranges in stored element order (host)
  int *el2nod = nullptr;              // [10][nel], 0-based, stored (colour) order
  int *perm = nullptr;                // stored -> original element id
  int *invperm = nullptr;             // original -> stored
  uint8_t *freemask = nullptr;        // [ndof], 1 = free dof
  double *K64 = nullptr;              // [465][nel] rotated, masked element matrices
  float *K32 = nullptr;
  float *KL32 = nullptr;              // K64 - K32 rounded to FP32 (finest level, mixed precision)
  double *Dinv64 = nullptr;           // [ndof] inverse diagonal (0 on fixed dofs)
  float *Dinv32 = nullptr;
  // children (coarse levels): fine stored index of child k, and parent-local vertex indices
  int *child = nullptr;               // [8][nel]
  uint32_t *child_vloc = nullptr;     // [8][nel], 4 x 4-bit parent-local node index (0..9)
  // transfer to the next coarser level (levels 0..nmg-2)
  int *P_ptr = nullptr, *P_col = nullptr;   // fine node rows
  float *P_w = nullptr;
  int *R_ptr = nullptr, *R_col = nullptr;   // coarse node rows (transpose)
  float *R_w = nullptr;
  // assembled 3x3-block CSR of the level operator (coarse levels): one launch per application
  int nnzb = 0;
  int *bsr_ptr = nullptr, *bsr_col = nullptr;   // [nnod+1], [nnzb]
  int *bsr_cptr = nullptr, *bsr_contrib = nullptr;   // per block: contributions e*100 + a*10 + b
  double *B64 = nullptr;                         // [nnzb][9]
  float *B32 = nullptr;
  // streamed apply (finest level): phase 1 streams the element matrices in chunks of 32 stored
  // elements and writes element outputs Ye; phase 2 sums them per node in a fixed order
  int nchunk = 0, sa_grid = 0;
  int *chunk_conn = nullptr;          // [nchunk][10][32] node ids of the chunk's elements (0: unused lane)
  float *ye32 = nullptr;              // [nel][30] element outputs
  int nchunk8 = 0;                    // FP64-accurate operators: chunks of 8 elements
  int *chunk_conn8 = nullptr;         // [nchunk8][10][8]
  double *ye64 = nullptr;             // [nel][30]
  int *g_ptr = nullptr;               // [nnod + 1] node -> incident (element, local node) entries
  int *g_idx = nullptr;               // [10 nel] offsets e * 30 + 3 * local node into Ye, element order
  int *sa_err = nullptr;              // bounded waits of the streamed apply that gave up (bit mask)
  // partially assembled FP32 operator (finest level): per integration point the 3x3 factor
  // sqrt(w eta) d xi / d x, [NIP][9][nel]; per element the free-dof bits; per node RR's angles
  float *pa32 = nullptr;
  int pa_ld = 0;                      // row stride of pa32 (floats, multiple of 4)
  uint32_t *pa_emask = nullptr;       // [nel] bit 3 n + c set when dof c of local node n is free
  float4 *pa_trig = nullptr;          // [nnod] (cos theta, sin theta, cos phi, sin phi)
  bool pa_ready = false;              // pa32 / pa_emask written by the last operator set-up
  // host copies needed at set-up
  std::vector<int> h_el2nod_orig;     // [nel][10] original order, 0-based
};

struct Finest {
  double *gcoord = nullptr;           // [3][nnod]
  double *gcoord_sph = nullptr;       // [3][nnod]
  double *RR = nullptr;               // [9][nnod] (theta,phi,r)->(x,y,z), row-major 3x3
  uint8_t *cls = nullptr;             // [nel] stored order
  int *iso_slot = nullptr;            // [nel] stored order, -1 if not iso
  double *cubic = nullptr;            // [60][niso] (theta,phi,r) x 20 nodes, X-90 frame
  int niso = 0;
  double *visc = nullptr, *dens = nullptr;  // [nvnod]
  double *G64 = nullptr;              // [120][nel]: G[p][3n+c]
  double *M64 = nullptr;              // [10][nel] packed lower 4x4
  double *Fbe = nullptr;              // [30][nel]
  double *BCe = nullptr;              // [30][nel] K_unmasked * Ufix per element
  double *Fb = nullptr;               // [ndof] assembled, rotated
  double *LiMM = nullptr;             // [nvnod] inverse lumped M
  int *err = nullptr;                 // device error flags
};

struct Coarse {
  int n = 0;                          // dofs of the coarsest level
  int nf = 0;                         // its free dofs: the dense inverse is nf x nf
  int *fidx = nullptr;                // [nf] compact -> level dof
  int *cmap = nullptr;                // [n] level dof -> compact index, -1 for a fixed dof
  double *A64 = nullptr;              // dense inverse (n x n)
  float *A32 = nullptr;
  bool refine64 = false;              // FP64 path: FP32 inverse + iterative refinement against B64
  float *B32tmp = nullptr;            // [9][nnzb] FP32 copy of the coarsest FP64 blocks (refinement)
  double *t64 = nullptr;              // [n] refinement residual
};

struct SetupArgs {
  int nel, nnod;
  const int *el2nod;        // [10][nel] stored order
  const uint8_t *cls;
  const int *iso_slot;
  const double *cubic;      // [60][niso]
  int niso;
  const double *gcoord, *gcoord_sph, *RR;
  const double *visc, *dens;
  const uint8_t *freemask;
  double g, Bscale, Dens0, minVisc, maxVisc;
  double *K64; float *K32; double *G64; double *M64; double *Fbe;
  float *KL32;              // low FP32 part of K64 - K32 (double-float outer operator) or nullptr
  float *PA32;              // [NIP * 9][pa_ld] partially assembled factors or nullptr
  int pa_ld;
  uint32_t *emask;          // [nel] free-dof bits or nullptr
  const double *ufix;       // [3*nnod] prescribed values (rotated frame) or nullptr
  double *BCe;              // [30][nel] element K_unmasked * ufix (when ufix != nullptr)
  int *err;
};

int slm_build(m3sph_mesh *M, const m3sph_level &f0);
int slm_advect_resident(m3sph_mesh *M, const double *U_soa, double *T, double dt, const m3sph_slm_opts *o,
                        bool first_step, m3sph_locate_info *info);
int stokes_velocity_soa(m3sph_mesh *M, double *dst);
int stokes_resident_solve(m3sph_mesh *M, const m3sph_opts *opts, bool zero_p, m3sph_info &inf);
int stokes_calc_dt(m3sph_mesh *M, double dt_adv_limit, double dtmax, double *dt, double *dt_adv);
int diffusion_resident(m3sph_mesh *M, double *T, double dt, int *nit);
int stokes_set_pressure(m3sph_mesh *M, const double *P);
int ml_build(m3sph_mesh *M);
int ml_features(m3sph_mesh *M, const double *h_visc);
template <typename T> int ml_sweep(m3sph_mesh *M, int j, const T *r0, const T *kd, const T *Dinv, T *tmp, T *d);
int ml_init_kernels();
int ml_set_infer(int v);
int ml_check(m3sph_mesh *M);
bool ml_ready(m3sph_mesh *M);
int ml_add_samples(m3sph_mesh *M, const double *r, const double *err, int stride, int offset);
int ml_reserve(m3sph_mesh *M, long cap);
int ml_set_params(m3sph_mesh *M, const float *h);
int ml_get_params(m3sph_mesh *M, float *h);
int ml_epoch(m3sph_mesh *M, int batch, float lr, unsigned long long seed, double *mse);
int ml_gradients(m3sph_mesh *M, const float *hX, const float *hT, int n, float *hgrad, double *loss);
int ml_forward(m3sph_mesh *M, const float *hX, int n, float *hY);
int ml_nparam();
long ml_count(m3sph_mesh *M);
void ml_mark_trained(m3sph_mesh *M, bool t);

}  // namespace m3sph

struct m3sph_mesh {
  int device = 0;
  int nmg = 0;
  cudaStream_t stream = nullptr;
  std::vector<m3sph::Level> lev;
  m3sph::Finest fin;
  m3sph::Coarse coarse;
  int precision = 0;                  // 0 fp64, 1 fp32 V-cycle
  m3sph_physics phys{};
  double last_setup_ms = 0.0;
  bool have_operator = false;
  std::vector<int> h_ifix;            // 0-based fixed dofs (rotated frame)
  std::vector<double> h_vfix;
  double *Ufix = nullptr;             // [ndof0] prescribed values (rotated frame)
  double *bc_rhs = nullptr;           // K1_full * Ufix
  bool has_nonzero_fix = false;
  bool bc_stale = false;              // prescribed values changed since the last operator rebuild
  // scratch
  std::vector<void *> work;           // device buffers owned by the workspace
  void *wk = nullptr;                 // host-side workspace descriptor
  void (*wk_free)(void *) = nullptr;
  std::vector<std::pair<double *, cudaGraphExec_t>> graphs;   // captured MG-PCG iterations
  bool use_graphs = true;
  bool df_outer = true;               // double-float outer operator on the mixed path
  bool split_apply = true;            // 4-warp split element-by-element kernels on the finest level
  int ml_schedule = 1;                // learned smoothing per side: 0 learned-Jacobi-learned, 1 one learned sweep
  float ml_omega = 1.0f;              // relaxation weight of the learned correction
  unsigned long long graph_kernels = 0;   // kernel launches per captured iteration
  void *ml = nullptr;                 // learned smoother state
  void (*ml_free)(void *) = nullptr;
  int smoother = 0;                   // 0 Jacobi, 1 learned smoother on the two finest levels
  bool smoother_active = false;       // learned smoother in use for the current solve
  int smoother_fallbacks = 0;
  double r_min = 0.0, r_max = 0.0;    // shell radii (features)
  double Lx = 0.0, Ly = 0.0, Lz = 0.0; // extents of the finest mesh (MESH.Lx/Ly/Lz, init_mesh_curved_p.m:264-272)
  double rad_max = 0.0;               // largest node radius sqrt(x^2+y^2+z^2) (rock_prop.m:10-11)
  double *T = nullptr;                // [nnod] resident temperature of the time step
  double *Usoa = nullptr;             // [3][nnod] Cartesian velocity handed to the advection
  long long ts_steps = 0;             // time steps taken since the temperature was set
  double ts_time = 0.0;               // model time accumulated by the time steps
  void *diff = nullptr;               // thermal-diffusion state
  void (*diff_free)(void *) = nullptr;
  void *slm = nullptr;                // advection / point-location state
  void (*slm_free)(void *) = nullptr;
  double *red = nullptr;              // reduction partials
  double *scal = nullptr;             // device scalars
  double *h_scal = nullptr;           // pinned host mirror
};
