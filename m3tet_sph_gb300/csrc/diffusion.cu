// Thermal diffusion half step (diffusion3d_p.m with the reference's default options): linear
// elements on the 8-child split of every P2 tetrahedron, double-Jacobian element integrals,
// lumped capacity, theta scheme, Dirichlet temperatures, Jacobi-preconditioned Polak-Ribiere CG.
//
// Layout: split elements `sub` [4][nsub] (node ids), packed conductivity C [10][nsub] (entries
// (i,j), i >= j, in the order 00 10 11 20 21 22 30 31 32 33), element products ye [4][nsub], and a
// node -> (local, element) list in element order for the fixed-order node sums (no atomics). One
// operator application reads 80 B of C, 16 B of ids and 32 B of gathered T per element and writes /
// re-reads 32 B of ye: HBM-bound.
#include <cmath>
#include <string>
#include <vector>

#include "common.cuh"

namespace m3sph {

int dot(const double *a, const double *b, size_t n, double *partials, double *out, cudaStream_t s);

// children of a P2 tetrahedron (local node numbers 0..9) for the three interior diagonals, and the
// diagonals' end nodes (tetmesh_p2_to_p1.m): the table that the reference's split follows
static const int EL2CHILD[3][8][4] = {
    {{0, 4, 8, 7}, {4, 1, 5, 9}, {8, 5, 2, 6}, {7, 9, 6, 3}, {9, 7, 6, 4}, {5, 8, 4, 6}, {7, 6, 4, 8}, {9, 4, 6, 5}},
    {{0, 4, 8, 7}, {4, 1, 5, 9}, {8, 5, 2, 6}, {7, 9, 6, 3}, {4, 8, 7, 5}, {9, 6, 5, 7}, {8, 7, 5, 6}, {4, 5, 7, 9}},
    {{0, 4, 8, 7}, {4, 1, 5, 9}, {8, 5, 2, 6}, {7, 9, 6, 3}, {7, 4, 8, 9}, {6, 5, 9, 8}, {4, 8, 9, 5}, {8, 9, 6, 7}}};
static const int DIAG2NOD[3][2] = {{4, 6}, {5, 7}, {8, 9}};

struct DiffState {
  int nsub = 0, nnod = 0, nfix = 0;
  double kappa = 0.0, theta = 1.0, tol = 1e-8;
  int itmax = 500;
  int *sub = nullptr;                  // [4][nsub]
  uint8_t *cls = nullptr;              // [nsub]
  double *C = nullptr;                 // [10][nsub]
  double *ye = nullptr;                // [4][nsub]
  int *gptr = nullptr, *gidx = nullptr;  // [nnod+1], [4 nsub]: local * nsub + element
  double *ML = nullptr, *Cdiag = nullptr;  // [nnod]
  uint8_t *fixmask = nullptr;          // [nnod]
  int *ifix = nullptr;                 // [nfix]
  double *vfix = nullptr;              // [nfix]
  double *rhs = nullptr, *x = nullptr, *r = nullptr, *d = nullptr, *q = nullptr, *Aq = nullptr, *rl = nullptr;
  int *err = nullptr;
};

static DiffState *diff_state(m3sph_mesh *M) { return reinterpret_cast<DiffState *>(M->diff); }

static void diff_free(void *p) {
  DiffState *D = reinterpret_cast<DiffState *>(p);
  for (void *q : {(void *)D->sub, (void *)D->cls, (void *)D->C, (void *)D->ye, (void *)D->gptr, (void *)D->gidx,
                  (void *)D->ML, (void *)D->Cdiag, (void *)D->fixmask, (void *)D->ifix, (void *)D->vfix, (void *)D->rhs,
                  (void *)D->x, (void *)D->r, (void *)D->d, (void *)D->q, (void *)D->Aq, (void *)D->rl, (void *)D->err})
    if (q) cudaFree(q);
  delete D;
}

__device__ __forceinline__ void c2s_d(double x, double y, double z, double &th, double &ph, double &r) {
  r = sqrt(x * x + y * y + z * z);
  th = atan2(sqrt(x * x + y * y), z);
  ph = atan2(y, x);
  if (ph < 0.0) ph += 2.0 * M_PI;
}

// element integrals of one split element (assembly_diffusion_els_*_opt.m): vertex (theta, phi, r)
// in the element's frame, J_SL from them, J_CS at each of the 4 points of ip_tetrahedron(4)
__global__ void k_diff_setup(int nsub, const int *__restrict__ sub, const uint8_t *__restrict__ cls,
                             const double *__restrict__ X, const double *__restrict__ S, int nnod, double kappa,
                             double *__restrict__ C, double *__restrict__ Me, int *err) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nsub) return;
  const int c = cls[e];
  double V[3][4];
  for (int i = 0; i < 4; ++i) {
    const int n = sub[(size_t)i * nsub + e];
    if (c <= 1) {
      V[0][i] = S[n];
      V[1][i] = S[nnod + n];
      V[2][i] = S[2 * (size_t)nnod + n];
      if (c == 1) {
        V[1][i] += M_PI;
        if (V[1][i] > 2.0 * M_PI) V[1][i] -= 2.0 * M_PI;
      }
    } else {   // X-90-rotated frame: (x, -z, y)
      c2s_d(X[n], -X[2 * (size_t)nnod + n], X[nnod + n], V[0][i], V[1][i], V[2][i]);
    }
  }
  // J_SL[j][k] = d sph_k / d loc_j with dN4 = [I; -1 -1 -1]
  double J[3][3];
  for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 3; ++k) J[j][k] = V[k][j] - V[k][3];
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  if (det < 0.0) atomicOr(err, 1);
  const double id = 1.0 / det;
  double Li[3][3];   // inverse of J_SL: Li[k][j] = d loc_j / d sph_k
  Li[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
  Li[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
  Li[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  Li[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
  Li[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  Li[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
  Li[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
  Li[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
  Li[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  const double a = (5.0 + 3.0 * sqrt(5.0)) / 20.0, b = (5.0 - sqrt(5.0)) / 20.0;
  double Cp[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0}, Ml[4] = {0, 0, 0, 0};
  for (int ip = 0; ip < 4; ++ip) {
    const double N[4] = {ip == 0 ? a : b, ip == 1 ? a : b, ip == 2 ? a : b, ip == 3 ? a : b};
    double sp[3];
    for (int k = 0; k < 3; ++k) sp[k] = V[k][0] * N[0] + V[k][1] * N[1] + V[k][2] * N[2] + V[k][3] * N[3];
    const double th = sp[0], ph = sp[1], rr = sp[2];
    if (th == 0.0) atomicOr(err, 2);
    double st, ct, sph, cph;
    sincos(th, &st, &ct);
    sincos(ph, &sph, &cph);
    const double dCS = rr * rr * st;
    const double SC[3][3] = {{rr * st * ct * cph / dCS, -rr * sph / dCS, rr * rr * st * st * cph / dCS},
                             {rr * st * ct * sph / dCS, rr * cph / dCS, rr * rr * st * st * sph / dCS},
                             {-rr * st * st / dCS, 0.0, rr * rr * st * ct / dCS}};
    double Jd[3][3];   // Jd[x][j] = d loc_j / d cart_x
    for (int x = 0; x < 3; ++x)
      for (int j = 0; j < 3; ++j) Jd[x][j] = SC[x][0] * Li[0][j] + SC[x][1] * Li[1][j] + SC[x][2] * Li[2][j];
    double g[4][3];
    for (int x = 0; x < 3; ++x) {
      g[0][x] = Jd[x][0];
      g[1][x] = Jd[x][1];
      g[2][x] = Jd[x][2];
      g[3][x] = -Jd[x][0] - Jd[x][1] - Jd[x][2];
    }
    const double w = dCS * det * 0.25;
    int k = 0;
    for (int i = 0; i < 4; ++i) {
      for (int j = 0; j <= i; ++j, ++k) Cp[k] += kappa * w * (g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2]);
      Ml[i] += w * N[i];   // row sum of w N_i N_j (sum_j N_j = 1)
    }
  }
  for (int k = 0; k < 10; ++k) C[(size_t)k * nsub + e] = Cp[k];
  for (int i = 0; i < 4; ++i) Me[(size_t)i * nsub + e] = Ml[i];
}

__device__ __forceinline__ int pk(int i, int j) { return i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

// ye_e = C_e x_e
__global__ void k_diff_elem(int nsub, const int *__restrict__ sub, const double *__restrict__ C,
                            const double *__restrict__ x, double *__restrict__ ye) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nsub) return;
  double xe[4], c[10];
  for (int i = 0; i < 4; ++i) xe[i] = x[sub[(size_t)i * nsub + e]];
  for (int k = 0; k < 10; ++k) c[k] = C[(size_t)k * nsub + e];
  for (int i = 0; i < 4; ++i) {
    double s = 0.0;
    for (int j = 0; j < 4; ++j) s += c[pk(i, j)] * xe[j];
    ye[(size_t)i * nsub + e] = s;
  }
}

// y_n = a ML_n x_n + c sum(ye) over the node's entries in element order; fixed rows 0 if masked
__global__ void k_diff_gather(int nnod, const int *__restrict__ gptr, const int *__restrict__ gidx,
                              const double *__restrict__ ye, const double *__restrict__ ML, const double *__restrict__ x,
                              double a, double c, const uint8_t *__restrict__ fixmask, double *__restrict__ y) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnod) return;
  double s = 0.0;
  for (int k = gptr[n]; k < gptr[n + 1]; ++k) s += ye[gidx[k]];
  const double v = (a != 0.0 ? a * ML[n] * x[n] : 0.0) + c * s;
  y[n] = (fixmask && fixmask[n]) ? 0.0 : v;
}

__global__ void k_diff_jacobi(int n, const double *ML, const double *Cdiag, double c, const uint8_t *fixmask,
                              const double *r, double *d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = fixmask[i] ? 0.0 : r[i] / (ML[i] + c * Cdiag[i]);
}
__global__ void k_diff_sub(int n, const double *a, const double *b, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}
// r = rhs - Ax on the free rows, 0 on the fixed ones
__global__ void k_diff_resid(int n, const double *rhs, const double *Ax, const uint8_t *fixmask, double *r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) r[i] = fixmask[i] ? 0.0 : rhs[i] - Ax[i];
}
__global__ void k_diff_setfix(const int *ifix, const double *vfix, int nfix, double *x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nfix) x[ifix[i]] = vfix[i];
}
__global__ void k_diff_dir(int n, const double *d, double beta, double *q, int first) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) q[i] = first ? d[i] : d[i] + beta * q[i];
}
__global__ void k_diff_step(int n, double alpha, const double *q, const double *Aq, double *x, double *r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    x[i] += alpha * q[i];
    r[i] -= alpha * Aq[i];
  }
}

static int dalloc_d(void **p, size_t bytes) {
  M3_CUDA(cudaMalloc(p, bytes ? bytes : 1));
  return M3SPH_OK;
}

static int diff_build(m3sph_mesh *M, DiffState *D, double theta_cone) {
  cudaStream_t s = M->stream;
  Level &L0 = M->lev[0];
  const int nel = L0.nel, nnod = L0.nnod;
  std::vector<double> X(3 * (size_t)nnod), S(3 * (size_t)nnod);
  M3_CUDA(cudaMemcpyAsync(X.data(), M->fin.gcoord, X.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaMemcpyAsync(S.data(), M->fin.gcoord_sph, S.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  const std::vector<int> &el = L0.h_el2nod_orig;   // [nel][10]
  const size_t nsub = 8 * (size_t)nel;
  if (nsub > (size_t)(1u << 31) / 4) {
    set_error("mesh too large for the diffusion split");
    return M3SPH_ERR_BAD_INPUT;
  }
  std::vector<int> sub(4 * nsub);
  std::vector<uint8_t> cls(nsub);
  const double tc = theta_cone * M_PI / 180.0;
  for (int e = 0; e < nel; ++e) {
    const int *en = &el[(size_t)e * 10];
    // shortest interior diagonal (Cartesian), the first on ties (tetmesh_p2_to_p1.m)
    int isp = 0;
    double best = 0.0;
    for (int k = 0; k < 3; ++k) {
      const int a = en[DIAG2NOD[k][0]], b = en[DIAG2NOD[k][1]];
      double d2 = 0.0;
      for (int c = 0; c < 3; ++c) {
        const double dd = X[(size_t)c * nnod + a] - X[(size_t)c * nnod + b];
        d2 += dd * dd;
      }
      const double len = std::sqrt(d2);
      if (k == 0 || len < best) {
        best = len;
        isp = k;
      }
    }
    for (int k = 0; k < 8; ++k) {
      const size_t se = 8 * (size_t)e + k;
      int nin = 0;
      bool cross = false;
      double ph[4];
      for (int i = 0; i < 4; ++i) {
        const int n = en[EL2CHILD[isp][k][i]];
        sub[(size_t)i * nsub + se] = n;
        const double th = S[n];
        ph[i] = S[nnod + n];
        nin += (th <= tc || th >= M_PI - tc) ? 1 : 0;
      }
      const int pairs[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
      for (const auto &pp : pairs) cross |= std::fabs(ph[pp[0]] - ph[pp[1]]) > M_PI;
      // check_els_in_cone.m / check_phi.m on the split elements
      cls[se] = (uint8_t)(nin == 0 ? (cross ? 1 : 0) : (nin < 3 ? 3 : 2));
    }
  }
  // node -> (local, element) entries in element order
  std::vector<int> ptr(nnod + 1, 0), idx(4 * nsub);
  for (size_t e = 0; e < nsub; ++e)
    for (int i = 0; i < 4; ++i) ptr[sub[(size_t)i * nsub + e] + 1]++;
  for (int n = 0; n < nnod; ++n) ptr[n + 1] += ptr[n];
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (size_t e = 0; e < nsub; ++e)
    for (int i = 0; i < 4; ++i) idx[fill[sub[(size_t)i * nsub + e]]++] = (int)((size_t)i * nsub + e);
  D->nsub = (int)nsub;
  D->nnod = nnod;
  int st;
  if ((st = dalloc_d((void **)&D->sub, sub.size() * sizeof(int))) ||
      (st = dalloc_d((void **)&D->cls, cls.size())) || (st = dalloc_d((void **)&D->C, 10 * nsub * sizeof(double))) ||
      (st = dalloc_d((void **)&D->ye, 4 * nsub * sizeof(double))) ||
      (st = dalloc_d((void **)&D->gptr, ptr.size() * sizeof(int))) ||
      (st = dalloc_d((void **)&D->gidx, idx.size() * sizeof(int))) ||
      (st = dalloc_d((void **)&D->ML, nnod * sizeof(double))) || (st = dalloc_d((void **)&D->Cdiag, nnod * sizeof(double))) ||
      (st = dalloc_d((void **)&D->fixmask, nnod)) || (st = dalloc_d((void **)&D->err, sizeof(int))))
    return st;
  for (double **p : {&D->rhs, &D->x, &D->r, &D->d, &D->q, &D->Aq, &D->rl})
    if ((st = dalloc_d((void **)p, nnod * sizeof(double)))) return st;
  M3_CUDA(cudaMemcpyAsync(D->sub, sub.data(), sub.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(D->cls, cls.data(), cls.size(), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(D->gptr, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(D->gidx, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

// element integrals, lumped capacity and conductivity diagonal for the diffusivity kappa
static int diff_integrate(m3sph_mesh *M, DiffState *D) {
  cudaStream_t s = M->stream;
  const int nsub = D->nsub, nnod = D->nnod;
  M3_CUDA(cudaMemsetAsync(D->err, 0, sizeof(int), s));
  // the lumped element capacities go through ye, then the fixed-order node sums
  k_diff_setup<<<(nsub + 127) / 128, 128, 0, s>>>(nsub, D->sub, D->cls, M->fin.gcoord, M->fin.gcoord_sph, nnod, D->kappa,
                                                  D->C, D->ye, D->err); count_launch();
  k_diff_gather<<<(nnod + 255) / 256, 256, 0, s>>>(nnod, D->gptr, D->gidx, D->ye, nullptr, nullptr, 0.0, 1.0, nullptr,
                                                   D->ML); count_launch();
  M3_CUDA(cudaGetLastError());
  int herr = 0;
  M3_CUDA(cudaMemcpyAsync(&herr, D->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  if (herr & 1) {
    set_error("negative Jacobi");
    return M3SPH_ERR_NEGATIVE_JACOBIAN;
  }
  if (herr & 2) {
    set_error("integration point with theta = 0 (det(J_CS) = Inf)");
    return M3SPH_ERR_BAD_INPUT;
  }
  return M3SPH_OK;
}

__global__ void k_diff_diag_elem(int nsub, const double *__restrict__ C, double *__restrict__ ye) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nsub) return;
  const int dk[4] = {0, 2, 5, 9};
  for (int i = 0; i < 4; ++i) ye[(size_t)i * nsub + e] = C[(size_t)dk[i] * nsub + e];
}

// conductivity diagonal: per node the sum of its elements' packed diagonal entries (00 11 22 33)
static int diff_diag(m3sph_mesh *M, DiffState *D) {
  cudaStream_t s = M->stream;
  k_diff_diag_elem<<<(D->nsub + 127) / 128, 128, 0, s>>>(D->nsub, D->C, D->ye); count_launch();
  k_diff_gather<<<(D->nnod + 255) / 256, 256, 0, s>>>(D->nnod, D->gptr, D->gidx, D->ye, nullptr, nullptr, 0.0, 1.0,
                                                      nullptr, D->Cdiag); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// y = a ML x + c C x (fixed rows zeroed when masked)
static int diff_apply(m3sph_mesh *M, DiffState *D, const double *x, double a, double c, bool masked, double *y) {
  cudaStream_t s = M->stream;
  k_diff_elem<<<(D->nsub + 127) / 128, 128, 0, s>>>(D->nsub, D->sub, D->C, x, D->ye); count_launch();
  k_diff_gather<<<(D->nnod + 255) / 256, 256, 0, s>>>(D->nnod, D->gptr, D->gidx, D->ye, D->ML, x, a, c,
                                                      masked ? D->fixmask : nullptr, y); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

static int read2(m3sph_mesh *M, int idx, double &v) {
  M3_CUDA(cudaMemcpyAsync(M->h_scal + idx, M->scal + idx, sizeof(double), cudaMemcpyDeviceToHost, M->stream));
  M3_CUDA(cudaStreamSynchronize(M->stream));
  v = M->h_scal[idx];
  return M3SPH_OK;
}

// one diffusion3d_p step on the device-resident T (nnod) over dt; *nit = PCG iterations
int diffusion_resident(m3sph_mesh *M, double *T, double dt, int *nit) {
  DiffState *D = diff_state(M);
  if (!D) {
    set_error("diffusion not set up (call m3sph_diffusion_setup)");
    return M3SPH_ERR_BAD_INPUT;
  }
  cudaStream_t s = M->stream;
  const int n = D->nnod;
  const unsigned g = (unsigned)((n + 255) / 256);
  const double c = dt * D->theta;
  // rhs = M T - dt (1 - theta) C T (diffusion3d_p.m:96-97)
  M3_TRY(diff_apply(M, D, T, 1.0, -dt * (1.0 - D->theta), false, D->rhs));
  // T(ifix) = vfix; r = rhs - A T on the free rows (A(:,ifix) vfix moves to the rhs through T)
  if (D->nfix) k_diff_setfix<<<(D->nfix + 255) / 256, 256, 0, s>>>(D->ifix, D->vfix, D->nfix, T); count_launch();
  M3_TRY(diff_apply(M, D, T, 1.0, c, true, D->Aq));
  k_diff_resid<<<g, 256, 0, s>>>(n, D->rhs, D->Aq, D->fixmask, D->r); count_launch();
  M3_CUDA(cudaMemsetAsync(D->q, 0, n * sizeof(double), s));
  // pcg_solver_p.m: tol relative to normdf of the initial residual over the free rows
  const int nfree = n - D->nfix;
  const double sq = std::sqrt((double)std::max(1, nfree));
  double rr = 0.0;
  M3_TRY(dot(D->r, D->r, n, M->red, M->scal + 20, s));
  M3_TRY(read2(M, 20, rr));
  double norm_r = std::sqrt(rr) / sq;
  const double tol = D->tol * norm_r;
  int it = 0;
  double rd = 0.0;
  // an exactly zero initial residual (a field the step leaves unchanged, e.g. a constant one) is
  // converged: pcg_solver_p.m would test 0 < 0 and go on to alpha = 0/0
  if (!(norm_r < tol) && norm_r > 0.0) {
    for (it = 1; it <= D->itmax; ++it) {
      k_diff_jacobi<<<g, 256, 0, s>>>(n, D->ML, D->Cdiag, c, D->fixmask, D->r, D->d); count_launch();
      double beta = 0.0;
      if (it > 1) {
        // beta = (r - rlast) . d / rdlast (Polak-Ribiere)
        k_diff_sub<<<g, 256, 0, s>>>(n, D->r, D->rl, D->Aq); count_launch();
        double num;
        M3_TRY(dot(D->Aq, D->d, n, M->red, M->scal + 21, s));
        M3_TRY(read2(M, 21, num));
        beta = num / rd;
      }
      k_diff_dir<<<g, 256, 0, s>>>(n, D->d, beta, D->q, it == 1); count_launch();
      M3_TRY(dot(D->r, D->d, n, M->red, M->scal + 22, s));
      M3_TRY(read2(M, 22, rd));
      M3_TRY(diff_apply(M, D, D->q, 1.0, c, true, D->Aq));
      double qAq;
      M3_TRY(dot(D->q, D->Aq, n, M->red, M->scal + 23, s));
      M3_TRY(read2(M, 23, qAq));
      M3_CUDA(cudaMemcpyAsync(D->rl, D->r, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      const double alpha = rd / qAq;
      k_diff_step<<<g, 256, 0, s>>>(n, alpha, D->q, D->Aq, T, D->r); count_launch();
      M3_TRY(dot(D->r, D->r, n, M->red, M->scal + 20, s));
      M3_TRY(read2(M, 20, rr));
      norm_r = std::sqrt(rr) / sq;
      if (std::isnan(norm_r)) {
        set_error("NaN in the diffusion solve");
        return M3SPH_ERR_NAN;
      }
      if (norm_r < tol) break;
    }
    it = std::min(it, D->itmax);
  }
  M3_CUDA(cudaGetLastError());
  if (nit) *nit = it;
  return M3SPH_OK;
}

}  // namespace m3sph

using namespace m3sph;

extern "C" int m3sph_diffusion_setup(m3sph_mesh *M, const m3sph_diffusion_opts *o, const int32_t *ifix,
                                     const double *vfix, int32_t nfix) {
  if (!M || !o || nfix < 0 || (nfix > 0 && (!ifix || !vfix)) || !(o->kappa >= 0.0)) {
    set_error("m3sph_diffusion_setup: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  cudaStream_t s = M->stream;
  DiffState *D = diff_state(M);
  if (!D) {
    D = new DiffState();
    M->diff = D;
    M->diff_free = diff_free;
    M3_TRY(diff_build(M, D, o->theta_cone > 0 ? o->theta_cone : 45.0));
  }
  D->kappa = o->kappa;
  D->theta = o->theta;
  D->tol = o->tol > 0 ? o->tol : 1e-8;
  D->itmax = o->itmax > 0 ? o->itmax : 500;
  std::vector<int> fx(nfix);
  std::vector<uint8_t> mask(D->nnod, 0);
  for (int i = 0; i < nfix; ++i) {
    if (ifix[i] < 1 || ifix[i] > D->nnod) {
      set_error("m3sph_diffusion_setup: ifix entry out of range");
      return M3SPH_ERR_BAD_INPUT;
    }
    fx[i] = ifix[i] - 1;
    mask[fx[i]] = 1;
  }
  if (D->ifix) cudaFree(D->ifix);
  if (D->vfix) cudaFree(D->vfix);
  D->ifix = nullptr;
  D->vfix = nullptr;
  D->nfix = nfix;
  M3_TRY(dalloc_d((void **)&D->ifix, std::max(1, nfix) * sizeof(int)));
  M3_TRY(dalloc_d((void **)&D->vfix, std::max(1, nfix) * sizeof(double)));
  if (nfix) {
    M3_CUDA(cudaMemcpyAsync(D->ifix, fx.data(), nfix * sizeof(int), cudaMemcpyHostToDevice, s));
    M3_CUDA(cudaMemcpyAsync(D->vfix, vfix, nfix * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  M3_CUDA(cudaMemcpyAsync(D->fixmask, mask.data(), D->nnod, cudaMemcpyHostToDevice, s));
  M3_TRY(diff_integrate(M, D));
  M3_TRY(diff_diag(M, D));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

extern "C" int m3sph_diffusion3d(m3sph_mesh *M, double *T, double dt, int32_t *nit) {
  if (!M || !T) {
    set_error("m3sph_diffusion3d: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  DiffState *D = diff_state(M);
  if (!D) {
    set_error("m3sph_diffusion3d: call m3sph_diffusion_setup first");
    return M3SPH_ERR_BAD_INPUT;
  }
  cudaStream_t s = M->stream;
  double *Td = nullptr;
  M3_CUDA(cudaMalloc(&Td, D->nnod * sizeof(double)));
  int st = M3SPH_OK, it = 0;
  if (cudaMemcpyAsync(Td, T, D->nnod * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess)
    st = cuda_fail(cudaGetLastError(), "m3sph_diffusion3d upload");
  if (!st && D->kappa > 0.0) st = diffusion_resident(M, Td, dt, &it);
  if (!st && (cudaMemcpyAsync(T, Td, D->nnod * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
              cudaStreamSynchronize(s) != cudaSuccess))
    st = cuda_fail(cudaGetLastError(), "m3sph_diffusion3d download");
  cudaFree(Td);
  if (nit) *nit = it;
  return st;
}
