// Element-level kernels: curved P2P1 element matrices (double Jacobian), element-by-element
// operator application with a coloured, atomic-free scatter, and element-wise Galerkin
// coarse operators.
//
// Reference behaviour restated (paths inside the reference project):
//   mfiles_SPH/assembly_stokes_els_out_cone_no_cross_2pi_opt.m:93-356  element integrals
//   mfiles_SPH/assembly_stokes_els_out_cone_cross_2pi_opt.m:96-101,385-429  Z-180 frame
//   mfiles_SPH/assembly_stokes_els_in_cone_no_iso_opt.m:93-106,390-496      X-90 frame
//   mfiles_SPH/assembly_stokes_els_in_cone_iso_20_nodes_opt.m:97-157        20-node Jacobian
//   mfiles_M3TET/calc_element_visc.m:5-7,43-48, calc_element_dens.m:5-7
//   mfiles_M3TET/flow3d_patera_mg_sph_p.m:225-243 (K1 = RR' K RR), :294-298 (free dofs)
//   mfiles_M3TET/restrict_stiffmat.m:118-127 (KK{k+1} = Ic2f' KK{k} Ic2f)
#include <utility>

#include "common.cuh"

namespace m3sph {

__constant__ ShapeTables c_sf;

int upload_shape_tables() {
  ShapeTables t;
  build_shape_tables(t);
  M3_CUDA(cudaMemcpyToSymbol(c_sf, &t, sizeof(t)));
  return M3SPH_OK;
}

// ----------------------------------------------------------------------------------------
// element matrix set-up (FP64): one CTA handles EB elements
// ----------------------------------------------------------------------------------------
constexpr int EB = 32;
constexpr int SETUP_THREADS = 256;
// shared-memory layout per CTA, all arrays [..][EB]
constexpr int SM_DN = NIP * 10 * 3;     // dN/dx at each IP
constexpr int SM_W = NIP;               // weight
constexpr int SM_W2 = NIP;              // weight * viscosity
constexpr int SM_W3 = NIP;              // weight / viscosity
constexpr int SM_FG = NIP;              // weight * buoyancy
constexpr int SM_DIR = NIP * 3;         // radial unit vector in element frame
constexpr int SM_VC = 60;               // frame (theta,phi,r) of 4 (or 20) geometry nodes
constexpr int SM_Q = 90;                // per node: Q = R_cls * RR (3x3)
constexpr int SM_BC = 30;               // unmasked K * Ufix per element dof
constexpr int SM_PER_EL = SM_DN + SM_W + SM_W2 + SM_W3 + SM_FG + SM_DIR + SM_VC + SM_Q + SM_BC;
size_t element_setup_smem() { return sizeof(double) * SM_PER_EL * EB + sizeof(int) * 2 * EB; }



__device__ __forceinline__ void cart2sph_d(double x, double y, double z, double &th, double &ph, double &r) {
  r = sqrt(x * x + y * y + z * z);
  th = atan2(sqrt(x * x + y * y), z);
  ph = atan2(y, x);
  if (ph < 0.0) ph += 2.0 * M_PI;
}

__global__ void __launch_bounds__(SETUP_THREADS) k_element_setup(SetupArgs a) {
  extern __shared__ double sm[];
  double *sDN = sm;                          // [ip][n][k][EB]
  double *sW = sDN + SM_DN * EB;
  double *sW2 = sW + SM_W * EB;
  double *sW3 = sW2 + SM_W2 * EB;
  double *sFG = sW3 + SM_W3 * EB;
  double *sDIR = sFG + SM_FG * EB;           // [ip][3][EB]
  double *sVC = sDIR + SM_DIR * EB;          // [k][node][EB], node < 4 (or 20 for iso)
  double *sQ = sVC + SM_VC * EB;             // [n][9][EB]
  double *sBC = sQ + SM_Q * EB;              // [30][EB]
  int *sMask = reinterpret_cast<int *>(sBC + SM_BC * EB);
  int *sCls = sMask + EB;
  const int e0 = blockIdx.x * EB;
  const int tid = threadIdx.x;
  const int nel = a.nel;

  // phase 0: frame coordinates, per-node rotations and dof masks
  if (tid < EB) {
    const int el = tid, e = e0 + el;
    int cls = 0, mask = 0;
    if (e < nel) {
      cls = a.cls[e];
      int v[4];
      for (int i = 0; i < 4; ++i) v[i] = a.el2nod[i * nel + e];
      if (cls == M3SPH_IN_CONE_ISO) {
        const int s = a.iso_slot[e];
        for (int q = 0; q < 60; ++q) sVC[q * EB + el] = a.cubic[(size_t)q * a.niso + s];
      } else {
        for (int i = 0; i < 4; ++i) {
          double th, ph, r;
          if (cls == M3SPH_OUT_CONE_NO_CROSS_2PI || cls == M3SPH_OUT_CONE_CROSS_2PI) {
            th = a.gcoord_sph[v[i]];
            ph = a.gcoord_sph[a.nnod + v[i]];
            r = a.gcoord_sph[2 * a.nnod + v[i]];
            if (cls == M3SPH_OUT_CONE_CROSS_2PI) {   // 180 deg rotation about z: phi + pi
              ph += M_PI;
              if (ph > 2.0 * M_PI) ph -= 2.0 * M_PI;
            }
          } else {                                   // 90 deg rotation about x: (x, -z, y)
            const double x = a.gcoord[v[i]], y = a.gcoord[a.nnod + v[i]], z = a.gcoord[2 * a.nnod + v[i]];
            cart2sph_d(x, -z, y, th, ph, r);
          }
          // layout [k][node]: k*20 + node
          sVC[(0 * 20 + i) * EB + el] = th;
          sVC[(1 * 20 + i) * EB + el] = ph;
          sVC[(2 * 20 + i) * EB + el] = r;
        }
      }
      // Q_n = R_cls * RR_n, v_frame = Q_n v_local
      for (int n = 0; n < 10; ++n) {
        const int nod = a.el2nod[n * nel + e];
        double R[9];
        for (int q = 0; q < 9; ++q) R[q] = a.RR[(size_t)q * a.nnod + nod];
        double Q[9];
        if (cls == M3SPH_OUT_CONE_NO_CROSS_2PI) {
          for (int q = 0; q < 9; ++q) Q[q] = R[q];
        } else if (cls == M3SPH_OUT_CONE_CROSS_2PI) {      // diag(-1,-1,1)
          for (int q = 0; q < 3; ++q) { Q[q] = -R[q]; Q[3 + q] = -R[3 + q]; Q[6 + q] = R[6 + q]; }
        } else {                                            // [1 0 0; 0 0 -1; 0 1 0]
          for (int q = 0; q < 3; ++q) { Q[q] = R[q]; Q[3 + q] = -R[6 + q]; Q[6 + q] = R[3 + q]; }
        }
        for (int q = 0; q < 9; ++q) sQ[(n * 9 + q) * EB + el] = Q[q];
        for (int c = 0; c < 3; ++c)
          if (a.freemask[3 * nod + c]) mask |= 1 << (3 * n + c);
      }
    }
    sMask[el] = mask;
    sCls[el] = cls;
    if (a.emask && e < nel) a.emask[e] = (uint32_t)mask;
    for (int q = 0; q < 30; ++q) sBC[q * EB + el] = 0.0;
  }
  __syncthreads();

  // phase 1: geometry and material at each (IP, element)
  for (int t = tid; t < NIP * EB; t += SETUP_THREADS) {
    const int ip = t / EB, el = t % EB, e = e0 + el;
    if (e >= nel) continue;
    const int cls = sCls[el];
    double J[3][3];       // J[i][k] = d sph_k / d loc_i
    double sph[3];
    if (cls == M3SPH_IN_CONE_ISO) {
      for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) {
          double s = 0.0;
          for (int n = 0; n < 20; ++n) s += c_sf.dN20[ip][n][i] * sVC[(k * 20 + n) * EB + el];
          J[i][k] = s;
        }
      for (int k = 0; k < 3; ++k) {
        double s = 0.0;
        for (int n = 0; n < 20; ++n) s += c_sf.N20[ip][n] * sVC[(k * 20 + n) * EB + el];
        sph[k] = s;
      }
    } else {
      for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) J[i][k] = sVC[(k * 20 + i) * EB + el] - sVC[(k * 20 + 3) * EB + el];
      for (int k = 0; k < 3; ++k) {
        double s = 0.0;
        for (int n = 0; n < 4; ++n) s += c_sf.NP[ip][n] * sVC[(k * 20 + n) * EB + el];
        sph[k] = s;
      }
    }
    const double detSL = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    if (detSL < 0.0) atomicOr(a.err, 1);
    const double id = 1.0 / detSL;
    double Ji[3][3];      // inverse: Ji[k][j] = d loc_j / d sph_k
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    const double th = sph[0], ph = sph[1], r = sph[2];
    if (th == 0.0) atomicOr(a.err, 2);
    double st, ct, sp, cp;
    sincos(th, &st, &ct);
    sincos(ph, &sp, &cp);
    const double detCS = r * r * st;
    const double ic = 1.0 / detCS;
    // J_SC[c][k] = d sph_k / d cart_c (assembly_stokes_els_*_opt.m:136-138)
    double JSC[3][3];
    JSC[0][0] = r * st * ct * cp * ic; JSC[0][1] = -r * sp * ic; JSC[0][2] = r * r * st * st * cp * ic;
    JSC[1][0] = r * st * ct * sp * ic; JSC[1][1] = r * cp * ic;  JSC[1][2] = r * r * st * st * sp * ic;
    JSC[2][0] = -r * st * st * ic;     JSC[2][1] = 0.0;          JSC[2][2] = r * r * st * ct * ic;
    double Jd[3][3];      // Jd[c][j] = d loc_j / d cart_c
    for (int c = 0; c < 3; ++c)
      for (int j = 0; j < 3; ++j) Jd[c][j] = JSC[c][0] * Ji[0][j] + JSC[c][1] * Ji[1][j] + JSC[c][2] * Ji[2][j];
    for (int n = 0; n < 10; ++n)
      for (int c = 0; c < 3; ++c)
        sDN[((ip * 10 + n) * 3 + c) * EB + el] =
            Jd[c][0] * c_sf.dNU[ip][n][0] + Jd[c][1] * c_sf.dNU[ip][n][1] + Jd[c][2] * c_sf.dNU[ip][n][2];
    const double w = detCS * detSL * c_sf.ipw[ip];
    double visc = 0.0, dens = 0.0;
    for (int v = 0; v < 4; ++v) {
      const int nod = a.el2nod[v * nel + e];
      visc += a.visc[nod] * c_sf.NP[ip][v];
      dens += a.dens[nod] * c_sf.NP[ip][v];
    }
    if (a.minVisc > 0.0) visc = fmax(visc, a.minVisc);
    if (a.maxVisc > 0.0) visc = fmin(visc, a.maxVisc);
    if (!(visc > 0.0)) atomicOr(a.err, 4);
    sW[ip * EB + el] = w;
    sW2[ip * EB + el] = w * visc;
    if (a.PA32) {
      // sqrt(w eta) d xi_j / d x_c in global Cartesian components: frame = R_cls global, so
      // d xi / d x_global = R_cls^T Jd (Z-180: diag(-1,-1,1); X-90: frame (x, -z, y))
      const double sq = sqrt(w * visc);
      for (int j = 0; j < 3; ++j) {
        double g0 = Jd[0][j], g1 = Jd[1][j], g2 = Jd[2][j];
        if (cls == M3SPH_OUT_CONE_CROSS_2PI) {
          g0 = -g0;
          g1 = -g1;
        } else if (cls != M3SPH_OUT_CONE_NO_CROSS_2PI) {
          const double t1 = g1;
          g1 = Jd[2][j];
          g2 = -t1;
        }
        a.PA32[((size_t)ip * 9 + 0 * 3 + j) * a.pa_ld + e] = (float)(sq * g0);
        a.PA32[((size_t)ip * 9 + 1 * 3 + j) * a.pa_ld + e] = (float)(sq * g1);
        a.PA32[((size_t)ip * 9 + 2 * 3 + j) * a.pa_ld + e] = (float)(sq * g2);
      }
    }
    sW3[ip * EB + el] = w / visc;
    sFG[ip * EB + el] = w * a.g * a.Bscale * (dens - a.Dens0);
    sDIR[(ip * 3 + 0) * EB + el] = st * cp;
    sDIR[(ip * 3 + 1) * EB + el] = st * sp;
    sDIR[(ip * 3 + 2) * EB + el] = ct;
  }
  __syncthreads();

  // phase 2a: stiffness blocks (i >= j), rotated to node frames and masked
  constexpr double C2 = -2.0 / 3.0;
  for (int t = tid; t < 55 * EB; t += SETUP_THREADS) {
    const int blk = t / EB, el = t % EB, e = e0 + el;
    if (e >= nel) continue;
    int i = 0, rem = blk;
    while (rem > i) { rem -= i + 1; ++i; }        // blk -> (i, j), j <= i
    const int j = rem;
    double B[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int ip = 0; ip < NIP; ++ip) {
      const double w2 = sW2[ip * EB + el];
      double di[3], dj[3];
      for (int c = 0; c < 3; ++c) {
        di[c] = sDN[((ip * 10 + i) * 3 + c) * EB + el];
        dj[c] = sDN[((ip * 10 + j) * 3 + c) * EB + el];
      }
      const double lap = di[0] * dj[0] + di[1] * dj[1] + di[2] * dj[2];
      for (int p = 0; p < 3; ++p)
        for (int q = 0; q < 3; ++q) {
          // K[(i,p),(j,q)] = w2 (d_pq gradNi.gradNj + d_q Ni d_p Nj - 2/3 d_p Ni d_q Nj)
          double v = di[q] * dj[p] + C2 * di[p] * dj[q];
          if (p == q) v += lap;
          B[p][q] += w2 * v;
        }
    }
    double Qi[9], Qj[9];
    for (int q = 0; q < 9; ++q) { Qi[q] = sQ[(i * 9 + q) * EB + el]; Qj[q] = sQ[(j * 9 + q) * EB + el]; }
    // T = B Qj ; Kl = Qi^T T
    double T[3][3];
    for (int p = 0; p < 3; ++p)
      for (int q = 0; q < 3; ++q) T[p][q] = B[p][0] * Qj[0 * 3 + q] + B[p][1] * Qj[1 * 3 + q] + B[p][2] * Qj[2 * 3 + q];
    const int mask = sMask[el];
    const bool bc = a.ufix != nullptr;
    int ni = 0, nj = 0;
    if (bc) {
      ni = a.el2nod[(size_t)i * nel + e];
      nj = a.el2nod[(size_t)j * nel + e];
    }
    for (int p = 0; p < 3; ++p)
      for (int q = 0; q < 3; ++q) {
        const int rr = 3 * i + p, cc = 3 * j + q;
        double v = Qi[0 * 3 + p] * T[0][q] + Qi[1 * 3 + p] * T[1][q] + Qi[2 * 3 + p] * T[2][q];
        if (bc) {
          // boundary-condition rhs from the unmasked operator: K(:,ifix) * Ufix
          // (flow3d_patera_mg_sph_p.m:269-283); each (i,j) block also stands for (j,i) when i > j
          atomicAdd(&sBC[rr * EB + el], v * a.ufix[3 * nj + q]);
          if (i != j) atomicAdd(&sBC[cc * EB + el], v * a.ufix[3 * ni + p]);
        }
        if (rr < cc) continue;
        if (!((mask >> rr) & 1) || !((mask >> cc) & 1)) v = 0.0;
        const int k = pack_idx(rr, cc);
        a.K64[kidx<double>(k, e, nel)] = v;
        const float hi = (float)v;
        a.K32[kidx<float>(k, e, nel)] = hi;
        if (a.KL32) a.KL32[kidx<float>(k, e, nel)] = (float)(v - (double)hi);
      }
  }
  // phase 2b: gradient matrix G[p][3n+c'] (rotated, not masked)
  for (int t = tid; t < 40 * EB; t += SETUP_THREADS) {
    const int q = t / EB, el = t % EB, e = e0 + el;
    if (e >= nel) continue;
    const int n = q / 4, p = q % 4;
    double Gf[3] = {0, 0, 0};
    for (int ip = 0; ip < NIP; ++ip) {
      const double wn = sW[ip * EB + el] * c_sf.NP[ip][p];
      for (int c = 0; c < 3; ++c) Gf[c] += wn * sDN[((ip * 10 + n) * 3 + c) * EB + el];
    }
    for (int cc = 0; cc < 3; ++cc) {
      double v = 0.0;
      for (int c = 0; c < 3; ++c) v += sQ[(n * 9 + c * 3 + cc) * EB + el] * Gf[c];
      a.G64[(size_t)(p * 30 + 3 * n + cc) * nel + e] = v;
    }
  }
  // phase 2c: (1/viscosity)-scaled pressure mass matrix, packed lower 4x4
  for (int t = tid; t < 10 * EB; t += SETUP_THREADS) {
    const int q = t / EB, el = t % EB, e = e0 + el;
    if (e >= nel) continue;
    int c = 0, rem = q;
    while (rem >= 4 - c) { rem -= 4 - c; ++c; }
    const int r = c + rem;
    double v = 0.0;
    for (int ip = 0; ip < NIP; ++ip) v += sW3[ip * EB + el] * c_sf.NP[ip][r] * c_sf.NP[ip][c];
    a.M64[(size_t)q * nel + e] = v;
  }
  // phase 2d: buoyancy force (rotated)
  for (int t = tid; t < 10 * EB; t += SETUP_THREADS) {
    const int n = t / EB, el = t % EB, e = e0 + el;
    if (e >= nel) continue;
    double F[3] = {0, 0, 0};
    for (int ip = 0; ip < NIP; ++ip) {
      const double f = sFG[ip * EB + el] * c_sf.NU[ip][n];
      for (int c = 0; c < 3; ++c) F[c] += f * sDIR[(ip * 3 + c) * EB + el];
    }
    for (int cc = 0; cc < 3; ++cc) {
      double v = 0.0;
      for (int c = 0; c < 3; ++c) v += sQ[(n * 9 + c * 3 + cc) * EB + el] * F[c];
      a.Fbe[(size_t)(3 * n + cc) * nel + e] = v;
    }
  }
  if (a.ufix) {
    __syncthreads();
    for (int t = tid; t < 30 * EB; t += SETUP_THREADS) {
      const int q = t / EB, el = t % EB, e = e0 + el;
      if (e < nel) a.BCe[(size_t)q * nel + e] = sBC[q * EB + el];
    }
  }
}

int launch_element_setup(const SetupArgs &a, cudaStream_t s) {
  const size_t smem = element_setup_smem();
  M3_CUDA(cudaFuncSetAttribute(k_element_setup, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = (a.nel + EB - 1) / EB;
  k_element_setup<<<grid, SETUP_THREADS, smem, s>>>(a); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// ----------------------------------------------------------------------------------------
// element-by-element y += K x over one colour (no two elements of a colour share a node)
// ----------------------------------------------------------------------------------------
template <typename T> struct Vec;
template <> struct Vec<float> { using type = float4; };
template <> struct Vec<double> { using type = double2; };
template <typename V, typename T> __device__ __forceinline__ T lane(const V &v, int i);
template <> __device__ __forceinline__ float lane<float4, float>(const float4 &v, int i) {
  return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}
template <> __device__ __forceinline__ double lane<double2, double>(const double2 &v, int i) {
  return i == 0 ? v.x : v.y;
}

template <typename T>
__global__ void __launch_bounds__(128) k_ebe_apply(const T *__restrict__ K, const int *__restrict__ el2nod, int nel,
                                                   int e_begin, int e_end, const T *__restrict__ x, T *__restrict__ y) {
  using VT = typename Vec<T>::type;
  constexpr int V = KVec<T>::V;
  const int e = e_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= e_end) return;
  int nod[10];
#pragma unroll
  for (int n = 0; n < 10; ++n) nod[n] = __ldg(el2nod + (size_t)n * nel + e);
  T xe[30], ye[30];
#pragma unroll
  for (int n = 0; n < 10; ++n)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      xe[3 * n + c] = x[3 * nod[n] + c];
      ye[3 * n + c] = T(0);
    }
  const VT *Kv = reinterpret_cast<const VT *>(K) + e;
  VT v4;
  int k = 0;
#pragma unroll
  for (int c = 0; c < 30; ++c) {
#pragma unroll
    for (int r = c; r < 30; ++r) {
      if (k % V == 0) v4 = __ldcs(Kv + (size_t)(k / V) * nel);
      const T v = lane<VT, T>(v4, k % V);
      ye[r] += v * xe[c];
      if (r != c) ye[c] += v * xe[r];
      ++k;
    }
  }
#pragma unroll
  for (int n = 0; n < 10; ++n)
#pragma unroll
    for (int c = 0; c < 3; ++c) y[3 * nod[n] + c] += ye[3 * n + c];
}

// y += K x in FP64 accuracy from FP32 arithmetic: K = hi + lo (two FP32 arrays, hi is the FP32
// operator of the V-cycle), x split the same way at the gather; each product is formed exactly
// (FMA error term) and accumulated in double-float (Knuth two-sum). ~10 FP32 operations per
// multiply-add instead of one FP64 FMA, which GB300 issues at 1/62 of its FP32 rate.

__global__ void __launch_bounds__(128) k_ebe_apply_df(const float *__restrict__ Kh, const float *__restrict__ Kl,
                                                      const int *__restrict__ el2nod, int nel, int e_begin, int e_end,
                                                      const double *__restrict__ x, double *__restrict__ y) {
  const int e = e_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= e_end) return;
  int nod[10];
#pragma unroll
  for (int n = 0; n < 10; ++n) nod[n] = __ldg(el2nod + (size_t)n * nel + e);
  float xh[30], xl[30], sh[30], sl[30];
#pragma unroll
  for (int n = 0; n < 10; ++n)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double xv = x[3 * nod[n] + c];
      const float h = (float)xv;
      xh[3 * n + c] = h;
      xl[3 * n + c] = (float)(xv - (double)h);
      sh[3 * n + c] = 0.f;
      sl[3 * n + c] = 0.f;
    }
  const float4 *Hv = reinterpret_cast<const float4 *>(Kh) + e;
  const float4 *Lv = reinterpret_cast<const float4 *>(Kl) + e;
  float4 h4, l4;
  int k = 0;
#pragma unroll
  for (int c = 0; c < 30; ++c) {
#pragma unroll
    for (int r = c; r < 30; ++r) {
      if (k % 4 == 0) {
        h4 = __ldcs(Hv + (size_t)(k / 4) * nel);
        l4 = __ldcs(Lv + (size_t)(k / 4) * nel);
      }
      const float vh = lane<float4, float>(h4, k % 4), vl = lane<float4, float>(l4, k % 4);
      df_mac(vh, vl, xh[c], xl[c], sh[r], sl[r]);
      if (r != c) df_mac(vh, vl, xh[r], xl[r], sh[c], sl[c]);
      ++k;
    }
  }
#pragma unroll
  for (int n = 0; n < 10; ++n)
#pragma unroll
    for (int c = 0; c < 3; ++c) y[3 * nod[n] + c] += (double)sh[3 * n + c] + (double)sl[3 * n + c];
}

int ebe_apply_df(const Level &L, const float *Kh, const float *Kl, const double *x, double *y, cudaStream_t s) {
  M3_CUDA(cudaMemsetAsync(y, 0, sizeof(double) * L.ndof, s));
  const int nc = (int)L.cstart.size() - 1;
  for (int c = 0; c < nc; ++c) {
    const int b = L.cstart[c], e = L.cstart[c + 1];
    if (e <= b) continue;
    k_ebe_apply_df<<<(e - b + 127) / 128, 128, 0, s>>>(Kh, Kl, L.el2nod, L.nel, b, e, x, y); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// ----------------------------------------------------------------------------------------
// split element-by-element apply: a CTA of 4 warps handles 32 elements of one colour; warp w
// streams the w-th quarter of the packed matrix (lanes = elements, so every load of a warp is
// one contiguous 512-byte segment), partial results are summed in shared memory and scattered.
// Packed entry k -> (row, col) is resolved at compile time.
// ----------------------------------------------------------------------------------------

struct OpF32 {   // FP32 V-cycle operator
  using acc_t = float;
  static constexpr bool two_part = false;
  static constexpr int V = 4;
  static constexpr int NCH = 117;
  const float4 *K;
  __device__ __forceinline__ void init(float (&y)[30], float (&)[30]) const {
#pragma unroll
    for (int i = 0; i < 30; ++i) y[i] = 0.f;
  }
  template <int Q>
  __device__ __forceinline__ void chunk(size_t off, const float (&xh)[30], const float (&)[30], float (&y)[30],
                                        float (&)[30]) const {
    const float4 v = __ldcs(K + off);
    entry<4 * Q + 0>(v.x, xh, y);
    entry<4 * Q + 1>(v.y, xh, y);
    entry<4 * Q + 2>(v.z, xh, y);
    entry<4 * Q + 3>(v.w, xh, y);
  }
  template <int k>
  __device__ __forceinline__ static void entry(float v, const float (&x)[30], float (&y)[30]) {
    if constexpr (k < NPACK) {
      constexpr int c = unpack_c(k), r = unpack_r(k);
      y[r] += v * x[c];
      if constexpr (r != c) y[c] += v * x[r];
    }
  }
};

struct OpF64 {   // native FP64 operator (plain path)
  using acc_t = double;
  static constexpr bool two_part = false;
  static constexpr int V = 2;
  static constexpr int NCH = 233;
  const double2 *K;
  __device__ __forceinline__ void init(double (&y)[30], double (&)[30]) const {
#pragma unroll
    for (int i = 0; i < 30; ++i) y[i] = 0.0;
  }
  template <int Q>
  __device__ __forceinline__ void chunk(size_t off, const double (&xh)[30], const double (&)[30], double (&y)[30],
                                        double (&)[30]) const {
    const double2 v = __ldcs(K + off);
    entry<2 * Q + 0>(v.x, xh, y);
    entry<2 * Q + 1>(v.y, xh, y);
  }
  template <int k>
  __device__ __forceinline__ static void entry(double v, const double (&x)[30], double (&y)[30]) {
    if constexpr (k < NPACK) {
      constexpr int c = unpack_c(k), r = unpack_r(k);
      y[r] += v * x[c];
      if constexpr (r != c) y[c] += v * x[r];
    }
  }
};

struct OpDF {    // double-float operator (mixed path, outer iterations)
  using acc_t = float;
  static constexpr bool two_part = true;
  static constexpr int V = 4;
  static constexpr int NCH = 117;
  const float4 *Kh, *Kl;
  __device__ __forceinline__ void init(float (&sh)[30], float (&sl)[30]) const {
#pragma unroll
    for (int i = 0; i < 30; ++i) { sh[i] = 0.f; sl[i] = 0.f; }
  }
  template <int Q>
  __device__ __forceinline__ void chunk(size_t off, const float (&xh)[30], const float (&xl)[30], float (&sh)[30],
                                        float (&sl)[30]) const {
    const float4 h = __ldcs(Kh + off), l = __ldcs(Kl + off);
    entry<4 * Q + 0>(h.x, l.x, xh, xl, sh, sl);
    entry<4 * Q + 1>(h.y, l.y, xh, xl, sh, sl);
    entry<4 * Q + 2>(h.z, l.z, xh, xl, sh, sl);
    entry<4 * Q + 3>(h.w, l.w, xh, xl, sh, sl);
  }
  template <int k>
  __device__ __forceinline__ static void entry(float vh, float vl, const float (&xh)[30], const float (&xl)[30],
                                               float (&sh)[30], float (&sl)[30]) {
    if constexpr (k < NPACK) {
      constexpr int c = unpack_c(k), r = unpack_r(k);
      df_mac(vh, vl, xh[c], xl[c], sh[r], sl[r]);
      if constexpr (r != c) df_mac(vh, vl, xh[r], xl[r], sh[c], sl[c]);
    }
  }
};

template <class Op, int Q0, int... Is>
__device__ __forceinline__ void run_chunks(const Op &op, int e, size_t nel, const typename Op::acc_t (&xh)[30],
                                           const typename Op::acc_t (&xl)[30], typename Op::acc_t (&y)[30],
                                           typename Op::acc_t (&yl)[30], std::integer_sequence<int, Is...>) {
  (op.template chunk<Q0 + Is>((size_t)(Q0 + Is) * nel + e, xh, xl, y, yl), ...);
}

template <class Op, int P>
__device__ __forceinline__ void run_part(const Op &op, int e, size_t nel, const typename Op::acc_t (&xh)[30],
                                         const typename Op::acc_t (&xl)[30], typename Op::acc_t (&y)[30],
                                         typename Op::acc_t (&yl)[30]) {
  constexpr int b = (Op::NCH * P) / 4, en = (Op::NCH * (P + 1)) / 4;
  run_chunks<Op, b>(op, e, nel, xh, xl, y, yl, std::make_integer_sequence<int, en - b>{});
}

template <class Op, typename XT>
__global__ void __launch_bounds__(128) k_ebe_apply_split(Op op, const int *__restrict__ el2nod, int nel, int e_begin,
                                                         int e_end, const XT *__restrict__ x, XT *__restrict__ y) {
  using A = typename Op::acc_t;
  __shared__ XT sY[4][30][33];
  __shared__ int sNod[10][32];
  const int lane = threadIdx.x & 31, part = threadIdx.x >> 5;
  const int e0 = e_begin + blockIdx.x * 32;
  const int e = e0 + lane;
  const bool valid = e < e_end;
  if (part == 0)
#pragma unroll
    for (int n = 0; n < 10; ++n) sNod[n][lane] = valid ? __ldg(el2nod + (size_t)n * nel + e) : 0;
  __syncthreads();
  A xh[30], xl[30], yh[30], yl[30];
  op.init(yh, yl);
  if (valid) {
#pragma unroll
    for (int n = 0; n < 10; ++n)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const XT xv = x[3 * sNod[n][lane] + c];
        const A h = (A)xv;
        xh[3 * n + c] = h;
        xl[3 * n + c] = (A)(xv - (XT)h);
      }
    switch (part) {
      case 0: run_part<Op, 0>(op, e, nel, xh, xl, yh, yl); break;
      case 1: run_part<Op, 1>(op, e, nel, xh, xl, yh, yl); break;
      case 2: run_part<Op, 2>(op, e, nel, xh, xl, yh, yl); break;
      default: run_part<Op, 3>(op, e, nel, xh, xl, yh, yl); break;
    }
  }
#pragma unroll
  for (int q = 0; q < 30; ++q) {
    if constexpr (Op::two_part)
      sY[part][q][lane] = (XT)yh[q] + (XT)yl[q];
    else
      sY[part][q][lane] = (XT)yh[q];
  }
  __syncthreads();
  for (int o = threadIdx.x; o < 30 * 32; o += 128) {
    const int q = o >> 5, el = o & 31;
    if (e0 + el >= e_end) continue;
    const XT v = sY[0][q][el] + sY[1][q][el] + sY[2][q][el] + sY[3][q][el];
    y[3 * sNod[q / 3][el] + q % 3] += v;
  }
}

template <class Op, typename XT>
static int ebe_apply_split(const Level &L, const Op &op, const XT *x, XT *y, cudaStream_t s) {
  M3_CUDA(cudaMemsetAsync(y, 0, sizeof(XT) * L.ndof, s));
  const int nc = (int)L.cstart.size() - 1;
  for (int c = 0; c < nc; ++c) {
    const int b = L.cstart[c], e = L.cstart[c + 1];
    if (e <= b) continue;
    k_ebe_apply_split<Op, XT><<<(e - b + 31) / 32, 128, 0, s>>>(op, L.el2nod, L.nel, b, e, x, y); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

int ebe_apply_split_f32(const Level &L, const float *K, const float *x, float *y, cudaStream_t s) {
  return ebe_apply_split(L, OpF32{reinterpret_cast<const float4 *>(K)}, x, y, s);
}
int ebe_apply_split_f64(const Level &L, const double *K, const double *x, double *y, cudaStream_t s) {
  return ebe_apply_split(L, OpF64{reinterpret_cast<const double2 *>(K)}, x, y, s);
}
int ebe_apply_split_df(const Level &L, const float *Kh, const float *Kl, const double *x, double *y, cudaStream_t s) {
  return ebe_apply_split(L, OpDF{reinterpret_cast<const float4 *>(Kh), reinterpret_cast<const float4 *>(Kl)}, x, y, s);
}

template <typename T>
int ebe_apply(const Level &L, const T *K, const T *x, T *y, cudaStream_t s) {
  M3_CUDA(cudaMemsetAsync(y, 0, sizeof(T) * L.ndof, s));
  const int nc = (int)L.cstart.size() - 1;
  for (int c = 0; c < nc; ++c) {
    const int b = L.cstart[c], e = L.cstart[c + 1];
    if (e <= b) continue;
    k_ebe_apply<T><<<(e - b + 127) / 128, 128, 0, s>>>(K, L.el2nod, L.nel, b, e, x, y); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template int ebe_apply<double>(const Level &, const double *, const double *, double *, cudaStream_t);
template int ebe_apply<float>(const Level &, const float *, const float *, float *, cudaStream_t);

// assemble element vectors V[q][nel] (q < nq) into node dofs / pressure nodes, per colour
__global__ void k_scatter_elvec(const double *__restrict__ V, int nq, int per_node, const int *__restrict__ el2nod,
                                int nel, int e_begin, int e_end, double *__restrict__ out) {
  const int e = e_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= e_end) return;
  for (int q = 0; q < nq; ++q) {
    const int n = q / per_node, c = q % per_node;
    const int nod = el2nod[(size_t)n * nel + e];
    out[per_node * nod + c] += V[(size_t)q * nel + e];
  }
}

int scatter_elvec(const Level &L, const double *V, int nq, int per_node, double *out, size_t nout, cudaStream_t s) {
  M3_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * nout, s));
  const int nc = (int)L.cstart.size() - 1;
  for (int c = 0; c < nc; ++c) {
    const int b = L.cstart[c], e = L.cstart[c + 1];
    if (e <= b) continue;
    k_scatter_elvec<<<(e - b + 127) / 128, 128, 0, s>>>(V, nq, per_node, L.el2nod, L.nel, b, e, out); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// diagonal of the element matrices -> inverse diagonal (0 on fixed dofs)
template <typename T>
__global__ void k_diag_scatter(const T *__restrict__ K, const int *__restrict__ el2nod, int nel, int e_begin,
                               int e_end, double *__restrict__ D) {
  const int e = e_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= e_end) return;
  for (int q = 0; q < 30; ++q) {
    const int nod = el2nod[(size_t)(q / 3) * nel + e];
    D[3 * nod + q % 3] += (double)K[kidx<T>(pack_idx(q, q), e, nel)];
  }
}

__global__ void k_invert_diag(const double *D, const uint8_t *mask, int n, double *Di64, float *Di32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = (mask[i] && D[i] != 0.0) ? 1.0 / D[i] : 0.0;
  if (Di64) Di64[i] = v;
  if (Di32) Di32[i] = (float)v;
}

template <typename T>
int level_inverse_diag(Level &L, const T *K, double *work, cudaStream_t s) {
  M3_CUDA(cudaMemsetAsync(work, 0, sizeof(double) * L.ndof, s));
  const int nc = (int)L.cstart.size() - 1;
  for (int c = 0; c < nc; ++c) {
    const int b = L.cstart[c], e = L.cstart[c + 1];
    if (e <= b) continue;
    k_diag_scatter<T><<<(e - b + 127) / 128, 128, 0, s>>>(K, L.el2nod, L.nel, b, e, work); count_launch();
  }
  k_invert_diag<<<(L.ndof + 255) / 256, 256, 0, s>>>(work, L.freemask, L.ndof, L.Dinv64, L.Dinv32); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template int level_inverse_diag<double>(Level &, const double *, double *, cudaStream_t);
template int level_inverse_diag<float>(Level &, const float *, double *, cudaStream_t);

// ----------------------------------------------------------------------------------------
// gradient / divergence / pressure-mass applications (finest level, per colour)
// ----------------------------------------------------------------------------------------
// y(3*nnod) += G q  (G[p][3n+c])
__global__ void k_grad(const double *__restrict__ G, const int *__restrict__ el2nod, int nel, int eb, int ee,
                       const double *__restrict__ q, double *__restrict__ y) {
  const int e = eb + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ee) return;
  double qe[4];
  for (int p = 0; p < 4; ++p) qe[p] = q[el2nod[(size_t)p * nel + e]];
  for (int n = 0; n < 10; ++n) {
    const int nod = el2nod[(size_t)n * nel + e];
    for (int c = 0; c < 3; ++c) {
      double v = 0.0;
      for (int p = 0; p < 4; ++p) v += G[(size_t)(p * 30 + 3 * n + c) * nel + e] * qe[p];
      y[3 * nod + c] += v;
    }
  }
}
// s(nvnod) += G^T z
__global__ void k_div(const double *__restrict__ G, const int *__restrict__ el2nod, int nel, int eb, int ee,
                      const double *__restrict__ z, double *__restrict__ s) {
  const int e = eb + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ee) return;
  double ze[30];
  for (int n = 0; n < 10; ++n) {
    const int nod = el2nod[(size_t)n * nel + e];
    for (int c = 0; c < 3; ++c) ze[3 * n + c] = z[3 * nod + c];
  }
  for (int p = 0; p < 4; ++p) {
    double v = 0.0;
    for (int q = 0; q < 30; ++q) v += G[(size_t)(p * 30 + q) * nel + e] * ze[q];
    s[el2nod[(size_t)p * nel + e]] += v;
  }
}
// y(nvnod) += M d (packed lower 4x4) or lumped row sums if d == nullptr
__global__ void k_mass(const double *__restrict__ M, const int *__restrict__ el2nod, int nel, int eb, int ee,
                       const double *__restrict__ d, double *__restrict__ y) {
  const int e = eb + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ee) return;
  double de[4], ye[4] = {0, 0, 0, 0};
  int nod[4];
  for (int p = 0; p < 4; ++p) {
    nod[p] = el2nod[(size_t)p * nel + e];
    de[p] = d ? d[nod[p]] : 1.0;
  }
  int k = 0;
  for (int c = 0; c < 4; ++c)
    for (int r = c; r < 4; ++r) {
      const double v = M[(size_t)k * nel + e];
      ++k;
      ye[r] += v * de[c];
      if (r != c) ye[c] += v * de[r];
    }
  for (int p = 0; p < 4; ++p) y[nod[p]] += ye[p];
}

int grad_apply(const Level &L, const double *G, const double *q, double *y, cudaStream_t s) {
  M3_CUDA(cudaMemsetAsync(y, 0, sizeof(double) * L.ndof, s));
  for (size_t c = 0; c + 1 < L.cstart.size(); ++c) {
    const int b = L.cstart[c], e = L.cstart[c + 1];
    if (e > b) k_grad<<<(e - b + 127) / 128, 128, 0, s>>>(G, L.el2nod, L.nel, b, e, q, y); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
int div_apply(const Level &L, const double *G, const double *z, double *out, cudaStream_t s) {
  M3_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * L.nvnod, s));
  for (size_t c = 0; c + 1 < L.cstart.size(); ++c) {
    const int b = L.cstart[c], e = L.cstart[c + 1];
    if (e > b) k_div<<<(e - b + 127) / 128, 128, 0, s>>>(G, L.el2nod, L.nel, b, e, z, out); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
int mass_apply(const Level &L, const double *M, const double *d, double *out, cudaStream_t s) {
  M3_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * L.nvnod, s));
  for (size_t c = 0; c + 1 < L.cstart.size(); ++c) {
    const int b = L.cstart[c], e = L.cstart[c + 1];
    if (e > b) k_mass<<<(e - b + 127) / 128, 128, 0, s>>>(M, L.el2nod, L.nel, b, e, d, out); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

// ----------------------------------------------------------------------------------------
// element-wise Galerkin coarse operator: Kc(p) = sum_k W_k^T Kf(child k) W_k (per component),
// then coarse dofs that are fixed are zeroed. One CTA per coarse element.
// ----------------------------------------------------------------------------------------
__constant__ double c_p2lc[10][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0},   {.5, .5, 0},
                                     {0, .5, .5}, {0, 0, .5}, {.5, 0, 0}, {.5, 0, .5}, {0, .5, 0}};
__constant__ int c_edges[6][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 2}, {3, 1}};

__device__ __forceinline__ void sf10_d(double r, double s, double t, double *N) {
  const double u = 1.0 - r - s - t;
  N[0] = r * (2 * r - 1); N[1] = s * (2 * s - 1); N[2] = t * (2 * t - 1); N[3] = u * (2 * u - 1);
  N[4] = 4 * r * s; N[5] = 4 * s * t; N[6] = 4 * t * u; N[7] = 4 * r * u; N[8] = 4 * r * t; N[9] = 4 * s * u;
}

template <typename T>
__global__ void __launch_bounds__(256) k_galerkin(const T *__restrict__ Kf, int nel_f, const int *__restrict__ child,
                                                  const uint32_t *__restrict__ child_vloc, int nel_c,
                                                  const int *__restrict__ el2nod_c, const uint8_t *__restrict__ mask_c,
                                                  T *__restrict__ Kc) {
  __shared__ T sK[30][31];
  __shared__ T sT[30][31];
  __shared__ T sW[10][10];
  __shared__ T sAcc[NPACK];
  const int pc = blockIdx.x;
  const int tid = threadIdx.x;
  for (int q = tid; q < NPACK; q += blockDim.x) sAcc[q] = T(0);
  for (int k = 0; k < 8; ++k) {
    const int fe = child[(size_t)k * nel_c + pc];
    const uint32_t vl = child_vloc[(size_t)k * nel_c + pc];
    __syncthreads();
    // prolongation weights of this child: W[i][j] = N_j(parent) at lattice of child node i
    if (tid < 10) {
      const int i = tid;
      double lc[3];
      if (i < 4) {
        const int pn = (vl >> (4 * i)) & 15;
        for (int d = 0; d < 3; ++d) lc[d] = c_p2lc[pn][d];
      } else {
        const int a0 = (vl >> (4 * c_edges[i - 4][0])) & 15, a1 = (vl >> (4 * c_edges[i - 4][1])) & 15;
        for (int d = 0; d < 3; ++d) lc[d] = 0.5 * (c_p2lc[a0][d] + c_p2lc[a1][d]);
      }
      double N[10];
      sf10_d(lc[0], lc[1], lc[2], N);
      for (int j = 0; j < 10; ++j) sW[i][j] = (T)N[j];
    }
    for (int q = tid; q < 900; q += blockDim.x) {
      const int r = q / 30, c = q % 30;
      const int rr = r > c ? r : c, cc = r > c ? c : r;
      sK[r][c] = Kf[kidx<T>(pack_idx(rr, cc), fe, nel_f)];
    }
    __syncthreads();
    // T[a][(j,c)] = sum_i K[a][(i,c)] W[i][j]
    for (int q = tid; q < 900; q += blockDim.x) {
      const int aa = q / 30, jc = q % 30, j = jc / 3, c = jc % 3;
      T v = T(0);
#pragma unroll
      for (int i = 0; i < 10; ++i) v += sK[aa][3 * i + c] * sW[i][j];
      sT[aa][jc] = v;
    }
    __syncthreads();
    // Acc[(j,c)][(l,d)] += sum_i W[i][j] T[(i,c)][(l,d)]  (lower part)
    for (int q = tid; q < NPACK; q += blockDim.x) {
      int cc = 0, rem = q;
      while (rem >= 30 - cc) { rem -= 30 - cc; ++cc; }
      const int rr = cc + rem;
      const int j = rr / 3, c = rr % 3;
      T v = T(0);
#pragma unroll
      for (int i = 0; i < 10; ++i) v += sW[i][j] * sT[3 * i + c][cc];
      sAcc[q] += v;
    }
  }
  __syncthreads();
  for (int q = tid; q < NPACK; q += blockDim.x) {
    int cc = 0, rem = q;
    while (rem >= 30 - cc) { rem -= 30 - cc; ++cc; }
    const int rr = cc + rem;
    const int nr = el2nod_c[(size_t)(rr / 3) * nel_c + pc], nc = el2nod_c[(size_t)(cc / 3) * nel_c + pc];
    T v = sAcc[q];
    if (!mask_c[3 * nr + rr % 3] || !mask_c[3 * nc + cc % 3]) v = T(0);
    Kc[kidx<T>(q, pc, nel_c)] = v;
  }
}

template <typename T>
int galerkin(const Level &F, const T *Kf, Level &C, T *Kc, cudaStream_t s) {
  k_galerkin<T><<<C.nel, 256, 0, s>>>(Kf, F.nel, C.child, C.child_vloc, C.nel, C.el2nod, C.freemask, Kc); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template int galerkin<double>(const Level &, const double *, Level &, double *, cudaStream_t);
template int galerkin<float>(const Level &, const float *, Level &, float *, cudaStream_t);

// ----------------------------------------------------------------------------------------
// assembled block operator for coarse levels: gather-assembly (deterministic, no atomics) and
// block-row SpMV. Block (i,j) of the level operator is the sum over elements containing nodes i
// and j of the element block (a,b) with node(a) = i, node(b) = j.
// ----------------------------------------------------------------------------------------
template <typename T>
__global__ void k_bsr_assemble(const T *__restrict__ K, int nel, int nnzb, const int *__restrict__ cptr,
                               const int *__restrict__ contrib, T *__restrict__ B) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnzb) return;
  T acc[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) acc[q] = T(0);
  for (int c = cptr[k]; c < cptr[k + 1]; ++c) {
    const int code = contrib[c];
    const int p = code / 100, a = (code / 10) % 10, b = code % 10;
#pragma unroll
    for (int pp = 0; pp < 3; ++pp)
#pragma unroll
      for (int qq = 0; qq < 3; ++qq) {
        const int r = 3 * a + pp, cc = 3 * b + qq;
        const int idx = r >= cc ? pack_idx(r, cc) : pack_idx(cc, r);
        acc[pp * 3 + qq] += K[kidx<T>(idx, p, nel)];
      }
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) B[(size_t)q * nnzb + k] = acc[q];   // [9][nnzb]
}

// y = B x for a 3x3-block CSR matrix with blocks stored [9][nnzb]: one warp per block row, lane l
// takes blocks ptr[i] + l, ptr[i] + l + 32, ... (all loads of a warp coalesced), then a shuffle sum
template <typename T>
__global__ void __launch_bounds__(256) k_bsr_spmv(const int *__restrict__ ptr, const int *__restrict__ col,
                                                  const T *__restrict__ B, int nrow, size_t nnzb,
                                                  const T *__restrict__ x, T *__restrict__ y) {
  const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= nrow) return;
  T s0 = 0, s1 = 0, s2 = 0;
  const int kb = ptr[i], ke = ptr[i + 1];
  for (int k = kb + lane; k < ke; k += 32) {
    const int j = col[k];
    const T x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
    s0 += B[k] * x0 + B[nnzb + k] * x1 + B[2 * nnzb + k] * x2;
    s1 += B[3 * nnzb + k] * x0 + B[4 * nnzb + k] * x1 + B[5 * nnzb + k] * x2;
    s2 += B[6 * nnzb + k] * x0 + B[7 * nnzb + k] * x1 + B[8 * nnzb + k] * x2;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if (lane < 3) y[3 * (size_t)i + lane] = lane == 0 ? s0 : lane == 1 ? s1 : s2;
}

template <typename T>
int bsr_assemble(const Level &L, const T *K, T *B, cudaStream_t s) {
  k_bsr_assemble<T><<<(L.nnzb + 127) / 128, 128, 0, s>>>(K, L.nel, L.nnzb, L.bsr_cptr, L.bsr_contrib, B); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template <typename T>
int bsr_apply(const Level &L, const T *B, const T *x, T *y, cudaStream_t s) {
  k_bsr_spmv<T><<<(unsigned)(((size_t)L.nnod * 32 + 255) / 256), 256, 0, s>>>(L.bsr_ptr, L.bsr_col, B, L.nnod,
                                                                             (size_t)L.nnzb, x, y);
  count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}
template int bsr_assemble<double>(const Level &, const double *, double *, cudaStream_t);
template int bsr_assemble<float>(const Level &, const float *, float *, cudaStream_t);
template int bsr_apply<double>(const Level &, const double *, const double *, double *, cudaStream_t);
template int bsr_apply<float>(const Level &, const float *, const float *, float *, cudaStream_t);

__global__ void k_f64_to_f32(const double *a, float *b, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}
int convert_f64_f32(const double *a, float *b, size_t n, cudaStream_t s) {
  k_f64_to_f32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, b, n); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

}  // namespace m3sph
