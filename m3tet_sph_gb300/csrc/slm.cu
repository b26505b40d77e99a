// Semi-Lagrangian thermal advection on the curved shell: PC2 departure points, curved-element
// point location by neighbour walk, P2 and quasi-cubic interpolation.
//
// Reference behaviour restated (paths inside the reference project):
//   mfiles_SPH/advect3d_slm_p_sph.m:165-242 (PC2), :298-410 (predictor), :412-440 (corrector)
//   mfiles_SPH/find_pts_outside_domain_sph.m:27-98 (radial clamp)
//   mfiles_SPH/local_coords_3d_sph.m:28-147 (per-class frames, barycentric determinant ratios)
//   mfiles_SPH/local_coords_curved_3d_sph.m:36-168 (Newton on the 10-node map, X-90 frame)
//   mfiles_SPH/locate_points_interp_vars_3d_sph.m:34-207, mfiles_SPH/tsearch2_sph.m:374-404
//   mfiles_M3TET/locate_points_in_neighboring_element.m:1-158 (tolerance growth to 15e-3)
//   mfiles_M3TET/interp3d_tet.m:39-69, mfiles_M3TET/interp3d_cubic_p.m:80-382
//
// Point location contract: a point gets the element whose own-frame barycentric coordinates all
// lie in [0,1]; if several do (points on shared faces), non-isoparametric elements win, then
// the largest element id; if none does, the vertex-neighbours of the last walked element are
// searched with a tolerance grown in 1e-6 steps up to 15e-3. Every walk has a step limit.
#include <mutex>

#include "common.cuh"

namespace m3sph {

constexpr int WALK_MAX_STEPS = 512;
constexpr float WALK32_MARGIN = 1e-4f;   // FP32 barycentric margin before the FP64 walk takes over
// Point-location rule (the oracle states the same rule):
//  1. C = {e : need(e) <= TIE_BAND}, need = max(-min barycentric, max barycentric - 1) in the
//     element's own frame. Non-empty C (tsearch2_sph.m:374-404): drop isoparametric elements if a
//     non-isoparametric one is in C (:380-382); if the point is at a vertex of every remaining
//     element keep those of the first frame in the reference's pass order (X-90, original, Z-180;
//     :383-386); take the largest id (:404).
//  2. Else tolerance in 1e-6 steps up to 15e-3 (locate_points_in_neighboring_element.m): among the
//     elements of the smallest step count, the smallest last Newton step if all are isoparametric,
//     else the smallest non-isoparametric id.
constexpr double TIE_BAND = 1e-10;
constexpr double TIE_TRIGGER = 1e-7;     // closer than this to the found element's boundary: resolve
constexpr double IFACE_TRIGGER = 15e-3;  // the same for elements next to another frame or to iso elements
constexpr double GAP_STEP = 1e-6;
constexpr int GAP_QMAX = 15000;          // 15e-3 in 1e-6 steps
constexpr int MAX_CAND = 64;             // candidates within the tie band kept per point
constexpr int MAX_RING_VERTS = 96;       // vertices of the 1-ring gathered for the 2-ring search

struct SlmMesh {
  int nel, nnod, nvnod;
  const int *el2nod;     // [10][nel] original order
  const int *nbr;        // [4][nel] neighbour across the face opposite local vertex k, -1 on the boundary
  const uint8_t *cls;    // [nel]
  const double *S0;      // [3][nvnod] GCOORD_SPH of vertices
  const double *SZ;      // [3][nvnod] Z-180 frame of vertices
  const double *SX;      // [3][nnod]  X-90 frame of all nodes
  const int *v2e_ptr;    // [nvnod+1]
  const int *v2e;        // vertex -> elements
  const uint8_t *iface;  // [nel] bit k: face k has a vertex shared with an element of another frame or iso-ness
  const float *S0f, *SZf, *SXf;   // FP32 copies of S0, SZ, SX (the FP32 part of the walk)
  // start grid for walks without a guess: cells equal in cos(theta), phi and r
  const int *grid;       // [gnr][gnt][gnp] element id
  int gnt, gnp, gnr;
  double grmin, grmax;
};

__host__ __device__ inline int grid_cell(int gnt, int gnp, int gnr, double grmin, double grmax, double ct, double ph,
                                         double r) {
  const double two_pi = 6.283185307179586;
  int it = (int)((1.0 - ct) * 0.5 * gnt);
  double p = fmod(ph, two_pi);
  if (p < 0) p += two_pi;
  int ip = (int)(p / two_pi * gnp);
  int ir = (int)((r - grmin) / (grmax - grmin) * gnr);
  it = it < 0 ? 0 : (it >= gnt ? gnt - 1 : it);
  ip = ip < 0 ? 0 : (ip >= gnp ? gnp - 1 : ip);
  ir = ir < 0 ? 0 : (ir >= gnr ? gnr - 1 : ir);
  return (ir * gnt + it) * gnp + ip;
}

__device__ __forceinline__ void sph2cart_d(double th, double ph, double r, double &x, double &y, double &z) {
  double st, ct, sp, cp;
  sincos(th, &st, &ct);
  sincos(ph, &sp, &cp);
  x = r * st * cp;
  y = r * st * sp;
  z = r * ct;
}
__device__ __forceinline__ void c2s(double x, double y, double z, double &th, double &ph, double &r) {
  r = sqrt(x * x + y * y + z * z);
  th = atan2(sqrt(x * x + y * y), z);
  ph = atan2(y, x);
  if (ph < 0.0) ph += 2.0 * M_PI;
}

template <typename R> struct PointFramesT {
  R p0[3], pz[3], px[3];
};
using PointFrames = PointFramesT<double>;

__device__ __forceinline__ void point_frames(double th, double ph, double r, PointFrames &f) {
  f.p0[0] = th; f.p0[1] = ph; f.p0[2] = r;
  double x, y, z;
  sph2cart_d(th, ph, r, x, y, z);
  c2s(-x, -y, z, f.pz[0], f.pz[1], f.pz[2]);     // 180 deg about z
  c2s(x, -z, y, f.px[0], f.px[1], f.px[2]);      // 90 deg about x
}

// barycentric determinant ratio of local_coords_3d_sph.m:94-147 for vertex a (b,c,d the others)
template <typename R>
__device__ __forceinline__ R dratio(const R (&t)[4], const R (&p)[4], const R (&q)[4], int b, int c, int d, R tp, R pp,
                                    R rp, int a) {
  auto D = [&](R ta, R pa, R ra) {
    return (t[b] - ta) * (p[c] - pa) * (q[d] - ra) + (t[c] - ta) * (p[d] - pa) * (q[b] - ra) +
           (t[d] - ta) * (p[b] - pa) * (q[c] - ra) - (q[b] - ra) * (p[c] - pa) * (t[d] - ta) -
           (q[c] - ra) * (p[d] - pa) * (t[b] - ta) - (q[d] - ra) * (p[b] - pa) * (t[c] - ta);
  };
  return D(tp, pp, rp) / D(t[a], p[a], q[a]);
}

template <typename R>
__device__ __forceinline__ void lc_straight(const R (&t)[4], const R (&p)[4], const R (&q)[4], const R *pt, R *lc) {
  lc[0] = dratio<R>(t, p, q, 1, 2, 3, pt[0], pt[1], pt[2], 0);
  lc[1] = dratio<R>(t, p, q, 0, 2, 3, pt[0], pt[1], pt[2], 1);
  lc[2] = dratio<R>(t, p, q, 0, 1, 3, pt[0], pt[1], pt[2], 2);
}

// own-frame local coordinates of point f in element e from the frame coordinates S0/SZ/SX (FP64 or
// their FP32 copies); returns the Newton step size for iso elements
template <typename R>
__device__ R local_coords_t(const SlmMesh &m, const R *S0, const R *SZ, const R *SX, int e, const PointFramesT<R> &f,
                            R *lc) {
  const int cls = m.cls[e];
  R t[4], p[4], q[4];
  int v[4];
  for (int i = 0; i < 4; ++i) v[i] = m.el2nod[(size_t)i * m.nel + e];
  if (cls == M3SPH_OUT_CONE_NO_CROSS_2PI) {
    for (int i = 0; i < 4; ++i) { t[i] = S0[v[i]]; p[i] = S0[m.nvnod + v[i]]; q[i] = S0[2 * m.nvnod + v[i]]; }
    lc_straight<R>(t, p, q, f.p0, lc);
    return R(0);
  }
  if (cls == M3SPH_OUT_CONE_CROSS_2PI) {
    for (int i = 0; i < 4; ++i) { t[i] = SZ[v[i]]; p[i] = SZ[m.nvnod + v[i]]; q[i] = SZ[2 * m.nvnod + v[i]]; }
    lc_straight<R>(t, p, q, f.pz, lc);
    return R(0);
  }
  for (int i = 0; i < 4; ++i) { t[i] = SX[v[i]]; p[i] = SX[m.nnod + v[i]]; q[i] = SX[2 * m.nnod + v[i]]; }
  lc_straight<R>(t, p, q, f.px, lc);
  if (cls != M3SPH_IN_CONE_ISO) return R(0);
  // Newton on the 10-node map (local_coords_curved_3d_sph.m:45-168): up to 6 steps, tol 1e-8
  R G[3][10];
  for (int n = 0; n < 10; ++n) {
    const int nod = m.el2nod[(size_t)n * m.nel + e];
    for (int k = 0; k < 3; ++k) G[k][n] = SX[(size_t)k * m.nnod + nod];
  }
  R step = R(0);
  for (int it = 0; it < 6; ++it) {
    const R r = lc[0], s = lc[1], tt = lc[2], u = R(1) - r - s - tt;
    const R N[10] = {r * (2 * r - 1), s * (2 * s - 1), tt * (2 * tt - 1), u * (2 * u - 1), 4 * r * s,
                     4 * s * tt, 4 * tt * u, 4 * r * u, 4 * r * tt, 4 * s * u};
    const R dN[10][3] = {{4 * r - 1, 0, 0}, {0, 4 * s - 1, 0}, {0, 0, 4 * tt - 1},
                         {1 - 4 * u, 1 - 4 * u, 1 - 4 * u}, {4 * s, 4 * r, 0}, {0, 4 * tt, 4 * s},
                         {-4 * tt, -4 * tt, 4 * (u - tt)}, {4 * (u - r), -4 * r, -4 * r},
                         {4 * tt, 0, 4 * r}, {-4 * s, 4 * (u - s), -4 * s}};
    R d[3], J[3][3];
    for (int k = 0; k < 3; ++k) {
      R s0 = R(0);
      for (int n = 0; n < 10; ++n) s0 += G[k][n] * N[n];
      d[k] = f.px[k] - s0;
      for (int j = 0; j < 3; ++j) {
        R sj = R(0);
        for (int n = 0; n < 10; ++n) sj += G[k][n] * dN[n][j];
        J[k][j] = sj;
      }
    }
    if (sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) < R(1e-8)) break;
    const R det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                  J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    const R id = R(1) / det;
    const R ds0 = id * ((J[1][1] * J[2][2] - J[1][2] * J[2][1]) * d[0] + (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * d[1] +
                        (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * d[2]);
    const R ds1 = id * ((J[1][2] * J[2][0] - J[1][0] * J[2][2]) * d[0] + (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * d[1] +
                        (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * d[2]);
    const R ds2 = id * ((J[1][0] * J[2][1] - J[1][1] * J[2][0]) * d[0] + (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * d[1] +
                        (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * d[2]);
    lc[0] += ds0;
    lc[1] += ds1;
    lc[2] += ds2;
    step = fabs(ds0) + fabs(ds1) + fabs(ds2);
  }
  return step;
}
__device__ __forceinline__ double local_coords(const SlmMesh &m, int e, const PointFrames &f, double *lc) {
  return local_coords_t<double>(m, m.S0, m.SZ, m.SX, e, f, lc);
}

__device__ __forceinline__ void bary_minmax(const double *lc, double &mn, double &mx, int &argmn) {
  const double l4 = 1.0 - lc[0] - lc[1] - lc[2];
  const double b[4] = {lc[0], lc[1], lc[2], l4};
  mn = b[0];
  mx = b[0];
  argmn = 0;
  for (int k = 1; k < 4; ++k) {
    if (b[k] < mn) { mn = b[k]; argmn = k; }
    mx = fmax(mx, b[k]);
  }
}

// frame of each class in the reference's pass order: X-90 (cone classes) 0, original 1, Z-180 2
__device__ __forceinline__ int frame_rank(int cls) { return cls >= M3SPH_IN_CONE_NO_ISO ? 0 : (cls == 0 ? 1 : 2); }

// candidate flags: bit 0 isoparametric, bits 1-2 frame rank, bit 3 point at one of its vertices

// rule 1 over n candidates; *ambiguous: neither the iso drop nor the shared-vertex drop applied and
// the remaining candidates span frames (the reference's error('no good'), tsearch2_sph.m:387-392)
__device__ int tie_rule(const int *id, const uint8_t *fl, int n, int *ambiguous) {
  bool any_iso = false, any_non = false;
  for (int k = 0; k < n; ++k) {
    if (fl[k] & 1) any_iso = true; else any_non = true;
  }
  const bool drop_iso = any_iso && any_non;
  bool all_vtx = true;
  int rmin = 3, rmax = -1;
  for (int k = 0; k < n; ++k) {
    if (drop_iso && (fl[k] & 1)) continue;
    if (!(fl[k] & 8)) all_vtx = false;
    const int r = (fl[k] >> 1) & 3;
    rmin = min(rmin, r);
    rmax = max(rmax, r);
  }
  const bool vtx_drop = all_vtx && n >= 2;
  int best = -1;
  for (int k = 0; k < n; ++k) {
    if (drop_iso && (fl[k] & 1)) continue;
    if (vtx_drop && ((fl[k] >> 1) & 3) != rmin) continue;
    best = max(best, id[k]);
  }
  *ambiguous = (n >= 2 && !drop_iso && !all_vtx && rmax > rmin) ? 1 : 0;
  return best;
}

// smallest quantised tolerance and, at that tolerance, the best isoparametric (smallest Newton
// step, then smallest id) and non-isoparametric (smallest id) elements
struct GapBest {
  int q = GAP_QMAX + 1, non = -1, iso = -1;
  double iso_step = 1e300;
  __device__ void add(int e, int qe, bool is_iso, double step) {
    if (qe > GAP_QMAX) return;
    if (qe < q) { q = qe; non = -1; iso = -1; iso_step = 1e300; }
    if (qe != q) return;
    if (!is_iso) {
      if (non < 0 || e < non) non = e;
    } else if (step < iso_step || (step == iso_step && e < iso)) {
      iso = e;
      iso_step = step;
    }
  }
  __device__ int pick() const { return non >= 0 ? non : iso; }
};

// one element of a ring or of the brute-force set: a candidate (within the tie band, appended to the
// warp's shared list; the rule does not depend on the order) or a gap contender
// an FP32 pre-filter skips the FP64 evaluation of elements the point is far from: FP32 barycentrics
// err by ~1e-5 here, so an element whose FP32 need exceeds the largest gap tolerance by PRE_MARGIN
// can be neither a tie candidate nor a gap contender in FP64
constexpr float PRE_MARGIN = 1e-3f;
__device__ __forceinline__ PointFramesT<float> frames_f32(const PointFrames &f) {
  PointFramesT<float> g;
  for (int k = 0; k < 3; ++k) {
    g.p0[k] = (float)f.p0[k];
    g.pz[k] = (float)f.pz[k];
    g.px[k] = (float)f.px[k];
  }
  return g;
}
__device__ __forceinline__ void eval_shared(const SlmMesh &m, int e, const PointFrames &f,
                                            const PointFramesT<float> &g, int *ids, uint8_t *fl, int *n,
                                            GapBest &G) {
  {
    float l[3];
    local_coords_t<float>(m, m.S0f, m.SZf, m.SXf, e, g, l);
    const float l4 = 1.0f - l[0] - l[1] - l[2];
    const float nf = fmaxf(fmaxf(-fminf(fminf(l[0], l[1]), fminf(l[2], l4)), 0.0f),
                           fmaxf(fmaxf(l[0], l[1]), fmaxf(l[2], l4)) - 1.0f);
    if (nf > (float)((GAP_QMAX + 1) * GAP_STEP) + PRE_MARGIN) return;   // NaN falls through to FP64
  }
  double lc[3], mn, mx;
  int am;
  const double step = local_coords(m, e, f, lc);
  bary_minmax(lc, mn, mx, am);
  const double need = fmax(-mn, mx - 1.0);
  const int cls = m.cls[e];
  const bool iso = cls == M3SPH_IN_CONE_ISO;
  if (need <= TIE_BAND) {
    const int slot = atomicAdd(n, 1);
    if (slot < MAX_CAND) {
      ids[slot] = e;
      fl[slot] = (uint8_t)((iso ? 1 : 0) | (frame_rank(cls) << 1) | (mx >= 1.0 - TIE_BAND ? 8 : 0));
    }
  } else if (need <= (GAP_QMAX + 1) * GAP_STEP) {
    G.add(e, (int)ceil(need / GAP_STEP - 1e-9), iso, step);
  }
}

// warp reduction of the gap choice: the smallest step count, then at that count the smallest
// non-isoparametric id and the isoparametric element of the smallest Newton step (then id)
__device__ __forceinline__ int gap_reduce(const GapBest &G, int &q) {
  q = G.q;
  for (int o = 16; o > 0; o >>= 1) q = min(q, __shfl_xor_sync(0xffffffffu, q, o));
  int non = (G.q == q) ? G.non : -1;
  int iso_e = (G.q == q) ? G.iso : -1;
  double iso_s = (G.q == q) ? G.iso_step : 1e300;
  for (int o = 16; o > 0; o >>= 1) {
    const int on = __shfl_xor_sync(0xffffffffu, non, o);
    const int oi = __shfl_xor_sync(0xffffffffu, iso_e, o);
    const double os = __shfl_xor_sync(0xffffffffu, iso_s, o);
    if (on >= 0 && (non < 0 || on < non)) non = on;
    if (oi >= 0 && (iso_e < 0 || os < iso_s || (os == iso_s && oi < iso_e))) { iso_e = oi; iso_s = os; }
  }
  return non >= 0 ? non : iso_e;
}

// rule 1 / rule 2 on the warp's shared candidate list (duplicates removed first), by lane 0;
// writes the point's element, local coordinates and status (base_status: 1 placed by a ring, 16 by
// the brute force)
__device__ void finish_point(const SlmMesh &m, const PointFrames &f, int i, int npt, int *ids, uint8_t *fl, int nc,
                             int gap_e, int q, int base_status, int adjust, int *els, double *lc_out, uint8_t *status) {
  int kind = nc > MAX_CAND ? 64 : 0;
  nc = min(nc, MAX_CAND);
  int u = 0;
  for (int a = 0; a < nc; ++a) {
    bool dup = false;
    for (int b = 0; b < u; ++b) dup |= ids[b] == ids[a];
    if (!dup) {
      ids[u] = ids[a];
      fl[u] = fl[a];
      ++u;
    }
  }
  int e = -1;
  if (u > 0) {
    int amb = 0;
    e = tie_rule(ids, fl, u, &amb);
    kind |= base_status | (u >= 2 ? 2 : 0) | (amb ? 32 : 0);
  } else if (q <= GAP_QMAX && gap_e >= 0) {
    e = gap_e;
    kind |= (base_status & 16) | 4;
  }
  if (e < 0) {
    status[i] = (uint8_t)(8 | (kind & 64));
    return;
  }
  double lc[3];
  local_coords(m, e, f, lc);
  if (adjust) {   // adjust_local_coords (locate_points_interp_vars_3d_sph.m:180-198)
    for (int k = 0; k < 3; ++k) lc[k] = fmin(fmax(lc[k], 0.0), 1.0);
    const double sm = lc[0] + lc[1] + lc[2];
    if (sm > 1.0) for (int k = 0; k < 3; ++k) lc[k] /= sm;
  }
  els[i] = e;
  lc_out[i] = lc[0];
  lc_out[npt + i] = lc[1];
  lc_out[2 * npt + i] = lc[2];
  status[i] = (uint8_t)kind;
}

// Rules 1-2 for the points k_locate listed: one warp per point over the elements sharing a vertex
// with the walk's element (placed points) or with any of those (points the walk could not place).
constexpr int RING_WARPS = 8;
constexpr int RING_VTAB = 256;   // open-addressing table of the 1-ring's vertices (2-ring search)
__global__ void __launch_bounds__(RING_WARPS * 32) k_resolve_ring(SlmMesh m, const double *__restrict__ P, int npt,
                                                                 const int *__restrict__ todo, int ntodo,
                                                                 int *__restrict__ els, double *__restrict__ lc_out,
                                                                 uint8_t *__restrict__ status, int adjust) {
  __shared__ int s_id[RING_WARPS][MAX_CAND];
  __shared__ uint8_t s_fl[RING_WARPS][MAX_CAND];
  __shared__ int s_n[RING_WARPS];
  __shared__ int s_vt[RING_WARPS][RING_VTAB];
  const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * RING_WARPS + wl;
  if (w >= ntodo) return;
  const int i = todo[w];
  const int e0 = els[i];
  const int depth = (status[i] & 1) ? 1 : 2;
  if (lane == 0) s_n[wl] = 0;
  PointFrames f;
  point_frames(P[i], P[npt + i], P[2 * npt + i], f);
  const PointFramesT<float> g32 = frames_f32(f);
  int v0[4], len[4];
  for (int k = 0; k < 4; ++k) {
    v0[k] = m.el2nod[(size_t)k * m.nel + e0];
    len[k] = m.v2e_ptr[v0[k] + 1] - m.v2e_ptr[v0[k]];
  }
  const int tot = len[0] + len[1] + len[2] + len[3];
  GapBest G;
  __syncwarp();
  if (depth == 1) {
    // an element of the 1-ring is visited once: from the first of e0's vertices it contains
    for (int t = lane; t < tot; t += 32) {
      int k = 0, o = t;
      while (o >= len[k]) o -= len[k++];
      const int e1 = m.v2e[m.v2e_ptr[v0[k]] + o];
      bool dup = false;
      for (int j = 0; j < 4; ++j) {
        const int v = m.el2nod[(size_t)j * m.nel + e1];
        for (int kk = 0; kk < k; ++kk) dup |= v == v0[kk];
      }
      if (!dup) eval_shared(m, e1, f, g32, s_id[wl], s_fl[wl], &s_n[wl], G);
    }
  } else {
    // vertices of the 1-ring, deduplicated in a shared hash table (-1 = empty)
    for (int t = lane; t < RING_VTAB; t += 32) s_vt[wl][t] = -1;
    __syncwarp();
    for (int t = lane; t < tot; t += 32) {
      int k = 0, o = t;
      while (o >= len[k]) o -= len[k++];
      const int e1 = m.v2e[m.v2e_ptr[v0[k]] + o];
      for (int j = 0; j < 4; ++j) {
        const int v = m.el2nod[(size_t)j * m.nel + e1];
        int h = (int)(((unsigned)v * 2654435761u) % RING_VTAB);
        for (int probe = 0; probe < RING_VTAB; ++probe) {
          const int old = atomicCAS(&s_vt[wl][h], -1, v);
          if (old == -1 || old == v) break;
          h = (h + 1) % RING_VTAB;
        }
      }
    }
    __syncwarp();
    // an element of the 2-ring is visited once: from the vertex in the table's lowest slot
    for (int slot = 0; slot < RING_VTAB; ++slot) {
      const int v = s_vt[wl][slot];
      if (v < 0) continue;
      for (int k = m.v2e_ptr[v] + lane; k < m.v2e_ptr[v + 1]; k += 32) {
        const int e1 = m.v2e[k];
        bool dup = false;
        for (int j = 0; j < 4 && !dup; ++j) {
          const int vj = m.el2nod[(size_t)j * m.nel + e1];
          if (vj == v) continue;
          int h = (int)(((unsigned)vj * 2654435761u) % RING_VTAB);
          for (int probe = 0; probe < RING_VTAB; ++probe) {
            const int tv = s_vt[wl][h];
            if (tv < 0) break;
            if (tv == vj) {
              dup = h < slot;
              break;
            }
            h = (h + 1) % RING_VTAB;
          }
        }
        if (!dup) eval_shared(m, e1, f, g32, s_id[wl], s_fl[wl], &s_n[wl], G);
      }
    }
  }
  __syncwarp();
  int q;
  const int gap_e = gap_reduce(G, q);
  if (lane != 0) return;
  finish_point(m, f, i, npt, s_id[wl], s_fl[wl], s_n[wl], gap_e, q, 1, adjust, els, lc_out, status);
}

// one thread per point: walk from the guess to the containing element; points that may tie and
// points the walk could not place are listed for k_resolve_ring.
// status bits: 1 placed, 2 tie, 4 gap (tolerance), 8 not placed yet (brute force next), 16 placed by
// brute force, 32 ambiguous for the reference, 64 candidate list overflow, 128 ring resolution pending
__global__ void k_locate(SlmMesh m, const double *__restrict__ P, int npt, const int *__restrict__ guess,
                         const int *__restrict__ node_guess, int *__restrict__ els, double *__restrict__ lc_out,
                         uint8_t *__restrict__ status, int adjust, int *__restrict__ ring_todo,
                         int *__restrict__ ring_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npt) return;
  PointFrames f;
  point_frames(P[i], P[npt + i], P[2 * npt + i], f);
  int e = guess ? guess[i] : -1;
  if ((e < 0 || e >= m.nel) && node_guess) e = node_guess[i];
  if ((e < 0 || e >= m.nel) && m.grid)
    e = m.grid[grid_cell(m.gnt, m.gnp, m.gnr, m.grmin, m.grmax, cos(P[i]), P[npt + i], P[2 * npt + i])];
  if (e < 0 || e >= m.nel) e = 0;
  int prev = -1, found = -1;
  // walk in FP32 (the FP64 pipe issues at 1/64 of the FP32 rate) until the FP32 barycentrics place
  // the point inside within a margin well above their rounding; the FP64 walk below then decides
  int steps32 = 0;
  {
    PointFramesT<float> g;
    for (int k = 0; k < 3; ++k) {
      g.p0[k] = (float)f.p0[k];
      g.pz[k] = (float)f.pz[k];
      g.px[k] = (float)f.px[k];
    }
    for (; steps32 < WALK_MAX_STEPS; ++steps32) {
      float l[3];
      local_coords_t<float>(m, m.S0f, m.SZf, m.SXf, e, g, l);
      const float b[4] = {l[0], l[1], l[2], 1.0f - l[0] - l[1] - l[2]};
      int am = 0;
      float mn = b[0];
      for (int k = 1; k < 4; ++k)
        if (b[k] < mn) { mn = b[k]; am = k; }
      if (!(mn < -WALK32_MARGIN)) break;   // inside (or NaN): hand over to FP64
      int nb = m.nbr[(size_t)am * m.nel + e];
      if (nb == prev || nb < 0) {
        int alt = -1;
        float amin = 1e30f;
        for (int k = 0; k < 4; ++k) {
          if (k == am || !(b[k] < 0.0f)) continue;
          const int c = m.nbr[(size_t)k * m.nel + e];
          if (c >= 0 && c != prev && b[k] < amin) { amin = b[k]; alt = c; }
        }
        if (alt < 0) break;
        nb = alt;
      }
      prev = e;
      e = nb;
    }
  }
  prev = -1;
  double lc[3] = {0, 0, 0};
  uint8_t st = 0;
  for (int step = 0; step < WALK_MAX_STEPS; ++step) {
    double mn, mx;
    int am;
    local_coords(m, e, f, lc);
    bary_minmax(lc, mn, mx, am);
    if (mn >= 0.0 && mx <= 1.0) {
      found = e;
      break;
    }
    // leave through the face opposite the most negative barycentric; avoid stepping straight back
    int nb = m.nbr[(size_t)am * m.nel + e];
    if (nb == prev || nb < 0) {
      const double b[4] = {lc[0], lc[1], lc[2], 1.0 - lc[0] - lc[1] - lc[2]};
      int alt = -1;
      double amin = 1e300;
      for (int k = 0; k < 4; ++k) {
        if (k == am || b[k] >= 0.0) continue;
        const int c = m.nbr[(size_t)k * m.nel + e];
        if (c >= 0 && c != prev && b[k] < amin) { amin = b[k]; alt = c; }
      }
      if (alt < 0) break;
      nb = alt;
    }
    prev = e;
    e = nb;
  }
  if (found >= 0) {
    st = 1;
    // the point may tie with other elements (within the band of a face, edge or vertex, or inside a
    // face that borders another frame or an isoparametric element, where the own-frame shapes
    // overlap): the ring is resolved by k_resolve_ring, one warp per such point
    const double b[4] = {lc[0], lc[1], lc[2], 1.0 - lc[0] - lc[1] - lc[2]};
    bool trig = false;
    const uint8_t fmask = m.iface[found];
    for (int k = 0; k < 4; ++k)
      trig |= b[k] < TIE_TRIGGER || b[k] > 1.0 - TIE_TRIGGER || (((fmask >> k) & 1) && b[k] < IFACE_TRIGGER);
    if (trig) {
      st = 1 | 128;
      ring_todo[atomicAdd(ring_count, 1)] = i;
    }
  } else {
    found = e;                   // the walk's last element: centre of the 2-ring search
    st = 128;
    ring_todo[atomicAdd(ring_count, 1)] = i;
  }
  if (st & 128) {                // resolved later from the centre element stored in els
    els[i] = found;
    status[i] = st;
    return;
  }
  els[i] = found;
  lc_out[i] = lc[0];
  lc_out[npt + i] = lc[1];
  lc_out[2 * npt + i] = lc[2];
  status[i] = st;
}

// brute force over all elements for points no ring could place (status 8): one warp per point, the
// same rule over every element
constexpr int BRUTE_WARPS = 8;
__global__ void __launch_bounds__(BRUTE_WARPS * 32) k_locate_brute(SlmMesh m, const double *__restrict__ P, int npt,
                                                                  const int *__restrict__ todo, int ntodo,
                                                                  int *__restrict__ els, double *__restrict__ lc_out,
                                                                  uint8_t *status, int adjust) {
  __shared__ int s_id[BRUTE_WARPS][MAX_CAND];
  __shared__ uint8_t s_fl[BRUTE_WARPS][MAX_CAND];
  __shared__ int s_n[BRUTE_WARPS];
  const int wl = threadIdx.x >> 5;
  const int w = blockIdx.x * BRUTE_WARPS + wl;
  const int lane = threadIdx.x & 31;
  if (w >= ntodo) return;
  if (lane == 0) s_n[wl] = 0;
  __syncwarp();
  const int i = todo[w];
  PointFrames f;
  point_frames(P[i], P[npt + i], P[2 * npt + i], f);
  GapBest G;
  const PointFramesT<float> g32 = frames_f32(f);
  for (int e = lane; e < m.nel; e += 32) eval_shared(m, e, f, g32, s_id[wl], s_fl[wl], &s_n[wl], G);
  __syncwarp();
  int q;
  const int gap_e = gap_reduce(G, q);
  if (lane != 0) return;
  finish_point(m, f, i, npt, s_id[wl], s_fl[wl], s_n[wl], gap_e, q, 16, adjust, els, lc_out, status);
}

// P2 interpolation (interp3d_tet.m:39-69): V is [nvar][nnod], out [nvar][npt]
__global__ void k_interp_p2(SlmMesh m, const int *__restrict__ els, const double *__restrict__ lc, int npt,
                            const double *__restrict__ V, int nvar, int monotonic, double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npt) return;
  const int e = els[i];
  if (e < 0 || e >= m.nel) {
    for (int k = 0; k < nvar; ++k) out[(size_t)k * npt + i] = nan("");
    return;
  }
  const double r = lc[i], s = lc[npt + i], t = lc[2 * npt + i], u = 1.0 - r - s - t;
  const double N[10] = {r * (2 * r - 1), s * (2 * s - 1), t * (2 * t - 1), u * (2 * u - 1), 4 * r * s,
                        4 * s * t, 4 * t * u, 4 * r * u, 4 * r * t, 4 * s * u};
  int nod[10];
  for (int n = 0; n < 10; ++n) nod[n] = m.el2nod[(size_t)n * m.nel + e];
  for (int k = 0; k < nvar; ++k) {
    const double *Vk = V + (size_t)k * m.nnod;
    double v = 0.0, lo = 1e300, hi = -1e300;
    for (int n = 0; n < 10; ++n) {
      const double x = Vk[nod[n]];
      v += N[n] * x;
      lo = fmin(lo, x);
      hi = fmax(hi, x);
    }
    if (monotonic) v = fmin(fmax(v, lo), hi);
    out[(size_t)k * npt + i] = v;
  }
}

// quasi-cubic: element P1 gradients of vertex values and distance weights, per element (original
// ids); the nodal sums are gathered per colour of the Stokes colouring (atomic-free)
__global__ void k_cubic_elgrad(SlmMesh m, const double *__restrict__ X, const double *__restrict__ B,
                               int method_wght, double *__restrict__ gel, double *__restrict__ wel) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nel) return;
  double x[4], y[4], z[4], b[4];
  for (int i = 0; i < 4; ++i) {
    const int v = m.el2nod[(size_t)i * m.nel + e];
    x[i] = X[v]; y[i] = X[m.nnod + v]; z[i] = X[2 * m.nnod + v];
    b[i] = B[v];
  }
  // gradient of the linear interpolant: solve [x_i - x_4] g = b_i - b_4
  const double a00 = x[0] - x[3], a01 = y[0] - y[3], a02 = z[0] - z[3];
  const double a10 = x[1] - x[3], a11 = y[1] - y[3], a12 = z[1] - z[3];
  const double a20 = x[2] - x[3], a21 = y[2] - y[3], a22 = z[2] - z[3];
  const double r0 = b[0] - b[3], r1 = b[1] - b[3], r2 = b[2] - b[3];
  const double det = a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) + a02 * (a10 * a21 - a11 * a20);
  const double id = 1.0 / det;
  const double gx = id * ((a11 * a22 - a12 * a21) * r0 + (a02 * a21 - a01 * a22) * r1 + (a01 * a12 - a02 * a11) * r2);
  const double gy = id * ((a12 * a20 - a10 * a22) * r0 + (a00 * a22 - a02 * a20) * r1 + (a02 * a10 - a00 * a12) * r2);
  const double gz = id * ((a10 * a21 - a11 * a20) * r0 + (a01 * a20 - a00 * a21) * r1 + (a00 * a11 - a01 * a10) * r2);
  gel[e] = gx; gel[m.nel + e] = gy; gel[2 * (size_t)m.nel + e] = gz;
  const double cx = 0.25 * (x[0] + x[1] + x[2] + x[3]), cy = 0.25 * (y[0] + y[1] + y[2] + y[3]),
               cz = 0.25 * (z[0] + z[1] + z[2] + z[3]);
  for (int i = 0; i < 4; ++i) {
    double w = 1.0;
    if (method_wght) w = 1.0 / sqrt((x[i] - cx) * (x[i] - cx) + (y[i] - cy) * (y[i] - cy) + (z[i] - cz) * (z[i] - cz));
    wel[(size_t)i * m.nel + e] = w;
  }
}
// per colour of the Stokes level-0 colouring (stored order -> original ids via perm)
__global__ void k_cubic_scatter(const int *__restrict__ perm, int nel, int eb, int ee, const int *__restrict__ el2nod_orig,
                                const double *__restrict__ gel, const double *__restrict__ wel, double *__restrict__ gn,
                                double *__restrict__ wn, int nvnod) {
  const int p = eb + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ee) return;
  const int e = perm[p];
  for (int i = 0; i < 4; ++i) {
    const int v = el2nod_orig[(size_t)i * nel + e];
    const double w = wel[(size_t)i * nel + e];
    gn[v] += w * gel[e];
    gn[nvnod + v] += w * gel[nel + e];
    gn[2 * (size_t)nvnod + v] += w * gel[2 * (size_t)nel + e];
    wn[v] += w;
  }
}

__global__ void k_cubic_interp(SlmMesh m, const double *__restrict__ X, const int *__restrict__ els,
                               const double *__restrict__ lc, int npt, const double *__restrict__ B,
                               const double *__restrict__ gn, const double *__restrict__ wn,
                               const double *__restrict__ gel, int monotonic, double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npt) return;
  const int e = els[i];
  if (e < 0 || e >= m.nel) {
    out[i] = nan("");
    return;
  }
  const double r = lc[i], s = lc[npt + i], t = lc[2 * npt + i], u = 1.0 - r - s - t;
  const double q2 = 1.4142135623730951;   // sqrt(2)
  const double N[16] = {r, s, t, u, q2 * r * s, q2 * s * t, t * u, r * u, q2 * r * t, s * u,
                        q2 * s * r * (s - r), q2 * s * t * (t - s), t * u * (u - t), r * u * (u - r),
                        q2 * r * t * (t - r), s * u * (u - s)};
  int v[4];
  double x[4], y[4], z[4], b[4], dB[4][3];
  for (int k = 0; k < 4; ++k) {
    v[k] = m.el2nod[(size_t)k * m.nel + e];
    x[k] = X[v[k]]; y[k] = X[m.nnod + v[k]]; z[k] = X[2 * m.nnod + v[k]];
    b[k] = B[v[k]];
    const double wk = wn[v[k]];
    for (int c = 0; c < 3; ++c) dB[k][c] = gn[(size_t)c * m.nvnod + v[k]] / wk - gel[(size_t)c * m.nel + e];
  }
  double sr[4], ss[4], st[4];
  for (int k = 0; k < 4; ++k) {
    sr[k] = (x[0] - x[3]) * dB[k][0] + (y[0] - y[3]) * dB[k][1] + (z[0] - z[3]) * dB[k][2];
    ss[k] = (x[1] - x[3]) * dB[k][0] + (y[1] - y[3]) * dB[k][1] + (z[1] - z[3]) * dB[k][2];
    st[k] = (x[2] - x[3]) * dB[k][0] + (y[2] - y[3]) * dB[k][1] + (z[2] - z[3]) * dB[k][2];
  }
  const double h = 0.7071067811865476;    // sqrt(1/2)
  const double q1n2 = h * sr[1] - h * ss[1], q1n1 = h * sr[0] - h * ss[0];
  const double q2n3 = h * ss[2] - h * st[2], q2n2 = h * ss[1] - h * st[1];
  const double q5n3 = h * sr[2] - h * st[2], q5n1 = h * sr[0] - h * st[0];
  const double info[12] = {(q1n2 - q1n1) / 2, (q2n3 - q2n2) / 2, (st[3] - st[2]) / 2, (sr[3] - sr[0]) / 2,
                           (q5n3 - q5n1) / 2, (ss[3] - ss[1]) / 2, (q1n2 + q1n1) / 2, (q2n3 + q2n2) / 2,
                           (st[3] + st[2]) / 2, (sr[3] + sr[0]) / 2, (q5n3 + q5n1) / 2, (ss[3] + ss[1]) / 2};
  double val = N[0] * b[0] + N[1] * b[1] + N[2] * b[2] + N[3] * b[3];
  for (int k = 0; k < 12; ++k) val += N[4 + k] * info[k];
  if (monotonic) {
    const double lo = fmin(fmin(b[0], b[1]), fmin(b[2], b[3])), hi = fmax(fmax(b[0], b[1]), fmax(b[2], b[3]));
    val = fmin(fmax(val, lo), hi);
  }
  out[i] = val;
}

// PC2 predictor (advect3d_slm_p_sph.m:298-410): U [3][nnod] Cartesian; writes P (3,npt)
// (theta,phi,r), the unit perpendicular direction and the predicted unit radius vector.
__global__ void k_predictor(const double *__restrict__ X, const double *__restrict__ S, int nnod,
                            const double *__restrict__ U, double dt, double r_cmb, double r_surf,
                            double *__restrict__ P, double *__restrict__ upu, double *__restrict__ rpu) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnod) return;
  const double rr = S[2 * nnod + i];
  const double x[3] = {X[i], X[nnod + i], X[2 * nnod + i]};
  const double u[3] = {U[i], U[nnod + i], U[2 * nnod + i]};
  double ru[3] = {x[0] / rr, x[1] / rr, x[2] / rr};
  const double nru2 = ru[0] * ru[0] + ru[1] * ru[1] + ru[2] * ru[2];
  const double ud = u[0] * ru[0] + u[1] * ru[1] + u[2] * ru[2];
  double upar[3], uperp[3];
  for (int k = 0; k < 3; ++k) {
    upar[k] = ud * ru[k] / nru2;
    uperp[k] = u[k] - upar[k];
  }
  const double np = sqrt(uperp[0] * uperp[0] + uperp[1] * uperp[1] + uperp[2] * uperp[2]);
  double e[3];
  for (int k = 0; k < 3; ++k) e[k] = np > 0.0 ? uperp[k] / np : 0.0;
  const double lpar = sqrt(upar[0] * upar[0] + upar[1] * upar[1] + upar[2] * upar[2]) * 0.5 * dt;
  const double lperp = np * 0.5 * dt;
  const double lprime = rr * tan(lperp / rr);
  double rp[3];
  for (int k = 0; k < 3; ++k) rp[k] = x[k] - e[k] * lprime;
  const double nrp = sqrt(rp[0] * rp[0] + rp[1] * rp[1] + rp[2] * rp[2]);
  const double rad = fabs(rr - lpar);
  double th, ph, r;
  c2s(rp[0] / nrp * rad, rp[1] / nrp * rad, rp[2] / nrp * rad, th, ph, r);
  const double rtol = 1e-12 * (r_surf - r_cmb);
  if (r <= r_cmb + rtol) r = r_cmb + rtol;
  if (r >= r_surf - rtol) r = r_surf - rtol;
  P[i] = th; P[nnod + i] = ph; P[2 * nnod + i] = r;
  for (int k = 0; k < 3; ++k) {
    upu[(size_t)k * nnod + i] = e[k];
    rpu[(size_t)k * nnod + i] = rp[k] / nrp;
  }
}
// PC2 corrector (advect3d_slm_p_sph.m:412-440): Ubt [3][nnod] velocity at predictor points
__global__ void k_corrector(const double *__restrict__ X, const double *__restrict__ S, int nnod,
                            const double *__restrict__ Ubt, const double *__restrict__ upu,
                            const double *__restrict__ rpu, double dt, double r_cmb, double r_surf,
                            double *__restrict__ P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnod) return;
  const double rr = S[2 * nnod + i];
  const double x[3] = {X[i], X[nnod + i], X[2 * nnod + i]};
  const double u[3] = {Ubt[i], Ubt[nnod + i], Ubt[2 * nnod + i]};
  const double q[3] = {rpu[i], rpu[nnod + i], rpu[2 * nnod + i]};
  const double e[3] = {upu[i], upu[nnod + i], upu[2 * nnod + i]};
  const double nq2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
  const double ud = u[0] * q[0] + u[1] * q[1] + u[2] * q[2];
  double upar[3], uperp[3];
  for (int k = 0; k < 3; ++k) {
    upar[k] = ud * q[k] / nq2;
    uperp[k] = u[k] - upar[k];
  }
  const double lpar = sqrt(upar[0] * upar[0] + upar[1] * upar[1] + upar[2] * upar[2]) * dt;
  const double lperp = sqrt(uperp[0] * uperp[0] + uperp[1] * uperp[1] + uperp[2] * uperp[2]) * dt;
  const double lprime = rr * tan(lperp / rr);
  double rp[3];
  for (int k = 0; k < 3; ++k) rp[k] = x[k] - e[k] * lprime;
  const double nrp = sqrt(rp[0] * rp[0] + rp[1] * rp[1] + rp[2] * rp[2]);
  const double rad = fabs(rr - lpar);
  double th, ph, r;
  c2s(rp[0] / nrp * rad, rp[1] / nrp * rad, rp[2] / nrp * rad, th, ph, r);
  const double rtol = 1e-12 * (r_surf - r_cmb);
  if (r <= r_cmb + rtol) r = r_cmb + rtol;
  if (r >= r_surf - rtol) r = r_surf - rtol;
  P[i] = th; P[nnod + i] = ph; P[2 * nnod + i] = r;
}

// RK4 backtracking (no working counterpart in the reference: advect3d_slm_p_sph.m:103-104 stops
// with 'RK4 is not working for spherical coordinates'). Each substep of length h integrates
// dx/dt = U(x) backwards in Cartesian coordinates with the classical RK4 weights; every stage
// point is moved radially into [r_cmb + tol, r_surf - tol] (find_pts_outside_domain_sph.m rule)
// before it is located and U is interpolated there.
__global__ void k_rk_point(const double *__restrict__ Xc, const double *__restrict__ k, int n, double c, double r_cmb,
                           double r_surf, double *__restrict__ P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = Xc[i] - c * k[i], y = Xc[n + i] - c * k[n + i], z = Xc[2 * n + i] - c * k[2 * n + i];
  double th, ph, r;
  c2s(x, y, z, th, ph, r);
  const double rtol = 1e-12 * (r_surf - r_cmb);
  if (r <= r_cmb + rtol) r = r_cmb + rtol;
  if (r >= r_surf - rtol) r = r_surf - rtol;
  P[i] = th; P[n + i] = ph; P[2 * n + i] = r;
}
// acc = (first ? 0 : acc) + w * k
__global__ void k_rk_accum(double *__restrict__ acc, const double *__restrict__ k, int n3, double w, int first) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  acc[i] = (first ? 0.0 : acc[i]) + w * k[i];
}
// Xc -= h/6 acc, radius clamped
__global__ void k_rk_update(double *__restrict__ Xc, const double *__restrict__ acc, int n, double h, double r_cmb,
                            double r_surf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x = Xc[i] - h / 6.0 * acc[i], y = Xc[n + i] - h / 6.0 * acc[n + i], z = Xc[2 * n + i] - h / 6.0 * acc[2 * n + i];
  const double r = sqrt(x * x + y * y + z * z);
  const double rtol = 1e-12 * (r_surf - r_cmb);
  const double rc = fmin(fmax(r, r_cmb + rtol), r_surf - rtol);
  const double f = rc / r;
  Xc[i] = x * f; Xc[n + i] = y * f; Xc[2 * n + i] = z * f;
}
__global__ void k_cart_to_sph(const double *__restrict__ Xc, int n, double *__restrict__ P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double th, ph, r;
  c2s(Xc[i], Xc[n + i], Xc[2 * n + i], th, ph, r);
  P[i] = th; P[n + i] = ph; P[2 * n + i] = r;
}

// ======================================================================================
// host side
// ======================================================================================
struct SlmState {
  bool built = false;
  int *el2nod = nullptr, *nbr = nullptr, *v2e_ptr = nullptr, *v2e = nullptr, *node_guess = nullptr, *grid = nullptr;
  float *S0f = nullptr, *SZf = nullptr, *SXf = nullptr;
  uint8_t *cls = nullptr, *iface = nullptr;
  int *ring_count = nullptr;          // [16]: 0 points listed for k_resolve_ring, 1 for the brute force,
                                      // 2.. status counts (k_status_counts)
  double *S0 = nullptr, *SZ = nullptr, *SX = nullptr;
  // work
  double *P = nullptr, *lc = nullptr, *V = nullptr, *out = nullptr, *upu = nullptr, *rpu = nullptr, *U = nullptr;
  double *gel = nullptr, *wel = nullptr, *gn = nullptr, *wn = nullptr;
  double *Xc = nullptr, *kk = nullptr, *acc = nullptr;   // RK4 point, stage slope, weighted sum
  int *els = nullptr, *guess = nullptr, *todo = nullptr;
  uint8_t *status = nullptr;
  size_t cap = 0;
  SlmMesh view{};
};

}  // namespace m3sph

namespace m3sph {

template <typename T>
static int sl_alloc(T **p, size_t n) {
  *p = nullptr;
  M3_CUDA(cudaMalloc((void **)p, sizeof(T) * (n ? n : 1)));
  return M3SPH_OK;
}
template <typename T>
static int sl_upload(T **p, const T *h, size_t n, cudaStream_t s) {
  int st = sl_alloc(p, n);
  if (st) return st;
  M3_CUDA(cudaMemcpyAsync(*p, h, sizeof(T) * n, cudaMemcpyHostToDevice, s));
  return M3SPH_OK;
}

static int noalloc_prepare(int device);

// face neighbours, vertex->element adjacency, per-frame node coordinates (set-up, host + upload)
int slm_build(m3sph_mesh *M, const m3sph_level &f0) {
  SlmState *S = new SlmState();
  M->slm = S;
  M->slm_free = [](void *p) {
    SlmState *S = reinterpret_cast<SlmState *>(p);
    for (void *q : {(void *)S->el2nod, (void *)S->nbr, (void *)S->v2e_ptr, (void *)S->v2e, (void *)S->node_guess,
                    (void *)S->cls, (void *)S->S0, (void *)S->SZ, (void *)S->SX, (void *)S->P, (void *)S->lc,
                    (void *)S->V, (void *)S->out, (void *)S->upu, (void *)S->rpu, (void *)S->U, (void *)S->gel,
                    (void *)S->wel, (void *)S->gn, (void *)S->wn, (void *)S->Xc, (void *)S->kk, (void *)S->acc,
                    (void *)S->els, (void *)S->guess,
                    (void *)S->todo, (void *)S->status, (void *)S->grid, (void *)S->S0f, (void *)S->SZf,
                    (void *)S->SXf, (void *)S->iface, (void *)S->ring_count})
      if (q) cudaFree(q);
    delete S;
  };
  cudaStream_t s = M->stream;
  const int nel = f0.nel, nnod = f0.nnod, nv = f0.nvnod;
  const std::vector<int> &el = M->lev[0].h_el2nod_orig;   // [nel][10]
  std::vector<int> soa((size_t)nel * 10);
  for (int e = 0; e < nel; ++e)
    for (int n = 0; n < 10; ++n) soa[(size_t)n * nel + e] = el[(size_t)e * 10 + n];
  // face neighbours: face k is opposite local vertex k
  struct Face { uint64_t key; int c; int ek; };
  std::vector<Face> faces((size_t)nel * 4);
  for (int e = 0; e < nel; ++e)
    for (int k = 0; k < 4; ++k) {
      int v[3], j = 0;
      for (int i = 0; i < 4; ++i)
        if (i != k) v[j++] = el[(size_t)e * 10 + i];
      std::sort(v, v + 3);
      faces[(size_t)e * 4 + k] = {(uint64_t)v[0] * (uint64_t)nv + (uint64_t)v[1], v[2], e * 4 + k};
    }
  std::sort(faces.begin(), faces.end(), [](const Face &a, const Face &b) {
    return a.key < b.key || (a.key == b.key && (a.c < b.c || (a.c == b.c && a.ek < b.ek)));
  });
  std::vector<int> nbr((size_t)nel * 4, -1);
  for (size_t i = 0; i + 1 < faces.size(); ++i)
    if (faces[i].key == faces[i + 1].key && faces[i].c == faces[i + 1].c) {
      const int a = faces[i].ek, b = faces[i + 1].ek;
      nbr[(size_t)(a % 4) * nel + a / 4] = b / 4;
      nbr[(size_t)(b % 4) * nel + b / 4] = a / 4;
      ++i;
    }
  // vertex -> elements
  std::vector<int> ptr(nv + 1, 0), adj((size_t)nel * 4);
  for (int e = 0; e < nel; ++e)
    for (int i = 0; i < 4; ++i) ptr[el[(size_t)e * 10 + i] + 1]++;
  for (int v = 0; v < nv; ++v) ptr[v + 1] += ptr[v];
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int e = 0; e < nel; ++e)
    for (int i = 0; i < 4; ++i) adj[fill[el[(size_t)e * 10 + i]]++] = e;
  // first element listing each node (guess_elems, locate_points_interp_vars_3d_sph.m:203-207)
  std::vector<int> first(nnod, -1);
  for (size_t i = 0; i < (size_t)nel * 10; ++i)
    if (first[el[i]] < 0) first[el[i]] = (int)(i / 10);
  // frames
  std::vector<double> S0(3 * (size_t)nv), SZ(3 * (size_t)nv), SX(3 * (size_t)nnod);
  for (int n = 0; n < nnod; ++n) {
    const double x = f0.GCOORD[3 * (size_t)n], y = f0.GCOORD[3 * (size_t)n + 1], z = f0.GCOORD[3 * (size_t)n + 2];
    auto c2sh = [](double a, double b, double c, double *o) {
      o[2] = std::sqrt(a * a + b * b + c * c);
      o[0] = std::atan2(std::sqrt(a * a + b * b), c);
      o[1] = std::atan2(b, a);
      if (o[1] < 0) o[1] += 2 * M_PI;
    };
    double o[3];
    c2sh(x, -z, y, o);
    for (int k = 0; k < 3; ++k) SX[(size_t)k * nnod + n] = o[k];
    if (n < nv) {
      c2sh(-x, -y, z, o);
      for (int k = 0; k < 3; ++k) {
        SZ[(size_t)k * nv + n] = o[k];
        S0[(size_t)k * nv + n] = f0.GCOORD_SPH[3 * (size_t)n + k];
      }
    }
  }
  // start grid: each cell holds the largest id of the elements whose vertex centroid falls in it;
  // empty cells take the first filled face neighbour (fixed order, repeated passes)
  double grmin = 1e300, grmax = -1e300;
  for (int v = 0; v < nv; ++v) {
    grmin = std::min(grmin, S0[2 * (size_t)nv + v]);
    grmax = std::max(grmax, S0[2 * (size_t)nv + v]);
  }
  if (!(grmax > grmin)) grmax = grmin + 1.0;
  const double target = std::max(1.0, nel / 4.0);
  const int gnr = std::min(64, std::max(2, (int)std::lround(std::cbrt(target) / 4.0)));
  const int gnt = std::max(2, (int)std::lround(std::sqrt(target / gnr / 2.0)));
  const int gnp = 2 * gnt;
  std::vector<int> grid((size_t)gnt * gnp * gnr, -1);
  for (int e = 0; e < nel; ++e) {
    double c[3] = {0, 0, 0};
    for (int i = 0; i < 4; ++i)
      for (int k = 0; k < 3; ++k) c[k] += 0.25 * f0.GCOORD[3 * (size_t)el[(size_t)e * 10 + i] + k];
    const double r = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    const int cell = grid_cell(gnt, gnp, gnr, grmin, grmax, r > 0 ? c[2] / r : 1.0, std::atan2(c[1], c[0]), r);
    grid[cell] = std::max(grid[cell], e);
  }
  for (bool again = true; again;) {
    again = false;
    std::vector<int> g2 = grid;
    for (int ir = 0; ir < gnr; ++ir)
      for (int it = 0; it < gnt; ++it)
        for (int ip = 0; ip < gnp; ++ip) {
          const size_t c = ((size_t)ir * gnt + it) * gnp + ip;
          if (grid[c] >= 0) continue;
          const int nb[6][3] = {{ir, it, (ip + 1) % gnp}, {ir, it, (ip + gnp - 1) % gnp}, {ir, it + 1, ip},
                                {ir, it - 1, ip},         {ir + 1, it, ip},                 {ir - 1, it, ip}};
          for (const auto &q : nb)
            if (q[0] >= 0 && q[0] < gnr && q[1] >= 0 && q[1] < gnt) {
              const int v = grid[((size_t)q[0] * gnt + q[1]) * gnp + q[2]];
              if (v >= 0) {
                g2[c] = v;
                break;
              }
            }
          if (g2[c] < 0) again = true;
        }
    grid.swap(g2);
  }
  std::vector<uint8_t> cls(f0.elclass, f0.elclass + nel);
  // interface elements: some element sharing a vertex has another frame or another iso-ness (the
  // own-frame shapes of such neighbours overlap or leave gaps)
  // (face k, opposite local vertex k, borders another frame or iso-ness if one of its vertices is
  // shared with such an element: bit k of iface)
  std::vector<uint8_t> vmask(nv, 0), iface(nel, 0);
  auto key = [&](int e) { const int c = cls[e]; return (c >= 2 ? 0 : (c == 0 ? 1 : 2)) * 2 + (c == 3 ? 1 : 0); };
  for (int e = 0; e < nel; ++e)
    for (int i = 0; i < 4; ++i) vmask[el[(size_t)e * 10 + i]] |= (uint8_t)(1u << key(e));
  for (int e = 0; e < nel; ++e)
    for (int i = 0; i < 4; ++i) {
      const uint8_t mk = vmask[el[(size_t)e * 10 + i]];
      if (mk & (mk - 1))
        for (int k = 0; k < 4; ++k)
          if (k != i) iface[e] |= (uint8_t)(1u << k);
    }
  int st;
  if ((st = sl_upload(&S->el2nod, soa.data(), soa.size(), s)) || (st = sl_upload(&S->nbr, nbr.data(), nbr.size(), s)) ||
      (st = sl_upload(&S->v2e_ptr, ptr.data(), ptr.size(), s)) || (st = sl_upload(&S->v2e, adj.data(), adj.size(), s)) ||
      (st = sl_upload(&S->node_guess, first.data(), first.size(), s)) ||
      (st = sl_upload(&S->cls, cls.data(), cls.size(), s)) || (st = sl_upload(&S->S0, S0.data(), S0.size(), s)) ||
      (st = sl_upload(&S->SZ, SZ.data(), SZ.size(), s)) || (st = sl_upload(&S->SX, SX.data(), SX.size(), s)) ||
      (st = sl_upload(&S->grid, grid.data(), grid.size(), s)) ||
      (st = sl_upload(&S->iface, iface.data(), iface.size(), s)) || (st = sl_alloc(&S->ring_count, 16)))
    return st;
  const std::vector<float> S0f(S0.begin(), S0.end()), SZf(SZ.begin(), SZ.end()), SXf(SX.begin(), SX.end());
  if ((st = sl_upload(&S->S0f, S0f.data(), S0f.size(), s)) || (st = sl_upload(&S->SZf, SZf.data(), SZf.size(), s)) ||
      (st = sl_upload(&S->SXf, SXf.data(), SXf.size(), s)))
    return st;
  M3_CUDA(cudaStreamSynchronize(s));
  S->view = SlmMesh{nel, nnod, nv, S->el2nod, S->nbr, S->cls, S->S0, S->SZ, S->SX, S->v2e_ptr, S->v2e, S->iface,
                    S->S0f, S->SZf, S->SXf, S->grid, gnt, gnp, gnr, grmin, grmax};
  S->built = true;
  // the allocation-free interpolation's scratch address and kernels are resolved here, at handle
  // creation, so that its calls never load code or commit memory later
  return noalloc_prepare(M->device);
}

static int slm_reserve(SlmState *S, size_t npt, int nel, int nnod, int nv) {
  if (npt <= S->cap && S->P) return M3SPH_OK;
  for (void *q : {(void *)S->P, (void *)S->lc, (void *)S->V, (void *)S->out, (void *)S->upu, (void *)S->rpu,
                  (void *)S->U, (void *)S->els, (void *)S->guess, (void *)S->todo, (void *)S->status})
    if (q) cudaFree(q);
  const size_t n = std::max(npt, (size_t)nnod);
  int st;
  if ((st = sl_alloc(&S->P, 3 * n)) || (st = sl_alloc(&S->lc, 3 * n)) || (st = sl_alloc(&S->V, 3 * (size_t)nnod)) ||
      (st = sl_alloc(&S->out, 3 * n)) || (st = sl_alloc(&S->upu, 3 * (size_t)nnod)) ||
      (st = sl_alloc(&S->rpu, 3 * (size_t)nnod)) || (st = sl_alloc(&S->U, 3 * (size_t)nnod)) ||
      (st = sl_alloc(&S->els, n)) || (st = sl_alloc(&S->guess, n)) || (st = sl_alloc(&S->todo, n)) ||
      (st = sl_alloc(&S->status, n)))
    return st;
  if (!S->gel) {
    if ((st = sl_alloc(&S->gel, 3 * (size_t)nel)) || (st = sl_alloc(&S->wel, 4 * (size_t)nel)) ||
        (st = sl_alloc(&S->gn, 3 * (size_t)nv)) || (st = sl_alloc(&S->wn, (size_t)nv)) ||
        (st = sl_alloc(&S->Xc, 3 * (size_t)nnod)) || (st = sl_alloc(&S->kk, 3 * (size_t)nnod)) ||
        (st = sl_alloc(&S->acc, 3 * (size_t)nnod)))
      return st;
  }
  S->cap = n;
  return M3SPH_OK;
}

__global__ void k_aos3_to_soa(const double *__restrict__ a, int n, double *__restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  b[i] = a[3 * (size_t)i];
  b[n + (size_t)i] = a[3 * (size_t)i + 1];
  b[2 * (size_t)n + i] = a[3 * (size_t)i + 2];
}
__global__ void k_soa3_to_aos(const double *__restrict__ b, int n, double *__restrict__ a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  a[3 * (size_t)i] = b[i];
  a[3 * (size_t)i + 1] = b[n + (size_t)i];
  a[3 * (size_t)i + 2] = b[2 * (size_t)n + i];
}
__global__ void k_add_int(int *v, int n, int d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] += d;
}

// points the walk and the rings left unplaced (status bit 8), listed for the brute force; the
// order of the list does not matter (each point is resolved on its own)
__global__ void k_status_compact(const uint8_t *__restrict__ status, int npt, int *__restrict__ todo,
                                 int *__restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < npt && (status[i] & 8)) todo[atomicAdd(cnt, 1)] = i;
}
// status counts: [0] walk / ring placed (1), [1] ties (2), [2] gaps (4), [3] brute force (16),
// [4] lost (8 without 16), [5] ambiguous for the reference (32), [6] candidate overflow (64)
__global__ void k_status_counts(const uint8_t *__restrict__ status, int npt, int *__restrict__ cnt) {
  int c[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npt; i += gridDim.x * blockDim.x) {
    const int st = status[i];
    c[0] += st & 1;
    c[1] += (st >> 1) & 1;
    c[2] += (st >> 2) & 1;
    c[3] += (st >> 4) & 1;
    c[4] += (st & 8) && !(st & 16);
    c[5] += (st >> 5) & 1;
    c[6] += (st >> 6) & 1;
  }
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    int v = c[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(cnt + k, v);
  }
}

// locate S->P (npt points) with optional guesses (S->guess valid if use_guess), writing S->els,
// S->lc, S->status; unplaced points get a brute-force pass. Returns counts in info.
static int slm_locate(m3sph_mesh *M, SlmState *S, int npt, bool use_guess, bool node_guess, bool adjust,
                      m3sph_locate_info *info) {
  cudaStream_t s = M->stream;
  M3_CUDA(cudaMemsetAsync(S->ring_count, 0, 16 * sizeof(int), s));
  k_locate<<<(npt + 127) / 128, 128, 0, s>>>(S->view, S->P, npt, use_guess ? S->guess : nullptr,
                                              node_guess ? S->node_guess : nullptr, S->els, S->lc, S->status,
                                              adjust ? 1 : 0, S->todo, S->ring_count); count_launch();
  M3_CUDA(cudaGetLastError());
  int nring = 0;
  M3_CUDA(cudaMemcpyAsync(&nring, S->ring_count, sizeof(int), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  if (nring > 0) {
    k_resolve_ring<<<(nring + RING_WARPS - 1) / RING_WARPS, RING_WARPS * 32, 0, s>>>(S->view, S->P, npt, S->todo, nring,
                                                                                     S->els, S->lc, S->status,
                                                                                     adjust ? 1 : 0); count_launch();
    M3_CUDA(cudaGetLastError());
  }
  // unplaced points: listed on the device, brute force over the list
  k_status_compact<<<(npt + 255) / 256, 256, 0, s>>>(S->status, npt, S->todo, S->ring_count + 1); count_launch();
  int nt = 0;
  M3_CUDA(cudaMemcpyAsync(&nt, S->ring_count + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  if (nt > 0) {
    k_locate_brute<<<(nt + BRUTE_WARPS - 1) / BRUTE_WARPS, BRUTE_WARPS * 32, 0, s>>>(S->view, S->P, npt, S->todo, nt,
                                                                                    S->els, S->lc, S->status,
                                                                                    adjust ? 1 : 0); count_launch();
    M3_CUDA(cudaGetLastError());
  }
  k_status_counts<<<std::min((npt + 255) / 256, 1216), 256, 0, s>>>(S->status, npt, S->ring_count + 2); count_launch();
  int hc[7];
  M3_CUDA(cudaMemcpyAsync(hc, S->ring_count + 2, sizeof(hc), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  const int nwalk = hc[0], ntie = hc[1], ngap = hc[2], nbrute = hc[3], nlost = hc[4], nambig = hc[5],
            noverflow = hc[6];
  if (info) {
    info->npt = npt;
    info->nwalk = nwalk;
    info->nties = ntie;
    info->ngap = ngap;
    info->nbrute = nbrute;
    info->nlost = nlost;
    info->nambig = nambig;
  }
  if (noverflow) {
    set_error("point location: more than " + std::to_string(MAX_CAND) + " elements tie at " +
              std::to_string(noverflow) + " points");
    return M3SPH_ERR_BAD_INPUT;
  }
  if (nlost) {
    set_error("some nodes have not been located");
    return M3SPH_ERR_POINT_NOT_FOUND;
  }
  return M3SPH_OK;
}

static int slm_cubic_gradients(m3sph_mesh *M, SlmState *S, const double *B, int method_wght) {
  cudaStream_t s = M->stream;
  Level &L0 = M->lev[0];
  const int nel = L0.nel, nv = L0.nvnod;
  k_cubic_elgrad<<<(nel + 127) / 128, 128, 0, s>>>(S->view, M->fin.gcoord, B, method_wght, S->gel, S->wel); count_launch();
  M3_CUDA(cudaMemsetAsync(S->gn, 0, sizeof(double) * 3 * nv, s));
  M3_CUDA(cudaMemsetAsync(S->wn, 0, sizeof(double) * nv, s));
  for (size_t c = 0; c + 1 < L0.cstart.size(); ++c) {
    const int b = L0.cstart[c], e = L0.cstart[c + 1];
    if (e > b) k_cubic_scatter<<<(e - b + 127) / 128, 128, 0, s>>>(L0.perm, nel, b, e, S->el2nod, S->gel, S->wel,
                                                                   S->gn, S->wn, nv); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

static SlmState *slm_state(m3sph_mesh *M) { return reinterpret_cast<SlmState *>(M->slm); }

}  // namespace m3sph

using namespace m3sph;

// element ids of interp3d_tet / interp3d_cubic_p callers: 1-based, within the mesh (the reference
// indexes EL2NOD with them, so any other value is an error there too)
static int check_element_ids(const int32_t *els, int npt, int nel, const char *fn) {
  for (int i = 0; i < npt; ++i)
    if (els[i] < 1 || els[i] > nel) {
      set_error(std::string(fn) + ": element id " + std::to_string(els[i]) + " at point " + std::to_string(i + 1) +
                " is outside 1.." + std::to_string(nel));
      return M3SPH_ERR_BAD_INPUT;
    }
  return M3SPH_OK;
}

static int slm_check(m3sph_mesh *M) {
  if (!M || !M->slm) {
    set_error("mesh handle without advection data");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  return M3SPH_OK;
}

extern "C" int m3sph_tsearch_sph(m3sph_mesh *M, const double *thphr, int32_t npt, const int32_t *els_guess,
                                 int32_t *els_out, double *lc_out, m3sph_locate_info *info) {
  int st = slm_check(M);
  if (st) return st;
  if (npt < 0 || (npt > 0 && (!thphr || !els_out))) {
    set_error("m3sph_tsearch_sph: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  if (npt == 0) return M3SPH_OK;
  SlmState *S = slm_state(M);
  Level &L0 = M->lev[0];
  if ((st = slm_reserve(S, npt, L0.nel, L0.nnod, L0.nvnod))) return st;
  cudaStream_t s = M->stream;
  // points arrive point-major (th ph r per point); S->lc stages them for the transpose to S->P
  M3_CUDA(cudaMemcpyAsync(S->lc, thphr, sizeof(double) * 3 * (size_t)npt, cudaMemcpyHostToDevice, s));
  k_aos3_to_soa<<<(npt + 255) / 256, 256, 0, s>>>(S->lc, npt, S->P); count_launch();
  if (els_guess) {
    M3_CUDA(cudaMemcpyAsync(S->guess, els_guess, sizeof(int) * npt, cudaMemcpyHostToDevice, s));
    k_add_int<<<(npt + 255) / 256, 256, 0, s>>>(S->guess, npt, -1); count_launch();
  }
  st = slm_locate(M, S, npt, els_guess != nullptr, npt == L0.nnod, false, info);
  if (st && st != M3SPH_ERR_POINT_NOT_FOUND) return st;
  // 1-based ids; local coordinates back to point-major order (S->P is free now)
  k_add_int<<<(npt + 255) / 256, 256, 0, s>>>(S->els, npt, 1); count_launch();
  M3_CUDA(cudaMemcpyAsync(els_out, S->els, sizeof(int) * npt, cudaMemcpyDeviceToHost, s));
  if (lc_out) {
    k_soa3_to_aos<<<(npt + 255) / 256, 256, 0, s>>>(S->lc, npt, S->P); count_launch();
    M3_CUDA(cudaMemcpyAsync(lc_out, S->P, sizeof(double) * 3 * (size_t)npt, cudaMemcpyDeviceToHost, s));
  }
  M3_CUDA(cudaStreamSynchronize(s));
  return st;
}

extern "C" int m3sph_locate_timing(m3sph_mesh *M, const double *thphr, int32_t npt, int32_t nrep, double *ms,
                                   m3sph_locate_info *info) {
  int st = slm_check(M);
  if (st) return st;
  if (npt <= 0 || nrep <= 0 || !thphr || !ms) {
    set_error("m3sph_locate_timing: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  SlmState *S = slm_state(M);
  Level &L0 = M->lev[0];
  if ((st = slm_reserve(S, npt, L0.nel, L0.nnod, L0.nvnod))) return st;
  cudaStream_t s = M->stream;
  M3_CUDA(cudaMemcpyAsync(S->lc, thphr, sizeof(double) * 3 * (size_t)npt, cudaMemcpyHostToDevice, s));
  k_aos3_to_soa<<<(npt + 255) / 256, 256, 0, s>>>(S->lc, npt, S->P); count_launch();
  st = slm_locate(M, S, npt, false, false, false, info);       // warm-up
  if (st) return st;
  cudaEvent_t e0, e1;
  M3_CUDA(cudaEventCreate(&e0));
  M3_CUDA(cudaEventCreate(&e1));
  M3_CUDA(cudaEventRecord(e0, s));
  for (int r = 0; r < nrep && !st; ++r) st = slm_locate(M, S, npt, false, false, false, info);
  M3_CUDA(cudaEventRecord(e1, s));
  M3_CUDA(cudaEventSynchronize(e1));
  float t = 0.f;
  M3_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t / nrep;
  return st;
}

extern "C" int m3sph_interp3d_tet(m3sph_mesh *M, const int32_t *els, const double *lc, int32_t npt, const double *V,
                                  int32_t nvar, int32_t monotonic, double *Vi) {
  int st = slm_check(M);
  if (st) return st;
  if (npt < 0 || nvar < 1 || nvar > 3 || (npt > 0 && (!els || !lc || !V || !Vi))) {
    set_error("m3sph_interp3d_tet: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  if (npt == 0) return M3SPH_OK;
  SlmState *S = slm_state(M);
  Level &L0 = M->lev[0];
  if ((st = check_element_ids(els, npt, L0.nel, "m3sph_interp3d_tet"))) return st;
  if ((st = slm_reserve(S, npt, L0.nel, L0.nnod, L0.nvnod))) return st;
  cudaStream_t s = M->stream;
  std::vector<int> e(npt);
  std::vector<double> l(3 * (size_t)npt), v((size_t)nvar * L0.nnod);
  for (int i = 0; i < npt; ++i) {
    e[i] = els[i] - 1;
    for (int k = 0; k < 3; ++k) l[(size_t)k * npt + i] = lc[3 * (size_t)i + k];
  }
  for (int n = 0; n < L0.nnod; ++n)
    for (int k = 0; k < nvar; ++k) v[(size_t)k * L0.nnod + n] = V[(size_t)n * nvar + k];
  M3_CUDA(cudaMemcpyAsync(S->els, e.data(), sizeof(int) * npt, cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(S->lc, l.data(), sizeof(double) * l.size(), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(S->V, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice, s));
  k_interp_p2<<<(npt + 127) / 128, 128, 0, s>>>(S->view, S->els, S->lc, npt, S->V, nvar, monotonic, S->out); count_launch();
  M3_CUDA(cudaGetLastError());
  std::vector<double> o((size_t)nvar * npt);
  M3_CUDA(cudaMemcpyAsync(o.data(), S->out, sizeof(double) * o.size(), cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < npt; ++i)
    for (int k = 0; k < nvar; ++k) Vi[(size_t)i * nvar + k] = o[(size_t)k * npt + i];
  return M3SPH_OK;
}

extern "C" int m3sph_interp3d_cubic(m3sph_mesh *M, const int32_t *els, const double *lc, int32_t npt, const double *V,
                                    int32_t monotonic, int32_t method_wght, double *Vi) {
  int st = slm_check(M);
  if (st) return st;
  if (npt < 0 || (npt > 0 && (!els || !lc || !V || !Vi))) {
    set_error("m3sph_interp3d_cubic: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  if (npt == 0) return M3SPH_OK;
  SlmState *S = slm_state(M);
  Level &L0 = M->lev[0];
  if ((st = check_element_ids(els, npt, L0.nel, "m3sph_interp3d_cubic"))) return st;
  if ((st = slm_reserve(S, npt, L0.nel, L0.nnod, L0.nvnod))) return st;
  cudaStream_t s = M->stream;
  std::vector<int> e(npt);
  std::vector<double> l(3 * (size_t)npt);
  for (int i = 0; i < npt; ++i) {
    e[i] = els[i] - 1;
    for (int k = 0; k < 3; ++k) l[(size_t)k * npt + i] = lc[3 * (size_t)i + k];
  }
  M3_CUDA(cudaMemcpyAsync(S->els, e.data(), sizeof(int) * npt, cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(S->lc, l.data(), sizeof(double) * l.size(), cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(S->V, V, sizeof(double) * L0.nnod, cudaMemcpyHostToDevice, s));
  if ((st = slm_cubic_gradients(M, S, S->V, method_wght))) return st;
  k_cubic_interp<<<(npt + 127) / 128, 128, 0, s>>>(S->view, M->fin.gcoord, S->els, S->lc, npt, S->V, S->gn, S->wn,
                                                    S->gel, monotonic, S->out); count_launch();
  M3_CUDA(cudaGetLastError());
  M3_CUDA(cudaMemcpyAsync(Vi, S->out, sizeof(double) * npt, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}

// advect3d_slm_p_sph with PC2 backtracking: T (nnod) updated in place; els_BT / els_INTERP
// (nnod, 1-based, 0 = none) are the WS_SLM guesses, updated on return.
static int advect_device(m3sph_mesh *M, double dt, const m3sph_slm_opts *o, bool use_ws, m3sph_locate_info *info) {
  SlmState *S = slm_state(M);
  Level &L0 = M->lev[0];
  cudaStream_t s = M->stream;
  const int n = L0.nnod;
  k_predictor<<<(n + 127) / 128, 128, 0, s>>>(M->fin.gcoord, M->fin.gcoord_sph, n, S->U, dt, o->r_cmb, o->r_surf,
                                               S->P, S->upu, S->rpu); count_launch();
  M3_CUDA(cudaGetLastError());
  m3sph_locate_info i1{}, i2{};
  M3_TRY(slm_locate(M, S, n, use_ws, true, true, &i1));
  // guesses for the next step's predictor search (els_BT) are this step's predictor elements
  k_interp_p2<<<(n + 127) / 128, 128, 0, s>>>(S->view, S->els, S->lc, n, S->U, 3, 0, S->out); count_launch();
  M3_CUDA(cudaMemcpyAsync(S->guess, S->els, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
  k_corrector<<<(n + 127) / 128, 128, 0, s>>>(M->fin.gcoord, M->fin.gcoord_sph, n, S->out, S->upu, S->rpu, dt,
                                               o->r_cmb, o->r_surf, S->P); count_launch();
  M3_CUDA(cudaGetLastError());
  M3_TRY(slm_locate(M, S, n, true, true, true, &i2));
  if (o->method_interp == 1) {
    M3_TRY(slm_cubic_gradients(M, S, S->V, o->method_wght));
    k_cubic_interp<<<(n + 127) / 128, 128, 0, s>>>(S->view, M->fin.gcoord, S->els, S->lc, n, S->V, S->gn, S->wn,
                                                    S->gel, o->monotonic, S->out); count_launch();
  } else {
    k_interp_p2<<<(n + 127) / 128, 128, 0, s>>>(S->view, S->els, S->lc, n, S->V, 1, o->monotonic, S->out); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  if (info) {
    info->npt = i1.npt + i2.npt;
    info->nwalk = i1.nwalk + i2.nwalk;
    info->nties = i1.nties + i2.nties;
    info->ngap = i1.ngap + i2.ngap;
    info->nbrute = i1.nbrute + i2.nbrute;
    info->nlost = i1.nlost + i2.nlost;
    info->nambig = i1.nambig + i2.nambig;
  }
  return M3SPH_OK;
}

static void add_info(m3sph_locate_info &a, const m3sph_locate_info &b) {
  a.npt += b.npt; a.nwalk += b.nwalk; a.nties += b.nties; a.ngap += b.ngap; a.nbrute += b.nbrute; a.nlost += b.nlost;
  a.nambig += b.nambig;
}

static int advect_device_rk4(m3sph_mesh *M, double dt, const m3sph_slm_opts *o, int nsub, bool use_ws,
                             m3sph_locate_info *info) {
  SlmState *S = slm_state(M);
  Level &L0 = M->lev[0];
  cudaStream_t s = M->stream;
  const int n = L0.nnod;
  const unsigned gb = (unsigned)((n + 127) / 128), gb3 = (unsigned)((3 * n + 127) / 128);
  const double h = dt / nsub;
  const double cst[4] = {0.0, 0.5, 0.5, 1.0}, wst[4] = {1.0, 2.0, 2.0, 1.0};
  m3sph_locate_info tot{};
  M3_CUDA(cudaMemcpyAsync(S->Xc, M->fin.gcoord, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, s));
  bool have_guess = use_ws;
  for (int sub = 0; sub < nsub; ++sub) {
    for (int st = 0; st < 4; ++st) {
      if (sub == 0 && st == 0) {
        M3_CUDA(cudaMemcpyAsync(S->kk, S->U, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, s));
      } else {
        // stage point x - c h k_prev (k_prev in kk), located and U interpolated there
        // stage 0 of later substeps: U at the new point (c = 0)
        k_rk_point<<<gb, 128, 0, s>>>(S->Xc, S->kk, n, cst[st] * h, o->r_cmb, o->r_surf, S->P); count_launch();
        m3sph_locate_info li{};
        M3_TRY(slm_locate(M, S, n, have_guess, true, true, &li));
        add_info(tot, li);
        M3_CUDA(cudaMemcpyAsync(S->guess, S->els, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
        have_guess = true;
        k_interp_p2<<<gb, 128, 0, s>>>(S->view, S->els, S->lc, n, S->U, 3, 0, S->kk); count_launch();
      }
      k_rk_accum<<<gb3, 128, 0, s>>>(S->acc, S->kk, 3 * n, wst[st], st == 0); count_launch();
    }
    k_rk_update<<<gb, 128, 0, s>>>(S->Xc, S->acc, n, h, o->r_cmb, o->r_surf); count_launch();
  }
  // departure points -> T
  k_cart_to_sph<<<gb, 128, 0, s>>>(S->Xc, n, S->P); count_launch();
  m3sph_locate_info li{};
  M3_TRY(slm_locate(M, S, n, true, true, true, &li));
  add_info(tot, li);
  if (o->method_interp == 1) {
    M3_TRY(slm_cubic_gradients(M, S, S->V, o->method_wght));
    k_cubic_interp<<<gb, 128, 0, s>>>(S->view, M->fin.gcoord, S->els, S->lc, n, S->V, S->gn, S->wn, S->gel,
                                      o->monotonic, S->out); count_launch();
  } else {
    k_interp_p2<<<gb, 128, 0, s>>>(S->view, S->els, S->lc, n, S->V, 1, o->monotonic, S->out); count_launch();
  }
  M3_CUDA(cudaGetLastError());
  if (info) *info = tot;
  return M3SPH_OK;
}

namespace m3sph {
// advect3d_slm_p_sph on device-resident data (the time step): U_soa [3][nnod] Cartesian nodal
// velocity, T (nnod) advected in place. The search guesses carry over from the previous call of the
// same handle (the reference's WS_SLM) unless first_step.
int slm_advect_resident(m3sph_mesh *M, const double *U_soa, double *T, double dt, const m3sph_slm_opts *o,
                        bool first_step, m3sph_locate_info *info) {
  int st = slm_check(M);
  if (st) return st;
  if (o->method_BT != 1 && o->method_BT != 2) {
    set_error("method_BT must be 1 (PC2) or 2 (RK4, 3 substeps)");
    return M3SPH_ERR_BAD_INPUT;
  }
  SlmState *S = slm_state(M);
  Level &L0 = M->lev[0];
  const int n = L0.nnod;
  if ((st = slm_reserve(S, n, L0.nel, n, L0.nvnod))) return st;
  cudaStream_t s = M->stream;
  M3_CUDA(cudaMemcpyAsync(S->U, U_soa, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToDevice, s));
  M3_CUDA(cudaMemcpyAsync(S->V, T, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  if (o->method_BT == 2) {
    M3_TRY(advect_device_rk4(M, dt, o, 3, !first_step, info));
  } else {
    M3_TRY(advect_device(M, dt, o, !first_step, info));
  }
  M3_CUDA(cudaMemcpyAsync(T, S->out, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  return M3SPH_OK;
}
}  // namespace m3sph

extern "C" int m3sph_advect_slm(m3sph_mesh *M, const double *Ux, const double *Uy, const double *Uz, double *T,
                                double dt, const m3sph_slm_opts *o, int32_t *els_BT, int32_t *els_INTERP,
                                m3sph_locate_info *info) {
  int st = slm_check(M);
  if (st) return st;
  if (!Ux || !Uy || !Uz || !T || !o) {
    set_error("m3sph_advect_slm: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  if (o->method_BT != 1 && o->method_BT != 2) {
    set_error("m3sph_advect_slm: method_BT must be 1 (PC2) or 2 (RK4, 3 substeps)");
    return M3SPH_ERR_BAD_INPUT;
  }
  SlmState *S = slm_state(M);
  Level &L0 = M->lev[0];
  const int n = L0.nnod;
  if ((st = slm_reserve(S, n, L0.nel, n, L0.nvnod))) return st;
  cudaStream_t s = M->stream;
  M3_CUDA(cudaMemcpyAsync(S->U, Ux, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(S->U + n, Uy, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(S->U + 2 * (size_t)n, Uz, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  M3_CUDA(cudaMemcpyAsync(S->V, T, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  bool use_ws = false;
  if (els_BT) {
    std::vector<int> g(n);
    bool any = false;
    for (int i = 0; i < n; ++i) {
      g[i] = (int)els_BT[i] - 1;
      any |= g[i] >= 0;
    }
    if (any) {
      use_ws = true;
      M3_CUDA(cudaMemcpyAsync(S->guess, g.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    }
  }
  if (o->method_BT == 2) {
    M3_TRY(advect_device_rk4(M, dt, o, 3, use_ws, info));
  } else {
    M3_TRY(advect_device(M, dt, o, use_ws, info));
  }
  std::vector<int> e(n);
  M3_CUDA(cudaMemcpyAsync(T, S->out, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaMemcpyAsync(e.data(), S->els, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  std::vector<int> g(n);
  M3_CUDA(cudaMemcpyAsync(g.data(), S->guess, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  M3_CUDA(cudaStreamSynchronize(s));
  // WS_SLM: els_BT = predictor elements (still in `guess`), els_INTERP = departure elements
  for (int i = 0; i < n; ++i) {
    if (els_BT) els_BT[i] = g[i] + 1;
    if (els_INTERP) els_INTERP[i] = e[i] + 1;
  }
  return M3SPH_OK;
}

// ======================================================================================
// Allocation-free quasi-cubic interpolation.
//
// Some callers of this library cannot allocate device memory once they are running: a host
// whose device memory is entirely owned by its own pool allocator (a stray cudaMalloc would fail
// or fragment that pool), a solver loop that must keep its memory footprint fixed after start-up,
// or a host with work in flight on other streams that a cudaMalloc / cudaFree (which may
// synchronise the device) would stall. m3sph_interp3d_cubic grows the handle's work buffers on demand
// (cudaMalloc); this variant keeps its scratch -- element gradients and weights, nodal gradient
// sums -- in the fixed file-scope array below, and takes inputs and outputs in memory the caller
// already owns and the device can read and write.
// ======================================================================================
namespace m3sph {

constexpr size_t NOALLOC_SCRATCH_DOUBLES = size_t(1) << 20;   // 8 MiB per device, held until exit
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static double *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {nullptr};
static std::mutex g_noalloc_mu;

// Device address of the scratch array on `device`, looked up once per device with that device
// current (in host code the symbol name is only a host-side stand-in, never a device address).
static int noalloc_scratch(int device, double **out) {
  if (device < 0 || device >= NOALLOC_MAX_DEVICES) {
    set_error("device id out of range for the allocation-free scratch table");
    return M3SPH_ERR_BAD_INPUT;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    int cur = -1;
    M3_CUDA(cudaGetDevice(&cur));
    if (cur != device) M3_CUDA(cudaSetDevice(device));
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (cur != device) cudaSetDevice(cur);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_ptr[device] = static_cast<double *>(p);
  }
  *out = g_noalloc_ptr[device];
  return M3SPH_OK;
}

__global__ void k_cubic_interp_caller(SlmMesh m, const double *__restrict__ X, const int32_t *__restrict__ els,
                                      const double *__restrict__ lc, int npt, const double *__restrict__ B,
                                      const double *__restrict__ gn, const double *__restrict__ wn,
                                      const double *__restrict__ gel, int monotonic, double *__restrict__ out);

// zero n doubles (the nodal sums): a kernel of this module rather than cudaMemsetAsync, so that
// nothing the call uses is loaded outside noalloc_prepare
__global__ void k_noalloc_zero(double *a, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) a[i] = 0.0;
}

// Run once per handle, from m3sph_mesh_create with the handle's device current. With CUDA's lazy
// module loading, the first use of this file's module -- the scratch lookup or the first launch of
// one of its kernels -- is where the driver loads the code and commits the 8 MiB array; doing both
// here keeps those allocations out of m3sph_interp3d_cubic_noalloc.
static int noalloc_prepare(int device) {
  double *scr = nullptr;
  int st = noalloc_scratch(device, &scr);
  if (st) return st;
  cudaFuncAttributes fa;
  M3_CUDA(cudaFuncGetAttributes(&fa, k_cubic_elgrad));
  M3_CUDA(cudaFuncGetAttributes(&fa, k_cubic_scatter));
  M3_CUDA(cudaFuncGetAttributes(&fa, k_cubic_interp_caller));
  M3_CUDA(cudaFuncGetAttributes(&fa, k_noalloc_zero));
  return M3SPH_OK;
}

// quasi-cubic value at one point of element e with local coordinates (r,s,t): the same arithmetic
// as k_cubic_interp (interp3d_cubic_p.m:243-382)
__device__ double cubic_point(const SlmMesh &m, const double *__restrict__ X, int e, double r, double s, double t,
                              const double *__restrict__ B, const double *__restrict__ gn,
                              const double *__restrict__ wn, const double *__restrict__ gel, int monotonic) {
  const double u = 1.0 - r - s - t;
  const double q2 = 1.4142135623730951;   // sqrt(2)
  const double N[16] = {r, s, t, u, q2 * r * s, q2 * s * t, t * u, r * u, q2 * r * t, s * u,
                        q2 * s * r * (s - r), q2 * s * t * (t - s), t * u * (u - t), r * u * (u - r),
                        q2 * r * t * (t - r), s * u * (u - s)};
  int v[4];
  double x[4], y[4], z[4], b[4], dB[4][3];
  for (int k = 0; k < 4; ++k) {
    v[k] = m.el2nod[(size_t)k * m.nel + e];
    x[k] = X[v[k]]; y[k] = X[m.nnod + v[k]]; z[k] = X[2 * m.nnod + v[k]];
    b[k] = B[v[k]];
    const double wk = wn[v[k]];
    for (int c = 0; c < 3; ++c) dB[k][c] = gn[(size_t)c * m.nvnod + v[k]] / wk - gel[(size_t)c * m.nel + e];
  }
  double sr[4], ss[4], st[4];
  for (int k = 0; k < 4; ++k) {
    sr[k] = (x[0] - x[3]) * dB[k][0] + (y[0] - y[3]) * dB[k][1] + (z[0] - z[3]) * dB[k][2];
    ss[k] = (x[1] - x[3]) * dB[k][0] + (y[1] - y[3]) * dB[k][1] + (z[1] - z[3]) * dB[k][2];
    st[k] = (x[2] - x[3]) * dB[k][0] + (y[2] - y[3]) * dB[k][1] + (z[2] - z[3]) * dB[k][2];
  }
  const double h = 0.7071067811865476;    // sqrt(1/2)
  const double q1n2 = h * sr[1] - h * ss[1], q1n1 = h * sr[0] - h * ss[0];
  const double q2n3 = h * ss[2] - h * st[2], q2n2 = h * ss[1] - h * st[1];
  const double q5n3 = h * sr[2] - h * st[2], q5n1 = h * sr[0] - h * st[0];
  const double info[12] = {(q1n2 - q1n1) / 2, (q2n3 - q2n2) / 2, (st[3] - st[2]) / 2, (sr[3] - sr[0]) / 2,
                           (q5n3 - q5n1) / 2, (ss[3] - ss[1]) / 2, (q1n2 + q1n1) / 2, (q2n3 + q2n2) / 2,
                           (st[3] + st[2]) / 2, (sr[3] + sr[0]) / 2, (q5n3 + q5n1) / 2, (ss[3] + ss[1]) / 2};
  double val = N[0] * b[0] + N[1] * b[1] + N[2] * b[2] + N[3] * b[3];
  for (int k = 0; k < 12; ++k) val += N[4 + k] * info[k];
  if (monotonic) {
    const double lo = fmin(fmin(b[0], b[1]), fmin(b[2], b[3])), hi = fmax(fmax(b[0], b[1]), fmax(b[2], b[3]));
    val = fmin(fmax(val, lo), hi);
  }
  return val;
}

// caller-layout variant: 1-based element ids, local coordinates as npt x 3
__global__ void k_cubic_interp_caller(SlmMesh m, const double *__restrict__ X, const int32_t *__restrict__ els,
                                      const double *__restrict__ lc, int npt, const double *__restrict__ B,
                                      const double *__restrict__ gn, const double *__restrict__ wn,
                                      const double *__restrict__ gel, int monotonic, double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npt) return;
  const int e = els[i] - 1;
  if (e < 0 || e >= m.nel) {
    out[i] = nan("");
    return;
  }
  out[i] = cubic_point(m, X, e, lc[3 * (size_t)i], lc[3 * (size_t)i + 1], lc[3 * (size_t)i + 2], B, gn, wn, gel,
                       monotonic);
}

}  // namespace m3sph

extern "C" int m3sph_interp3d_cubic_noalloc(m3sph_mesh *M, const int32_t *els, const double *lc, int32_t npt,
                                            const double *V, int32_t monotonic, int32_t method_wght, double *Vi) {
  int st = slm_check(M);
  if (st) return st;
  if (npt < 0 || (npt > 0 && (!els || !lc || !V || !Vi))) {
    set_error("m3sph_interp3d_cubic_noalloc: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  if (npt == 0) return M3SPH_OK;
  SlmState *S = slm_state(M);
  Level &L0 = M->lev[0];
  const size_t nel = L0.nel, nv = L0.nvnod;
  const size_t need = 7 * nel + 4 * nv;   // element gradients (3) and weights (4), nodal sums (3) and weights (1)
  if (need > NOALLOC_SCRATCH_DOUBLES) {
    set_error("m3sph_interp3d_cubic_noalloc: this mesh needs " + std::to_string(need) +
              " scratch values but the fixed scratch holds " + std::to_string(NOALLOC_SCRATCH_DOUBLES) +
              " (7 per element + 4 per vertex); use m3sph_interp3d_cubic");
    return M3SPH_ERR_BAD_INPUT;
  }
  double *scr = nullptr;
  if ((st = noalloc_scratch(M->device, &scr))) return st;
  double *gel = scr, *wel = gel + 3 * nel, *gn = wel + 4 * nel, *wn = gn + 3 * nv;
  cudaStream_t s = M->stream;
  k_cubic_elgrad<<<(unsigned)((nel + 127) / 128), 128, 0, s>>>(S->view, M->fin.gcoord, V, method_wght, gel, wel); count_launch();
  // the array keeps the previous call's contents: the nodal sums must start at zero
  k_noalloc_zero<<<(unsigned)std::min<size_t>((4 * nv + 255) / 256, 1024), 256, 0, s>>>(gn, 4 * nv); count_launch();
  // (gn (3 nv) and wn (nv) are contiguous)
  for (size_t c = 0; c + 1 < L0.cstart.size(); ++c) {
    const int b = L0.cstart[c], e = L0.cstart[c + 1];
    if (e > b) k_cubic_scatter<<<(e - b + 127) / 128, 128, 0, s>>>(L0.perm, (int)nel, b, e, S->el2nod, gel, wel, gn,
                                                                   wn, (int)nv); count_launch();
  }
  k_cubic_interp_caller<<<(npt + 127) / 128, 128, 0, s>>>(S->view, M->fin.gcoord, els, lc, npt, V, gn, wn, gel,
                                                           monotonic, Vi); count_launch();
  M3_CUDA(cudaGetLastError());
  M3_CUDA(cudaStreamSynchronize(s));
  return M3SPH_OK;
}
