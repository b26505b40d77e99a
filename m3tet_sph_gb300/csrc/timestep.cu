// Rock properties and the device-resident time step.
//
// rock_prop (rock_prop.m:5-66) is one elementwise pass over the nodes (HBM-bound: 8 B of T and
// 24 B of coordinates read, 16 B written per node). The time step chains the hot-path calls of the
// reference's time loop (M3TET_SPH_SOUTH_ATLANTIC_PLUME.m:213-296) without leaving the device:
// rock_prop -> Stokes (operator rebuild + Patera) -> calculate_dt -> semi-Lagrangian advection.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>

#include "common.cuh"

namespace m3sph {

constexpr double ROCK_R = 8.314472;   // J/(mol K), rock_prop.m

struct RockArgs {
  double Visc0, Dens0, T_ref, alpha, Ea, Va, g, L0, a_UM2LM;
  double minDens, maxDens, minVisc, maxVisc;   // NaN: no cut-off
  double rad_max;
};

// Dens and Visc of node n (rock_prop.m:14-62), in the reference's order of operations
__global__ void k_rock_prop(const double *__restrict__ T, const double *__restrict__ X, int nnod, RockArgs a,
                            double *__restrict__ visc, double *__restrict__ dens) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnod) return;
  const double t = T[n];
  double d = a.Dens0 * (1.0 - a.alpha * (t - a.T_ref));
  if (!isnan(a.maxDens)) d = fmin(d, a.maxDens);
  if (!isnan(a.minDens)) d = fmax(d, a.minDens);
  const double T0_K = a.T_ref + 273.0;
  double v = 1.0;
  if (a.Ea > 0.0) {
    const double T_K = t + 273.0;
    const double eta = a.Ea / (ROCK_R * T0_K);
    v = v * exp(eta * ((T0_K / T_K) - 1.0));
    v = fmin(v, 1e8);
    v = fmax(v, 1e-8);
  }
  double v2 = v;
  if (a.Va > 0.0) {
    const double x = X[n], y = X[nnod + n], z = X[2 * (size_t)nnod + n];
    const double depth = a.rad_max - sqrt(x * x + y * y + z * z);
    const double P = fabs(a.g * a.Dens0 * a.L0 * depth);
    v2 = v2 * exp(P * a.Va / (ROCK_R * T0_K));
  }
  double v3 = v;
  if (a.a_UM2LM > 0.0) v3 = v3 * a.a_UM2LM;
  double mu = fmin(v2, v3) * a.Visc0;
  if (!isnan(a.maxVisc)) mu = fmin(mu, a.maxVisc);
  if (!isnan(a.minVisc)) mu = fmax(mu, a.minVisc);
  visc[n] = mu;
  dens[n] = d;
}

static int rock_args(const m3sph_mesh *M, const m3sph_rock_params *p, RockArgs &a) {
  if (p->Ea > 0.0 && p->Ea < 1000.0) {
    set_error(" Activation energy PHYSICS.Ea seems to be in kJ/mol. Convert to J/mol.");
    return M3SPH_ERR_BAD_INPUT;
  }
  a = RockArgs{p->Visc0, p->Dens0, p->T_ref, p->alpha, p->Ea, p->Va, p->g, p->L0, p->a_UM2LM,
               p->minDens, p->maxDens, p->minVisc, p->maxVisc, M->rad_max};
  return M3SPH_OK;
}

static int rock_prop_device(m3sph_mesh *M, const m3sph_rock_params *p, const double *T, double *visc, double *dens) {
  RockArgs a;
  M3_TRY(rock_args(M, p, a));
  const int n = M->lev[0].nnod;
  k_rock_prop<<<(n + 255) / 256, 256, 0, M->stream>>>(T, M->fin.gcoord, n, a, visc, dens); count_launch();
  M3_CUDA(cudaGetLastError());
  return M3SPH_OK;
}

static int elapsed(cudaEvent_t a, cudaEvent_t b, double &ms) {
  float f = 0.f;
  M3_CUDA(cudaEventElapsedTime(&f, a, b));
  ms = f;
  return M3SPH_OK;
}

}  // namespace m3sph

using namespace m3sph;

extern "C" int m3sph_rock_prop(m3sph_mesh *M, const m3sph_rock_params *p, const double *T, double *Visc,
                               double *Dens) {
  if (!M || !p || !T || !Visc || !Dens) {
    set_error("m3sph_rock_prop: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  const size_t n = M->lev[0].nnod;
  cudaStream_t s = M->stream;
  double *d = nullptr;
  M3_CUDA(cudaMalloc(&d, 3 * n * sizeof(double)));
  int st = M3SPH_OK;
  if (cudaMemcpyAsync(d, T, n * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess)
    st = cuda_fail(cudaGetLastError(), "m3sph_rock_prop upload");
  if (!st) st = rock_prop_device(M, p, d, d + n, d + 2 * n);
  if (!st && (cudaMemcpyAsync(Visc, d + n, n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
              cudaMemcpyAsync(Dens, d + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
              cudaStreamSynchronize(s) != cudaSuccess))
    st = cuda_fail(cudaGetLastError(), "m3sph_rock_prop download");
  cudaFree(d);
  return st;
}

extern "C" int m3sph_set_temperature(m3sph_mesh *M, const double *T, double time) {
  if (!M || !T) {
    set_error("m3sph_set_temperature: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  const size_t n = M->lev[0].nnod;
  if (!M->T) M3_CUDA(cudaMalloc(&M->T, n * sizeof(double)));
  if (!M->Usoa) M3_CUDA(cudaMalloc(&M->Usoa, 3 * n * sizeof(double)));
  M3_CUDA(cudaMemcpyAsync(M->T, T, n * sizeof(double), cudaMemcpyHostToDevice, M->stream));
  M3_CUDA(cudaStreamSynchronize(M->stream));
  M->ts_steps = 0;
  M->ts_time = time;
  return M3SPH_OK;
}

extern "C" int m3sph_get_temperature(m3sph_mesh *M, double *T) {
  if (!M || !T || !M->T) {
    set_error("m3sph_get_temperature: no resident temperature (call m3sph_set_temperature)");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  M3_CUDA(cudaMemcpyAsync(T, M->T, M->lev[0].nnod * sizeof(double), cudaMemcpyDeviceToHost, M->stream));
  M3_CUDA(cudaStreamSynchronize(M->stream));
  return M3SPH_OK;
}

extern "C" int m3sph_get_properties(m3sph_mesh *M, double *Visc, double *Dens) {
  if (!M || !M->have_operator) {
    set_error("m3sph_get_properties: call m3sph_stokes_setup first");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  const size_t n = M->lev[0].nnod;
  if (Visc) M3_CUDA(cudaMemcpyAsync(Visc, M->fin.visc, n * sizeof(double), cudaMemcpyDeviceToHost, M->stream));
  if (Dens) M3_CUDA(cudaMemcpyAsync(Dens, M->fin.dens, n * sizeof(double), cudaMemcpyDeviceToHost, M->stream));
  M3_CUDA(cudaStreamSynchronize(M->stream));
  return M3SPH_OK;
}

extern "C" int m3sph_set_pressure(m3sph_mesh *M, const double *P) {
  if (!M || !P || !M->have_operator) {
    set_error("m3sph_set_pressure: call m3sph_stokes_setup first");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  M3_TRY(stokes_set_pressure(M, P));
  M->ts_steps = std::max<long long>(M->ts_steps, 1);   // the next time step starts from this pressure
  return M3SPH_OK;
}

extern "C" int m3sph_time_step(m3sph_mesh *M, const m3sph_step_opts *o, m3sph_step_info *info) {
  if (!M || !o) {
    set_error("m3sph_time_step: bad arguments");
    return M3SPH_ERR_BAD_INPUT;
  }
  if (!M->have_operator || !M->T) {
    set_error("m3sph_time_step: call m3sph_stokes_setup and m3sph_set_temperature first");
    return M3SPH_ERR_BAD_INPUT;
  }
  if ((o->stokes.precision ? 1 : 0) != M->precision) {
    set_error("m3sph_time_step: opts.stokes.precision differs from the set-up's");
    return M3SPH_ERR_BAD_INPUT;
  }
  M3_CUDA(cudaSetDevice(M->device));
  cudaStream_t s = M->stream;
  m3sph_step_info inf{};
  cudaEvent_t ev[5];
  for (auto &e : ev) M3_CUDA(cudaEventCreate(&e));
  struct Guard {
    cudaEvent_t *e;
    ~Guard() { for (int i = 0; i < 5; ++i) cudaEventDestroy(e[i]); }
  } guard{ev};
  M3_CUDA(cudaEventRecord(ev[0], s));
  // UPDATE VISCOSITY AND DENSITY (rock_prop)
  if (o->rock_prop) {
    M3_TRY(rock_prop_device(M, &o->rock, M->T, M->fin.visc, M->fin.dens));
    M3_TRY(ml_features(M, nullptr));
  }
  M3_CUDA(cudaEventRecord(ev[1], s));
  // SOLVE FOR VISCOUS FLOW: first step from P = 0, later ones from the previous pressure
  const int st = stokes_resident_solve(M, &o->stokes, M->ts_steps == 0, inf.stokes);
  if (st && st != M3SPH_ERR_NOT_CONVERGED) return st;
  M3_CUDA(cudaEventRecord(ev[2], s));
  // CALCULATE TIME STEP
  M3_TRY(stokes_calc_dt(M, o->dt_adv_limit, o->dtmax, &inf.dt, &inf.dt_adv));
  M3_CUDA(cudaEventRecord(ev[3], s));
  // THERMAL ADVECTION-DIFFUSION in the new velocity (thermal_advdiff_3d_p.m)
  double t_diff = 0.0;
  auto half_step = [&](void) -> int {
    if (!o->diffusion) return M3SPH_OK;
    const auto h0 = std::chrono::steady_clock::now();
    int it = 0;
    const int r = diffusion_resident(M, M->T, 0.5 * inf.dt, &it);
    inf.diffusion_its += it;
    t_diff += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - h0).count();
    return r;
  };
  M3_TRY(half_step());
  M3_TRY(stokes_velocity_soa(M, M->Usoa));
  M3_TRY(slm_advect_resident(M, M->Usoa, M->T, inf.dt, &o->slm, M->ts_steps == 0, &inf.locate));
  M3_TRY(half_step());
  M3_CUDA(cudaEventRecord(ev[4], s));
  M3_CUDA(cudaEventSynchronize(ev[4]));
  inf.t_diffusion_ms = t_diff;
  M3_TRY(elapsed(ev[0], ev[1], inf.t_rock_ms));
  M3_TRY(elapsed(ev[1], ev[2], inf.t_stokes_ms));
  M3_TRY(elapsed(ev[2], ev[3], inf.t_dt_ms));
  M3_TRY(elapsed(ev[3], ev[4], inf.t_advect_ms));
  M3_TRY(elapsed(ev[0], ev[4], inf.t_total_ms));
  M->ts_steps++;
  M->ts_time += inf.dt;
  inf.time = M->ts_time;
  inf.status = st;
  if (info) *info = inf;
  if (st) set_error("m3sph_time_step: Patera iteration not converged in this step");
  return st;
}
