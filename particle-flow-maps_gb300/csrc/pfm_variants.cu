// Kernels of the reference's alternative ("evolve m" / grad-T) dataflow, which its live step does
// not call (their call sites in 3D/run_3D.py:795-808 are commented out):
//   * RK4_T_and_T_grad_m_forward (3D/run_3D.py:221-292): one RK4 that advances the positions and two
//     Jacobian sets (T and T_grad_m) with the same interpolated velocity gradient;
//   * update_particles_imp (3D/run_3D.py:395-401): imp = cols(T) @ init_imp;
//   * update_particles_grad_m (3D/run_3D.py:412-428): C_r = grad_T_init_r @ init_imp + (T^T C0 T)_r;
//   * compute_dT_dx (3D/run_3D.py:353-390): a particle-neighbourhood estimate of grad T_init.
// Particle layouts as in pfm.h: vectors [3][P], vector triples [3][3][P], and the per-particle
// 3x3 matrices grad_T_init_{x,y,z} as [3 (r)][3 (a)][3 (b)][P].
#include "pfm_internal.cuh"

namespace pfm {

constexpr int kVThreads = 128;

// RK4_T_and_T_grad_m_forward: the RK4 of RK4_T_forward applied to two Jacobian sets at once, with
// the reference's constants (half_dt = 0.5 dt, the third stage over dt, and the final step
// dt * f32(1/6), one_sixth = 1./6 in run_3D.py:21).
__global__ void __launch_bounds__(kVThreads) k_rk4_T2_forward3(float* __restrict__ pos, float* __restrict__ T,
                                                              float* __restrict__ T2, int64_t P, MacFields3 F,
                                                              MacGeom g, float dt) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  float p0[3] = {pos[q], pos[P + q], pos[2 * P + q]};
  float T0[2][3][3];
#pragma unroll
  for (int v = 0; v < 3; ++v)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T0[0][v][c] = T[(v * 3 + c) * P + q];
      T0[1][v][c] = T2[(v * 3 + c) * P + q];
    }
  float pk[3] = {p0[0], p0[1], p0[2]};
  float Tk[2][3][3], sT[2][3][3];
  float su[3];
#pragma unroll
  for (int s2 = 0; s2 < 2; ++s2)
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
      for (int c = 0; c < 3; ++c) Tk[s2][v][c] = T0[s2][v][c];
  const float half_dt = 0.5f * dt;
#pragma unroll 1
  for (int s = 0; s < 4; ++s) {
    float u[3], G[3][3];
    interp_mac3(F, g, pk, u, G, true);
    const float wgt = (s == 0 || s == 3) ? 1.f : 2.f;
    const float cdt = (s < 2) ? half_dt : dt;
#pragma unroll
    for (int c = 0; c < 3; ++c) su[c] = (s == 0) ? u[c] : su[c] + wgt * u[c];
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2)
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        float dT[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) dT[r] = G[0][r] * Tk[s2][v][0] + G[1][r] * Tk[s2][v][1] + G[2][r] * Tk[s2][v][2];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          sT[s2][v][c] = (s == 0) ? dT[c] : sT[s2][v][c] + wgt * dT[c];
          if (s < 3) Tk[s2][v][c] = T0[s2][v][c] - cdt * dT[c];
        }
      }
    if (s < 3) {
#pragma unroll
      for (int c = 0; c < 3; ++c) pk[c] = p0[c] + cdt * u[c];
    }
  }
  const float coef = dt * (float)(1.0 / 6.0);
#pragma unroll
  for (int c = 0; c < 3; ++c) pos[c * P + q] = p0[c] + coef * su[c];
#pragma unroll
  for (int v = 0; v < 3; ++v)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T[(v * 3 + c) * P + q] = T0[0][v][c] - coef * sT[0][v][c];
      T2[(v * 3 + c) * P + q] = T0[1][v][c] - coef * sT[1][v][c];
    }
}

// update_particles_imp (3D/run_3D.py:395-401): imp[r] = T_x[r] m0[0] + T_y[r] m0[1] + T_z[r] m0[2]
__global__ void __launch_bounds__(256) k_update_imp3(float* __restrict__ imp, const float* __restrict__ m0,
                                                     const float* __restrict__ T, int64_t P) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  const float a = m0[q], b = m0[P + q], c = m0[2 * P + q];
#pragma unroll
  for (int r = 0; r < 3; ++r) imp[r * P + q] = T[(0 * 3 + r) * P + q] * a + T[(1 * 3 + r) * P + q] * b + T[(2 * 3 + r) * P + q] * c;
}

// update_particles_grad_m (3D/run_3D.py:412-428): with A = rows(T), C_r = grad_T_init_r @ init_imp +
// (A^T (rows(init_C) A))[r, :]; gT may be null (grad_T_init = 0).
__global__ void __launch_bounds__(256) k_update_grad_m3(float* __restrict__ C, const float* __restrict__ C0,
                                                        const float* __restrict__ Tg, const float* __restrict__ gT,
                                                        const float* __restrict__ m0, int64_t P) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  float A[3][3], Cm[3][3], CA[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      A[r][c] = Tg[(r * 3 + c) * P + q];
      Cm[r][c] = C0[(r * 3 + c) * P + q];
    }
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) CA[r][c] = Cm[r][0] * A[0][c] + Cm[r][1] * A[1][c] + Cm[r][2] * A[2][c];
  const float m[3] = {m0[q], m0[P + q], m0[2 * P + q]};
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float tct = A[0][r] * CA[0][a] + A[1][r] * CA[1][a] + A[2][r] * CA[2][a];
      float gm = 0.f;
      if (gT) {
        const float* G = gT + (int64_t)((r * 3 + a) * 3) * P + q;
        gm = G[0] * m[0] + G[P] * m[1] + G[2 * P] * m[2];
      }
      C[(r * 3 + a) * P + q] = gm + tct;
    }
}

// compute_dT_dx (3D/run_3D.py:353-390).  For particle i with base cell int(x0_i / dx), the cells
// base - 1 .. base + 2 per axis (i, j, k order) and, in each, the first `cap` particles of its cell
// list (the bins of the sort of the current positions, particle-index order: the reference's
// sequential arrival order): with d = x0_n - x0_i in world units (as the reference writes it) and
// dw = (1/dx) (dN_2(d_x) N_2(d_y) N_2(d_z), N_2 dN_2 N_2, N_2 N_2 dN_2),
//   grad_T_init_r[a][b] += dw[a] * T_b(n)[r]   (T = cols(T_x, T_y, T_z) of the neighbour).
// Neighbour cells outside the grid are skipped (the reference indexes its fields out of range
// there).
__global__ void __launch_bounds__(kVThreads) k_compute_dT_dx3(const float* __restrict__ x0, const float* __restrict__ T,
                                                             const int* __restrict__ start,
                                                             const int* __restrict__ order, int64_t P, MacGeom g,
                                                             float inv_dx, int cap, float* __restrict__ gT) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  const float xi[3] = {x0[q], x0[P + q], x0[2 * P + q]};
  int base[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) base[a] = __float2int_rz(xi[a] / g.dx);
  float acc[3][3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) acc[r][a][b] = 0.f;
  for (int oi = -1; oi < 3; ++oi)
    for (int oj = -1; oj < 3; ++oj)
      for (int ok = -1; ok < 3; ++ok) {
        const int ci = base[0] + oi, cj = base[1] + oj, ck = base[2] + ok;
        if (ci < 0 || ci >= g.N[0] || cj < 0 || cj >= g.N[1] || ck < 0 || ck >= g.N[2]) continue;
        const int cell = (ci * g.N[1] + cj) * g.N[2] + ck;
        const int sb = start[cell];
        int se = start[cell + 1];
        if (se - sb > cap) se = sb + cap;
        for (int s = sb; s < se; ++s) {
          const int n = order[s];
          const float dxv = x0[n] - xi[0], dyv = x0[P + n] - xi[1], dzv = x0[2 * P + n] - xi[2];
          const float nx = N2(dxv), ny = N2(dyv), nz = N2(dzv);
          const float dw[3] = {inv_dx * dN2(dxv) * ny * nz, inv_dx * nx * dN2(dyv) * nz, inv_dx * nx * ny * dN2(dzv)};
#pragma unroll
          for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int r = 0; r < 3; ++r) {
              const float t = T[(b * 3 + r) * P + n];  // T[r][b] = T_b[r]
#pragma unroll
              for (int a = 0; a < 3; ++a) acc[r][a][b] += dw[a] * t;
            }
        }
      }
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) gT[((r * 3 + a) * 3 + b) * P + q] = acc[r][a][b];
}

static int need3(pfm_handle* h, const char* what) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, std::string(what) + " on a 2D handle");
  return PFM_OK;
}

}  // namespace pfm

using namespace pfm;

extern "C" {

int pfm3_rk4_T_and_T_grad_m_forward(pfm_handle* h, float* pos, float* T, float* T_grad_m, const float* u_x,
                                    const float* u_y, const float* u_z, float dt, void* stream) {
  int s = need3(h, "pfm3_rk4_T_and_T_grad_m_forward");
  if (s) return s;
  if (!u_x || !u_y || !u_z) return set_error(h, PFM_ERR_NULL, "pfm3_rk4_T_and_T_grad_m_forward: null grid");
  if (h->P == 0) return PFM_OK;
  if (!pos || !T || !T_grad_m) return set_error(h, PFM_ERR_NULL, "pfm3_rk4_T_and_T_grad_m_forward: null particle field");
  if (T == T_grad_m) return set_error(h, PFM_ERR_ARG, "pfm3_rk4_T_and_T_grad_m_forward: T and T_grad_m must not alias");
  const MacFields3 F{{u_x, u_y, u_z}};
  launch(h, k_rk4_T2_forward3, grid_for(h->P, kVThreads), kVThreads, 0, (cudaStream_t)stream, pos, T, T_grad_m, h->P, F,
         h->geom, dt);
  return launch_check(h, "k_rk4_T2_forward3");
}

int pfm3_update_imp(pfm_handle* h, float* imp, const float* init_imp, const float* T, void* stream) {
  int s = need3(h, "pfm3_update_imp");
  if (s) return s;
  if (h->P == 0) return PFM_OK;
  if (!imp || !init_imp || !T) return set_error(h, PFM_ERR_NULL, "pfm3_update_imp: null input");
  launch(h, k_update_imp3, grid_for(h->P, 256), 256, 0, (cudaStream_t)stream, imp, init_imp, T, h->P);
  return launch_check(h, "k_update_imp3");
}

int pfm3_update_grad_m(pfm_handle* h, float* C, const float* init_C, const float* T, const float* grad_T_init,
                       const float* init_imp, void* stream) {
  int s = need3(h, "pfm3_update_grad_m");
  if (s) return s;
  if (h->P == 0) return PFM_OK;
  if (!C || !init_C || !T || (grad_T_init && !init_imp))
    return set_error(h, PFM_ERR_NULL, "pfm3_update_grad_m: null input");
  launch(h, k_update_grad_m3, grid_for(h->P, 256), 256, 0, (cudaStream_t)stream, C, init_C, T, grad_T_init, init_imp,
         h->P);
  return launch_check(h, "k_update_grad_m3");
}

int pfm3_compute_dT_dx(pfm_handle* h, const float* pos, const float* init_pos, const float* T, int cap,
                       float* grad_T_init, void* stream) {
  int s = need3(h, "pfm3_compute_dT_dx");
  if (s) return s;
  if (cap < 0) return set_error(h, PFM_ERR_ARG, "pfm3_compute_dT_dx: cap < 0");
  if (h->P == 0) return PFM_OK;
  if (!pos || !init_pos || !T || !grad_T_init) return set_error(h, PFM_ERR_NULL, "pfm3_compute_dT_dx: null input");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = sort_particles(h, pos, st);
  if (rc) return rc;
  const float inv_dx = (float)(1.0 / h->cfg.dx);
  launch(h, k_compute_dT_dx3, grid_for(h->P, kVThreads), kVThreads, 0, st, init_pos, T, ws_ptr<int>(h, h->o_start),
         ws_ptr<int>(h, h->o_order), h->P, h->geom, inv_dx, cap, grad_T_init);
  return launch_check(h, "k_compute_dT_dx3");
}

}  // extern "C"
