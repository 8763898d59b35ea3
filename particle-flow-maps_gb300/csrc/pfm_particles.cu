// Per-particle kernels of the particle-flow-map step: G2P of velocity and its gradient, the
// flow-map Jacobian composition/reset, and the forward RK4 of positions and T.
// Particle fields are SoA ([n][P]); see include/pfm.h.
#include "pfm_internal.cuh"

namespace pfm {

constexpr int kPThreads = 128;
// Block size of the RK4 kernel and the resident blocks per SM it is compiled for.  64 threads x
// 10 blocks caps it at 96 registers (20 warps per SM; the cube-extent instances spill 8 bytes, and
// with a cap of 9 blocks the compiler still picks 96).  Measured at 256^3 (the gradient-reinit +
// RK4 + records kernel, strides read at run time): 128 x 4 (128 registers) 19.2 ms, 128 x 5
// 18.0 ms, 128 x 6 (80 registers, spills) 18.8 ms, 256 x 2 20.9 ms, 64 x 10 17.6 ms.
#ifndef PFM_RK4_MINB
#define PFM_RK4_MINB 10
#endif
#ifndef PFM_RK4_THREADS
#define PFM_RK4_THREADS 64
#endif
constexpr int kRK4Threads = PFM_RK4_THREADS;

// ---------------------------------------------------------------------------------------------
// 3D
// ---------------------------------------------------------------------------------------------

// init_particles_imp / init_particles_imp_grad_m (3D/init_conditions.py:254-273) via
// interp_u_MAC_grad_imp (3D/taichi_utils.py:371-376): imp = u(p); C rows = grad u_c(p)
// (new_C and the gradient are the same sum).
__global__ void __launch_bounds__(kPThreads) k_g2p3(const float* __restrict__ pos, int64_t P,
                                                   MacFields3 F, MacGeom g, float* __restrict__ imp,
                                                   float* __restrict__ C) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  float p[3] = {pos[q], pos[P + q], pos[2 * P + q]};
  float u[3], G[3][3];
  interp_mac3(F, g, p, u, G, true);
  if (imp) {
#pragma unroll
    for (int c = 0; c < 3; ++c) imp[c * P + q] = u[c];
  }
  if (C) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int r = 0; r < 3; ++r) C[(c * 3 + r) * P + q] = G[c][r];
  }
}

// update_T (3D/run_3D.py:430-439) + optional reset_T_to_identity of T_gm (3D/run_3D.py:133-140).
// cols(T_gm) @ cols(T_init): new T_init_c[r] = sum_k T_gm_k[r] * T_init_c[k].
__global__ void __launch_bounds__(256) k_update_T3(float* __restrict__ Ti, float* __restrict__ Tg,
                                                   int64_t P, int reset) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  float M[3][3], N[3][3];
#pragma unroll
  for (int v = 0; v < 3; ++v)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      M[c][v] = Tg[(v * 3 + c) * P + q];  // M[r][k] = T_gm_k[r]
      N[c][v] = Ti[(v * 3 + c) * P + q];  // N[k][c] = T_init_c[k]
    }
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r)
      Ti[(c * 3 + r) * P + q] = M[r][0] * N[0][c] + M[r][1] * N[1][c] + M[r][2] * N[2][c];
  if (reset) {
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
      for (int c = 0; c < 3; ++c) Tg[(v * 3 + c) * P + q] = (v == c) ? 1.f : 0.f;
  }
}

template <int D>
__global__ void __launch_bounds__(256) k_reset_T(float* __restrict__ T, int64_t P) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
#pragma unroll
  for (int v = 0; v < D; ++v)
#pragma unroll
    for (int c = 0; c < D; ++c) T[(v * D + c) * P + q] = (v == c) ? 1.f : 0.f;
}

// RK4_T_forward (3D/run_3D.py:175-219): the gradient is taken in the transpose form
// (interp_u_MAC_grad_transpose, 3D/taichi_utils.py:319-324), so dT_v/dt[r] = sum_c du_c/dx_r T_v[c].
// The stage sums (k1 + 2 k2 + 2 k3 + k4) accumulate in the reference's left-to-right order.
// With PAY the kernel also writes the P2G record and cell key of the advected particle
// (write_p2g_record3), the input of the P2G tiles that follow RK4_T_forward in the step.
// With GRADM it first does the flow-map gradient reinitialisation of the step
// (3D/run_3D.py:768-772): init_C rows = grad u(p) in the velocity Fg (init_particles_imp_grad_m,
// as k_g2p3), T_init <- cols(T_gm) @ cols(T_init) (update_T, as k_update_T3) and T_gm <- I, so the
// RK4 starts from the identity without reading T_gm back.
// NC: the grid's cube extent when the interpolation is compiled for it (interp_mac3_taps<NC>), else 0.
template <bool PAY, bool GRADM, int NC>
__global__ void __launch_bounds__(kRK4Threads, PFM_RK4_MINB) k_rk4_T_forward3(float* __restrict__ pos, float* __restrict__ T,
                                                             int64_t P, MacFields3 F, MacGeom g, float dt,
                                                             P2GRecords3 R, MacFields3 Fg,
                                                             const float* __restrict__ dt_dev) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  if (dt_dev) dt = *dt_dev;  // the whole-step graph keeps dt on the device
  float p0[3] = {ld_stream(pos + q), ld_stream(pos + P + q), ld_stream(pos + 2 * P + q)};
  float T0[3][3];
  float u[3], G[3][3];  // the RK4 stage's velocity and gradient
  if (GRADM) {
    {
      // grad u(p0) of the pre-midpoint velocity and the first RK4 stage's u_mid(p0) share their
      // taps, and their loads are independent: both gathers are issued together
      Axis3 A0[3], A1[3];
      mac_taps3(g, p0, A0, A1);
      float ug[3], Gg[3][3];
      interp_mac3_taps<NC>(Fg, g, A0, A1, ug, Gg, true);
      interp_mac3_taps<NC>(F, g, A0, A1, u, G, true);
      float* C = const_cast<float*>(R.C);
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) C[(c * 3 + r) * P + q] = Gg[c][r];
    }
    float* Ti = const_cast<float*>(R.Ti);
    float M[3][3], N[3][3];
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        M[c][v] = ld_stream(T + (v * 3 + c) * P + q);   // M[r][k] = T_gm_k[r]
        N[c][v] = ld_stream(Ti + (v * 3 + c) * P + q);  // N[k][c] = T_init_c[k]
      }
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int r = 0; r < 3; ++r)
        Ti[(c * 3 + r) * P + q] = M[r][0] * N[0][c] + M[r][1] * N[1][c] + M[r][2] * N[2][c];
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
      for (int c = 0; c < 3; ++c) T0[v][c] = (v == c) ? 1.f : 0.f;
  } else {
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
      for (int c = 0; c < 3; ++c) T0[v][c] = ld_stream(T + (v * 3 + c) * P + q);
  }
  float pk[3] = {p0[0], p0[1], p0[2]};
  float Tk[3][3];
#pragma unroll
  for (int v = 0; v < 3; ++v)
#pragma unroll
    for (int c = 0; c < 3; ++c) Tk[v][c] = T0[v][c];
  float su[3] = {0.f, 0.f, 0.f}, sT[3][3];
#pragma unroll
  for (int v = 0; v < 3; ++v)
#pragma unroll
    for (int c = 0; c < 3; ++c) sT[v][c] = 0.f;
  const float half_dt = 0.5f * dt;
#pragma unroll 1
  for (int s = 0; s < 4; ++s) {
    if (!GRADM || s > 0) interp_mac3<NC>(F, g, pk, u, G, true);
    float dT[3][3];
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
      for (int r = 0; r < 3; ++r) dT[v][r] = G[0][r] * Tk[v][0] + G[1][r] * Tk[v][1] + G[2][r] * Tk[v][2];
    const float wgt = (s == 0 || s == 3) ? 1.f : 2.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) su[c] = (s == 0) ? u[c] : su[c] + wgt * u[c];
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
      for (int c = 0; c < 3; ++c) sT[v][c] = (s == 0) ? dT[v][c] : sT[v][c] + wgt * dT[v][c];
    if (s < 3) {
      const float cdt = (s < 2) ? half_dt : dt;
#pragma unroll
      for (int c = 0; c < 3; ++c) pk[c] = p0[c] + cdt * u[c];
#pragma unroll
      for (int v = 0; v < 3; ++v)
#pragma unroll
        for (int c = 0; c < 3; ++c) Tk[v][c] = T0[v][c] - cdt * dT[v][c];
    }
  }
  const float coef = dt / 6.f;
  float pn[3], Tn[3][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    pn[c] = p0[c] + coef * su[c];
    st_stream(pos + c * P + q, pn[c]);
  }
#pragma unroll
  for (int v = 0; v < 3; ++v)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Tn[v][c] = T0[v][c] - coef * sT[v][c];
      st_stream(T + (v * 3 + c) * P + q, Tn[v][c]);
    }
  if (PAY) {
    const float v[3] = {pn[0] / g.dx, pn[1] / g.dx, pn[2] / g.dx};
    write_p2g_record3(R, q, P, g, v, Tn);
  }
}

// ---------------------------------------------------------------------------------------------
// 2D
// ---------------------------------------------------------------------------------------------

// init_particles_imp / _grad_m (2D/init_conditions.py:184-210)
__global__ void __launch_bounds__(kPThreads) k_g2p2(const float* __restrict__ pos, int64_t P, MacFields2 F,
                                                   MacGeom g, float* __restrict__ imp, float* __restrict__ C) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  float p[2] = {pos[q], pos[P + q]};
  float u[2], G[2][2];
  interp_mac2(F, g, p, u, G);
  if (imp) {
    imp[q] = u[0];
    imp[P + q] = u[1];
  }
  if (C) {
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
      for (int r = 0; r < 2; ++r) C[(c * 2 + r) * P + q] = G[c][r];
  }
}

// RK4_T_forward 2D (2D/run_2D.py:304-341): interp_u_MAC_grad (rows) then grad^T @ T.
__global__ void __launch_bounds__(kPThreads) k_rk4_T_forward2(float* __restrict__ pos, float* __restrict__ T,
                                                             int64_t P, MacFields2 F, MacGeom g, float dt,
                                                             int advect_psi, const float* __restrict__ dt_dev) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  if (dt_dev) dt = *dt_dev;
  float p0[2] = {pos[q], pos[P + q]};
  float T0[2][2] = {{T[q], T[P + q]}, {T[2 * P + q], T[3 * P + q]}};
  float pk[2] = {p0[0], p0[1]};
  float Tk[2][2] = {{T0[0][0], T0[0][1]}, {T0[1][0], T0[1][1]}};
  float su[2] = {0.f, 0.f}, sT[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
  const float half_dt = 0.5f * dt;
#pragma unroll 1
  for (int s = 0; s < 4; ++s) {
    float u[2], G[2][2];
    interp_mac2(F, g, pk, u, G);
    float dT[2][2];
#pragma unroll
    for (int v = 0; v < 2; ++v)
#pragma unroll
      for (int r = 0; r < 2; ++r) dT[v][r] = G[0][r] * Tk[v][0] + G[1][r] * Tk[v][1];
    const float wgt = (s == 0 || s == 3) ? 1.f : 2.f;
#pragma unroll
    for (int c = 0; c < 2; ++c) su[c] = (s == 0) ? u[c] : su[c] + wgt * u[c];
#pragma unroll
    for (int v = 0; v < 2; ++v)
#pragma unroll
      for (int c = 0; c < 2; ++c) sT[v][c] = (s == 0) ? dT[v][c] : sT[v][c] + wgt * dT[v][c];
    if (s < 3) {
      const float cdt = (s < 2) ? half_dt : dt;
#pragma unroll
      for (int c = 0; c < 2; ++c) pk[c] = p0[c] + cdt * u[c];
#pragma unroll
      for (int v = 0; v < 2; ++v)
#pragma unroll
        for (int c = 0; c < 2; ++c) Tk[v][c] = T0[v][c] - cdt * dT[v][c];
    }
  }
  const float coef = dt / 6.f;
  if (advect_psi) {
    pos[q] = p0[0] + coef * su[0];
    pos[P + q] = p0[1] + coef * su[1];
  }
#pragma unroll
  for (int v = 0; v < 2; ++v)
#pragma unroll
    for (int c = 0; c < 2; ++c) T[(v * 2 + c) * P + q] = T0[v][c] - coef * sT[v][c];
}

// update_particles_grad_m (2D/run_2D.py:526-536): C = cols(T) @ (rows(C0) @ rows(T))
__global__ void __launch_bounds__(256) k_update_grad_m2(float* __restrict__ C, const float* __restrict__ C0,
                                                        const float* __restrict__ Tg, int64_t P) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  float A[2][2], Cm[2][2];
#pragma unroll
  for (int v = 0; v < 2; ++v)
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      A[v][c] = Tg[(v * 2 + c) * P + q];   // rows(T): A[r][c] = T_r[c]
      Cm[v][c] = C0[(v * 2 + c) * P + q];  // rows(C0)
    }
  float CA[2][2];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 2; ++c) CA[r][c] = Cm[r][0] * A[0][c] + Cm[r][1] * A[1][c];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 2; ++c) C[(r * 2 + c) * P + q] = A[0][r] * CA[0][c] + A[1][r] * CA[1][c];
}

// update_T 2D (2D/run_2D.py:538-546): T = cols(T_gm) @ cols(T_init)
__global__ void __launch_bounds__(256) k_update_T2(float* __restrict__ T, const float* __restrict__ Ti,
                                                   const float* __restrict__ Tg, int64_t P) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  float M[2][2], N[2][2];
#pragma unroll
  for (int v = 0; v < 2; ++v)
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      M[c][v] = Tg[(v * 2 + c) * P + q];
      N[c][v] = Ti[(v * 2 + c) * P + q];
    }
#pragma unroll
  for (int c = 0; c < 2; ++c)
#pragma unroll
    for (int r = 0; r < 2; ++r) T[(c * 2 + r) * P + q] = M[r][0] * N[0][c] + M[r][1] * N[1][c];
}

// update_particles_imp 2D (2D/run_2D.py:517-524): imp = cols(T_x, T_y) @ init_imp
__global__ void __launch_bounds__(256) k_update_imp2(float* __restrict__ imp, const float* __restrict__ m0,
                                                     const float* __restrict__ T, int64_t P) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  float a = m0[q], b = m0[P + q];
  imp[q] = T[q] * a + T[2 * P + q] * b;
  imp[P + q] = T[P + q] * a + T[3 * P + q] * b;
}

static int check_dim(pfm_handle* h, int D) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != D) return set_error(h, PFM_ERR_SHAPE, "handle dimension does not match the call");
  return PFM_OK;
}

}  // namespace pfm

using namespace pfm;

namespace pfm {

int launch_rk4_T_forward3(pfm_handle* h, float* pos, float* T, const MacFields3& F, float dt, const P2GRecords3* R,
                          const MacFields3* Fg, cudaStream_t st, const float* dt_dev) {
  if (h->P == 0) return PFM_OK;
  const unsigned nb = grid_for(h->P, kRK4Threads);
  with_cube(h, [&](auto nc) {
    constexpr int NC = decltype(nc)::value;
    if (R && Fg)
      launch(h, k_rk4_T_forward3<true, true, NC>, nb, kRK4Threads, 0, st, pos, T, h->P, F, h->geom, dt, *R, *Fg,
             dt_dev);
    else if (R)
      launch(h, k_rk4_T_forward3<true, false, NC>, nb, kRK4Threads, 0, st, pos, T, h->P, F, h->geom, dt, *R,
             MacFields3{}, dt_dev);
    else
      launch(h, k_rk4_T_forward3<false, false, NC>, nb, kRK4Threads, 0, st, pos, T, h->P, F, h->geom, dt,
             P2GRecords3{}, MacFields3{}, dt_dev);
  });
  return launch_check(h, "k_rk4_T_forward3");
}

int launch_rk4_T_forward2(pfm_handle* h, float* pos, float* T, const MacFields2& F, float dt, int advect_psi,
                          cudaStream_t st, const float* dt_dev) {
  if (h->P == 0) return PFM_OK;
  launch(h, k_rk4_T_forward2, grid_for(h->P, kPThreads), kPThreads, 0, st, pos, T, h->P, F, h->geom, dt, advect_psi,
         dt_dev);
  return launch_check(h, "k_rk4_T_forward2");
}

}  // namespace pfm

extern "C" {

int pfm3_g2p(pfm_handle* h, const float* pos, const float* u_x, const float* u_y, const float* u_z,
             float* imp_out, float* C_out, void* stream) {
  int s = check_dim(h, 3);
  if (s) return s;
  if (!pos || !u_x || !u_y || !u_z) return set_error(h, PFM_ERR_NULL, "pfm3_g2p: null input");
  if (h->P == 0 || (!imp_out && !C_out)) return PFM_OK;
  MacFields3 F{{u_x, u_y, u_z}};
  launch(h, k_g2p3, grid_for(h->P, kPThreads), kPThreads, 0, (cudaStream_t)stream, pos, h->P, F, h->geom, imp_out, C_out);
  return launch_check(h, "k_g2p3");
}

int pfm3_update_T(pfm_handle* h, float* T_init, float* T_gm, int reset_gm, void* stream) {
  int s = check_dim(h, 3);
  if (s) return s;
  if (!T_init || !T_gm) return set_error(h, PFM_ERR_NULL, "pfm3_update_T: null input");
  if (h->P == 0) return PFM_OK;
  launch(h, k_update_T3, grid_for(h->P, 256), 256, 0, (cudaStream_t)stream, T_init, T_gm, h->P, reset_gm);
  return launch_check(h, "k_update_T3");
}

int pfm3_reset_T(pfm_handle* h, float* T, void* stream) {
  int s = check_dim(h, 3);
  if (s) return s;
  if (!T) return set_error(h, PFM_ERR_NULL, "pfm3_reset_T: null input");
  if (h->P == 0) return PFM_OK;
  launch(h, k_reset_T<3>, grid_for(h->P, 256), 256, 0, (cudaStream_t)stream, T, h->P);
  return launch_check(h, "k_reset_T<3>");
}

int pfm3_rk4_T_forward(pfm_handle* h, float* pos, float* T, const float* u_x, const float* u_y,
                       const float* u_z, float dt, void* stream) {
  int s = check_dim(h, 3);
  if (s) return s;
  if (!pos || !T || !u_x || !u_y || !u_z) return set_error(h, PFM_ERR_NULL, "pfm3_rk4_T_forward: null input");
  if (h->P == 0) return PFM_OK;
  MacFields3 F{{u_x, u_y, u_z}};
  return launch_rk4_T_forward3(h, pos, T, F, dt, nullptr, nullptr, (cudaStream_t)stream);
}

int pfm2_g2p(pfm_handle* h, const float* pos, const float* u_x, const float* u_y, float* imp_out,
             float* C_out, void* stream) {
  int s = check_dim(h, 2);
  if (s) return s;
  if (!pos || !u_x || !u_y) return set_error(h, PFM_ERR_NULL, "pfm2_g2p: null input");
  if (h->P == 0 || (!imp_out && !C_out)) return PFM_OK;
  MacFields2 F{{u_x, u_y}};
  launch(h, k_g2p2, grid_for(h->P, kPThreads), kPThreads, 0, (cudaStream_t)stream, pos, h->P, F, h->geom, imp_out, C_out);
  return launch_check(h, "k_g2p2");
}

int pfm2_rk4_T_forward(pfm_handle* h, float* pos, float* T, const float* u_x, const float* u_y, float dt,
                       int advect_psi, void* stream) {
  int s = check_dim(h, 2);
  if (s) return s;
  if (!pos || !T || !u_x || !u_y) return set_error(h, PFM_ERR_NULL, "pfm2_rk4_T_forward: null input");
  if (h->P == 0) return PFM_OK;
  MacFields2 F{{u_x, u_y}};
  launch(h, k_rk4_T_forward2, grid_for(h->P, kPThreads), kPThreads, 0, (cudaStream_t)stream, pos, T, h->P, F, h->geom,
         dt, advect_psi, (const float*)nullptr);
  return launch_check(h, "k_rk4_T_forward2");
}

int pfm2_update_grad_m(pfm_handle* h, float* C, const float* init_C, const float* T_gm, void* stream) {
  int s = check_dim(h, 2);
  if (s) return s;
  if (!C || !init_C || !T_gm) return set_error(h, PFM_ERR_NULL, "pfm2_update_grad_m: null input");
  if (h->P == 0) return PFM_OK;
  launch(h, k_update_grad_m2, grid_for(h->P, 256), 256, 0, (cudaStream_t)stream, C, init_C, T_gm, h->P);
  return launch_check(h, "k_update_grad_m2");
}

int pfm2_update_T(pfm_handle* h, float* T, const float* T_init, const float* T_gm, void* stream) {
  int s = check_dim(h, 2);
  if (s) return s;
  if (!T || !T_init || !T_gm) return set_error(h, PFM_ERR_NULL, "pfm2_update_T: null input");
  if (h->P == 0) return PFM_OK;
  launch(h, k_update_T2, grid_for(h->P, 256), 256, 0, (cudaStream_t)stream, T, T_init, T_gm, h->P);
  return launch_check(h, "k_update_T2");
}

int pfm2_update_imp(pfm_handle* h, float* imp, const float* init_imp, const float* T, void* stream) {
  int s = check_dim(h, 2);
  if (s) return s;
  if (!imp || !init_imp || !T) return set_error(h, PFM_ERR_NULL, "pfm2_update_imp: null input");
  if (h->P == 0) return PFM_OK;
  launch(h, k_update_imp2, grid_for(h->P, 256), 256, 0, (cudaStream_t)stream, imp, init_imp, T, h->P);
  return launch_check(h, "k_update_imp2");
}

int pfm2_reset_T(pfm_handle* h, float* T, void* stream) {
  int s = check_dim(h, 2);
  if (s) return s;
  if (!T) return set_error(h, PFM_ERR_NULL, "pfm2_reset_T: null input");
  if (h->P == 0) return PFM_OK;
  launch(h, k_reset_T<2>, grid_for(h->P, 256), 256, 0, (cudaStream_t)stream, T, h->P);
  return launch_check(h, "k_reset_T<2>");
}

}  // extern "C"
