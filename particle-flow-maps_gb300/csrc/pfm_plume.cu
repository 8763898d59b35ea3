// The Boussinesq smoke plume that generates and evaluates the pressure warm start: a density
// source, semi-Lagrangian transport of the density, and the buoyancy force carried by the
// particles' impulse.  The reference solver has no external forces or plume; these kernels add
// them around its unchanged step.
//
// A force f acting over dt changes the impulse a particle carries now by f dt.  In the
// particle-flow-map step the impulse handed to P2G is M init_imp with M = cols(T_gm) cols(T_init)
// (3D/run_3D.py:462-475, the same composition update_T stores, 3D/run_3D.py:430-439), and M is
// the map accumulated up to the current time; adding M^-1 f dt to init_imp therefore adds f dt to
// the current impulse and lets the following RK4 steps transport it like the rest of the impulse.
// The force is applied at the start of a step (before the RK4), at the particles' positions.
#include "pfm_internal.cuh"

namespace pfm {

constexpr int kPlThreads = 256;

// trilinear sample of a cell-centred field at world position (x, y, z), clamped to the centres
__device__ __forceinline__ float sample_cells(const float* __restrict__ f, const MacGeom& g, float x, float y,
                                              float z) {
  const float s[3] = {x * g.inv_dx - 0.5f, y * g.inv_dx - 0.5f, z * g.inv_dx - 0.5f};
  int i0[3];
  float t[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float hi = (float)(g.N[a] - 1);
    const float c = fminf(fmaxf(s[a], 0.f), hi);
    int b = (int)floorf(c);
    if (b > g.N[a] - 2) b = g.N[a] - 2;
    if (b < 0) b = 0;
    i0[a] = b;
    t[a] = g.N[a] > 1 ? c - (float)b : 0.f;
  }
  const int N1 = g.N[1], N2 = g.N[2];
  const int i1 = min(i0[0] + 1, g.N[0] - 1), j1 = min(i0[1] + 1, N1 - 1), k1 = min(i0[2] + 1, N2 - 1);
  auto at = [&](int i, int j, int k) { return f[((int64_t)i * N1 + j) * N2 + k]; };
  const float c00 = at(i0[0], i0[1], i0[2]) * (1.f - t[2]) + at(i0[0], i0[1], k1) * t[2];
  const float c01 = at(i0[0], j1, i0[2]) * (1.f - t[2]) + at(i0[0], j1, k1) * t[2];
  const float c10 = at(i1, i0[1], i0[2]) * (1.f - t[2]) + at(i1, i0[1], k1) * t[2];
  const float c11 = at(i1, j1, i0[2]) * (1.f - t[2]) + at(i1, j1, k1) * t[2];
  const float c0 = c00 * (1.f - t[1]) + c01 * t[1];
  const float c1 = c10 * (1.f - t[1]) + c11 * t[1];
  return c0 * (1.f - t[0]) + c1 * t[0];
}

// rho = value inside the sphere |x - c| < radius (cell centres)
__global__ void __launch_bounds__(kPlThreads) k_plume_source(float* __restrict__ rho, MacGeom g, float cx, float cy,
                                                             float cz, float r2, float value) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)g.N[0] * g.N[1] * g.N[2]) return;
  int i, j, k;
  split3((unsigned)e, g.dN[1], g.dN[2], i, j, k);
  const float x = ((float)i + 0.5f) * g.dx - cx, y = ((float)j + 0.5f) * g.dx - cy, z = ((float)k + 0.5f) * g.dx - cz;
  if (x * x + y * y + z * z < r2) rho[e] = value;
}

// rho1(x) = rho0(x - dt u(x)), u the face average at the cell centre
__global__ void __launch_bounds__(kPlThreads) k_advect_density(const float* __restrict__ rho0, float* __restrict__ rho1,
                                                               const float* __restrict__ ux,
                                                               const float* __restrict__ uy,
                                                               const float* __restrict__ uz, MacGeom g, float dt) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)g.N[0] * g.N[1] * g.N[2]) return;
  int i, j, k;
  split3((unsigned)e, g.dN[1], g.dN[2], i, j, k);
  const int N1 = g.N[1], N2 = g.N[2];
  const float vx = 0.5f * (ux[((int64_t)i * N1 + j) * N2 + k] + ux[((int64_t)(i + 1) * N1 + j) * N2 + k]);
  const float vy = 0.5f * (uy[((int64_t)i * (N1 + 1) + j) * N2 + k] + uy[((int64_t)i * (N1 + 1) + j + 1) * N2 + k]);
  const float vz = 0.5f * (uz[((int64_t)i * N1 + j) * (N2 + 1) + k] + uz[((int64_t)i * N1 + j) * (N2 + 1) + k + 1]);
  const float x = ((float)i + 0.5f) * g.dx - dt * vx;
  const float y = ((float)j + 0.5f) * g.dx - dt * vy;
  const float z = ((float)k + 0.5f) * g.dx - dt * vz;
  rho1[e] = sample_cells(rho0, g, x, y, z);
}

// init_imp += M^-1 (coef rho(x_p) e_axis), M = cols(T_gm) cols(T_init); particles whose M is
// singular (|det| <= 1e-20) are left unchanged
__global__ void __launch_bounds__(kPlThreads) k_buoyancy_impulse(const float* __restrict__ pos,
                                                                 const float* __restrict__ Tgm,
                                                                 const float* __restrict__ Tin, float* __restrict__ imp,
                                                                 const float* __restrict__ rho, MacGeom g, int64_t P,
                                                                 float coef, int axis) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  const float f = coef * sample_cells(rho, g, pos[q], pos[P + q], pos[2 * P + q]);
  if (f == 0.f) return;
  // A[r][k] = cols(T_gm)[r][k] = T_gm vector k, component r; B likewise for T_init
  float A[3][3], B[3][3], M[3][3];
#pragma unroll
  for (int v = 0; v < 3; ++v)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      A[c][v] = Tgm[(v * 3 + c) * P + q];
      B[c][v] = Tin[(v * 3 + c) * P + q];
    }
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int s = 0; s < 3; ++s) M[r][s] = A[r][0] * B[0][s] + A[r][1] * B[1][s] + A[r][2] * B[2][s];
  // adjugate solve: delta = adj(M) (f e_axis) / det M = column `axis` of adj(M) times f / det
  const float c00 = M[1][1] * M[2][2] - M[1][2] * M[2][1];
  const float c01 = M[1][2] * M[2][0] - M[1][0] * M[2][2];
  const float c02 = M[1][0] * M[2][1] - M[1][1] * M[2][0];
  const float det = M[0][0] * c00 + M[0][1] * c01 + M[0][2] * c02;
  if (!(fabsf(det) > 1e-20f)) return;
  float adj_col[3];  // adj(M)[r][axis] = cofactor of M[axis][r]
  if (axis == 0) {
    adj_col[0] = c00;
    adj_col[1] = c01;
    adj_col[2] = c02;
  } else if (axis == 1) {
    adj_col[0] = M[0][2] * M[2][1] - M[0][1] * M[2][2];
    adj_col[1] = M[0][0] * M[2][2] - M[0][2] * M[2][0];
    adj_col[2] = M[0][1] * M[2][0] - M[0][0] * M[2][1];
  } else {
    adj_col[0] = M[0][1] * M[1][2] - M[0][2] * M[1][1];
    adj_col[1] = M[0][2] * M[1][0] - M[0][0] * M[1][2];
    adj_col[2] = M[0][0] * M[1][1] - M[0][1] * M[1][0];
  }
  const float s = f / det;
#pragma unroll
  for (int r = 0; r < 3; ++r) imp[r * P + q] += adj_col[r] * s;
}

}  // namespace pfm

using namespace pfm;

int pfm3_plume_source(pfm_handle* h, float* rho, float cx, float cy, float cz, float radius, float value,
                      void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_plume_source on a 2D handle");
  if (!rho) return set_error(h, PFM_ERR_NULL, "pfm3_plume_source: null rho");
  if (!(radius >= 0.f)) return set_error(h, PFM_ERR_ARG, "pfm3_plume_source: radius < 0");
  launch(h, k_plume_source, grid_for(h->cells, kPlThreads), kPlThreads, 0, (cudaStream_t)stream, rho, h->geom, cx, cy,
         cz, radius * radius, value);
  return launch_check(h, "k_plume_source");
}

int pfm3_advect_density(pfm_handle* h, const float* rho0, float* rho1, const float* u_x, const float* u_y,
                        const float* u_z, float dt, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_advect_density on a 2D handle");
  if (!rho0 || !rho1 || !u_x || !u_y || !u_z) return set_error(h, PFM_ERR_NULL, "pfm3_advect_density: null input");
  if (rho0 == rho1) return set_error(h, PFM_ERR_ARG, "pfm3_advect_density: rho0 and rho1 must not alias");
  launch(h, k_advect_density, grid_for(h->cells, kPlThreads), kPlThreads, 0, (cudaStream_t)stream, rho0, rho1, u_x,
         u_y, u_z, h->geom, dt);
  return launch_check(h, "k_advect_density");
}

int pfm3_add_buoyancy_impulse(pfm_handle* h, const float* pos, const float* T_gm, const float* T_init, float* init_imp,
                              const float* rho, float coef, int axis, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_add_buoyancy_impulse on a 2D handle");
  if (!pos || !T_gm || !T_init || !init_imp || !rho)
    return set_error(h, PFM_ERR_NULL, "pfm3_add_buoyancy_impulse: null input");
  if (axis < 0 || axis > 2) return set_error(h, PFM_ERR_ARG, "pfm3_add_buoyancy_impulse: axis not 0, 1 or 2");
  if (h->P == 0) return PFM_OK;
  launch(h, k_buoyancy_impulse, grid_for(h->P, kPlThreads), kPlThreads, 0, (cudaStream_t)stream, pos, T_gm, T_init,
         init_imp, rho, h->geom, h->P, coef, axis);
  return launch_check(h, "k_buoyancy_impulse");
}
