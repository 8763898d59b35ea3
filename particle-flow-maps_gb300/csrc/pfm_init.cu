// Initial-condition kernels used to set up large scenes on the device: the vortex-ring
// Biot-Savart sum (add_vortex_ring, 3D/init_conditions.py:10-22; with the smoke marker,
// add_vortex_ring_and_smoke, 3D/init_conditions.py:29-56) and the centre-to-face split
// (split_central_vector, 3D/taichi_utils.py:87-100; 2D/taichi_utils.py:56-67).
#include "pfm_internal.cuh"

namespace pfm {

// vf[i,j,k] += sum_l curve_length * (-1/(4 pi r^3) * (1 - exp(-(r/delta)^3))) * (p - p_l) x w_l
// with p the cell centre (I + 0.5) * dx (center_coords_func, 3D/taichi_utils.py:28-31).
// SMOKE (add_vortex_ring_and_smoke, 3D/init_conditions.py:29-56, first loop) also adds
// curve_length * exp(-(r/delta)^3) to smoke[3] sample by sample; the velocity arithmetic is the
// same code in both forms, so their velocities are bitwise equal.
template <bool SMOKE>
__global__ void __launch_bounds__(256) k_vortex_ring(float* __restrict__ vc, float* __restrict__ smoke, MacGeom g,
                                                     float w, float rad, float delta, float3 c, float3 ux, float3 uy,
                                                     int num_samples) {
  const int64_t C = (int64_t)g.N[0] * g.N[1] * g.N[2];
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= C) return;
  int i, j, k;
  split3((unsigned)e, g.dN[1], g.dN[2], i, j, k);
  const float px = ((float)i + 0.5f) * g.dx, py = ((float)j + 0.5f) * g.dx, pz = ((float)k + 0.5f) * g.dx;
  const float pi = 3.14159265358979323846f;
  const float curve_length = (2.f * pi * rad) / (float)num_samples;
  float ax = 0.f, ay = 0.f, az = 0.f;
  float s3 = SMOKE ? smoke[e * 4 + 3] : 0.f;
  for (int l = 0; l < num_samples; ++l) {
    float theta = (float)l / (float)num_samples * 2.f * pi;
    float ct = cosf(theta), st = sinf(theta);
    float sx = rad * (ct * ux.x + st * uy.x) + c.x;
    float sy = rad * (ct * ux.y + st * uy.y) + c.y;
    float sz = rad * (ct * ux.z + st * uy.z) + c.z;
    float dx = px - sx, dy = py - sy, dz = pz - sz;
    float r = sqrtf(dx * dx + dy * dy + dz * dz);
    float wx = w * (-st * ux.x + ct * uy.x), wy = w * (-st * ux.y + ct * uy.y), wz = w * (-st * ux.z + ct * uy.z);
    float rd = r / delta;
    float ex = expf(-(rd * rd * rd));
    float f = curve_length * (-1.f / (4.f * pi * r * r * r) * (1.f - ex));
    ax += f * (dy * wz - dz * wy);
    ay += f * (dz * wx - dx * wz);
    az += f * (dx * wy - dy * wx);
    if (SMOKE) s3 += curve_length * ex;
  }
  vc[e * 3 + 0] += ax;
  vc[e * 3 + 1] += ay;
  vc[e * 3 + 2] += az;
  if (SMOKE) smoke[e * 4 + 3] = s3;
}

// add_vortex_ring_and_smoke, second loop: cells whose marker exceeds 0.002 become (color, 1),
// the others 0.
__global__ void __launch_bounds__(256) k_smoke_marker(float4* __restrict__ smoke, int64_t C, float3 color) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= C) return;
  const float4 s = smoke[e];
  smoke[e] = (s.w > 0.002f) ? make_float4(color.x, color.y, color.z, 1.f) : make_float4(0.f, 0.f, 0.f, 0.f);
}

// split_central_vector: face = 0.5 * (sample(vc, I) + sample(vc, I - e_fam)) with clamped samples
template <int D>
__global__ void __launch_bounds__(256) k_split_central(const float* __restrict__ vc, MacGeom g, int fam,
                                                       float* __restrict__ out) {
  const int n0 = g.n[fam][0], n1 = g.n[fam][1], n2 = g.n[fam][2];
  const int64_t nf = (int64_t)n0 * n1 * n2;
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nf) return;
  int idx[3];
  split3((unsigned)e, g.dn[fam][1], g.dn[fam][2], idx[0], idx[1], idx[2]);
  int a[3] = {idx[0], idx[1], idx[2]}, b[3] = {idx[0], idx[1], idx[2]};
  b[fam] -= 1;
  for (int d = 0; d < 3; ++d) {
    a[d] = a[d] < 0 ? 0 : (a[d] > g.N[d] - 1 ? g.N[d] - 1 : a[d]);
    b[d] = b[d] < 0 ? 0 : (b[d] > g.N[d] - 1 ? g.N[d] - 1 : b[d]);
  }
  const int64_t ea = ((int64_t)a[0] * g.N[1] + a[1]) * g.N[2] + a[2];
  const int64_t eb = ((int64_t)b[0] * g.N[1] + b[1]) * g.N[2] + b[2];
  out[e] = 0.5f * (vc[ea * D + fam] + vc[eb * D + fam]);
}

// Counter-based uniform in [0, 1) with 24 random bits (splitmix64 finaliser of seed and index).
__device__ __forceinline__ float hash_uniform(uint64_t seed, uint64_t n) {
  uint64_t z = seed * 0xD1B54A32D192ED03ull + n + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return (float)(z >> 40) * (1.0f / 16777216.0f);
}

// Stratified jittered seeding: every cell holds ppc = ppc_axis^D particles, one per sub-cell of a
// ppc_axis^D lattice, at (lattice index + U) * dx / ppc_axis.  Particle order: the lines of cells
// along the last axis one after another; each line in groups of kSeedGroup cells (the last group
// takes the remainder); inside a group, order [leading sub-indices][cell][last sub-index].  With 8
// particles per cell a warp's 32 particles are then 16 neighbouring cells along the last axis with
// the same leading sub-cell, so the rows their interpolation stencils read are shared by the whole
// warp: the RK4 kernel's gathers touch fewer cache lines per instruction than with the 8 particles
// of each cell consecutive (a warp then spans 4 cells and both halves of each, two rows per stencil
// row for the staggered components).
constexpr int kSeedGroup = 16;

template <int D>
__global__ void __launch_bounds__(256) k_seed_jittered(float* __restrict__ pos, int64_t P, MacGeom g, uint64_t seed,
                                                       int axis, float h_sub) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  const int nl = g.N[D - 1];                 // cells along the last axis
  const int ppc = axis * axis * (D == 3 ? axis : 1);
  const int64_t line_len = (int64_t)nl * ppc;
  const int64_t line = q / line_len;
  const int64_t rem = q - line * line_len;
  const int gi = (int)(rem / ((int64_t)kSeedGroup * ppc));
  const int r = (int)(rem - (int64_t)gi * kSeedGroup * ppc);
  const int k0 = gi * kSeedGroup;
  const int gsz = nl - k0 < kSeedGroup ? nl - k0 : kSeedGroup;
  const int s_last = r % axis;
  const int t = r / axis;
  const int kk = t % gsz;
  const int o = t / gsz;  // leading sub-indices
  int ci[3], si[3];
  if (D == 3) {
    ci[0] = (int)(line / g.N[1]);
    ci[1] = (int)(line - (int64_t)ci[0] * g.N[1]);
    ci[2] = k0 + kk;
    si[0] = o / axis;
    si[1] = o % axis;
    si[2] = s_last;
  } else {
    ci[0] = (int)line;
    ci[1] = k0 + kk;
    si[0] = o;
    si[1] = s_last;
  }
#pragma unroll
  for (int d = 0; d < D; ++d) {
    float lat = (float)(ci[d] * axis + si[d]);
    float u = hash_uniform(seed, (uint64_t)q * D + d);
    pos[d * P + q] = __fmul_rn(__fadd_rn(lat, u), h_sub);
  }
}

}  // namespace pfm

using namespace pfm;

extern "C" {

int pfm3_add_vortex_ring(pfm_handle* h, float w, float rad, float delta, const float c[3], const float unit_x[3],
                         const float unit_y[3], int num_samples, float* vc, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_add_vortex_ring on a 2D handle");
  if (!c || !unit_x || !unit_y || !vc) return set_error(h, PFM_ERR_NULL, "pfm3_add_vortex_ring: null input");
  if (num_samples < 1) return set_error(h, PFM_ERR_ARG, "pfm3_add_vortex_ring: num_samples < 1");
  launch(h, k_vortex_ring<false>, grid_for(h->cells, 256), 256, 0, (cudaStream_t)stream, vc, (float*)nullptr, h->geom,
         w, rad, delta, make_float3(c[0], c[1], c[2]), make_float3(unit_x[0], unit_x[1], unit_x[2]),
         make_float3(unit_y[0], unit_y[1], unit_y[2]), num_samples);
  return launch_check(h, "k_vortex_ring");
}

int pfm3_add_vortex_ring_and_smoke(pfm_handle* h, float w, float rad, float delta, const float c[3],
                                   const float unit_x[3], const float unit_y[3], const float color[3], int num_samples,
                                   float* vc, float* smoke, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_add_vortex_ring_and_smoke on a 2D handle");
  if (!c || !unit_x || !unit_y || !color || !vc || !smoke)
    return set_error(h, PFM_ERR_NULL, "pfm3_add_vortex_ring_and_smoke: null input");
  if (num_samples < 1) return set_error(h, PFM_ERR_ARG, "pfm3_add_vortex_ring_and_smoke: num_samples < 1");
  if (((uintptr_t)smoke) & 15) return set_error(h, PFM_ERR_ARG, "pfm3_add_vortex_ring_and_smoke: smoke not 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned gr = grid_for(h->cells, 256);
  launch(h, k_vortex_ring<true>, gr, 256, 0, st, vc, smoke, h->geom, w, rad, delta, make_float3(c[0], c[1], c[2]),
         make_float3(unit_x[0], unit_x[1], unit_x[2]), make_float3(unit_y[0], unit_y[1], unit_y[2]), num_samples);
  launch(h, k_smoke_marker, gr, 256, 0, st, reinterpret_cast<float4*>(smoke), h->cells,
         make_float3(color[0], color[1], color[2]));
  return launch_check(h, "k_vortex_ring<true>");
}

int pfm_split_central_vector(pfm_handle* h, const float* vc, float* u_x, float* u_y, float* u_z, void* stream) {
  if (!h) return PFM_ERR_NULL;
  const int D = h->cfg.dim;
  if (!vc || !u_x || !u_y || (D == 3 && !u_z)) return set_error(h, PFM_ERR_NULL, "pfm_split_central_vector: null");
  float* outs[3] = {u_x, u_y, u_z};
  for (int f = 0; f < D; ++f) {
    int64_t nf = (int64_t)h->geom.n[f][0] * h->geom.n[f][1] * h->geom.n[f][2];
    if (D == 3)
      launch(h, k_split_central<3>, grid_for(nf, 256), 256, 0, (cudaStream_t)stream, vc, h->geom, f, outs[f]);
    else
      launch(h, k_split_central<2>, grid_for(nf, 256), 256, 0, (cudaStream_t)stream, vc, h->geom, f, outs[f]);
  }
  return launch_check(h, "k_split_central");
}

int pfm_seed_jittered(pfm_handle* h, uint64_t seed, int ppc_axis, float* pos, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (!pos && h->P > 0) return set_error(h, PFM_ERR_NULL, "pfm_seed_jittered: null pos");
  if (ppc_axis < 1) return set_error(h, PFM_ERR_ARG, "pfm_seed_jittered: ppc_axis < 1");
  const int D = h->cfg.dim;
  int64_t ppc = (int64_t)ppc_axis * ppc_axis * (D == 3 ? ppc_axis : 1);
  if (h->P != ppc * h->cells) return set_error(h, PFM_ERR_SHAPE, "pfm_seed_jittered: particles != ppc * cells");
  if (h->P == 0) return PFM_OK;
  const float h_sub = (float)(h->cfg.dx / ppc_axis);
  if (D == 3)
    launch(h, k_seed_jittered<3>, grid_for(h->P, 256), 256, 0, (cudaStream_t)stream, pos, h->P, h->geom, seed,
           ppc_axis, h_sub);
  else
    launch(h, k_seed_jittered<2>, grid_for(h->P, 256), 256, 0, (cudaStream_t)stream, pos, h->P, h->geom, seed,
           ppc_axis, h_sub);
  return launch_check(h, "k_seed_jittered");
}

}  // extern "C"
