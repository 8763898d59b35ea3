// Scalar (smoke) transport and the vorticity diagnostics of the particle-flow-map solver:
//   * init_particles_smoke (3D/init_conditions.py:275-279): G2P of the 4-channel cell-centred smoke
//     and its gradient (interp_grad_2_smoke, 3D/taichi_utils.py:379-420);
//   * advect_smoke / clamp_smoke (3D/run_3D.py:315-334; 2D/run_2D.py:444-450): semi-Lagrangian
//     transport of a cell field through the face-averaged backward map, trilinear
//     (interp_1 / sample_min_max_1, 3D/taichi_utils.py:192-250; 2D/taichi_utils.py:118-143);
//   * get_central_vector and curl (3D/taichi_utils.py:56-85; 2D/taichi_utils.py:50-55, 96-104).
// Smoke grids are AoS like the reference's vector fields: [nx][ny][nz][4] (3D), [nx][ny][3] (2D),
// so one 3D cell is one 16-byte load.  P2G_smoke lives with the other P2G kernels (pfm_p2g.cu).
// The grid kernels here are HBM-bound stencils (one pass over their inputs and outputs).
#include "pfm_internal.cuh"

namespace pfm {

constexpr int kFThreads = 256;

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ int64_t cell3(const MacGeom& g, int i, int j, int k) {
  return ((int64_t)i * g.N[1] + j) * g.N[2] + k;
}

// ---------------------------------------------------------------------------------------------
// diagnostics
// ---------------------------------------------------------------------------------------------

// get_central_vector (3D/taichi_utils.py:80-85): vc = average of the two faces of each cell.
__global__ void __launch_bounds__(kFThreads) k_central3(const float* __restrict__ ux, const float* __restrict__ uy,
                                                        const float* __restrict__ uz, MacGeom g,
                                                        float* __restrict__ vc) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)g.N[0] * g.N[1] * g.N[2]) return;
  int i, j, k;
  split3((unsigned)e, g.dN[1], g.dN[2], i, j, k);
  const int N1 = g.N[1], N2 = g.N[2];
  const float a = ux[((int64_t)(i + 1) * N1 + j) * N2 + k], b = ux[((int64_t)i * N1 + j) * N2 + k];
  const float c = uy[((int64_t)i * (N1 + 1) + j + 1) * N2 + k], d = uy[((int64_t)i * (N1 + 1) + j) * N2 + k];
  const float f = uz[((int64_t)i * N1 + j) * (N2 + 1) + k + 1], h = uz[((int64_t)i * N1 + j) * (N2 + 1) + k];
  vc[e * 3 + 0] = 0.5f * (a + b);
  vc[e * 3 + 1] = 0.5f * (c + d);
  vc[e * 3 + 2] = 0.5f * (f + h);
}

// curl (3D/taichi_utils.py:56-78): central differences of the cell-centred vc, indices clamped
// by sample(); inv_dist = f32(1 / f32(2 dx)).  Products are rounded before the differences.
__global__ void __launch_bounds__(kFThreads) k_curl3(const float* __restrict__ vc, MacGeom g, float inv_dist,
                                                     float* __restrict__ w) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)g.N[0] * g.N[1] * g.N[2]) return;
  int i, j, k;
  split3((unsigned)e, g.dN[1], g.dN[2], i, j, k);
  const int m0 = g.N[0] - 1, m1 = g.N[1] - 1, m2 = g.N[2] - 1;
  const float* vr = vc + 3 * cell3(g, clampi(i + 1, 0, m0), j, k);
  const float* vl = vc + 3 * cell3(g, clampi(i - 1, 0, m0), j, k);
  const float* vt = vc + 3 * cell3(g, i, clampi(j + 1, 0, m1), k);
  const float* vb = vc + 3 * cell3(g, i, clampi(j - 1, 0, m1), k);
  const float* vf = vc + 3 * cell3(g, i, j, clampi(k + 1, 0, m2));
  const float* va = vc + 3 * cell3(g, i, j, clampi(k - 1, 0, m2));
  const float d_vx_dz = __fmul_rn(inv_dist, vf[0] - va[0]);
  const float d_vx_dy = __fmul_rn(inv_dist, vt[0] - vb[0]);
  const float d_vy_dx = __fmul_rn(inv_dist, vr[1] - vl[1]);
  const float d_vy_dz = __fmul_rn(inv_dist, vf[1] - va[1]);
  const float d_vz_dx = __fmul_rn(inv_dist, vr[2] - vl[2]);
  const float d_vz_dy = __fmul_rn(inv_dist, vt[2] - vb[2]);
  w[e * 3 + 0] = d_vz_dy - d_vy_dz;
  w[e * 3 + 1] = d_vx_dz - d_vz_dx;
  w[e * 3 + 2] = d_vy_dx - d_vx_dy;
}

// get_central_vector (2D/taichi_utils.py:50-55)
__global__ void __launch_bounds__(kFThreads) k_central2(const float* __restrict__ ux, const float* __restrict__ uy,
                                                        MacGeom g, float* __restrict__ vc) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)g.N[0] * g.N[1]) return;
  const int i = (int)udiv((unsigned)e, g.dN[1]), j = (int)((unsigned)e - (unsigned)i * (unsigned)g.N[1]);
  const int N1 = g.N[1];
  vc[e * 2 + 0] = 0.5f * (ux[(int64_t)(i + 1) * N1 + j] + ux[(int64_t)i * N1 + j]);
  vc[e * 2 + 1] = 0.5f * (uy[(int64_t)i * (N1 + 1) + j + 1] + uy[(int64_t)i * (N1 + 1) + j]);
}

// curl (2D/taichi_utils.py:96-104): w = (vr.y - vl.y - vt.x + vb.x) / (2 dx), left to right.
__global__ void __launch_bounds__(kFThreads) k_curl2(const float* __restrict__ vc, MacGeom g, float two_dx,
                                                     float* __restrict__ w) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)g.N[0] * g.N[1]) return;
  const int i = (int)udiv((unsigned)e, g.dN[1]), j = (int)((unsigned)e - (unsigned)i * (unsigned)g.N[1]);
  const int m0 = g.N[0] - 1, m1 = g.N[1] - 1, N1 = g.N[1];
  const float* vl = vc + 2 * ((int64_t)clampi(i - 1, 0, m0) * N1 + j);
  const float* vr = vc + 2 * ((int64_t)clampi(i + 1, 0, m0) * N1 + j);
  const float* vb = vc + 2 * ((int64_t)i * N1 + clampi(j - 1, 0, m1));
  const float* vt = vc + 2 * ((int64_t)i * N1 + clampi(j + 1, 0, m1));
  w[e] = (((vr[1] - vl[1]) - vt[0]) + vb[0]) / two_dx;
}

// ---------------------------------------------------------------------------------------------
// smoke
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ float4 f4fma(float a, float4 v, float4 acc) {
  return make_float4(fmaf(a, v.x, acc.x), fmaf(a, v.y, acc.y), fmaf(a, v.z, acc.z), fmaf(a, v.w, acc.w));
}
__device__ __forceinline__ float4 f4mul(float a, float4 v) { return make_float4(a * v.x, a * v.y, a * v.z, a * v.w); }

// init_particles_smoke (3D/init_conditions.py:275-279) with interp_grad_2_smoke
// (3D/taichi_utils.py:379-420): per particle the smoke value (4 channels) and
// grad[r][ch] = sum over the 27 non-zero taps of dw_r * value[ch], dw_x = (1/dx) dN_2 N_2 N_2.
// BL = 0.5 on every axis, position clamped to [1, n - 2 - eps] of the cell grid; the three
// non-zero taps per axis come from axis_taps (bitwise the reference's per-tap weights).  The tap
// sums are factorised axis by axis (z, y, x) like interp_mac3: rounding-level differences only.
__global__ void __launch_bounds__(128) k_g2p_smoke3(const float* __restrict__ pos, int64_t P, MacGeom g,
                                                    float dxf, const float4* __restrict__ smoke,
                                                    float* __restrict__ s_out, float* __restrict__ grad_out) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  Axis3 A[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float u = pos[a * P + q] / dxf;  // u, v, w = p / dx
    axis_taps(u - 0.5f, (float)((double)g.N[a] - 2.0 - 1e-6), A[a]);
  }
  const int N1 = g.N[1], N2 = g.N[2];
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 V = z4, GX = z4, GY = z4, GZ = z4;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float4 Aa = z4, Ba = z4, Ca = z4;
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const float4* row = smoke + (((int64_t)(A[0].first + a) * N1 + (A[1].first + b)) * N2 + A[2].first);
      const float4 v0 = __ldg(row), v1 = __ldg(row + 1), v2 = __ldg(row + 2);
      const float4 tn = f4fma(A[2].w[2], v2, f4fma(A[2].w[1], v1, f4mul(A[2].w[0], v0)));
      const float4 td = f4fma(A[2].dw[2], v2, f4fma(A[2].dw[1], v1, f4mul(A[2].dw[0], v0)));
      Aa = f4fma(A[1].w[b], tn, Aa);
      Ba = f4fma(A[1].dw[b], tn, Ba);
      Ca = f4fma(A[1].w[b], td, Ca);
    }
    V = f4fma(A[0].w[a], Aa, V);
    GX = f4fma(A[0].dw[a], Aa, GX);
    GY = f4fma(A[0].w[a], Ba, GY);
    GZ = f4fma(A[0].w[a], Ca, GZ);
  }
  const float inv_dx = 1.f / dxf;  // 1. / dx
  if (s_out) {
    s_out[q] = V.x;
    s_out[P + q] = V.y;
    s_out[2 * P + q] = V.z;
    s_out[3 * P + q] = V.w;
  }
  if (grad_out) {
    const float4 Gr[3] = {GX, GY, GZ};
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      grad_out[(r * 4 + 0) * P + q] = Gr[r].x * inv_dx;
      grad_out[(r * 4 + 1) * P + q] = Gr[r].y * inv_dx;
      grad_out[(r * 4 + 2) * P + q] = Gr[r].z * inv_dx;
      grad_out[(r * 4 + 3) * P + q] = Gr[r].w * inv_dx;
    }
  }
}

// The cell-centre backward map of advect_smoke / clamp_smoke (3D/run_3D.py:318-320):
// psi_c = f32(1/6) * (psi_x[i] + psi_x[i+1] + psi_y[j] + psi_y[j+1] + psi_z[k] + psi_z[k+1]),
// summed left to right; psi grids are [F][3].
__device__ __forceinline__ void psi_centre3(const float* __restrict__ px, const float* __restrict__ py,
                                            const float* __restrict__ pz, const MacGeom& g, int i, int j, int k,
                                            float c[3]) {
  const int N1 = g.N[1], N2 = g.N[2];
  const float* a = px + 3 * (((int64_t)i * N1 + j) * N2 + k);
  const float* b = px + 3 * (((int64_t)(i + 1) * N1 + j) * N2 + k);
  const float* e = py + 3 * (((int64_t)i * (N1 + 1) + j) * N2 + k);
  const float* f = py + 3 * (((int64_t)i * (N1 + 1) + j + 1) * N2 + k);
  const float* h = pz + 3 * (((int64_t)i * N1 + j) * (N2 + 1) + k);
  const float* l = pz + 3 * (((int64_t)i * N1 + j) * (N2 + 1) + k + 1);
  const float sixth = (float)(1.0 / 6.0);
#pragma unroll
  for (int d = 0; d < 3; ++d)
    c[d] = __fmul_rn(sixth, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(a[d], b[d]), e[d]), f[d]), h[d]), l[d]));
}

// Trilinear corner of interp_1 / sample_min_max_1 (3D/taichi_utils.py:192-250): s clamped to
// [lo, n - 1 - eps], iu = floor(s); the corners iu, iu+1 are in range, so sample()'s clamp is
// the identity.
__device__ __forceinline__ void lin_axis(float u, float lo, float hi, int& i0, float& s, float& iu) {
  s = fmaxf(lo, fminf(u, hi));
  iu = floorf(s);
  i0 = __float2int_rz(iu);
}

__device__ __forceinline__ float N1f(float x) { return __fsub_rn(1.f, fabsf(x)); }

// advect_smoke (3D/run_3D.py:315-323): smoke1[c] = interp_1(smoke0, psi_c, dx);
// clamp_smoke (3D/run_3D.py:326-334): smoke1[c] = clamp(smoke1[c], min, max of the 8 corners).
// Both evaluate the reference's expressions in its order: interped starts at 0 * corner(0,0,0) and
// adds ((value * N_1(x)) * N_1(y)) * N_1(z) over i, j, k.
template <bool CLAMP>
__global__ void __launch_bounds__(kFThreads) k_smoke_semilag3(const float4* __restrict__ s0, float4* __restrict__ s1,
                                                              const float* __restrict__ px, const float* __restrict__ py,
                                                              const float* __restrict__ pz, MacGeom g, float dxf) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)g.N[0] * g.N[1] * g.N[2]) return;
  int i, j, k;
  split3((unsigned)e, g.dN[1], g.dN[2], i, j, k);
  float c[3];
  psi_centre3(px, py, pz, g, i, j, k, c);
  int i0[3];
  float s[3], iu[3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
    lin_axis(__fsub_rn(__fdiv_rn(c[a], dxf), 0.5f), 1.f, (float)((double)g.N[a] - 1.0 - 1e-6), i0[a], s[a], iu[a]);
  if (!CLAMP) {
    float4 acc = s0[cell3(g, i0[0], i0[1], i0[2])];
    acc = make_float4(0.f * acc.x, 0.f * acc.y, 0.f * acc.z, 0.f * acc.w);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int d = 0; d < 2; ++d) {
          const float nx = N1f(__fsub_rn(s[0], __fadd_rn(iu[0], (float)a)));
          const float ny = N1f(__fsub_rn(s[1], __fadd_rn(iu[1], (float)b)));
          const float nz = N1f(__fsub_rn(s[2], __fadd_rn(iu[2], (float)d)));
          const float4 v = s0[cell3(g, i0[0] + a, i0[1] + b, i0[2] + d)];
          acc.x = __fadd_rn(acc.x, __fmul_rn(__fmul_rn(__fmul_rn(v.x, nx), ny), nz));
          acc.y = __fadd_rn(acc.y, __fmul_rn(__fmul_rn(__fmul_rn(v.y, nx), ny), nz));
          acc.z = __fadd_rn(acc.z, __fmul_rn(__fmul_rn(__fmul_rn(v.z, nx), ny), nz));
          acc.w = __fadd_rn(acc.w, __fmul_rn(__fmul_rn(__fmul_rn(v.w, nx), ny), nz));
        }
    s1[e] = acc;
  } else {
    float4 mn = s0[cell3(g, i0[0], i0[1], i0[2])], mx = mn;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int d = 0; d < 2; ++d) {
          const float4 v = s0[cell3(g, i0[0] + a, i0[1] + b, i0[2] + d)];
          mn = make_float4(fminf(mn.x, v.x), fminf(mn.y, v.y), fminf(mn.z, v.z), fminf(mn.w, v.w));
          mx = make_float4(fmaxf(mx.x, v.x), fmaxf(mx.y, v.y), fmaxf(mx.z, v.z), fmaxf(mx.w, v.w));
        }
    float4 x = s1[e];
    x = make_float4(fminf(fmaxf(x.x, mn.x), mx.x), fminf(fmaxf(x.y, mn.y), mx.y), fminf(fmaxf(x.z, mn.z), mx.z),
                    fminf(fmaxf(x.w, mn.w), mx.w));
    s1[e] = x;
  }
}

// advect_smoke (2D/run_2D.py:444-450): psi_c = 0.25 * (psi_x[i] + psi_x[i+1] + psi_y[j] + psi_y[j+1]),
// then interp_1 (2D/taichi_utils.py:118-143): s clamped to [0, n - 1 - eps], four corners
// a*N1(fu)*N1(fv) + b*N1(fu-1)*N1(fv) + c*N1(fu)*N1(fv-1) + d*N1(fu-1)*N1(fv-1).  3 channels.
__global__ void __launch_bounds__(kFThreads) k_advect_smoke2(const float* __restrict__ s0, float* __restrict__ s1,
                                                             const float* __restrict__ px,
                                                             const float* __restrict__ py, MacGeom g, float dxf) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)g.N[0] * g.N[1]) return;
  const int i = (int)udiv((unsigned)e, g.dN[1]), j = (int)((unsigned)e - (unsigned)i * (unsigned)g.N[1]);
  const int N1 = g.N[1];
  const float* a = px + 2 * ((int64_t)i * N1 + j);
  const float* b = px + 2 * ((int64_t)(i + 1) * N1 + j);
  const float* c = py + 2 * ((int64_t)i * (N1 + 1) + j);
  const float* d = py + 2 * ((int64_t)i * (N1 + 1) + j + 1);
  int i0[2];
  float s[2], iu[2];
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const float pc = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(a[t], b[t]), c[t]), d[t]));
    lin_axis(__fsub_rn(__fdiv_rn(pc, dxf), 0.5f), 0.f, (float)((double)g.N[t] - 1.0 - 1e-6), i0[t], s[t], iu[t]);
  }
  const float fu = __fsub_rn(s[0], iu[0]), fv = __fsub_rn(s[1], iu[1]);
  const float n0u = N1f(fu), n1u = N1f(__fsub_rn(fu, 1.f)), n0v = N1f(fv), n1v = N1f(__fsub_rn(fv, 1.f));
  const float* ca = s0 + 3 * ((int64_t)i0[0] * N1 + i0[1]);
  const float* cb = s0 + 3 * ((int64_t)(i0[0] + 1) * N1 + i0[1]);
  const float* cc = s0 + 3 * ((int64_t)i0[0] * N1 + i0[1] + 1);
  const float* cd = s0 + 3 * ((int64_t)(i0[0] + 1) * N1 + i0[1] + 1);
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    const float t0 = __fmul_rn(__fmul_rn(ca[ch], n0u), n0v);
    const float t1 = __fmul_rn(__fmul_rn(cb[ch], n1u), n0v);
    const float t2 = __fmul_rn(__fmul_rn(cc[ch], n0u), n1v);
    const float t3 = __fmul_rn(__fmul_rn(cd[ch], n1u), n1v);
    s1[e * 3 + ch] = __fadd_rn(__fadd_rn(__fadd_rn(t0, t1), t2), t3);
  }
}

static bool aligned16(const void* p) { return (((uintptr_t)p) & 15) == 0; }

// add_fields / scale_field (3D/taichi_utils.py:13-21, 2D/taichi_utils.py:9-16): elementwise over
// any field, f32, the product rounded before the sum (no contraction), in the reference's order.
__global__ void __launch_bounds__(256) k_add_fields(const float* __restrict__ f1, const float* __restrict__ f2,
                                                    float multiplier, float* __restrict__ dest, int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    dest[e] = __fadd_rn(f1[e], __fmul_rn(multiplier, f2[e]));
}

__global__ void __launch_bounds__(256) k_scale_field(const float* __restrict__ a, float alpha,
                                                     float* __restrict__ result, int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    result[e] = __fmul_rn(alpha, a[e]);
}

static unsigned elementwise_blocks(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (unsigned)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

}  // namespace pfm

using namespace pfm;

extern "C" {

int pfm3_get_central_vector(pfm_handle* h, const float* u_x, const float* u_y, const float* u_z, float* vc,
                            void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_get_central_vector on a 2D handle");
  if (!u_x || !u_y || !u_z || !vc) return set_error(h, PFM_ERR_NULL, "pfm3_get_central_vector: null input");
  launch(h, k_central3, grid_for(h->cells, kFThreads), kFThreads, 0, (cudaStream_t)stream, u_x, u_y, u_z, h->geom, vc);
  return launch_check(h, "k_central3");
}

int pfm3_curl(pfm_handle* h, const float* vc, float* w, float dx, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_curl on a 2D handle");
  if (!vc || !w) return set_error(h, PFM_ERR_NULL, "pfm3_curl: null input");
  if (vc == w) return set_error(h, PFM_ERR_ARG, "pfm3_curl: vc and w must not alias");
  const float inv_dist = 1.f / (2.f * dx);
  launch(h, k_curl3, grid_for(h->cells, kFThreads), kFThreads, 0, (cudaStream_t)stream, vc, h->geom, inv_dist, w);
  return launch_check(h, "k_curl3");
}

int pfm2_get_central_vector(pfm_handle* h, const float* u_x, const float* u_y, float* vc, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 2) return set_error(h, PFM_ERR_SHAPE, "pfm2_get_central_vector on a 3D handle");
  if (!u_x || !u_y || !vc) return set_error(h, PFM_ERR_NULL, "pfm2_get_central_vector: null input");
  launch(h, k_central2, grid_for(h->cells, kFThreads), kFThreads, 0, (cudaStream_t)stream, u_x, u_y, h->geom, vc);
  return launch_check(h, "k_central2");
}

int pfm2_curl(pfm_handle* h, const float* vc, float* w, float dx, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 2) return set_error(h, PFM_ERR_SHAPE, "pfm2_curl on a 3D handle");
  if (!vc || !w) return set_error(h, PFM_ERR_NULL, "pfm2_curl: null input");
  if (vc == w) return set_error(h, PFM_ERR_ARG, "pfm2_curl: vc and w must not alias");
  launch(h, k_curl2, grid_for(h->cells, kFThreads), kFThreads, 0, (cudaStream_t)stream, vc, h->geom, 2.f * dx, w);
  return launch_check(h, "k_curl2");
}

int pfm3_init_particles_smoke(pfm_handle* h, const float* pos, const float* smoke, float* smoke_p, float* grad_smoke,
                              void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_init_particles_smoke on a 2D handle");
  if (h->P > 0 && (!pos || !smoke)) return set_error(h, PFM_ERR_NULL, "pfm3_init_particles_smoke: null input");
  if (smoke && !aligned16(smoke)) return set_error(h, PFM_ERR_ARG, "pfm3_init_particles_smoke: smoke not 16-byte aligned");
  if (h->P == 0) return PFM_OK;
  launch(h, k_g2p_smoke3, grid_for(h->P, 128), 128, 0, (cudaStream_t)stream, pos, h->P, h->geom, h->geom.dx,
         reinterpret_cast<const float4*>(smoke), smoke_p, grad_smoke);
  return launch_check(h, "k_g2p_smoke3");
}

static int smoke_semilag3(pfm_handle* h, const float* smoke0, float* smoke1, const float* psi_x, const float* psi_y,
                          const float* psi_z, float dx, bool clamp, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "3D smoke transport on a 2D handle");
  if (!smoke0 || !smoke1 || !psi_x || !psi_y || !psi_z) return set_error(h, PFM_ERR_NULL, "smoke transport: null input");
  if (smoke0 == smoke1) return set_error(h, PFM_ERR_ARG, "smoke transport: smoke0 and smoke1 must not alias");
  if (!aligned16(smoke0) || !aligned16(smoke1)) return set_error(h, PFM_ERR_ARG, "smoke grids must be 16-byte aligned");
  const float4* s0 = reinterpret_cast<const float4*>(smoke0);
  float4* s1 = reinterpret_cast<float4*>(smoke1);
  const unsigned gr = grid_for(h->cells, kFThreads);
  if (clamp)
    launch(h, k_smoke_semilag3<true>, gr, kFThreads, 0, (cudaStream_t)stream, s0, s1, psi_x, psi_y, psi_z, h->geom, dx);
  else
    launch(h, k_smoke_semilag3<false>, gr, kFThreads, 0, (cudaStream_t)stream, s0, s1, psi_x, psi_y, psi_z, h->geom, dx);
  return launch_check(h, "k_smoke_semilag3");
}

int pfm3_advect_smoke(pfm_handle* h, const float* smoke0, float* smoke1, const float* psi_x, const float* psi_y,
                      const float* psi_z, float dx, void* stream) {
  return smoke_semilag3(h, smoke0, smoke1, psi_x, psi_y, psi_z, dx, false, stream);
}

int pfm3_clamp_smoke(pfm_handle* h, const float* smoke0, float* smoke1, const float* psi_x, const float* psi_y,
                     const float* psi_z, float dx, void* stream) {
  return smoke_semilag3(h, smoke0, smoke1, psi_x, psi_y, psi_z, dx, true, stream);
}

int pfm2_advect_smoke(pfm_handle* h, const float* smoke0, float* smoke1, const float* psi_x, const float* psi_y,
                      float dx, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 2) return set_error(h, PFM_ERR_SHAPE, "pfm2_advect_smoke on a 3D handle");
  if (!smoke0 || !smoke1 || !psi_x || !psi_y) return set_error(h, PFM_ERR_NULL, "pfm2_advect_smoke: null input");
  if (smoke0 == smoke1) return set_error(h, PFM_ERR_ARG, "pfm2_advect_smoke: smoke0 and smoke1 must not alias");
  launch(h, k_advect_smoke2, grid_for(h->cells, kFThreads), kFThreads, 0, (cudaStream_t)stream, smoke0, smoke1, psi_x,
         psi_y, h->geom, dx);
  return launch_check(h, "k_advect_smoke2");
}


int pfm_add_fields(const float* f1, const float* f2, float multiplier, float* dest, int64_t n, void* stream) {
  if (n < 0) return PFM_ERR_ARG;
  if (n == 0) return PFM_OK;
  if (!f1 || !f2 || !dest) return PFM_ERR_NULL;
  k_add_fields<<<elementwise_blocks(n), 256, 0, (cudaStream_t)stream>>>(f1, f2, multiplier, dest, n);
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}

int pfm_scale_field(const float* a, float alpha, float* result, int64_t n, void* stream) {
  if (n < 0) return PFM_ERR_ARG;
  if (n == 0) return PFM_OK;
  if (!a || !result) return PFM_ERR_NULL;
  k_scale_field<<<elementwise_blocks(n), 256, 0, (cudaStream_t)stream>>>(a, alpha, result, n);
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}

}  // extern "C"
