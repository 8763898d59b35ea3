// Grid kernels of the step: CFL max speed and the midpoint velocity (backward RK4 of the face
// positions and Jacobians, then the advection u1 = T . u0(psi)).
#include "pfm_internal.cuh"

namespace pfm {

constexpr int kGThreads = 128;
// Resident blocks per SM the 3D midpoint kernel is compiled for: 5 (94 registers, no spills).  With
// the strides of a cube grid compiled in (interp_mac3_taps<NC>) it measured 3.90 ms at 256^3
// against 3.96 ms at 6 (80 registers, a 20-byte spill).  With strides read at run time, 6 measured
// 4.39 ms against 4.43-4.86 ms uncapped (88 registers, 5 blocks) and 4.61 ms at 8 (64 registers,
// spills).
#ifndef PFM_MID_MINB
#define PFM_MID_MINB 5
#endif

// calc_max_speed (3D/run_3D.py:95-103; 2D/run_2D.py:101-108).  Max is order independent, so the
// per-block maxima are combined by the last block without atomics on floats.
template <int D>
__global__ void __launch_bounds__(256) k_max_speed(const float* __restrict__ ux, const float* __restrict__ uy,
                                                   const float* __restrict__ uz, MacGeom g,
                                                   float* __restrict__ partial, unsigned* ticket,
                                                   float* __restrict__ out) {
  const int64_t C = (int64_t)g.N[0] * g.N[1] * g.N[2];
  float m = 1.e-3f;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < C; e += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    split3((unsigned)e, g.dN[1], g.dN[2], i, j, k);
    float u, v, sp;
    if (D == 3) {
      float w;
      u = 0.5f * (ux[((int64_t)i * g.N[1] + j) * g.N[2] + k] + ux[((int64_t)(i + 1) * g.N[1] + j) * g.N[2] + k]);
      v = 0.5f * (uy[((int64_t)i * (g.N[1] + 1) + j) * g.N[2] + k] +
                  uy[((int64_t)i * (g.N[1] + 1) + j + 1) * g.N[2] + k]);
      w = 0.5f * (uz[((int64_t)i * g.N[1] + j) * (g.N[2] + 1) + k] +
                  uz[((int64_t)i * g.N[1] + j) * (g.N[2] + 1) + k + 1]);
      sp = sqrtf(u * u + v * v + w * w);
    } else {
      u = 0.5f * (ux[(int64_t)i * g.N[1] + j] + ux[(int64_t)(i + 1) * g.N[1] + j]);
      v = 0.5f * (uy[(int64_t)i * (g.N[1] + 1) + j] + uy[(int64_t)i * (g.N[1] + 1) + j + 1]);
      sp = sqrtf(u * u + v * v);
    }
    m = fmaxf(m, sp);
  }
  __shared__ float sm[256];
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] = fmaxf(sm[threadIdx.x], sm[threadIdx.x + s]);
    __syncthreads();
  }
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = sm[0];
    __threadfence();
    unsigned t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  float mm = 1.e-3f;
  for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x) mm = fmaxf(mm, ((volatile float*)partial)[b]);
  sm[threadIdx.x] = mm;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] = fmaxf(sm[threadIdx.x], sm[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *out = sm[0];
    *ticket = 0u;
  }
}

// Midpoint for face family `fam` (3D/run_3D.py:106-120, 144-173, 296-312): psi starts at the face
// centre X_fam (taichi_utils.py:33-46), T at the unit vector e_fam; RK4 over -dt_half with the
// rows-form gradient (dT/dt = grad u . T); then u1 = T . u0(psi).
// One component of interp_mac3_taps (value and gradient) at a sample on whole or half cells whose
// clamp does not bind: per axis the three taps are the C set (s whole: t = 0, weights 1/8, 3/4,
// 1/8, derivatives -1/2, -0, 1/2) or the H set (s half: t = -1/2, weights 1/2, 1/2, 0,
// derivatives -1, 1, 0), the weights interp_mac3's closed form gives there.  The sums are
// interp_mac3_taps' own, term for term and in its order, less the terms whose weight is zero
// (which add a zero): the same results, with the zero-weight loads and FMAs left out (12 of the 27
// rows and taps of a component with two H axes).  b: the component's first tap; sx, sy: its
// strides along x and y.
template <bool CX, bool CY, bool CZ>
__device__ __forceinline__ void centre_component(const float* __restrict__ b, int sx, int sy, float& v, float& gx,
                                                 float& gy, float& gz) {
  constexpr int NA = CX ? 3 : 2, NB = CY ? 3 : 2;
  float v_ = 0.f, x_ = 0.f, y_ = 0.f, z_ = 0.f;
#pragma unroll
  for (int a = 0; a < NA; ++a) {
    float Aa = 0.f, Ba = 0.f, Ca = 0.f;
#pragma unroll
    for (int bb = 0; bb < NB; ++bb) {
      const float* __restrict__ row = b + (a * sx + bb * sy);
      const float v0 = __ldg(row), v1 = __ldg(row + 1);
      float tn, td;
      if (CZ) {
        const float v2 = __ldg(row + 2);
        tn = fmaf(v2, 0.125f, fmaf(v1, 0.75f, v0 * 0.125f));
        td = fmaf(v2, 0.5f, v0 * -0.5f);
      } else {
        tn = fmaf(v1, 0.5f, v0 * 0.5f);
        td = fmaf(v1, 1.f, v0 * -1.f);
      }
      const float wy = CY ? (bb == 1 ? 0.75f : 0.125f) : 0.5f;
      Aa = fmaf(wy, tn, Aa);
      if (!CY || bb != 1) Ba = fmaf(CY ? (bb == 0 ? -0.5f : 0.5f) : (bb == 0 ? -1.f : 1.f), tn, Ba);
      Ca = fmaf(wy, td, Ca);
    }
    const float wx = CX ? (a == 1 ? 0.75f : 0.125f) : 0.5f;
    v_ = fmaf(wx, Aa, v_);
    if (!CX || a != 1) x_ = fmaf(CX ? (a == 0 ? -0.5f : 0.5f) : (a == 0 ? -1.f : 1.f), Aa, x_);
    y_ = fmaf(wx, Ba, y_);
    z_ = fmaf(wx, Ca, z_);
  }
  v = v_;
  gx = x_;
  gy = y_;
  gz = z_;
}

// interp_mac3<NC>(want_grad) at the centre of face (i, j, k) of family fam, when the sample is
// that face centre exactly (p / dx gives back the face's coordinates) and no clamp binds; else
// false (the caller interpolates generically).  Component c samples axis a at s = X_a - BL(c, a),
// X the face centre (whole on the family's axis, half elsewhere), BL = 0 on a = c, 1/2 elsewhere:
// s is whole (C taps, first tap s - 1) when a is both or neither of fam and c, else half (H taps,
// first tap s - 1/2).
template <int fam, int NC>
__device__ __forceinline__ bool interp_face_centre(const MacFields3& F, const MacGeom& g, const float p[3],
                                                   const int I[3], float uo[3], float G[3][3]) {
  bool ok = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float u = p[a] * g.inv_dx;
    const float X = (float)I[a] + (a == fam ? 0.f : 0.5f);
    ok = ok && (u == X);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float sv = (a == c) ? u - 0.0f : u - 0.5f;
      ok = ok && sv >= 1.f && sv <= g.hi[c][a];
    }
  }
  if (!ok) return false;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    int first[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) first[a] = (a == fam || a != c) ? I[a] - 1 : I[a];
    const int m1 = NC ? (c == 1 ? NC + 1 : NC) : g.n[c][1], m2 = NC ? (c == 2 ? NC + 1 : NC) : g.n[c][2];
    const float* __restrict__ base = F.u[c] + ((first[0] * m1 + first[1]) * m2 + first[2]);
    const int sx = m1 * m2;
    float v, gx, gy, gz;
    // axis a takes the C set when (a == fam) == (a == c)
    if (c == fam)
      centre_component<true, true, true>(base, sx, m2, v, gx, gy, gz);
    else if (fam == 0 && c == 1)
      centre_component<false, false, true>(base, sx, m2, v, gx, gy, gz);
    else if (fam == 0 && c == 2)
      centre_component<false, true, false>(base, sx, m2, v, gx, gy, gz);
    else if (fam == 1 && c == 0)
      centre_component<false, false, true>(base, sx, m2, v, gx, gy, gz);
    else if (fam == 1 && c == 2)
      centre_component<true, false, false>(base, sx, m2, v, gx, gy, gz);
    else if (fam == 2 && c == 0)
      centre_component<false, true, false>(base, sx, m2, v, gx, gy, gz);
    else
      centre_component<true, false, false>(base, sx, m2, v, gx, gy, gz);
    uo[c] = v;
    G[c][0] = gx * g.inv_dx;
    G[c][1] = gy * g.inv_dx;
    G[c][2] = gz * g.inv_dx;
  }
  return true;
}

// NC: the grid's cube extent when the interpolation is compiled for it (interp_mac3_taps<NC>), else 0.
// centre != 0: the first stage at the face centre in the constant-weight form (interp_face_centre).
template <int fam, int NC>
__global__ void __launch_bounds__(kGThreads, PFM_MID_MINB) k_midpoint3(MacFields3 F, MacGeom g, float dt_half,
                                                        float* __restrict__ u1, float* __restrict__ psi_out,
                                                        float* __restrict__ T_out,
                                                        const float* __restrict__ dt_half_dev, int centre) {
  if (dt_half_dev) dt_half = *dt_half_dev;  // the whole-step graph keeps dt on the device
  const int n0 = g.n[fam][0], n1 = g.n[fam][1], n2 = g.n[fam][2];
  const int64_t nf = (int64_t)n0 * n1 * n2;
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nf) return;
  int i, j, k;
  split3((unsigned)e, g.dn[fam][1], g.dn[fam][2], i, j, k);
  float X[3] = {(float)i, (float)j, (float)k};
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (d != fam) X[d] = X[d] + 0.5f;
  float p0[3] = {X[0] * g.dx, X[1] * g.dx, X[2] * g.dx};
  float T0[3] = {fam == 0 ? 1.f : 0.f, fam == 1 ? 1.f : 0.f, fam == 2 ? 1.f : 0.f};
  const float neg_dt = -1.f * dt_half;
  const float half = 0.5f * neg_dt;
  float pk[3] = {p0[0], p0[1], p0[2]}, Tk[3] = {T0[0], T0[1], T0[2]};
  float su[3], sT[3];
  const int I[3] = {i, j, k};
#pragma unroll 1
  for (int s = 0; s < 4; ++s) {
    float u[3], G[3][3];
    // the first stage samples the face centre itself: constant weights, a third of the rows fewer
    if (s > 0 || !centre || !interp_face_centre<fam, NC>(F, g, pk, I, u, G)) interp_mac3<NC>(F, g, pk, u, G, true);
    float dT[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) dT[c] = G[c][0] * Tk[0] + G[c][1] * Tk[1] + G[c][2] * Tk[2];
    const float wgt = (s == 0 || s == 3) ? 1.f : 2.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      su[c] = (s == 0) ? u[c] : su[c] + wgt * u[c];
      sT[c] = (s == 0) ? dT[c] : sT[c] + wgt * dT[c];
    }
    if (s < 3) {
      const float cdt = (s < 2) ? half : neg_dt;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        pk[c] = p0[c] + cdt * u[c];
        Tk[c] = T0[c] + cdt * dT[c];
      }
    }
  }
  const float coef = neg_dt / 6.f;
  float pf[3], Tf[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    pf[c] = p0[c] + coef * su[c];
    Tf[c] = T0[c] + coef * sT[c];
  }
  if (psi_out) {
#pragma unroll
    for (int c = 0; c < 3; ++c) psi_out[e * 3 + c] = pf[c];
  }
  if (T_out) {
#pragma unroll
    for (int c = 0; c < 3; ++c) T_out[e * 3 + c] = Tf[c];
  }
  float ua[3], G[3][3];
  interp_mac3<NC>(F, g, pf, ua, G, false);
  u1[e] = Tf[0] * ua[0] + Tf[1] * ua[1] + Tf[2] * ua[2];
}

// 2D midpoint (2D/run_2D.py:120-129, 233-261, 429-441)
template <int fam>
__global__ void __launch_bounds__(kGThreads) k_midpoint2(MacFields2 F, MacGeom g, float dt_half,
                                                        float* __restrict__ u1, float* __restrict__ psi_out,
                                                        float* __restrict__ T_out,
                                                        const float* __restrict__ dt_half_dev) {
  if (dt_half_dev) dt_half = *dt_half_dev;
  const int n0 = g.n[fam][0], n1 = g.n[fam][1];
  const int64_t nf = (int64_t)n0 * n1;
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nf) return;
  const int i = (int)udiv((unsigned)e, g.dn[fam][1]);
  const int j = (int)((unsigned)e - (unsigned)i * (unsigned)n1);
  float X[2] = {(float)i, (float)j};
  X[1 - fam] = X[1 - fam] + 0.5f;
  float p0[2] = {X[0] * g.dx, X[1] * g.dx};
  float T0[2] = {fam == 0 ? 1.f : 0.f, fam == 1 ? 1.f : 0.f};
  const float neg_dt = -1.f * dt_half;
  const float half = 0.5f * neg_dt;
  float pk[2] = {p0[0], p0[1]}, Tk[2] = {T0[0], T0[1]};
  float su[2], sT[2];
#pragma unroll 1
  for (int s = 0; s < 4; ++s) {
    float u[2], G[2][2];
    interp_mac2(F, g, pk, u, G);
    float dT[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) dT[c] = G[c][0] * Tk[0] + G[c][1] * Tk[1];
    const float wgt = (s == 0 || s == 3) ? 1.f : 2.f;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      su[c] = (s == 0) ? u[c] : su[c] + wgt * u[c];
      sT[c] = (s == 0) ? dT[c] : sT[c] + wgt * dT[c];
    }
    if (s < 3) {
      const float cdt = (s < 2) ? half : neg_dt;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        pk[c] = p0[c] + cdt * u[c];
        Tk[c] = T0[c] + cdt * dT[c];
      }
    }
  }
  const float coef = neg_dt / 6.f;
  float pf[2] = {p0[0] + coef * su[0], p0[1] + coef * su[1]};
  float Tf[2] = {T0[0] + coef * sT[0], T0[1] + coef * sT[1]};
  if (psi_out) {
    psi_out[e * 2] = pf[0];
    psi_out[e * 2 + 1] = pf[1];
  }
  if (T_out) {
    T_out[e * 2] = Tf[0];
    T_out[e * 2 + 1] = Tf[1];
  }
  float ua[2], G[2][2];
  interp_mac2(F, g, pf, ua, G);
  u1[e] = Tf[0] * ua[0] + Tf[1] * ua[1];
}

// k_midpoint3 of face family fam, instantiated for the grid's cube extent when there is one.
static void launch_midpoint3(pfm_handle* h, int fam, dim3 gr, cudaStream_t st, const MacFields3& F, float dt_half,
                             float* u1, float* psi_out, float* T_out, const float* dt_half_dev) {
  with_cube(h, [&](auto nc) {
    constexpr int NC = decltype(nc)::value;
    const int c = h->mid_centre;
    if (fam == 0)
      launch(h, k_midpoint3<0, NC>, gr, kGThreads, 0, st, F, h->geom, dt_half, u1, psi_out, T_out, dt_half_dev, c);
    if (fam == 1)
      launch(h, k_midpoint3<1, NC>, gr, kGThreads, 0, st, F, h->geom, dt_half, u1, psi_out, T_out, dt_half_dev, c);
    if (fam == 2)
      launch(h, k_midpoint3<2, NC>, gr, kGThreads, 0, st, F, h->geom, dt_half, u1, psi_out, T_out, dt_half_dev, c);
  });
}

// The midpoint kernels of every face family, dt_half from the host value or (dt_half_dev non-null)
// from device memory.
int launch_midpoint(pfm_handle* h, const float* const* u0, float* const* u1, float dt_half, const float* dt_half_dev,
                    cudaStream_t st) {
  const int D = h->cfg.dim;
  for (int fam = 0; fam < D; ++fam) {
    const int64_t nf = (int64_t)h->geom.n[fam][0] * h->geom.n[fam][1] * h->geom.n[fam][2];
    const dim3 gr(grid_for(nf, kGThreads));
    if (D == 3) {
      const MacFields3 F{{u0[0], u0[1], u0[2]}};
      launch_midpoint3(h, fam, gr, st, F, dt_half, u1[fam], nullptr, nullptr, dt_half_dev);
    } else {
      const MacFields2 F{{u0[0], u0[1]}};
      if (fam == 0) launch(h, k_midpoint2<0>, gr, kGThreads, 0, st, F, h->geom, dt_half, u1[0], (float*)nullptr,
                           (float*)nullptr, dt_half_dev);
      if (fam == 1) launch(h, k_midpoint2<1>, gr, kGThreads, 0, st, F, h->geom, dt_half, u1[1], (float*)nullptr,
                           (float*)nullptr, dt_half_dev);
    }
  }
  return launch_check(h, "midpoint");
}

int max_speed_async(pfm_handle* h, const float* ux, const float* uy, const float* uz, float* out,
                    cudaStream_t st) {
  int s = require_ws(h);
  if (s) return s;
  float* part = ws_ptr<float>(h, h->o_maxpart);
  unsigned* ticket = reinterpret_cast<unsigned*>(part + kReduceBlocks);
  unsigned blocks = grid_for(h->cells, 256);
  if (blocks > (unsigned)kReduceBlocks) blocks = kReduceBlocks;
  s = check_cuda(h, cudaMemsetAsync(ticket, 0, sizeof(unsigned), st), "memset ticket");
  if (s) return s;
  if (h->cfg.dim == 3)
    launch(h, k_max_speed<3>, blocks, 256, 0, st, ux, uy, uz, h->geom, part, ticket, out);
  else
    launch(h, k_max_speed<2>, blocks, 256, 0, st, ux, uy, uz, h->geom, part, ticket, out);
  return launch_check(h, "k_max_speed");
}

}  // namespace pfm

using namespace pfm;

extern "C" {

int pfm3_calc_max_speed(pfm_handle* h, const float* u_x, const float* u_y, const float* u_z, float* max_dev,
                        void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_calc_max_speed on a 2D handle");
  if (!u_x || !u_y || !u_z || !max_dev) return set_error(h, PFM_ERR_NULL, "pfm3_calc_max_speed: null input");
  return max_speed_async(h, u_x, u_y, u_z, max_dev, (cudaStream_t)stream);
}

int pfm2_calc_max_speed(pfm_handle* h, const float* u_x, const float* u_y, float* max_dev, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 2) return set_error(h, PFM_ERR_SHAPE, "pfm2_calc_max_speed on a 3D handle");
  if (!u_x || !u_y || !max_dev) return set_error(h, PFM_ERR_NULL, "pfm2_calc_max_speed: null input");
  return max_speed_async(h, u_x, u_y, nullptr, max_dev, (cudaStream_t)stream);
}

int pfm3_midpoint(pfm_handle* h, const float* u0_x, const float* u0_y, const float* u0_z, float* u1_x,
                  float* u1_y, float* u1_z, float dt_half, float* psi_out[3], float* T_out[3], void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_midpoint on a 2D handle");
  if (!u0_x || !u0_y || !u0_z || !u1_x || !u1_y || !u1_z)
    return set_error(h, PFM_ERR_NULL, "pfm3_midpoint: null input");
  if (u0_x == u1_x || u0_y == u1_y || u0_z == u1_z)
    return set_error(h, PFM_ERR_ARG, "pfm3_midpoint: u0 and u1 must not alias");
  MacFields3 F{{u0_x, u0_y, u0_z}};
  float* outs[3] = {u1_x, u1_y, u1_z};
  for (int fam = 0; fam < 3; ++fam) {
    int64_t nf = (int64_t)h->geom.n[fam][0] * h->geom.n[fam][1] * h->geom.n[fam][2];
    float* po = psi_out ? psi_out[fam] : nullptr;
    float* to = T_out ? T_out[fam] : nullptr;
    dim3 gr(grid_for(nf, kGThreads));
    launch_midpoint3(h, fam, gr, (cudaStream_t)stream, F, dt_half, outs[fam], po, to, nullptr);
    int s = launch_check(h, "k_midpoint3");
    if (s) return s;
  }
  return PFM_OK;
}

int pfm2_midpoint(pfm_handle* h, const float* u0_x, const float* u0_y, float* u1_x, float* u1_y, float dt_half,
                  float* psi_out[2], float* T_out[2], void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 2) return set_error(h, PFM_ERR_SHAPE, "pfm2_midpoint on a 3D handle");
  if (!u0_x || !u0_y || !u1_x || !u1_y) return set_error(h, PFM_ERR_NULL, "pfm2_midpoint: null input");
  if (u0_x == u1_x || u0_y == u1_y) return set_error(h, PFM_ERR_ARG, "pfm2_midpoint: u0 and u1 must not alias");
  MacFields2 F{{u0_x, u0_y}};
  float* outs[2] = {u1_x, u1_y};
  for (int fam = 0; fam < 2; ++fam) {
    int64_t nf = (int64_t)h->geom.n[fam][0] * h->geom.n[fam][1];
    float* po = psi_out ? psi_out[fam] : nullptr;
    float* to = T_out ? T_out[fam] : nullptr;
    dim3 gr(grid_for(nf, kGThreads));
    cudaStream_t st = (cudaStream_t)stream;
    if (fam == 0) launch(h, k_midpoint2<0>, gr, kGThreads, 0, st, F, h->geom, dt_half, outs[fam], po, to,
                       (const float*)nullptr);
    if (fam == 1) launch(h, k_midpoint2<1>, gr, kGThreads, 0, st, F, h->geom, dt_half, outs[fam], po, to,
                       (const float*)nullptr);
    int s = launch_check(h, "k_midpoint2");
    if (s) return s;
  }
  return PFM_OK;
}

}  // extern "C"
