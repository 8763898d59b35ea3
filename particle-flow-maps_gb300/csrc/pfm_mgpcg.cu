// MGPCG pressure projection on the MAC grid (3D/mgpcg.py, 2D/mgpcg.py).
//
// Structure follows MGPCG.solve (3D/mgpcg.py:202-280) exactly, with these GB300 choices:
//  * alpha/beta/convergence live in a device SolveState, and the iteration loop runs on the
//    device: a CUDA graph WHILE node repeats the iteration until the convergence test (or the
//    iteration limit) clears its condition, so the host waits once per solve and the stopping
//    iteration is the reference's;
//  * every reduction is deterministic: a fixed block partition, per-thread f32 partials,
//    f64 block and grid combination in block order (no float atomics);
//  * the restriction scatter (r_{l+1}[I//2] += res/(dim-1), 3D/mgpcg.py:152-158) is a gather
//    over the 8 (4 in 2D) children, so it needs no atomics either.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <algorithm>
#include <atomic>
#include <type_traits>
#include <vector>

#include "pfm_internal.cuh"
#include "pfm_tma.cuh"

namespace pfm {

struct Lvl {
  int n0, n1, n2;
  int64_t count;
  Div32 d1, d2;  // divisors n1, n2
  Div32 dh;      // divisor (last extent + 1) / 2: the cell pairs of a smoothing sweep
};

static inline Lvl make_lvl(int n0, int n1, int n2, int D) {
  const int last = (D == 3) ? n2 : n1;
  return Lvl{n0, n1, n2, (int64_t)n0 * n1 * n2, make_div32((unsigned)n1), make_div32((unsigned)n2),
             make_div32((unsigned)((last + 1) >> 1))};
}

struct BC {
  int lo[3], hi[3];  // 2 = Neumann
};

static inline Lvl lvl_of(const pfm_handle* h, int l) {
  return make_lvl(h->lv[l].n[0], h->lv[l].n[1], h->lv[l].n[2], h->cfg.dim);
}

// Multigrid level storage: FP32 (the reference), or FP16 / BF16 in the mixed-precision solve;
// values are widened to FP32 on load and rounded to nearest on store.
__device__ __forceinline__ float ldv(const float* p) { return *p; }
__device__ __forceinline__ float ldv(const __half* p) { return __half2float(*p); }
__device__ __forceinline__ float ldv(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ void stv(float* p, float v) { *p = v; }
__device__ __forceinline__ void stv(__half* p, float v) { *p = __float2half_rn(v); }
__device__ __forceinline__ void stv(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }

// neighbor_sum / num_fluid_neighbors (3D/mgpcg.py:92-115)
template <int D, typename S>
__device__ __forceinline__ void stencil(const S* __restrict__ f, const Lvl& L, const BC& bc, int i, int j,
                                        int k, int64_t e, float& nb, float& mult) {
  float ret = 0.f;
  float num = 2.f * D;
  const int64_t sx = (int64_t)L.n1 * L.n2, sy = L.n2;
  if (i < L.n0 - 1) ret += ldv(f + e + sx);
  if (i > 0) ret += ldv(f + e - sx);
  if (D == 3) {
    if (j < L.n1 - 1) ret += ldv(f + e + sy);
    if (j > 0) ret += ldv(f + e - sy);
    if (k < L.n2 - 1) ret += ldv(f + e + 1);
    if (k > 0) ret += ldv(f + e - 1);
  } else {
    if (j < L.n1 - 1) ret += ldv(f + e + sy);
    if (j > 0) ret += ldv(f + e - sy);
  }
  if (i <= 0 && bc.lo[0] == 2) num -= 1.f;
  if (i >= L.n0 - 1 && bc.hi[0] == 2) num -= 1.f;
  if (j <= 0 && bc.lo[1] == 2) num -= 1.f;
  if (j >= L.n1 - 1 && bc.hi[1] == 2) num -= 1.f;
  if (D == 3) {
    if (k <= 0 && bc.lo[2] == 2) num -= 1.f;
    if (k >= L.n2 - 1 && bc.hi[2] == 2) num -= 1.f;
  }
  nb = ret;
  mult = num;
}

// num_fluid_neighbors alone (the mult of stencil<D>, no loads)
template <int D>
__device__ __forceinline__ float stencil_mult(const Lvl& L, const BC& bc, int i, int j, int k) {
  float num = 2.f * D;
  if (i <= 0 && bc.lo[0] == 2) num -= 1.f;
  if (i >= L.n0 - 1 && bc.hi[0] == 2) num -= 1.f;
  if (j <= 0 && bc.lo[1] == 2) num -= 1.f;
  if (j >= L.n1 - 1 && bc.hi[1] == 2) num -= 1.f;
  if (D == 3) {
    if (k <= 0 && bc.lo[2] == 2) num -= 1.f;
    if (k >= L.n2 - 1 && bc.hi[2] == 2) num -= 1.f;
  }
  return num;
}

__device__ __forceinline__ void decode(const Lvl& L, int64_t e, int& i, int& j, int& k) {
  split3((unsigned)e, L.d1, L.d2, i, j, k);
}

// ---------------------------------------------------------------------------------------------
// deterministic block/grid reduction
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Sums `v` over the `nb` blocks of a fixed partition (this block is `bid`).  Returns true in the
// last block to finish, where *total holds the sum (combined in block order): bitwise
// reproducible.  A batched launch passes each scene's own partition (bid, nb) of its work items.
__device__ bool grid_sum(double v, double* partials, unsigned* ticket, double* total, unsigned bid, unsigned nb) {
  __shared__ double ws[32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) ws[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double b = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0.0;
    b = warp_sum(b);
    if (lane == 0) {
      partials[bid] = b;
      __threadfence();
      unsigned t = atomicAdd(ticket, 1u);
      last = (t == nb - 1);
    }
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double s = 0.0;
  for (int b = threadIdx.x; b < (int)nb; b += blockDim.x) s += ((volatile double*)partials)[b];
  s = warp_sum(s);
  if (lane == 0) ws[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
    *total = t;
    *ticket = 0u;
  }
  __syncthreads();
  return true;
}

// Two sums of the same partition at once: each is reduced exactly as grid_sum reduces it (the
// same warp trees, block order and final combination), the second through partials[nb ..).
__device__ bool grid_sum2(double v0, double v1, double* partials, unsigned* ticket, double* total0, double* total1,
                          unsigned bid, unsigned nb) {
  __shared__ double ws[2][32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v0 = warp_sum(v0);
  v1 = warp_sum(v1);
  if (lane == 0) {
    ws[0][wid] = v0;
    ws[1][wid] = v1;
  }
  __syncthreads();
  if (wid == 0) {
    double b0 = lane < (int)(blockDim.x >> 5) ? ws[0][lane] : 0.0;
    double b1 = lane < (int)(blockDim.x >> 5) ? ws[1][lane] : 0.0;
    b0 = warp_sum(b0);
    b1 = warp_sum(b1);
    if (lane == 0) {
      partials[bid] = b0;
      partials[nb + bid] = b1;
      __threadfence();
      unsigned t = atomicAdd(ticket, 1u);
      last = (t == nb - 1);
    }
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double s0 = 0.0, s1 = 0.0;
  for (int b = threadIdx.x; b < (int)nb; b += blockDim.x) {
    s0 += ((volatile double*)partials)[b];
    s1 += ((volatile double*)partials)[nb + b];
  }
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  __syncthreads();  // every thread is done reading ws before it is reused
  if (lane == 0) {
    ws[0][wid] = s0;
    ws[1][wid] = s1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      t0 += ws[0][w];
      t1 += ws[1][w];
    }
    *total0 = t0;
    *total1 = t1;
    *ticket = 0u;
  }
  __syncthreads();
  return true;
}

struct RedBuf {
  double* partials;  // 2 x kReduceBlocks
  SolveState* st;
};

// ---------------------------------------------------------------------------------------------
// Poisson pieces: apply_bc, divergence, subtract_grad_p (3D/mgpcg.py:359-418; 2D 293-335)
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void k_apply_bc(float* __restrict__ u, int fam, MacGeom g, int lo_neu, int hi_neu) {
  // faces with index 0 or n along `fam`
  const int n0 = g.n[fam][0], n1 = g.n[fam][1], n2 = g.n[fam][2];
  int a1 = (fam == 0) ? 1 : 0, a2 = (fam == 2) ? 1 : 2;
  if (D == 2) a2 = 2;
  const int m1 = g.n[fam][a1], m2 = (D == 3) ? g.n[fam][a2] : 1;
  const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned plane = (unsigned)m1 * (unsigned)m2;
  if (e >= 2 * plane) return;
  const int side = (int)(e / plane);
  const unsigned r = e - (unsigned)side * plane;
  const int c1 = (int)(r / (unsigned)m2), c2 = (int)(r % (unsigned)m2);
  int idx[3] = {0, 0, 0};
  idx[fam] = side ? g.n[fam][fam] - 1 : 0;
  idx[a1] = c1;
  if (D == 3) idx[a2] = c2;
  if ((side == 0 && lo_neu) || (side == 1 && hi_neu)) u[((int64_t)idx[0] * n1 + idx[1]) * n2 + idx[2]] = 0.f;
  (void)n0;
}

// divergence (3D/mgpcg.py:380-390) times scale: scale = -1 fuses init(u_div, -1), r0 = -(vr - vl + ...)
template <int D>
__global__ void k_divergence(const float* __restrict__ ux, const float* __restrict__ uy,
                             const float* __restrict__ uz, Lvl L, float* __restrict__ r0, float scale) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= L.count) return;
  int i, j, k;
  decode(L, e, i, j, k);
  float div;
  if (D == 3) {
    float vl = ux[((int64_t)i * L.n1 + j) * L.n2 + k], vr = ux[((int64_t)(i + 1) * L.n1 + j) * L.n2 + k];
    float vb = uy[((int64_t)i * (L.n1 + 1) + j) * L.n2 + k], vt = uy[((int64_t)i * (L.n1 + 1) + j + 1) * L.n2 + k];
    float va = uz[((int64_t)i * L.n1 + j) * (L.n2 + 1) + k], vc = uz[((int64_t)i * L.n1 + j) * (L.n2 + 1) + k + 1];
    div = vr - vl + vt - vb + vc - va;
  } else {
    float vl = ux[(int64_t)i * L.n1 + j], vr = ux[(int64_t)(i + 1) * L.n1 + j];
    float vb = uy[(int64_t)i * (L.n1 + 1) + j], vt = uy[(int64_t)i * (L.n1 + 1) + j + 1];
    div = vr - vl + vt - vb;
  }
  r0[e] = div * scale;
}

// subtract_grad_p for family `fam`, followed by apply_bc on that family's boundary faces.
template <int D, int fam>
__global__ void __launch_bounds__(256) k_subtract_grad_p(float* __restrict__ u, const float* __restrict__ p, MacGeom g,
                                                         int lo_neu, int hi_neu) {
  const unsigned nf = (unsigned)g.n[fam][0] * g.n[fam][1] * g.n[fam][2];
  const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nf) return;
  int idx[3];
  split3(e, g.dn[fam][1], g.dn[fam][2], idx[0], idx[1], idx[2]);
  const int N[3] = {g.N[0], g.N[1], g.N[2]};
  // sample(p, I) and sample(p, I - e_fam): clamped indices, then the explicit zeros
  int hiI[3] = {idx[0], idx[1], idx[2]}, loI[3] = {idx[0], idx[1], idx[2]};
  loI[fam] -= 1;
  int a = idx[fam];
  auto clampi = [](int v, int n) { return v < 0 ? 0 : (v > n - 1 ? n - 1 : v); };
  hiI[fam] = clampi(hiI[fam], N[fam]);
  loI[fam] = clampi(loI[fam], N[fam]);
  float pr = p[((int64_t)hiI[0] * N[1] + hiI[1]) * N[2] + hiI[2]];
  float pl = p[((int64_t)loI[0] * N[1] + loI[1]) * N[2] + loI[2]];
  if (a - 1 < 0) pl = 0.f;
  if (a >= N[fam]) pr = 0.f;
  float v = u[e] - (pr - pl);
  if ((a == 0 && lo_neu) || (a == N[fam] && hi_neu)) v = 0.f;
  u[e] = v;
}

// ---------------------------------------------------------------------------------------------
// multigrid V-cycle kernels (3D/mgpcg.py:152-200)
// ---------------------------------------------------------------------------------------------

// Every kernel of the solver iteration is an operation struct whose run(bid, nb) does the work of
// block `bid` of an `nb`-block launch; the kernel is run(blockIdx.x, gridDim.x), and a batched
// launch (k_worklist) runs the blocks of many scenes' operations from one work list.

// smooth(l, phase): z = (r + nbsum(z)) / mult on cells with (i+j+k)&1 == phase.  One thread per
// pair of cells along the last axis; the thread updates the member of the right colour.  `fresh`:
// the level's z is to start at zero (the V-cycle zeroes a level before its first sweep), so the
// sweep reads no neighbours -- every neighbour sum is 0 -- and writes zero to the other colour:
// bitwise the zeroing launch followed by the sweep, in one pass.
template <int D, typename S>
__device__ __forceinline__ void smooth_blk(S* __restrict__ z, const S* __restrict__ r, const Lvl& L, const BC& bc,
                                           int phase, const SolveState* st, unsigned bid, bool fresh = false) {
  if (st && st->done) return;
  const int nl = (D == 3) ? L.n2 : L.n1;
  const int half = (nl + 1) >> 1;
  const int64_t npairs = (D == 3) ? (int64_t)L.n0 * L.n1 * half : (int64_t)L.n0 * half;
  const unsigned e = bid * blockDim.x + threadIdx.x;
  if (e >= (unsigned)npairs) return;
  int i, j, k;
  const unsigned t = udiv(e, L.dh);
  const int m = (int)(e - t * (unsigned)half);
  int other;  // the pair's member of the other colour along the last axis
  if (D == 3) {
    const unsigned q = udiv(t, L.d1);
    j = (int)(t - q * (unsigned)L.n1);
    i = (int)q;
    k = 2 * m + ((i + j + phase) & 1);
    other = k ^ 1;
    if (fresh && other < L.n2) stv(z + ((int64_t)i * L.n1 + j) * L.n2 + other, 0.f);
    if (k >= L.n2) return;
  } else {
    i = (int)t;
    j = 2 * m + ((i + phase) & 1);
    k = 0;
    other = j ^ 1;
    if (fresh && other < L.n1) stv(z + (int64_t)i * L.n1 + other, 0.f);
    if (j >= L.n1) return;
  }
  const int64_t c = ((int64_t)i * L.n1 + j) * L.n2 + k;
  if (fresh) {
    stv(z + c, (ldv(r + c) + 0.f) / stencil_mult<D>(L, bc, i, j, k));
    return;
  }
  float nb, mult;
  stencil<D>(z, L, bc, i, j, k, c, nb, mult);
  stv(z + c, (ldv(r + c) + nb) / mult);
}

template <int D, typename S>
struct OpSmooth {
  S* z;
  const S* r;
  Lvl L;
  BC bc;
  int phase;
  const SolveState* st;
  __device__ __forceinline__ void run(unsigned bid, unsigned) const { smooth_blk<D, S>(z, r, L, bc, phase, st, bid); }
};

template <int D, typename S>
__global__ void __launch_bounds__(256) k_smooth(S* __restrict__ z, const S* __restrict__ r, Lvl L,
                                                BC bc, int phase, const SolveState* st, int fresh) {
  smooth_blk<D, S>(z, r, L, bc, phase, st, blockIdx.x, fresh != 0);
}

// Eight consecutive values along the last axis (n2 % 8 == 0, so a run is 16- or 32-byte aligned).
__device__ __forceinline__ void ld8(const float* p, float (&v)[8]) {
  const float4 a = *reinterpret_cast<const float4*>(p), b = *reinterpret_cast<const float4*>(p + 4);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void st8(float* p, const float (&v)[8]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  *reinterpret_cast<float4*>(p + 4) = make_float4(v[4], v[5], v[6], v[7]);
}
template <typename H>
__device__ __forceinline__ void ld8h(const H* p, float (&v)[8]) {
  const uint4 u = *reinterpret_cast<const uint4*>(p);
  const H* h = reinterpret_cast<const H*>(&u);
#pragma unroll
  for (int q = 0; q < 8; ++q) v[q] = ldv(h + q);
}
template <typename H>
__device__ __forceinline__ void st8h(H* p, const float (&v)[8]) {
  uint4 u;
  H* h = reinterpret_cast<H*>(&u);
#pragma unroll
  for (int q = 0; q < 8; ++q) stv(h + q, v[q]);
  *reinterpret_cast<uint4*>(p) = u;
}
__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
template <typename H>
__device__ __forceinline__ void ld4h(const H* p, float (&v)[4]) {
  const uint2 u = *reinterpret_cast<const uint2*>(p);
  const H* h = reinterpret_cast<const H*>(&u);
#pragma unroll
  for (int q = 0; q < 4; ++q) v[q] = ldv(h + q);
}
__device__ __forceinline__ void ld4(const __half* p, float (&v)[4]) { ld4h(p, v); }
__device__ __forceinline__ void ld4(const __nv_bfloat16* p, float (&v)[4]) { ld4h(p, v); }
__device__ __forceinline__ void ld8(const __half* p, float (&v)[8]) { ld8h(p, v); }
__device__ __forceinline__ void ld8(const __nv_bfloat16* p, float (&v)[8]) { ld8h(p, v); }
__device__ __forceinline__ void st8(__half* p, const float (&v)[8]) { st8h(p, v); }
__device__ __forceinline__ void st8(__nv_bfloat16* p, const float (&v)[8]) { st8h(p, v); }

// k_divergence in 3D with one thread per run of eight cells along the last axis (Lv.n2 % 8 == 0):
// whole vectors of the x and y faces on either side, the nine z faces of the run one by one (their
// rows are n2 + 1 long).  The same sum, in the same order, per cell.
__global__ void __launch_bounds__(256) k_divergence8(const float* __restrict__ ux, const float* __restrict__ uy,
                                                     const float* __restrict__ uz, Lvl L, float* __restrict__ r0,
                                                     float scale) {
  const int runs = L.n2 >> 3;
  const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
  if ((int64_t)e >= (int64_t)L.n0 * L.n1 * runs) return;
  const unsigned row = e / (unsigned)runs;
  const int k0 = (int)(e - row * (unsigned)runs) * 8;
  const unsigned i_ = udiv(row, L.d1);
  const int i = (int)i_, j = (int)(row - i_ * (unsigned)L.n1);
  float vl[8], vr[8], vb[8], vt[8], z[9], out[8];
  ld8(ux + ((int64_t)i * L.n1 + j) * L.n2 + k0, vl);
  ld8(ux + ((int64_t)(i + 1) * L.n1 + j) * L.n2 + k0, vr);
  ld8(uy + ((int64_t)i * (L.n1 + 1) + j) * L.n2 + k0, vb);
  ld8(uy + ((int64_t)i * (L.n1 + 1) + j + 1) * L.n2 + k0, vt);
  const float* zr = uz + ((int64_t)i * L.n1 + j) * (L.n2 + 1) + k0;
#pragma unroll
  for (int q = 0; q < 9; ++q) z[q] = zr[q];
#pragma unroll
  for (int q = 0; q < 8; ++q) out[q] = (vr[q] - vl[q] + vt[q] - vb[q] + z[q + 1] - z[q]) * scale;
  st8(r0 + ((int64_t)i * L.n1 + j) * L.n2 + k0, out);
}

// k_residual in 3D with one thread per run of eight cells along the last axis (L.n2 % 8 == 0):
// x, b and the four neighbouring runs of x as whole vectors, each cell's neighbour sum in
// stencil<3>'s order.  The same residual per cell.
__global__ void __launch_bounds__(256) k_residual8(float* __restrict__ r, const float* __restrict__ b,
                                                   const float* __restrict__ x, Lvl L, BC bc) {
  const int runs = L.n2 >> 3;
  const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
  if ((int64_t)e >= (int64_t)L.n0 * L.n1 * runs) return;
  const unsigned row = e / (unsigned)runs;
  const int k0 = (int)(e - row * (unsigned)runs) * 8;
  const unsigned i_ = udiv(row, L.d1);
  const int i = (int)i_, j = (int)(row - i_ * (unsigned)L.n1);
  const int64_t sx = (int64_t)L.n1 * L.n2, sy = L.n2;
  const int64_t c0 = ((int64_t)i * L.n1 + j) * L.n2 + k0;
  float xc[8], bb[8], xp[8], xm[8], yp[8], ym[8], out[8];
  ld8(x + c0, xc);
  ld8(b + c0, bb);
  const bool hx = i < L.n0 - 1, lx = i > 0, hy = j < L.n1 - 1, ly = j > 0;
  if (hx) ld8(x + c0 + sx, xp);
  if (lx) ld8(x + c0 - sx, xm);
  if (hy) ld8(x + c0 + sy, yp);
  if (ly) ld8(x + c0 - sy, ym);
  const float zl = k0 > 0 ? x[c0 - 1] : 0.f;
  const float zr = k0 + 8 < L.n2 ? x[c0 + 8] : 0.f;
  float base = 6.f;
  if (i <= 0 && bc.lo[0] == 2) base -= 1.f;
  if (i >= L.n0 - 1 && bc.hi[0] == 2) base -= 1.f;
  if (j <= 0 && bc.lo[1] == 2) base -= 1.f;
  if (j >= L.n1 - 1 && bc.hi[1] == 2) base -= 1.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int k = k0 + q;
    float nb = 0.f;
    if (hx) nb += xp[q];
    if (lx) nb += xm[q];
    if (hy) nb += yp[q];
    if (ly) nb += ym[q];
    if (k < L.n2 - 1) nb += (q < 7) ? xc[q + 1] : zr;
    if (k > 0) nb += (q > 0) ? xc[q - 1] : zl;
    float mult = base;
    if (k <= 0 && bc.lo[2] == 2) mult -= 1.f;
    if (k >= L.n2 - 1 && bc.hi[2] == 2) mult -= 1.f;
    out[q] = bb[q] - (mult * xc[q] - nb);
  }
  st8(r + c0, out);
}

// The divergence of the finest level times scale into out, as runs of eight cells where the grid
// allows.
template <int D>
static void launch_divergence(pfm_handle* h, const float* ux, const float* uy, const float* uz, float* out,
                              float scale, cudaStream_t s) {
  const Lvl L = lvl_of(h, 0);
  if (D == 3 && L.n2 % 8 == 0)
    launch(h, k_divergence8, grid_for(L.count / 8, 256), 256, 0, s, ux, uy, uz, L, out, scale);
  else
    launch(h, k_divergence<D>, grid_for(h->cells, 256), 256, 0, s, ux, uy, uz, L, out, scale);
}

// The same update in 3D for the x and y face families with one thread per run of eight faces
// along the last axis (whole vectors of u and of the two pressure rows; the row index decides the
// boundary terms for the whole run); needs N2 % 8 == 0.  Element for element k_subtract_grad_p.
template <int fam>
__global__ void __launch_bounds__(256) k_subtract_grad_p8(float* __restrict__ u, const float* __restrict__ p,
                                                          MacGeom g, int lo_neu, int hi_neu) {
  static_assert(fam == 0 || fam == 1, "runs along the last axis: the x and y faces");
  const int N0 = g.N[0], N1 = g.N[1], N2 = g.N[2];
  const int n1 = g.n[fam][1], runs = N2 >> 3;
  const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
  if ((int64_t)e >= (int64_t)g.n[fam][0] * n1 * runs) return;
  const unsigned row = e / (unsigned)runs;
  const int k0 = (int)(e - row * (unsigned)runs) * 8;
  const unsigned i_ = udiv(row, g.dn[fam][1]);
  const int i = (int)i_, j = (int)(row - i_ * (unsigned)n1);
  const int a = fam == 0 ? i : j, Nf = fam == 0 ? N0 : N1;
  auto clampi = [](int v, int n) { return v < 0 ? 0 : (v > n - 1 ? n - 1 : v); };
  const int hi_a = clampi(a, Nf), lo_a = clampi(a - 1, Nf);
  const int64_t pr_row = fam == 0 ? ((int64_t)hi_a * N1 + j) * N2 : ((int64_t)i * N1 + hi_a) * N2;
  const int64_t pl_row = fam == 0 ? ((int64_t)lo_a * N1 + j) * N2 : ((int64_t)i * N1 + lo_a) * N2;
  const int64_t c0 = ((int64_t)i * n1 + j) * N2 + k0;
  float uv[8], pr[8], pl[8];
  ld8(u + c0, uv);
  ld8(p + pr_row + k0, pr);
  ld8(p + pl_row + k0, pl);
  const bool zl = a - 1 < 0, zr = a >= Nf, wall = (a == 0 && lo_neu) || (a == Nf && hi_neu);
  float out[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float r = zr ? 0.f : pr[q], l = zl ? 0.f : pl[q];
    out[q] = wall ? 0.f : uv[q] - (r - l);
  }
  st8(u + c0, out);
}

// k_subtract_grad_p of face family f, as runs of eight faces where the family and grid allow
template <int D>
static void launch_subtract_grad_p(pfm_handle* h, int f, float* u, const float* p, int lo, int hi, cudaStream_t s) {
  const MacGeom& g = h->geom;
  const int64_t nf = (int64_t)g.n[f][0] * g.n[f][1] * g.n[f][2];
  if (D == 3 && f < 2 && g.N[2] % 8 == 0) {
    const unsigned nb = grid_for(nf / 8, 256);
    if (f == 0) launch(h, k_subtract_grad_p8<0>, nb, 256, 0, s, u, p, g, lo, hi);
    if (f == 1) launch(h, k_subtract_grad_p8<1>, nb, 256, 0, s, u, p, g, lo, hi);
    return;
  }
  if (f == 0) launch(h, k_subtract_grad_p<D, 0>, grid_for(nf, 256), 256, 0, s, u, p, g, lo, hi);
  if (f == 1) launch(h, k_subtract_grad_p<D, 1>, grid_for(nf, 256), 256, 0, s, u, p, g, lo, hi);
  if (D == 3 && f == 2) launch(h, k_subtract_grad_p<3, 2>, grid_for(nf, 256), 256, 0, s, u, p, g, lo, hi);
}


// smooth(l, phase) in 3D with one thread per run of eight cells along the last axis: the run, r
// and the four neighbouring runs are read as whole vectors (the cells of the other colour, which a
// half-sweep never changes, are written back unchanged) and each cell of the colour is updated
// with the same sum, in the same order, as stencil<3> -- bitwise the result of k_smooth.
// Eight consecutive elements of a level vector as loaded (16-bit storage: one 16-byte word, four
// registers; f32: eight), converted to f32 element by element where they are used.
template <typename S>
struct Raw8 {
  uint4 u;
  __device__ __forceinline__ void load(const S* p) { u = *reinterpret_cast<const uint4*>(p); }
  __device__ __forceinline__ float operator[](int q) const { return ldv(reinterpret_cast<const S*>(&u) + q); }
};
template <>
struct Raw8<float> {
  float v[8];
  __device__ __forceinline__ void load(const float* p) { ld8(p, v); }
  __device__ __forceinline__ float operator[](int q) const { return v[q]; }
};

template <typename S>
__device__ __forceinline__ void smooth8_blk(S* __restrict__ z, const S* __restrict__ r, const Lvl& L, const BC& bc,
                                            int phase, const SolveState* st, unsigned bid, bool fresh = false) {
  if (st && st->done) return;
  const int runs = L.n2 >> 3;
  const unsigned e = bid * blockDim.x + threadIdx.x;
  if ((int64_t)e >= (int64_t)L.n0 * L.n1 * runs) return;
  const unsigned row = e / (unsigned)runs;
  const int k0 = (int)(e - row * (unsigned)runs) * 8;
  const unsigned i_ = udiv(row, L.d1);
  const int i = (int)i_, j = (int)(row - i_ * (unsigned)L.n1);
  const int64_t sx = (int64_t)L.n1 * L.n2, sy = L.n2;
  const int64_t c0 = ((int64_t)i * L.n1 + j) * L.n2 + k0;
  Raw8<S> rr, zc, xp, xm, yp, ym;
  rr.load(r + c0);
  float base = 6.f;
  if (i <= 0 && bc.lo[0] == 2) base -= 1.f;
  if (i >= L.n0 - 1 && bc.hi[0] == 2) base -= 1.f;
  if (j <= 0 && bc.lo[1] == 2) base -= 1.f;
  if (j >= L.n1 - 1 && bc.hi[1] == 2) base -= 1.f;
  const int first = (i + j + k0 + phase) & 1;  // run offset of the first cell of the colour
  float out[8];
  if (fresh) {  // z starts at zero: the colour gets (r + 0) / mult, the other colour zero
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = k0 + q;
      float num = base;
      if (k <= 0 && bc.lo[2] == 2) num -= 1.f;
      if (k >= L.n2 - 1 && bc.hi[2] == 2) num -= 1.f;
      out[q] = ((q & 1) == first) ? (rr[q] + 0.f) / num : 0.f;
    }
    st8(z + c0, out);
    return;
  }
  zc.load(z + c0);
  const bool hx = i < L.n0 - 1, lx = i > 0, hy = j < L.n1 - 1, ly = j > 0;
  if (hx) xp.load(z + c0 + sx);
  if (lx) xm.load(z + c0 - sx);
  if (hy) yp.load(z + c0 + sy);
  if (ly) ym.load(z + c0 - sy);
  const float zl = k0 > 0 ? ldv(z + c0 - 1) : 0.f;
  const float zr = k0 + 8 < L.n2 ? ldv(z + c0 + 8) : 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    out[q] = zc[q];
    if ((q & 1) != first) continue;
    const int k = k0 + q;
    float ret = 0.f;
    if (hx) ret += xp[q];
    if (lx) ret += xm[q];
    if (hy) ret += yp[q];
    if (ly) ret += ym[q];
    if (k < L.n2 - 1) ret += (q < 7) ? zc[q + 1] : zr;
    if (k > 0) ret += (q > 0) ? zc[q - 1] : zl;
    float num = base;
    if (k <= 0 && bc.lo[2] == 2) num -= 1.f;
    if (k >= L.n2 - 1 && bc.hi[2] == 2) num -= 1.f;
    out[q] = (rr[q] + ret) / num;
  }
  st8(z + c0, out);
}

template <typename S>
struct OpSmooth8 {
  S* z;
  const S* r;
  Lvl L;
  BC bc;
  int phase;
  const SolveState* st;
  __device__ __forceinline__ void run(unsigned bid, unsigned) const { smooth8_blk<S>(z, r, L, bc, phase, st, bid); }
};

// Resident blocks per SM the smoother is compiled for: f32 levels 3 (72 registers, no spill),
// 16-bit levels PFM_SMOOTH8_MINB16.
#ifndef PFM_SMOOTH8_MINB16
#define PFM_SMOOTH8_MINB16 4
#endif
template <typename S>
constexpr int smooth8_min_blocks() { return sizeof(S) == 2 ? PFM_SMOOTH8_MINB16 : 3; }

template <typename S>
__global__ void __launch_bounds__(256, smooth8_min_blocks<S>()) k_smooth8(S* __restrict__ z, const S* __restrict__ r, Lvl L, BC bc,
                                                 int phase, const SolveState* st, int fresh) {
  smooth8_blk<S>(z, r, L, bc, phase, st, blockIdx.x, fresh != 0);
}

// smooth(l, phase) in 3D for 16-bit level storage with the tile staged by the TMA: a block owns
// 4 x 8 x TK cells; one tiled load brings z over the tile and its one-cell halo (the innermost
// coordinate starts 8 cells early so that it stays 16-byte aligned; zero fill outside the level,
// where the stencil reads nothing) and one brings r over the tile.  Each thread then updates the
// cells of the colour in its run of 8 from shared memory, with the sums of stencil<3> in their
// order, and stores the run (the other colour unchanged) -- bitwise the result of k_smooth8.
// The one wait is bounded: on expiry the solve ends with code 4.
constexpr int kTmaI = 4, kTmaJ = 8, kTmaMaxK = 64;

template <typename S>
__global__ void __launch_bounds__(256) k_smooth_tma(const __grid_constant__ CUtensorMap tz,
                                                    const __grid_constant__ CUtensorMap tr, S* __restrict__ z, Lvl L,
                                                    BC bc, int phase, SolveState* st, int TK) {
  __shared__ __align__(128) S zb[(kTmaI + 2) * (kTmaJ + 2) * (kTmaMaxK + 16)];
  __shared__ __align__(128) S rb[kTmaI * kTmaJ * kTmaMaxK];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_skip;
  if (threadIdx.x == 0) s_skip = st ? *(volatile int*)&st->done : 0;
  __syncthreads();
  if (s_skip) return;
  const int tk = L.n2 / TK, tj = (L.n1 + kTmaJ - 1) / kTmaJ;
  const int b = blockIdx.x;
  const int bk = b % tk, bj = (b / tk) % tj, bi = b / (tk * tj);
  const int i0 = bi * kTmaI, j0 = bj * kTmaJ, k0 = bk * TK;
  const int W = TK + 16;  // brick row: 8 cells of halo room on each side
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bar, (uint32_t)(((kTmaI + 2) * (kTmaJ + 2) * W + kTmaI * kTmaJ * TK) * sizeof(S)));
    tma_load_3d(zb, &tz, k0 - 8, j0 - 1, i0 - 1, &bar);
    tma_load_3d(rb, &tr, k0, j0, i0, &bar);
  }
  bool ok = mbar_try_wait(&bar, 0);
  if (!ok) {
    const unsigned long long t0 = now_ns();
    while (!(ok = mbar_try_wait(&bar, 0)) && now_ns() - t0 < kWaitNs) {
    }
    if (!ok && st) atomicCAS(&st->done, 0, 4);
  }
  if (__syncthreads_or(!ok)) return;  // the copies never arrived: nothing is written
  const int R = TK >> 3;
  const int t = threadIdx.x;
  if (t >= kTmaI * kTmaJ * R) return;
  const int ii = t / (kTmaJ * R), jj = (t / R) % kTmaJ, run = t % R;
  const int i = i0 + ii, j = j0 + jj, k0r = k0 + 8 * run;
  if (i >= L.n0 || j >= L.n1) return;
  const S* row = zb + ((ii + 1) * (kTmaJ + 2) + (jj + 1)) * W + 8 + 8 * run;  // this run in the brick
  const int pw = (kTmaJ + 2) * W;                                            // brick plane
  float zc[8], rr[8], xp[8], xm[8], yp[8], ym[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    zc[q] = ldv(row + q);
    xp[q] = ldv(row + pw + q);
    xm[q] = ldv(row - pw + q);
    yp[q] = ldv(row + W + q);
    ym[q] = ldv(row - W + q);
    rr[q] = ldv(rb + (ii * kTmaJ + jj) * TK + 8 * run + q);
  }
  const float zl = ldv(row - 1), zr = ldv(row + 8);
  const bool hx = i < L.n0 - 1, lx = i > 0, hy = j < L.n1 - 1, ly = j > 0;
  float base = 6.f;
  if (i <= 0 && bc.lo[0] == 2) base -= 1.f;
  if (i >= L.n0 - 1 && bc.hi[0] == 2) base -= 1.f;
  if (j <= 0 && bc.lo[1] == 2) base -= 1.f;
  if (j >= L.n1 - 1 && bc.hi[1] == 2) base -= 1.f;
  const int first = (i + j + k0r + phase) & 1;
  float out[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) out[q] = zc[q];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if ((q & 1) != first) continue;
    const int k = k0r + q;
    float ret = 0.f;
    if (hx) ret += xp[q];
    if (lx) ret += xm[q];
    if (hy) ret += yp[q];
    if (ly) ret += ym[q];
    if (k < L.n2 - 1) ret += (q < 7) ? zc[q + 1] : zr;
    if (k > 0) ret += (q > 0) ? zc[q - 1] : zl;
    float num = base;
    if (k <= 0 && bc.lo[2] == 2) num -= 1.f;
    if (k >= L.n2 - 1 && bc.hi[2] == 2) num -= 1.f;
    out[q] = (rr[q] + ret) / num;
  }
  st8(z + ((int64_t)i * L.n1 + j) * L.n2 + k0r, out);
}

// restrict(l) as a gather: rc[I] = sum over children (fine-index order) of res/(dim-1),
// res = r - (mult z - nbsum(z)).
template <int D, typename S>
__device__ __forceinline__ void restrict_blk(const S* __restrict__ zf, const S* __restrict__ rf, const Lvl& Lf,
                                             S* __restrict__ rc, const Lvl& Lc, const BC& bc, const SolveState* st,
                                             unsigned bid) {
  if (st && st->done) return;
  int64_t e = (int64_t)bid * blockDim.x + threadIdx.x;
  if (e >= Lc.count) return;
  int I, J, K;
  decode(Lc, e, I, J, K);
  float acc = 0.f;
  const float den = (float)D - 1.0f;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int cc = 0; cc < (D == 3 ? 2 : 1); ++cc) {
        int i = 2 * I + a, j = 2 * J + b, k = (D == 3) ? 2 * K + cc : 0;
        if (i >= Lf.n0 || j >= Lf.n1 || k >= Lf.n2) continue;
        const int64_t c = ((int64_t)i * Lf.n1 + j) * Lf.n2 + k;
        float nb, mult;
        stencil<D>(zf, Lf, bc, i, j, k, c, nb, mult);
        float res = ldv(rf + c) - (mult * ldv(zf + c) - nb);
        acc += res * 1.0f / den;
      }
  stv(rc + e, acc);
}

// The same restriction in 3D with one thread per run of four coarse cells along the last axis:
// each of the 2 x 2 fine rows under them is read as whole 8-element vectors (z, r and the four
// neighbouring rows) and its eight residuals are formed as stencil<3> forms them (the same
// neighbour order); each coarse cell sums its eight in restrict_blk's order.  Needs Lf.n2 % 8 == 0.
template <typename S>
__device__ __forceinline__ void restrict8_blk(const S* __restrict__ zf, const S* __restrict__ rf, const Lvl& Lf,
                                              S* __restrict__ rc, const Lvl& Lc, const BC& bc, const SolveState* st,
                                              unsigned bid) {
  if (st && st->done) return;
  const int runs = Lc.n2 >> 2;
  const unsigned e = bid * blockDim.x + threadIdx.x;
  if ((int64_t)e >= (int64_t)Lc.n0 * Lc.n1 * runs) return;
  const unsigned row = e / (unsigned)runs;
  const int K0 = (int)(e - row * (unsigned)runs) * 4;
  const unsigned I_ = udiv(row, Lc.d1);
  const int I = (int)I_, J = (int)(row - I_ * (unsigned)Lc.n1);
  const int k0 = 2 * K0;
  const int64_t sx = (int64_t)Lf.n1 * Lf.n2, sy = Lf.n2;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const float den = 2.0f;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const int i = 2 * I + a, j = 2 * J + b;
      if (i >= Lf.n0 || j >= Lf.n1) continue;
      const int64_t c0 = ((int64_t)i * Lf.n1 + j) * Lf.n2 + k0;
      float zc[8], rr[8], xp[8], xm[8], yp[8], ym[8];
      ld8(zf + c0, zc);
      ld8(rf + c0, rr);
      const bool hx = i < Lf.n0 - 1, lx = i > 0, hy = j < Lf.n1 - 1, ly = j > 0;
      if (hx) ld8(zf + c0 + sx, xp);
      if (lx) ld8(zf + c0 - sx, xm);
      if (hy) ld8(zf + c0 + sy, yp);
      if (ly) ld8(zf + c0 - sy, ym);
      const float zl = k0 > 0 ? ldv(zf + c0 - 1) : 0.f;
      const float zr = k0 + 8 < Lf.n2 ? ldv(zf + c0 + 8) : 0.f;
      float base = 6.f;
      if (i <= 0 && bc.lo[0] == 2) base -= 1.f;
      if (i >= Lf.n0 - 1 && bc.hi[0] == 2) base -= 1.f;
      if (j <= 0 && bc.lo[1] == 2) base -= 1.f;
      if (j >= Lf.n1 - 1 && bc.hi[1] == 2) base -= 1.f;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int k = k0 + q;
        float nb = 0.f;
        if (hx) nb += xp[q];
        if (lx) nb += xm[q];
        if (hy) nb += yp[q];
        if (ly) nb += ym[q];
        if (k < Lf.n2 - 1) nb += (q < 7) ? zc[q + 1] : zr;
        if (k > 0) nb += (q > 0) ? zc[q - 1] : zl;
        float mult = base;
        if (k <= 0 && bc.lo[2] == 2) mult -= 1.f;
        if (k >= Lf.n2 - 1 && bc.hi[2] == 2) mult -= 1.f;
        const float res = rr[q] - (mult * zc[q] - nb);
        acc[q >> 1] += res * 1.0f / den;
      }
    }
  const int64_t cc = ((int64_t)I * Lc.n1 + J) * Lc.n2 + K0;
#pragma unroll
  for (int q = 0; q < 4; ++q) stv(rc + cc + q, acc[q]);
}

template <typename S>
struct OpRestrict8 {
  const S* zf;
  const S* rf;
  Lvl Lf;
  S* rc;
  Lvl Lc;
  BC bc;
  const SolveState* st;
  __device__ __forceinline__ void run(unsigned bid, unsigned) const { restrict8_blk<S>(zf, rf, Lf, rc, Lc, bc, st, bid); }
};

template <typename S>
__global__ void __launch_bounds__(256) k_restrict8(const S* __restrict__ zf, const S* __restrict__ rf, Lvl Lf,
                                                   S* __restrict__ rc, Lvl Lc, BC bc, const SolveState* st) {
  restrict8_blk<S>(zf, rf, Lf, rc, Lc, bc, st, blockIdx.x);
}

template <int D, typename S>
struct OpRestrict {
  const S* zf;
  const S* rf;
  Lvl Lf;
  S* rc;
  Lvl Lc;
  BC bc;
  const SolveState* st;
  __device__ __forceinline__ void run(unsigned bid, unsigned) const { restrict_blk<D, S>(zf, rf, Lf, rc, Lc, bc, st, bid); }
};

template <int D, typename S>
__global__ void __launch_bounds__(256) k_restrict(const S* __restrict__ zf, const S* __restrict__ rf,
                                                  Lvl Lf, S* __restrict__ rc, Lvl Lc, BC bc,
                                                  const SolveState* st) {
  restrict_blk<D, S>(zf, rf, Lf, rc, Lc, bc, st, blockIdx.x);
}

// prolongate(l): z_l[I] += z_{l+1}[I//2]
template <int D, typename S>
__device__ __forceinline__ void prolong_blk(S* __restrict__ zf, const Lvl& Lf, const S* __restrict__ zc,
                                            const Lvl& Lc, const SolveState* st, unsigned bid) {
  if (st && st->done) return;
  int64_t e = (int64_t)bid * blockDim.x + threadIdx.x;
  if (e >= Lf.count) return;
  int i, j, k;
  decode(Lf, e, i, j, k);
  int64_t ce = (D == 3) ? ((int64_t)(i >> 1) * Lc.n1 + (j >> 1)) * Lc.n2 + (k >> 1)
                        : (int64_t)(i >> 1) * Lc.n1 + (j >> 1);
  stv(zf + e, ldv(zf + e) + ldv(zc + ce));
}

template <int D, typename S>
struct OpProlong {
  S* zf;
  Lvl Lf;
  const S* zc;
  Lvl Lc;
  const SolveState* st;
  __device__ __forceinline__ void run(unsigned bid, unsigned) const { prolong_blk<D, S>(zf, Lf, zc, Lc, st, bid); }
};

template <int D, typename S>
__global__ void __launch_bounds__(256) k_prolong(S* __restrict__ zf, Lvl Lf, const S* __restrict__ zc,
                                                 Lvl Lc, const SolveState* st) {
  prolong_blk<D, S>(zf, Lf, zc, Lc, st, blockIdx.x);
}

// The same update in 3D with one thread per run of eight fine cells along the last axis (whole
// 8-element vectors of z_l, the four coarse cells under them as one vector of z_{l+1}); needs
// Lf.n2 % 8 == 0.  Element for element the sum of prolong_blk.
template <typename S>
__device__ __forceinline__ void prolong8_blk(S* __restrict__ zf, const Lvl& Lf, const S* __restrict__ zc,
                                             const Lvl& Lc, const SolveState* st, unsigned bid) {
  if (st && st->done) return;
  const int runs = Lf.n2 >> 3;
  const unsigned e = bid * blockDim.x + threadIdx.x;
  if ((int64_t)e >= (int64_t)Lf.n0 * Lf.n1 * runs) return;
  const unsigned row = e / (unsigned)runs;
  const int k0 = (int)(e - row * (unsigned)runs) * 8;
  const unsigned i_ = udiv(row, Lf.d1);
  const int i = (int)i_, j = (int)(row - i_ * (unsigned)Lf.n1);
  const int64_t c0 = ((int64_t)i * Lf.n1 + j) * Lf.n2 + k0;
  const int64_t cc = ((int64_t)(i >> 1) * Lc.n1 + (j >> 1)) * Lc.n2 + (k0 >> 1);
  float a[8], out[8], b[4];
  ld8(zf + c0, a);
  ld4(zc + cc, b);
#pragma unroll
  for (int q = 0; q < 8; ++q) out[q] = a[q] + b[q >> 1];
  st8(zf + c0, out);
}

template <typename S>
struct OpProlong8 {
  S* zf;
  Lvl Lf;
  const S* zc;
  Lvl Lc;
  const SolveState* st;
  __device__ __forceinline__ void run(unsigned bid, unsigned) const { prolong8_blk<S>(zf, Lf, zc, Lc, st, bid); }
};

template <typename S>
__global__ void __launch_bounds__(256) k_prolong8(S* __restrict__ zf, Lvl Lf, const S* __restrict__ zc, Lvl Lc,
                                                  const SolveState* st) {
  prolong8_blk<S>(zf, Lf, zc, Lc, st, blockIdx.x);
}

// init(r, k) (3D/mgpcg.py:71-79): r0 = r * k
__global__ void __launch_bounds__(256) k_scale(float* __restrict__ out, const float* __restrict__ in, int64_t n,
                                              float k) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = in[e] * k;
}

template <typename S>
__device__ __forceinline__ void zero_blk(S* __restrict__ a, int64_t n, const SolveState* st, unsigned bid, unsigned nb) {
  if (st && st->done) return;
  for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < n; e += (int64_t)nb * blockDim.x) stv(a + e, 0.f);
}

template <typename S>
struct OpZero {
  S* a;
  int64_t n;
  const SolveState* st;
  __device__ __forceinline__ void run(unsigned bid, unsigned nb) const { zero_blk<S>(a, n, st, bid, nb); }
};

template <typename S>
__global__ void __launch_bounds__(256) k_zero(S* __restrict__ a, int64_t n, const SolveState* st) {
  zero_blk<S>(a, n, st, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------------------------
// PCG kernels with fused reductions and device-side scalar updates
// ---------------------------------------------------------------------------------------------
enum RedKind { RED_ZTR_INIT = 0, RED_ZTR = 1, RED_RTR0 = 2, RED_MEAN = 3, RED_BTB = 4 };

// Per-thread partial sums of the mixed solve: Neumaier-compensated f32 (each thread adds at most a
// few hundred terms; the block and grid sums are f64).  Per-element f64 arithmetic would run on
// GB300's narrow FP64 pipe and cost about 0.1 ms per PCG iteration at 256^3.
struct CompSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = s + x;
    c += (fabsf(s) >= fabsf(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// the stopping rule of k_update_xr / k_true_residual; the relative rules accept an exactly zero
// residual, so a zero right-hand side (a fluid at rest) ends at the first check
__device__ __forceinline__ bool converged(double rTr, const SolveState* st, double tol, int tol_mode) {
  if (tol_mode == 0) return rTr < tol;
  const double ref = (tol_mode == 1) ? st->rTr0 : st->bTb;
  return rTr == 0.0 || sqrt(rTr) < tol * sqrt(ref);
}

// sum(a*b) (or sum(a) for RED_MEAN) with a finalizer that updates the solve state.  Per-thread
// partials accumulate in f32 (the reference solve) or f64 (f64 != 0, the mixed solve).
template <typename SA>
__device__ __forceinline__ void dot_blk(const SA* __restrict__ a, const float* __restrict__ b, int64_t n, RedBuf rb,
                                        int kind, double eps, double inv_n, int max_iters, int f64, unsigned bid,
                                        unsigned nb) {
  SolveState* st = rb.st;
  if (st->done) return;
  double total;
  if (f64) {
    // a 16-bit level vector (z) holds the scaled values: undo the scale of the residual it answers
    const double us = (sizeof(SA) == 2) ? 1.0 / (double)st->hscale : 1.0;
    CompSum acc;
    for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < n; e += (int64_t)nb * blockDim.x)
      acc.add((kind == RED_MEAN) ? ldv(a + e) : ldv(a + e) * b[e]);
    if (!grid_sum(acc.value() * us, rb.partials, &st->ticket, &total, bid, nb)) return;
  } else {
    float acc = 0.f;
    for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < n; e += (int64_t)nb * blockDim.x)
      acc += (kind == RED_MEAN) ? ldv(a + e) : ldv(a + e) * b[e];
    if (!grid_sum((double)acc, rb.partials, &st->ticket, &total, bid, nb)) return;
  }
  if (threadIdx.x != 0) return;
  if (kind == RED_ZTR_INIT) {
    st->zTr_old = total;
    if (max_iters == 0) {  // for i in range(0): no iteration at all
      st->done = 2;
      st->conv_it = 0;
    }
  } else if (kind == RED_ZTR) {
    // beta = new_zTr / (old_zTr + eps); p update follows (3D/mgpcg.py:268-275)
    st->beta = (float)(total / (st->zTr_old + eps));
    st->zTr_old = total;
    st->it += 1;
    if (max_iters >= 0 && st->it >= max_iters) {  // the reference's loop ends here (limit)
      st->done = 2;
      st->conv_it = st->it;
    }
  } else if (kind == RED_RTR0) {
    st->rTr0 = total;
    st->rTr = total;
    st->hscale = total > 0.0 ? (float)(1.0 / sqrt(total * inv_n)) : 1.f;
  } else if (kind == RED_BTB) {
    st->bTb = total;
  } else {
    st->mean = (float)(total * inv_n);
  }
}

template <typename SA>
struct OpDot {
  const SA* a;
  const float* b;
  int64_t n;
  RedBuf rb;
  int kind;
  double eps, inv_n;
  int max_iters, f64;
  __device__ __forceinline__ void run(unsigned bid, unsigned nb) const {
    dot_blk<SA>(a, b, n, rb, kind, eps, inv_n, max_iters, f64, bid, nb);
  }
};

template <typename SA>
__global__ void __launch_bounds__(kReduceThreads, kReduceResident) k_dot(const SA* __restrict__ a, const float* __restrict__ b,
                                                        int64_t n, RedBuf rb, int kind, double eps, double inv_n,
                                                        int max_iters, int f64) {
  dot_blk<SA>(a, b, n, rb, kind, eps, inv_n, max_iters, f64, blockIdx.x, gridDim.x);
}

// recenter (3D/mgpcg.py:174-180): r -= mean; with rh, also the level-storage copy of r that the
// mixed-precision V-cycle smooths against
template <typename S>
__device__ __forceinline__ void sub_mean_blk(float* __restrict__ r, S* __restrict__ rh, int64_t n,
                                             const SolveState* st, unsigned bid, unsigned nb) {
  if (st->done) return;
  const float m = st->mean;
  const float hs = (sizeof(S) == 2) ? st->hscale : 1.f;
  for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < n; e += (int64_t)nb * blockDim.x) {
    const float v = r[e] - m;
    r[e] = v;
    if (rh) stv(rh + e, v * hs);
  }
}

template <typename S>
struct OpSubMean {
  float* r;
  S* rh;
  int64_t n;
  const SolveState* st;
  __device__ __forceinline__ void run(unsigned bid, unsigned nb) const { sub_mean_blk<S>(r, rh, n, st, bid, nb); }
};

template <typename S>
__global__ void __launch_bounds__(256) k_sub_mean(float* __restrict__ r, S* __restrict__ rh, int64_t n,
                                                  const SolveState* st) {
  sub_mean_blk<S>(r, rh, n, st, blockIdx.x, gridDim.x);
}

// the level-storage copy of r (mixed solve without recentring)
template <typename S>
__device__ __forceinline__ void to_storage_blk(S* __restrict__ out, const float* __restrict__ in, int64_t n,
                                               const SolveState* st, unsigned bid, unsigned nb) {
  if (st->done) return;
  const float hs = (sizeof(S) == 2) ? st->hscale : 1.f;
  for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < n; e += (int64_t)nb * blockDim.x)
    stv(out + e, in[e] * hs);
}

template <typename S>
struct OpToStorage {
  S* out;
  const float* in;
  int64_t n;
  const SolveState* st;
  __device__ __forceinline__ void run(unsigned bid, unsigned nb) const { to_storage_blk<S>(out, in, n, st, bid, nb); }
};

template <typename S>
__global__ void __launch_bounds__(256) k_to_storage(S* __restrict__ out, const float* __restrict__ in, int64_t n,
                                                    const SolveState* st) {
  to_storage_blk<S>(out, in, n, st, blockIdx.x, gridDim.x);
}

// compute_Ap + reduce(p, Ap) + alpha = zTr / (pAp + eps)   (3D/mgpcg.py:237-240)
template <int D>
__device__ __forceinline__ void Ap_dot_blk(const float* __restrict__ p, float* __restrict__ Ap, const Lvl& L,
                                           const BC& bc, RedBuf rb, double eps, int f64, unsigned bid, unsigned nb) {
  SolveState* st = rb.st;
  if (st->done) return;
  float acc = 0.f;
  CompSum cacc;
  for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < L.count; e += (int64_t)nb * blockDim.x) {
    int i, j, k;
    decode(L, e, i, j, k);
    float nbs, mult;
    stencil<D>(p, L, bc, i, j, k, e, nbs, mult);
    float pe = p[e];
    float ap = mult * pe - nbs;
    Ap[e] = ap;
    if (f64) cacc.add(pe * ap);
    else acc += pe * ap;
  }
  double total;
  if (!grid_sum(f64 ? cacc.value() : (double)acc, rb.partials, &st->ticket, &total, bid, nb)) return;
  if (threadIdx.x == 0) {
    st->pAp = total;
    st->alpha = (float)(st->zTr_old / (total + eps));
  }
}

template <int D>
struct OpApDot {
  const float* p;
  float* Ap;
  Lvl L;
  BC bc;
  RedBuf rb;
  double eps;
  int f64;
  __device__ __forceinline__ void run(unsigned bid, unsigned nb) const { Ap_dot_blk<D>(p, Ap, L, bc, rb, eps, f64, bid, nb); }
};

template <int D>
__global__ void __launch_bounds__(kReduceThreads, kReduceResident) k_Ap_dot(const float* __restrict__ p, float* __restrict__ Ap,
                                                           Lvl L, BC bc, RedBuf rb, double eps, int f64) {
  Ap_dot_blk<D>(p, Ap, L, bc, rb, eps, f64, blockIdx.x, gridDim.x);
}

// update_x, update_r, reduce(r, r) and the convergence test (3D/mgpcg.py:243-258).  With x64
// (the residual-replacement solve) x accumulates in FP64 and a passing test only marks the solve
// for verification (done = 5): k_true_residual, next in the iteration, decides on the true residual.
// With want_mean the pass also sums the new r for the next recenter (sum(r) / n into st->mean),
// accumulated and reduced exactly as dot_blk's RED_MEAN pass over the same r would: the same mean.
__device__ __forceinline__ void update_xr_blk(float* __restrict__ x, const float* __restrict__ p, float* __restrict__ r,
                                              const float* __restrict__ Ap, int64_t n, RedBuf rb, double tol,
                                              int tol_mode, int f64, double inv_n, unsigned bid, unsigned nb,
                                              double* __restrict__ x64 = nullptr, bool want_mean = false) {
  SolveState* st = rb.st;
  if (st->done) return;
  const float alpha = st->alpha;
  float acc = 0.f, macc = 0.f;
  CompSum cacc, cmacc;
  for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < n; e += (int64_t)nb * blockDim.x) {
    if (x64)
      x64[e] = fma((double)alpha, (double)p[e], x64[e]);
    else
      x[e] += alpha * p[e];
    float re = r[e] - alpha * Ap[e];
    r[e] = re;
    if (f64) {
      cacc.add(re * re);
      if (want_mean) cmacc.add(re);
    } else {
      acc += re * re;
      if (want_mean) macc += re;
    }
  }
  double total, tmean = 0.0;
  if (want_mean) {
    if (!grid_sum2(f64 ? cacc.value() : (double)acc, f64 ? cmacc.value() * 1.0 : (double)macc, rb.partials,
                   &st->ticket, &total, &tmean, bid, nb))
      return;
  } else if (!grid_sum(f64 ? cacc.value() : (double)acc, rb.partials, &st->ticket, &total, bid, nb)) {
    return;
  }
  if (threadIdx.x == 0) {
    if (want_mean) st->mean = (float)(tmean * inv_n);
    st->rTr = total;
    if (total > 0.0) st->hscale = (float)(1.0 / sqrt(total * inv_n));
    if (!isfinite(total)) {
      st->done = 3;
      st->conv_it = st->it;
    } else if (converged(total, st, tol, tol_mode)) {
      st->done = x64 ? 5 : 1;
      st->conv_it = st->it;
    }
  }
}

struct OpUpdateXr {
  float* x;
  const float* p;
  float* r;
  const float* Ap;
  int64_t n;
  RedBuf rb;
  double tol;
  int tol_mode, f64;
  double inv_n;
  double* x64;
  __device__ __forceinline__ void run(unsigned bid, unsigned nb) const {
    update_xr_blk(x, p, r, Ap, n, rb, tol, tol_mode, f64, inv_n, bid, nb, x64);
  }
};

__global__ void __launch_bounds__(kReduceThreads, kReduceResident) k_update_xr(float* __restrict__ x, const float* __restrict__ p,
                                                              float* __restrict__ r, const float* __restrict__ Ap,
                                                              int64_t n, RedBuf rb, double tol, int tol_mode,
                                                              int f64, double inv_n, double* x64, int want_mean) {
  update_xr_blk(x, p, r, Ap, n, rb, tol, tol_mode, f64, inv_n, blockIdx.x, gridDim.x, x64, want_mean != 0);
}

// FP32 <-> FP64 copies of x for the residual-replacement solve
__global__ void __launch_bounds__(256) k_x_to64(double* __restrict__ x64, const float* __restrict__ x, int64_t n,
                                                const SolveState* st) {
  if (st->done) return;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    x64[e] = (double)x[e];
}

__global__ void __launch_bounds__(256) k_x_from64(float* __restrict__ x, const double* __restrict__ x64, int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    x[e] = (float)x64[e];
}

// r = b - A x: the initial residual of a warm-started solve
template <int D>
__global__ void __launch_bounds__(256) k_residual(float* __restrict__ r, const float* __restrict__ b,
                                                  const float* __restrict__ x, Lvl L, BC bc) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < L.count; e += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    decode(L, e, i, j, k);
    float nb, mult;
    stencil<D>(x, L, bc, i, j, k, e, nb, mult);
    r[e] = b[e] - (mult * x[e] - nb);
  }
}

// True-residual check: |b - A x|^2 (compensated f32 partials, f64 combination) into rTr_true,
// every `every` iterations and, with every < 0, unconditionally (after the loop).  It reports and
// does not steer: x is stored in f32, which puts a floor under the true residual (about 2e-5
// relative at 64^3 for a smooth pressure, more at 256^3) below the reference's recursive 1e-6
// rule, so replacing the recursive residual by it would hold every solve above its tolerance.
// With x64 and r (the residual-replacement solve, every > 0): the residual b - A x is formed in
// FP64 from the FP64 x, replaces the recursive residual r, and its norm decides convergence --
// every `every` iterations and whenever k_update_xr marked the solve for verification (done 5).
template <int D>
__device__ __forceinline__ void true_residual_replace_blk(const float* __restrict__ b, const double* __restrict__ x64,
                                                          float* __restrict__ r, const Lvl& L, const BC& bc,
                                                          RedBuf rb, int every, double tol, int tol_mode,
                                                          double inv_n, unsigned bid, unsigned nb) {
  SolveState* st = rb.st;
  const int done = st->done;
  if (!(done == 5 || (done == 0 && (st->it + 1) % every == 0))) return;
  double acc = 0.0;
  const int64_t sx = (int64_t)L.n1 * L.n2, sy = L.n2;
  for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < L.count; e += (int64_t)nb * blockDim.x) {
    int i, j, k;
    decode(L, e, i, j, k);
    double nbs = 0.0;
    if (i < L.n0 - 1) nbs += x64[e + sx];
    if (i > 0) nbs += x64[e - sx];
    if (j < L.n1 - 1) nbs += x64[e + sy];
    if (j > 0) nbs += x64[e - sy];
    if (D == 3) {
      if (k < L.n2 - 1) nbs += x64[e + 1];
      if (k > 0) nbs += x64[e - 1];
    }
    const double re = (double)b[e] - ((double)stencil_mult<D>(L, bc, i, j, k) * x64[e] - nbs);
    r[e] = (float)re;
    acc += re * re;
  }
  double total;
  if (!grid_sum(acc, rb.partials, &st->ticket, &total, bid, nb)) return;
  if (threadIdx.x == 0) {
    st->rTr_true = total;
    st->rTr = total;
    if (total > 0.0) st->hscale = (float)(1.0 / sqrt(total * inv_n));
    if (!isfinite(total)) {
      st->done = 3;
      st->conv_it = st->it;
    } else if (converged(total, st, tol, tol_mode)) {
      st->done = 1;
      st->conv_it = st->it;
    } else {
      st->done = 0;  // the recursive residual had drifted below the true one: iterate on
    }
  }
}

template <int D>
__device__ __forceinline__ void true_residual_blk(const float* __restrict__ b, const float* __restrict__ x,
                                                  const Lvl& L, const BC& bc, RedBuf rb, int every, unsigned bid,
                                                  unsigned nb) {
  SolveState* st = rb.st;
  if (every > 0 && (st->done != 0 || (st->it + 1) % every != 0)) return;
  CompSum acc;
  for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < L.count; e += (int64_t)nb * blockDim.x) {
    int i, j, k;
    decode(L, e, i, j, k);
    float nbs, mult;
    stencil<D>(x, L, bc, i, j, k, e, nbs, mult);
    const float re = b[e] - (mult * x[e] - nbs);
    acc.add(re * re);
  }
  double total;
  if (!grid_sum(acc.value(), rb.partials, &st->ticket, &total, bid, nb)) return;
  if (threadIdx.x == 0) st->rTr_true = total;
}

template <int D>
struct OpTrueResidual {
  const float* b;
  const float* x;
  Lvl L;
  BC bc;
  RedBuf rb;
  int every;
  const double* x64;  // non-null: the replacement form
  float* r;
  double tol;
  int tol_mode;
  double inv_n;
  __device__ __forceinline__ void run(unsigned bid, unsigned nb) const {
    if (x64)
      true_residual_replace_blk<D>(b, x64, r, L, bc, rb, every, tol, tol_mode, inv_n, bid, nb);
    else
      true_residual_blk<D>(b, x, L, bc, rb, every, bid, nb);
  }
};

template <int D>
__global__ void __launch_bounds__(kReduceThreads, kReduceResident) k_true_residual(const float* __restrict__ b,
                                                                  const float* __restrict__ x, Lvl L, BC bc,
                                                                  RedBuf rb, int every) {
  true_residual_blk<D>(b, x, L, bc, rb, every, blockIdx.x, gridDim.x);
}

template <int D>
__global__ void __launch_bounds__(kReduceThreads, kReduceResident) k_true_residual_replace(const float* __restrict__ b,
                                                                          const double* __restrict__ x64,
                                                                          float* __restrict__ r, Lvl L, BC bc,
                                                                          RedBuf rb, int every, double tol,
                                                                          int tol_mode, double inv_n) {
  true_residual_replace_blk<D>(b, x64, r, L, bc, rb, every, tol, tol_mode, inv_n, blockIdx.x, gridDim.x);
}

// update_p: p = z + beta p (3D/mgpcg.py:147-150)
template <typename SZ>
__device__ __forceinline__ void update_p_blk(float* __restrict__ p, const SZ* __restrict__ z, int64_t n,
                                             const SolveState* st, unsigned bid, unsigned nb) {
  if (st->done) return;
  const float beta = st->beta;
  if (sizeof(SZ) == 2) {  // z answers the scaled residual
    const float us = 1.f / st->hscale;
    for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < n; e += (int64_t)nb * blockDim.x)
      p[e] = ldv(z + e) * us + beta * p[e];
  } else {
    for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < n; e += (int64_t)nb * blockDim.x)
      p[e] = ldv(z + e) + beta * p[e];
  }
}

template <typename SZ>
struct OpUpdateP {
  float* p;
  const SZ* z;
  int64_t n;
  const SolveState* st;
  __device__ __forceinline__ void run(unsigned bid, unsigned nb) const { update_p_blk<SZ>(p, z, n, st, bid, nb); }
};

template <typename SZ>
__global__ void __launch_bounds__(256) k_update_p(float* __restrict__ p, const SZ* __restrict__ z, int64_t n,
                                                  const SolveState* st) {
  update_p_blk<SZ>(p, z, n, st, blockIdx.x, gridDim.x);
}

// Device loop control.  The loop body is the second half of iteration k (recenter, V-cycle, beta,
// p update) followed by the first half of iteration k+1 (Ap, alpha, x/r update, convergence
// test), so the WHILE condition is evaluated exactly where the reference breaks.  One launch of
// the loop runs at most `chunk` bodies.
__global__ void k_loop_begin(SolveState* st, int chunk, cudaGraphConditionalHandle cond) {
  st->it_stop = st->it + chunk;
  cudaGraphSetConditional(cond, (st->done == 0 && chunk > 0) ? 1u : 0u);
}

__global__ void k_loop_cond(const SolveState* st, cudaGraphConditionalHandle cond) {
  cudaGraphSetConditional(cond, (st->done == 0 && st->it < st->it_stop) ? 1u : 0u);
}

// ---------------------------------------------------------------------------------------------
// coarse-level V-cycle tail in one CTA
// ---------------------------------------------------------------------------------------------
// Levels whose cell count fits the handle's tail_cells (4096 by default) run the rest of the V-cycle (pre-smoothing,
// restriction, the bottom sweeps, prolongation, post-smoothing; 3D/mgpcg.py:182-200) inside one
// thread block, with the level vectors in shared memory and __syncthreads() between half-sweeps.
// Each cell update is the same expression as in the grid-wide kernels, in the same sweep order.
constexpr int kTailThreads = 1024;

struct TailPlan {
  int l0, L;           // levels l0 .. L-1 live in shared memory
  Lvl lv[kMaxLevels];
  int off[kMaxLevels]; // offset of level l in each of the z and r shared arrays
  int total;           // floats per array
};

template <int D>
__device__ void tail_smooth(float* z, const float* r, const Lvl& L, const BC& bc, int phase) {
  for (int e = threadIdx.x; e < (int)L.count; e += blockDim.x) {
    int i, j, k;
    decode(L, e, i, j, k);
    if (((i + j + k) & 1) == phase) {
      float nb, mult;
      stencil<D>(z, L, bc, i, j, k, e, nb, mult);
      z[e] = (r[e] + nb) / mult;
    }
  }
  __syncthreads();
}

// `iters` red-black sweeps (colour `first`, then the other) of one tail level.  When the level has
// at most kTailCpt cells per thread, each thread decodes its cells once and keeps their offsets,
// colours, neighbour masks, neighbour counts and r in registers for all the sweeps; every update
// sums the neighbours in stencil<D>'s order and divides as tail_smooth does (the same results).
constexpr int kTailCpt = 4;

template <int D>
__device__ void tail_sweeps(float* z, const float* r, const Lvl& L, const BC& bc, int iters, int first) {
  if ((int)L.count > kTailCpt * (int)blockDim.x) {  // block-uniform
    for (int it = 0; it < iters; ++it) {
      tail_smooth<D>(z, r, L, bc, first);
      tail_smooth<D>(z, r, L, bc, first ^ 1);
    }
    return;
  }
  const int sx = L.n1 * L.n2, sy = L.n2;  // a tail level holds at most kTailCpt * 1024 cells
  // per cell: bits 0-5 the neighbours present (+x, -x, +y, -y, +z, -z), bit 6 the colour, bit 7
  // the cell exists; the cell is threadIdx.x + c * blockDim.x
  unsigned msk[kTailCpt];
  float rc[kTailCpt], mc[kTailCpt];
#pragma unroll
  for (int c = 0; c < kTailCpt; ++c) {
    const int e = threadIdx.x + c * blockDim.x;
    msk[c] = 0;
    rc[c] = 0.f;
    mc[c] = 1.f;
    if (e < (int)L.count) {
      int i, j, k;
      decode(L, e, i, j, k);
      float nb, mult;
      stencil<D>(z, L, bc, i, j, k, e, nb, mult);
      msk[c] = (i < L.n0 - 1 ? 1u : 0u) | (i > 0 ? 2u : 0u) | (j < L.n1 - 1 ? 4u : 0u) | (j > 0 ? 8u : 0u) |
               (D == 3 && k < L.n2 - 1 ? 16u : 0u) | (D == 3 && k > 0 ? 32u : 0u) |
               ((unsigned)((i + j + k) & 1) << 6) | 128u;
      rc[c] = r[e];
      mc[c] = mult;
    }
  }
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const unsigned want = 128u | ((unsigned)(first ^ h) << 6);
#pragma unroll
      for (int c = 0; c < kTailCpt; ++c) {
        if ((msk[c] & 192u) == want) {
          const int e = threadIdx.x + c * blockDim.x;
          float ret = 0.f;
          if (msk[c] & 1u) ret += z[e + sx];
          if (msk[c] & 2u) ret += z[e - sx];
          if (msk[c] & 4u) ret += z[e + sy];
          if (msk[c] & 8u) ret += z[e - sy];
          if (msk[c] & 16u) ret += z[e + 1];
          if (msk[c] & 32u) ret += z[e - 1];
          z[e] = (rc[c] + ret) / mc[c];
        }
      }
      __syncthreads();
    }
}

template <int D, typename S>
__device__ __forceinline__ void tail_blk(S* __restrict__ zg, const S* __restrict__ rg, const TailPlan& T, const BC& bc,
                                         int pre_post, int bottom, const SolveState* st) {
  if (st && st->done) return;
  extern __shared__ float sh[];
  float* Z = sh;
  float* R = sh + T.total;
  const int l0 = T.l0;
  for (int e = threadIdx.x; e < (int)T.lv[l0].count; e += blockDim.x) {
    R[T.off[l0] + e] = ldv(rg + e);
    Z[T.off[l0] + e] = 0.f;
  }
  __syncthreads();
  for (int l = l0; l < T.L - 1; ++l) {
    float* z = Z + T.off[l];
    const float* r = R + T.off[l];
    tail_sweeps<D>(z, r, T.lv[l], bc, pre_post, 0);
    const Lvl Lf = T.lv[l], Lc = T.lv[l + 1];
    float* zc = Z + T.off[l + 1];
    float* rc = R + T.off[l + 1];
    for (int e = threadIdx.x; e < (int)Lc.count; e += blockDim.x) {
      int I, J, K;
      decode(Lc, e, I, J, K);
      float acc = 0.f;
      for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
          for (int cc = 0; cc < (D == 3 ? 2 : 1); ++cc) {
            int i = 2 * I + a, j = 2 * J + b, k = (D == 3) ? 2 * K + cc : 0;
            if (i >= Lf.n0 || j >= Lf.n1 || k >= Lf.n2) continue;
            const int64_t c = ((int64_t)i * Lf.n1 + j) * Lf.n2 + k;
            float nb, mult;
            stencil<D>(z, Lf, bc, i, j, k, c, nb, mult);
            float res = r[c] - (mult * z[c] - nb);
            acc += res * 1.0f / ((float)D - 1.0f);
          }
      rc[e] = acc;
      zc[e] = 0.f;
    }
    __syncthreads();
  }
  {
    float* z = Z + T.off[T.L - 1];
    const float* r = R + T.off[T.L - 1];
    tail_sweeps<D>(z, r, T.lv[T.L - 1], bc, bottom, 0);
  }
  for (int l = T.L - 2; l >= l0; --l) {
    float* z = Z + T.off[l];
    const float* r = R + T.off[l];
    const Lvl Lf = T.lv[l], Lc = T.lv[l + 1];
    const float* zc = Z + T.off[l + 1];
    for (int e = threadIdx.x; e < (int)Lf.count; e += blockDim.x) {
      int i, j, k;
      decode(Lf, e, i, j, k);
      int64_t ce = (D == 3) ? ((int64_t)(i >> 1) * Lc.n1 + (j >> 1)) * Lc.n2 + (k >> 1)
                            : (int64_t)(i >> 1) * Lc.n1 + (j >> 1);
      z[e] += zc[ce];
    }
    __syncthreads();
    tail_sweeps<D>(z, r, Lf, bc, pre_post, 1);
  }
  for (int e = threadIdx.x; e < (int)T.lv[l0].count; e += blockDim.x) stv(zg + e, Z[T.off[l0] + e]);
}

template <int D, typename S>
__global__ void __launch_bounds__(kTailThreads) k_vcycle_tail(S* __restrict__ zg, const S* __restrict__ rg,
                                                              TailPlan T, BC bc, int pre_post, int bottom,
                                                              const SolveState* st) {
  tail_blk<D, S>(zg, rg, T, bc, pre_post, bottom, st);
}

// The tail of one scene in a batched launch (one work item): the level extents travel in the work
// list and the block rebuilds the TailPlan (levels, divisors, offsets) in shared memory.
template <int D, typename S>
struct OpTail {
  S* zg;
  const S* rg;
  int l0, L;
  int n[kMaxLevels][3];
  BC bc;
  int pre_post, bottom;
  const SolveState* st;
  __device__ __forceinline__ void run(unsigned, unsigned) const {
    __shared__ TailPlan T;
    if (threadIdx.x == 0) {
      T.l0 = l0;
      T.L = L;
      int off = 0;
      for (int l = l0; l < L; ++l) {
        const int last = (D == 3) ? n[l][2] : n[l][1];
        T.lv[l] = Lvl{n[l][0], n[l][1], n[l][2], (int64_t)n[l][0] * n[l][1] * n[l][2], make_div32((unsigned)n[l][1]),
                      make_div32((unsigned)n[l][2]), make_div32((unsigned)((last + 1) >> 1))};
        T.off[l] = off;
        off += n[l][0] * n[l][1] * n[l][2];
      }
      T.total = off;
    }
    __syncthreads();
    tail_blk<D, S>(zg, rg, T, bc, pre_post, bottom, st);
  }
};

// ---------------------------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------------------------
static BC bc_of(const pfm_handle* h) {
  BC b;
  for (int d = 0; d < 3; ++d) {
    b.lo[d] = (d < h->cfg.dim) ? h->cfg.boundary[d][0] : 2;
    b.hi[d] = (d < h->cfg.dim) ? h->cfg.boundary[d][1] : 2;
  }
  return b;
}

static unsigned red_blocks(int64_t n) {
  unsigned b = grid_for(n, kReduceThreads);
  return b > (unsigned)kReduceBlocks ? (unsigned)kReduceBlocks : b;
}

// Elementwise kernels: one wave of 8 resident 256-thread blocks per SM (every block loops over an
// equal share, so no partial last wave idles most of the GPU).
static unsigned stream_blocks(int64_t n) {
  unsigned b = grid_for(n, 256);
  return b > 152u * 8u ? 152u * 8u : b;
}

// Level l's z and r in storage S.  Level 0's r is the PCG residual in the FP32 solve; the mixed
// solve smooths against its level-storage copy, kept in the upper half of level 0's z buffer
// (level-0 z uses the lower half).
template <typename S>
static S* level_z(pfm_handle* h, int l) {
  return ws_ptr<S>(h, h->o_z[l]);
}

template <typename S>
static S* level_r(pfm_handle* h, int l) {
  if (l == 0 && sizeof(S) == 2) return ws_ptr<S>(h, h->o_z[0]) + h->lv[0].count;
  return ws_ptr<S>(h, h->o_r[l]);
}

template <typename S>
static void zero_launch(pfm_handle* h, int l, const SolveState* st, cudaStream_t s) {
  launch(h, k_zero<S>, stream_blocks(h->lv[l].count), 256, 0, s, level_z<S>(h, l), h->lv[l].count, st);
}

// One red-black half-sweep of level l.  With *zero_first set, the level's z is due to be zeroed
// first: the grid-wide smoothers do both in one pass (`fresh`), the TMA-staged one after a zeroing
// launch; either way *zero_first is cleared.
template <int D, typename S>
static void smooth_launch(pfm_handle* h, int l, int phase, const SolveState* st, cudaStream_t s,
                          bool* zero_first = nullptr) {
  Lvl L = lvl_of(h, l);
  const int nl = (D == 3) ? L.n2 : L.n1;
  int64_t npairs = (D == 3) ? (int64_t)L.n0 * L.n1 * ((nl + 1) / 2) : (int64_t)L.n0 * ((nl + 1) / 2);
  int fresh = 0;
  if (zero_first && *zero_first) {
    *zero_first = false;
    fresh = 1;
  }
  if (D == 3 && sizeof(S) == 2 && L.n2 % 8 == 0 && h->smooth_tma) {  // 16-bit levels: the TMA-staged tile
    if (fresh) zero_launch<S>(h, l, st, s);
    fresh = 0;
    const int TK = L.n2 % 64 == 0 ? 64 : (L.n2 % 32 == 0 ? 32 : (L.n2 % 16 == 0 ? 16 : 8));
    CUtensorMap tz, tr;
    const bool bf = sizeof(S) == 2 && !std::is_same<S, __half>::value;
    if (make_map_3d_16bit(&tz, level_z<S>(h, l), bf, L.n0, L.n1, L.n2, kTmaI + 2, kTmaJ + 2, TK + 16) &&
        make_map_3d_16bit(&tr, level_r<S>(h, l), bf, L.n0, L.n1, L.n2, kTmaI, kTmaJ, TK)) {
      const int64_t blocks = (int64_t)((L.n0 + kTmaI - 1) / kTmaI) * ((L.n1 + kTmaJ - 1) / kTmaJ) * (L.n2 / TK);
      launch(h, k_smooth_tma<S>, (unsigned)blocks, 256, 0, s, tz, tr, level_z<S>(h, l), L, bc_of(h), phase,
             const_cast<SolveState*>(st), TK);
      return;
    }
  }
  if (D == 3 && L.n2 % 8 == 0) {
    const int64_t nvec = (int64_t)L.n0 * L.n1 * (L.n2 / 8);
    launch(h, k_smooth8<S>, grid_for(nvec, 256), 256, 0, s, level_z<S>(h, l), (const S*)level_r<S>(h, l), L,
           bc_of(h), phase, st, fresh);
    return;
  }
  launch(h, k_smooth<D, S>, grid_for(npairs, 256), 256, 0, s, level_z<S>(h, l), (const S*)level_r<S>(h, l), L,
         bc_of(h), phase, st, fresh);
}

static int tail_level(const pfm_handle* h) {
  for (int l = 0; l < h->L; ++l)
    if (h->lv[l].count <= h->tail_cells) return l;
  return h->L;  // no level small enough: every level runs as grid-wide kernels
}

// Shared memory of the tail kernel (z and r of the tail levels, f32) for a threshold.
static size_t tail_smem(const pfm_handle* h, int cells) {
  size_t total = 0;
  bool in = false;
  for (int l = 0; l < h->L; ++l) {
    if (h->lv[l].count <= cells) in = true;
    if (in) total += (size_t)h->lv[l].count;
  }
  return total * 2 * sizeof(float);
}

template <int D, typename S>
static cudaError_t allow_tail_smem(size_t bytes) {
  return cudaFuncSetAttribute(k_vcycle_tail<D, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

int set_tail_cells(pfm_handle* h, int cells) {
  if (cells < 0) return set_error(h, PFM_ERR_ARG, "tail_cells must be >= 0");
  const size_t bytes = tail_smem(h, cells);
  if (bytes > 227 * 1024) return set_error(h, PFM_ERR_ARG, "tail_cells: the tail levels exceed 227 KB of shared memory");
  if (bytes > 48 * 1024) {  // above the default dynamic shared-memory limit: opt in (once per kernel)
    cudaError_t e = h->cfg.dim == 3 ? allow_tail_smem<3, float>(bytes) : allow_tail_smem<2, float>(bytes);
    if (e == cudaSuccess) e = h->cfg.dim == 3 ? allow_tail_smem<3, __half>(bytes) : allow_tail_smem<2, __half>(bytes);
    if (e == cudaSuccess)
      e = h->cfg.dim == 3 ? allow_tail_smem<3, __nv_bfloat16>(bytes) : allow_tail_smem<2, __nv_bfloat16>(bytes);
    int rc = check_cuda(h, e, "tail shared memory");
    if (rc) return rc;
  }
  h->tail_cells = cells;
  return PFM_OK;
}

// apply_preconditioner (3D/mgpcg.py:182-200) with level storage S
// The levels' z start at zero: each level's zeroing is folded into its first half-sweep (which
// then reads no neighbours), or launched on its own where the level's first use is not a sweep
// (no pre-smoothing); the updates are the same, two to four launches fewer per V-cycle.
template <int D, typename S>
static void vcycle(pfm_handle* h, const SolveState* st, cudaStream_t s) {
  const int L = h->L;
  const BC bc = bc_of(h);
  const int l0 = tail_level(h);
  bool zero_first[kMaxLevels] = {};
  auto flush = [&](int l) {  // a use of z_l other than a half-sweep: zero it now if still due
    if (zero_first[l]) {
      zero_launch<S>(h, l, st, s);
      zero_first[l] = false;
    }
  };
  zero_first[0] = true;
  const int down_end = l0 < L ? l0 : L - 1;  // grid-wide levels that restrict to a coarser one
  for (int l = 0; l < down_end; ++l) {
    for (int i = 0; i < h->cfg.pre_post_smoothing; ++i) {
      smooth_launch<D, S>(h, l, 0, st, s, &zero_first[l]);
      smooth_launch<D, S>(h, l, 1, st, s);
    }
    flush(l);  // the restriction reads z_l
    if (l + 1 != l0) zero_first[l + 1] = true;
    Lvl Lf = lvl_of(h, l), Lc = lvl_of(h, l + 1);
    if (D == 3 && Lf.n2 % 8 == 0)
      launch(h, k_restrict8<S>, grid_for((int64_t)Lc.n0 * Lc.n1 * (Lc.n2 / 4), 256), 256, 0, s,
             (const S*)level_z<S>(h, l), (const S*)level_r<S>(h, l), Lf, level_r<S>(h, l + 1), Lc, bc, st);
    else
      launch(h, k_restrict<D, S>, grid_for(Lc.count, 256), 256, 0, s, (const S*)level_z<S>(h, l),
             (const S*)level_r<S>(h, l), Lf, level_r<S>(h, l + 1), Lc, bc, st);
  }
  if (l0 < L) {
    TailPlan T{};
    T.l0 = l0;
    T.L = L;
    int off = 0;
    for (int l = l0; l < L; ++l) {
      T.lv[l] = lvl_of(h, l);
      T.off[l] = off;
      off += (int)h->lv[l].count;
    }
    T.total = off;
    const size_t smem = (size_t)off * 2 * sizeof(float);
    zero_first[l0] = false;  // the tail starts its levels from zero and writes all of z_l0
    launch(h, k_vcycle_tail<D, S>, 1, kTailThreads, smem, s, level_z<S>(h, l0), (const S*)level_r<S>(h, l0), T, bc,
           h->cfg.pre_post_smoothing, h->cfg.bottom_smoothing, st);
  } else {
    for (int i = 0; i < h->cfg.bottom_smoothing; ++i) {
      smooth_launch<D, S>(h, L - 1, 0, st, s, &zero_first[L - 1]);
      smooth_launch<D, S>(h, L - 1, 1, st, s);
    }
    flush(L - 1);
  }
  for (int l = down_end - 1; l >= 0; --l) {
    Lvl Lf = lvl_of(h, l), Lc = lvl_of(h, l + 1);
    flush(l);  // the prolongation reads z_l and z_{l+1}
    flush(l + 1);
    if (D == 3 && Lf.n2 % 8 == 0)
      launch(h, k_prolong8<S>, grid_for((int64_t)Lf.n0 * Lf.n1 * (Lf.n2 / 8), 256), 256, 0, s, level_z<S>(h, l), Lf,
             (const S*)level_z<S>(h, l + 1), Lc, st);
    else
      launch(h, k_prolong<D, S>, grid_for(Lf.count, 256), 256, 0, s, level_z<S>(h, l), Lf,
             (const S*)level_z<S>(h, l + 1), Lc, st);
    for (int i = 0; i < h->cfg.pre_post_smoothing; ++i) {
      smooth_launch<D, S>(h, l, 1, st, s);
      smooth_launch<D, S>(h, l, 0, st, s);
    }
  }
}

static bool all_neumann(const pfm_handle* h) {
  for (int d = 0; d < h->cfg.dim; ++d)
    if (h->cfg.boundary[d][0] != 2 || h->cfg.boundary[d][1] != 2) return false;
  return true;
}

// Captures `body` (kernels only) on the handle's capture stream into an executable graph.
template <class F>
static int capture(pfm_handle* h, F&& body, cudaGraphExec_t* exec, int* nodes) {
  if (!h->cap_stream) {
    int rc = check_cuda(h, cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking), "capture stream");
    if (rc) return rc;
  }
  cudaGraph_t g = nullptr;
  int rc = check_cuda(h, cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  if (rc) return rc;
  const uint64_t before = h->launches;
  body(h->cap_stream);
  *nodes = (int)(h->launches - before);
  h->launches = before;
  rc = check_cuda(h, cudaStreamEndCapture(h->cap_stream, &g), "end capture");
  if (rc) return rc;
  rc = check_cuda(h, cudaGraphInstantiate(exec, g, 0), "graph instantiate");
  cudaGraphDestroy(g);
  return rc;
}

static int run_graph(pfm_handle* h, cudaGraphExec_t exec, int nodes, cudaStream_t s) {
  h->launches += (uint64_t)nodes;
  return check_cuda(h, cudaGraphLaunch(exec, s), "graph launch");
}

// k_loop_begin, the WHILE node whose body is one solver iteration, and the solve's finish, appended
// to the graph behind the cursor.  Returns the body's kernel count.
template <class K>
static int append_solve_loop(GraphCursor& gc, K& k) {
  pfm_handle* h = gc.h;
  cudaGraphConditionalHandle cond{};
  if (!gc.rc) gc.rc = check_cuda(h, cudaGraphConditionalHandleCreate(&cond, gc.G, 0, 0), "conditional handle");
  if (gc.rc) return 0;
  launch(h, k_loop_begin, 1, 1, 0, gc.seg(), k.st, k.chunk, cond);
  cudaGraph_t body = gc.add_conditional(cond, cudaGraphCondTypeWhile);
  if (gc.rc) return 0;
  const uint64_t b0 = h->launches;
  gc.capture_body(body, [&](cudaStream_t q) { k.body(q, cond); });
  const int nodes = (int)(h->launches - b0);
  if (!gc.rc) k.finish(gc.seg());
  return nodes;
}

// The kernels of one MGPCG.solve (3D/mgpcg.py:202-280) with level storage S (float: the reference
// solve; __half / __nv_bfloat16: the mixed solve, which also accumulates every inner product in
// f64), grouped as the graphs use them:
//   setup:  x (unless warm-started) = p = 0, recenter, [b = r0, b.b, r0 = b - A x for a warm
//           start], r0.r0, first V-cycle, p = z, z.r, and the first half of iteration 1 (Ap,
//           alpha, x/r update, convergence test [, true residual]);
//   body:   one WHILE iteration: the second half of iteration k and the first half of k+1, then
//           k_loop_cond clears the loop condition once converged or at the iteration limit;
//   finish: the final true residual (when monitored).
template <int D, typename S>
struct SolveKernels {
  pfm_handle* h;
  pfm_solve_opts o;
  bool mixed, warm, true_res, keep_b, neu, replace;
  // the next recenter's mean is summed by k_update_xr (all-Neumann; not when the true-residual
  // replacement rewrites r after it)
  bool fuse_mean;
  int f64, chunk, mi;
  int64_t n;
  double inv_n;
  SolveState* st;
  RedBuf rb;
  float *r0, *x, *p, *Ap, *bvec;
  double* x64;  // the residual-replacement solve's FP64 x (else null)
  S *z0, *rh;
  Lvl L0;
  BC bc;

  SolveKernels(pfm_handle* hh, const pfm_solve_opts& oo) : h(hh), o(oo) {
    mixed = sizeof(S) == 2;
    f64 = mixed ? 1 : 0;
    warm = o.warm_start != 0;
    true_res = o.true_residual_every > 0;
    replace = mixed && true_res && o.true_residual_replace != 0;
    keep_b = warm || true_res || o.tol_mode == 2;
    chunk = o.max_iters >= 0 ? o.max_iters + 1 : o.check_every;
    mi = o.max_iters;
    n = h->cells;
    inv_n = 1.0 / (double)n;
    neu = all_neumann(h);
    fuse_mean = neu && !replace;
    st = ws_ptr<SolveState>(h, h->o_state);
    rb = RedBuf{ws_ptr<double>(h, h->o_partials), st};
    r0 = ws_ptr<float>(h, h->o_r[0]);
    z0 = level_z<S>(h, 0);
    rh = mixed ? level_r<S>(h, 0) : nullptr;
    x = ws_ptr<float>(h, h->o_x);
    p = ws_ptr<float>(h, h->o_p);
    Ap = ws_ptr<float>(h, h->o_Ap);
    bvec = ws_ptr<float>(h, h->o_b);
    x64 = replace ? ws_ptr<double>(h, h->o_x64) : nullptr;
    L0 = lvl_of(h, 0);
    bc = bc_of(h);
  }
  // recenter r0 (all-Neumann) and, in the mixed solve with `storage`, refresh its scaled
  // level-storage copy.  With mean_ready the mean was summed by the k_update_xr that wrote r0.
  void recenter(cudaStream_t q, bool storage, bool mean_ready = false) {
    S* out = (mixed && storage) ? rh : nullptr;
    if (neu) {
      if (!mean_ready)
        launch(h, k_dot<float>, red_blocks(n), kReduceThreads, 0, q, (const float*)r0, (const float*)nullptr, n, rb,
               (int)RED_MEAN, o.eps, inv_n, mi, f64);
      launch(h, k_sub_mean<S>, stream_blocks(n), 256, 0, q, r0, out, n, (const SolveState*)st);
    } else if (out) {
      launch(h, k_to_storage<S>, stream_blocks(n), 256, 0, q, out, (const float*)r0, n, (const SolveState*)st);
    }
  }
  void first_half(cudaStream_t q) {
    launch(h, k_Ap_dot<D>, red_blocks(n), kReduceThreads, 0, q, (const float*)p, Ap, L0, bc, rb, o.eps, f64);
    launch(h, k_update_xr, red_blocks(n), kReduceThreads, 0, q, x, (const float*)p, r0, (const float*)Ap, n, rb, o.tol,
           o.tol_mode, f64, inv_n, x64, fuse_mean ? 1 : 0);
    if (replace)
      launch(h, k_true_residual_replace<D>, red_blocks(n), kReduceThreads, 0, q, (const float*)bvec,
             (const double*)x64, r0, L0, bc, rb, o.true_residual_every, o.tol, o.tol_mode, inv_n);
    else if (true_res)
      launch(h, k_true_residual<D>, red_blocks(n), kReduceThreads, 0, q, (const float*)bvec, (const float*)x, L0, bc, rb,
             o.true_residual_every);
  }
  void setup(cudaStream_t q) {
    // init(): x = p = Ap = 0 (3D/mgpcg.py:63-79); z0 is zeroed by the V-cycle, and Ap needs no
    // zeroing: k_Ap_dot writes every element before k_update_xr reads it
    cudaMemsetAsync(st, 0, sizeof(SolveState), q);
    if (!warm) cudaMemsetAsync(x, 0, n * 4, q);
    cudaMemsetAsync(p, 0, n * 4, q);
    recenter(q, false);
    if (keep_b) {
      cudaMemcpyAsync(bvec, r0, n * 4, cudaMemcpyDeviceToDevice, q);
      launch(h, k_dot<float>, red_blocks(n), kReduceThreads, 0, q, (const float*)bvec, (const float*)bvec, n, rb,
             (int)RED_BTB, o.eps, inv_n, mi, 1);
    }
    if (warm) {
      if (D == 3 && L0.n2 % 8 == 0)
        launch(h, k_residual8, grid_for(n / 8, 256), 256, 0, q, r0, (const float*)bvec, (const float*)x, L0, bc);
      else
        launch(h, k_residual<D>, stream_blocks(n), 256, 0, q, r0, (const float*)bvec, (const float*)x, L0, bc);
    }
    if (replace) launch(h, k_x_to64, stream_blocks(n), 256, 0, q, x64, (const float*)x, n, (const SolveState*)st);
    launch(h, k_dot<float>, red_blocks(n), kReduceThreads, 0, q, (const float*)r0, (const float*)r0, n, rb,
           (int)RED_RTR0, o.eps, inv_n, mi, f64);
    // the scaled level-storage copy of r0, once r0.r0 (and so the scale) is known
    if (mixed) launch(h, k_to_storage<S>, stream_blocks(n), 256, 0, q, rh, (const float*)r0, n, (const SolveState*)st);
    vcycle<D, S>(h, st, q);
    launch(h, k_update_p<S>, stream_blocks(n), 256, 0, q, p, (const S*)z0, n, (const SolveState*)st);
    launch(h, k_dot<S>, red_blocks(n), kReduceThreads, 0, q, (const S*)z0, (const float*)r0, n, rb, (int)RED_ZTR_INIT,
           o.eps, inv_n, mi, f64);
    first_half(q);
  }
  void body(cudaStream_t q, cudaGraphConditionalHandle cond) {
    recenter(q, true, fuse_mean);
    vcycle<D, S>(h, st, q);
    launch(h, k_dot<S>, red_blocks(n), kReduceThreads, 0, q, (const S*)z0, (const float*)r0, n, rb, (int)RED_ZTR, o.eps,
           inv_n, mi, f64);
    launch(h, k_update_p<S>, stream_blocks(n), 256, 0, q, p, (const S*)z0, n, (const SolveState*)st);
    first_half(q);
    launch(h, k_loop_cond, 1, 1, 0, q, (const SolveState*)st, cond);
  }
  void finish(cudaStream_t q) {
    if (replace)  // the FP32 pressure the caller receives
      launch(h, k_x_from64, stream_blocks(n), 256, 0, q, x, (const double*)x64, n);
    if (true_res)  // the final true residual of the solve (of the FP32 pressure)
      launch(h, k_true_residual<D>, red_blocks(n), kReduceThreads, 0, q, (const float*)bvec, (const float*)x, L0, bc, rb,
             -1);
  }
};

// MGPCG.solve (3D/mgpcg.py:202-280) on r_0 (already k r); the solution is left in the workspace
// vector x.  Two graphs per handle, captured once per option set: the setup graph and the loop
// graph (k_loop_begin -> WHILE(not done and it < it_stop) { body } -> finish -> the device state
// copied to pinned host memory).  With a finite max_iters one loop launch finishes the solve;
// with max_iters = -1 the host relaunches the loop every check_every iterations until the state
// reports convergence.
template <int D, typename S>
static int solve_impl(pfm_handle* h, const pfm_solve_opts& o, pfm_solve_stats* stats, cudaStream_t s) {
  SolveKernels<D, S> K(h, o);
  const int mi = K.mi;
  const int chunk = K.chunk;
  SolveState* hs = h->h_state;
  const int key_mode = (o.precision & 3) | (K.warm ? 4 : 0) | (K.replace ? 8 : 0);
  if (!h->g_valid || h->g_eps != o.eps || h->g_tol != o.tol || h->g_mode != o.tol_mode || h->g_max_iters != mi ||
      h->g_chunk != chunk || h->g_variant != key_mode || h->g_true_every != o.true_residual_every) {
    if (h->g_setup) cudaGraphExecDestroy(h->g_setup);
    if (h->g_loop) cudaGraphExecDestroy(h->g_loop);
    h->g_setup = h->g_loop = nullptr;
    h->g_valid = 0;
    int rc = capture(h, [&](cudaStream_t q) { K.setup(q); }, &h->g_setup, &h->g_setup_nodes);
    if (rc) return rc;
    cudaGraph_t top = nullptr;
    rc = check_cuda(h, cudaGraphCreate(&top, 0), "graph create");
    if (rc) return rc;
    GraphCursor gc(h, top, h->cap_stream);
    const uint64_t before = h->launches;
    h->g_body_nodes = append_solve_loop(gc, K);
    if (!gc.rc) cudaMemcpyAsync(hs, K.st, sizeof(SolveState), cudaMemcpyDeviceToHost, gc.seg());
    gc.close();
    h->launches = before;
    rc = gc.rc;
    if (!rc) rc = check_cuda(h, cudaGraphInstantiate(&h->g_loop, top, 0), "loop graph instantiate");
    cudaGraphDestroy(top);
    if (rc) return rc;
    h->g_eps = o.eps;
    h->g_tol = o.tol;
    h->g_mode = o.tol_mode;
    h->g_max_iters = mi;
    h->g_chunk = chunk;
    h->g_variant = key_mode;
    h->g_true_every = o.true_residual_every;
    h->g_valid = 1;
  }
  int rc = run_graph(h, h->g_setup, h->g_setup_nodes, s);
  if (rc) return rc;
  int it_before = 0;
  while (true) {
    rc = check_cuda(h, cudaGraphLaunch(h->g_loop, s), "loop graph launch");
    if (rc) return rc;
    rc = check_cuda(h, cudaStreamSynchronize(s), "mgpcg sync");
    if (rc) return rc;
    // kernels launched: k_loop_begin, one body per completed iteration (k_loop_cond inside), and
    // the final true-residual check
    h->launches += 1 + (uint64_t)h->g_body_nodes * (uint64_t)(hs->it - it_before) + (K.true_res ? 1 : 0) + (K.replace ? 1 : 0);
    it_before = hs->it;
    if (hs->done || mi >= 0) break;
  }
  if (stats) {
    stats->converged = hs->done == 1;
    stats->iterations = hs->done ? hs->conv_it : hs->it;
    stats->rTr = hs->rTr;
    stats->rTr0 = hs->rTr0;
    stats->bTb = hs->bTb;
    stats->rTr_true = K.true_res ? hs->rTr_true : -1.0;
  }
  if (hs->done == 3) return set_error(h, PFM_ERR_NONFINITE, "MGPCG: non-finite residual");
  if (hs->done == 4) return set_error(h, PFM_ERR_CUDA, "MGPCG: a smoother's tile copy did not arrive");
  if (hs->done != 1) return set_error(h, PFM_ERR_NOT_CONVERGED, "MGPCG: iteration limit reached");
  return PFM_OK;
}

template <int D>
static int solve_dispatch(pfm_handle* h, const pfm_solve_opts* opts, pfm_solve_stats* stats, cudaStream_t s) {
  pfm_solve_opts o{400, 1e-12, 1e-12, 0, 4, 0, 0, 0, 0};
  if (opts) o = *opts;
  if (o.check_every < 1) o.check_every = 1;
  if (o.tol_mode < 0 || o.tol_mode > 2) return set_error(h, PFM_ERR_ARG, "MGPCG: tol_mode must be 0, 1 or 2");
  if (o.precision == 1) return solve_impl<D, __half>(h, o, stats, s);
  if (o.precision == 2) return solve_impl<D, __nv_bfloat16>(h, o, stats, s);
  if (o.precision != 0) return set_error(h, PFM_ERR_ARG, "MGPCG: precision must be 0 (FP32), 1 (FP16) or 2 (BF16)");
  return solve_impl<D, float>(h, o, stats, s);
}

// The warm-start guess from the buffer's current pressure p and the slot's history (h1 the solution
// before p, h2 the one before h1; `count` of them are valid): MODE 2 x = 2 p - h1, the linear
// extrapolation; MODE 3 x = 3 (p - h1) + h2, the quadratic one through the three solutions (with
// fewer solutions kept, the highest order they allow; with none, x = p).  The history then
// shifts (h2 = h1, h1 = p) in both modes, so either may follow the other; k_bump_count counts it.
template <int MODE>
__global__ void __launch_bounds__(256) k_warm_extrap(float* __restrict__ x, float* __restrict__ h1,
                                                     float* __restrict__ h2, const float* __restrict__ p, int64_t n,
                                                     const int* count) {
  const int c = *count;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const float v = p[e];
    if (c == 0) {
      x[e] = v;
    } else {
      const float a = h1[e];
      if (MODE == 3 && c >= 2)
        x[e] = __fadd_rn(__fmul_rn(3.f, __fsub_rn(v, a)), h2[e]);
      else
        x[e] = __fsub_rn(2.f * v, a);
      h2[e] = a;
    }
    h1[e] = v;
  }
}

__global__ void k_bump_count(int* count) { *count = *count < 2 ? *count + 1 : 2; }

int warm_start_init(pfm_handle* h, float* x, const float* p_io, int mode, cudaStream_t s) {
  if (!p_io) return set_error(h, PFM_ERR_NULL, "MGPCG: warm_start needs the pressure buffer");
  if (mode == 1)
    return check_cuda(h, cudaMemcpyAsync(x, p_io, h->cells * 4, cudaMemcpyDeviceToDevice, s), "copy initial guess");
  int slot = -1;
  for (int k = 0; k < 2 && slot < 0; ++k)
    if (h->hist_ptr[k] == p_io) slot = k;
  for (int k = 0; k < 2 && slot < 0; ++k)
    if (!h->hist_ptr[k]) {
      h->hist_ptr[k] = p_io;
      slot = k;
    }
  if (slot < 0)
    return set_error(h, PFM_ERR_ARG,
                     "MGPCG: warm_start 2 and 3 keep the history of at most two pressure buffers per handle");
  float* h1 = ws_ptr<float>(h, h->o_hist) + (size_t)(2 * slot) * h->cells;
  float* h2 = h1 + h->cells;
  int* count = ws_ptr<int>(h, h->o_hist_flag) + slot;
  if (mode == 3)
    launch(h, k_warm_extrap<3>, stream_blocks(h->cells), 256, 0, s, x, h1, h2, p_io, (int64_t)h->cells,
           (const int*)count);
  else
    launch(h, k_warm_extrap<2>, stream_blocks(h->cells), 256, 0, s, x, h1, h2, p_io, (int64_t)h->cells,
           (const int*)count);
  launch(h, k_bump_count, 1, 1, 0, s, count);
  return launch_check(h, "warm start");
}

int mgpcg_solve_in_place(pfm_handle* h, float* x_out, const pfm_solve_opts* opts, pfm_solve_stats* stats,
                         cudaStream_t s) {
  if (opts && (opts->warm_start < 0 || opts->warm_start > 3))
    return set_error(h, PFM_ERR_ARG, "MGPCG: warm_start must be 0, 1, 2 or 3");
  if (opts && opts->warm_start) {  // the initial guess from the caller's current x_out
    int c = warm_start_init(h, ws_ptr<float>(h, h->o_x), x_out, opts->warm_start, s);
    if (c) return c;
  }
  int rc = h->cfg.dim == 3 ? solve_dispatch<3>(h, opts, stats, s) : solve_dispatch<2>(h, opts, stats, s);
  if (rc != PFM_OK && rc != PFM_ERR_NOT_CONVERGED) return rc;
  if (x_out) {
    int c = check_cuda(h, cudaMemcpyAsync(x_out, ws_ptr<float>(h, h->o_x), h->cells * 4, cudaMemcpyDeviceToDevice, s),
                       "copy pressure");
    if (c) return c;
  }
  return rc;
}

template <int D>
static int poisson_impl(pfm_handle* h, float* const* u, float* p_out, const pfm_solve_opts* opts,
                        pfm_solve_stats* stats, cudaStream_t s) {
  int rc = require_ws(h);
  if (rc) return rc;
  const MacGeom& g = h->geom;
  for (int f = 0; f < D; ++f) {
    int a1 = (f == 0) ? 1 : 0, a2 = (f == 2) ? 1 : 2;
    int64_t plane = (int64_t)g.n[f][a1] * (D == 3 ? g.n[f][a2] : 1);
    launch(h, k_apply_bc<D>, grid_for(2 * plane, 256), 256, 0, s, u[f], f, g, h->cfg.boundary[f][0] == 2,
                                                          h->cfg.boundary[f][1] == 2);
  }
  float* r0 = ws_ptr<float>(h, h->o_r[0]);
  launch_divergence<D>(h, u[0], u[1], D == 3 ? u[2] : nullptr, r0, -1.f, s);
  rc = launch_check(h, "divergence");
  if (rc) return rc;
  int solve_rc = mgpcg_solve_in_place(h, p_out, opts, stats, s);
  const float* x = ws_ptr<float>(h, h->o_x);
  if (solve_rc != PFM_OK && solve_rc != PFM_ERR_NOT_CONVERGED) return solve_rc;
  for (int f = 0; f < D; ++f) {
    const int lo = h->cfg.boundary[f][0] == 2, hi = h->cfg.boundary[f][1] == 2;
    launch_subtract_grad_p<D>(h, f, u[f], x, lo, hi, s);
  }
  rc = launch_check(h, "subtract_grad_p");
  if (rc) return rc;
  return solve_rc;
}

// Records the finished solve in the step state: iterations, done code, final r.r, and the kernels
// its WHILE body ran (iterations x body).
__global__ void k_record_solve(StepCtl* ctl, const SolveState* st, int which, int body_nodes) {
  ctl->iters[which] = st->done ? st->conv_it : st->it;
  ctl->history[(ctl->i & 63)][which] = ctl->iters[which];
  ctl->done[which] = st->done;
  ctl->rTr[which] = st->rTr;
  ctl->kernels += (unsigned long long)st->it * (unsigned long long)body_nodes;
}

template <int D, typename S>
static void append_solve(GraphCursor& gc, const pfm_solve_opts& o, StepCtl* ctl, int which) {
  SolveKernels<D, S> K(gc.h, o);
  const int body = append_solve_loop(gc, K);
  if (gc.rc) return;
  launch(gc.h, k_record_solve, 1, 1, 0, gc.seg(), ctl, (const SolveState*)K.st, which, body);
}

template <class F>
static void dispatch_solve(int D, int precision, F&& f) {
  if (D == 3) {
    if (precision == 1) f(std::integral_constant<int, 3>(), __half());
    else if (precision == 2) f(std::integral_constant<int, 3>(), __nv_bfloat16());
    else f(std::integral_constant<int, 3>(), float());
  } else {
    if (precision == 1) f(std::integral_constant<int, 2>(), __half());
    else if (precision == 2) f(std::integral_constant<int, 2>(), __nv_bfloat16());
    else f(std::integral_constant<int, 2>(), float());
  }
}

// MGPCG_3/MGPCG_2.Poisson appended to a whole-step graph in three parts -- pre: apply_bc,
// divergence, [warm start from p_io], the solve's setup; loop: the device iteration loop and the
// statistics to ctl (slot `which`); post: [pressure to p_io], subtract_grad_p with the wall reset.
// Nothing waits on the host.  A batch in work-list mode emits every scene's pre and post parts in
// the scene's own branch and one batched loop for all of them (append_batched_loop).
int append_poisson_pre(GraphCursor& gc, float* const* u, float* p_io, const pfm_solve_opts& opts) {
  pfm_handle* h = gc.h;
  const int D = h->cfg.dim;
  const MacGeom& g = h->geom;
  pfm_solve_opts o = opts;
  if (!p_io) o.warm_start = 0;
  cudaStream_t q = gc.seg();
  for (int f = 0; f < D; ++f) {
    const int a1 = (f == 0) ? 1 : 0, a2 = (f == 2) ? 1 : 2;
    const int64_t plane = (int64_t)g.n[f][a1] * (D == 3 ? g.n[f][a2] : 1);
    if (D == 3)
      launch(h, k_apply_bc<3>, grid_for(2 * plane, 256), 256, 0, q, u[f], f, g, h->cfg.boundary[f][0] == 2,
             h->cfg.boundary[f][1] == 2);
    else
      launch(h, k_apply_bc<2>, grid_for(2 * plane, 256), 256, 0, q, u[f], f, g, h->cfg.boundary[f][0] == 2,
             h->cfg.boundary[f][1] == 2);
  }
  float* r0 = ws_ptr<float>(h, h->o_r[0]);
  float* x = ws_ptr<float>(h, h->o_x);
  if (D == 3)
    launch_divergence<3>(h, u[0], u[1], u[2], r0, -1.f, q);
  else
    launch_divergence<2>(h, u[0], u[1], nullptr, r0, -1.f, q);
  if (o.warm_start && !gc.rc) gc.rc = warm_start_init(h, x, p_io, o.warm_start, q);
  dispatch_solve(D, o.precision, [&](auto dd, auto ss) {
    SolveKernels<decltype(dd)::value, decltype(ss)> K(h, o);
    K.setup(gc.seg());
  });
  return gc.rc;
}

int append_poisson_loop(GraphCursor& gc, const pfm_solve_opts& opts, float* p_io, StepCtl* ctl, int which) {
  pfm_solve_opts o = opts;
  if (!p_io) o.warm_start = 0;
  dispatch_solve(gc.h->cfg.dim, o.precision,
                 [&](auto dd, auto ss) { append_solve<decltype(dd)::value, decltype(ss)>(gc, o, ctl, which); });
  return gc.rc;
}

int append_poisson_post(GraphCursor& gc, float* const* u, float* p_io) {
  pfm_handle* h = gc.h;
  if (gc.rc) return gc.rc;
  const int D = h->cfg.dim;
  float* x = ws_ptr<float>(h, h->o_x);
  cudaStream_t q = gc.seg();
  if (p_io) cudaMemcpyAsync(p_io, x, h->cells * 4, cudaMemcpyDeviceToDevice, q);
  for (int f = 0; f < D; ++f) {
    const int lo = h->cfg.boundary[f][0] == 2, hi = h->cfg.boundary[f][1] == 2;
    if (D == 3) launch_subtract_grad_p<3>(h, f, u[f], x, lo, hi, q);
    else launch_subtract_grad_p<2>(h, f, u[f], x, lo, hi, q);
  }
  return gc.rc;
}

int append_poisson(GraphCursor& gc, float* const* u, float* p_io, const pfm_solve_opts& opts, StepCtl* ctl,
                   int which) {
  append_poisson_pre(gc, u, p_io, opts);
  if (gc.rc) return gc.rc;
  append_poisson_loop(gc, opts, p_io, ctl, which);
  if (gc.rc) return gc.rc;
  return append_poisson_post(gc, u, p_io);
}

// ---------------------------------------------------------------------------------------------
// batched MGPCG iterations: persistent kernels over a work list of (scene, block) items
// ---------------------------------------------------------------------------------------------
// A work list: scene s owns items [prefix[s], prefix[s+1]), item w of it is block w - prefix[s] of
// the scene's own launch of the operation (the same partition as the scene's standalone kernel,
// so its reductions combine the same partials in the same order: bitwise the standalone result).
// The list travels as the kernel's parameter (no device allocation): at most kBatchMax scenes per
// launch.
constexpr int kBatchMax = 64;

template <class Op>
struct WorkList {
  int n;
  int prefix[kBatchMax + 1];
  Op op[kBatchMax];
};

// A grid sized for the GPU's resident blocks walks the list; a scene whose solve has finished
// costs one read of its done flag per item (every operation starts with that test).
template <class Op, int THREADS>
__global__ void __launch_bounds__(THREADS) k_worklist(const __grid_constant__ WorkList<Op> wl) {
  const int total = wl.prefix[wl.n];
  for (int w = blockIdx.x; w < total; w += gridDim.x) {
    int lo = 0, hi = wl.n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (wl.prefix[mid] <= w) lo = mid;
      else hi = mid - 1;
    }
    wl.op[lo].run((unsigned)(w - wl.prefix[lo]), (unsigned)(wl.prefix[lo + 1] - wl.prefix[lo]));
    __syncthreads();
  }
}

template <class Op>
struct WorkItems {
  std::vector<Op> ops;
  std::vector<unsigned> blocks;
  void add(const Op& op, unsigned nb) {
    if (nb == 0) return;
    ops.push_back(op);
    blocks.push_back(nb);
  }
};

template <class Op, int THREADS>
static void launch_worklist(pfm_handle* h, cudaStream_t q, const WorkItems<Op>& it, size_t smem = 0) {
  constexpr unsigned kResident = 152u * (2048u / THREADS);  // resident blocks of the 152 SMs
  for (size_t c0 = 0; c0 < it.ops.size(); c0 += kBatchMax) {
    WorkList<Op> wl{};
    wl.n = (int)std::min<size_t>(kBatchMax, it.ops.size() - c0);
    int tot = 0;
    for (int i = 0; i < wl.n; ++i) {
      wl.prefix[i] = tot;
      wl.op[i] = it.ops[c0 + i];
      tot += (int)it.blocks[c0 + i];
    }
    wl.prefix[wl.n] = tot;
    if (tot == 0) continue;
    launch(h, k_worklist<Op, THREADS>, std::min((unsigned)tot, kResident), THREADS, smem, q, wl);
  }
}

// Loop control over every scene of the batch: the WHILE condition holds while any scene's solve
// is running (not done, under its iteration limit); the batched body's kernels are counted on the
// first scene's step state.
constexpr int kBatchScenes = 2 * kBatchMax;

struct LoopAll {
  int n;
  SolveState* st[kBatchScenes];
};

__global__ void k_loop_begin_all(LoopAll la, int chunk, cudaGraphConditionalHandle cond) {
  unsigned any = 0;
  for (int s = 0; s < la.n; ++s) {
    SolveState* st = la.st[s];
    st->it_stop = st->it + chunk;
    if (st->done == 0 && chunk > 0) any = 1;
  }
  cudaGraphSetConditional(cond, any);
}

__global__ void k_loop_cond_all(LoopAll la, cudaGraphConditionalHandle cond, StepCtl* ctl0,
                                unsigned long long body_nodes) {
  unsigned any = 0;
  for (int s = 0; s < la.n; ++s) {
    const SolveState* st = la.st[s];
    if (st->done == 0 && st->it < st->it_stop) any = 1;
  }
  cudaGraphSetConditional(cond, any);
  if (ctl0) ctl0->kernels += body_nodes;
}

// One scene of a batched solve: its kernels' arguments and the shape of its V-cycle.
template <int D, typename S>
struct BatchScene {
  SolveKernels<D, S> K;
  int L, l0, down_end;
  BatchScene(pfm_handle* h, const pfm_solve_opts& o) : K(h, o) {
    L = h->L;
    l0 = tail_level(h);
    down_end = l0 < L ? l0 : L - 1;
  }
};

// One red-black half-sweep for the scenes `level` picks: level(scene) is the level to smooth, or -1
// to leave the scene out.  The kernel of each scene is the one smooth_launch picks.
template <int D, typename S, class Level>
static void batched_smooth(std::vector<BatchScene<D, S>>& B, cudaStream_t q, int phase, Level level) {
  WorkItems<OpSmooth<D, S>> wide;
  WorkItems<OpSmooth8<S>> runs;
  for (auto& b : B) {
    const int lv = level(b);
    if (lv < 0) continue;
    pfm_handle* h = b.K.h;
    const Lvl L = lvl_of(h, lv);
    if (D == 3 && L.n2 % 8 == 0) {
      const int64_t nvec = (int64_t)L.n0 * L.n1 * (L.n2 / 8);
      runs.add(OpSmooth8<S>{level_z<S>(h, lv), level_r<S>(h, lv), L, b.K.bc, phase, b.K.st}, grid_for(nvec, 256));
    } else {
      const int nl = (D == 3) ? L.n2 : L.n1;
      const int64_t npairs = (D == 3) ? (int64_t)L.n0 * L.n1 * ((nl + 1) / 2) : (int64_t)L.n0 * ((nl + 1) / 2);
      wide.add(OpSmooth<D, S>{level_z<S>(h, lv), level_r<S>(h, lv), L, b.K.bc, phase, b.K.st}, grid_for(npairs, 256));
    }
  }
  pfm_handle* h0 = B[0].K.h;
  launch_worklist<OpSmooth<D, S>, 256>(h0, q, wide);
  launch_worklist<OpSmooth8<S>, 256>(h0, q, runs);
}

// apply_preconditioner for every scene of the batch: each scene's kernels in the order of vcycle()
// (the batched schedule interleaves the scenes level by level; a scene takes part in the steps its
// own hierarchy has, so its own sequence of updates is unchanged).
template <int D, typename S>
static void batched_vcycle(std::vector<BatchScene<D, S>>& B, cudaStream_t q) {
  pfm_handle* h0 = B[0].K.h;
  int dmax = 0, pmax = 0, bmax = 0;
  for (auto& b : B) {
    dmax = std::max(dmax, b.down_end);
    pmax = std::max(pmax, b.K.h->cfg.pre_post_smoothing);
    bmax = std::max(bmax, b.K.h->cfg.bottom_smoothing);
  }
  {
    WorkItems<OpZero<S>> z;
    for (auto& b : B)
      z.add(OpZero<S>{level_z<S>(b.K.h, 0), b.K.h->lv[0].count, b.K.st}, stream_blocks(b.K.h->lv[0].count));
    launch_worklist<OpZero<S>, 256>(h0, q, z);
  }
  for (int l = 0; l < dmax; ++l) {
    for (int i = 0; i < pmax; ++i) {
      auto pre = [&](const BatchScene<D, S>& b) { return (l < b.down_end && i < b.K.h->cfg.pre_post_smoothing) ? l : -1; };
      batched_smooth<D, S>(B, q, 0, pre);
      batched_smooth<D, S>(B, q, 1, pre);
    }
    WorkItems<OpZero<S>> z;
    WorkItems<OpRestrict<D, S>> r;
    for (auto& b : B) {
      if (l >= b.down_end) continue;
      pfm_handle* h = b.K.h;
      if (l + 1 != b.l0)
        z.add(OpZero<S>{level_z<S>(h, l + 1), h->lv[l + 1].count, b.K.st}, stream_blocks(h->lv[l + 1].count));
      const Lvl Lf = lvl_of(h, l), Lc = lvl_of(h, l + 1);
      r.add(OpRestrict<D, S>{level_z<S>(h, l), level_r<S>(h, l), Lf, level_r<S>(h, l + 1), Lc, b.K.bc, b.K.st},
            grid_for(Lc.count, 256));
    }
    launch_worklist<OpZero<S>, 256>(h0, q, z);
    launch_worklist<OpRestrict<D, S>, 256>(h0, q, r);
  }
  // the coarse levels: one block per scene that has a tail, the bottom sweeps for the others
  WorkItems<OpTail<D, S>> t;
  size_t tail_smem_max = 0;
  for (auto& b : B) {
    if (b.l0 >= b.L) continue;
    pfm_handle* h = b.K.h;
    OpTail<D, S> op{};
    op.zg = level_z<S>(h, b.l0);
    op.rg = level_r<S>(h, b.l0);
    op.l0 = b.l0;
    op.L = b.L;
    size_t cells = 0;
    for (int l = 0; l < b.L; ++l) {
      for (int a = 0; a < 3; ++a) op.n[l][a] = h->lv[l].n[a];
      if (l >= b.l0) cells += (size_t)h->lv[l].count;
    }
    op.bc = b.K.bc;
    op.pre_post = h->cfg.pre_post_smoothing;
    op.bottom = h->cfg.bottom_smoothing;
    op.st = b.K.st;
    t.add(op, 1);
    tail_smem_max = std::max(tail_smem_max, cells * 2 * sizeof(float));
  }
  if (!t.ops.empty()) {
    static std::atomic<unsigned long long> attr{0};  // above the default 48 KB: opt in per device
    if (tail_smem_max > 48 * 1024) opt_in_smem(k_worklist<OpTail<D, S>, kTailThreads>, 227 * 1024, attr);
    launch_worklist<OpTail<D, S>, kTailThreads>(h0, q, t, tail_smem_max);
  }
  for (int i = 0; i < bmax; ++i) {
    auto bottom = [&](const BatchScene<D, S>& b) {
      return (b.l0 >= b.L && i < b.K.h->cfg.bottom_smoothing) ? b.L - 1 : -1;
    };
    batched_smooth<D, S>(B, q, 0, bottom);
    batched_smooth<D, S>(B, q, 1, bottom);
  }
  for (int l = dmax - 1; l >= 0; --l) {
    WorkItems<OpProlong<D, S>> pr;
    for (auto& b : B) {
      if (l >= b.down_end) continue;
      pfm_handle* h = b.K.h;
      const Lvl Lf = lvl_of(h, l), Lc = lvl_of(h, l + 1);
      pr.add(OpProlong<D, S>{level_z<S>(h, l), Lf, level_z<S>(h, l + 1), Lc, b.K.st}, grid_for(Lf.count, 256));
    }
    launch_worklist<OpProlong<D, S>, 256>(h0, q, pr);
    for (int i = 0; i < pmax; ++i) {
      auto post = [&](const BatchScene<D, S>& b) { return (l < b.down_end && i < b.K.h->cfg.pre_post_smoothing) ? l : -1; };
      batched_smooth<D, S>(B, q, 1, post);
      batched_smooth<D, S>(B, q, 0, post);
    }
  }
}

// One WHILE iteration for every scene: SolveKernels::body's kernels, each one batched launch.
template <int D, typename S>
static void batched_body(std::vector<BatchScene<D, S>>& B, cudaStream_t q) {
  pfm_handle* h0 = B[0].K.h;
  {  // recenter with the level-storage copy
    WorkItems<OpDot<float>> mean;
    WorkItems<OpSubMean<S>> sub;
    WorkItems<OpToStorage<S>> sto;
    for (auto& b : B) {
      auto& K = b.K;
      if (K.neu) {
        mean.add(OpDot<float>{K.r0, nullptr, K.n, K.rb, (int)RED_MEAN, K.o.eps, K.inv_n, K.mi, K.f64}, red_blocks(K.n));
        sub.add(OpSubMean<S>{K.r0, K.mixed ? K.rh : nullptr, K.n, K.st}, stream_blocks(K.n));
      } else if (K.mixed) {
        sto.add(OpToStorage<S>{K.rh, K.r0, K.n, K.st}, stream_blocks(K.n));
      }
    }
    launch_worklist<OpDot<float>, kReduceThreads>(h0, q, mean);
    launch_worklist<OpSubMean<S>, 256>(h0, q, sub);
    launch_worklist<OpToStorage<S>, 256>(h0, q, sto);
  }
  batched_vcycle<D, S>(B, q);
  WorkItems<OpDot<S>> ztr;
  WorkItems<OpUpdateP<S>> up;
  WorkItems<OpApDot<D>> ap;
  WorkItems<OpUpdateXr> xr;
  WorkItems<OpTrueResidual<D>> tr;
  for (auto& b : B) {
    auto& K = b.K;
    ztr.add(OpDot<S>{K.z0, K.r0, K.n, K.rb, (int)RED_ZTR, K.o.eps, K.inv_n, K.mi, K.f64}, red_blocks(K.n));
    up.add(OpUpdateP<S>{K.p, K.z0, K.n, K.st}, stream_blocks(K.n));
    ap.add(OpApDot<D>{K.p, K.Ap, K.L0, K.bc, K.rb, K.o.eps, K.f64}, red_blocks(K.n));
    xr.add(OpUpdateXr{K.x, K.p, K.r0, K.Ap, K.n, K.rb, K.o.tol, K.o.tol_mode, K.f64, K.inv_n, K.x64}, red_blocks(K.n));
    if (K.true_res)
      tr.add(OpTrueResidual<D>{K.bvec, K.x, K.L0, K.bc, K.rb, K.o.true_residual_every, K.x64, K.r0, K.o.tol,
                               K.o.tol_mode, K.inv_n},
             red_blocks(K.n));
  }
  launch_worklist<OpDot<S>, kReduceThreads>(h0, q, ztr);
  launch_worklist<OpUpdateP<S>, 256>(h0, q, up);
  launch_worklist<OpApDot<D>, kReduceThreads>(h0, q, ap);
  launch_worklist<OpUpdateXr, kReduceThreads>(h0, q, xr);
  launch_worklist<OpTrueResidual<D>, kReduceThreads>(h0, q, tr);
}

template <int D, typename S>
static int append_batched_loop_t(GraphCursor& gc, pfm_handle* const* hs, int n, const pfm_solve_opts& o,
                                 StepCtl* const* ctls, int which) {
  pfm_handle* h0 = gc.h;
  std::vector<BatchScene<D, S>> B;
  B.reserve(n);
  for (int s = 0; s < n; ++s) B.emplace_back(hs[s], o);
  LoopAll la{};
  la.n = n;
  for (int s = 0; s < n; ++s) la.st[s] = B[s].K.st;
  cudaGraphConditionalHandle cond{};
  if (!gc.rc) gc.rc = check_cuda(h0, cudaGraphConditionalHandleCreate(&cond, gc.G, 0, 0), "conditional handle");
  if (gc.rc) return gc.rc;
  launch(h0, k_loop_begin_all, 1, 1, 0, gc.seg(), la, B[0].K.chunk, cond);
  cudaGraph_t body = gc.add_conditional(cond, cudaGraphCondTypeWhile);
  if (gc.rc) return gc.rc;
  // the body's kernels are counted by k_loop_cond_all on the device, once per iteration
  uint64_t nodes = 0;
  const uint64_t b0 = h0->launches;
  gc.capture_body(body, [&](cudaStream_t q) {
    batched_body<D, S>(B, q);
    nodes = h0->launches - b0 + 1;
    launch(h0, k_loop_cond_all, 1, 1, 0, q, la, cond, ctls[0], (unsigned long long)nodes);
  });
  return gc.rc;
}

// The iteration loops of n scenes' solves as one WHILE node whose body is batched launches; every
// scene's setup must already be in the graph behind the cursor, and its post part follows.  The
// scenes share dim, precision and options (pfm_batch checks).
int append_batched_loop(GraphCursor& gc, pfm_handle* const* hs, int n, const pfm_solve_opts& opts,
                        StepCtl* const* ctls, int which) {
  if (n < 1 || n > kBatchScenes) return set_error(gc.h, PFM_ERR_ARG, "batched solve: 1 to 128 scenes");
  int rc = PFM_OK;
  dispatch_solve(gc.h->cfg.dim, opts.precision, [&](auto dd, auto ss) {
    rc = append_batched_loop_t<decltype(dd)::value, decltype(ss)>(gc, hs, n, opts, ctls, which);
  });
  return rc ? rc : gc.rc;
}

// A scene's part after a batched loop: the solve's finish (the final true residual) and its
// statistics in the step state (the loop's kernels are counted by the loop itself).
int append_poisson_finish(GraphCursor& gc, const pfm_solve_opts& opts, float* p_io, StepCtl* ctl, int which) {
  pfm_solve_opts o = opts;
  if (!p_io) o.warm_start = 0;
  dispatch_solve(gc.h->cfg.dim, o.precision, [&](auto dd, auto ss) {
    SolveKernels<decltype(dd)::value, decltype(ss)> K(gc.h, o);
    cudaStream_t q = gc.seg();
    K.finish(q);
    launch(gc.h, k_record_solve, 1, 1, 0, q, ctl, (const SolveState*)K.st, which, 0);
  });
  return gc.rc;
}

}  // namespace pfm

using namespace pfm;

extern "C" {

int pfm3_poisson(pfm_handle* h, float* u_x, float* u_y, float* u_z, float* p_out, const pfm_solve_opts* opts,
                 pfm_solve_stats* stats, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_poisson on a 2D handle");
  if (!u_x || !u_y || !u_z) return set_error(h, PFM_ERR_NULL, "pfm3_poisson: null velocity");
  float* u[3] = {u_x, u_y, u_z};
  return poisson_impl<3>(h, u, p_out, opts, stats, (cudaStream_t)stream);
}

int pfm2_poisson(pfm_handle* h, float* u_x, float* u_y, float* p_out, const pfm_solve_opts* opts,
                 pfm_solve_stats* stats, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 2) return set_error(h, PFM_ERR_SHAPE, "pfm2_poisson on a 3D handle");
  if (!u_x || !u_y) return set_error(h, PFM_ERR_NULL, "pfm2_poisson: null velocity");
  float* u[2] = {u_x, u_y};
  return poisson_impl<2>(h, u, p_out, opts, stats, (cudaStream_t)stream);
}

int pfm_mgpcg_solve(pfm_handle* h, const float* r, float k, float* x_out, const pfm_solve_opts* opts,
                    pfm_solve_stats* stats, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (!r || !x_out) return set_error(h, PFM_ERR_NULL, "pfm_mgpcg_solve: null input");
  int rc = require_ws(h);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  float* r0 = ws_ptr<float>(h, h->o_r[0]);
  // init(r, k): r0 = k r (3D/mgpcg.py:71-79)
  launch(h, k_scale, stream_blocks(h->cells), 256, 0, s, r0, r, h->cells, k);
  rc = launch_check(h, "k_scale");
  if (rc) return rc;
  return mgpcg_solve_in_place(h, x_out, opts, stats, s);
}

int pfm_apply_bc(pfm_handle* h, float* u_x, float* u_y, float* u_z, void* stream) {
  if (!h) return PFM_ERR_NULL;
  const int D = h->cfg.dim;
  if (!u_x || !u_y || (D == 3 && !u_z)) return set_error(h, PFM_ERR_NULL, "pfm_apply_bc: null velocity");
  float* u[3] = {u_x, u_y, u_z};
  const MacGeom& g = h->geom;
  cudaStream_t s = (cudaStream_t)stream;
  for (int f = 0; f < D; ++f) {
    const int a1 = (f == 0) ? 1 : 0, a2 = (f == 2) ? 1 : 2;
    const int64_t plane = (int64_t)g.n[f][a1] * (D == 3 ? g.n[f][a2] : 1);
    const int lo = h->cfg.boundary[f][0] == 2, hi = h->cfg.boundary[f][1] == 2;
    if (D == 3) launch(h, k_apply_bc<3>, grid_for(2 * plane, 256), 256, 0, s, u[f], f, g, lo, hi);
    else launch(h, k_apply_bc<2>, grid_for(2 * plane, 256), 256, 0, s, u[f], f, g, lo, hi);
  }
  return launch_check(h, "pfm_apply_bc");
}

int pfm_divergence(pfm_handle* h, const float* u_x, const float* u_y, const float* u_z, float* div_out,
                   void* stream) {
  if (!h) return PFM_ERR_NULL;
  const int D = h->cfg.dim;
  if (!u_x || !u_y || (D == 3 && !u_z) || !div_out) return set_error(h, PFM_ERR_NULL, "pfm_divergence: null input");
  cudaStream_t s = (cudaStream_t)stream;
  if (D == 3)
    launch_divergence<3>(h, u_x, u_y, u_z, div_out, 1.f, s);
  else
    launch_divergence<2>(h, u_x, u_y, nullptr, div_out, 1.f, s);
  return launch_check(h, "pfm_divergence");
}

int pfm_subtract_grad_p(pfm_handle* h, float* u_x, float* u_y, float* u_z, const float* p, void* stream) {
  if (!h) return PFM_ERR_NULL;
  const int D = h->cfg.dim;
  if (!u_x || !u_y || (D == 3 && !u_z) || !p) return set_error(h, PFM_ERR_NULL, "pfm_subtract_grad_p: null input");
  cudaStream_t s = (cudaStream_t)stream;
  float* u[3] = {u_x, u_y, u_z};
  for (int f = 0; f < D; ++f) {
    // lo/hi = 0: the gradient subtraction alone; the boundary faces are left to pfm_apply_bc
    if (D == 3) launch_subtract_grad_p<3>(h, f, u[f], p, 0, 0, s);
    else launch_subtract_grad_p<2>(h, f, u[f], p, 0, 0, s);
  }
  return launch_check(h, "pfm_subtract_grad_p");
}

}  // extern "C"
