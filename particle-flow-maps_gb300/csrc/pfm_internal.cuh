// Internal definitions shared by the libpfm.so translation units: the handle, the workspace
// layout, grid geometry and the quadratic-B-spline interpolation device code.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <type_traits>

#include "../../include/pfm.h"

namespace pfm {

constexpr int kMaxLevels = 16;
constexpr int kReduceBlocks = 1024;  // fixed partition of every deterministic reduction
constexpr int kReduceThreads = 256;
// The reduction kernels are compiled for 8 resident blocks per SM (at most 32 registers), so the
// 1024 blocks of the partition run in one wave on GB300's 152 SMs instead of 912 + 112.
constexpr int kReduceResident = 8;
constexpr int kScanItems = 8;        // items per thread in the cell-count scan
constexpr int kScanThreads = 1024;

// Device-resident state of one MGPCG solve (3D/mgpcg.py:202-280).  Scalars that the reference
// keeps as Python floats (zTr, pAp, rTr) are doubles; alpha/beta are stored to f32 fields in the
// reference (self.alpha[None] = ...), so they are f32 here too.
struct SolveState {
  double zTr_old;
  double pAp;
  double rTr;
  double rTr0;
  double bTb;      // b.b of the recentred right-hand side (mixed / warm-started solves)
  double rTr_true; // |b - A x|^2 at the last true-residual check
  double sum;      // scratch result of the last reduction
  float alpha;
  float beta;
  float mean;      // recenter mean
  float hscale;    // 16-bit level storage holds r * hscale (unit RMS), z is read back / hscale
  int it;          // completed iterations
  int done;        // 1 converged, 2 iteration limit, 3 non-finite, 4 a tile copy did not arrive
  int conv_it;     // iteration index at convergence
  unsigned ticket; // last-block counter of the reductions
  int it_stop;     // the device loop pauses when `it` reaches this count
};

// Unsigned division by a divisor that is fixed for a launch, with one multiply-high (Granlund and
// Montgomery, "Division by invariant integers using multiplication", PLDI 1994): with
// s = ceil(log2 d) and m = floor(2^32 (2^s - d) / d) + 1, n / d = (umulhi(n, m) + n) >> s for
// every 0 <= n < 2^31.  Grid and level indices stay below 2^31 (pfm_create rejects larger grids).
struct Div32 {
  unsigned d, m, s;
};

__host__ __device__ inline Div32 make_div32(unsigned d) {
  unsigned s = 0;
  while ((1ull << s) < d) ++s;
  const unsigned long long m = ((1ull << 32) * ((1ull << s) - d)) / d + 1;
  return Div32{d, (unsigned)m, s};
}

__device__ __forceinline__ unsigned udiv(unsigned n, const Div32& D) { return (__umulhi(n, D.m) + n) >> D.s; }

// e = (i * n1 + j) * n2 + k  ->  (i, j, k), with d1 / d2 the divisors n1 / n2
__device__ __forceinline__ void split3(unsigned e, const Div32& d1, const Div32& d2, int& i, int& j, int& k) {
  const unsigned t = udiv(e, d2);
  k = (int)(e - t * d2.d);
  const unsigned u = udiv(t, d1);
  j = (int)(t - u * d1.d);
  i = (int)u;
}

// Device state of the whole-step graph (pfm3_step / pfm2_step): the frame clock of
// 3D/run_3D.py:725-743 (2D/run_2D.py:782-799) in double precision, this step's dt, the reinit
// flags, and the statistics of the step's two MGPCG solves.
struct StepCtl {
  double sub_t;        // time since the last frame
  double curr_dt;      // this step's dt (CFL dx / max_speed, clamped to the frame)
  double rTr[2];       // final r.r of the midpoint [0] and final [1] solves
  unsigned long long kernels;  // kernels the step graphs ran since the host last read this
  float max_speed;     // calc_max_speed of this step
  float dt;            // f32(curr_dt)
  float dt_half;       // f32(0.5 curr_dt)
  int i, ik, frame_idx, output_frame;
  int reinit, repos, gradm;
  int iters[2];        // MGPCG iterations of the two solves
  int done[2];         // their end codes (1 converged, 2 iteration limit, 3 non-finite)
  int history[64][2];  // iterations of step s's two solves at s % 64
};

struct LevelDims {
  int n[3];
  int64_t count;
};

// Face-grid geometry (3D/run_3D.py:73-75) and the f32 clamp constants of interp_grad_2
// (3D/taichi_utils.py:282-284): hi[c][a] = f32(dim_a(field c) - 2 - 1e-6), formed in double.
struct MacGeom {
  int dim;
  int N[3];        // res
  int n[3][3];     // n[c][a]: extent of face field c along axis a
  float hi[3][3];  // interpolation clamp constants
  float dx;        // f32(dx)
  float inv_dx;    // f32(1/dx)
  Div32 dN[3];     // divisors N[a]
  Div32 dn[3][3];  // divisors n[c][a]
};

}  // namespace pfm

struct pfm_handle {
  pfm_config cfg;
  pfm::MacGeom geom;
  int64_t P;
  int64_t cells;
  int L;
  pfm::LevelDims lv[pfm::kMaxLevels];
  // workspace
  char* ws;
  size_t ws_bytes;
  size_t ws_need;
  // workspace offsets
  size_t o_key, o_slot, o_order, o_count, o_start, o_blocksums, o_payload;
  size_t o_r[pfm::kMaxLevels], o_z[pfm::kMaxLevels];
  size_t o_x, o_p, o_Ap, o_b, o_partials, o_state, o_maxpart, o_step;
  // warm_start 2: the previous solution of up to two pressure buffers (the caller's pointers name
  // the slots) and a device flag per slot saying whether it holds one
  size_t o_hist, o_hist_flag;
  size_t o_x64;
  const float* hist_ptr[2];

  // pinned host mirror of the solve state
  pfm::SolveState* h_state;
  // kernels launched through this handle (reported by pfm_launch_count)
  uint64_t launches;
  int rec_valid;  // 3D P2G records and cell keys of the last RK4/payload pass are in the workspace
  // CUDA graphs of the MGPCG setup and of one PCG iteration (captured on first use)
  cudaStream_t cap_stream;
  cudaGraphExec_t g_setup, g_loop;  // setup + first half-iteration; device-side PCG loop
  int g_setup_nodes, g_body_nodes;
  double g_eps, g_tol;
  int g_mode, g_valid, g_max_iters, g_chunk, g_variant, g_true_every;
  // tunables (pfm_set_tuning): faces per thread of the 2D P2G column gather; MGPCG levels with at
  // most tail_cells cells run in one thread block
  int p2g2_column;
  int tail_cells;
  int smooth_tma;  // 3D 16-bit MGPCG levels smoothed from TMA-staged tiles (same results)
  int cube_kernels;  // 3D interpolating kernels instantiated for the grid's cube extent (same results)
  int mid_centre;    // 3D midpoint's first stage at the face centre in constant-weight form (same results)
  // whole-step graph (pfm3_step / pfm2_step), rebuilt when its fields or parameters change
  cudaGraphExec_t g_step;
  std::string step_key;
  int step_clock_init;  // the step state has been initialised (pfm_step_reset or the first step)
  std::string err;
};

namespace pfm {

int set_error(pfm_handle* h, int status, const std::string& msg);
int check_cuda(pfm_handle* h, cudaError_t e, const char* what);
int require_ws(pfm_handle* h);

template <class T>
inline T* ws_ptr(pfm_handle* h, size_t off) {
  return reinterpret_cast<T*>(h->ws + off);
}

// Launches `kernel` and counts it on the handle.
template <typename... KArgs, typename... Args>
inline void launch(pfm_handle* h, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                   Args... args) {
  kernel<<<grid, block, smem, st>>>(args...);
  h->launches++;
}

// Appends work to a CUDA graph G behind a set of dependency nodes: seg() opens a stream-capture
// segment (cudaStreamBeginCaptureToGraph) on the handle's capture stream, add_conditional()
// closes it and adds an IF/WHILE node, capture_body() fills a conditional node's body graph.
// The first error is kept in rc; later calls do nothing.
struct GraphCursor {
  pfm_handle* h;
  cudaGraph_t G;
  cudaStream_t cs;
  cudaGraphNode_t deps[256];  // a batch joins one node per scene
  size_t ndeps = 0;
  bool open = false;
  int rc = 0;
  cudaGraph_t junk = nullptr;  // after an error, segments are captured here and discarded
  uint64_t body_launches = 0;  // kernels launched into conditional bodies
  GraphCursor(pfm_handle* hh, cudaGraph_t g, cudaStream_t s) : h(hh), G(g), cs(s) {}
  cudaStream_t seg();
  void close();
  cudaGraph_t add_conditional(cudaGraphConditionalHandle cond, cudaGraphConditionalNodeType type);
  template <class F>
  void capture_body(cudaGraph_t body, F&& f) {
    if (rc) return;
    close();
    rc = begin_body(body);
    if (rc) return;
    const uint64_t b0 = h->launches;
    f(cs);
    body_launches += h->launches - b0;
    rc = end_body();
  }
  int begin_body(cudaGraph_t body);
  int end_body();
};

// cudaFuncSetAttribute acts on the current device's context only, so a kernel that needs more than
// the default 48 KB of dynamic shared memory is opted in once per device: `done` holds a bit per
// device ordinal (ordinals of 64 and above are opted in on every call).
template <class K>
inline cudaError_t opt_in_smem(K* kernel, int bytes, std::atomic<unsigned long long>& done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

inline unsigned grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return (unsigned)(b < 1 ? 1 : b);
}

// ------------------------------------------------------------------------------------------
// Quadratic B-spline (3D/taichi_utils.py:252-272).  Branch structure as in the reference.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float N2(float x) {
  float ax = fabsf(x);
  float r = 0.f;
  if (ax < 0.5f)
    r = 0.75f - ax * ax;
  else if (ax < 1.5f)
    r = 0.5f * ((1.5f - ax) * (1.5f - ax));
  return r;
}

__device__ __forceinline__ float dN2(float x) {
  float ax = fabsf(x);
  float r = 0.f;
  if (ax < 0.5f)
    r = -2.f * ax;
  else if (ax < 1.5f)
    r = 0.5f * (2.f * ax - 3.f);
  if (x < 0.f) r = -r;
  return r;
}

// One axis of the interp_grad_2 stencil (3D/taichi_utils.py:278-305).  The reference visits
// the four taps iu-1..iu+2 of the clamped sample position s; exactly one of the outer two has
// |x| >= 1.5, where N_2 and dN_2 are exactly zero, so only the three taps around the middle tap
// m (|s - m| <= 0.5) are kept.  With t = s - m in [-0.5, 0.5) the three taps sit at x = t+1, t,
// t-1, where the branches of N_2 / dN_2 reduce to
//   N_2:  0.5 (0.5 - t)^2,  0.75 - t^2,  0.5 (0.5 + t)^2
//   dN_2: t - 0.5,          -2 t,        t + 0.5
// (the |x| = 0.5 and 1.5 boundary cases included).  For s >= 1 every subtraction involved is
// exact, so the weights are bitwise those of the reference's per-tap evaluation.
// sample() clamps every tap index to [0, n-1] (3D/taichi_utils.py:48-54), but the position is
// first clamped to [1, n - 2 - eps], so floor(s) lies in [1, n-3] and the three taps
// first .. first+2 always lie in [0, n-1] (n >= 4 is enforced when the handle is created; a NaN
// or infinite position clamps to an end of the range too).  The clamp never changes an index, so
// only the first tap is stored and the taps of a row are three consecutive floats.
struct Axis3 {
  int first;
  float w[3];
  float dw[3];
};

__device__ __forceinline__ void axis_taps(float u, float hi, Axis3& a) {
  const float s = fmaxf(1.f, fminf(u, hi));
  const float iu = floorf(s);
  const float frac = s - iu;
  const bool lo = frac < 0.5f;
  const float t = lo ? frac : frac - 1.f;
  const float l = 0.5f - t, r = 0.5f + t;
  a.w[0] = 0.5f * (l * l);
  a.w[1] = 0.75f - t * t;
  a.w[2] = 0.5f * (r * r);
  a.dw[0] = t - 0.5f;
  a.dw[1] = -2.f * t;
  a.dw[2] = t + 0.5f;
  a.first = __float2int_rz(iu) + (lo ? -1 : 0);
}

// interp_u_MAC_grad (3D/taichi_utils.py:312-317): u at p and G[c][r] = d u_c / d x_r.
// The two distinct tap sets per axis are shared: component c uses the BL = 0 set on axis c
// and the BL = 0.5 set on the others.
struct MacFields3 {
  const float* u[3];
};

// The 27-tap sums are evaluated axis by axis (z taps, then y, then x): per component
//   tn_ab = sum_k wz_k f_abk,  td_ab = sum_k dwz_k f_abk,
//   A_a = sum_b wy_b tn_ab,  B_a = sum_b dwy_b tn_ab,  C_a = sum_b wy_b td_ab,
//   u = sum_a wx_a A_a,  du/dx = sum_a dwx_a A_a / dx,  du/dy = sum_a wx_a B_a / dx,
//   du/dz = sum_a wx_a C_a / dx,
// the same terms as the reference's triple loop in a different association (rounding-level
// differences only).  Components x and y share the z tap set (BL = 0.5 along z) and their
// x/y weights form natural pairs, so they run together on packed f32x2 FMAs; z runs scalar.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// The two tap sets per axis at p (A0: the component along the axis, A1: the others).
__device__ __forceinline__ void mac_taps3(const MacGeom& g, const float p[3], Axis3 A0[3], Axis3 A1[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float u = p[a] * g.inv_dx;  // = p / dx exactly when dx is a power of two
    axis_taps(u - 0.0f, g.hi[a][a], A0[a]);            // the component along a
    axis_taps(u - 0.5f, g.hi[(a + 1) % 3][a], A1[a]);  // the others
  }
}

// The tap sums of interp_mac3 for taps already computed (two fields of the same shape sampled at
// one position share them).  NC > 0: the grid is NC^3 cells, so the face fields' strides are
// compile-time constants and every row of a field is its base pointer plus a load immediate (the
// same loads and sums as NC = 0, which reads the strides from g).
template <int NC = 0>
__device__ __forceinline__ void interp_mac3_taps(const MacFields3& F, const MacGeom& g, const Axis3 A0[3],
                                                 const Axis3 A1[3], float uo[3], float G[3][3], bool want_grad);

template <int NC = 0>
__device__ __forceinline__ void interp_mac3(const MacFields3& F, const MacGeom& g, const float p[3],
                                            float uo[3], float G[3][3], bool want_grad) {
  Axis3 A0[3], A1[3];
  mac_taps3(g, p, A0, A1);
  interp_mac3_taps<NC>(F, g, A0, A1, uo, G, want_grad);
}

template <int NC>
__device__ __forceinline__ void interp_mac3_taps(const MacFields3& F, const MacGeom& g, const Axis3 A0[3],
                                                 const Axis3 A1[3], float uo[3], float G[3][3], bool want_grad) {
  const float inv_dx = g.inv_dx;
  // ---- components x and y together: x uses (A0x, A1y, A1z), y uses (A1x, A0y, A1z)
  {
    const float* __restrict__ f0 = F.u[0];
    const float* __restrict__ f1 = F.u[1];
    const int m01 = NC ? NC : g.n[0][1], m02 = NC ? NC : g.n[0][2];
    const int m11 = NC ? NC + 1 : g.n[1][1], m12 = NC ? NC : g.n[1][2];
    const Axis3& Z = A1[2];
    const float* __restrict__ b0 = f0 + ((A0[0].first * m01 + A1[1].first) * m02 + Z.first);
    const float* __restrict__ b1 = f1 + ((A1[0].first * m11 + A0[1].first) * m12 + Z.first);
    const int sx0 = m01 * m02, sx1 = m11 * m12;
    const float2 zw0 = f2(Z.w[0], Z.w[0]), zw1 = f2(Z.w[1], Z.w[1]), zw2 = f2(Z.w[2], Z.w[2]);
    float2 V = f2(0.f, 0.f), GX = V, GY = V, GZ = V;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float2 Aa = f2(0.f, 0.f), Ba = Aa, Ca = Aa;
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const float* __restrict__ r0 = b0 + (a * sx0 + b * m02);
        const float* __restrict__ r1 = b1 + (a * sx1 + b * m12);
        const float2 v0 = f2(__ldg(r0), __ldg(r1));
        const float2 v1 = f2(__ldg(r0 + 1), __ldg(r1 + 1));
        const float2 v2 = f2(__ldg(r0 + 2), __ldg(r1 + 2));
        float2 tn = __fmul2_rn(v0, zw0);
        tn = __ffma2_rn(v1, zw1, tn);
        tn = __ffma2_rn(v2, zw2, tn);
        const float2 wy = f2(A1[1].w[b], A0[1].w[b]);
        Aa = __ffma2_rn(wy, tn, Aa);
        if (want_grad) {
          const float2 zd0 = f2(Z.dw[0], Z.dw[0]), zd1 = f2(Z.dw[1], Z.dw[1]), zd2 = f2(Z.dw[2], Z.dw[2]);
          float2 td = __fmul2_rn(v0, zd0);
          td = __ffma2_rn(v1, zd1, td);
          td = __ffma2_rn(v2, zd2, td);
          Ba = __ffma2_rn(f2(A1[1].dw[b], A0[1].dw[b]), tn, Ba);
          Ca = __ffma2_rn(wy, td, Ca);
        }
      }
      const float2 wx = f2(A0[0].w[a], A1[0].w[a]);
      V = __ffma2_rn(wx, Aa, V);
      if (want_grad) {
        GX = __ffma2_rn(f2(A0[0].dw[a], A1[0].dw[a]), Aa, GX);
        GY = __ffma2_rn(wx, Ba, GY);
        GZ = __ffma2_rn(wx, Ca, GZ);
      }
    }
    uo[0] = V.x;
    uo[1] = V.y;
    if (want_grad) {
      G[0][0] = GX.x * inv_dx;
      G[1][0] = GX.y * inv_dx;
      G[0][1] = GY.x * inv_dx;
      G[1][1] = GY.y * inv_dx;
      G[0][2] = GZ.x * inv_dx;
      G[1][2] = GZ.y * inv_dx;
    }
  }
  // ---- component z: (A1x, A1y, A0z)
  {
    const float* __restrict__ f = F.u[2];
    const int m1 = NC ? NC : g.n[2][1], m2 = NC ? NC + 1 : g.n[2][2];
    const Axis3 &X = A1[0], &Y = A1[1], &Z = A0[2];
    const float* __restrict__ base = f + ((X.first * m1 + Y.first) * m2 + Z.first);
    const int sx = m1 * m2;
    float v_ = 0.f, x_ = 0.f, y_ = 0.f, z_ = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float Aa = 0.f, Ba = 0.f, Ca = 0.f;
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const float* __restrict__ row = base + (a * sx + b * m2);
        const float v0 = __ldg(row), v1 = __ldg(row + 1), v2 = __ldg(row + 2);
        const float tn = fmaf(v2, Z.w[2], fmaf(v1, Z.w[1], v0 * Z.w[0]));
        Aa = fmaf(Y.w[b], tn, Aa);
        if (want_grad) {
          const float td = fmaf(v2, Z.dw[2], fmaf(v1, Z.dw[1], v0 * Z.dw[0]));
          Ba = fmaf(Y.dw[b], tn, Ba);
          Ca = fmaf(Y.w[b], td, Ca);
        }
      }
      v_ = fmaf(X.w[a], Aa, v_);
      if (want_grad) {
        x_ = fmaf(X.dw[a], Aa, x_);
        y_ = fmaf(X.w[a], Ba, y_);
        z_ = fmaf(X.w[a], Ca, z_);
      }
    }
    uo[2] = v_;
    if (want_grad) {
      G[2][0] = x_ * inv_dx;
      G[2][1] = y_ * inv_dx;
      G[2][2] = z_ * inv_dx;
    }
  }
}

// The cube extents the 3D interpolating kernels are instantiated for (interp_mac3_taps<NC>).
// with_cube(h, f) calls f(std::integral_constant<int, NC>()) with NC the grid's extent when the grid
// is a cube of one of them (and the handle's PFM_TUNE_CUBE_KERNELS is on), else with NC = 0
// (strides from the geometry).
inline int cube_extent(const MacGeom& g) {
  const int n = g.N[0];
  if (g.dim != 3 || g.N[1] != n || g.N[2] != n) return 0;
  return (n == 64 || n == 128 || n == 256 || n == 512) ? n : 0;
}

template <class Fn>
inline void with_cube(const pfm_handle* h, Fn&& f) {
  switch (h->cube_kernels ? cube_extent(h->geom) : 0) {
    case 64: f(std::integral_constant<int, 64>()); break;
    case 128: f(std::integral_constant<int, 128>()); break;
    case 256: f(std::integral_constant<int, 256>()); break;
    case 512: f(std::integral_constant<int, 512>()); break;
    default: f(std::integral_constant<int, 0>()); break;
  }
}

// Loads and stores of particle state that a thread touches once (the RK4's inputs and outputs):
// the evict-first (streaming) cache operators, so that they do not displace the grid rows the
// interpolations reuse (RK4 at 256^3: 14.83 against 15.12 ms with the default operators).
__device__ __forceinline__ float ld_stream(const float* p) { return __ldcs(p); }
template <class T>
__device__ __forceinline__ void st_stream(T* p, T v) { __stcs(p, v); }

// P2G particle record and cell key (3D), shared by the payload pass and the fused RK4 + P2G:
//   pos4[q]      = (pos/dx, 0)
//   famrec[f][q] = (m_f, dx (T C T)_f row), m = T_gm^T-composed init_imp, T C T = T_gm^T init_C T_gm
//                  (the row pre-scaled by dx: the tiles take face offsets in grid units)
//                  (3D/run_3D.py:462-479)
//   key[q]       = linear cell of int(pos/dx) clamped to the grid (3D/run_3D.py:348),
//   slot[q]      = arrival index in its bin (atomic on the bin count; fixed later by the sort).
// A[r][c] = T_gm_r[c] (rows of T_gm); v = pos / dx.
struct P2GRecords3 {
  const float* imp0;  // init_imp [3][P]
  const float* Ti;    // T_init [3][3][P]
  const float* C;     // init_C [3][3][P]
  float4* pos4;       // [P]
  float4* famrec;     // [3][P]
  int* key;
  int* slot;
  int* count;
};

__device__ __forceinline__ void write_p2g_record3(const P2GRecords3& R, int64_t q, int64_t P, const MacGeom& g,
                                                  const float v[3], const float A[3][3]) {
  int c[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int ci = __float2int_rz(v[a]);
    c[a] = ci < 0 ? 0 : (ci > g.N[a] - 1 ? g.N[a] - 1 : ci);
  }
  const int k = (c[0] * g.N[1] + c[1]) * g.N[2] + c[2];
  st_stream(R.key + q, k);
  R.slot[q] = atomicAdd(&R.count[k], 1);
  float Cm[3][3], N[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
      Cm[r][cc] = R.C[(r * 3 + cc) * P + q];   // rows(init_C)
      N[cc][r] = R.Ti[(r * 3 + cc) * P + q];   // cols(T_init): N[k][c'] = T_init_c'[k]
    }
  // TCT = A^T (C A); T_transpose = A^T N; m = T_transpose init_imp
  float CA[3][3], TCT[3][3], TT[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) CA[r][cc] = Cm[r][0] * A[0][cc] + Cm[r][1] * A[1][cc] + Cm[r][2] * A[2][cc];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
      TCT[r][cc] = A[0][r] * CA[0][cc] + A[1][r] * CA[1][cc] + A[2][r] * CA[2][cc];
      TT[r][cc] = A[0][r] * N[0][cc] + A[1][r] * N[1][cc] + A[2][r] * N[2][cc];
    }
  const float m0[3] = {ld_stream(R.imp0 + q), ld_stream(R.imp0 + P + q), ld_stream(R.imp0 + 2 * P + q)};
  float m[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) m[r] = TT[r][0] * m0[0] + TT[r][1] * m0[1] + TT[r][2] * m0[2];
  st_stream(R.pos4 + q, make_float4(v[0], v[1], v[2], 0.f));
#pragma unroll
  for (int f = 0; f < 3; ++f)
    st_stream(R.famrec + f * P + q, make_float4(m[f], TCT[f][0] * g.dx, TCT[f][1] * g.dx, TCT[f][2] * g.dx));
}

// Launches RK4_T_forward (3D); with R non-null the kernel also writes the P2G records and keys
// of the advected particles, and with Fg non-null it first does the flow-map gradient
// reinitialisation (init_C = grad u(p) in Fg, update_T, T_gm = I) (defined in pfm_particles.cu).
int launch_rk4_T_forward3(pfm_handle* h, float* pos, float* T, const MacFields3& F, float dt, const P2GRecords3* R,
                          const MacFields3* Fg, cudaStream_t st, const float* dt_dev = nullptr);

// ------------------------------------------------------------------------------------------
// 2D (2D/taichi_utils.py:214-261)
// ------------------------------------------------------------------------------------------
struct MacFields2 {
  const float* u[2];
};

__device__ __forceinline__ void interp2_component(const float* __restrict__ f, int n1, const Axis3& X,
                                                  const Axis3& Y, float inv_dx, float& val, float& gx,
                                                  float& gy) {
  float v_ = 0.f, x_ = 0.f, y_ = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float* __restrict__ row = f + ((X.first + a) * n1 + Y.first);
    float v0 = __ldg(row), v1 = __ldg(row + 1), v2 = __ldg(row + 2);
    float tn = v0 * Y.w[0] + v1 * Y.w[1] + v2 * Y.w[2];
    float td = v0 * Y.dw[0] + v1 * Y.dw[1] + v2 * Y.dw[2];
    v_ += X.w[a] * tn;
    x_ += X.dw[a] * tn;
    y_ += X.w[a] * td;
  }
  val = v_;
  gx = x_ * inv_dx;
  gy = y_ * inv_dx;
}

__device__ __forceinline__ void interp_mac2(const MacFields2& F, const MacGeom& g, const float p[2],
                                            float uo[2], float G[2][2]) {
  Axis3 A0[2], A1[2];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    float u = p[a] * g.inv_dx;  // = p / dx exactly when dx is a power of two
    axis_taps(u - 0.0f, g.hi[a][a], A0[a]);
    axis_taps(u - 0.5f, g.hi[1 - a][a], A1[a]);
  }
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const Axis3& X = (c == 0) ? A0[0] : A1[0];
    const Axis3& Y = (c == 1) ? A0[1] : A1[1];
    interp2_component(F.u[c], g.n[c][1], X, Y, g.inv_dx, uo[c], G[c][0], G[c][1]);
  }
}

// ------------------------------------------------------------------------------------------
// host-side launch helpers (defined in the .cu files)
// ------------------------------------------------------------------------------------------
int launch_check(pfm_handle* h, const char* what);

// MGPCG entry used by the Poisson wrappers (pfm_mgpcg.cu): solves A x = -div where div is in
// r_0 of the workspace (already written).  x may be a caller buffer.
int mgpcg_solve_in_place(pfm_handle* h, float* x, const pfm_solve_opts* opts, pfm_solve_stats* stats,
                         cudaStream_t st);

// The whole-step graph's pieces (pfm_step.cu): Poisson with a device-side solve (pfm_mgpcg.cu), the
// midpoint kernels and calc_max_speed (pfm_grid.cu), the 3D P2G tiles from records (pfm_p2g.cu),
// the 2D RK4 (pfm_particles.cu).
int append_poisson(GraphCursor& gc, float* const* u, float* p_io, const pfm_solve_opts& opts, StepCtl* ctl,
                   int which);
// append_poisson in its three parts (pre: apply_bc, divergence, warm start, the solve's setup;
// loop: the WHILE node and the statistics; post: the pressure copy and subtract_grad_p), and the
// loops of many scenes' solves as one WHILE node of batched work-list kernels.
int append_poisson_pre(GraphCursor& gc, float* const* u, float* p_io, const pfm_solve_opts& opts);
int append_poisson_loop(GraphCursor& gc, const pfm_solve_opts& opts, float* p_io, StepCtl* ctl, int which);
int append_poisson_post(GraphCursor& gc, float* const* u, float* p_io);
int append_batched_loop(GraphCursor& gc, pfm_handle* const* hs, int n, const pfm_solve_opts& opts,
                        StepCtl* const* ctls, int which);
int append_poisson_finish(GraphCursor& gc, const pfm_solve_opts& opts, float* p_io, StepCtl* ctl, int which);
int launch_midpoint(pfm_handle* h, const float* const* u0, float* const* u1, float dt_half, const float* dt_half_dev,
                    cudaStream_t st);
int max_speed_async(pfm_handle* h, const float* ux, const float* uy, const float* uz, float* out, cudaStream_t st);
int p2g3_from_records(pfm_handle* h, float* const* us, float* const* ws, cudaStream_t st);
P2GRecords3 records3(pfm_handle* h, const float* init_imp, const float* T_init, const float* init_C);
int launch_rk4_T_forward2(pfm_handle* h, float* pos, float* T, const MacFields2& F, float dt, int advect_psi,
                          cudaStream_t st, const float* dt_dev);

// Sets the MGPCG tail threshold and the shared-memory limit of the one-block V-cycle tail
// (pfm_mgpcg.cu).
int set_tail_cells(pfm_handle* h, int cells);

// Initial guess of a warm-started solve into x (pfm_mgpcg.cu): mode 1 copies the caller's pressure
// p_io, mode 2 extrapolates 2 p_io - (the solution before it) once that history exists.
int warm_start_init(pfm_handle* h, float* x, const float* p_io, int mode, cudaStream_t st);

// Counting sort of the particle cells (pfm_p2g.cu).
int sort_particles(pfm_handle* h, const float* pos, cudaStream_t st);

}  // namespace pfm
