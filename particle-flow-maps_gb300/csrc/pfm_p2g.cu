// Deterministic APIC particle-to-grid transfer (3D/run_3D.py:441-552, 2D/run_2D.py:548-611).
//
// The reference scatters 3 x 64 taps per particle with float atomic adds, so its sums depend on
// thread scheduling.  Here:
//  1. every particle gets the key int(pos/dx) (its cell, clamped to the grid) and a counting
//     sort with one digit of radix = number of cells bins the particles; each bin is then put in
//     particle-index order, so the permutation equals a stable CPU sort of the same keys;
//  2. a payload pass evaluates each particle's impulse m = T_gm^T-composed init_imp and affine
//     matrix T_gm^T C T_gm once, in sorted order (AoS float4 records);
//  3. one thread per face gathers, in (cell, particle-index) order, every particle of the cells
//     that can reach the face: for the face's own axis the cells idx-2..idx+1, for the others
//     idx-1..idx+1 (|x| < 1.5 support of N_2).  Particles outside the grid keep a clamped key,
//     which stays inside every neighbourhood they can reach, and their weights come from their
//     real positions, exactly as the reference's bounds-checked scatter.
#include "pfm_internal.cuh"

namespace pfm {

constexpr int kBinThreads = 256;

// cell key + slot in the bin (slot order is arbitrary here; fixed by k_cell_sort)
template <int D>
__global__ void __launch_bounds__(kBinThreads) k_bin_keys(const float* __restrict__ pos, int64_t P, MacGeom g,
                                                          int* __restrict__ key, int* __restrict__ slot,
                                                          int* __restrict__ count) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  int c[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    float v = pos[a * P + q] / g.dx;  // int(particles_pos[i] / dx), 3D/run_3D.py:348
    int ci = __float2int_rz(v);
    ci = ci < 0 ? 0 : (ci > g.N[a] - 1 ? g.N[a] - 1 : ci);
    c[a] = ci;
  }
  int k = (D == 3) ? (c[0] * g.N[1] + c[1]) * g.N[2] + c[2] : c[0] * g.N[1] + c[1];
  key[q] = k;
  slot[q] = atomicAdd(&count[k], 1);
}

// exclusive scan of the bin counts: block sums, one-block scan of the sums, block-local scan
__global__ void __launch_bounds__(kScanThreads) k_scan_blocksums(const int* __restrict__ in, int64_t n,
                                                                 int* __restrict__ bsum) {
  const int64_t base = (int64_t)blockIdx.x * kScanThreads * kScanItems;
  int s = 0;
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    int64_t e = base + (int64_t)t * kScanThreads + threadIdx.x;
    if (e < n) s += in[e];
  }
  __shared__ int sm[kScanThreads / 32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    int v = threadIdx.x < kScanThreads / 32 ? sm[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) bsum[blockIdx.x] = v;
  }
}

__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
  __shared__ int sm[kScanThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < kScanThreads / 32 ? sm[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kScanThreads / 32) sm[lane] = w;
  }
  __syncthreads();
  int prefix = wid > 0 ? sm[wid - 1] : 0;
  if (total) *total = sm[kScanThreads / 32 - 1];
  __syncthreads();
  return prefix + x - v;
}

// one block: exclusive scan of nb block sums in place (nb <= kScanThreads * kScanItems)
__global__ void __launch_bounds__(kScanThreads) k_scan_top(int* __restrict__ bsum, int nb) {
  int vals[kScanItems];
  int loc = 0;
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    int e = threadIdx.x * kScanItems + t;
    vals[t] = e < nb ? bsum[e] : 0;
    loc += vals[t];
  }
  int total;
  int ex = block_exclusive_scan(loc, &total);
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    int e = threadIdx.x * kScanItems + t;
    if (e < nb) bsum[e] = ex;
    ex += vals[t];
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int* __restrict__ in, int64_t n,
                                                             const int* __restrict__ boff, int* __restrict__ out,
                                                             int total_P) {
  const int64_t base = (int64_t)blockIdx.x * kScanThreads * kScanItems;
  int vals[kScanItems];
  int loc = 0;
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    int64_t e = base + (int64_t)threadIdx.x * kScanItems + t;
    vals[t] = e < n ? in[e] : 0;
    loc += vals[t];
  }
  int ex = block_exclusive_scan(loc, nullptr) + boff[blockIdx.x];
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    int64_t e = base + (int64_t)threadIdx.x * kScanItems + t;
    if (e < n) out[e] = ex;
    ex += vals[t];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = total_P;
}

__global__ void __launch_bounds__(kBinThreads) k_scatter_order(const int* __restrict__ key, const int* __restrict__ slot,
                                                               const int* __restrict__ start, int64_t P,
                                                               int* __restrict__ order) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  order[start[key[q]] + slot[q]] = (int)q;
}

// each bin in ascending particle index: the stable order of a CPU counting sort
__global__ void __launch_bounds__(kBinThreads) k_cell_sort(const int* __restrict__ start, int64_t C,
                                                           int* __restrict__ order) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int b = start[c], e = start[c + 1];
  for (int i = b + 1; i < e; ++i) {
    int v = order[i];
    int j = i - 1;
    while (j >= b && order[j] > v) {
      order[j + 1] = order[j];
      --j;
    }
    order[j + 1] = v;
  }
}

// Payload (3D): per sorted slot s, record 0 = pos/dx, records 1..3 = (m_c, (T C T)_c row) for the
// three face families (3D/run_3D.py:462-479).
__global__ void __launch_bounds__(kBinThreads) k_payload3(const int* __restrict__ order, int64_t P, MacGeom g,
                                                          const float* __restrict__ pos, const float* __restrict__ imp0,
                                                          const float* __restrict__ Tg, const float* __restrict__ Ti,
                                                          const float* __restrict__ C, float4* __restrict__ pay) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= P) return;
  const int64_t q = order[s];
  float A[3][3], Cm[3][3], N[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      A[r][c] = Tg[(r * 3 + c) * P + q];   // rows(T_gm): A[r][c] = T_gm_r[c]
      Cm[r][c] = C[(r * 3 + c) * P + q];   // rows(init_C)
      N[c][r] = Ti[(r * 3 + c) * P + q];   // cols(T_init): N[k][c'] = T_init_c'[k]
    }
  // TCT = A^T (C A); T_transpose = A^T N; m = T_transpose init_imp
  float CA[3][3], TCT[3][3], TT[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) CA[r][c] = Cm[r][0] * A[0][c] + Cm[r][1] * A[1][c] + Cm[r][2] * A[2][c];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      TCT[r][c] = A[0][r] * CA[0][c] + A[1][r] * CA[1][c] + A[2][r] * CA[2][c];
      TT[r][c] = A[0][r] * N[0][c] + A[1][r] * N[1][c] + A[2][r] * N[2][c];
    }
  float m0[3] = {imp0[q], imp0[P + q], imp0[2 * P + q]};
  float m[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) m[r] = TT[r][0] * m0[0] + TT[r][1] * m0[1] + TT[r][2] * m0[2];
  float4* o = pay + s * 4;
  o[0] = make_float4(pos[q] / g.dx, pos[P + q] / g.dx, pos[2 * P + q] / g.dx, 0.f);
#pragma unroll
  for (int f = 0; f < 3; ++f) o[1 + f] = make_float4(m[f], TCT[f][0], TCT[f][1], TCT[f][2]);
}

// Payload (2D): record 0 = (pos/dx, psi), records 1..2 = (imp_c, C_c row, 0)
__global__ void __launch_bounds__(kBinThreads) k_payload2(const int* __restrict__ order, int64_t P, MacGeom g,
                                                          const float* __restrict__ pos, const float* __restrict__ imp,
                                                          const float* __restrict__ C, const float* __restrict__ psi,
                                                          float4* __restrict__ pay) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= P) return;
  const int64_t q = order[s];
  float4* o = pay + s * 3;
  o[0] = make_float4(pos[q] / g.dx, pos[P + q] / g.dx, psi ? psi[q] : 0.f, psi ? psi[P + q] : 0.f);
  o[1] = make_float4(imp[q], C[q], C[P + q], 0.f);
  o[2] = make_float4(imp[P + q], C[2 * P + q], C[3 * P + q], 0.f);
}

// per-face gather (3D), one face family per launch
template <int fam>
__global__ void __launch_bounds__(128) k_gather3(const float4* __restrict__ pay, const int* __restrict__ start,
                                                 MacGeom g, int use_apic, float* __restrict__ u,
                                                 float* __restrict__ w) {
  const int n0 = g.n[fam][0], n1 = g.n[fam][1], n2 = g.n[fam][2];
  const int64_t nf = (int64_t)n0 * n1 * n2;
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nf) return;
  int f[3];
  f[2] = (int)(e % n2);
  int64_t t = e / n2;
  f[1] = (int)(t % n1);
  f[0] = (int)(t / n1);
  int lo[3], hi[3];

#pragma unroll
  for (int a = 0; a < 3; ++a) {
    lo[a] = f[a] - (a == fam ? 2 : 1);
    hi[a] = f[a] + 1;
    lo[a] = lo[a] < 0 ? 0 : lo[a];
    hi[a] = hi[a] > g.N[a] - 1 ? g.N[a] - 1 : hi[a];

  }
  const float ff[3] = {(float)f[0], (float)f[1], (float)f[2]};
  float num = 0.f, den = 0.f;
  for (int ci = lo[0]; ci <= hi[0]; ++ci)
    for (int cj = lo[1]; cj <= hi[1]; ++cj) {
      const int rowc = (ci * g.N[1] + cj) * g.N[2];
      const int sb = __ldg(start + rowc + lo[2]), se = __ldg(start + rowc + hi[2] + 1);
      for (int s = sb; s < se; ++s) {  // the cells of a (ci, cj) row are contiguous in sorted order
        const float4 p0 = __ldg(pay + (int64_t)s * 4);
        const float pp[3] = {p0.x, p0.y, p0.z};
        float wgt = 1.f;
        float dp[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          float arg = (a == fam) ? (pp[a] - ff[a]) : ((pp[a] - ff[a]) - 0.5f);
          wgt *= N2(arg);
          dp[a] = ((a == fam) ? (ff[a] - pp[a]) : ((ff[a] + 0.5f) - pp[a])) * g.dx;
        }
        if (wgt == 0.f) continue;
        const float4 pf = __ldg(pay + (int64_t)s * 4 + 1 + fam);
        float delta = pf.y * dp[0] + pf.z * dp[1] + pf.w * dp[2];
        den += wgt;
        num += (use_apic ? (pf.x + delta) : pf.x) * wgt;
      }
    }
  w[e] = den;
  u[e] = den > 0.f ? num / den : num;  // 3D normalises by division (run_3D.py:530-552)
}

template <int fam>
__global__ void __launch_bounds__(128) k_gather2(const float4* __restrict__ pay, const int* __restrict__ start,
                                                 MacGeom g, int use_apic, float* __restrict__ u,
                                                 float* __restrict__ w, float* __restrict__ psig) {
  const int n0 = g.n[fam][0], n1 = g.n[fam][1];
  const int64_t nf = (int64_t)n0 * n1;
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nf) return;
  int f[2] = {(int)(e / n1), (int)(e % n1)};
  int lo[2], hi[2];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    lo[a] = f[a] - (a == fam ? 2 : 1);
    hi[a] = f[a] + 1;
    lo[a] = lo[a] < 0 ? 0 : lo[a];
    hi[a] = hi[a] > g.N[a] - 1 ? g.N[a] - 1 : hi[a];
  }
  const float ff[2] = {(float)f[0], (float)f[1]};
  float num = 0.f, den = 0.f, s0 = 0.f, s1 = 0.f;
  for (int ci = lo[0]; ci <= hi[0]; ++ci) {
    const int rowc = ci * g.N[1];
    const int sb = __ldg(start + rowc + lo[1]), se = __ldg(start + rowc + hi[1] + 1);
    for (int s = sb; s < se; ++s) {
      const float4 p0 = __ldg(pay + (int64_t)s * 3);
      const float pp[2] = {p0.x, p0.y};
      float wgt = 1.f, dp[2];
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        float arg = (a == fam) ? (pp[a] - ff[a]) : ((pp[a] - ff[a]) - 0.5f);
        wgt *= N2(arg);
        dp[a] = ((a == fam) ? (ff[a] - pp[a]) : ((ff[a] + 0.5f) - pp[a])) * g.dx;
      }
      if (wgt == 0.f) continue;
      const float4 pf = __ldg(pay + (int64_t)s * 3 + 1 + fam);
      float delta = pf.y * dp[0] + pf.z * dp[1];
      den += wgt;
      num += (use_apic ? (pf.x + delta) : pf.x) * wgt;
      s0 += p0.z * wgt;
      s1 += p0.w * wgt;
    }
  }
  w[e] = den;
  if (den > 0.f) {  // 2D normalises with scale = 1/w (run_2D.py:599-611)
    float scale = 1.f / den;
    num *= scale;
    s0 *= scale;
    s1 *= scale;
  }
  u[e] = num;
  if (psig) {
    psig[e * 2] = s0;
    psig[e * 2 + 1] = s1;
  }
}

int sort_particles(pfm_handle* h, const float* pos, cudaStream_t st) {
  int rc = require_ws(h);
  if (rc) return rc;
  const int64_t P = h->P, C = h->cells;
  int* key = ws_ptr<int>(h, h->o_key);
  int* slot = ws_ptr<int>(h, h->o_slot);
  int* order = ws_ptr<int>(h, h->o_order);
  int* count = ws_ptr<int>(h, h->o_count);
  int* start = ws_ptr<int>(h, h->o_start);
  int* bsum = ws_ptr<int>(h, h->o_blocksums);
  rc = check_cuda(h, cudaMemsetAsync(count, 0, C * 4, st), "memset counts");
  if (rc) return rc;
  if (P > 0) {
    if (h->cfg.dim == 3)
      launch(h, k_bin_keys<3>, grid_for(P, kBinThreads), kBinThreads, 0, st, pos, P, h->geom, key, slot, count);
    else
      launch(h, k_bin_keys<2>, grid_for(P, kBinThreads), kBinThreads, 0, st, pos, P, h->geom, key, slot, count);
  }
  const int64_t per_block = (int64_t)kScanThreads * kScanItems;
  const int nb = (int)((C + per_block - 1) / per_block);
  if (nb > kScanThreads * kScanItems) return set_error(h, PFM_ERR_SHAPE, "too many cells for the bin scan");
  launch(h, k_scan_blocksums, nb, kScanThreads, 0, st, count, C, bsum);
  launch(h, k_scan_top, 1, kScanThreads, 0, st, bsum, nb);
  launch(h, k_scan_apply, nb, kScanThreads, 0, st, count, C, bsum, start, (int)P);
  if (P > 0) {
    launch(h, k_scatter_order, grid_for(P, kBinThreads), kBinThreads, 0, st, key, slot, start, P, order);
    launch(h, k_cell_sort, grid_for(C, kBinThreads), kBinThreads, 0, st, start, C, order);
  }
  return launch_check(h, "sort_particles");
}

static int copy_sort_out(pfm_handle* h, int* cell_count, int* order, cudaStream_t st) {
  if (cell_count) {
    int rc = check_cuda(h, cudaMemcpyAsync(cell_count, ws_ptr<int>(h, h->o_count), h->cells * 4,
                                           cudaMemcpyDeviceToDevice, st), "copy counts");
    if (rc) return rc;
  }
  if (order && h->P > 0) {
    int rc = check_cuda(h, cudaMemcpyAsync(order, ws_ptr<int>(h, h->o_order), h->P * 4, cudaMemcpyDeviceToDevice, st),
                        "copy order");
    if (rc) return rc;
  }
  return PFM_OK;
}

}  // namespace pfm

using namespace pfm;

extern "C" {

int pfm3_sort_particles(pfm_handle* h, const float* pos, int* cell_count, int* order, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_sort_particles on a 2D handle");
  if (!pos && h->P > 0) return set_error(h, PFM_ERR_NULL, "pfm3_sort_particles: null pos");
  int rc = sort_particles(h, pos, (cudaStream_t)stream);
  if (rc) return rc;
  return copy_sort_out(h, cell_count, order, (cudaStream_t)stream);
}

int pfm2_sort_particles(pfm_handle* h, const float* pos, int* cell_count, int* order, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 2) return set_error(h, PFM_ERR_SHAPE, "pfm2_sort_particles on a 3D handle");
  if (!pos && h->P > 0) return set_error(h, PFM_ERR_NULL, "pfm2_sort_particles: null pos");
  int rc = sort_particles(h, pos, (cudaStream_t)stream);
  if (rc) return rc;
  return copy_sort_out(h, cell_count, order, (cudaStream_t)stream);
}

int pfm3_p2g(pfm_handle* h, const float* init_imp, const float* pos, const float* T_gm, const float* T_init,
             const float* init_C, float* u_x, float* u_y, float* u_z, float* w_x, float* w_y, float* w_z,
             void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_p2g on a 2D handle");
  if (!u_x || !u_y || !u_z || !w_x || !w_y || !w_z) return set_error(h, PFM_ERR_NULL, "pfm3_p2g: null grid");
  if (h->P > 0 && (!init_imp || !pos || !T_gm || !T_init || !init_C))
    return set_error(h, PFM_ERR_NULL, "pfm3_p2g: null particle field");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = sort_particles(h, pos, st);
  if (rc) return rc;
  float4* pay = ws_ptr<float4>(h, h->o_payload);
  if (h->P > 0)
    launch(h, k_payload3, grid_for(h->P, kBinThreads), kBinThreads, 0, st, ws_ptr<int>(h, h->o_order), h->P, h->geom, pos,
                                                                    init_imp, T_gm, T_init, init_C, pay);
  float* us[3] = {u_x, u_y, u_z};
  float* ws[3] = {w_x, w_y, w_z};
  for (int f = 0; f < 3; ++f) {
    int64_t nf = (int64_t)h->geom.n[f][0] * h->geom.n[f][1] * h->geom.n[f][2];
    const int* start = ws_ptr<int>(h, h->o_start);
    if (f == 0) launch(h, k_gather3<0>, grid_for(nf, 128), 128, 0, st, pay, start, h->geom, h->cfg.use_apic, us[f], ws[f]);
    if (f == 1) launch(h, k_gather3<1>, grid_for(nf, 128), 128, 0, st, pay, start, h->geom, h->cfg.use_apic, us[f], ws[f]);
    if (f == 2) launch(h, k_gather3<2>, grid_for(nf, 128), 128, 0, st, pay, start, h->geom, h->cfg.use_apic, us[f], ws[f]);
  }
  return launch_check(h, "pfm3_p2g");
}

int pfm2_p2g(pfm_handle* h, const float* imp, const float* pos, const float* C, const float* psi, float* u_x,
             float* u_y, float* psi_x, float* psi_y, float* w_x, float* w_y, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 2) return set_error(h, PFM_ERR_SHAPE, "pfm2_p2g on a 3D handle");
  if (!u_x || !u_y || !w_x || !w_y) return set_error(h, PFM_ERR_NULL, "pfm2_p2g: null grid");
  if (h->P > 0 && (!imp || !pos || !C)) return set_error(h, PFM_ERR_NULL, "pfm2_p2g: null particle field");
  if ((psi_x || psi_y) && !psi) return set_error(h, PFM_ERR_NULL, "pfm2_p2g: psi grids need particle psi");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = sort_particles(h, pos, st);
  if (rc) return rc;
  float4* pay = ws_ptr<float4>(h, h->o_payload);
  if (h->P > 0)
    launch(h, k_payload2, grid_for(h->P, kBinThreads), kBinThreads, 0, st, ws_ptr<int>(h, h->o_order), h->P, h->geom, pos,
                                                                    imp, C, psi, pay);
  float* us[2] = {u_x, u_y};
  float* ws[2] = {w_x, w_y};
  float* ps[2] = {psi_x, psi_y};
  for (int f = 0; f < 2; ++f) {
    int64_t nf = (int64_t)h->geom.n[f][0] * h->geom.n[f][1];
    const int* start = ws_ptr<int>(h, h->o_start);
    if (f == 0) launch(h, k_gather2<0>, grid_for(nf, 128), 128, 0, st, pay, start, h->geom, h->cfg.use_apic, us[f], ws[f], ps[f]);
    if (f == 1) launch(h, k_gather2<1>, grid_for(nf, 128), 128, 0, st, pay, start, h->geom, h->cfg.use_apic, us[f], ws[f], ps[f]);
  }
  return launch_check(h, "pfm2_p2g");
}

}  // extern "C"
