// Deterministic APIC particle-to-grid transfer (3D/run_3D.py:441-552, 2D/run_2D.py:548-611).
//
// The reference scatters 3 x 64 taps per particle with float atomic adds, so its sums depend on
// thread scheduling.  Here:
//  1. every particle gets the key int(pos/dx) (its cell, clamped to the grid) and a counting
//     sort with one digit of radix = number of cells bins the particles; each bin is then put in
//     particle-index order, so the permutation equals a stable CPU sort of the same keys;
//  2. a payload pass evaluates each particle's impulse m = T_gm^T-composed init_imp and affine
//     matrix T_gm^T C T_gm once, in sorted order (float4 records);
//  3. 3D: one thread per cell sums its particles into the window of faces they reach and cell
//     tiles merge the windows in shared memory in a fixed order (k_tile3); 2D: one thread per
//     face column gathers the particles of the cells that reach it (k_gather2).
//     Particles outside the grid keep a clamped key, which stays inside every neighbourhood they
//     can reach, and their weights come from their real positions, exactly as the reference's
//     bounds-checked scatter.
#include <climits>
#include <mutex>

#include "pfm_binsort.cuh"
#include "pfm_internal.cuh"

namespace pfm {

constexpr int kBinThreads = 256;

// cell key + slot in the bin (slot order is arbitrary here; fixed by k_cell_sort_staged)
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

// one block: exclusive scan of nb block sums in place, kScanThreads * kScanItems at a time with the
// running total carried between chunks (more than one chunk from 512^3 cells on)
__global__ void __launch_bounds__(kScanThreads) k_scan_top(int* __restrict__ bsum, int nb) {
  int carry = 0;
  for (int c0 = 0; c0 < nb; c0 += kScanThreads * kScanItems) {
    int vals[kScanItems];
    int loc = 0;
#pragma unroll
    for (int t = 0; t < kScanItems; ++t) {
      int e = c0 + threadIdx.x * kScanItems + t;
      vals[t] = e < nb ? bsum[e] : 0;
      loc += vals[t];
    }
    int total;
    int ex = block_exclusive_scan(loc, &total) + carry;
#pragma unroll
    for (int t = 0; t < kScanItems; ++t) {
      int e = c0 + threadIdx.x * kScanItems + t;
      if (e < nb) bsum[e] = ex;
      ex += vals[t];
    }
    carry += total;
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

// The same scatter for four consecutive particles per thread (16-byte loads of their keys and
// slots, the four bin-start lookups in flight together); needs P % 4 == 0.
__global__ void __launch_bounds__(kBinThreads) k_scatter_order4(const int4* __restrict__ key4,
                                                                const int4* __restrict__ slot4,
                                                                const int* __restrict__ start, int64_t P4,
                                                                int* __restrict__ order) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P4) return;
  const int4 k = key4[t], sl = slot4[t];
  const int s0 = start[k.x], s1 = start[k.y], s2 = start[k.z], s3 = start[k.w];
  const int q = (int)(4 * t);
  order[s0 + sl.x] = q;
  order[s1 + sl.y] = q + 1;
  order[s2 + sl.z] = q + 2;
  order[s3 + sl.w] = q + 3;
}

// Each bin in ascending particle index: the stable order of a CPU counting sort.  One thread per
// bin of up to kSmallBin entries (larger ones are left to k_bin_sort_big, pfm_binsort.cuh), with
// the block's span of `order` staged in shared memory: the 256 consecutive bins of a block are one
// contiguous run of entries, read and written back with coalesced accesses, and each thread sorts
// its bin there.  A block whose run exceeds the stage (large bins among its cells) sorts its bins
// in global memory.
constexpr int kSortStage = 4096;  // entries a block stages (16 KB; 8 per cell on average is 2,048)
__global__ void __launch_bounds__(kBinThreads) k_cell_sort_staged(const int* __restrict__ start, int64_t C,
                                                                  int* __restrict__ order) {
  __shared__ int stage[kSortStage];
  const int64_t c0 = (int64_t)blockIdx.x * kBinThreads, c = c0 + threadIdx.x;
  const int64_t cend = C < c0 + kBinThreads ? C : c0 + kBinThreads;
  const int base = start[c0], span = start[cend] - base;
  const int b = c < C ? start[c] : 0, e = c < C ? start[c + 1] : 0;
  if (span > kSortStage) {  // the same for the whole block
    if (c < C) sort_bin_by_thread(order, b, e - b);
    return;
  }
  for (int i = threadIdx.x; i < span; i += kBinThreads) stage[i] = order[base + i];
  __syncthreads();
  if (c < C) sort_bin_by_thread(stage, b - base, e - b);
  __syncthreads();
  for (int i = threadIdx.x; i < span; i += kBinThreads) order[base + i] = stage[i];
}

// Payload and cell keys (3D), one pass in particle order q (coalesced reads and writes); the
// record layout is write_p2g_record3's.
__global__ void __launch_bounds__(kBinThreads) k_payload_keys3(int64_t P, MacGeom g, const float* __restrict__ pos,
                                                               const float* __restrict__ Tg, P2GRecords3 R) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  const float v[3] = {pos[q] / g.dx, pos[P + q] / g.dx, pos[2 * P + q] / g.dx};
  float A[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) A[r][c] = Tg[(r * 3 + c) * P + q];  // rows(T_gm)
  write_p2g_record3(R, q, P, g, v, A);
}

// Payload (2D): pos4 = (pos/dx, psi), famrec[f] = (imp_f, C_f row, 0)
__global__ void __launch_bounds__(kBinThreads) k_payload2(const int* __restrict__ order, int64_t P, MacGeom g,
                                                          const float* __restrict__ pos, const float* __restrict__ imp,
                                                          const float* __restrict__ C, const float* __restrict__ psi,
                                                          float4* __restrict__ pos4, float4* __restrict__ famrec) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= P) return;
  const int64_t q = order[s];
  pos4[s] = make_float4(pos[q] / g.dx, pos[P + q] / g.dx, psi ? psi[q] : 0.f, psi ? psi[P + q] : 0.f);
  famrec[s] = make_float4(imp[q], C[q], C[P + q], 0.f);
  famrec[P + s] = make_float4(imp[P + q], C[2 * P + q], C[3 * P + q], 0.f);
}

// Tiled P2G (3D).  Cells are grouped in kTX x kTY x kTZ tiles, one thread per cell.  For each
// face family the thread sums its cell's particles (particle-index order) into a register window
// of the 4 x 3 x 3 faces they can reach (4 along the family's own axis: faces c-1 .. c+2; 3 along
// the others: c-1 .. c+1), every thread stores its window in shared memory (36 slots per cell),
// and after one barrier each face of the region around the tile sums the slots of the cells that
// reach it, in slot order, and adds the sum into the face grids.  Tiles run in 8 launches by the
// parity of their tile coordinates: tiles of one parity are a tile apart and their face regions
// (one face below, two above) never overlap, so no atomics are needed.  Each face sums in a fixed
// order (launch, pass, particle index): the result is bitwise reproducible (the same sums, in the
// same order, as merging the windows into a shared copy of the region in 36 passes with a barrier
// between passes).  Particles outside the grid sit in the clamped edge cell, whose window still
// holds every in-grid face they reach; their weights come from their real positions.
//
// Record staging: a cell's particles are gathered through the sorted order, so each one costs a
// memory round trip.  Every thread keeps a ring of kRing particle slots in shared memory (pos4 and
// the family record, 32 B) filled by 16-byte asynchronous copies (cp.async, no registers held), so
// kRing - 1 particles are in flight while one is summed; the next slot's particle index is read one
// iteration ahead.  The first kRing copies of the next family are issued before the window merge
// and face add-back of the current one, so that memory latency overlaps the merge.
//
// Tile of 4 x 4 x 16 cells (256 threads, 128 registers each): 16 along the last axis, the length
// of the seeding order's cell groups (pfm_seed_jittered), so the records of a group's particles
// are read by one tile in one launch (with 8-cell tiles a group's 128-particle runs are split
// between tiles of different parity launches and every record line is fetched twice).  With a
// ring of 2 a block holds 90 KB of shared memory, so two blocks share an SM and one block's
// barriers and window merge overlap the other's particle loop.  Measured at 256^3 (the P2G phase:
// sort, 8 tile launches, normalisation): 4 x 8 x 16 cells with a ring of 5 (one 224 KB block per
// SM) 10.33 ms; 4 x 4 x 16 with rings of 4 / 3 / 2 / 1 (two blocks per SM) 9.65 / 9.37 / 9.25 /
// 10.96 ms; 4 x 3 x 16 with rings of 5 / 4: 11.14 / 10.82 ms.
#ifndef PFM_TILE_X
#define PFM_TILE_X 4
#endif
#ifndef PFM_TILE_Y
#define PFM_TILE_Y 4
#endif
#ifndef PFM_TILE_Z
#define PFM_TILE_Z 16
#endif
constexpr int kTX = PFM_TILE_X, kTY = PFM_TILE_Y, kTZ = PFM_TILE_Z;
constexpr int kTileThreads = kTX * kTY * kTZ;
static_assert(kTileThreads % 32 == 0 && kTileThreads <= 512, "the P2G tiles are whole warps, at most 512 cells");
static_assert(kTX >= 3 && kTY >= 3 && kTZ >= 3, "same-parity tiles must be far enough apart for their face regions");
constexpr int kTileBlocksPerSM = 512 / kTileThreads;  // resident tile blocks per SM (128 registers a thread)
constexpr int kWinSlots = 4 * 3 * 3;                   // window faces per cell
#ifndef PFM_TILE_RING
#define PFM_TILE_RING 2
#endif
constexpr int kRing = PFM_TILE_RING;                                              // staged particles per thread
constexpr size_t kWinBytes = (size_t)kWinSlots * kTileThreads * sizeof(float2);  // 73,728 B
constexpr size_t kRingBytes = (size_t)kRing * 2 * kTileThreads * sizeof(float4);  // 16,384 B
constexpr size_t kTileSmem = kWinBytes + kRingBytes;                              // 92,160 B
static_assert(kTileSmem <= 227 * 1024, "k_tile3 exceeds the 227 KB of shared memory of a block");

struct FaceOut3 {
  float* u[3];
  float* w[3];
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Ring slot d of this thread: ring[(2 d) * kTileThreads + t] = pos4, ring[(2 d + 1) * kTileThreads + t] = record
// (a warp's 32 lanes read 512 contiguous bytes per slot array: no bank conflicts).
__device__ __forceinline__ void ring_fill(float4* ring, int d, const float4* __restrict__ pos4,
                                          const float4* __restrict__ rec, int q) {
  cp_async16(ring + (2 * d) * kTileThreads + threadIdx.x, pos4 + q);
  cp_async16(ring + (2 * d + 1) * kTileThreads + threadIdx.x, rec + q);
}

// The first kRing particles of a family's loop; one commit group per slot (empty past the end).
// Returns the particle index of slot sb + kRing (read ahead for the loop).
__device__ __forceinline__ int ring_prologue(float4* ring, const float4* __restrict__ pos4,
                                             const float4* __restrict__ rec, const int* __restrict__ order, int sb,
                                             int se) {
#pragma unroll
  for (int d = 0; d < kRing; ++d) {
    if (sb + d < se) ring_fill(ring, d, pos4, rec, __ldg(order + sb + d));
    cp_async_commit();
  }
  return sb + kRing < se ? __ldg(order + sb + kRing) : 0;
}

// Weights and offsets of the window faces c-1 .. c-1+W-1 along one axis (N_2 of 3D/run_3D.py:486).
// The offsets are face minus particle position in grid units: the records carry the affine rows
// already multiplied by dx (write_p2g_record3), so c (x_face - x_p) is formed without a multiply by
// dx per face (the same products when dx is a power of two, where both scalings are exact).
template <bool OWN>
__device__ __forceinline__ void tile_axis(float p, int c, float* w, float* d) {
  constexpr int W = OWN ? 4 : 3;
  const float fz = p - (float)c;
  if (c >= 1 && fz >= 0.f && fz < 1.f) {  // closed form of the branches (exact subtractions)
    if (OWN) {  // faces c-1 .. c+2 at x = fz+1, fz, fz-1, fz-2
      const bool lo = fz < 0.5f;
      const float t = lo ? fz : fz - 1.f;
      const float l = 0.5f - t, r = 0.5f + t;
      const float w0 = 0.5f * (l * l), w1 = 0.75f - t * t, w2 = 0.5f * (r * r);
      w[0] = lo ? w0 : 0.f;
      w[1] = lo ? w1 : w0;
      w[2] = lo ? w2 : w1;
      w[W - 1] = lo ? 0.f : w2;
    } else {  // faces c-1 .. c+1 at (x - 1/2) = t+1, t, t-1 with t = fz - 1/2
      const float t = fz - 0.5f;
      const float l = 0.5f - t, r = 0.5f + t;
      w[0] = 0.5f * (l * l);
      w[1] = 0.75f - t * t;
      w[2] = 0.5f * (r * r);
    }
  } else {  // first cell or outside the grid: per-face N_2 as the reference
#pragma unroll
    for (int o = 0; o < W; ++o) {
      const float t = (float)(c - 1 + o);
      w[o] = OWN ? N2(p - t) : N2((p - t) - 0.5f);
    }
  }
#pragma unroll
  for (int o = 0; o < W; ++o) {
    const float t = (float)(c - 1 + o);
    d[o] = OWN ? (t - p) : ((t + 0.5f) - p);
  }
}

// One family: the particle loop from the ring (whose prologue was issued earlier; qn is the index
// of slot sb + kRing), the window store, and -- after the barrier -- the next family's ring
// prologue (NEXT >= 0), the window merge and the face add-back.
template <int FAM, int NEXT, bool APIC>
__device__ __forceinline__ int tile_family(float2* __restrict__ win, float4* ring, const float4* __restrict__ pos4,
                                           const float4* __restrict__ rec, const float4* __restrict__ rec_next,
                                           const int* __restrict__ order, int sb, int se, int qn, int ci, int cj,
                                           int ck, int x0, int y0, int z0, const MacGeom& g,
                                           float* __restrict__ u, float* __restrict__ w) {
  constexpr int W0 = FAM == 0 ? 4 : 3, W1 = FAM == 1 ? 4 : 3, W2 = FAM == 2 ? 4 : 3;
  constexpr int E0 = kTX + W0 - 1, E1 = kTY + W1 - 1, E2 = kTZ + W2 - 1, NE = E0 * E1 * E2;
  static_assert(W0 * W1 * W2 <= kWinSlots, "window exceeds the shared buffer");
  float2 acc[W0][W1][W2];  // (numerator, weight sum) of each window face
#pragma unroll
  for (int a = 0; a < W0; ++a)
#pragma unroll
    for (int b = 0; b < W1; ++b)
#pragma unroll
      for (int k = 0; k < W2; ++k) acc[a][b][k] = make_float2(0.f, 0.f);
  int d = 0;
  for (int s = sb; s < se; ++s) {
    cp_async_wait<kRing - 1>();  // slot d (group s - sb of this family) has landed
    const float4 p = ring[(2 * d) * kTileThreads + threadIdx.x];
    const float4 fr = ring[(2 * d + 1) * kTileThreads + threadIdx.x];
    float w0[W0], d0[W0], w1[W1], d1[W1], w2[W2], d2[W2];
    tile_axis<FAM == 0>(p.x, ci, w0, d0);
    tile_axis<FAM == 1>(p.y, cj, w1, d1);
    tile_axis<FAM == 2>(p.z, ck, w2, d2);
    // Face (a, b, k) receives w0[a] w1[b] w2[k] (m + c1 d0[a] + c2 d1[b] + c3 d2[k]) with
    // (m, c1, c2, c3) the record (APIC: run_3D.py:486-528); factored per axis as
    // w2[k] P_ab + (w2[k] d2[k]) Q_ab, P_ab = w1[b] (m w0[a] + c1 w0[a] d0[a]) + c2 w0[a] (w1[b] d1[b]),
    // Q_ab = c3 w0[a] w1[b], the weight sum w0[a] w1[b] w2[k] riding in the same packed FMA:
    // two instructions per face instead of five (the same terms, associated differently).
    const float m = fr.x;
    const float c1 = APIC ? fr.y : 0.f, c2 = APIC ? fr.z : 0.f, c3 = APIC ? fr.w : 0.f;
    float e1[W1], e2[W2];
#pragma unroll
    for (int b = 0; b < W1; ++b) e1[b] = w1[b] * d1[b];
#pragma unroll
    for (int k = 0; k < W2; ++k) e2[k] = w2[k] * d2[k];
#pragma unroll
    for (int a = 0; a < W0; ++a) {
      const float alpha = fmaf(c1, w0[a] * d0[a], m * w0[a]);
      const float beta = c2 * w0[a], gamma = c3 * w0[a];
#pragma unroll
      for (int b = 0; b < W1; ++b) {
        const float2 pw = make_float2(fmaf(beta, e1[b], alpha * w1[b]), w0[a] * w1[b]);
        const float Q = gamma * w1[b];
#pragma unroll
        for (int k = 0; k < W2; ++k) {
          acc[a][b][k] = __ffma2_rn(make_float2(w2[k], w2[k]), pw, acc[a][b][k]);
          if (APIC) acc[a][b][k].x = fmaf(e2[k], Q, acc[a][b][k].x);  // without APIC Q = 0: adds 0
        }
      }
    }
    // refill the slot just read with particle s + kRing.  The empty asm takes sums that depend on
    // every value read from the slot, so those reads have completed before the copy is issued.
    asm volatile("" ::"f"(acc[W0 - 1][W1 - 1][W2 - 1].x), "f"(acc[W0 - 1][W1 - 1][W2 - 1].y) : "memory");
    if (s + kRing < se) {
      ring_fill(ring, d, pos4, rec, qn);
      if (s + kRing + 1 < se) qn = __ldg(order + s + kRing + 1);
    }
    cp_async_commit();
    d = d + 1 == kRing ? 0 : d + 1;
  }
#pragma unroll
  for (int a = 0; a < W0; ++a)
#pragma unroll
    for (int b = 0; b < W1; ++b)
#pragma unroll
      for (int k = 0; k < W2; ++k)
        win[((a * W1 + b) * W2 + k) * kTileThreads + threadIdx.x] = acc[a][b][k];
  __syncthreads();
  int qnext = 0;
  if (NEXT >= 0) qnext = ring_prologue(ring, pos4, rec_next, order, sb, se);
  // Face e of the tile's region (origin one face below the tile) takes window slot (a, b, k) of
  // the cell e - (a, b, k), summed from zero in slot order (a, then b, then k)
  const int n0 = g.n[FAM][0], n1 = g.n[FAM][1], n2 = g.n[FAM][2];
  constexpr int NPT = (NE + kTileThreads - 1) / kTileThreads;
  int64_t qs[NPT];
  float2 vs[NPT];
#pragma unroll
  for (int j = 0; j < NPT; ++j) {
    const int e = threadIdx.x + j * kTileThreads;
    const int ez = e % E2, r = e / E2, ey = r % E1, ex = r / E1;
    const int gi = x0 - 1 + ex, gj = y0 - 1 + ey, gk = z0 - 1 + ez;
    qs[j] = -1;
    if (e < NE && gi >= 0 && gi < n0 && gj >= 0 && gj < n1 && gk >= 0 && gk < n2) {
      qs[j] = ((int64_t)gi * n1 + gj) * n2 + gk;
      float2 v = make_float2(0.f, 0.f);
#pragma unroll
      for (int a = 0; a < W0; ++a) {
        const int sx = ex - a;
        if (sx < 0 || sx >= kTX) continue;
#pragma unroll
        for (int b = 0; b < W1; ++b) {
          const int sy = ey - b;
          if (sy < 0 || sy >= kTY) continue;
#pragma unroll
          for (int k = 0; k < W2; ++k) {
            const int sz = ez - k;
            if (sz < 0 || sz >= kTZ) continue;
            v = __fadd2_rn(v, win[((a * W1 + b) * W2 + k) * kTileThreads + (sx * kTY + sy) * kTZ + sz]);
          }
        }
      }
      vs[j] = make_float2(v.x + u[qs[j]], v.y + w[qs[j]]);
    }
  }
#pragma unroll
  for (int j = 0; j < NPT; ++j) {
    if (qs[j] >= 0) {
      u[qs[j]] = vs[j].x;
      w[qs[j]] = vs[j].y;
    }
  }
  __syncthreads();
  return qnext;
}

// One parity class (px, py, pz) of tiles; grid = (tiles along z, y, x of that parity).
template <bool APIC>
__global__ void __launch_bounds__(kTileThreads, kTileBlocksPerSM) k_tile3(const float4* __restrict__ pos4,
                                                           const float4* __restrict__ famrec,
                                                           const int* __restrict__ order,
                                                           const int* __restrict__ start, MacGeom g,
                                                           int64_t P, int px, int py, int pz, FaceOut3 out) {
  extern __shared__ __align__(16) unsigned char tile_smem[];
  float2* win = reinterpret_cast<float2*>(tile_smem);  // kWinSlots x kTileThreads window values (num, den)
  float4* ring = reinterpret_cast<float4*>(tile_smem + kWinBytes);
  const int x0 = (2 * (int)blockIdx.z + px) * kTX, y0 = (2 * (int)blockIdx.y + py) * kTY;
  const int z0 = (2 * (int)blockIdx.x + pz) * kTZ;
  const int lz = threadIdx.x % kTZ, ly = (threadIdx.x / kTZ) % kTY, lx = threadIdx.x / (kTZ * kTY);
  const int ci = x0 + lx, cj = y0 + ly, ck = z0 + lz;
  int sb = 0, se = 0;
  if (ci < g.N[0] && cj < g.N[1] && ck < g.N[2]) {
    const int c = (ci * g.N[1] + cj) * g.N[2] + ck;
    sb = __ldg(start + c);
    se = __ldg(start + c + 1);
  }
  const float4* r0 = famrec;
  const float4* r1 = famrec + P;
  const float4* r2 = famrec + 2 * P;
  int qn = ring_prologue(ring, pos4, r0, order, sb, se);
  qn = tile_family<0, 1, APIC>(win, ring, pos4, r0, r1, order, sb, se, qn, ci, cj, ck, x0, y0, z0, g, out.u[0],
                               out.w[0]);
  qn = tile_family<1, 2, APIC>(win, ring, pos4, r1, r2, order, sb, se, qn, ci, cj, ck, x0, y0, z0, g, out.u[1],
                               out.w[1]);
  tile_family<2, -1, APIC>(win, ring, pos4, r2, r2, order, sb, se, qn, ci, cj, ck, x0, y0, z0, g, out.u[2],
                           out.w[2]);
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------------------------
// P2G_smoke (3D/run_3D.py:554-593): the cell-centred 4-channel smoke field with the APIC term
// delta = dpos . (T_transpose @ init_grad_smoke), T_transpose = cols(T_gm) @ cols(T_init), weights
// N_2(pos - I - 1/2) per axis, normalised by the weight sum and clamped to [0, 1] where it is
// positive.  Same deterministic scheme as the impulse: bin sort, per-cell register windows (the
// 3 x 3 x 3 cells a particle cell reaches), parity-ordered cell tiles, no float atomics.
// ---------------------------------------------------------------------------------------------

// Record pass in particle order: pos4 = (pos/dx, 0), chrec[ch][q] = (s_ch, M[0][ch], M[1][ch],
// M[2][ch]) with M = T_transpose @ init_grad_smoke; cell key + bin slot as k_bin_keys.
__global__ void __launch_bounds__(kBinThreads) k_payload_smoke3(int64_t P, MacGeom g, const float* __restrict__ pos,
                                                                const float* __restrict__ Tg,
                                                                const float* __restrict__ Ti,
                                                                const float* __restrict__ s,
                                                                const float* __restrict__ Gs, float4* __restrict__ pos4,
                                                                float4* __restrict__ chrec, int* __restrict__ key,
                                                                int* __restrict__ slot, int* __restrict__ count) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  float v[3];
  int c[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    v[a] = pos[a * P + q] / g.dx;
    const int ci = __float2int_rz(v[a]);
    c[a] = ci < 0 ? 0 : (ci > g.N[a] - 1 ? g.N[a] - 1 : ci);
  }
  const int k = (c[0] * g.N[1] + c[1]) * g.N[2] + c[2];
  key[q] = k;
  slot[q] = atomicAdd(&count[k], 1);
  // TT[r][cc] = sum_k T_gm_k[r] * T_init_cc[k]
  float M[3][3], N[3][3], TT[3][3];
#pragma unroll
  for (int vv = 0; vv < 3; ++vv)
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
      M[cc][vv] = Tg[(vv * 3 + cc) * P + q];
      N[cc][vv] = Ti[(vv * 3 + cc) * P + q];
    }
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) TT[r][cc] = M[r][0] * N[0][cc] + M[r][1] * N[1][cc] + M[r][2] * N[2][cc];
  pos4[q] = make_float4(v[0], v[1], v[2], 0.f);
#pragma unroll
  for (int ch = 0; ch < 4; ++ch) {
    const float g0 = Gs[(0 * 4 + ch) * P + q], g1 = Gs[(1 * 4 + ch) * P + q], g2 = Gs[(2 * 4 + ch) * P + q];
    float m[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) m[r] = TT[r][0] * g0 + TT[r][1] * g1 + TT[r][2] * g2;
    chrec[ch * P + q] = make_float4(s[ch * P + q], m[0], m[1], m[2]);
  }
}


// One channel of one tile: window sums of (s + delta) w (and, with DEN, of w) over the 3 x 3 x 3
// cells; every thread stores its window in shared memory (27 slots x 512 cells) and after one
// barrier each cell of the tile's region sums the slots that reach it, from zero in slot order --
// the sums, in the order, of merging the windows in 27 barrier-separated passes -- and adds the
// sum into smoke[.][ch] (and the weight grid for ch 0).  The weights do not depend on the channel,
// so only channel 0 sums them.
template <bool DEN>
__device__ __forceinline__ void tile_smoke_channel(float2* __restrict__ win, const float4* __restrict__ pos4,
                                                   const float4* __restrict__ rec, const int* __restrict__ order,
                                                   int sb, int se, int ci, int cj, int ck, int x0, int y0, int z0,
                                                   const MacGeom& g, int use_apic, int ch,
                                                   float* __restrict__ smoke, float* __restrict__ wsum) {
  constexpr int E0 = kTX + 2, E1 = kTY + 2, E2 = kTZ + 2, NE = E0 * E1 * E2;
  float num[3][3][3], den[3][3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int k = 0; k < 3; ++k) num[a][b][k] = den[a][b][k] = 0.f;
  const float dx = g.dx;
  int qn = sb < se ? __ldg(order + sb) : 0;  // next slot's particle read one iteration ahead
  for (int s = sb; s < se; ++s) {
    const int q = qn;
    if (s + 1 < se) qn = __ldg(order + s + 1);
    const float4 p = __ldg(pos4 + q);
    const float4 fr = __ldg(rec + q);
    float w0[3], d0[3], w1[3], d1[3], w2[3], d2[3];
    tile_axis<false>(p.x, ci, w0, d0);
    tile_axis<false>(p.y, cj, w1, d1);
    tile_axis<false>(p.z, ck, w2, d2);
#pragma unroll
    for (int o = 0; o < 3; ++o) {  // the smoke records are not pre-scaled: offsets in world units
      d0[o] *= dx;
      d1[o] *= dx;
      d2[o] *= dx;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const float w01 = w0[a] * w1[b];
        const float d01 = fr.y * d0[a] + fr.z * d1[b];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float wt = w01 * w2[k];
          const float delta = d01 + fr.w * d2[k];
          num[a][b][k] += (use_apic ? (fr.x + delta) : fr.x) * wt;
          if (DEN) den[a][b][k] += wt;
        }
      }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        win[((a * 3 + b) * 3 + k) * kTileThreads + threadIdx.x] = make_float2(num[a][b][k], den[a][b][k]);
  __syncthreads();
  const int n0 = g.N[0], n1 = g.N[1], n2 = g.N[2];
  constexpr int NPT = (NE + kTileThreads - 1) / kTileThreads;
  int64_t qs[NPT];
  float2 vs[NPT];
#pragma unroll
  for (int j = 0; j < NPT; ++j) {
    const int e = threadIdx.x + j * kTileThreads;
    const int ez = e % E2, r = e / E2, ey = r % E1, ex = r / E1;
    const int gi = x0 - 1 + ex, gj = y0 - 1 + ey, gk = z0 - 1 + ez;
    qs[j] = -1;
    if (e < NE && gi >= 0 && gi < n0 && gj >= 0 && gj < n1 && gk >= 0 && gk < n2) {
      qs[j] = ((int64_t)gi * n1 + gj) * n2 + gk;
      float2 v = make_float2(0.f, 0.f);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const int sx = ex - a;
        if (sx < 0 || sx >= kTX) continue;
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          const int sy = ey - b;
          if (sy < 0 || sy >= kTY) continue;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const int sz = ez - k;
            if (sz < 0 || sz >= kTZ) continue;
            const float2 f = win[((a * 3 + b) * 3 + k) * kTileThreads + (sx * kTY + sy) * kTZ + sz];
            v.x += f.x;
            if (DEN) v.y += f.y;
          }
        }
      }
      vs[j] = make_float2(v.x + smoke[qs[j] * 4 + ch], DEN ? v.y + wsum[qs[j]] : 0.f);
    }
  }
#pragma unroll
  for (int j = 0; j < NPT; ++j) {
    if (qs[j] >= 0) {
      smoke[qs[j] * 4 + ch] = vs[j].x;
      if (DEN) wsum[qs[j]] = vs[j].y;
    }
  }
  __syncthreads();
}

constexpr size_t kSmokeTileSmem = (size_t)27 * kTileThreads * sizeof(float2);  // 55,296 B

__global__ void __launch_bounds__(kTileThreads, kTileBlocksPerSM) k_tile_smoke3(const float4* __restrict__ pos4,
                                                                 const float4* __restrict__ chrec,
                                                                 const int* __restrict__ order,
                                                                 const int* __restrict__ start, MacGeom g, int use_apic,
                                                                 int64_t P, int px, int py, int pz,
                                                                 float* __restrict__ smoke, float* __restrict__ wsum) {
  extern __shared__ float2 win[];  // 27 x kTileThreads window values (num, den)
  const int x0 = (2 * (int)blockIdx.z + px) * kTX, y0 = (2 * (int)blockIdx.y + py) * kTY;
  const int z0 = (2 * (int)blockIdx.x + pz) * kTZ;
  const int lz = threadIdx.x % kTZ, ly = (threadIdx.x / kTZ) % kTY, lx = threadIdx.x / (kTZ * kTY);
  const int ci = x0 + lx, cj = y0 + ly, ck = z0 + lz;
  int sb = 0, se = 0;
  if (ci < g.N[0] && cj < g.N[1] && ck < g.N[2]) {
    const int c = (ci * g.N[1] + cj) * g.N[2] + ck;
    sb = __ldg(start + c);
    se = __ldg(start + c + 1);
  }
  tile_smoke_channel<true>(win, pos4, chrec, order, sb, se, ci, cj, ck, x0, y0, z0, g, use_apic, 0, smoke, wsum);
#pragma unroll 1
  for (int ch = 1; ch < 4; ++ch)
    tile_smoke_channel<false>(win, pos4, chrec + ch * P, order, sb, se, ci, cj, ck, x0, y0, z0, g, use_apic, ch,
                              smoke, wsum);
}

// smoke /= w and clamp every channel to [0, 1] where w > 0 (3D/run_3D.py:584-591)
__global__ void __launch_bounds__(kBinThreads) k_normalize_smoke3(float4* __restrict__ smoke,
                                                                  const float* __restrict__ wsum, int64_t C) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= C) return;
  const float w = wsum[e];
  if (!(w > 0.f)) return;
  float4 s = smoke[e];
  float* c = reinterpret_cast<float*>(&s);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    float x = c[j] / w;
    if (x < 0.f) x = 0.f;
    if (x > 1.f) x = 1.f;
    c[j] = x;
  }
  smoke[e] = s;
}

// u = u / w where w > 0 (3D/run_3D.py:530-552), all three families in one pass
__global__ void __launch_bounds__(kBinThreads) k_normalize3(FaceOut3 out, int64_t F0, int64_t F1, int64_t F2) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int f = 0;
  if (e >= F0) {
    e -= F0;
    f = 1;
    if (e >= F1) {
      e -= F1;
      f = 2;
      if (e >= F2) return;
    }
  }
  float* u = f == 0 ? out.u[0] : (f == 1 ? out.u[1] : out.u[2]);
  const float* w = f == 0 ? out.w[0] : (f == 1 ? out.w[1] : out.w[2]);
  const float wv = w[e];
  if (wv > 0.f) u[e] = u[e] / wv;
}

// The same division four faces at a time (16-byte vectors of u and w; every family's face count a
// multiple of 4 and the six arrays 16-byte aligned): element for element k_normalize3.
__global__ void __launch_bounds__(kBinThreads) k_normalize3v(FaceOut3 out, int64_t Q0, int64_t Q1, int64_t Q2) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int f = 0;
  if (e >= Q0) {
    e -= Q0;
    f = 1;
    if (e >= Q1) {
      e -= Q1;
      f = 2;
      if (e >= Q2) return;
    }
  }
  float4* u = reinterpret_cast<float4*>(f == 0 ? out.u[0] : (f == 1 ? out.u[1] : out.u[2]));
  const float4* w = reinterpret_cast<const float4*>(f == 0 ? out.w[0] : (f == 1 ? out.w[1] : out.w[2]));
  const float4 wv = w[e];
  float4 uv = u[e];
  if (wv.x > 0.f) uv.x = uv.x / wv.x;
  if (wv.y > 0.f) uv.y = uv.y / wv.y;
  if (wv.z > 0.f) uv.z = uv.z / wv.z;
  if (wv.w > 0.f) uv.w = uv.w / wv.w;
  u[e] = uv;
}

// Column gather (2D): columns along j; 2D normalises with scale = 1/w (run_2D.py:599-611) and
// also carries the reference map psi.
template <int fam>
__global__ void __launch_bounds__(128) k_gather2(const float4* __restrict__ pos4, const float4* __restrict__ famrec,
                                                 const int* __restrict__ start, MacGeom g, int K, int use_apic,
                                                 int64_t P, float* __restrict__ u, float* __restrict__ w,
                                                 float* __restrict__ psig) {
  constexpr int WIN = (fam == 1) ? 4 : 3;
  const int n0 = g.n[fam][0], n1 = g.n[fam][1];
  const int nseg = (n1 + K - 1) / K;
  const int64_t ncol = (int64_t)n0 * nseg;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncol) return;
  const int i = (int)(t % n0);
  const int seg = (int)(t / n0);
  const int j0 = seg * K, j1 = min(j0 + K, n1);
  const int G0 = g.N[0], G1 = g.N[1];
  const int ci_lo = max(i - (fam == 0 ? 2 : 1), 0), ci_hi = min(i + 1, G0 - 1);
  const int cj_lo = max(j0 - (fam == 1 ? 2 : 1), 0), cj_hi = min(j1, G1 - 1);
  const float fi = (float)i, dx = g.dx;
  float num[WIN], den[WIN], s0[WIN], s1[WIN];
#pragma unroll
  for (int q = 0; q < WIN; ++q) num[q] = den[q] = s0[q] = s1[q] = 0.f;
  auto flush = [&](int jf, int q) {
    if (jf >= j0 && jf < j1) {
      const int64_t e = (int64_t)i * n1 + jf;
      float a = num[q], b0 = s0[q], b1 = s1[q];
      if (den[q] > 0.f) {
        float scale = 1.f / den[q];
        a *= scale;
        b0 *= scale;
        b1 *= scale;
      }
      w[e] = den[q];
      u[e] = a;
      if (psig) {
        psig[e * 2] = b0;
        psig[e * 2 + 1] = b1;
      }
    }
  };
  int jb = cj_lo - 1;
  for (int cj = cj_lo; cj <= cj_hi; ++cj) {
    while (jb < cj - 1) {
      flush(jb, 0);
#pragma unroll
      for (int q = 0; q < WIN - 1; ++q) {
        num[q] = num[q + 1];
        den[q] = den[q + 1];
        s0[q] = s0[q + 1];
        s1[q] = s1[q + 1];
      }
      num[WIN - 1] = den[WIN - 1] = s0[WIN - 1] = s1[WIN - 1] = 0.f;
      ++jb;
    }
    const float fj0 = (float)(cj - 1);
    for (int ci = ci_lo; ci <= ci_hi; ++ci) {
      const int c = ci * G1 + cj;
      const int sb = __ldg(start + c), se = __ldg(start + c + 1);
      for (int s = sb; s < se; ++s) {
        const float4 p = __ldg(pos4 + s);
        float wi, di;
        if (fam == 0) {
          wi = N2(p.x - fi);
          di = (fi - p.x) * dx;
        } else {
          wi = N2((p.x - fi) - 0.5f);
          di = ((fi + 0.5f) - p.x) * dx;
        }
        if (wi == 0.f) continue;
        const float4 fr = __ldg(famrec + (int64_t)fam * P + s);
#pragma unroll
        for (int q = 0; q < WIN; ++q) {
          const float fj = fj0 + (float)q;
          float wj, dj;
          if (fam == 1) {
            wj = N2(p.y - fj);
            dj = (fj - p.y) * dx;
          } else {
            wj = N2((p.y - fj) - 0.5f);
            dj = ((fj + 0.5f) - p.y) * dx;
          }
          const float wt = wi * wj;
          const float delta = fr.y * di + fr.z * dj;
          num[q] += (use_apic ? (fr.x + delta) : fr.x) * wt;
          den[q] += wt;
          s0[q] += p.z * wt;
          s1[q] += p.w * wt;
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < WIN; ++q) flush(jb + q, q);
}

// Bins with counted keys/slots -> bin starts and the stable order (scan, scatter, per-bin sort).
static int sort_from_keys(pfm_handle* h, cudaStream_t st) {
  const int64_t P = h->P, C = h->cells;
  const int* key = ws_ptr<int>(h, h->o_key);
  const int* slot = ws_ptr<int>(h, h->o_slot);
  int* order = ws_ptr<int>(h, h->o_order);
  int* count = ws_ptr<int>(h, h->o_count);
  int* start = ws_ptr<int>(h, h->o_start);
  int* bsum = ws_ptr<int>(h, h->o_blocksums);
  const int64_t per_block = (int64_t)kScanThreads * kScanItems;
  const int nb = (int)((C + per_block - 1) / per_block);
  launch(h, k_scan_blocksums, nb, kScanThreads, 0, st, (const int*)count, C, bsum);
  launch(h, k_scan_top, 1, kScanThreads, 0, st, bsum, nb);
  launch(h, k_scan_apply, nb, kScanThreads, 0, st, (const int*)count, C, (const int*)bsum, start, (int)P);
  if (P > 0) {
    if (P % 4 == 0 && ((uintptr_t)key | (uintptr_t)slot) % 16 == 0)
      launch(h, k_scatter_order4, grid_for(P / 4, kBinThreads), kBinThreads, 0, st, (const int4*)key,
             (const int4*)slot, (const int*)start, P / 4, order);
    else
      launch(h, k_scatter_order, grid_for(P, kBinThreads), kBinThreads, 0, st, key, slot, (const int*)start, P, order);
    launch(h, k_cell_sort_staged, grid_for(C, kBinThreads), kBinThreads, 0, st, (const int*)start, C, order);
    launch(h, k_bin_sort_big, grid_for(C, kBigThreads), kBigThreads, 0, st, (const int*)start, C, order);
  }
  return launch_check(h, "sort_particles");
}

int sort_particles(pfm_handle* h, const float* pos, cudaStream_t st) {
  int rc = require_ws(h);
  if (rc) return rc;
  const int64_t P = h->P;
  int* key = ws_ptr<int>(h, h->o_key);
  int* slot = ws_ptr<int>(h, h->o_slot);
  int* count = ws_ptr<int>(h, h->o_count);
  h->rec_valid = 0;  // the keys of the P2G records are overwritten
  rc = check_cuda(h, cudaMemsetAsync(count, 0, h->cells * 4, st), "memset counts");
  if (rc) return rc;
  if (P > 0) {
    if (h->cfg.dim == 3)
      launch(h, k_bin_keys<3>, grid_for(P, kBinThreads), kBinThreads, 0, st, pos, P, h->geom, key, slot, count);
    else
      launch(h, k_bin_keys<2>, grid_for(P, kBinThreads), kBinThreads, 0, st, pos, P, h->geom, key, slot, count);
  }
  return sort_from_keys(h, st);
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

P2GRecords3 records3(pfm_handle* h, const float* init_imp, const float* T_init, const float* init_C) {
  float4* pos4 = ws_ptr<float4>(h, h->o_payload);
  return P2GRecords3{init_imp, T_init, init_C, pos4, pos4 + h->P, ws_ptr<int>(h, h->o_key), ws_ptr<int>(h, h->o_slot),
                     ws_ptr<int>(h, h->o_count)};
}

// P2G from records and keys already in the workspace: bin sort, tiles, normalisation.
int p2g3_from_records(pfm_handle* h, float* const* us, float* const* ws, cudaStream_t st) {
  int rc = sort_from_keys(h, st);
  if (rc) return rc;
  const float4* pos4 = ws_ptr<float4>(h, h->o_payload);
  const float4* famrec = pos4 + h->P;
  const int* start = ws_ptr<int>(h, h->o_start);
  const int* order = ws_ptr<int>(h, h->o_order);
  FaceOut3 out{{us[0], us[1], us[2]}, {ws[0], ws[1], ws[2]}};
  int64_t F[3];
  for (int f = 0; f < 3; ++f) {
    F[f] = (int64_t)h->geom.n[f][0] * h->geom.n[f][1] * h->geom.n[f][2];
    rc = check_cuda(h, cudaMemsetAsync(us[f], 0, F[f] * 4, st), "zero u");
    if (!rc) rc = check_cuda(h, cudaMemsetAsync(ws[f], 0, F[f] * 4, st), "zero w");
    if (rc) return rc;
  }
  if (h->P > 0) {
    static std::atomic<unsigned long long> attr{0};  // above the default 48 KB: opt in per device
    auto tile = h->cfg.use_apic ? k_tile3<true> : k_tile3<false>;
    rc = check_cuda(h, opt_in_smem(tile, (int)kTileSmem, attr), "k_tile3 shared-memory attribute");
    if (rc) return rc;
    const int nt[3] = {(h->geom.N[0] + kTX - 1) / kTX, (h->geom.N[1] + kTY - 1) / kTY, (h->geom.N[2] + kTZ - 1) / kTZ};
    for (int px = 0; px < 2; ++px)
      for (int py = 0; py < 2; ++py)
        for (int pz = 0; pz < 2; ++pz) {
          const unsigned bx = (nt[0] - px + 1) / 2, by = (nt[1] - py + 1) / 2, bz = (nt[2] - pz + 1) / 2;
          if (!bx || !by || !bz) continue;
          launch(h, tile, dim3(bz, by, bx), kTileThreads, kTileSmem, st, pos4, famrec, order, start, h->geom, h->P,
                 px, py, pz, out);
        }
    bool vec = true;
    for (int f = 0; f < 3; ++f)
      vec = vec && F[f] % 4 == 0 && ((uintptr_t)us[f] | (uintptr_t)ws[f]) % 16 == 0;
    if (vec)
      launch(h, k_normalize3v, grid_for((F[0] + F[1] + F[2]) / 4, kBinThreads), kBinThreads, 0, st, out, F[0] / 4,
             F[1] / 4, F[2] / 4);
    else
      launch(h, k_normalize3, grid_for(F[0] + F[1] + F[2], kBinThreads), kBinThreads, 0, st, out, F[0], F[1], F[2]);
  }
  return launch_check(h, "p2g3");
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
  int rc = require_ws(h);
  if (rc) return rc;
  rc = check_cuda(h, cudaMemsetAsync(ws_ptr<int>(h, h->o_count), 0, h->cells * 4, st), "memset counts");
  if (rc) return rc;
  const P2GRecords3 R = records3(h, init_imp, T_init, init_C);
  if (h->P > 0)
    launch(h, k_payload_keys3, grid_for(h->P, kBinThreads), kBinThreads, 0, st, h->P, h->geom, pos, T_gm, R);
  h->rec_valid = 1;
  float* u[3] = {u_x, u_y, u_z};
  float* w[3] = {w_x, w_y, w_z};
  return p2g3_from_records(h, u, w, st);
}

int pfm3_rk4_p2g_records(pfm_handle* h, float* pos, float* T_gm, const float* ua_x, const float* ua_y,
                         const float* ua_z, float dt, const float* init_imp, const float* T_init, const float* init_C,
                         void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_rk4_p2g_records on a 2D handle");
  if (!ua_x || !ua_y || !ua_z) return set_error(h, PFM_ERR_NULL, "pfm3_rk4_p2g_records: null grid");
  if (h->P > 0 && (!init_imp || !pos || !T_gm || !T_init || !init_C))
    return set_error(h, PFM_ERR_NULL, "pfm3_rk4_p2g_records: null particle field");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = require_ws(h);
  if (rc) return rc;
  rc = check_cuda(h, cudaMemsetAsync(ws_ptr<int>(h, h->o_count), 0, h->cells * 4, st), "memset counts");
  if (rc) return rc;
  const P2GRecords3 R = records3(h, init_imp, T_init, init_C);
  const MacFields3 F{{ua_x, ua_y, ua_z}};
  rc = launch_rk4_T_forward3(h, pos, T_gm, F, dt, &R, nullptr, st);
  if (rc) return rc;
  h->rec_valid = 1;
  return PFM_OK;
}

int pfm3_gradm_rk4_p2g_records(pfm_handle* h, float* pos, float* T_gm, float* T_init, float* init_C,
                               const float* init_imp, const float* u_x, const float* u_y, const float* u_z,
                               const float* ua_x, const float* ua_y, const float* ua_z, float dt, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_gradm_rk4_p2g_records on a 2D handle");
  if (!u_x || !u_y || !u_z || !ua_x || !ua_y || !ua_z)
    return set_error(h, PFM_ERR_NULL, "pfm3_gradm_rk4_p2g_records: null grid");
  if (h->P > 0 && (!init_imp || !pos || !T_gm || !T_init || !init_C))
    return set_error(h, PFM_ERR_NULL, "pfm3_gradm_rk4_p2g_records: null particle field");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = require_ws(h);
  if (rc) return rc;
  rc = check_cuda(h, cudaMemsetAsync(ws_ptr<int>(h, h->o_count), 0, h->cells * 4, st), "memset counts");
  if (rc) return rc;
  const P2GRecords3 R = records3(h, init_imp, T_init, init_C);
  const MacFields3 F{{ua_x, ua_y, ua_z}}, Fg{{u_x, u_y, u_z}};
  rc = launch_rk4_T_forward3(h, pos, T_gm, F, dt, &R, &Fg, st);
  if (rc) return rc;
  h->rec_valid = 1;
  return PFM_OK;
}

int pfm3_p2g_from_records(pfm_handle* h, float* u_x, float* u_y, float* u_z, float* w_x, float* w_y, float* w_z,
                          void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_p2g_from_records on a 2D handle");
  if (!u_x || !u_y || !u_z || !w_x || !w_y || !w_z) return set_error(h, PFM_ERR_NULL, "pfm3_p2g_from_records: null grid");
  int rc = require_ws(h);
  if (rc) return rc;
  if (!h->rec_valid)
    return set_error(h, PFM_ERR_ARG, "pfm3_p2g_from_records: no P2G records in the workspace (call "
                                     "pfm3_rk4_p2g_records first; a sort or 2D P2G call overwrites them)");
  float* u[3] = {u_x, u_y, u_z};
  float* w[3] = {w_x, w_y, w_z};
  return p2g3_from_records(h, u, w, (cudaStream_t)stream);
}

int pfm3_rk4_p2g(pfm_handle* h, float* pos, float* T_gm, const float* ua_x, const float* ua_y, const float* ua_z,
                 float dt, const float* init_imp, const float* T_init, const float* init_C, float* u_x, float* u_y,
                 float* u_z, float* w_x, float* w_y, float* w_z, void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (!u_x || !u_y || !u_z || !w_x || !w_y || !w_z) return set_error(h, PFM_ERR_NULL, "pfm3_rk4_p2g: null grid");
  int rc = pfm3_rk4_p2g_records(h, pos, T_gm, ua_x, ua_y, ua_z, dt, init_imp, T_init, init_C, stream);
  if (rc) return rc;
  return pfm3_p2g_from_records(h, u_x, u_y, u_z, w_x, w_y, w_z, stream);
}

int pfm3_p2g_smoke(pfm_handle* h, const float* smoke_p, const float* init_grad_smoke, const float* pos,
                   const float* T_gm, const float* T_init, int use_apic_smoke, float* smoke, float* weight,
                   void* stream) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_p2g_smoke on a 2D handle");
  if (!smoke || !weight) return set_error(h, PFM_ERR_NULL, "pfm3_p2g_smoke: null grid");
  if (((uintptr_t)smoke) & 15) return set_error(h, PFM_ERR_ARG, "pfm3_p2g_smoke: smoke not 16-byte aligned");
  if (h->P > 0 && (!smoke_p || !init_grad_smoke || !pos || !T_gm || !T_init))
    return set_error(h, PFM_ERR_NULL, "pfm3_p2g_smoke: null particle field");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = require_ws(h);
  if (rc) return rc;
  rc = check_cuda(h, cudaMemsetAsync(ws_ptr<int>(h, h->o_count), 0, h->cells * 4, st), "memset counts");
  if (!rc) rc = check_cuda(h, cudaMemsetAsync(smoke, 0, h->cells * 16, st), "zero smoke");
  if (!rc) rc = check_cuda(h, cudaMemsetAsync(weight, 0, h->cells * 4, st), "zero weight");
  if (rc) return rc;
  h->rec_valid = 0;  // the impulse records share the payload
  float4* pos4 = ws_ptr<float4>(h, h->o_payload);
  float4* chrec = pos4 + h->P;
  if (h->P > 0)
    launch(h, k_payload_smoke3, grid_for(h->P, kBinThreads), kBinThreads, 0, st, h->P, h->geom, pos, T_gm, T_init,
           smoke_p, init_grad_smoke, pos4, chrec, ws_ptr<int>(h, h->o_key), ws_ptr<int>(h, h->o_slot),
           ws_ptr<int>(h, h->o_count));
  rc = sort_from_keys(h, st);
  if (rc) return rc;
  if (h->P > 0) {
    const int* start = ws_ptr<int>(h, h->o_start);
    const int* order = ws_ptr<int>(h, h->o_order);
    static std::atomic<unsigned long long> attr{0};  // above the default 48 KB: opt in per device
    rc = check_cuda(h, opt_in_smem(k_tile_smoke3, (int)kSmokeTileSmem, attr), "k_tile_smoke3 shared-memory attribute");
    if (rc) return rc;
    const int nt[3] = {(h->geom.N[0] + kTX - 1) / kTX, (h->geom.N[1] + kTY - 1) / kTY, (h->geom.N[2] + kTZ - 1) / kTZ};
    for (int px = 0; px < 2; ++px)
      for (int py = 0; py < 2; ++py)
        for (int pz = 0; pz < 2; ++pz) {
          const unsigned bx = (nt[0] - px + 1) / 2, by = (nt[1] - py + 1) / 2, bz = (nt[2] - pz + 1) / 2;
          if (!bx || !by || !bz) continue;
          launch(h, k_tile_smoke3, dim3(bz, by, bx), kTileThreads, kSmokeTileSmem, st, (const float4*)pos4,
                 (const float4*)chrec, order, start, h->geom, use_apic_smoke ? 1 : 0, h->P, px, py, pz, smoke,
                 weight);
        }
    launch(h, k_normalize_smoke3, grid_for(h->cells, kBinThreads), kBinThreads, 0, st,
           reinterpret_cast<float4*>(smoke), (const float*)weight, h->cells);
  }
  return launch_check(h, "pfm3_p2g_smoke");
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
  float4* pos4 = ws_ptr<float4>(h, h->o_payload);
  float4* famrec = pos4 + h->P;
  h->rec_valid = 0;
  if (h->P > 0)
    launch(h, k_payload2, grid_for(h->P, kBinThreads), kBinThreads, 0, st, ws_ptr<int>(h, h->o_order), h->P, h->geom,
           pos, imp, C, psi, pos4, famrec);
  float* us[2] = {u_x, u_y};
  float* ws[2] = {w_x, w_y};
  float* ps[2] = {psi_x, psi_y};
  const int* start = ws_ptr<int>(h, h->o_start);
  for (int f = 0; f < 2; ++f) {
    const int n1 = h->geom.n[f][1];
    const int K = n1 < h->p2g2_column ? n1 : h->p2g2_column;
    const int64_t ncol = (int64_t)h->geom.n[f][0] * ((n1 + K - 1) / K);
    if (f == 0) launch(h, k_gather2<0>, grid_for(ncol, 128), 128, 0, st, pos4, famrec, start, h->geom, K,
                       h->cfg.use_apic, h->P, us[f], ws[f], ps[f]);
    if (f == 1) launch(h, k_gather2<1>, grid_for(ncol, 128), 128, 0, st, pos4, famrec, start, h->geom, K,
                       h->cfg.use_apic, h->P, us[f], ws[f], ps[f]);
  }
  return launch_check(h, "pfm2_p2g");
}

}  // extern "C"
