// Learned warm start for the pressure solve: the layers of a 3D convolutional U-Net in BF16 with
// FP32 accumulation, forward and backward, on the fifth-generation tensor cores.
//
// Activation layout ("channel-blocked"): a tensor with C channels on an n0 x n1 x n2 grid is
// [C/8][n0][n1][n2][8] bf16 -- eight channels (16 bytes) per voxel per block.  This makes every
// operand an MMA needs a canonical no-swizzle K-major tile in shared memory without any copy:
//
//  * Forward / data-gradient convolution (k_conv3_fwd): implicit GEMM D[voxel][cout] =
//    sum over 27 taps and cin of X[voxel + tap][ci] W[tap][co][ci].  A CTA owns 128 output voxels
//    (one d0 plane, 16 rows of 8 along d2).  One TMA tiled load brings the 3 x 18 x 10 input brick
//    with its halo (zero fill outside the grid is the convolution's padding) as
//    [cin/8][3][18][10][8]: for a fixed 8-channel block, 8 consecutive voxels along d2 are 8
//    consecutive 16-byte rows, i.e. an 8x16B "core matrix"; the 16 rows of the tile are 160 bytes
//    apart and the channel blocks 8640 bytes apart.  Each tap is then just another start address of
//    the same shared-memory descriptor (LBO 8640, SBO 160): no im2col in memory or in shared
//    memory.  The weights of one tap, [cin/8][npad][8], are a plain bulk copy (cp.async.bulk) into a
//    four-stage ring.  One thread issues tcgen05.mma (M 128, N npad, K 16, kind::f16 BF16 x BF16 ->
//    F32) into a TMEM accumulator; four warps read it back with tcgen05.ld for the epilogue (bias,
//    ReLU, BF16 or F32 store).  The data gradient is the same kernel on the output gradient with the
//    weights flipped and transposed (k_nn_pack_w).
//  * Weight gradient (k_conv3_wgrad): D[(tap, ci)][co] = sum over voxels X[v + tap][ci] dY[v][co],
//    K = voxels.  The operands need voxels along the 16-byte rows, so the CTA transposes 8x8 blocks
//    of the TMA-loaded brick and output-gradient tile into K-major core matrices in shared memory
//    (one 128-byte core per thread step), then issues M 128 x N npad x K 16 MMAs; each CTA sums a
//    strided set of voxel tiles for a group of M tiles and a deterministic reduction sums the CTAs.
//
// Every wait (TMA, MMA completion) is bounded by wall time; on expiry the kernel raises a flag in
// device memory, skips its remaining work, frees its TMEM and returns, and later CTAs see the flag
// and return at once.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "pfm_internal.cuh"
#include "pfm_tma.cuh"

namespace pfm {
namespace nn {

constexpr int kThreads = 128;
constexpr int kTileD1 = 16, kTileD2 = 8;  // 128 output voxels per CTA
constexpr int kBoxD0 = 3, kBoxD1 = kTileD1 + 2, kBoxD2 = kTileD2 + 2;
constexpr int kBoxVox = kBoxD0 * kBoxD1 * kBoxD2;  // 540
constexpr int kChunkBytes = kBoxVox * 16;          // one 8-channel block of the brick: 8640 B
constexpr int kRowBytes = kBoxD2 * 16;             // one brick row along d2: 160 B
constexpr int kStages = 4;                         // weight ring depth
constexpr int kMaxCin = 128, kMaxNpad = 128;
constexpr int kSmPerGpuSmem = 233472;                  // shared memory per SM (228 KB)
constexpr int kMaxDynSmem = 232448 - 64;               // per-CTA limit (227 KB) less the static flag

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, M 128, BF16 inputs, F32 accumulator
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// arrives on `bar` once every tcgen05.mma this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}

// 16 consecutive 32-bit TMEM columns of this warp's 32 lanes (lane = thread)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor, no swizzle: start address, leading-dimension byte offset (the
// stride between core matrices along K) and stride-dimension byte offset (between 8-row groups
// along M or N), all in 16-byte units; bit 46 is the descriptor version of this architecture.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: F32 accumulator (bits 4-5 = 1), BF16 A and B (bits 7-9,
// 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

struct ConvFwdParams {
  int n0, n1, n2;
  int tiles2;          // tiles along d2 (8 voxels each); blockIdx.x = t1 * tiles2 + t2
  int cin, c1;         // input channels (x1 holds the first c1)
  int npad, cout;      // MMA N (multiple of 16) and real output channels
  int ncols;           // TMEM columns allocated
  int nstage;          // weight ring depth in taps (27: every tap's weights loaded up front)
  uint32_t idesc;
  const __nv_bfloat16* w;  // [27][cin/8][npad][8]
  const float* bias;       // [cout] or null
  int relu;
  __nv_bfloat16* y1;  // channel-blocked output, channels [0, cy1)
  int cy1;
  __nv_bfloat16* y2;  // channels [cy1, cout), or null
  float* yf;          // if set: f32 planar output [cout][n0][n1][n2] instead of y1/y2
  const float* yf_scale;  // device scalar multiplying yf (or null)
  int* err;
};

__global__ void __launch_bounds__(kThreads) k_conv3_fwd(const __grid_constant__ CUtensorMap tm1,
                                                        const __grid_constant__ CUtensorMap tm2,
                                                        const ConvFwdParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  __shared__ int s_skip;
  if (tid == 0) s_skip = *(volatile int*)p.err;
  __syncthreads();
  if (s_skip) return;  // an earlier CTA gave up: do nothing (uniform over the CTA)

  const int nchunk = p.cin >> 3;
  const uint32_t box_bytes = (uint32_t)nchunk * kChunkBytes;
  const uint32_t stage_bytes = (uint32_t)p.npad * p.cin * 2;
  unsigned char* box = smem;
  unsigned char* wring = smem + ((box_bytes + 127) & ~127u);
  const int ns = p.nstage;
  uint64_t* bars = (uint64_t*)(wring + ns * stage_bytes);
  uint64_t* box_bar = bars;
  uint64_t* full = bars + 1;
  uint64_t* done = bars + 1 + ns;
  uint64_t* final_bar = bars + 1 + 2 * ns;
  uint32_t* slot = (uint32_t*)(bars + 2 + 2 * ns);

  const int t1 = blockIdx.x / p.tiles2, t2 = blockIdx.x - t1 * p.tiles2;
  const int z = blockIdx.y, y0 = t1 * kTileD1, x0 = t2 * kTileD2;

  if (tid == 0) {
    mbar_init(box_bar, 1);
    for (int s = 0; s < ns; ++s) {
      mbar_init(full + s, 1);
      mbar_init(done + s, 1);
    }
    mbar_init(final_bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(slot, (uint32_t)p.ncols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;

  if (tid == 0) {
    bool ok = true;
    mbar_expect_tx(box_bar, box_bytes);
    tma_load_5d(box, &tm1, 0, x0 - 1, y0 - 1, z - 1, 0, box_bar);
    if (p.cin > p.c1) tma_load_5d(box + (size_t)(p.c1 >> 3) * kChunkBytes, &tm2, 0, x0 - 1, y0 - 1, z - 1, 0, box_bar);
    for (int t = 0; t < ns; ++t) {
      mbar_expect_tx(full + t, stage_bytes);
      bulk_load(wring + t * stage_bytes, (const unsigned char*)p.w + (size_t)t * stage_bytes, stage_bytes, full + t);
    }
    ok = mbar_wait(box_bar, 0, p.err, 1);
    const uint32_t box_addr = su32(box), ring_addr = su32(wring);
    const uint32_t blbo = (uint32_t)p.npad * 16;
    for (int t = 0; t < 27 && ok; ++t) {
      const int s = t % ns;
      ok = mbar_wait(full + s, (t / ns) & 1, p.err, 2);
      if (!ok) break;
      tc_fence_after();
      const int a = t / 9, b = (t / 3) % 3, c = t % 3;
      const uint32_t a0 = box_addr + (uint32_t)(((a * kBoxD1 + b) * kBoxD2 + c) * 16);
      const uint32_t b0 = ring_addr + (uint32_t)s * stage_bytes;
      for (int j = 0; j < (p.cin >> 4); ++j) {
        const uint64_t ad = smem_desc(a0 + (uint32_t)(2 * j) * kChunkBytes, kChunkBytes, kRowBytes);
        const uint64_t bd = smem_desc(b0 + (uint32_t)(2 * j) * blbo, blbo, 128);
        mma_bf16(tmem, ad, bd, p.idesc, (t | j) != 0);
      }
      mma_commit(done + s);
      // refill the stage the previous tap used once its MMAs have completed
      if (t >= 1 && t - 1 + ns < 27) {
        const int sp = (t - 1) % ns;
        ok = mbar_wait(done + sp, ((t - 1) / ns) & 1, p.err, 3);
        if (!ok) break;
        mbar_expect_tx(full + sp, stage_bytes);
        bulk_load(wring + sp * stage_bytes, (const unsigned char*)p.w + (size_t)(t - 1 + ns) * stage_bytes,
                  stage_bytes, full + sp);
      }
    }
    mma_commit(final_bar);
  }
  const bool fin = mbar_wait(final_bar, 0, p.err, 4);
  tc_fence_after();

  // epilogue: warp w holds TMEM lanes 32w..32w+31 = output voxels m = 32w + lane
  const int m = warp * 32 + lane;
  const int yy = y0 + (m >> 3), xx = x0 + (m & 7);
  const bool valid = fin && yy < p.n1 && xx < p.n2;
  const size_t V = (size_t)p.n0 * p.n1 * p.n2;
  const size_t vox = ((size_t)z * p.n1 + yy) * p.n2 + xx;
  const float scale = (p.yf && p.yf_scale) ? *p.yf_scale : 1.f;
  for (int c0 = 0; c0 < p.npad; c0 += 16) {
    float v[16];
    tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
    if (!valid) continue;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int nb = c0 + 8 * q;
      if (nb >= p.cout) break;
      float o[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        float r = v[8 * q + e];
        if (p.bias && nb + e < p.cout) r += p.bias[nb + e];
        if (p.relu) r = fmaxf(r, 0.f);
        o[e] = r;
      }
      if (p.yf) {
        for (int e = 0; e < 8 && nb + e < p.cout; ++e) p.yf[(size_t)(nb + e) * V + vox] = o[e] * scale;
      } else {
        uint4 pk;
        __nv_bfloat162 h0 = __floats2bfloat162_rn(o[0], o[1]), h1 = __floats2bfloat162_rn(o[2], o[3]);
        __nv_bfloat162 h2 = __floats2bfloat162_rn(o[4], o[5]), h3 = __floats2bfloat162_rn(o[6], o[7]);
        pk.x = *(uint32_t*)&h0;
        pk.y = *(uint32_t*)&h1;
        pk.z = *(uint32_t*)&h2;
        pk.w = *(uint32_t*)&h3;
        __nv_bfloat16* dst = nb < p.cy1 ? p.y1 + ((size_t)(nb >> 3) * V + vox) * 8
                                        : p.y2 + ((size_t)((nb - p.cy1) >> 3) * V + vox) * 8;
        *(uint4*)dst = pk;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, (uint32_t)p.ncols);
}

// ---------------------------------------------------------------------------------------------
// weight gradient

struct ConvWgradParams {
  int n0, n1, n2, tiles2, ntiles;  // voxel tiles of 1 x 16 x 8
  int cin, c1, cdy, npad;          // input channels, dY channels (multiple of 8), MMA N
  int mtiles, mt_per_cta;          // M tiles of 128 (tap, ci) rows; per CTA group (blockIdx.y)
  int nabuf;                       // operand buffers for A (2: staging overlaps the MMAs; 1: more CTAs per SM)
  int ncols;
  uint32_t idesc;
  float* partial;  // [gridDim.x][mtiles * 128][npad]
  int* err;
};

// 8x8 transpose of 16-bit elements: in[v] holds 8 channels of voxel v, out[e] 8 voxels of channel e
__device__ __forceinline__ void transpose8x8(const uint4 (&in)[8], uint4 (&out)[8]) {
  const uint32_t* w = reinterpret_cast<const uint32_t*>(in);  // w[v * 4 + e / 2]
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const uint32_t sel = (e & 1) ? 0x7632u : 0x5410u;
    uint32_t o[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = __byte_perm(w[(2 * q) * 4 + (e >> 1)], w[(2 * q + 1) * 4 + (e >> 1)], sel);
    out[e] = make_uint4(o[0], o[1], o[2], o[3]);
  }
}

__device__ __forceinline__ void copy_core_T(const unsigned char* src, unsigned char* dst) {
  uint4 in[8], out[8];
#pragma unroll
  for (int v = 0; v < 8; ++v) in[v] = *(const uint4*)(src + 16 * v);
  transpose8x8(in, out);
#pragma unroll
  for (int e = 0; e < 8; ++e) *(uint4*)(dst + 16 * e) = out[e];
}

constexpr int kCoresA = 16 * 16;           // 16 row groups x 16 voxel groups per M tile
constexpr int kAbufBytes = kCoresA * 128;  // 32 KB

constexpr int kWgThreads = 256;  // 8 warps stage the operand cores; warps 0-3 also drain TMEM

__global__ void __launch_bounds__(kWgThreads) k_conv3_wgrad(const __grid_constant__ CUtensorMap tm1,
                                                          const __grid_constant__ CUtensorMap tm2,
                                                          const __grid_constant__ CUtensorMap tmdy,
                                                          const ConvWgradParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  __shared__ int s_skip;
  if (tid == 0) s_skip = *(volatile int*)p.err;
  __syncthreads();
  if (s_skip) return;

  const int nchunk = p.cin >> 3, dchunk = p.cdy >> 3, ngrp = p.npad >> 3;
  const uint32_t box_bytes = (uint32_t)nchunk * kChunkBytes;
  const uint32_t dy_bytes = (uint32_t)dchunk * 2048;
  unsigned char* box = smem;
  unsigned char* dybox = box + ((box_bytes + 127) & ~127u);
  unsigned char* bcore = dybox + dy_bytes;           // [16 voxel groups][npad/8][128 B]
  unsigned char* abuf = bcore + (size_t)p.npad * 256;  // nabuf x [16 voxel groups][16 row groups][128 B]
  uint64_t* bars = (uint64_t*)(abuf + p.nabuf * kAbufBytes);
  uint64_t* box_bar = bars;
  uint64_t* done = bars + 1;  // [2], one per A buffer
  uint64_t* final_bar = bars + 3;
  uint32_t* slot = (uint32_t*)(bars + 4);

  const int mt0 = blockIdx.y * p.mt_per_cta;
  const int nmt = min(p.mt_per_cta, p.mtiles - mt0);

  if (tid == 0) {
    mbar_init(box_bar, 1);
    mbar_init(done, 1);
    mbar_init(done + 1, 1);
    mbar_init(final_bar, 1);
    fence_mbar_init();
  }
  // B groups beyond the dY channels stay zero
  for (int i = tid; i < p.npad * 16; i += blockDim.x) ((uint4*)bcore)[i] = make_uint4(0, 0, 0, 0);
  if (warp == 0) tmem_alloc(slot, (uint32_t)p.ncols);
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;

  bool ok = true;
  bool first = true;
  unsigned box_phase = 0;
  int uses[2] = {0, 0};
  int last = -1;  // A buffer of the last commit
  const uint32_t idesc = p.idesc;
  const uint32_t blbo = (uint32_t)ngrp * 128;
  for (int tile = blockIdx.x; tile < p.ntiles && ok; tile += gridDim.x) {
    const int pl = tile / ((p.n1 + kTileD1 - 1) / kTileD1 * p.tiles2);
    const int r = tile - pl * ((p.n1 + kTileD1 - 1) / kTileD1 * p.tiles2);
    const int t1 = r / p.tiles2, t2 = r - t1 * p.tiles2;
    const int z = pl, y0 = t1 * kTileD1, x0 = t2 * kTileD2;
    if (tid == 0) {
      fence_proxy_async();
      mbar_expect_tx(box_bar, box_bytes + dy_bytes);
      tma_load_5d(box, &tm1, 0, x0 - 1, y0 - 1, z - 1, 0, box_bar);
      if (p.cin > p.c1) tma_load_5d(box + (size_t)(p.c1 >> 3) * kChunkBytes, &tm2, 0, x0 - 1, y0 - 1, z - 1, 0, box_bar);
      tma_load_5d(dybox, &tmdy, 0, x0, y0, z, 0, box_bar);
    }
    bool w = mbar_wait(box_bar, box_phase, p.err, 11);
    box_phase ^= 1;
    // the previous tile's MMAs read bcore: wait for the last of them before restaging it
    if (w && last >= 0) w = mbar_wait(done + last, (uses[last] - 1) & 1, p.err, 12);
    ok = __syncthreads_and(w) != 0;  // every thread takes the same path through the barriers below
    if (!ok) break;
    for (int i = tid; i < dchunk * 16; i += blockDim.x) {  // B core (channel group g, voxel group k)
      const int g = i % dchunk, k = i / dchunk;
      copy_core_T(dybox + g * 2048 + k * 128, bcore + k * blbo + g * 128);
    }
    for (int mi = 0; mi < nmt && ok; ++mi) {
      const int buf = p.nabuf == 2 ? ((uses[0] + uses[1]) & 1) : 0;
      bool wb = true;
      if (uses[buf] > 0) wb = mbar_wait(done + buf, (uses[buf] - 1) & 1, p.err, 13);
      ok = __syncthreads_and(wb) != 0;
      if (!ok) break;
      unsigned char* A = abuf + buf * kAbufBytes;
      for (int i = tid; i < kCoresA; i += blockDim.x) {  // A core (row group g, voxel group k)
        const int g = i & 15, k = i >> 4;
        const int G = (mt0 + mi) * 16 + g;
        const int tap = G / nchunk, ch = G - tap * nchunk;
        unsigned char* dst = A + k * 2048 + g * 128;
        if (tap < 27) {
          const int a = tap / 9, b = (tap / 3) % 3, c = tap % 3;
          copy_core_T(box + (size_t)ch * kChunkBytes + ((a * kBoxD1 + k + b) * kBoxD2 + c) * 16, dst);
        } else {
#pragma unroll
          for (int e = 0; e < 8; ++e) *(uint4*)(dst + 16 * e) = make_uint4(0, 0, 0, 0);
        }
      }
      fence_proxy_async();
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      if (tid == 0) {
        const uint32_t a_addr = su32(A), b_addr = su32(bcore);
        for (int kk = 0; kk < 8; ++kk) {
          const uint64_t ad = smem_desc(a_addr + (uint32_t)(2 * kk) * 2048, 2048, 128);
          const uint64_t bd = smem_desc(b_addr + (uint32_t)(2 * kk) * blbo, blbo, 128);
          mma_bf16(tmem + (uint32_t)(mi * p.npad), ad, bd, idesc, !(first && kk == 0));
        }
        mma_commit(done + buf);
      }
      uses[buf]++;
      last = buf;
    }
    first = false;
    __syncthreads();  // the brick and dY tile are consumed: the next TMA may overwrite them
  }
  if (tid == 0) mma_commit(final_bar);
  const bool fin = mbar_wait(final_bar, 0, p.err, 14);
  tc_fence_after();

  const int rows = p.mtiles * 128;
  for (int mi = 0; mi < nmt && warp < 4; ++mi) {  // TMEM lanes 32w..32w+31 belong to warp w % 4
    for (int c0 = 0; c0 < p.npad; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(mi * p.npad + c0), v);
      if (!fin) continue;
      const int R = (mt0 + mi) * 128 + warp * 32 + lane;
      float* dst = p.partial + ((size_t)blockIdx.x * rows + R) * p.npad + c0;
#pragma unroll
      for (int e = 0; e < 16; e += 4)
        *(float4*)(dst + e) = first ? make_float4(0.f, 0.f, 0.f, 0.f) : make_float4(v[e], v[e + 1], v[e + 2], v[e + 3]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, (uint32_t)p.ncols);
}

// dW[co][ci][tap] = sum over splits of partial[split][tap * cin + ci][co] (fixed order)
__global__ void k_wgrad_reduce(const float* __restrict__ partial, int splits, int rows, int npad, int cin, int cout,
                               float* __restrict__ dw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int total = cout * cin * 27;
  if (i >= total) return;
  const int tap = i % 27, ci = (i / 27) % cin, co = i / (27 * cin);
  const size_t R = (size_t)tap * cin + ci;
  float s = 0.f;
  for (int k = 0; k < splits; ++k) s += partial[((size_t)k * rows + R) * npad + co];
  dw[i] = s;
}

// ---------------------------------------------------------------------------------------------
// weight packing, element-wise layers and the optimizer

// wp[t][kc][n][e] = W'[n][kc*8+e][t] with W' = W ([cout][cin][27]) or, for the data gradient,
// W'[n][ci'][t] = W[ci'][n][26 - t] (n over the layer's input channels, ci' over its outputs).
__global__ void k_pack_w(const float* __restrict__ W, int cout, int cin, int flip, int kin, int npad,
                         __nv_bfloat16* __restrict__ wp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int total = 27 * kin * npad;
  if (i >= total) return;
  const int e = i & 7, n = (i >> 3) % npad, kc = (i >> 3) / npad % (kin >> 3), t = (i >> 3) / npad / (kin >> 3);
  const int k = kc * 8 + e;
  float v = 0.f;
  if (!flip) {
    if (n < cout && k < cin) v = W[((size_t)n * cin + k) * 27 + t];
  } else {
    if (n < cin && k < cout) v = W[((size_t)k * cin + n) * 27 + (26 - t)];
  }
  wp[i] = __float2bfloat16_rn(v);
}

// x (16 channels): channel 0 = f * (*inv_scale), channels 1..15 = 0
__global__ void k_pack_scalar(const float* __restrict__ f, size_t V, const float* __restrict__ inv_scale,
                              __nv_bfloat16* __restrict__ x) {
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  const float s = inv_scale ? *inv_scale : 1.f;
  __nv_bfloat162 h0 = __floats2bfloat162_rn(f[v] * s, 0.f);
  uint4 a = make_uint4(*(uint32_t*)&h0, 0, 0, 0), z = make_uint4(0, 0, 0, 0);
  ((uint4*)x)[v] = a;
  ((uint4*)x)[V + v] = z;
}

__device__ __forceinline__ void unpack8(uint4 u, float (&f)[8]) {
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    float2 t = __bfloat1622float2(h[q]);
    f[2 * q] = t.x;
    f[2 * q + 1] = t.y;
  }
}

__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
  uint4 u;
  uint32_t* w = reinterpret_cast<uint32_t*>(&u);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * q], f[2 * q + 1]);
    w[q] = *(uint32_t*)&h;
  }
  return u;
}

// 2x2x2 average pool (mode 0), its backward (mode 1: dx[v] = dy[v / 2] / 8), nearest upsampling
// (mode 2: y[v] = x[v / 2]) and its backward (mode 3: dx[V] = sum of the 8 children), one
// 8-channel block of one fine voxel (modes 1, 2) or one coarse voxel (modes 0, 3) per thread.
__global__ void k_resample(const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out, int chunks, int n0,
                           int n1, int n2, int mode) {
  const int m0 = n0 >> 1, m1 = n1 >> 1, m2 = n2 >> 1;
  const size_t Vf = (size_t)n0 * n1 * n2, Vc = (size_t)m0 * m1 * m2;
  const bool coarse = (mode == 0 || mode == 3);
  const size_t per = coarse ? Vc : Vf;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per * chunks) return;
  const int ch = (int)(i / per);
  const size_t v = i - (size_t)ch * per;
  const uint4* src = (const uint4*)in;
  uint4* dst = (uint4*)out;
  if (coarse) {
    const int k = (int)(v % m2), j = (int)((v / m2) % m1), ii = (int)(v / ((size_t)m1 * m2));
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b)
        for (int c = 0; c < 2; ++c) {
          float f[8];
          unpack8(src[(size_t)ch * Vf + ((size_t)(2 * ii + a) * n1 + 2 * j + b) * n2 + 2 * k + c], f);
#pragma unroll
          for (int e = 0; e < 8; ++e) acc[e] += f[e];
        }
    if (mode == 0)
#pragma unroll
      for (int e = 0; e < 8; ++e) acc[e] *= 0.125f;
    dst[(size_t)ch * Vc + v] = pack8(acc);
  } else {
    const int k = (int)(v % n2), j = (int)((v / n2) % n1), ii = (int)(v / ((size_t)n1 * n2));
    uint4 u = src[(size_t)ch * Vc + ((size_t)(ii >> 1) * m1 + (j >> 1)) * m2 + (k >> 1)];
    if (mode == 1) {
      float f[8];
      unpack8(u, f);
#pragma unroll
      for (int e = 0; e < 8; ++e) f[e] *= 0.125f;
      u = pack8(f);
    }
    dst[(size_t)ch * Vf + v] = u;
  }
}

// g = g * (y > 0) (mode 0, the ReLU backward) or a = a + b (mode 1), on 8-channel blocks
__global__ void k_elementwise(__nv_bfloat16* __restrict__ g, const __nv_bfloat16* __restrict__ y, size_t n8,
                              int mode) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n8) return;
  float a[8], b[8];
  unpack8(((const uint4*)g)[i], a);
  unpack8(((const uint4*)y)[i], b);
#pragma unroll
  for (int e = 0; e < 8; ++e) a[e] = mode == 0 ? (b[e] > 0.f ? a[e] : 0.f) : a[e] + b[e];
  ((uint4*)g)[i] = pack8(a);
}

constexpr int kRedBlocks = 296;  // 2 x 148: fixed partition of the deterministic reductions
constexpr int kRedThreads = 256;

__device__ __forceinline__ float block_sum(float v, float* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// bias gradient partials: part[block][c] = sum over this block's voxels of dy channel c
__global__ void k_bias_grad_part(const __nv_bfloat16* __restrict__ dy, int chunks, size_t V, float* __restrict__ part) {
  __shared__ float sh[32];
  for (int ch = 0; ch < chunks; ++ch) {
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
      float f[8];
      unpack8(((const uint4*)dy)[(size_t)ch * V + v], f);
#pragma unroll
      for (int e = 0; e < 8; ++e) acc[e] += f[e];
    }
    for (int e = 0; e < 8; ++e) {
      const float s = block_sum(acc[e], sh);
      if (threadIdx.x == 0) part[(size_t)blockIdx.x * chunks * 8 + ch * 8 + e] = s;
    }
  }
}

// out[c] = sum over parts of part[p][c], fixed order
__global__ void k_sum_parts(const float* __restrict__ part, int parts, int width, int n, float* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  float s = 0.f;
  for (int k = 0; k < parts; ++k) s += part[(size_t)k * width + c];
  out[c] = s;
}

// partial sums of e = pred - target * (*inv_scale) and e^2; part[block] = (sum e, sum e^2)
__global__ void k_loss_part(const float* __restrict__ pred, const float* __restrict__ target,
                            const float* __restrict__ inv_scale, size_t V, float* __restrict__ part) {
  __shared__ float sh[32];
  const float s = inv_scale ? *inv_scale : 1.f;
  float a = 0.f, b = 0.f;
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
    const float e = (pred ? pred[v] : 0.f) - target[v] * s;
    a += e;
    b += e * e;
  }
  a = block_sum(a, sh);
  b = block_sum(b, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

// the loss of a pressure guess up to a constant: out = {L, mean e, 1 / rms e, rms e} with
// L = mean(e^2) - mean(e)^2 (with pred = null, e = -target: out[2] is the inverse RMS of the
// target, the scale of a right-hand side); k_loss_grad writes dL/dpred = 2 (e - mean e) / V as
// channel 0 of a 16-channel block tensor.
__global__ void k_loss_final(const float* __restrict__ part, int parts, size_t V, float* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double a = 0.0, b = 0.0;
  for (int k = 0; k < parts; ++k) {
    a += part[2 * k];
    b += part[2 * k + 1];
  }
  const double me = a / (double)V, mse = b / (double)V;
  out[0] = (float)(mse - me * me);
  out[1] = (float)me;
  out[2] = (float)(mse > 0 ? 1.0 / sqrt(mse) : 1.0);
  out[3] = (float)(mse > 0 ? sqrt(mse) : 1.0);
}

__global__ void k_loss_grad(const float* __restrict__ pred, const float* __restrict__ target,
                            const float* __restrict__ inv_scale, const float* __restrict__ stats, size_t V,
                            __nv_bfloat16* __restrict__ g) {
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  const float s = inv_scale ? *inv_scale : 1.f;
  const float e = pred[v] - target[v] * s - stats[1];
  __nv_bfloat162 h0 = __floats2bfloat162_rn(2.f * e / (float)V, 0.f);
  ((uint4*)g)[v] = make_uint4(*(uint32_t*)&h0, 0, 0, 0);
  ((uint4*)g)[V + v] = make_uint4(0, 0, 0, 0);
}

// Adam (Kingma and Ba, 2015) on f32 master parameters, gradient scaled by gscale
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       size_t n, float lr, float b1, float b2, float eps, float c1, float c2, float gscale) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i] * gscale;
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// ---------------------------------------------------------------------------------------------
// host side

// tensor map of a channel-blocked bf16 tensor: dims (8, n2, n1, n0, C/8), box (8, b2, b1, b0, C/8)
bool make_map(CUtensorMap* tm, const void* base, int C, int n0, int n1, int n2, int b0, int b1, int b2) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[5] = {8, (cuuint64_t)n2, (cuuint64_t)n1, (cuuint64_t)n0, (cuuint64_t)(C / 8)};
  const cuuint64_t strides[4] = {16, (cuuint64_t)n2 * 16, (cuuint64_t)n1 * n2 * 16, (cuuint64_t)n0 * n1 * n2 * 16};
  const cuuint32_t box[5] = {8, (cuuint32_t)b2, (cuuint32_t)b1, (cuuint32_t)b0, (cuuint32_t)(C / 8)};
  const cuuint32_t es[5] = {1, 1, 1, 1, 1};
  return fn(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int pow2_cols(int n) {
  int c = 32;
  while (c < n) c <<= 1;
  return c;
}

// dynamic shared memory that also keeps resident CTAs x TMEM columns within the SM's 512 columns:
// at most k = 512 / ncols CTAs may share an SM, so k + 1 CTAs (each with 1 KB reserved) must not fit
size_t occupancy_smem(size_t need, int ncols) {
  const size_t k = 512 / (size_t)ncols;
  const size_t floor_bytes = (size_t)kSmPerGpuSmem / (k + 1) - 1024 + 1;
  return need > floor_bytes ? need : floor_bytes;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace nn
}  // namespace pfm

using namespace pfm::nn;

static int grid_ok(int n0, int n1, int n2) {
  return n0 > 0 && n1 > 0 && n2 > 0 && (long long)n0 * n1 * n2 < (1ll << 31);
}

extern "C" int pfm_nn_conv3(const pfm_conv3_args* a, void* stream) {
  if (!a || !a->x1 || !a->w || !a->err || (!a->y1 && !a->yf)) return PFM_ERR_NULL;
  if (!grid_ok(a->d0, a->d1, a->d2)) return PFM_ERR_SHAPE;
  const int cin = a->c1 + a->c2;
  if (a->c1 <= 0 || a->c1 % 16 || a->c2 < 0 || a->c2 % 16 || cin > kMaxCin || (a->c2 > 0 && !a->x2)) return PFM_ERR_SHAPE;
  if (a->cout <= 0 || a->cout > kMaxNpad) return PFM_ERR_SHAPE;
  const int npad = (a->cout + 15) / 16 * 16;
  if (!a->yf) {
    if (a->cout % 8 || a->cy1 <= 0 || a->cy1 % 8 || a->cy1 > a->cout || (a->cy1 < a->cout && !a->y2))
      return PFM_ERR_SHAPE;
  }
  if (!aligned16(a->x1) || (a->x2 && !aligned16(a->x2)) || !aligned16(a->w) || (a->y1 && !aligned16(a->y1)) ||
      (a->y2 && !aligned16(a->y2)))
    return PFM_ERR_ARG;
  CUtensorMap tm1, tm2;
  if (!make_map(&tm1, a->x1, a->c1, a->d0, a->d1, a->d2, kBoxD0, kBoxD1, kBoxD2)) return PFM_ERR_CUDA;
  if (a->c2 > 0) {
    if (!make_map(&tm2, a->x2, a->c2, a->d0, a->d1, a->d2, kBoxD0, kBoxD1, kBoxD2)) return PFM_ERR_CUDA;
  } else {
    tm2 = tm1;
  }
  ConvFwdParams p{};
  p.n0 = a->d0;
  p.n1 = a->d1;
  p.n2 = a->d2;
  p.tiles2 = (a->d2 + kTileD2 - 1) / kTileD2;
  const int tiles1 = (a->d1 + kTileD1 - 1) / kTileD1;
  p.cin = cin;
  p.c1 = a->c1;
  p.npad = npad;
  p.cout = a->cout;
  p.ncols = pow2_cols(npad);
  p.idesc = idesc_bf16(128, npad);
  p.w = (const __nv_bfloat16*)a->w;
  p.bias = a->bias;
  p.relu = a->relu;
  p.y1 = (__nv_bfloat16*)a->y1;
  p.cy1 = a->yf ? a->cout : a->cy1;
  p.y2 = (__nv_bfloat16*)a->y2;
  p.yf = a->yf;
  p.yf_scale = a->yf_scale;
  p.err = a->err;
  const size_t box = ((size_t)(cin / 8) * kChunkBytes + 127) & ~(size_t)127;
  // weight ring of 4 taps: deeper rings (up to all 27 taps) remove refill round trips but cost
  // shared memory, hence CTAs per SM, and concurrent CTAs are what keeps the tensor core busy
  const size_t stage = (size_t)npad * cin * 2;
  p.nstage = kStages;
  const size_t need = 1024 + box + (size_t)p.nstage * stage + 8 * (2 + 2 * p.nstage) + 16;
  const size_t smem = occupancy_smem(need, p.ncols);
  if (smem > kMaxDynSmem) return PFM_ERR_SHAPE;
  static std::atomic<unsigned long long> attr{0};  // above the default 48 KB: opt in per device
  if (pfm::opt_in_smem(k_conv3_fwd, kMaxDynSmem, attr) != cudaSuccess) return PFM_ERR_CUDA;
  dim3 grid((unsigned)(tiles1 * p.tiles2), (unsigned)a->d0);
  if (grid.y > 65535) return PFM_ERR_SHAPE;
  k_conv3_fwd<<<grid, kThreads, smem, (cudaStream_t)stream>>>(tm1, tm2, p);
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}

extern "C" int pfm_nn_wgrad_workspace(const pfm_conv3_wgrad_args* a, size_t* bytes) {
  if (!a || !bytes) return PFM_ERR_NULL;
  const int cin = a->c1 + a->c2;
  const int npad = (a->cdy + 15) / 16 * 16;
  const int mtiles = (27 * cin + 127) / 128;
  const int mt_per = std::min(mtiles, std::max(1, 256 / std::max(npad, 16)));
  const int gy = (mtiles + mt_per - 1) / mt_per;
  const long long ntiles = (long long)a->d0 * ((a->d1 + kTileD1 - 1) / kTileD1) * ((a->d2 + kTileD2 - 1) / kTileD2);
  const long long gx = std::min<long long>(ntiles, std::max(1, (4 * 148 + gy - 1) / gy));
  *bytes = (size_t)gx * mtiles * 128 * npad * sizeof(float);
  return PFM_OK;
}

extern "C" int pfm_nn_conv3_wgrad(const pfm_conv3_wgrad_args* a, void* stream) {
  if (!a || !a->x1 || !a->dy || !a->dw || !a->partial || !a->err) return PFM_ERR_NULL;
  if (!grid_ok(a->d0, a->d1, a->d2)) return PFM_ERR_SHAPE;
  const int cin = a->c1 + a->c2;
  if (a->c1 <= 0 || a->c1 % 16 || a->c2 < 0 || a->c2 % 16 || cin > kMaxCin || (a->c2 > 0 && !a->x2)) return PFM_ERR_SHAPE;
  if (a->cdy <= 0 || a->cdy % 8 || a->cdy > kMaxNpad || a->cout <= 0 || a->cout > a->cdy) return PFM_ERR_SHAPE;
  if (!aligned16(a->x1) || (a->x2 && !aligned16(a->x2)) || !aligned16(a->dy) || !aligned16(a->partial))
    return PFM_ERR_ARG;
  const int npad = (a->cdy + 15) / 16 * 16;
  CUtensorMap tm1, tm2, tmdy;
  if (!make_map(&tm1, a->x1, a->c1, a->d0, a->d1, a->d2, kBoxD0, kBoxD1, kBoxD2)) return PFM_ERR_CUDA;
  if (a->c2 > 0) {
    if (!make_map(&tm2, a->x2, a->c2, a->d0, a->d1, a->d2, kBoxD0, kBoxD1, kBoxD2)) return PFM_ERR_CUDA;
  } else {
    tm2 = tm1;
  }
  if (!make_map(&tmdy, a->dy, a->cdy, a->d0, a->d1, a->d2, 1, kTileD1, kTileD2)) return PFM_ERR_CUDA;
  ConvWgradParams p{};
  p.n0 = a->d0;
  p.n1 = a->d1;
  p.n2 = a->d2;
  p.tiles2 = (a->d2 + kTileD2 - 1) / kTileD2;
  p.ntiles = a->d0 * ((a->d1 + kTileD1 - 1) / kTileD1) * p.tiles2;
  p.cin = cin;
  p.c1 = a->c1;
  p.cdy = a->cdy;
  p.npad = npad;
  p.mtiles = (27 * cin + 127) / 128;
  p.mt_per_cta = std::min(p.mtiles, std::max(1, 256 / npad));
  p.ncols = pow2_cols(p.mt_per_cta * npad);
  p.idesc = idesc_bf16(128, npad);
  p.partial = a->partial;
  p.err = a->err;
  const int gy = (p.mtiles + p.mt_per_cta - 1) / p.mt_per_cta;
  const int gx = std::min(p.ntiles, std::max(1, (4 * 148 + gy - 1) / gy));
  size_t ws = 0;
  pfm_nn_wgrad_workspace(a, &ws);
  if (a->partial_bytes < ws) return PFM_ERR_WORKSPACE;
  const size_t box = ((size_t)(cin / 8) * kChunkBytes + 127) & ~(size_t)127;
  const size_t base = 1024 + box + (size_t)(a->cdy / 8) * 2048 + (size_t)npad * 256 + 8 * 4 + 16;
  // one A buffer when that lets two CTAs share an SM (their stagings then overlap each other)
  p.nabuf = (2 * (base + 2 * kAbufBytes + 1024) > (size_t)kSmPerGpuSmem && 2 * (base + kAbufBytes + 1024) <= (size_t)kSmPerGpuSmem) ? 1 : 2;
  const size_t need = base + (size_t)p.nabuf * kAbufBytes;
  const size_t smem = occupancy_smem(need, p.ncols);
  if (smem > kMaxDynSmem) return PFM_ERR_SHAPE;
  static std::atomic<unsigned long long> attr{0};  // above the default 48 KB: opt in per device
  if (pfm::opt_in_smem(k_conv3_wgrad, kMaxDynSmem, attr) != cudaSuccess) return PFM_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  k_conv3_wgrad<<<dim3((unsigned)gx, (unsigned)gy), kWgThreads, smem, st>>>(tm1, tm2, tmdy, p);
  const int total = a->cout * cin * 27;
  k_wgrad_reduce<<<(total + 255) / 256, 256, 0, st>>>(a->partial, gx, p.mtiles * 128, npad, cin, a->cout, a->dw);
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}

extern "C" int pfm_nn_pack_weights(const float* W, int cout, int cin, int flip, int kin, int npad, void* wp,
                                   void* stream) {
  if (!W || !wp) return PFM_ERR_NULL;
  if (cout <= 0 || cin <= 0 || kin % 16 || npad % 16 || npad <= 0 || kin <= 0) return PFM_ERR_SHAPE;
  if (!flip && (kin < cin || npad < cout)) return PFM_ERR_SHAPE;
  if (flip && (kin < cout || npad < cin)) return PFM_ERR_SHAPE;
  const int total = 27 * kin * npad;
  k_pack_w<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(W, cout, cin, flip, kin, npad, (__nv_bfloat16*)wp);
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}

extern "C" int pfm_nn_pack_scalar(const float* f, int d0, int d1, int d2, const float* inv_scale, void* x,
                                  void* stream) {
  if (!f || !x) return PFM_ERR_NULL;
  if (!grid_ok(d0, d1, d2)) return PFM_ERR_SHAPE;
  const size_t V = (size_t)d0 * d1 * d2;
  k_pack_scalar<<<(unsigned)((V + 255) / 256), 256, 0, (cudaStream_t)stream>>>(f, V, inv_scale, (__nv_bfloat16*)x);
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}

extern "C" int pfm_nn_resample(const void* in, void* out, int channels, int d0, int d1, int d2, int mode,
                               void* stream) {
  if (!in || !out) return PFM_ERR_NULL;
  if (!grid_ok(d0, d1, d2) || d0 % 2 || d1 % 2 || d2 % 2 || channels <= 0 || channels % 8 || mode < 0 || mode > 3)
    return PFM_ERR_SHAPE;
  const size_t Vf = (size_t)d0 * d1 * d2;
  const size_t per = (mode == 0 || mode == 3) ? Vf / 8 : Vf;
  const size_t n = per * (channels / 8);
  k_resample<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)in, (__nv_bfloat16*)out, channels / 8, d0, d1, d2, mode);
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}

extern "C" int pfm_nn_elementwise(void* g, const void* y, size_t elements, int mode, void* stream) {
  if (!g || !y) return PFM_ERR_NULL;
  if (elements % 8 || (mode != 0 && mode != 1)) return PFM_ERR_SHAPE;
  const size_t n8 = elements / 8;
  if (n8 == 0) return PFM_OK;
  k_elementwise<<<(unsigned)((n8 + 255) / 256), 256, 0, (cudaStream_t)stream>>>((__nv_bfloat16*)g,
                                                                                 (const __nv_bfloat16*)y, n8, mode);
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}

extern "C" size_t pfm_nn_scratch_floats(int channels) {
  return (size_t)kRedBlocks * (size_t)(channels > 2 ? channels : 2);
}

extern "C" int pfm_nn_bias_grad(const void* dy, int channels, int d0, int d1, int d2, int cout, float* db,
                                float* scratch, void* stream) {
  if (!dy || !db || !scratch) return PFM_ERR_NULL;
  if (!grid_ok(d0, d1, d2) || channels <= 0 || channels % 8 || cout <= 0 || cout > channels) return PFM_ERR_SHAPE;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t V = (size_t)d0 * d1 * d2;
  k_bias_grad_part<<<kRedBlocks, kRedThreads, 0, st>>>((const __nv_bfloat16*)dy, channels / 8, V, scratch);
  k_sum_parts<<<(cout + 127) / 128, 128, 0, st>>>(scratch, kRedBlocks, channels, cout, db);
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}

extern "C" int pfm_nn_loss(const float* pred, const float* target, const float* inv_scale, int d0, int d1, int d2,
                           float* out4, void* grad, float* scratch, void* stream) {
  if (!target || !out4 || !scratch || (grad && !pred)) return PFM_ERR_NULL;
  if (!grid_ok(d0, d1, d2)) return PFM_ERR_SHAPE;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t V = (size_t)d0 * d1 * d2;
  k_loss_part<<<kRedBlocks, kRedThreads, 0, st>>>(pred, target, inv_scale, V, scratch);
  k_loss_final<<<1, 32, 0, st>>>(scratch, kRedBlocks, V, out4);
  if (grad)
    k_loss_grad<<<(unsigned)((V + 255) / 256), 256, 0, st>>>(pred, target, inv_scale, out4, V, (__nv_bfloat16*)grad);
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}

extern "C" int pfm_nn_adam(float* p, const float* g, float* m, float* v, size_t n, float lr, float beta1, float beta2,
                           float eps, int step, float gscale, void* stream) {
  if (!p || !g || !m || !v) return PFM_ERR_NULL;
  if (step < 1 || n == 0) return PFM_ERR_ARG;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  k_adam<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr, beta1, beta2, eps, c1, c2,
                                                                         gscale);
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}
