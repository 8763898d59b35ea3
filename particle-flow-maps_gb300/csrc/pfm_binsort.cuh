// Per-bin ordering of the particle binning (get_particles_id_in_every_cell, 3D/run_3D.py:342-351):
// after the counting sort scatters each particle into its bin at the slot an atomic handed it,
// every bin is put in ascending particle index, so the permutation equals a stable CPU sort of the
// cell keys.  Shared by the workspace path (pfm_p2g.cu) and the allocation-free path
// (pfm_noalloc.cu).
//
//  * bins of at most 16 entries: one thread, entries loaded into registers, bitonic network;
//  * larger bins: k_bin_sort_big, a whole thread block per bin (each block scans 1024 cells and
//    sorts the large bins among them one after another), a bitonic network over the bin padded to a power of
//    two with virtual +inf entries.  The network is the form in which every comparator moves the
//    smaller value to the lower index (stage k: mirror comparator i <-> i ^ (k - 1), then
//    half-cleaners at strides k/4 .. 1), so a comparator that touches a virtual entry never moves
//    anything and the padding needs no storage.  Strides below kBigChunk run in shared memory on
//    chunks of the bin, larger strides directly on the bin in global memory with a block barrier
//    between passes.  Work O(n log^2 n) per bin with all of a block's threads on it: a bin of 2^21
//    entries takes milliseconds, not the O(n^2) dependent steps of an insertion sort.
#pragma once

#include <climits>
#include <stdint.h>

namespace pfm {
namespace {  // each translation unit that sorts bins gets its own copy of the kernels

constexpr int kBigThreads = 1024;  // block of k_bin_sort_big: the cells one block scans
constexpr int kBigChunk = 8192;    // entries of a bin sorted in shared memory at once (32 KB)
constexpr int kSmallBin = 16;      // bins up to this size are sorted by one thread

// Bins of at most N entries: all loads issued together into registers (INT_MAX past the end), a
// bitonic sorting network, and the first n values stored back.  The entries are distinct particle
// indices, so the result is the ascending order whatever the network.
template <int N>
__device__ __forceinline__ void sort_bin_small(int* __restrict__ order, int b, int n) {
  int v[N];
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = i < n ? order[b + i] : INT_MAX;
#pragma unroll
  for (int k = 2; k <= N; k <<= 1)
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const int l = i ^ j;
        if (l > i) {
          const int lo = min(v[i], v[l]), hi = max(v[i], v[l]);
          const bool up = (i & k) == 0;
          v[i] = up ? lo : hi;
          v[l] = up ? hi : lo;
        }
      }
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (i < n) order[b + i] = v[i];
}

// One thread's share of a bin of up to kSmallBin entries (larger bins are left to k_bin_sort_big).
__device__ __forceinline__ void sort_bin_by_thread(int* __restrict__ order, int b, int n) {
  if (n <= 1) return;
  if (n <= 8)
    sort_bin_small<8>(order, b, n);
  else if (n <= kSmallBin)
    sort_bin_small<16>(order, b, n);
}

// Comparator p of a pass over `m` (power of two) positions: stage size k, stride j; j == k/2 is the
// mirror pass of the stage.  Returns the pair (i, l), i < l.
__device__ __forceinline__ void pass_pair(int p, int k, int j, int& i, int& l) {
  if (j == (k >> 1)) {
    const int kb = p / j, t = p - kb * j;
    i = kb * k + t;
    l = kb * k + (k - 1 - t);
  } else {
    const int jb = p / j, t = p - jb * j;
    i = jb * 2 * j + t;
    l = i + j;
  }
}

// Passes with strides from j0 down to 1 of stage k (j0 == k/2 starts with the mirror pass) on a
// shared-memory chunk of S entries (S a power of two, virtual +inf already stored as INT_MAX).
__device__ __forceinline__ void smem_passes(int* s, int S, int k, int j0) {
  for (int j = j0; j >= 1; j >>= 1) {
    for (int p = threadIdx.x; p < S / 2; p += blockDim.x) {
      int i, l;
      pass_pair(p, k, j, i, l);
      int x = s[i], y = s[l];
      if (x > y) {
        s[i] = y;
        s[l] = x;
      }
    }
    __syncthreads();
  }
}

// Loads a[c0 .. c0 + S) (INT_MAX past n) into s, or stores the real part back.
__device__ __forceinline__ void chunk_load(const int* a, int n, int c0, int S, int* s) {
  for (int t = threadIdx.x; t < S; t += blockDim.x) s[t] = c0 + t < n ? a[c0 + t] : INT_MAX;
  __syncthreads();
}

__device__ __forceinline__ void chunk_store(int* a, int n, int c0, int S, const int* s) {
  for (int t = threadIdx.x; t < S && c0 + t < n; t += blockDim.x) a[c0 + t] = s[t];
  __syncthreads();
}

// The whole block sorts a[0 .. n) ascending (n > 1); s is kBigChunk ints of shared memory.
__device__ void block_sort_bin(int* a, int n, int* s) {
  int64_t m = 1;
  while (m < n) m <<= 1;
  const int S = m < kBigChunk ? (int)m : kBigChunk;
  // stages up to the chunk size, chunk by chunk in shared memory
  for (int c0 = 0; c0 < n; c0 += S) {
    chunk_load(a, n, c0, S, s);
    for (int k = 2; k <= S; k <<= 1) smem_passes(s, S, k, k >> 1);
    chunk_store(a, n, c0, S, s);
  }
  // larger stages: global passes down to the chunk size, then the rest of the stage per chunk
  // (64-bit comparator indices: m reaches 2^31 for bins of more than 2^30 entries)
  for (int64_t k = 2 * (int64_t)S; k <= m; k <<= 1) {
    for (int64_t j = k >> 1; j >= S; j >>= 1) {
      for (int64_t p = threadIdx.x; p < m / 2; p += blockDim.x) {
        int64_t i, l;
        if (j == (k >> 1)) {
          const int64_t kb = p / j, t = p - kb * j;
          i = kb * k + t;
          l = kb * k + (k - 1 - t);
        } else {
          const int64_t jb = p / j, t = p - jb * j;
          i = jb * 2 * j + t;
          l = i + j;
        }
        if (l < n) {
          int x = a[i], y = a[l];
          if (x > y) {
            a[i] = y;
            a[l] = x;
          }
        }
      }
      __syncthreads();
    }
    for (int c0 = 0; c0 < n; c0 += S) {
      chunk_load(a, n, c0, S, s);
      smem_passes(s, S, 2 * S, S >> 1);  // half-cleaners only: the stage size does not enter them
      chunk_store(a, n, c0, S, s);
    }
  }
}

// Every bin of more than kSmallBin entries, one block per bin: block b scans cells
// [b * kBigThreads, (b + 1) * kBigThreads) and sorts the large ones it found.  start has C + 1
// entries (bin c = order[start[c] .. start[c + 1])).
__global__ void __launch_bounds__(kBigThreads) k_bin_sort_big(const int* __restrict__ start, int64_t C,
                                                             int* order) {
  __shared__ int s_chunk[kBigChunk];
  __shared__ int s_list[kBigThreads];
  __shared__ int s_n;
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  const int64_t c = (int64_t)blockIdx.x * kBigThreads + threadIdx.x;
  if (c < C && start[c + 1] - start[c] > kSmallBin) s_list[atomicAdd(&s_n, 1)] = (int)(c - (int64_t)blockIdx.x * kBigThreads);
  __syncthreads();
  const int nb = s_n;
  for (int t = 0; t < nb; ++t) {
    const int64_t cc = (int64_t)blockIdx.x * kBigThreads + s_list[t];
    const int b = start[cc], e = start[cc + 1];
    block_sort_bin(order + b, e - b, s_chunk);
  }
}

}  // namespace
}  // namespace pfm
