// Sumcheck-side kernel templates of the WHIR prover path (instantiated in sumcheck.cu for the
// Goldilocks family and in sumcheck_mont.cu for Field192/Field256):
//   sumcheck round polynomial (c0, c2) and the in-place fold, fused as fold-then-compute
//     (reference src/algebra/sumcheck.rs:12-111, protocols/sumcheck.rs:104-155)
//   eq-weight accumulation (multilinear.rs:170-190, linear_form/multilinear_extension.rs:38-40)
//   geometric accumulation of STIR / OOD constraints (algebra/mod.rs:154-177)
//   base -> extension lift and vector RLC (algebra/mod.rs:51-98)
//   univariate (Horner) evaluation for out-of-domain samples (algebra/mod.rs:105-129)
// Every value is an exact field element, so the reduction order inside the kernels does not
// change any output bit relative to the reference's rayon split order.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "bulk.cuh"
#include "field.cuh"
#include "kernels.hpp"
#include "roots.cuh"
#include "wide.cuh"

namespace whir {

static constexpr int SC_THREADS = 256;
static constexpr size_t SC_MAX_BLOCKS = 152 * 8;

template <class T>
__device__ __forceinline__ T shfl_down_t(const T& x, int d) {
  T r;
  const uint64_t* src = reinterpret_cast<const uint64_t*>(&x);
  uint64_t* dst = reinterpret_cast<uint64_t*>(&r);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(T) / 8); ++i) dst[i] = __shfl_down_sync(0xffffffffu, src[i], d);
  return r;
}

template <class T>
__device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) x = x + shfl_down_t(x, d);
  return x;
}

// Block-wide sum; the result is valid in thread 0.
template <class T>
__device__ T block_sum(T x) {
  __shared__ T part[32];
  x = warp_sum(x);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) part[warp] = x;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  x = (threadIdx.x < nw) ? part[threadIdx.x] : T::zero();
  if (warp == 0) x = warp_sum(x);
  __syncthreads();
  return x;
}

// Two block-wide sums in one pass (one pair of barriers); the results are valid in thread 0.
template <class T>
__device__ void block_sum2(T& a, T& b) {
  __shared__ T part[2][32];
  a = warp_sum(a);
  b = warp_sum(b);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    part[0][warp] = a;
    part[1][warp] = b;
  }
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  a = (threadIdx.x < nw) ? part[0][threadIdx.x] : T::zero();
  b = (threadIdx.x < nw) ? part[1][threadIdx.x] : T::zero();
  if (warp == 0) {
    a = warp_sum(a);
    b = warp_sum(b);
  }
  __syncthreads();
}

template <class T>
__device__ __forceinline__ T ldcg_t(const T* p) {
  T r;
  const unsigned long long* s = reinterpret_cast<const unsigned long long*>(p);
  unsigned long long* d = reinterpret_cast<unsigned long long*>(&r);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(T) / 8); ++i) d[i] = __ldcg(s + i);
  return r;
}

// Publishes a round message written to out[0..2): bumps the launch sequence counter[1] and stores it
// in the word after out[1] once the values are visible system-wide. `out` may be host-mapped
// memory, which the host polls instead of copying and synchronising the stream.
template <class T>
__device__ __forceinline__ void publish_pair(T* out, unsigned int* counter) {
  const unsigned int seq = counter[1] + 1;
  counter[1] = seq;
  __threadfence_system();
  *reinterpret_cast<volatile unsigned int*>(out + 2) = seq;
}

// Sums the block's per-thread (c0, c2) accumulators and stores the block partial. With a counter,
// the last block to finish also sums all partials into out[0..2), re-arms counter[0] and publishes
// the pair (publish_pair), so one launch yields the round message. A one-block launch writes out
// directly.
template <class T>
__device__ void finish_pairs(T acc0, T acc2, T* partials, T* out, unsigned int* counter) {
  block_sum2(acc0, acc2);
  __shared__ bool am_last;
  if (gridDim.x == 1) {
    if (threadIdx.x == 0) {
      partials[0] = acc0;
      partials[1] = acc2;
      if (out) {
        out[0] = acc0;
        out[1] = acc2;
        if (counter) publish_pair(out, counter);
      }
    }
    return;
  }
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = acc0;
    partials[2 * blockIdx.x + 1] = acc2;
    am_last = false;
    if (counter) {
      __threadfence();
      am_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  T s0 = T::zero(), s2 = T::zero();
  for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
    s0 += ldcg_t(partials + 2 * i);
    s2 += ldcg_t(partials + 2 * i + 1);
  }
  block_sum2(s0, s2);
  if (threadIdx.x == 0) {
    out[0] = s0;
    out[1] = s2;
    counter[0] = 0;
    publish_pair(out, counter);
  }
}

template <class T>
__global__ void __launch_bounds__(SC_THREADS) sc_compute_kernel(const T* a, const T* b, uint64_t n, T* partials,
                                                                 T* out, unsigned int* counter) {
  WideAcc<T> w0, w2;
  w0.init();
  w2.init();
  if (n == 1) {
    if (blockIdx.x == 0 && threadIdx.x == 0) w0.mac(a[0], b[0]);
  } else {
    const uint64_t h = n >> 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < h; i += (uint64_t)gridDim.x * blockDim.x) {
      const T a0 = a[i], a1 = a[i + h], b0 = b[i], b1 = b[i + h];
      w0.mac(a0, b0);
      w2.mac(a1 - a0, b1 - b0);
    }
  }
  T acc0 = w0.get(), acc2 = w2.get();
  finish_pairs(acc0, acc2, partials, out, counter);
}

template <class T>
__global__ void __launch_bounds__(SC_THREADS) sc_fold_compute_kernel(T* a, T* b, uint64_t n, T r, T* partials,
                                                                      T* out, unsigned int* counter) {
  WideAcc<T> w0, w2;
  w0.init();
  w2.init();
  if (n <= 2) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (n == 2) {
        const T fa = a[0] + (a[1] - a[0]) * r, fb = b[0] + (b[1] - b[0]) * r;
        a[0] = fa;
        b[0] = fb;
        w0.mac(fa, fb);
      } else if (n == 1) {
        w0.mac(a[0], b[0]);
      }
    }
  } else {
    const uint64_t q = n >> 2, h = n >> 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < q; i += (uint64_t)gridDim.x * blockDim.x) {
      const T a0 = a[i], a1 = a[i + q], a2 = a[i + h], a3 = a[i + h + q];
      const T b0 = b[i], b1 = b[i + q], b2 = b[i + h], b3 = b[i + h + q];
      const T fa0 = a0 + (a2 - a0) * r, fa1 = a1 + (a3 - a1) * r;
      const T fb0 = b0 + (b2 - b0) * r, fb1 = b1 + (b3 - b1) * r;
      a[i] = fa0;
      a[i + q] = fa1;
      b[i] = fb0;
      b[i + q] = fb1;
      w0.mac(fa0, fb0);
      w2.mac(fa1 - fa0, fb1 - fb0);
    }
  }
  T acc0 = w0.get(), acc2 = w2.get();
  finish_pairs(acc0, acc2, partials, out, counter);
}

// Raises a kernel's dynamic shared-memory limit to `bytes` once per device (the flags and results
// belong to the caller's instantiation).
static constexpr int SC_MAX_DEVICES = 64;
template <class K>
static cudaError_t sc_smem_attr_once(K kernel, size_t bytes, std::once_flag* flags, cudaError_t* results) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= SC_MAX_DEVICES)
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  std::call_once(flags[dev], [&] {
    results[dev] = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  });
  return results[dev];
}

// Large rounds (n >= SC_BULK_MIN) with the operands staged by the bulk-copy engine. A tile is
// SC_THREADS consecutive items i (pairs (i, i + h) of a round without fold, quads
// (i, i + q, i + h, i + h + q) of a fold-and-compute round); its segments of a and b (4 KiB each for
// 16-byte elements) go through two shared-memory stages filled by cp.async.bulk against per-stage
// mbarriers, so the next tile's loads are in flight while this tile is folded and accumulated, with
// no registers held for them. CTAs take tiles t = blockIdx.x + k gridDim.x. Waits are bounded as in
// the tensor sums; a timeout sets the context's sticky device error word (counter[3]), which the
// next host-mapped publication reports, and the CTA stops reading.
static constexpr uint64_t SC_BULK_MIN = 1ull << 18;
static constexpr int SC_BULK_NST = 2;

template <class T, bool FOLD>
__global__ void __launch_bounds__(SC_THREADS, 2) sc_round_bulk_kernel(T* a, T* b, uint64_t n, T r, T* partials,
                                                                      T* out, unsigned int* counter) {
  constexpr int NSEG = FOLD ? 8 : 4;
  constexpr uint32_t SEG = SC_THREADS * sizeof(T), STAGE = NSEG * SEG;
  extern __shared__ __align__(128) unsigned char rb_smem[];
  __shared__ __align__(8) uint64_t bar[SC_BULK_NST];
  __shared__ int aborted;
  const uint64_t h = n >> 1, q = n >> 2, items = FOLD ? q : h;
  const uint64_t tiles = items / SC_THREADS;
  const int ntile = (int)((tiles - blockIdx.x + gridDim.x - 1) / gridDim.x);  // tiles of this CTA
  if (threadIdx.x == 0) {
    aborted = 0;
    for (int st = 0; st < SC_BULK_NST; ++st) mbar_init(&bar[st], 1);
    mbar_init_fence();
  }
  __syncthreads();
  // segment k of tile t starts at element off[k] + t * SC_THREADS of a (k < NSEG / 2) or b
  auto issue = [&](int k) {
    const int st = k % SC_BULK_NST;
    const uint64_t i0 = (blockIdx.x + (uint64_t)k * gridDim.x) * SC_THREADS;
    unsigned char* dst = rb_smem + (size_t)st * STAGE;
    mbar_arrive_expect_tx(&bar[st], STAGE);
#pragma unroll
    for (int sg = 0; sg < NSEG; ++sg) {
      const T* base = sg < NSEG / 2 ? a : b;
      const int part = sg % (NSEG / 2);
      const uint64_t off = FOLD ? ((part & 1) ? q : 0) + ((part & 2) ? h : 0) : (part ? h : 0);
      bulk_copy_g2s(dst + sg * SEG, base + off + i0, SEG, &bar[st]);
    }
  };
  if (threadIdx.x == 0)
    for (int k = 0; k < ntile && k < SC_BULK_NST; ++k) issue(k);
  WideAcc<T> w0, w2;
  w0.init();
  w2.init();
  int k = 0;
  for (; k < ntile; ++k) {
    const int st = k % SC_BULK_NST;
    if (mbar_wait(&bar[st], (uint32_t)(k / SC_BULK_NST) & 1)) {
      const T* v = reinterpret_cast<const T*>(rb_smem + (size_t)st * STAGE) + threadIdx.x;
      const uint64_t i = (blockIdx.x + (uint64_t)k * gridDim.x) * SC_THREADS + threadIdx.x;
      if constexpr (FOLD) {
        const T a0 = v[0], a1 = v[SC_THREADS], a2 = v[2 * SC_THREADS], a3 = v[3 * SC_THREADS];
        const T b0 = v[4 * SC_THREADS], b1 = v[5 * SC_THREADS], b2 = v[6 * SC_THREADS], b3 = v[7 * SC_THREADS];
        const T fa0 = a0 + (a2 - a0) * r, fa1 = a1 + (a3 - a1) * r;
        const T fb0 = b0 + (b2 - b0) * r, fb1 = b1 + (b3 - b1) * r;
        a[i] = fa0;
        a[i + q] = fa1;
        b[i] = fb0;
        b[i + q] = fb1;
        w0.mac(fa0, fb0);
        w2.mac(fa1 - fa0, fb1 - fb0);
      } else {
        const T a0 = v[0], a1 = v[SC_THREADS], b0 = v[2 * SC_THREADS], b1 = v[3 * SC_THREADS];
        w0.mac(a0, b0);
        w2.mac(a1 - a0, b1 - b0);
      }
    } else {
      aborted = 1;
    }
    __syncthreads();
    if (aborted) break;
    if (threadIdx.x == 0 && k + SC_BULK_NST < ntile) {
      fence_proxy_async_smem();
      issue(k + SC_BULK_NST);
    }
  }
  if (aborted && threadIdx.x == 0) {
    atomicExch(counter + 3, 1u);
    for (int j = k; j < ntile && j < k + SC_BULK_NST; ++j) mbar_wait(&bar[j % SC_BULK_NST], (uint32_t)(j / SC_BULK_NST) & 1);
  }
  T acc0 = w0.get(), acc2 = w2.get();
  finish_pairs(acc0, acc2, partials, out, counter);
}

template <class T, bool FOLD>
static cudaError_t run_round_bulk(T* a, T* b, size_t n, T r, T* partials, size_t* nparts, cudaStream_t s, T* out,
                                  unsigned int* counter) {
  static std::once_flag flags[SC_MAX_DEVICES];
  static cudaError_t results[SC_MAX_DEVICES];
  constexpr size_t smem = (size_t)SC_BULK_NST * (FOLD ? 8 : 4) * SC_THREADS * sizeof(T);
  cudaError_t e = sc_smem_attr_once(sc_round_bulk_kernel<T, FOLD>, smem, flags, results);
  if (e != cudaSuccess) return e;
  // Two resident CTAs per SM; tiles split evenly (a CTA with one tile more than the others would set
  // the time). The partials area holds SC_MAX_BLOCKS pairs.
  static const size_t slots = [] {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
        cudaSuccess || sms < 1)
      sms = 152;
    return (size_t)std::min<size_t>(2 * (size_t)sms, SC_MAX_BLOCKS);
  }();
  const uint64_t tiles = (FOLD ? n / 4 : n / 2) / SC_THREADS;
  const uint64_t per = (tiles + slots - 1) / slots;
  const size_t g = (size_t)std::max<uint64_t>(1, (tiles + per - 1) / per);
  sc_round_bulk_kernel<T, FOLD><<<(unsigned)g, SC_THREADS, smem, s>>>(a, b, n, r, partials, out, counter);
  note_launch();
  *nparts = g;
  return cudaGetLastError();
}

// The bulk-staged round takes power-of-two n >= SC_BULK_MIN and 16-byte aligned vectors.
template <class T>
static bool round_bulk_ok(const T* a, const T* b, size_t n) {
  // (segments of SC_THREADS elements and offsets that are multiples of SC_THREADS elements keep every
  // copy 16-byte aligned for 8-, 16-, 24- and 32-byte elements)
  return n >= SC_BULK_MIN && (n & (n - 1)) == 0 && sizeof(T) % 8 == 0 && sizeof(T) <= 32 &&
         reinterpret_cast<uintptr_t>(a) % 16 == 0 && reinterpret_cast<uintptr_t>(b) % 16 == 0;
}

// Rounds on vectors of at most SC_SMALL elements run in one warp: no shared memory, no barriers, no
// cross-block partials and little code to fetch. These launches are latency-bound: event-timed on a
// GB300, a fold-and-compute round at n = 16 takes 8.1 us this way against 12.6 us with the
// 256-thread kernel above (empty launch: 4.1 us); from n = 1024 on, several blocks are faster.
static constexpr uint64_t SC_SMALL = 512;
template <class T>
__global__ void __launch_bounds__(32) sc_small_kernel(T* a, T* b, uint64_t n, T r, int fold, T* partials, T* out,
                                                      unsigned int* counter) {
  const int lane = threadIdx.x;
  WideAcc<T> w0, w2;
  w0.init();
  w2.init();
  if (fold) {
    if (n <= 2) {
      if (lane == 0) {
        if (n == 2) {
          const T fa = a[0] + (a[1] - a[0]) * r, fb = b[0] + (b[1] - b[0]) * r;
          a[0] = fa;
          b[0] = fb;
          w0.mac(fa, fb);
        } else if (n == 1) {
          w0.mac(a[0], b[0]);
        }
      }
    } else {
      const uint64_t q = n >> 2, h = n >> 1;
#pragma unroll 1
      for (uint64_t i = lane; i < q; i += 32) {
        const T a0 = a[i], a1 = a[i + q], a2 = a[i + h], a3 = a[i + h + q];
        const T b0 = b[i], b1 = b[i + q], b2 = b[i + h], b3 = b[i + h + q];
        const T fa0 = a0 + (a2 - a0) * r, fa1 = a1 + (a3 - a1) * r;
        const T fb0 = b0 + (b2 - b0) * r, fb1 = b1 + (b3 - b1) * r;
        a[i] = fa0;
        a[i + q] = fa1;
        b[i] = fb0;
        b[i + q] = fb1;
        w0.mac(fa0, fb0);
        w2.mac(fa1 - fa0, fb1 - fb0);
      }
    }
  } else if (n == 1) {
    if (lane == 0) w0.mac(a[0], b[0]);
  } else {
    const uint64_t h = n >> 1;
#pragma unroll 1
    for (uint64_t i = lane; i < h; i += 32) {
      const T a0 = a[i], a1 = a[i + h], b0 = b[i], b1 = b[i + h];
      w0.mac(a0, b0);
      w2.mac(a1 - a0, b1 - b0);
    }
  }
  T acc0 = w0.get(), acc2 = w2.get();
#pragma unroll 1
  for (int d = 16; d > 0; d >>= 1) {
    acc0 = acc0 + shfl_down_t(acc0, d);
    acc2 = acc2 + shfl_down_t(acc2, d);
  }
  if (lane == 0) {
    if (partials) {
      partials[0] = acc0;
      partials[1] = acc2;
    }
    if (out) {
      out[0] = acc0;
      out[1] = acc2;
      if (counter) publish_pair(out, counter);
    }
  }
}

template <class T>
__global__ void __launch_bounds__(SC_THREADS) sc_fold_kernel(T* v, uint64_t n, T r) {
  const uint64_t h = n >> 1;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < h; i += (uint64_t)gridDim.x * blockDim.x) {
    const T lo = v[i], hi = v[i + h];
    v[i] = lo + (hi - lo) * r;
  }
}

template <class T>
__global__ void __launch_bounds__(SC_THREADS) sc_fold2_kernel(T* v, T* w, uint64_t n, T r) {
  const uint64_t h = n >> 1;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < h; i += (uint64_t)gridDim.x * blockDim.x) {
    const T vlo = v[i], vhi = v[i + h], wlo = w[i], whi = w[i + h];
    v[i] = vlo + (vhi - vlo) * r;
    w[i] = wlo + (whi - wlo) * r;
  }
}

template <class T>
__global__ void __launch_bounds__(SC_THREADS) reduce_pairs_kernel(const T* partials, uint64_t nparts, T* out) {
  T s0 = T::zero(), s2 = T::zero();
  for (uint64_t i = threadIdx.x; i < nparts; i += blockDim.x) {
    s0 += partials[2 * i];
    s2 += partials[2 * i + 1];
  }
  s0 = block_sum(s0);
  s2 = block_sum(s2);
  if (threadIdx.x == 0) {
    out[0] = s0;
    out[1] = s2;
  }
}

template <class T>
__global__ void __launch_bounds__(SC_THREADS) reduce_singles_kernel(const T* partials, uint64_t nparts, T* out) {
  T s = T::zero();
  for (uint64_t i = threadIdx.x; i < nparts; i += blockDim.x) s += partials[i];
  s = block_sum(s);
  if (threadIdx.x == 0) out[0] = s;
}

template <class T>
cudaError_t launch_sumcheck_compute(const T* a, const T* b, size_t n, T* partials, size_t* nparts, cudaStream_t s,
                                    T* out, unsigned int* counter) {
  if (n <= SC_SMALL) {
    sc_small_kernel<T><<<1, 32, 0, s>>>(const_cast<T*>(a), const_cast<T*>(b), n, T::zero(), 0, partials, out,
                                       counter);
    note_launch();
    *nparts = 1;
    return cudaGetLastError();
  }
  if (round_bulk_ok(a, b, n))
    return run_round_bulk<T, false>(const_cast<T*>(a), const_cast<T*>(b), n, T::zero(), partials, nparts, s, out,
                                    counter);
  size_t g = sumcheck_partials(n);
  sc_compute_kernel<T><<<(unsigned)g, SC_THREADS, 0, s>>>(a, b, n, partials, out, counter);
  note_launch();
  *nparts = g;
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_fold_compute(T* a, T* b, size_t n, T r, T* partials, size_t* nparts, cudaStream_t s, T* out,
                                unsigned int* counter) {
  if (n <= SC_SMALL) {
    sc_small_kernel<T><<<1, 32, 0, s>>>(a, b, n, r, 1, partials, out, counter);
    note_launch();
    *nparts = 1;
    return cudaGetLastError();
  }
  if (round_bulk_ok(a, b, n)) return run_round_bulk<T, true>(a, b, n, r, partials, nparts, s, out, counter);
  size_t g = sumcheck_partials(n);
  sc_fold_compute_kernel<T><<<(unsigned)g, SC_THREADS, 0, s>>>(a, b, n, r, partials, out, counter);
  note_launch();
  *nparts = g;
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_fold(T* v, size_t n, T r, cudaStream_t s) {
  if (n <= 1) return cudaSuccess;
  size_t g = std::min(SC_MAX_BLOCKS, (n / 2 + SC_THREADS - 1) / SC_THREADS);
  sc_fold_kernel<T><<<(unsigned)g, SC_THREADS, 0, s>>>(v, n, r);
  note_launch();
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_fold2(T* v, T* w, size_t n, T r, cudaStream_t s) {
  if (n <= 1) return cudaSuccess;
  size_t g = std::min(SC_MAX_BLOCKS, (n / 2 + SC_THREADS - 1) / SC_THREADS);
  sc_fold2_kernel<T><<<(unsigned)g, SC_THREADS, 0, s>>>(v, w, n, r);
  note_launch();
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_reduce_pairs(const T* partials, size_t nparts, T* out, cudaStream_t s) {
  reduce_pairs_kernel<T><<<1, SC_THREADS, 0, s>>>(partials, nparts, out);
  note_launch();
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_reduce_singles(const T* partials, size_t nparts, T* out, cudaStream_t s) {
  reduce_singles_kernel<T><<<1, SC_THREADS, 0, s>>>(partials, nparts, out);
  note_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// eq weights: acc[i] += hi[i >> l] * lo[i & (2^l - 1)], hi = scalar * eq(point[0..h)),
// lo = eq(point[h..nv)).
// ---------------------------------------------------------------------------------------------
template <class T>
__global__ void eq_table_kernel(const T* point, int off, int cnt, T scalar, T* table) {
  const uint64_t size = 1ull << cnt;
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < size; e += (uint64_t)gridDim.x * blockDim.x) {
    T v = scalar;
    for (int k = 0; k < cnt; ++k) {
      const T x = point[off + k];
      const bool bit = (e >> (cnt - 1 - k)) & 1;
      v = v * (bit ? x : (T::one() - x));
    }
    table[e] = v;
  }
}

template <class T>
__global__ void __launch_bounds__(SC_THREADS) eq_accumulate_kernel(T* acc, uint64_t n, const T* hi, const T* lo, int l) {
  const uint64_t mask = (1ull << l) - 1;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    acc[i] += hi[i >> l] * lo[i & mask];
}

template <class T>
cudaError_t launch_eval_eq(T* acc, const T* point, int nv, T scalar, T* tables, cudaStream_t s) {
  const int h = nv / 2, l = nv - h;
  T* hi = tables;
  T* lo = tables + (1ull << h);
  eq_table_kernel<T><<<(unsigned)std::max<size_t>(1, ((1ull << h) + 255) / 256), 256, 0, s>>>(point, 0, h, scalar, hi);
  note_launch();
  eq_table_kernel<T><<<(unsigned)std::max<size_t>(1, ((1ull << l) + 255) / 256), 256, 0, s>>>(point, h, l, T::one(), lo);
  note_launch();
  const uint64_t n = 1ull << nv;
  size_t g = std::min<size_t>(SC_MAX_BLOCKS * 2, (n + SC_THREADS - 1) / SC_THREADS);
  eq_accumulate_kernel<T><<<(unsigned)g, SC_THREADS, 0, s>>>(acc, n, hi, lo, l);
  note_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Geometric accumulation: acc[i] += sum_j s_j x_j^i. CTA covers GA_E * blockDim consecutive
// indices; thread t handles i = base + t + u * blockDim (u < GA_E) so every access is coalesced.
// Per point: p = s_j x_j^(base + t) then p *= x_j^blockDim per step.
// ---------------------------------------------------------------------------------------------
static constexpr int GA_E = 16;
static constexpr int GA_THREADS = 256;
static constexpr int GA_CHUNK = 64;  // points staged in shared memory at a time

template <class T>
__global__ void __launch_bounds__(GA_THREADS) geometric_kernel(T* acc, uint64_t n, const T* scalars, const T* points,
                                                               uint64_t m) {
  __shared__ T sA[GA_CHUNK];  // s_j * x_j^base
  __shared__ T sB[GA_CHUNK];  // x_j^blockDim
  __shared__ T sX[GA_CHUNK];  // x_j
  const uint64_t base = (uint64_t)blockIdx.x * GA_THREADS * GA_E;
  T accu[GA_E];
#pragma unroll
  for (int u = 0; u < GA_E; ++u) accu[u] = T::zero();
  for (uint64_t j0 = 0; j0 < m; j0 += GA_CHUNK) {
    const int cnt = (int)std::min<uint64_t>(GA_CHUNK, m - j0);
    __syncthreads();
    if (threadIdx.x < cnt) {
      const T x = points[j0 + threadIdx.x];
      sX[threadIdx.x] = x;
      sA[threadIdx.x] = scalars[j0 + threadIdx.x] * x.pow(base);
      sB[threadIdx.x] = x.pow(GA_THREADS);
    }
    __syncthreads();
    for (int j = 0; j < cnt; ++j) {
      T p = sA[j] * sX[j].pow(threadIdx.x);
      const T stepv = sB[j];
#pragma unroll
      for (int u = 0; u < GA_E; ++u) {
        accu[u] += p;
        p = p * stepv;
      }
    }
  }
#pragma unroll
  for (int u = 0; u < GA_E; ++u) {
    const uint64_t i = base + threadIdx.x + (uint64_t)u * GA_THREADS;
    if (i < n) acc[i] += accu[u];
  }
}

template <class T>
cudaError_t launch_geometric_accumulate(T* acc, size_t n, const T* scalars, const T* points, size_t m, cudaStream_t s) {
  if (m == 0 || n == 0) return cudaSuccess;
  const size_t per = (size_t)GA_THREADS * GA_E;
  geometric_kernel<T><<<(unsigned)((n + per - 1) / per), GA_THREADS, 0, s>>>(acc, n, scalars, points, m);
  note_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Geometric accumulation over in-domain points x_j = w_N^(e_j): thread t of a CTA covers
// i = base + t + u * blockDim (u < E); p = s_j w_N^(e_j i) starts from the root tables and is
// advanced by w_N^(e_j blockDim) (a base-field multiplier) for each u.
// ---------------------------------------------------------------------------------------------
static constexpr int GR_THREADS = 256;
static constexpr int GR_CHUNK = 256;

template <class T, int E>
__global__ void __launch_bounds__(GR_THREADS) geometric_roots_kernel(T* acc, uint64_t n, const T* scalars,
                                                                     const uint64_t* exps, uint64_t m, int logN,
                                                                     RootTab rt) {
  typedef typename T::Base B;
  __shared__ T sS[GR_CHUNK];
  __shared__ uint64_t sE[GR_CHUNK];
  __shared__ B sStep[GR_CHUNK];
  const uint64_t mask = (1ull << logN) - 1;
  const uint64_t base = (uint64_t)blockIdx.x * GR_THREADS * E;
  const uint64_t i0 = base + threadIdx.x;
  T accu[E];
#pragma unroll
  for (int u = 0; u < E; ++u) accu[u] = T::zero();
  for (uint64_t j0 = 0; j0 < m; j0 += GR_CHUNK) {
    const int cnt = (int)min((uint64_t)GR_CHUNK, m - j0);
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
      sS[k] = scalars[j0 + k];
      const uint64_t e = exps[j0 + k] & mask;
      sE[k] = e;
      sStep[k] = root_pow<B>(rt, logN, (e * GR_THREADS) & mask);
    }
    __syncthreads();
    if constexpr (E == 1) {
      // One index per thread: unreduced accumulation, with the root-table reads of 8 queries issued
      // together (they are independent, and their latency dominates this loop).
      WideAcc<T> w;
      w.init();
      int j = 0;
      for (; j + 8 <= cnt; j += 8) {
        B r[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) r[k] = root_pow<B>(rt, logN, (sE[j + k] * i0) & mask);
#pragma unroll
        for (int k = 0; k < 8; ++k) w.mac_mixed(sS[j + k], r[k]);
      }
      for (; j < cnt; ++j) w.mac_mixed(sS[j], root_pow<B>(rt, logN, (sE[j] * i0) & mask));
      accu[0] += w.get();
    } else {
      for (int j = 0; j < cnt; ++j) {
        T p = sS[j].mul_base(root_pow<B>(rt, logN, (sE[j] * i0) & mask));
        const B step = sStep[j];
#pragma unroll
        for (int u = 0; u < E; ++u) {
          accu[u] += p;
          if (u + 1 < E) p = p.mul_base(step);
        }
      }
    }
  }
#pragma unroll
  for (int u = 0; u < E; ++u) {
    const uint64_t i = i0 + (uint64_t)u * GR_THREADS;
    if (i < n) acc[i] += accu[u];
  }
}

// Split form (see geometric_split_plan): thread t of a CTA takes entry t mod 2^te_log of its tile
// and every (256 >> te_log)-th query of its group's slice; the subgroups' sums meet in shared
// memory, then either in acc directly (one group) or through the partials and the tile's last CTA.
template <class T>
__global__ void __launch_bounds__(GR_THREADS) geometric_roots_split_kernel(T* acc, uint64_t n, const T* scalars,
                                                                           const uint64_t* exps, uint64_t m,
                                                                           int logN, RootTab rt, int te_log,
                                                                           int groups, T* partials,
                                                                           unsigned int* counters) {
  typedef typename T::Base B;
  __shared__ T red[GR_THREADS];
  __shared__ bool am_last;
  const int te = 1 << te_log, sg = GR_THREADS >> te_log;
  const uint64_t tile = blockIdx.x / groups;
  const int g = (int)(blockIdx.x - tile * groups);
  const int e = threadIdx.x & (te - 1), sub = threadIdx.x >> te_log;
  const uint64_t i = (tile << te_log) + e;
  const uint64_t mask = (1ull << logN) - 1;
  const uint64_t q0 = m * g / groups, q1 = m * (g + 1) / groups;
  WideAcc<T> w;
  w.init();
  if (i < n) {
    uint64_t j = q0 + sub;
    // eight root-table reads issued together (their latency dominates)
    for (; j + 7 * (uint64_t)sg < q1; j += 8 * (uint64_t)sg) {
      B r[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) r[k] = root_pow<B>(rt, logN, (exps[j + k * sg] * i) & mask);
#pragma unroll
      for (int k = 0; k < 8; ++k) w.mac_mixed(scalars[j + k * sg], r[k]);
    }
    for (; j < q1; j += sg) w.mac_mixed(scalars[j], root_pow<B>(rt, logN, (exps[j] * i) & mask));
  }
  T v = w.get();
  if (sg > 1) {
    red[threadIdx.x] = v;
    __syncthreads();
    if (sub == 0)
      for (int t = 1; t < sg; ++t) v += red[threadIdx.x + (t << te_log)];
  }
  if (groups == 1) {
    if (sub == 0 && i < n) acc[i] += v;
    return;
  }
  if (sub == 0 && i < n) partials[(uint64_t)g * n + i] = v;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = atomicAdd(counters + tile, 1u) == (unsigned)groups - 1;
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  if (sub == 0 && i < n) {
    T t = acc[i];
    for (int gg = 0; gg < groups; ++gg) t += ldcg_t(partials + (uint64_t)gg * n + i);
    acc[i] = t;
  }
  if (threadIdx.x == 0) counters[tile] = 0;
}

template <class T>
cudaError_t launch_geometric_roots(T* acc, size_t n, const T* scalars, const uint64_t* exps, size_t m, int logN,
                                   RootTab rt, cudaStream_t s, T* partials, unsigned int* counters) {
  if (n == 0 || m == 0) return cudaSuccess;
  if (logN > rt.log_order) return cudaErrorInvalidValue;
  const GeometricSplit sp = geometric_split_plan(n, m, partials != nullptr && counters != nullptr);
  if (sp.split) {
    const size_t tiles = (n + ((size_t)1 << sp.te_log) - 1) >> sp.te_log;
    geometric_roots_split_kernel<T><<<(unsigned)(tiles * sp.groups), GR_THREADS, 0, s>>>(
        acc, n, scalars, exps, m, logN, rt, sp.te_log, sp.groups, partials, counters);
    note_launch();
    return cudaGetLastError();
  }
  int E = 1;
  while (E < 8 && n / ((size_t)GR_THREADS * E * 2) >= 304) E *= 2;
  const size_t per = (size_t)GR_THREADS * E;
  const unsigned grid = (unsigned)((n + per - 1) / per);
  switch (E) {
    case 1: geometric_roots_kernel<T, 1><<<grid, GR_THREADS, 0, s>>>(acc, n, scalars, exps, m, logN, rt); break;
    case 2: geometric_roots_kernel<T, 2><<<grid, GR_THREADS, 0, s>>>(acc, n, scalars, exps, m, logN, rt); break;
    case 4: geometric_roots_kernel<T, 4><<<grid, GR_THREADS, 0, s>>>(acc, n, scalars, exps, m, logN, rt); break;
    default: geometric_roots_kernel<T, 8><<<grid, GR_THREADS, 0, s>>>(acc, n, scalars, exps, m, logN, rt); break;
  }
  note_launch();
  return cudaGetLastError();
}

template <class T>
__global__ void scatter_kernel(T* dense, const uint64_t* idx, const T* vals, uint64_t m) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x)
    dense[idx[k]] = vals[k];
}
template <class T>
cudaError_t launch_scatter(T* dense, const uint64_t* idx, const T* vals, size_t m, cudaStream_t s) {
  if (!m) return cudaSuccess;
  scatter_kernel<T><<<(unsigned)((m + 255) / 256), 256, 0, s>>>(dense, idx, vals, m);
  note_launch();
  return cudaGetLastError();
}

template <class T>
__global__ void add_kernel(T* acc, const T* src, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    acc[i] += src[i];
}
template <class T>
cudaError_t launch_add(T* acc, const T* src, size_t n, cudaStream_t s) {
  if (!n) return cudaSuccess;
  size_t g = std::min<size_t>(SC_MAX_BLOCKS * 2, (n + SC_THREADS - 1) / SC_THREADS);
  add_kernel<T><<<(unsigned)g, SC_THREADS, 0, s>>>(acc, src, n);
  note_launch();
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_eq_table(const T* point, int off, int cnt, T scalar, T* table, cudaStream_t s) {
  eq_table_kernel<T><<<(unsigned)std::max<size_t>(1, ((1ull << cnt) + 255) / 256), 256, 0, s>>>(point, off, cnt,
                                                                                               scalar, table);
  note_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Fused first sumcheck rounds: a = map(x) and b = sum_l rlc_l eq(point_l, .) are evaluated on the
// fly from the coefficient vector and small eq tables instead of being written to HBM.
// ---------------------------------------------------------------------------------------------
// With eq(i) = sum_f hi_f[i >> l] lo_f[i & (2^l - 1)] and the folded (top) variables inside the hi
// index, every sum of the first two rounds factors into per-row sums of lo-weighted coefficients
// times one hi-side factor per row (R = 2^(h-1) rows in the half with top bit 0):
//   round 1: c0 = sum_H sum_f hi_f[H] * S_f(H, x),
//            c2 = sum_H sum_f (hi_f[H + R] - hi_f[H]) * S_f(H, x_top - x),   S_f(H, y) = sum_j lo_f[j] y[H 2^l + j];
//   round 2: the folded covector is b'(H 2^l + j) = sum_f lo_f[j] (hi_f[H] + r (hi_f[H + R] - hi_f[H])).
// Each coefficient then costs one product per form instead of two eq products and a fold. Work is
// split in units of (row, chunk of EQ_CHUNK columns); each thread multiplies its own partial row sums
// by the row factor (linearity), so no per-row block reduction is needed.
static constexpr uint64_t EQ_CHUNK = 2048;
static constexpr int EQ_MAX_FORMS = 16;
static constexpr int EQ_UNROLL = (int)(EQ_CHUNK / SC_THREADS);  // chunk elements per thread

template <class T, class S>
__global__ void __launch_bounds__(SC_THREADS) first_compute_eq_kernel(const S* x, uint64_t n, const T* tables,
                                                                      int nforms, int h, int l, T* partials,
                                                                      T* out, unsigned int* counter) {
  const uint64_t hs = 1ull << h, ls = 1ull << l, rows = hs >> 1, half = n >> 1;
  const uint64_t chunk = ls < EQ_CHUNK ? ls : EQ_CHUNK, per_row = ls / chunk, units = rows * per_row;
  T acc0 = T::zero(), acc2 = T::zero();
  for (uint64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const uint64_t H = u / per_row, j0 = (u - H * per_row) * chunk, base = H * ls;
    for (int f = 0; f < nforms; ++f) {
      const T* hi = tables + (uint64_t)f * (hs + ls);
      const T* lo = hi + hs;
      WideAcc<T> s0, s2;
      s0.init();
      s2.init();
      for (uint64_t j = j0 + threadIdx.x; j < j0 + chunk; j += blockDim.x) {
        const S x0 = x[base + j], x1 = x[base + half + j];
        const T w = lo[j];
        s0.mac_mixed(w, x0);
        s2.mac_mixed(w, x1 - x0);
      }
      const T h0 = hi[H];
      acc0 += h0 * s0.get();
      acc2 += (hi[H + rows] - h0) * s2.get();
    }
  }
  finish_pairs(acc0, acc2, partials, out, counter);
}

// Round 2 by rows (h >= 2, nforms <= EQ_MAX_FORMS): folds x and the covector with r into a_out /
// b_out (n/2 each) and computes (c0, c2) of the folded pair; rows H < R/2 pair with rows H + R/2
// (the second variable is the second bit of the hi index).
template <class T, class S>
__global__ void __launch_bounds__(SC_THREADS) first_fold_compute_rows_kernel(const S* x, uint64_t n, T r,
                                                                            const T* tables, int nforms, int h,
                                                                            int l, T* a_out, T* b_out,
                                                                            T* partials, T* out,
                                                                            unsigned int* counter) {
  __shared__ T rowf[2][EQ_MAX_FORMS];
  const uint64_t hs = 1ull << h, ls = 1ull << l, rows = hs >> 1, qr = hs >> 2;
  const uint64_t q = n >> 2, hf = n >> 1;
  const uint64_t chunk = ls < EQ_CHUNK ? ls : EQ_CHUNK, per_row = ls / chunk, units = qr * per_row;
  WideAcc<T> w0, w2;
  w0.init();
  w2.init();
  for (uint64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const uint64_t H = u / per_row, j0 = (u - H * per_row) * chunk, base = H * ls;
    __syncthreads();  // the previous unit's readers are done with rowf
    if (threadIdx.x < 2 * nforms) {
      const int f = threadIdx.x >> 1, side = threadIdx.x & 1;
      const T* hi = tables + (uint64_t)f * (hs + ls);
      const uint64_t R0 = H + side * qr;
      rowf[side][f] = hi[R0] + r * (hi[R0 + rows] - hi[R0]);
    }
    __syncthreads();
    for (uint64_t j = j0 + threadIdx.x; j < j0 + chunk; j += blockDim.x) {
      const uint64_t i = base + j;
      const S x0 = x[i], x1 = x[i + q], x2 = x[i + hf], x3 = x[i + hf + q];
      const T fa0 = Embed<T, S>::map(x0) + Embed<T, S>::mul(r, x2 - x0);
      const T fa1 = Embed<T, S>::map(x1) + Embed<T, S>::mul(r, x3 - x1);
      T fb0 = T::zero(), fb1 = T::zero();
      for (int f = 0; f < nforms; ++f) {
        const T w = tables[(uint64_t)f * (hs + ls) + hs + j];
        fb0 += w * rowf[0][f];
        fb1 += w * rowf[1][f];
      }
      a_out[i] = fa0;
      a_out[i + q] = fa1;
      b_out[i] = fb0;
      b_out[i + q] = fb1;
      w0.mac(fa0, fb0);
      w2.mac(fa1 - fa0, fb1 - fb0);
    }
  }
  T acc0 = w0.get(), acc2 = w2.get();
  finish_pairs(acc0, acc2, partials, out, counter);
}

// eq evaluated at one index (round 2 for small shapes or many forms, and the MLE dot product).
template <class T>
__device__ __forceinline__ T eq_on_the_fly(const T* tables, int nforms, int h, int l, uint64_t i) {
  const uint64_t hs = 1ull << h, ls = 1ull << l;
  T v = T::zero();
  for (int f = 0; f < nforms; ++f) {
    const T* hi = tables + (uint64_t)f * (hs + ls);
    v += hi[i >> l] * hi[hs + (i & (ls - 1))];
  }
  return v;
}

template <class T, class S>
__global__ void __launch_bounds__(SC_THREADS) first_fold_compute_eq_kernel(const S* x, uint64_t n, T r,
                                                                           const T* tables, int nforms, int h, int l,
                                                                           T* a_out, T* b_out, T* partials, T* out,
                                                                           unsigned int* counter) {
  WideAcc<T> w0, w2;
  w0.init();
  w2.init();
  const uint64_t q = n >> 2, hf = n >> 1;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < q; i += (uint64_t)gridDim.x * blockDim.x) {
    const S x0 = x[i], x1 = x[i + q], x2 = x[i + hf], x3 = x[i + hf + q];
    const T fa0 = Embed<T, S>::map(x0) + Embed<T, S>::mul(r, x2 - x0);
    const T fa1 = Embed<T, S>::map(x1) + Embed<T, S>::mul(r, x3 - x1);
    const T b0 = eq_on_the_fly(tables, nforms, h, l, i), b1 = eq_on_the_fly(tables, nforms, h, l, i + q);
    const T b2 = eq_on_the_fly(tables, nforms, h, l, i + hf), b3 = eq_on_the_fly(tables, nforms, h, l, i + hf + q);
    const T fb0 = b0 + (b2 - b0) * r, fb1 = b1 + (b3 - b1) * r;
    a_out[i] = fa0;
    a_out[i + q] = fa1;
    b_out[i] = fb0;
    b_out[i + q] = fb1;
    w0.mac(fa0, fb0);
    w2.mac(fa1 - fa0, fb1 - fb0);
  }
  T acc0 = w0.get(), acc2 = w2.get();
  finish_pairs(acc0, acc2, partials, out, counter);
}

// Later rounds of the fused initial sumcheck while the folded variables stay inside the hi index:
// the covector keeps the form b(H 2^l + j) = sum_f lo_f[j] F_f[H] with row factors F (F = hi for
// the unfolded covector), so folding it only folds F, and b is never written. One launch folds
// a_in (length m) with r into a_out (m/2, may alias a_in), folds F (2^rlog rows, per-form stride
// fstride) into F_next (per-form stride 2^h), and computes (c0, c2) of the next round from
// row sums of lo-weighted a values. Needs rlog >= 2 and nforms <= EQ_MAX_FORMS.
template <class T, class S>
__global__ void __launch_bounds__(SC_THREADS, sizeof(T) <= 16 ? 2 : 1) rows_fold_compute_kernel(const S* a_in, uint64_t m, T r, const T* F,
                                                                      uint64_t fstride, int rlog, const T* tables,
                                                                      int nforms, int h, int l, T* a_out,
                                                                      T* F_next, T* partials, T* out,
                                                                      unsigned int* counter) {
  __shared__ T rowf[2][EQ_MAX_FORMS];
  const uint64_t hs = 1ull << h, ls = 1ull << l;
  const uint64_t half_rows = (1ull << rlog) >> 1, qr = (1ull << rlog) >> 2;
  const uint64_t hf = m >> 1, q = m >> 2;
  const uint64_t chunk = ls < EQ_CHUNK ? ls : EQ_CHUNK, per_row = ls / chunk, units = qr * per_row;
  T acc0 = T::zero(), acc2 = T::zero();
  for (uint64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const uint64_t H = u / per_row, j0 = (u - H * per_row) * chunk, base = H * ls;
    __syncthreads();  // the previous unit's readers are done with rowf
    if (threadIdx.x < 2 * nforms) {
      const int f = threadIdx.x >> 1, side = threadIdx.x & 1;
      const T* Ff = F + (uint64_t)f * fstride;
      const uint64_t R0 = H + side * qr;
      const T v = Ff[R0] + r * (Ff[R0 + half_rows] - Ff[R0]);
      rowf[side][f] = v;
      if (j0 == 0) F_next[(uint64_t)f * hs + R0] = v;
    }
    __syncthreads();
    for (int f = 0; f < nforms; ++f) {
      const T* lo = tables + (uint64_t)f * (hs + ls) + hs;
      WideAcc<T> s0, s2;
      s0.init();
      s2.init();
      if (f == 0 && chunk == EQ_CHUNK && sizeof(T) <= 16) {
        // Full chunk of the first form: the fold's loads are issued in groups of RF_GROUP
        // iterations before any of their stores. a_out may alias a_in, but a thread's stores
        // (offsets i, i + q) never meet another iteration's loads (i', i' + q, i' + hf, i' + hf + q
        // with i' != i inside one chunk, q >= chunk), so hoisting the loads is safe.
        constexpr int RF_GROUP = sizeof(S) <= 8 ? 4 : 2;
#pragma unroll 1
        for (int k0 = 0; k0 < EQ_UNROLL; k0 += RF_GROUP) {
          S x0[RF_GROUP], x1[RF_GROUP], x2[RF_GROUP], x3[RF_GROUP];
#pragma unroll
          for (int k = 0; k < RF_GROUP; ++k) {
            const uint64_t i = base + j0 + threadIdx.x + (uint64_t)(k0 + k) * SC_THREADS;
            x0[k] = a_in[i];
            x1[k] = a_in[i + q];
            x2[k] = a_in[i + hf];
            x3[k] = a_in[i + hf + q];
          }
#pragma unroll
          for (int k = 0; k < RF_GROUP; ++k) {
            const uint64_t j = j0 + threadIdx.x + (uint64_t)(k0 + k) * SC_THREADS, i = base + j;
            const T fa0 = Embed<T, S>::map(x0[k]) + Embed<T, S>::mul(r, x2[k] - x0[k]);
            const T fa1 = Embed<T, S>::map(x1[k]) + Embed<T, S>::mul(r, x3[k] - x1[k]);
            a_out[i] = fa0;
            a_out[i + q] = fa1;
            const T w = lo[j];
            s0.mac(w, fa0);
            s2.mac(w, fa1 - fa0);
          }
        }
      } else {
        for (uint64_t j = j0 + threadIdx.x; j < j0 + chunk; j += blockDim.x) {
          const uint64_t i = base + j;
          T fa0, fa1;
          if (f == 0) {
            const S x0 = a_in[i], x1 = a_in[i + q], x2 = a_in[i + hf], x3 = a_in[i + hf + q];
            fa0 = Embed<T, S>::map(x0) + Embed<T, S>::mul(r, x2 - x0);
            fa1 = Embed<T, S>::map(x1) + Embed<T, S>::mul(r, x3 - x1);
            a_out[i] = fa0;
            a_out[i + q] = fa1;
          } else {
            fa0 = a_out[i];  // written by this thread in the first pass
            fa1 = a_out[i + q];
          }
          const T w = lo[j];
          s0.mac(w, fa0);
          s2.mac(w, fa1 - fa0);
        }
      }
      acc0 += rowf[0][f] * s0.get();
      acc2 += (rowf[1][f] - rowf[0][f]) * s2.get();
    }
  }
  finish_pairs(acc0, acc2, partials, out, counter);
}

// End of the row-factored rounds: folds a (length m) with r in place and writes the folded
// covector b_out[i] = sum_f lo_f[j] (F_f[H] + r (F_f[H + R/2] - F_f[H])), i = H 2^l + j < m/2,
// from row factors F with R = 2^rlog rows (per-form stride 2^h).
template <class T>
__global__ void __launch_bounds__(SC_THREADS) rows_finish_kernel(T* a, uint64_t m, T r, const T* F, int rlog,
                                                                 const T* tables, int nforms, int h, int l,
                                                                 T* b_out) {
  const uint64_t hs = 1ull << h, ls = 1ull << l, half_rows = (1ull << rlog) >> 1, hf = m >> 1;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < hf; i += (uint64_t)gridDim.x * blockDim.x) {
    const T lo = a[i], hi = a[i + hf];
    a[i] = lo + (hi - lo) * r;
    const uint64_t H = i >> l, j = i & (ls - 1);
    T v = T::zero();
    for (int f = 0; f < nforms; ++f) {
      const T* Ff = F + (uint64_t)f * hs;
      const T g = Ff[H] + r * (Ff[H + half_rows] - Ff[H]);
      v += tables[(uint64_t)f * (hs + ls) + hs + j] * g;
    }
    b_out[i] = v;
  }
}

template <class T, class S>
cudaError_t launch_first_compute_eq(const S* x, size_t n, const T* tables, int nforms, int nv, T* partials,
                                    size_t* nparts, cudaStream_t s, T* out, unsigned int* counter) {
  if (nv < 2 || n != (1ull << nv)) return cudaErrorInvalidValue;  // the row split needs h >= 1
  size_t g = sumcheck_partials(n);
  {
    const int h = nv / 2, l = nv - nv / 2;
    const uint64_t ls = 1ull << l, chunk = std::min<uint64_t>(ls, EQ_CHUNK);
    const uint64_t units = (1ull << (h - 1)) * (ls / chunk);
    g = std::max<size_t>(1, std::min<size_t>(g, units));
  }
  first_compute_eq_kernel<T, S><<<(unsigned)g, SC_THREADS, 0, s>>>(x, n, tables, nforms, nv / 2, nv - nv / 2,
                                                                    partials, out, counter);
  note_launch();
  *nparts = g;
  return cudaGetLastError();
}
template <class T, class S>
cudaError_t launch_first_fold_compute_eq(const S* x, size_t n, T r, const T* tables, int nforms, int nv, T* a_out,
                                         T* b_out, T* partials, size_t* nparts, cudaStream_t s, T* out,
                                         unsigned int* counter) {
  size_t g = sumcheck_partials(n);
  const int h = nv / 2, l = nv - nv / 2;
  if (h >= 2 && nforms <= EQ_MAX_FORMS && n == (1ull << nv)) {
    const uint64_t ls = 1ull << l, chunk = std::min<uint64_t>(ls, EQ_CHUNK);
    const uint64_t units = (1ull << (h - 2)) * (ls / chunk);
    g = std::max<size_t>(1, std::min<size_t>(g, units));
    first_fold_compute_rows_kernel<T, S><<<(unsigned)g, SC_THREADS, 0, s>>>(x, n, r, tables, nforms, h, l, a_out,
                                                                             b_out, partials, out, counter);
  } else {
    first_fold_compute_eq_kernel<T, S><<<(unsigned)g, SC_THREADS, 0, s>>>(x, n, r, tables, nforms, h, l, a_out,
                                                                           b_out, partials, out, counter);
  }
  note_launch();
  *nparts = g;
  return cudaGetLastError();
}

template <class T, class S>
cudaError_t launch_rows_fold_compute(const S* a_in, size_t m, T r, const T* F, size_t fstride, int rlog,
                                     const T* tables, int nforms, int nv, T* a_out, T* F_next, T* partials,
                                     size_t* nparts, cudaStream_t s, T* out, unsigned int* counter) {
  const int h = nv / 2, l = nv - nv / 2;
  if (rlog < 2 || rlog > h || nforms > EQ_MAX_FORMS || m != ((size_t)1 << (rlog + l))) return cudaErrorInvalidValue;
  const uint64_t ls = 1ull << l, chunk = std::min<uint64_t>(ls, EQ_CHUNK);
  const uint64_t units = (1ull << (rlog - 2)) * (ls / chunk);
  size_t g = std::max<size_t>(1, std::min<size_t>(sumcheck_partials(m), units));
  rows_fold_compute_kernel<T, S><<<(unsigned)g, SC_THREADS, 0, s>>>(a_in, m, r, F, fstride, rlog, tables, nforms, h, l,
                                                                     a_out, F_next, partials, out, counter);
  note_launch();
  *nparts = g;
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_rows_finish(T* a, size_t m, T r, const T* F, int rlog, const T* tables, int nforms, int nv,
                               T* b_out, cudaStream_t s) {
  const int h = nv / 2, l = nv - nv / 2;
  if (rlog < 1 || rlog > h || m != ((size_t)1 << (rlog + l))) return cudaErrorInvalidValue;
  const size_t g = std::max<size_t>(1, std::min(SC_MAX_BLOCKS, (m / 2 + SC_THREADS - 1) / SC_THREADS));
  rows_finish_kernel<T><<<(unsigned)g, SC_THREADS, 0, s>>>(a, m, r, F, rlog, tables, nforms, h, l, b_out);
  note_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Initial sumcheck over covectors that are sums of tensor products (reference
// protocols/sumcheck.rs:69-162 with a = sum_j c_j lift(x_j) and b = sum_f s_f B_f, where every form
// is B_f(y) = prod_t phi_{f,t}(y_t) with phi(0) = alpha_t, phi(1) = beta_t: an eq form
// eq(p, .) has (alpha, beta) = (1 - p_t, p_t), an out-of-domain geometric form x^i has
// (1, x^(2^(n-1-t))); variable t = 0 is the most significant index bit).
//
// Round t's polynomial depends on the data only through the 2^k sums
//   V_{j,f}(z) = sum_rest x_j(z, rest) * prod_{t >= k} phi_{f,t}(rest)      (z = top k index bits)
// (the k folded variables enter through the challenges, the rest through the tensor weights), so
// one pass over the vectors yields every round message of the k rounds, and a second pass after
// the last challenge writes the folded vector a'(rest) = sum_{j,z} c_j eq(r, z) x_j(z, rest) and the
// folded covector b'(rest) = sum_f K_f prod_{t >= k} phi_{f,t}(rest). The rest index is split into
// 2^R rows and 2^C columns; per form, `tables` holds the row weights (2^R) then the column weights
// (2^C) of the tensor over variables k.. n-1.
// ---------------------------------------------------------------------------------------------
// Loads CPT consecutive source elements (CPT == 2: one 16-byte load of two 8-byte elements).
template <class S, int CPT>
__device__ __forceinline__ void load_cols(const S* p, S* out) {
  if constexpr (CPT == 2 && sizeof(S) == 8) {
    const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(p);
    reinterpret_cast<uint64_t*>(out)[0] = v.x;
    reinterpret_cast<uint64_t*>(out)[1] = v.y;
  } else {
#pragma unroll
    for (int c = 0; c < CPT; ++c) out[c] = p[c];
  }
}

// Sums pass. CTA (j, z, row group g, column tile): thread = CPT adjacent columns, rows
// [g rpc, (g+1) rpc) of the z block; per form the thread accumulates sum_rows row_w[H] x(H, col)
// unreduced, then multiplies by its column weight; the CTA's per-form sums go to partials, and the
// last CTA adds the partials of every (j, f, z) into out[(j nforms + f) 2^k + z]. Rows are read in
// batches of TS_RB, the next batch's loads issued before the current batch is multiplied (the first
// version, one column per thread and no prefetch, ran at 16 % of DRAM peak, long-scoreboard bound).
// Block sums of the per-thread form sums go to partials[blockIdx.x * NF + f]; the last CTA to
// arrive adds them into out[(j NF + f) 2^k + z], writes out[nout] = 1 if any CTA of the launch
// recorded an error in counter[2] (else 0) and re-arms counter[0] and counter[2].
template <class T, int NF>
__device__ __forceinline__ void tensor_sums_finish(const T (&mine)[NF], const TensorShape& sh, T* partials, T* out,
                                                   unsigned int* counter, const MailSlot& mail) {
  __shared__ bool am_last;
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    const T s = block_sum(mine[f]);
    if (threadIdx.x == 0) partials[(uint64_t)blockIdx.x * NF + f] = s;
  }
  if (threadIdx.x == 0) {
    __threadfence();
    am_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  const uint64_t nz = 1ull << sh.k, groups = sh.row_groups * sh.col_tiles;
  const uint64_t nout = (uint64_t)sh.nvec * NF * nz;
  T* mo = reinterpret_cast<T*>(mail.data);  // host-mapped copy of out, when publishing
  for (uint64_t o = threadIdx.x; o < nout; o += blockDim.x) {
    const uint64_t zz = o % nz, f = (o / nz) % NF, jj = o / (nz * NF);
    const T* p = partials + ((jj * nz + zz) * groups) * NF + f;
    T s = T::zero();
    for (uint64_t q = 0; q < groups; ++q) s += ldcg_t(p + q * NF);
    out[o] = s;
    if (mo) mo[o] = s;
  }
  if (threadIdx.x == 0) {
    const unsigned int err = atomicExch(counter + 2, 0u);
    out[nout] = err ? T::one() : T::zero();
    if (mo) mo[nout] = out[nout];
    counter[0] = 0;
  }
  if (mo == nullptr) return;
  __threadfence_system();
  __syncthreads();
  if (threadIdx.x == 0) {
    reinterpret_cast<volatile unsigned int*>(mail.flag)[1] = *reinterpret_cast<const volatile unsigned int*>(mail.dev_err);
    __threadfence_system();
    *reinterpret_cast<volatile unsigned int*>(mail.flag) = mail.seq;
  }
}

static constexpr int TS_RB = 4;
template <class T, class S, int NF, int CPT>
__global__ void __launch_bounds__(TS_THREADS) tensor_sums_kernel(const S* x, TensorShape sh, const T* tables,
                                                                 T* partials, T* out, unsigned int* counter,
                                                                 MailSlot mail) {
  __shared__ T srow[NF][TS_MAX_RPC];
  const uint64_t rows = 1ull << sh.R, cols = 1ull << sh.C, per = rows + cols;
  uint64_t bid = blockIdx.x;
  const uint64_t tile = bid % sh.col_tiles;
  bid /= sh.col_tiles;
  const uint64_t g = bid % sh.row_groups;
  bid /= sh.row_groups;
  const uint64_t z = bid & ((1ull << sh.k) - 1), j = bid >> sh.k;
  const uint64_t col = (tile * blockDim.x + threadIdx.x) * CPT;
  const uint64_t r0 = g * sh.rpc;
  for (int e = threadIdx.x; e < NF * sh.rpc; e += blockDim.x) {
    const int f = e / sh.rpc, r = e - f * sh.rpc;
    srow[f][r] = tables[(uint64_t)f * per + r0 + r];
  }
  __syncthreads();
  WideAcc<T> acc[NF][CPT];
#pragma unroll
  for (int f = 0; f < NF; ++f)
#pragma unroll
    for (int c = 0; c < CPT; ++c) acc[f][c].init();
  if (col < cols) {
    const S* base = x + j * sh.vec_stride + ((z << sh.R) + r0) * cols + col;
    const int full = sh.rpc / TS_RB * TS_RB;
    S cur[TS_RB][CPT], nxt[TS_RB][CPT];
    if (full) {
#pragma unroll
      for (int u = 0; u < TS_RB; ++u) load_cols<S, CPT>(base + (uint64_t)u * cols, cur[u]);
    }
    for (int r = 0; r < full; r += TS_RB) {
      const bool more = r + TS_RB < full;
      if (more) {
#pragma unroll
        for (int u = 0; u < TS_RB; ++u) load_cols<S, CPT>(base + (uint64_t)(r + TS_RB + u) * cols, nxt[u]);
      }
#pragma unroll
      for (int u = 0; u < TS_RB; ++u)
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          const T w = srow[f][r + u];
#pragma unroll
          for (int c = 0; c < CPT; ++c) acc[f][c].mac_mixed(w, cur[u][c]);
        }
      if (more) {
#pragma unroll
        for (int u = 0; u < TS_RB; ++u)
#pragma unroll
          for (int c = 0; c < CPT; ++c) cur[u][c] = nxt[u][c];
      }
    }
    for (int r = full; r < sh.rpc; ++r) {
      S v[CPT];
      load_cols<S, CPT>(base + (uint64_t)r * cols, v);
#pragma unroll
      for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int c = 0; c < CPT; ++c) acc[f][c].mac_mixed(srow[f][r], v[c]);
    }
  }
  T mine[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    mine[f] = T::zero();
    if (col < cols) {
#pragma unroll
      for (int c = 0; c < CPT; ++c) mine[f] += tables[(uint64_t)f * per + rows + col + c] * acc[f][c].get();
    }
  }
  tensor_sums_finish<T, NF>(mine, sh, partials, out, counter, mail);
}

// Sums pass with the tile staged by the bulk-copy engine: CTA (j, z, row group, 512-column tile)
// streams its rpc rows of 4 KiB through TB_NST shared-memory stages of TB_RB rows. One thread issues
// a stage's row copies against the stage's mbarrier; every thread waits for the stage, reads its two
// columns of each row (one 16-byte shared load) and accumulates; after a CTA barrier the stage is
// refilled with the rows TB_NST stages ahead. Up to TB_NST x 16 KiB are in flight per CTA with no
// registers held for them (the register-prefetch version above keeps 64 bytes per thread in flight
// and runs two CTAs per SM at 100 registers).
// A stage wait that times out sets the context's error word (counter[2]); the CTA then stops reading,
// waits (bounded) for its copies still in flight and still takes part in the final reduction, whose
// last CTA reports the error in out[nout].
static constexpr int TB_RB = 4;
static constexpr int TB_NST = 3;
static constexpr int TB_COLS = 2 * TS_THREADS;
static constexpr uint32_t TB_ROW_BYTES = TB_COLS * 8;
static constexpr uint32_t TB_STAGE_BYTES = TB_RB * TB_ROW_BYTES;
static constexpr size_t TB_SMEM = (size_t)TB_NST * TB_STAGE_BYTES;

// Resident CTAs per SM the bulk kernel is compiled for: its registers are the NF x 2 wide
// accumulators plus addressing, so more forms or wider fields get fewer CTAs instead of spills.
template <class T, int NF>
struct TbMinCtas {
  static constexpr int value = (NF == 1 && sizeof(T) <= 16) ? 4 : (NF * sizeof(T) <= 32 ? 2 : 1);
};

template <class T, class S, int NF>
__global__ void __launch_bounds__(TS_THREADS, TbMinCtas<T, NF>::value) tensor_sums_bulk_kernel(const S* x, TensorShape sh, const T* tables,
                                                                         T* partials, T* out, unsigned int* counter,
                                                                         MailSlot mail) {
  static_assert(sizeof(S) == 8, "two 8-byte source elements per 16-byte shared load");
  extern __shared__ __align__(128) unsigned char tb_smem[];
  __shared__ T srow[NF][TS_MAX_RPC];
  __shared__ __align__(8) uint64_t bar[TB_NST];
  __shared__ int aborted;
  const uint64_t rows = 1ull << sh.R, cols = 1ull << sh.C, per = rows + cols;
  uint64_t bid = blockIdx.x;
  const uint64_t tile = bid % sh.col_tiles;
  bid /= sh.col_tiles;
  const uint64_t g = bid % sh.row_groups;
  bid /= sh.row_groups;
  const uint64_t z = bid & ((1ull << sh.k) - 1), j = bid >> sh.k;
  const uint64_t col0 = tile * TB_COLS, col = col0 + 2 * threadIdx.x;
  const uint64_t r0 = g * sh.rpc;
  const S* base = x + j * sh.vec_stride + ((z << sh.R) + r0) * cols + col0;
  const int nb = sh.rpc / TB_RB;
  if (threadIdx.x == 0) {
    aborted = 0;
#pragma unroll
    for (int st = 0; st < TB_NST; ++st) mbar_init(&bar[st], 1);
    mbar_init_fence();
  }
  for (int e = threadIdx.x; e < NF * sh.rpc; e += blockDim.x) {
    const int f = e / sh.rpc, r = e - f * sh.rpc;
    srow[f][r] = tables[(uint64_t)f * per + r0 + r];
  }
  __syncthreads();
  auto issue = [&](int b) {
    const int st = b % TB_NST;
    unsigned char* dst = tb_smem + (size_t)st * TB_STAGE_BYTES;
    mbar_arrive_expect_tx(&bar[st], TB_STAGE_BYTES);
#pragma unroll
    for (int u = 0; u < TB_RB; ++u)
      bulk_copy_g2s(dst + u * TB_ROW_BYTES, base + (uint64_t)(b * TB_RB + u) * cols, TB_ROW_BYTES, &bar[st]);
  };
  if (threadIdx.x == 0)
    for (int b = 0; b < nb && b < TB_NST; ++b) issue(b);
  WideAcc<T> acc[NF][2];
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    acc[f][0].init();
    acc[f][1].init();
  }
  int b = 0;
  for (; b < nb; ++b) {
    const int st = b % TB_NST;
    if (mbar_wait(&bar[st], (uint32_t)(b / TB_NST) & 1)) {
      const unsigned char* src = tb_smem + (size_t)st * TB_STAGE_BYTES + 16 * threadIdx.x;
#pragma unroll
      for (int u = 0; u < TB_RB; ++u) {
        const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(src + u * TB_ROW_BYTES);
        S x0, x1;
        reinterpret_cast<uint64_t*>(&x0)[0] = v.x;
        reinterpret_cast<uint64_t*>(&x1)[0] = v.y;
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          const T w = srow[f][b * TB_RB + u];
          acc[f][0].mac_mixed(w, x0);
          acc[f][1].mac_mixed(w, x1);
        }
      }
    } else {
      aborted = 1;
    }
    __syncthreads();
    if (aborted) break;
    if (threadIdx.x == 0 && b + TB_NST < nb) {
      fence_proxy_async_smem();
      issue(b + TB_NST);
    }
  }
  if (aborted && threadIdx.x == 0) {
    atomicExch(counter + 2, 1u);
    atomicExch(counter + 3, 1u);
    // the copies of the stage that timed out and of the stages issued after it
    for (int q = b; q < nb && q < b + TB_NST; ++q) mbar_wait(&bar[q % TB_NST], (uint32_t)(q / TB_NST) & 1);
  }
  T mine[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    mine[f] = T::zero();
    if (!aborted) {
      mine[f] += tables[(uint64_t)f * per + rows + col] * acc[f][0].get();
      mine[f] += tables[(uint64_t)f * per + rows + col + 1] * acc[f][1].get();
    }
  }
  tensor_sums_finish<T, NF>(mine, sh, partials, out, counter, mail);
}

// Fold pass: a_out[i] = sum_{j, z} w[j 2^k + z] x_j(z, i) and b_out[i] = sum_f kf[f] row_f[i >> C]
// col_f[i & (2^C - 1)] for i < 2^(R + C).
template <class T, class S>
__global__ void __launch_bounds__(TS_THREADS) tensor_fold_kernel(const S* x, TensorShape sh, const T* w,
                                                                 const T* kf, const T* tables, T* a_out,
                                                                 T* b_out) {
  extern __shared__ unsigned char ts_smem[];
  T* sw = reinterpret_cast<T*>(ts_smem);
  const int nw = sh.nvec << sh.k;
  for (int e = threadIdx.x; e < nw; e += blockDim.x) sw[e] = w[e];
  __syncthreads();
  const uint64_t rows = 1ull << sh.R, cols = 1ull << sh.C, per = rows + cols, len = rows * cols;
  const uint64_t zstride = len, nz = 1ull << sh.k;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < len; i += (uint64_t)gridDim.x * blockDim.x) {
    WideAcc<T> acc;
    acc.init();
    for (int j = 0; j < sh.nvec; ++j) {
      const S* xj = x + (uint64_t)j * sh.vec_stride + i;
      const T* wj = sw + ((uint64_t)j << sh.k);
      uint64_t z = 0;
      for (; z + 8 <= nz; z += 8) {
        S v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = xj[(z + u) * zstride];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc.mac_mixed(wj[z + u], v[u]);
      }
      for (; z < nz; ++z) acc.mac_mixed(wj[z], xj[z * zstride]);
    }
    a_out[i] = acc.get();
    const uint64_t H = i >> sh.C, c = i & (cols - 1);
    T bv = T::zero();
    for (int f = 0; f < sh.nforms; ++f) {
      const T* tf = tables + (uint64_t)f * per;
      bv += kf[f] * (tf[H] * tf[rows + c]);
    }
    b_out[i] = bv;
  }
}

// Fold pass with the source rows staged by the bulk-copy engine (8-byte sources, 512-output tiles):
// CTA = outputs [i0, i0 + 512); its nvec 2^k source rows x_j(z, i0 .. i0 + 511) (4 KiB each) stream
// through TB_NST shared-memory stages of TB_RB rows as in the sums pass, each thread accumulating
// two adjacent outputs. Waits are bounded as in tensor_sums_bulk_kernel; a timeout sets the error
// word counter[2], which the host reads back after the fold.
// Issues stage q % TB_NST of the fold: rows r = q TB_RB + u, row r = (vector r >> nz_log, z = the low
// bits), each TB_ROW_BYTES from x_j(z, i0).
template <class S>
__device__ __forceinline__ void fold_issue(unsigned char* smem, uint64_t* bar, int q, const S* xt, uint64_t vstride,
                                           uint64_t len, int nz_log) {
  const int st = q % TB_NST;
  unsigned char* dst = smem + (size_t)st * TB_STAGE_BYTES;
  mbar_arrive_expect_tx(&bar[st], TB_STAGE_BYTES);
#pragma unroll
  for (int u = 0; u < TB_RB; ++u) {
    const int r = q * TB_RB + u, j = r >> nz_log, z = r & ((1 << nz_log) - 1);
    bulk_copy_g2s(dst + u * TB_ROW_BYTES, xt + (uint64_t)j * vstride + (uint64_t)z * len, TB_ROW_BYTES, &bar[st]);
  }
}

template <class T, class S>
__global__ void __launch_bounds__(TS_THREADS, sizeof(T) <= 8 ? 4 : (sizeof(T) <= 16 ? 3 : 2)) tensor_fold_bulk_kernel(const S* x, TensorShape sh, const T* w,
                                                                        const T* kf, const T* tables, T* a_out,
                                                                        T* b_out, unsigned int* err) {
  static_assert(sizeof(S) == 8, "two 8-byte source elements per 16-byte shared load");
  extern __shared__ __align__(128) unsigned char tb_smem[];
  __shared__ __align__(8) uint64_t bar[TB_NST];
  __shared__ int aborted;
  const uint64_t rows = 1ull << sh.R, cols = 1ull << sh.C, per = rows + cols, len = rows * cols;
  const int nz_log = sh.k, nrows = sh.nvec << sh.k, nb = nrows / TB_RB;
  T* sw = reinterpret_cast<T*>(tb_smem + TB_SMEM);  // the nrows fold weights after the stages
  const uint64_t i0 = (uint64_t)blockIdx.x * TB_COLS;
  if (threadIdx.x == 0) {
    aborted = 0;
#pragma unroll
    for (int st = 0; st < TB_NST; ++st) mbar_init(&bar[st], 1);
    mbar_init_fence();
  }
  for (int e = threadIdx.x; e < nrows; e += blockDim.x) sw[e] = w[e];
  __syncthreads();
  const S* xt = x + i0;
  const uint64_t vstride = sh.vec_stride;
  if (threadIdx.x == 0)
    for (int q = 0; q < nb && q < TB_NST; ++q) fold_issue<S>(tb_smem, bar, q, xt, vstride, len, nz_log);
  WideAcc<T> acc0, acc1;
  acc0.init();
  acc1.init();
  int b = 0;
  for (; b < nb; ++b) {
    const int st = b % TB_NST;
    if (mbar_wait(&bar[st], (uint32_t)(b / TB_NST) & 1)) {
      const unsigned char* src = tb_smem + (size_t)st * TB_STAGE_BYTES + 16 * threadIdx.x;
#pragma unroll
      for (int u = 0; u < TB_RB; ++u) {
        const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(src + u * TB_ROW_BYTES);
        S x0, x1;
        reinterpret_cast<uint64_t*>(&x0)[0] = v.x;
        reinterpret_cast<uint64_t*>(&x1)[0] = v.y;
        const T wr = sw[b * TB_RB + u];
        acc0.mac_mixed(wr, x0);
        acc1.mac_mixed(wr, x1);
      }
    } else {
      aborted = 1;
    }
    __syncthreads();
    if (aborted) break;
    if (threadIdx.x == 0 && b + TB_NST < nb) {
      fence_proxy_async_smem();
      fold_issue<S>(tb_smem, bar, b + TB_NST, xt, vstride, len, nz_log);
    }
  }
  if (aborted) {
    if (threadIdx.x == 0) {
      atomicExch(err, 1u);
      for (int q = b; q < nb && q < b + TB_NST; ++q) mbar_wait(&bar[q % TB_NST], (uint32_t)(q / TB_NST) & 1);
    }
    return;
  }
  const uint64_t i = i0 + 2 * threadIdx.x;
  a_out[i] = acc0.get();
  a_out[i + 1] = acc1.get();
  const uint64_t H = i >> sh.C, c = i & (cols - 1);  // i and i + 1 share the row (cols >= 2)
  T b0 = T::zero(), b1 = T::zero();
  for (int f = 0; f < sh.nforms; ++f) {
    const T* tf = tables + (uint64_t)f * per;
    const T rowk = kf[f] * tf[H];
    b0 += rowk * tf[rows + c];
    b1 += rowk * tf[rows + c + 1];
  }
  b_out[i] = b0;
  b_out[i + 1] = b1;
}

template <class T, class S, int NF>
static cudaError_t run_tensor_sums_bulk(const S* x, const TensorShape& sh, const T* tables, T* partials, T* out,
                                        unsigned int* counter, cudaStream_t s, const MailSlot& mail) {
  static std::once_flag flags[SC_MAX_DEVICES];
  static cudaError_t results[SC_MAX_DEVICES];
  cudaError_t e = sc_smem_attr_once(tensor_sums_bulk_kernel<T, S, NF>, TB_SMEM, flags, results);
  if (e != cudaSuccess) return e;
  tensor_sums_bulk_kernel<T, S, NF><<<(unsigned)sh.grid(), TS_THREADS, TB_SMEM, s>>>(x, sh, tables, partials, out,
                                                                                     counter, mail);
  return cudaSuccess;
}

// The bulk-staged kernel takes full 512-column tiles of 8-byte elements at 16-byte aligned rows.
inline bool tensor_sums_bulk_ok(const TensorShape& sh, size_t src_bytes) {
  return sh.cpt == 2 && src_bytes == 8 && sh.threads == TS_THREADS && (1ull << sh.C) % TB_COLS == 0 &&
         sh.rpc % TB_RB == 0;
}

template <class T, class S>
cudaError_t launch_tensor_sums(const S* x, const TensorShape& sh, const T* tables, T* partials, T* out,
                               unsigned int* counter, cudaStream_t s, const MailSlot& mail) {
  const unsigned grid = (unsigned)sh.grid();
  const bool two = sh.cpt == 2;
  if (two && (sizeof(S) != 8 || reinterpret_cast<uintptr_t>(x) % 16)) return cudaErrorInvalidValue;
  if constexpr (sizeof(S) == 8) {
    if (tensor_sums_bulk_ok(sh, sizeof(S))) {
      cudaError_t e = cudaSuccess;
      switch (sh.nforms) {
        case 1: e = run_tensor_sums_bulk<T, S, 1>(x, sh, tables, partials, out, counter, s, mail); break;
        case 2: e = run_tensor_sums_bulk<T, S, 2>(x, sh, tables, partials, out, counter, s, mail); break;
        case 3: e = run_tensor_sums_bulk<T, S, 3>(x, sh, tables, partials, out, counter, s, mail); break;
        case 4: e = run_tensor_sums_bulk<T, S, 4>(x, sh, tables, partials, out, counter, s, mail); break;
        default: return cudaErrorInvalidValue;
      }
      if (e != cudaSuccess) return e;
      note_launch();
      return cudaGetLastError();
    }
  }
#define WHIR_TS_LAUNCH(NF)                                                                                        \
  if (two)                                                                                                        \
    tensor_sums_kernel<T, S, NF, 2><<<grid, sh.threads, 0, s>>>(x, sh, tables, partials, out, counter, mail);    \
  else                                                                                                            \
    tensor_sums_kernel<T, S, NF, 1><<<grid, sh.threads, 0, s>>>(x, sh, tables, partials, out, counter, mail);
  switch (sh.nforms) {
    case 1: WHIR_TS_LAUNCH(1) break;
    case 2: WHIR_TS_LAUNCH(2) break;
    case 3: WHIR_TS_LAUNCH(3) break;
    case 4: WHIR_TS_LAUNCH(4) break;
    default: return cudaErrorInvalidValue;
  }
#undef WHIR_TS_LAUNCH
  note_launch();
  return cudaGetLastError();
}

template <class T, class S>
static cudaError_t run_tensor_fold_bulk(const S* x, const TensorShape& sh, const T* w, const T* kf, const T* tables,
                                        T* a_out, T* b_out, unsigned int* err, cudaStream_t s) {
  static std::once_flag flags[SC_MAX_DEVICES];
  static cudaError_t results[SC_MAX_DEVICES];
  const size_t smem = TB_SMEM + ((size_t)sh.nvec << sh.k) * sizeof(T);
  cudaError_t e = sc_smem_attr_once(tensor_fold_bulk_kernel<T, S>, TB_SMEM + 48 * 1024, flags, results);
  if (e != cudaSuccess) return e;
  const uint64_t len = 1ull << (sh.R + sh.C);
  tensor_fold_bulk_kernel<T, S><<<(unsigned)(len / TB_COLS), TS_THREADS, smem, s>>>(x, sh, w, kf, tables, a_out, b_out,
                                                                                  err);
  return cudaSuccess;
}

template <class T, class S>
cudaError_t launch_tensor_fold(const S* x, const TensorShape& sh, const T* w, const T* kf, const T* tables, T* a_out,
                               T* b_out, unsigned int* err, cudaStream_t s) {
  const uint64_t len = 1ull << (sh.R + sh.C);
  const size_t smem = ((size_t)sh.nvec << sh.k) * sizeof(T);
  if (smem > 48 * 1024) return cudaErrorInvalidValue;
  if constexpr (sizeof(S) == 8) {
    // bulk-staged: whole 512-output tiles, 16-byte aligned rows, whole stages of rows
    if (err && len % TB_COLS == 0 && reinterpret_cast<uintptr_t>(x) % 16 == 0 && sh.vec_stride % 2 == 0 &&
        ((sh.nvec << sh.k) % TB_RB) == 0 && (1ull << sh.C) >= 2) {
      cudaError_t e = run_tensor_fold_bulk<T, S>(x, sh, w, kf, tables, a_out, b_out, err, s);
      if (e != cudaSuccess) return e;
      note_launch();
      return cudaGetLastError();
    }
  }
  const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((len + TS_THREADS - 1) / TS_THREADS,
                                                                           SC_MAX_BLOCKS * 4));
  tensor_fold_kernel<T, S><<<grid, TS_THREADS, smem, s>>>(x, sh, w, kf, tables, a_out, b_out);
  note_launch();
  return cudaGetLastError();
}

// Row and column tables of every form in one launch: form f's entries out[f (2^R + 2^C) + e] are its
// row table (e < 2^R: variables 0..R-1, pairs ab[f pf ..]) then its column table (variables R..R+C-1,
// pairs ab[f pf + 2R ..]), pf = 2 (R + C).
template <class T>
__global__ void tensor_tables_kernel(const T* ab, int nforms, int R, int C, T* out) {
  const uint64_t rows = 1ull << R, per = rows + (1ull << C), total = per * (uint64_t)nforms;
  const uint64_t pf = 2ull * (R + C);
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t f = t / per, e = t - f * per;
    const bool is_row = e < rows;
    const int cnt = is_row ? R : C;
    const uint64_t idx = is_row ? e : e - rows;
    const T* p = ab + f * pf + (is_row ? 0 : 2ull * R);
    T v = T::one();
    for (int q = 0; q < cnt; ++q) v = v * p[2 * q + ((idx >> (cnt - 1 - q)) & 1)];
    out[t] = v;
  }
}
template <class T>
cudaError_t launch_tensor_tables(const T* ab, int nforms, int R, int C, T* out, cudaStream_t s) {
  const uint64_t total = ((1ull << R) + (1ull << C)) * (uint64_t)nforms;
  if (total == 0) return cudaSuccess;
  tensor_tables_kernel<T><<<(unsigned)std::min<uint64_t>((total + 255) / 256, 4096), 256, 0, s>>>(ab, nforms, R, C, out);
  note_launch();
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------------------------
// Multilinear evaluation sum_i map(x_i) * eq(point, i) with the eq weights taken from one pair of
// hi / lo tables (tables[0..2^h) and tables[2^h .. 2^h + 2^l)); block sums go to partials.
// ---------------------------------------------------------------------------------------------
template <class T, class S>
__global__ void __launch_bounds__(SC_THREADS) mle_dot_kernel(const S* x, uint64_t n, const T* tables, int h, int l,
                                                             T* partials) {
  T acc = T::zero();
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    acc += Embed<T, S>::mul(eq_on_the_fly(tables, 1, h, l, i), x[i]);
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

template <class T, class S>
cudaError_t launch_mle_dot(const S* x, size_t n, const T* tables, int nv, T* partials, size_t* nparts,
                           cudaStream_t s) {
  size_t g = std::max<size_t>(1, std::min(SC_MAX_BLOCKS, (n + SC_THREADS - 1) / SC_THREADS));
  mle_dot_kernel<T, S><<<(unsigned)g, SC_THREADS, 0, s>>>(x, n, tables, nv / 2, nv - nv / 2, partials);
  note_launch();
  *nparts = g;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Lift + RLC
// ---------------------------------------------------------------------------------------------
template <class T, class S>
__global__ void lift_kernel(T* dst, const S* src, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = Embed<T, S>::map(src[i]);
}
template <class T, class S>
__global__ void axpy_kernel(T* dst, T c, const S* src, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] += Embed<T, S>::mul(c, src[i]);
}

template <class T, class S>
cudaError_t launch_lift_rlc(T* dst, const S* const* vecs, const T* coeffs, size_t nvec, size_t n, cudaStream_t s) {
  size_t g = std::min<size_t>(SC_MAX_BLOCKS * 2, (n + SC_THREADS - 1) / SC_THREADS);
  if (g == 0) return cudaSuccess;
  lift_kernel<T, S><<<(unsigned)g, SC_THREADS, 0, s>>>(dst, vecs[0], n);
  note_launch();
  for (size_t j = 1; j < nvec; ++j) {
    axpy_kernel<T, S><<<(unsigned)g, SC_THREADS, 0, s>>>(dst, coeffs[j], vecs[j], n);
    note_launch();
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Univariate evaluation: thread handles UE_E consecutive coefficients by Horner, scaled by
// x^(chunk start); block sums go to partials.
// ---------------------------------------------------------------------------------------------
static constexpr int UE_E = 32;

template <class T, class S>
__global__ void __launch_bounds__(SC_THREADS) univariate_kernel(const S* c, uint64_t n, T x, T* partials) {
  const uint64_t start = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * UE_E;
  T h = T::zero();
  if (start < n) {
    const uint64_t end = std::min<uint64_t>(start + UE_E, n);
    for (uint64_t i = end; i-- > start;) h = h * x + Embed<T, S>::map(c[i]);
    h = h * x.pow(start);
  }
  h = block_sum(h);
  if (threadIdx.x == 0) partials[blockIdx.x] = h;
}

template <class T, class S>
cudaError_t launch_univariate_eval(const S* coeffs, size_t n, T x, T* partials, size_t* nparts, cudaStream_t s) {
  size_t per = (size_t)SC_THREADS * UE_E;
  size_t g = std::max<size_t>(1, (n + per - 1) / per);
  univariate_kernel<T, S><<<(unsigned)g, SC_THREADS, 0, s>>>(coeffs, n, x, partials);
  note_launch();
  *nparts = g;
  return cudaGetLastError();
}

// Explicit-instantiation lists (used by sumcheck.cu and sumcheck_mont.cu).
#define WHIR_SC_INST(T)                                                                                          \
  template cudaError_t launch_sumcheck_compute<T>(const T*, const T*, size_t, T*, size_t*, cudaStream_t, T*,      \
                                                  unsigned int*);                                                \
  template cudaError_t launch_fold_compute<T>(T*, T*, size_t, T, T*, size_t*, cudaStream_t, T*, unsigned int*);  \
  template cudaError_t launch_fold<T>(T*, size_t, T, cudaStream_t);                                               \
  template cudaError_t launch_fold2<T>(T*, T*, size_t, T, cudaStream_t);                                          \
  template cudaError_t launch_reduce_pairs<T>(const T*, size_t, T*, cudaStream_t);                                \
  template cudaError_t launch_reduce_singles<T>(const T*, size_t, T*, cudaStream_t);                              \
  template cudaError_t launch_eval_eq<T>(T*, const T*, int, T, T*, cudaStream_t);                                 \
  template cudaError_t launch_geometric_accumulate<T>(T*, size_t, const T*, const T*, size_t, cudaStream_t);      \
  template cudaError_t launch_geometric_roots<T>(T*, size_t, const T*, const uint64_t*, size_t, int, RootTab,    \
                                                 cudaStream_t, T*, unsigned int*);                               \
  template cudaError_t launch_scatter<T>(T*, const uint64_t*, const T*, size_t, cudaStream_t);                   \
  template cudaError_t launch_add<T>(T*, const T*, size_t, cudaStream_t);                                        \
  template cudaError_t launch_eq_table<T>(const T*, int, int, T, T*, cudaStream_t);                              \
  template cudaError_t launch_rows_finish<T>(T*, size_t, T, const T*, int, const T*, int, int, T*, cudaStream_t);  \
  template cudaError_t launch_tensor_tables<T>(const T*, int, int, int, T*, cudaStream_t);

// Kernels that read coefficient vectors over S and compute over T.
#define WHIR_SC_EMBED_INST(T, S)                                                                                 \
  template cudaError_t launch_first_compute_eq<T, S>(const S*, size_t, const T*, int, int, T*, size_t*,          \
                                                     cudaStream_t, T*, unsigned int*);                           \
  template cudaError_t launch_first_fold_compute_eq<T, S>(const S*, size_t, T, const T*, int, int, T*, T*, T*,   \
                                                          size_t*, cudaStream_t, T*, unsigned int*);             \
  template cudaError_t launch_mle_dot<T, S>(const S*, size_t, const T*, int, T*, size_t*, cudaStream_t);         \
  template cudaError_t launch_lift_rlc<T, S>(T*, const S* const*, const T*, size_t, size_t, cudaStream_t);       \
  template cudaError_t launch_univariate_eval<T, S>(const S*, size_t, T, T*, size_t*, cudaStream_t);             \
  template cudaError_t launch_rows_fold_compute<T, S>(const S*, size_t, T, const T*, size_t, int, const T*, int,  \
                                                      int, T*, T*, T*, size_t*, cudaStream_t, T*, unsigned int*); \
  template cudaError_t launch_tensor_sums<T, S>(const S*, const TensorShape&, const T*, T*, T*, unsigned int*,     \
                                                cudaStream_t, const MailSlot&);                                                   \
  template cudaError_t launch_tensor_fold<T, S>(const S*, const TensorShape&, const T*, const T*, const T*, T*, T*, \
                                                unsigned int*, cudaStream_t);

}  // namespace whir
