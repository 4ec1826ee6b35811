// Commitment-side kernels: encode instantiations for the Goldilocks family (the encode kernels
// themselves, with the leaf hash fused into the kernel that writes each codeword row, are in
// encode.cuh), Merkle layers, generic hash_many, proof-of-work search and opening gathers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

#include "encode.cuh"
#include "field.cuh"
#include "hash.cuh"
#include "kernels.hpp"
#include "roots.cuh"
#include "status.hpp"

namespace whir {

static unsigned long long g_launches = 0;
uint64_t kernel_launches() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }
void note_launch() { __atomic_fetch_add(&g_launches, 1ull, __ATOMIC_RELAXED); }

static int ilog2(size_t x) {
  int l = 0;
  while (((size_t)1 << l) < x) ++l;
  return l;
}
static bool is_pow2(size_t x) { return x && !(x & (x - 1)); }

int plan_encode(size_t n_msgs, size_t msg_len, size_t codeword_len, size_t eb, EncodePlan* p) {
  if (n_msgs == 0 || codeword_len == 0) return WHIR_ERR_INVALID;
  if (!is_pow2(codeword_len) || codeword_len > (1ull << 32)) return WHIR_ERR_UNSUPPORTED;
  size_t C = 1;
  while (C < msg_len) C <<= 1;  // coset size: next power of two >= masked message length
  if (C > codeword_len) return WHIR_ERR_INVALID;
  p->logC = ilog2(C);
  p->logN = ilog2(codeword_len);
  size_t K = codeword_len / C;
  p->scratch_elems = 0;
  p->logC1 = p->logC2 = 0;
  p->cols_per_cta = 0;
  if (n_msgs * C * eb <= ENC_SMEM_BUDGET && p->logC <= ENC_MAX_LOGN_SMEM) {
    p->mode = 0;
    size_t G = std::max<size_t>(1, ENC_SMEM_BUDGET / (n_msgs * C * eb));
    size_t g2 = 1;
    while (g2 * 2 <= G) g2 *= 2;
    G = std::min(g2, K);
    // keep at least ~2 waves of CTAs when the shape allows it
    while (G > 1 && K / G < 304) G >>= 1;
    p->cosets_per_cta = (int)G;
    return 0;
  }
  size_t C2 = 1;
  while (n_msgs * (C2 * 2) * eb <= ENC_SMEM_BUDGET && C2 * 2 <= C && ilog2(C2 * 2) <= ENC_MAX_LOGN_SMEM) C2 *= 2;
  if (n_msgs * C2 * eb > ENC_SMEM_BUDGET) return WHIR_ERR_UNSUPPORTED;
  size_t C1 = C / C2;
  if (ilog2(C1) > ENC_MAX_LOGN_SMEM || C1 * eb > ENC_SMEM_BUDGET) return WHIR_ERR_UNSUPPORTED;
  size_t W = 1;
  while (W * 2 <= C2 && C1 * (W * 2) * eb <= ENC_SMEM_BUDGET) W *= 2;
  p->mode = 1;
  p->logC1 = ilog2(C1);
  p->logC2 = ilog2(C2);
  p->cosets_per_cta = 1;
  p->cols_per_cta = (int)W;
  p->scratch_elems = n_msgs * K * C;
  return 0;
}

WHIR_ENCODE_INST(Gl)
WHIR_ENCODE_INST(Gl2)
WHIR_ENCODE_INST(Gl3)


// ---------------------------------------------------------------------------------------------
// Merkle layers: each CTA hashes a tile of 2^k consecutive nodes of one layer up k layers in
// shared memory, writing every produced node to its slot.
// ---------------------------------------------------------------------------------------------
static constexpr int MK_THREADS = 256;
static constexpr int MK_TILE_LOG = 9;  // 512 input digests per CTA (16 KiB)

template <int KIND>
__global__ void __launch_bounds__(MK_THREADS) merkle_tile_kernel(uint32_t* nodes, int layers, int in_level,
                                                                 int nlev, uint64_t in_count) {
  __shared__ uint4 buf[(1 << MK_TILE_LOG) * 2];  // 512 digests
  const int tile_log = nlev;
  const uint64_t tile = 1ull << tile_log;
  // offset of level l: 2^(L+1) - 2^(L-l+1)
  auto level_off = [&](int l) -> uint64_t { return (2ull << layers) - (2ull << (layers - l)); };
  const uint64_t in_off = level_off(in_level);
  const uint64_t first = (uint64_t)blockIdx.x * tile;
  const uint4* src = reinterpret_cast<const uint4*>(nodes + (in_off + first) * 8);
  for (uint64_t i = threadIdx.x; i < tile * 2 && first + i / 2 < in_count; i += blockDim.x) buf[i] = src[i];
  __syncthreads();
  uint64_t cnt = tile;
  for (int l = 1; l <= nlev; ++l) {
    cnt >>= 1;
    const uint64_t out_off = level_off(in_level + l) + (first >> l);
    uint32_t h[8];
    uint4 r0, r1;
    const bool active = threadIdx.x < cnt;
    if (active) {
      uint32_t m[16];
      const uint4* p = buf + threadIdx.x * 4;
      uint4 q0 = p[0], q1 = p[1], q2 = p[2], q3 = p[3];
      m[0] = q0.x; m[1] = q0.y; m[2] = q0.z; m[3] = q0.w;
      m[4] = q1.x; m[5] = q1.y; m[6] = q1.z; m[7] = q1.w;
      m[8] = q2.x; m[9] = q2.y; m[10] = q2.z; m[11] = q2.w;
      m[12] = q3.x; m[13] = q3.y; m[14] = q3.z; m[15] = q3.w;
      hash64<KIND>(m, h);
      r0 = make_uint4(h[0], h[1], h[2], h[3]);
      r1 = make_uint4(h[4], h[5], h[6], h[7]);
      uint4* dst = reinterpret_cast<uint4*>(nodes + (out_off + threadIdx.x) * 8);
      dst[0] = r0;
      dst[1] = r1;
    }
    __syncthreads();
    if (active) {
      buf[threadIdx.x * 2] = r0;
      buf[threadIdx.x * 2 + 1] = r1;
    }
    __syncthreads();
  }
}

template <int KIND>
static cudaError_t merkle_run(uint32_t* nodes, int layers, cudaStream_t s) {
  int level = 0;
  while (level < layers) {
    int nlev = std::min(MK_TILE_LOG, layers - level);
    uint64_t in_count = 1ull << (layers - level);
    uint64_t grid = in_count >> nlev;
    merkle_tile_kernel<KIND><<<(unsigned)grid, MK_THREADS, 0, s>>>(nodes, layers, level, nlev, in_count);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    level += nlev;
  }
  return cudaSuccess;
}

cudaError_t launch_merkle(uint32_t* nodes, int layers, int kind, cudaStream_t s) {
  switch (kind) {
    case HASH_BLAKE3: return merkle_run<HASH_BLAKE3>(nodes, layers, s);
    case HASH_SHA2: return merkle_run<HASH_SHA2>(nodes, layers, s);
    case HASH_SHA3: return merkle_run<HASH_SHA3>(nodes, layers, s);
    case HASH_KECCAK: return merkle_run<HASH_KECCAK>(nodes, layers, s);
    default: return cudaErrorInvalidValue;  // Copy cannot hash 64-byte nodes
  }
}

// ---------------------------------------------------------------------------------------------
// hash_many: one thread per message (size % 4 == 0).
// ---------------------------------------------------------------------------------------------
template <int KIND>
__global__ void hash_many_kernel(const uint8_t* in, uint64_t size, uint64_t count, uint8_t* out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint8_t* p = in + i * size;
    WordHasher<KIND> h;
    h.init((uint32_t)size);
    for (uint64_t k = 0; k < size; k += 4)
      h.push((uint32_t)p[k] | ((uint32_t)p[k + 1] << 8) | ((uint32_t)p[k + 2] << 16) | ((uint32_t)p[k + 3] << 24));
    uint32_t o[8];
    h.finish(o);
    for (int q = 0; q < 8; ++q)
      for (int b = 0; b < 4; ++b) out[i * 32 + 4 * q + b] = (uint8_t)(o[q] >> (8 * b));
  }
}

cudaError_t launch_hash_many(const uint8_t* in, size_t size, size_t count, uint8_t* out, int kind, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  unsigned grid = (unsigned)std::min<size_t>((count + 255) / 256, 65535);
  switch (kind) {
    case HASH_BLAKE3: hash_many_kernel<HASH_BLAKE3><<<grid, 256, 0, s>>>(in, size, count, out); note_launch(); break;
    case HASH_SHA2: hash_many_kernel<HASH_SHA2><<<grid, 256, 0, s>>>(in, size, count, out); note_launch(); break;
    case HASH_SHA3: hash_many_kernel<HASH_SHA3><<<grid, 256, 0, s>>>(in, size, count, out); note_launch(); break;
    case HASH_KECCAK: hash_many_kernel<HASH_KECCAK><<<grid, 256, 0, s>>>(in, size, count, out); note_launch(); break;
    default: hash_many_kernel<HASH_COPY><<<grid, 256, 0, s>>>(in, size, count, out); note_launch(); break;
    note_launch();
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Proof of work: every nonce of the range is tested, so the minimum over the range is exact.
// ---------------------------------------------------------------------------------------------
struct PowArgs {
  uint32_t chal[8];
  uint32_t pre[16];  // Blake3: state after the nonce-independent part of round 1 (blake3_pow_prefix)
  uint64_t threshold, start, count;
  unsigned long long* best;
  unsigned long long* counter;
};

static constexpr int POW_THREADS = 256;
static constexpr int POW_PER_THREAD = 4;
static constexpr uint64_t POW_BLOCK = (uint64_t)POW_THREADS * POW_PER_THREAD;

// CTAs claim consecutive blocks of POW_BLOCK nonces in increasing order and stop at the first block
// that starts at or above the best nonce found so far. Every block below the final best has been
// searched completely, so the result is the lowest satisfying nonce of the range.
template <int KIND>
__global__ void __launch_bounds__(POW_THREADS) pow_kernel(PowArgs a) {
  __shared__ unsigned long long s_start;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned long long b = atomicAdd(a.counter, 1ull);
      const unsigned long long off = b * POW_BLOCK;
      const unsigned long long st = a.start + off;
      const unsigned long long best = *reinterpret_cast<volatile unsigned long long*>(a.best);
      s_start = (off >= a.count || st >= best) ? ~0ull : st;
    }
    __syncthreads();
    const unsigned long long st = s_start;
    __syncthreads();
    if (st == ~0ull) return;
    // The best nonce so far is re-read before every hash (the read of one iteration is used by the
    // next, so its latency hides behind a hash): once a satisfying nonce at or below this thread's
    // next nonce is known, the rest of the block cannot lower the result and is skipped. Without
    // this, every block claimed before the first hit ran to completion (about one full wave of
    // nonces beyond the answer).
    unsigned long long known = *reinterpret_cast<volatile unsigned long long*>(a.best);
#pragma unroll 1
    for (int q = 0; q < POW_PER_THREAD; ++q) {
      const uint64_t off = (uint64_t)q * POW_THREADS + threadIdx.x;
      if (st - a.start + off >= a.count) break;
      const uint64_t nonce = st + off;
      if (nonce >= known) break;
      known = *reinterpret_cast<volatile unsigned long long*>(a.best);
      uint32_t h[8];
      if constexpr (KIND == HASH_BLAKE3) {
        blake3_pow_tail(a.pre, a.chal, (uint32_t)nonce, (uint32_t)(nonce >> 32), h[0], h[1]);
      } else {
        uint32_t m[16];
#pragma unroll
        for (int w = 0; w < 8; ++w) m[w] = a.chal[w];
        m[8] = (uint32_t)nonce;
        m[9] = (uint32_t)(nonce >> 32);
#pragma unroll
        for (int w = 10; w < 16; ++w) m[w] = 0;
        hash64<KIND>(m, h);
      }
      const uint64_t v = (uint64_t)h[0] | ((uint64_t)h[1] << 32);
      if (v <= a.threshold) atomicMin(a.best, (unsigned long long)nonce);
    }
  }
}

cudaError_t launch_pow(const uint32_t challenge[8], uint64_t threshold, uint64_t start, uint64_t count,
                       unsigned long long* best, int kind, cudaStream_t s) {
  PowArgs a;
  for (int i = 0; i < 8; ++i) a.chal[i] = challenge[i];
  blake3_pow_prefix(a.chal, a.pre);
  a.threshold = threshold;
  a.start = start;
  a.count = count;
  a.best = best;
  a.counter = best + 1;  // the caller provides two words: best nonce, block counter (both reset)
  unsigned grid = (unsigned)std::min<uint64_t>((count + POW_BLOCK - 1) / POW_BLOCK, 152ull * 8);
  switch (kind) {
    case HASH_BLAKE3: pow_kernel<HASH_BLAKE3><<<grid, 256, 0, s>>>(a); note_launch(); break;
    case HASH_SHA2: pow_kernel<HASH_SHA2><<<grid, 256, 0, s>>>(a); note_launch(); break;
    case HASH_SHA3: pow_kernel<HASH_SHA3><<<grid, 256, 0, s>>>(a); note_launch(); break;
    case HASH_KECCAK: pow_kernel<HASH_KECCAK><<<grid, 256, 0, s>>>(a); note_launch(); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------

__global__ void gather_digests_kernel(const uint32_t* nodes, const uint64_t* idx, uint64_t n, uint32_t* out) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n * 8; t += (uint64_t)gridDim.x * blockDim.x)
    out[t] = nodes[idx[t >> 3] * 8 + (t & 7)];
}
cudaError_t launch_gather_digests(const uint32_t* nodes, const uint64_t* idx, size_t n, uint32_t* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  unsigned grid = (unsigned)std::min<size_t>((n * 8 + 255) / 256, 4096);
  gather_digests_kernel<<<grid, 256, 0, s>>>(nodes, idx, n, out);
  note_launch();
  return cudaGetLastError();
}

}  // namespace whir
