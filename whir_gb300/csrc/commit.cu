// Commitment-side kernels: interleaved Reed–Solomon encode with the leaf hash fused into the
// kernel that writes each codeword row, Merkle layers, generic hash_many, proof-of-work search and
// opening gathers.
//
// Encode (reference ntt/cooley_tukey.rs:411-477). For message m, coset c in [0, K) and t in [0, C)
// the codeword row c*C + t, column m holds P_m(w_N^c * w_C^t) = NTT_C(x_j * w_N^(c j))[t]: the
// coset twist is applied while loading, the size-C NTT runs in shared memory (radix-2
// decimation-in-frequency, natural order in, bit-reversed order out), and each CTA finishes whole
// codeword rows so it can write them with coalesced stores and hash them straight from shared
// memory (matrix_commit.rs:211-232 leaf hashing, merkle_tree.rs:82-127 leaves).
// Large C is split four-step as C = C1 * C2: pass 1 (cols) runs NTT_C1 over strided columns,
// applies the w_C^(j2 k1) twiddles and writes an intermediate; pass 2 (rows) runs NTT_C2 over
// contiguous rows and emits codeword rows t = k1 + C1 * k2.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

#include "field.cuh"
#include "hash.cuh"
#include "kernels.hpp"
#include "roots.cuh"
#include "status.hpp"

namespace whir {

static unsigned long long g_launches = 0;
uint64_t kernel_launches() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }
void note_launch() { __atomic_fetch_add(&g_launches, 1ull, __ATOMIC_RELAXED); }

static constexpr int ENC_THREADS = 256;
static constexpr size_t ENC_SMEM_BUDGET = 64 * 1024;  // data bytes per CTA
static constexpr int ENC_MAX_LOGN_SMEM = 12;          // largest in-CTA NTT


// LOGR consecutive decimation-in-frequency stages done in registers. The current sub-blocks have
// size B = 2^logB; a work item (vector v, sub-block blk, offset j < B/R) owns the R = 2^LOGR
// elements at offsets j + k*B/R, k < R, which are exactly the elements those stages combine.
// Stage st pairs k with k + R/2^(st+1) and multiplies the difference by w_(2h)^(offset mod 2h),
// 2h = B / 2^st, read from tw[q] = w_n^q.
template <class F, int LOGR>
__device__ __forceinline__ void dif_step(F* s, int logn, int logB, int nvec, int lognvec, int vs, int es,
                                         bool vec_fastest, const Gl* tw) {
  constexpr int R = 1 << LOGR;
  const int logstride = logB - LOGR;
  const int stride = 1 << logstride;
  const int items_log = logn - LOGR;  // work items per vector = n / R
  const int total = nvec << items_log;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int v, it;
    if (vec_fastest) {
      v = t & (nvec - 1);
      it = t >> lognvec;
    } else {
      v = t >> items_log;
      it = t & ((1 << items_log) - 1);
    }
    const int blk = it >> logstride, j = it & (stride - 1);
    F* base = s + v * vs + (((blk << logB) + j) * es);
    const int kstep = stride * es;
    F x[R];
#pragma unroll
    for (int k = 0; k < R; ++k) x[k] = base[k * kstep];
#pragma unroll
    for (int st = 0; st < LOGR; ++st) {
      const int half = R >> (st + 1);
      const int log2h = logB - st;
      const int tws = logn - log2h;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        if (k & half) continue;
        const int pos = (j + k * stride) & ((1 << log2h) - 1);
        const F u = x[k], w = x[k + half];
        x[k] = u + w;
        x[k + half] = (u - w).mul_base(tw[pos << tws]);
      }
    }
#pragma unroll
    for (int k = 0; k < R; ++k) base[k * kstep] = x[k];
  }
  __syncthreads();
}

// In-place DIF NTT of nvec vectors of size 2^logn in shared memory; element i of vector v lives at
// s[v*vs + i*es]. Output index k ends up at position brev(k). Stages are processed three at a time
// in registers (radix 8), with a radix-4 / radix-2 step for the remainder.
template <class F>
__device__ void smem_ntt_dif(F* s, int logn, int nvec, int vs, int es, bool vec_fastest, const Gl* tw) {
  int lognvec = 0;
  while ((1 << lognvec) < nvec) ++lognvec;
  int logB = logn;
  while (logB >= 3) {
    dif_step<F, 3>(s, logn, logB, nvec, lognvec, vs, es, vec_fastest, tw);
    logB -= 3;
  }
  if (logB == 2) dif_step<F, 2>(s, logn, logB, nvec, lognvec, vs, es, vec_fastest, tw);
  if (logB == 1) dif_step<F, 1>(s, logn, logB, nvec, lognvec, vs, es, vec_fastest, tw);
}

template <class F>
__device__ __forceinline__ void push_elem_words(const F& x, uint32_t* w);
template <>
__device__ __forceinline__ void push_elem_words<Gl>(const Gl& x, uint32_t* w) {
  w[0] = (uint32_t)x.v;
  w[1] = (uint32_t)(x.v >> 32);
}
template <>
__device__ __forceinline__ void push_elem_words<Gl2>(const Gl2& x, uint32_t* w) {
  w[0] = (uint32_t)x.c0;
  w[1] = (uint32_t)(x.c0 >> 32);
  w[2] = (uint32_t)x.c1;
  w[3] = (uint32_t)(x.c1 >> 32);
}
template <>
__device__ __forceinline__ void push_elem_words<Gl3>(const Gl3& x, uint32_t* w) {
  w[0] = (uint32_t)x.c0;
  w[1] = (uint32_t)(x.c0 >> 32);
  w[2] = (uint32_t)x.c1;
  w[3] = (uint32_t)(x.c1 >> 32);
  w[4] = (uint32_t)x.c2;
  w[5] = (uint32_t)(x.c2 >> 32);
}

template <class F>
struct EncArgs {
  const F* src;  // rows mode 0: messages; rows mode 1: intermediate; cols: messages
  F* dst;        // rows: codeword; cols: intermediate
  uint32_t* leaves;
  uint64_t msg_len;
  uint64_t K;  // number of cosets
  int M;       // messages = codeword columns
  int logC, logN, logC1, logC2;
  int mode;    // rows kernel: 0 single pass, 1 four-step pass 2
  int G;       // cosets per CTA (rows mode 0)
  int W;       // columns per CTA (cols kernel)
  RootTab rt;
};

// Produces whole codeword rows: writes them and (optionally) their leaf digests.
template <class F, int KIND>
__global__ void __launch_bounds__(ENC_THREADS) encode_rows_kernel(EncArgs<F> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  F* s = reinterpret_cast<F*>(smem_raw);
  const int M = a.M;
  const int logn = a.mode == 0 ? a.logC : a.logC2;
  const int n = 1 << logn;
  const int nvec = a.mode == 0 ? a.G * M : M;
  const int R = a.mode == 0 ? a.G * n : n;  // rows produced by this CTA
  Gl* tw = reinterpret_cast<Gl*>(smem_raw + (size_t)nvec * n * sizeof(F));
  const uint64_t C = 1ull << a.logC, N = 1ull << a.logN;
  for (int k = threadIdx.x; k < (n >> 1); k += blockDim.x) tw[k] = root_pow(a.rt, logn, (uint64_t)k);

  uint64_t c_base = 0, k1 = 0;
  if (a.mode == 0) {
    c_base = (uint64_t)blockIdx.x * a.G;
    for (int idx = threadIdx.x; idx < nvec * n; idx += blockDim.x) {
      const int vec = idx >> logn, j = idx & (n - 1);
      const int g = vec / M, m = vec - g * M;
      const uint64_t c = c_base + g;
      F x = (uint64_t)j < a.msg_len ? a.src[(uint64_t)m * a.msg_len + j] : F::zero();
      if (c != 0 && j != 0) x = x.mul_base(root_pow(a.rt, a.logN, (c * (uint64_t)j) & (N - 1)));
      s[idx] = x;
    }
  } else {
    const uint64_t C1 = 1ull << a.logC1;
    c_base = blockIdx.x >> a.logC1;
    k1 = blockIdx.x & (C1 - 1);
    for (int idx = threadIdx.x; idx < M * n; idx += blockDim.x) {
      const int m = idx >> logn, j2 = idx & (n - 1);
      s[idx] = a.src[((((uint64_t)m * a.K + c_base) << a.logC1) + k1) * n + j2];
    }
  }
  __syncthreads();
  smem_ntt_dif<F>(s, logn, nvec, n, 1, false, tw);

  // Coalesced row stores: consecutive threads write consecutive columns of consecutive rows.
  for (int idx = threadIdx.x; idx < R * M; idx += blockDim.x) {
    const int rho = idx / M, m = idx - rho * M;
    uint64_t row;
    int sidx;
    if (a.mode == 0) {
      const int g = rho >> logn, t = rho & (n - 1);
      row = (c_base + g) * C + t;
      sidx = ((g * M + m) << logn) + brev(t, logn);
    } else {
      row = c_base * C + k1 + ((uint64_t)rho << a.logC1);
      sidx = (m << logn) + brev(rho, logn);
    }
    a.dst[row * M + m] = s[sidx];
  }
  if (a.leaves == nullptr) return;
  // One thread per row: hash the row's canonical little-endian bytes.
  for (int rho = threadIdx.x; rho < R; rho += blockDim.x) {
    uint64_t row;
    int base, g = 0, t = rho;
    if (a.mode == 0) {
      g = rho >> logn;
      t = rho & (n - 1);
      row = (c_base + g) * C + t;
      base = ((g * M) << logn) + brev(t, logn);
    } else {
      row = c_base * C + k1 + ((uint64_t)rho << a.logC1);
      base = brev(rho, logn);
    }
    uint32_t out[8];
    if constexpr (KIND == HASH_BLAKE3) {
      // Message blocks assembled in registers (static indices) straight from shared memory:
      // block b holds u64 limbs 8b .. 8b+7 of the row (limb L = limb L % LIMBS of column L / LIMBS).
      const int limbs = M * F::LIMBS;
      const int nblocks = limbs == 0 ? 1 : (limbs + 7) / 8;
      blake3_iv(out);
      for (int b = 0; b < nblocks; ++b) {
        uint32_t mw[16];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int L = b * 8 + q;
          uint64_t limb = 0;
          if (L < limbs) {
            const int col = L / F::LIMBS, part = L - col * F::LIMBS;
            limb = reinterpret_cast<const uint64_t*>(&s[base + (col << logn)])[part];
          }
          mw[2 * q] = (uint32_t)limb;
          mw[2 * q + 1] = (uint32_t)(limb >> 32);
        }
        const bool last = b == nblocks - 1;
        const uint32_t blen = last ? (uint32_t)(limbs - b * 8) * 8 : 64;
        const uint32_t flags = (b == 0 ? B3_CHUNK_START : 0) | (last ? (B3_CHUNK_END | B3_ROOT) : 0);
        blake3_compress_cv(out, mw, 0, 0, blen, flags);
      }
    } else {
      WordHasher<KIND> h;
      h.init((uint32_t)(M * F::LIMBS * 8));
      for (int m = 0; m < M; ++m) {
        uint32_t w[2 * F::LIMBS];
        push_elem_words<F>(s[base + (m << logn)], w);
#pragma unroll
        for (int q = 0; q < 2 * F::LIMBS; ++q) h.push(w[q]);
      }
      h.finish(out);
    }
    uint4* dstw = reinterpret_cast<uint4*>(a.leaves + row * 8);
    dstw[0] = make_uint4(out[0], out[1], out[2], out[3]);
    dstw[1] = make_uint4(out[4], out[5], out[6], out[7]);
  }
}

// Four-step pass 1: NTT_C1 over columns j2 of the (C1 x C2) view of each twisted message,
// multiplied by w_C^(j2 k1); intermediate layout [m][c][k1][j2].
template <class F>
__global__ void __launch_bounds__(ENC_THREADS) encode_cols_kernel(EncArgs<F> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  F* s = reinterpret_cast<F*>(smem_raw);
  const int logn = a.logC1, n = 1 << logn, W = a.W;
  Gl* tw = reinterpret_cast<Gl*>(smem_raw + (size_t)W * n * sizeof(F));
  const uint64_t C2 = 1ull << a.logC2, N = 1ull << a.logN;
  const uint64_t tiles = C2 / W;
  const uint64_t tile = blockIdx.x % tiles;
  const uint64_t mc = blockIdx.x / tiles;  // m * K + c
  const uint64_t c = mc % a.K, m = mc / a.K;
  for (int k = threadIdx.x; k < (n >> 1); k += blockDim.x) tw[k] = root_pow(a.rt, logn, (uint64_t)k);
  for (int idx = threadIdx.x; idx < n * W; idx += blockDim.x) {
    const int j1 = idx / W, w = idx - j1 * W;
    const uint64_t j = ((uint64_t)j1 << a.logC2) + tile * W + w;
    F x = j < a.msg_len ? a.src[m * a.msg_len + j] : F::zero();
    if (c != 0 && j != 0) x = x.mul_base(root_pow(a.rt, a.logN, (c * j) & (N - 1)));
    s[idx] = x;
  }
  __syncthreads();
  smem_ntt_dif<F>(s, logn, W, 1, W, true, tw);
  for (int idx = threadIdx.x; idx < n * W; idx += blockDim.x) {
    const int k1 = idx / W, w = idx - k1 * W;
    const uint64_t j2 = tile * W + w;
    F v = s[brev(k1, logn) * W + w];
    const uint64_t e = j2 * (uint64_t)k1;
    if (e) v = v.mul_base(root_pow(a.rt, a.logC, e));
    a.dst[((mc << a.logC1) + k1) * C2 + j2] = v;
  }
}

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

template <class F, int KIND>
static cudaError_t run_rows(const EncArgs<F>& a, unsigned grid, size_t smem, cudaStream_t s) {
  // Set on every launch: the attribute is per device and this may run from several host threads.
  cudaError_t e = cudaFuncSetAttribute(encode_rows_kernel<F, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(ENC_SMEM_BUDGET + 32 * 1024));
  if (e != cudaSuccess) return e;
  encode_rows_kernel<F, KIND><<<grid, ENC_THREADS, smem, s>>>(a);
  note_launch();
  return cudaGetLastError();
}

template <class F>
static cudaError_t dispatch_rows(const EncArgs<F>& a, int kind, unsigned grid, size_t smem, cudaStream_t s) {
  switch (kind) {
    case HASH_BLAKE3: return run_rows<F, HASH_BLAKE3>(a, grid, smem, s);
    case HASH_SHA2: return run_rows<F, HASH_SHA2>(a, grid, smem, s);
    case HASH_SHA3: return run_rows<F, HASH_SHA3>(a, grid, smem, s);
    case HASH_KECCAK: return run_rows<F, HASH_KECCAK>(a, grid, smem, s);
    default: return run_rows<F, HASH_COPY>(a, grid, smem, s);
  }
}

template <class F>
cudaError_t launch_encode(const EncodePlan& p, const F* src, size_t n_msgs, size_t msg_len, F* dst,
                          uint32_t* leaves, int hash_kind, F* scratch, RootTab rt, cudaStream_t s) {
  EncArgs<F> a;
  a.leaves = leaves;
  a.msg_len = msg_len;
  a.M = (int)n_msgs;
  a.logC = p.logC;
  a.logN = p.logN;
  a.logC1 = p.logC1;
  a.logC2 = p.logC2;
  a.K = 1ull << (p.logN - p.logC);
  a.G = p.cosets_per_cta;
  a.W = p.cols_per_cta;
  a.rt = rt;
  if (p.mode == 0) {
    a.mode = 0;
    a.src = src;
    a.dst = dst;
    const size_t n = 1ull << p.logC;
    const size_t smem = (size_t)a.G * n_msgs * n * sizeof(F) + (n / 2) * sizeof(Gl) + 16;
    return dispatch_rows<F>(a, hash_kind, (unsigned)(a.K / a.G), smem, s);
  }
  // pass 1
  {
    cudaError_t ea = cudaFuncSetAttribute(encode_cols_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(ENC_SMEM_BUDGET + 32 * 1024));
    if (ea != cudaSuccess) return ea;
    EncArgs<F> c = a;
    c.src = src;
    c.dst = scratch;
    c.leaves = nullptr;
    const size_t C1 = 1ull << p.logC1, C2 = 1ull << p.logC2;
    const size_t smem = (size_t)a.W * C1 * sizeof(F) + (C1 / 2) * sizeof(Gl) + 16;
    const size_t grid = n_msgs * a.K * (C2 / a.W);
    encode_cols_kernel<F><<<(unsigned)grid, ENC_THREADS, smem, s>>>(c);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  // pass 2
  a.mode = 1;
  a.src = scratch;
  a.dst = dst;
  const size_t C1 = 1ull << p.logC1, C2 = 1ull << p.logC2;
  const size_t smem = n_msgs * C2 * sizeof(F) + (C2 / 2) * sizeof(Gl) + 16;
  return dispatch_rows<F>(a, hash_kind, (unsigned)(a.K * C1), smem, s);
}

template cudaError_t launch_encode<Gl>(const EncodePlan&, const Gl*, size_t, size_t, Gl*, uint32_t*, int, Gl*,
                                       RootTab, cudaStream_t);
template cudaError_t launch_encode<Gl2>(const EncodePlan&, const Gl2*, size_t, size_t, Gl2*, uint32_t*, int, Gl2*,
                                        RootTab, cudaStream_t);
template cudaError_t launch_encode<Gl3>(const EncodePlan&, const Gl3*, size_t, size_t, Gl3*, uint32_t*, int, Gl3*,
                                        RootTab, cudaStream_t);

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
#pragma unroll 1
    for (int q = 0; q < POW_PER_THREAD; ++q) {
      const uint64_t off = (uint64_t)q * POW_THREADS + threadIdx.x;
      if (st - a.start + off >= a.count) break;
      const uint64_t nonce = st + off;
      uint32_t m[16];
#pragma unroll
      for (int w = 0; w < 8; ++w) m[w] = a.chal[w];
      m[8] = (uint32_t)nonce;
      m[9] = (uint32_t)(nonce >> 32);
#pragma unroll
      for (int w = 10; w < 16; ++w) m[w] = 0;
      uint32_t h[8];
      hash64<KIND>(m, h);
      const uint64_t v = (uint64_t)h[0] | ((uint64_t)h[1] << 32);
      if (v <= a.threshold) atomicMin(a.best, (unsigned long long)nonce);
    }
  }
}

cudaError_t launch_pow(const uint32_t challenge[8], uint64_t threshold, uint64_t start, uint64_t count,
                       unsigned long long* best, int kind, cudaStream_t s) {
  PowArgs a;
  for (int i = 0; i < 8; ++i) a.chal[i] = challenge[i];
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
// Opening gathers
// ---------------------------------------------------------------------------------------------
template <class F>
__global__ void gather_rows_kernel(const F* matrix, uint64_t cols, const uint64_t* idx, uint64_t n, F* out) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n * cols; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = t / cols, c = t - i * cols;
    out[t] = matrix[idx[i] * cols + c];
  }
}
template <class F>
cudaError_t launch_gather_rows(const F* matrix, size_t cols, const uint64_t* idx, size_t n, F* out, cudaStream_t s) {
  if (n * cols == 0) return cudaSuccess;
  unsigned grid = (unsigned)std::min<size_t>((n * cols + 255) / 256, 4096);
  gather_rows_kernel<F><<<grid, 256, 0, s>>>(matrix, cols, idx, n, out);
  note_launch();
  return cudaGetLastError();
}
template cudaError_t launch_gather_rows<Gl>(const Gl*, size_t, const uint64_t*, size_t, Gl*, cudaStream_t);
template cudaError_t launch_gather_rows<Gl2>(const Gl2*, size_t, const uint64_t*, size_t, Gl2*, cudaStream_t);
template cudaError_t launch_gather_rows<Gl3>(const Gl3*, size_t, const uint64_t*, size_t, Gl3*, cudaStream_t);

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
