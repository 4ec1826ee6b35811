// Interleaved Reed–Solomon encode kernels, shared by the translation units that instantiate them
// for the Goldilocks family (commit.cu) and for the Montgomery fields (commit_mont.cu).
//
// Encode (reference ntt/cooley_tukey.rs:411-477). For message m, coset c in [0, K) and t in [0, C)
// the codeword row c*C + t, column m holds P_m(w_N^c * w_C^t) = NTT_C(x_j * w_N^(c j))[t]: the
// coset twist is applied while loading, the size-C NTT runs in shared memory (radix-8/4/2
// decimation-in-frequency steps in registers, natural order in, bit-reversed order out), and each
// CTA finishes whole codeword rows so it can write them with coalesced stores and hash them
// straight from shared memory (matrix_commit.rs:211-232 leaf hashing, merkle_tree.rs:82-127 leaves).
// Large C is split four-step as C = C1 * C2: pass 1 (cols) runs NTT_C1 over strided columns,
// applies the w_C^(j2 k1) twiddles and writes an intermediate; pass 2 (rows) runs NTT_C2 over
// contiguous rows and emits codeword rows t = k1 + C1 * k2.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "field.cuh"
#include "hash.cuh"
#include "kernels.hpp"
#include "roots.cuh"
#include "status.hpp"

namespace whir {

static constexpr int ENC_THREADS = 256;
static constexpr size_t ENC_SMEM_BUDGET = 64 * 1024;  // data bytes per CTA
static constexpr int ENC_MAX_LOGN_SMEM = ENC_MAX_NTT_LOG;  // largest in-CTA NTT
// Dynamic shared memory limit set on the encode kernels: the data tile plus at most as many bytes
// of twiddles (n - 1 base elements for a size-n NTT) plus alignment slack.
static constexpr size_t ENC_SMEM_ATTR = 2 * ENC_SMEM_BUDGET + 256;


// Shared-memory element index swizzle: the low SB bits of an element index are XORed with the XOR
// of its higher SB-bit groups (a bijection within each aligned block of 2^SB elements). The NTT
// steps' power-of-two strides, the bit-reversed row order of the row stores and of the leaf hashing,
// and the interleaved columns of the four-step pass then spread over the 32 banks instead of
// landing on one or two.
template <class F>
struct SwzBits {
  static constexpr int value = sizeof(F) == 16 ? 3 : (sizeof(F) == 32 ? 2 : 4);
};
template <class F>
__device__ __forceinline__ int swz(int L) {
  constexpr int SB = SwzBits<F>::value;
  int h = 0;
#pragma unroll
  for (int sh = SB; sh < 15; sh += SB) h ^= L >> sh;
  return L ^ (h & ((1 << SB) - 1));
}
// Shared-memory element access, 16-byte vectorised where the element size allows it.
template <class F>
__device__ __forceinline__ F lds(const F* s, int i) {
  if constexpr (sizeof(F) % 16 == 0) {
    F r;
    const ulonglong2* p = reinterpret_cast<const ulonglong2*>(s + i);
    ulonglong2* d = reinterpret_cast<ulonglong2*>(&r);
#pragma unroll
    for (int q = 0; q < (int)(sizeof(F) / 16); ++q) d[q] = p[q];
    return r;
  } else {
    return s[i];
  }
}
template <class F>
__device__ __forceinline__ void sts(F* s, int i, const F& x) {
  if constexpr (sizeof(F) % 16 == 0) {
    ulonglong2* p = reinterpret_cast<ulonglong2*>(s + i);
    const ulonglong2* d = reinterpret_cast<const ulonglong2*>(&x);
#pragma unroll
    for (int q = 0; q < (int)(sizeof(F) / 16); ++q) p[q] = d[q];
  } else {
    s[i] = x;
  }
}

// NTT twiddles by butterfly span: level L (span 2h = 2^L) holds w_(2h)^q for q < h at offset h - 1,
// so the threads of a warp read consecutive entries. The table is in shared memory, or (TWG) read
// through L1 from the global copy.
template <class B, bool TWG>
__device__ __forceinline__ B tw_at(const B* tw, int i) {
  if constexpr (TWG) {
    return ldg_elem(tw + i);
  } else {
    return tw[i];
  }
}

// LOGR consecutive decimation-in-frequency stages done in registers. The current sub-blocks have
// size B = 2^logB; a work item (vector v, sub-block blk, offset j < B/R) owns the R = 2^LOGR
// elements at offsets j + k*B/R, k < R, which are exactly the elements those stages combine.
// Stage st pairs k with k + R/2^(st+1) and multiplies the difference by w_(2h)^(offset mod 2h),
// 2h = B / 2^st.
// LAST marks the final step (B = R, so j = 0): its twiddles are w_(2h)^kk for 2h <= R, the R - 1
// first table entries, held in registers; the kk = 0 ones are 1 and their products are skipped
// (7 of the 12 products of a radix-8 step, 3 of 4 for radix 4, all of radix 2).
template <class F, int LOGR, bool TWG, bool LAST>
__device__ __forceinline__ void dif_step(F* s, int logn, int logB, int nvec, int lognvec, int vs, int es,
                                         bool vec_fastest, const typename F::Base* tw) {
  constexpr int R = 1 << LOGR;
  typedef typename F::Base B;
  B lt[R > 2 ? R - 1 : 1];
  if constexpr (LAST) {
#pragma unroll
    for (int i = 1; i < R - 1; ++i) lt[i] = tw_at<B, TWG>(tw, i);
  }
  const int logstride = logB - LOGR;
  const int stride = 1 << logstride;
  const int items_log = logn - LOGR;  // work items per vector = n / R
  const int total = nvec << items_log;
  const int kstep = stride * es;
  // swz is linear over GF(2), and an element index is the sum of disjoint bit fields (vector, block,
  // offset j < stride, k * stride, each scaled by the power-of-two strides vs / es), so
  // swz(base + k * kstep) = swz(base) ^ swz(k * kstep): the R per-k terms are shared by every work
  // item of the step, and an index costs one XOR.
  int kswz[R];
#pragma unroll
  for (int k = 0; k < R; ++k) kswz[k] = swz<F>(k * kstep);
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
    const int sbase = swz<F>(v * vs + (((blk << logB) + j) * es));
    int pidx[R];
    F x[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
      pidx[k] = sbase ^ kswz[k];
      x[k] = lds(s, pidx[k]);
    }
#pragma unroll
    for (int st = 0; st < LOGR; ++st) {
      const int half = R >> (st + 1);
      const int log2h = logB - st;
      // w_(2h)^pos with pos = (j + k * stride) mod 2^log2h = j + (k mod 2^(LOGR - st)) * stride.
      const int tw0 = (1 << (log2h - 1)) - 1 + j;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        if (k & half) continue;
        const int kk = k & ((1 << (LOGR - st)) - 1);
        const F u = x[k], w = x[k + half];
        x[k] = u + w;
        if constexpr (LAST) {
          x[k + half] = kk == 0 ? u - w : (u - w).mul_base(lt[(1 << (LOGR - st - 1)) - 1 + kk]);
        } else {
          x[k + half] = (u - w).mul_base(tw_at<B, TWG>(tw, tw0 + kk * stride));
        }
      }
    }
#pragma unroll
    for (int k = 0; k < R; ++k) sts(s, pidx[k], x[k]);
  }
  __syncthreads();
}

// In-place DIF NTT of nvec vectors of size 2^logn in shared memory; element i of vector v lives at
// s[swz(v*vs + i*es)]. Output index k ends up at position brev(k). Stages are processed three at a
// time in registers (radix 8), with a radix-4 / radix-2 step for the remainder.
template <class F, bool TWG>
__device__ void smem_ntt_dif(F* s, int logn, int nvec, int vs, int es, bool vec_fastest, const typename F::Base* tw) {
  int lognvec = 0;
  while ((1 << lognvec) < nvec) ++lognvec;
  // The radix-4 / radix-2 remainder goes first, so the last step is radix 8 whenever logn >= 3: its
  // twiddles are then 5 constant products per 8 elements, and its stride-1 accesses in the column
  // pass's interleaved layout (element v + i W) stay clear of bank conflicts after the swizzle.
  int logB = logn;
  if (logB > 3 && logB % 3 == 2) {
    dif_step<F, 2, TWG, false>(s, logn, logB, nvec, lognvec, vs, es, vec_fastest, tw);
    logB -= 2;
  } else if (logB > 3 && logB % 3 == 1) {
    dif_step<F, 1, TWG, false>(s, logn, logB, nvec, lognvec, vs, es, vec_fastest, tw);
    logB -= 1;
  }
  while (logB > 3) {
    dif_step<F, 3, TWG, false>(s, logn, logB, nvec, lognvec, vs, es, vec_fastest, tw);
    logB -= 3;
  }
  if (logB == 3) dif_step<F, 3, TWG, true>(s, logn, logB, nvec, lognvec, vs, es, vec_fastest, tw);
  if (logB == 2) dif_step<F, 2, TWG, true>(s, logn, logB, nvec, lognvec, vs, es, vec_fastest, tw);
  if (logB == 1) dif_step<F, 1, TWG, true>(s, logn, logB, nvec, lognvec, vs, es, vec_fastest, tw);
}

// Copies the twiddle levels 1..logn (entries [0, 2^logn - 1)) of the global table into shared memory.
template <class B>
__device__ __forceinline__ void load_twiddles(B* tw, const RootTab& rt, int logn) {
  const B* g = reinterpret_cast<const B*>(rt.ntt);
  for (int k = threadIdx.x; k < (1 << logn) - 1; k += blockDim.x) tw[k] = ldg_elem(g + k);
}

// 32-bit little-endian words of an element's u64 limbs (the element must already be canonical).
template <class F>
__device__ __forceinline__ void push_elem_words(const F& x, uint32_t* w) {
  const uint64_t* l = reinterpret_cast<const uint64_t*>(&x);
#pragma unroll
  for (int i = 0; i < F::LIMBS; ++i) {
    w[2 * i] = (uint32_t)l[i];
    w[2 * i + 1] = (uint32_t)(l[i] >> 32);
  }
}

// Quotient by the message count through its reciprocal (exact for the tile indices used here: they
// are below 2^13 and M <= 2^13, so i * M < 2^32); a runtime integer division costs ~20 instructions
// per element.
__device__ __forceinline__ int div_m(int i, uint64_t magic) { return (int)(((uint64_t)(uint32_t)i * magic) >> 32); }
inline uint64_t m_magic_of(uint64_t M) { return M ? ((1ull << 32) + M - 1) / M : 0; }

template <class F>
struct EncArgs {
  const F* src;  // rows mode 0: messages; rows mode 1: intermediate; cols: messages
  F* dst;        // rows: codeword; cols: intermediate
  uint32_t* leaves;
  uint64_t msg_len;
  uint64_t K;  // number of cosets
  int M;       // messages = codeword columns
  uint64_t m_magic;  // ceil(2^32 / M): i / M = (i * m_magic) >> 32 exactly for i * M < 2^32
  int logC, logN, logC1, logC2;
  int mode;    // rows kernel: 0 single pass, 1 four-step pass 2
  uint64_t add_rows;  // rows kernel without leaves: 0 stores the codeword; else adds rows < add_rows into dst
  int G;       // cosets per CTA (rows mode 0)
  int W;       // columns per CTA (cols kernel)
  RootTab rt;
};

// Produces whole codeword rows: writes them and (optionally) their leaf digests.
// Minimum resident CTAs per SM for the encode kernels: three for elements of up to 16 bytes (their
// 64 KB tiles fit three per SM; the register cap is then 85), two for the 24- and 32-byte fields
// (without a bound the 4-limb Montgomery field took ~165 registers per thread, one CTA per SM,
// measured 44 % slower).
template <class F>
struct EncMinCtas {
  static constexpr int value = sizeof(F) <= 16 ? 3 : 2;
};

template <class F, int KIND>
__device__ __forceinline__ void encode_rows_body(const EncArgs<F>& a, uint64_t bid, unsigned char* smem_raw) {
  F* s = reinterpret_cast<F*>(smem_raw);
  const int M = a.M;
  const int logn = a.mode == 0 ? a.logC : a.logC2;
  const int n = 1 << logn;
  const int nvec = a.mode == 0 ? a.G * M : M;
  const int R = a.mode == 0 ? a.G * n : n;  // rows produced by this CTA
  typedef typename F::Base B;
  B* tw = reinterpret_cast<B*>(smem_raw + (size_t)nvec * n * sizeof(F));
  const uint64_t C = 1ull << a.logC, N = 1ull << a.logN;
  load_twiddles<B>(tw, a.rt, logn);

  uint64_t c_base = 0, k1 = 0;
  if (a.mode == 0) {
    c_base = bid * a.G;
    #pragma unroll 4
    for (int idx = threadIdx.x; idx < nvec * n; idx += blockDim.x) {
      const int vec = idx >> logn, j = idx & (n - 1);
      const int g = div_m(vec, a.m_magic), m = vec - g * M;
      const uint64_t c = c_base + g;
      F x = (uint64_t)j < a.msg_len ? a.src[(uint64_t)m * a.msg_len + j] : F::zero();
      if (c != 0 && j != 0) x = x.mul_base(root_pow<B>(a.rt, a.logN, (c * (uint64_t)j) & (N - 1)));
      sts(s, swz<F>(idx), x);
    }
  } else {
    const uint64_t C1 = 1ull << a.logC1;
    c_base = bid >> a.logC1;
    k1 = bid & (C1 - 1);
    // Column factor w_N^(j2 (c + K k1)) of the four-step split (see encode_cols_body): one power
    // per column j2, shared by the M messages; all ones for c = k1 = 0.
    const uint64_t e = c_base + a.K * k1;
    const F* src = a.src + (((uint64_t)c_base << a.logC1) + k1) * n;
    const uint64_t mstride = (a.K << a.logC1) * (uint64_t)n;  // one message's intermediate block
    // Shared index (m << logn) + j2 with j2 < n: swz of it is swz(j2) ^ swz(m << logn), the second
    // term the same for every thread.
    if (n >= ENC_THREADS) {
      for (int j2 = threadIdx.x; j2 < n; j2 += ENC_THREADS) {
        const B f = root_pow<B>(a.rt, a.logN, (e * (uint64_t)j2) & (N - 1));
        const int sj = swz<F>(j2);
        const F* p = src + j2;
        #pragma unroll 4
        for (int m = 0; m < M; ++m) {
          F x = *p;
          p += mstride;
          if (e != 0) x = x.mul_base(f);
          sts(s, sj ^ swz<F>(m << logn), x);
        }
      }
    } else {
      // idx = threadIdx.x + ENC_THREADS i: column j2 fixed, message advancing by ENC_THREADS / n
      const int j2 = threadIdx.x & (n - 1);
      const B f = root_pow<B>(a.rt, a.logN, (e * (uint64_t)j2) & (N - 1));
      const int st = swz<F>(threadIdx.x), iters = (M * n + ENC_THREADS - 1) / ENC_THREADS;
      const F* p = src + (uint64_t)(threadIdx.x >> logn) * mstride + j2;
      const uint64_t pstep = (uint64_t)(ENC_THREADS >> logn) * mstride;
      #pragma unroll 4
      for (int i = 0; i < iters; ++i) {
        if (threadIdx.x + i * ENC_THREADS < M * n) {
          F x = *p;
          if (e != 0) x = x.mul_base(f);
          sts(s, st ^ swz<F>(i * ENC_THREADS), x);
        }
        p += pstep;
      }
    }
  }
  __syncthreads();
  smem_ntt_dif<F, false>(s, logn, nvec, n, 1, false, tw);

  // Coalesced row stores: consecutive threads write consecutive columns of consecutive rows.
  const bool m_pow2 = (M & (M - 1)) == 0;
  if (a.mode == 1 && m_pow2 && M <= ENC_THREADS) {
    // idx = threadIdx.x + ENC_THREADS i = rho M + m: the column m is fixed per thread and rho advances
    // by rs = ENC_THREADS / M. brev(rho) = brev(rho0) ^ brev(i rs) (rho0 < rs), so the shared index
    // (m << logn) + brev(rho) is the thread's first one XOR a term shared by all threads.
    const int logM = __ffs(M) - 1, m = threadIdx.x & (M - 1), rho0 = threadIdx.x >> logM;
    const int rs = ENC_THREADS >> logM, iters = (R * M + ENC_THREADS - 1) / ENC_THREADS;
    const int sb = swz<F>((m << logn) + brev(rho0, logn));
    const uint64_t row0 = c_base * C + k1 + ((uint64_t)rho0 << a.logC1), rstep = (uint64_t)rs << a.logC1;
    F* q = a.dst + row0 * M + m;
    const uint64_t qstep = rstep * M;
    if (a.add_rows) {
      for (int i = 0; i < iters; ++i) {
        if (threadIdx.x + i * ENC_THREADS < R * M && row0 + i * rstep < a.add_rows)
          *q = *q + lds(s, sb ^ swz<F>(brev(i * rs, logn)));
        q += qstep;
      }
    } else {
      #pragma unroll 4
      for (int i = 0; i < iters; ++i) {
        if (threadIdx.x + i * ENC_THREADS < R * M) *q = lds(s, sb ^ swz<F>(brev(i * rs, logn)));
        q += qstep;
      }
    }
  } else {
    #pragma unroll 4
    for (int idx = threadIdx.x; idx < R * M; idx += blockDim.x) {
      const int rho = div_m(idx, a.m_magic), m = idx - rho * M;
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
      if (a.add_rows == 0)
        a.dst[row * M + m] = lds(s, swz<F>(sidx));
      else if (row < a.add_rows)
        a.dst[row * M + m] = a.dst[row * M + m] + lds(s, swz<F>(sidx));
    }
  }
  if (a.leaves == nullptr) return;
  if constexpr (!Canon<F>::IDENTITY) {
    // Leaves hash canonical bytes: convert the tile in place once every row has been stored.
    __syncthreads();
    for (int idx = threadIdx.x; idx < nvec * n; idx += blockDim.x) {
      uint64_t c[F::LIMBS];
      Canon<F>::to(s[idx], c);
      uint64_t* d = reinterpret_cast<uint64_t*>(&s[idx]);
#pragma unroll
      for (int q = 0; q < F::LIMBS; ++q) d[q] = c[q];
    }
    __syncthreads();
  }
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
    // Column col of the row sits at base + (col << logn); when that sum has disjoint bit fields
    // (always in mode 1, where base < n; in mode 0 when M is a power of two) its swizzle is
    // swz(base) ^ swz(col << logn), the second term shared by all threads.
    const bool lin = a.mode == 1 || m_pow2;
    const int sbase = swz<F>(base);
    auto col_idx = [&](int col) { return lin ? sbase ^ swz<F>(col << logn) : swz<F>(base + (col << logn)); };
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
            limb = reinterpret_cast<const uint64_t*>(&s[col_idx(col)])[part];
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
        push_elem_words<F>(lds(s, col_idx(m)), w);
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

template <class F, int KIND>
__global__ void __launch_bounds__(ENC_THREADS, EncMinCtas<F>::value) encode_rows_kernel(EncArgs<F> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  encode_rows_body<F, KIND>(a, blockIdx.x, smem_raw);
}

// One encode pass over several jobs (independent codewords of possibly different shapes) in one
// launch: job j owns CTAs [jobs[j].cta_begin, jobs[j + 1].cta_begin) of the grid.
template <class F>
struct EncJob {
  EncArgs<F> args;
  uint64_t cta_begin;
};
template <class F>
__device__ __forceinline__ int enc_job_of(const EncJob<F>* jobs, int njobs, uint64_t bid) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].cta_begin <= bid)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}
template <class F, int KIND>
__global__ void __launch_bounds__(ENC_THREADS, EncMinCtas<F>::value) encode_rows_multi_kernel(const EncJob<F>* jobs,
                                                                                             int njobs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int j = enc_job_of(jobs, njobs, blockIdx.x);
  const EncArgs<F> a = jobs[j].args;
  encode_rows_body<F, KIND>(a, blockIdx.x - jobs[j].cta_begin, smem_raw);
}

// w_(2^lvl)^e for e < 2^lvl: from the in-CTA twiddle table (level lvl holds w^q for q < 2^(lvl-1),
// and w^(q + 2^(lvl-1)) = -w^q) when it has that level, else from the two root tables.
template <class B>
__device__ __forceinline__ B level_root(const RootTab& rt, int lvl, uint64_t e) {
  if (lvl <= NTT_TW_LEVELS) {
    const uint64_t h = 1ull << (lvl - 1);
    const B* t = reinterpret_cast<const B*>(rt.ntt) + (h - 1);
    return e < h ? ldg_elem(t + e) : -ldg_elem(t + (e - h));
  }
  return root_pow<B>(rt, lvl, e);
}

// Four-step pass 1: NTT_C1 over columns j2 of the (C1 x C2) view of each twisted message;
// intermediate layout [m][c][k1][j2].
// With j = j1 C2 + j2 and t = k1 + C1 k2 the codeword value is
//   sum_j2 w_C2^(k2 j2) * w_N^(j2 (c + K k1)) * sum_j1 w_C1^(k1 j1) * w_N^(c j1 C2) * x_j
// (w_C = w_N^K): this pass applies the row part of the coset twist, w_N^(c j1 C2) = w_(K C1)^(c j1),
// one table read and one product per element; the factor w_N^(j2 (c + K k1)) depends on j2 only
// within a row-pass CTA (fixed c, k1), so pass 2 applies it with one power per column shared by
// all messages.
template <class F>
__device__ __forceinline__ void encode_cols_body(const EncArgs<F>& a, uint64_t bid, unsigned char* smem_raw) {
  F* s = reinterpret_cast<F*>(smem_raw);
  const int logn = a.logC1, n = 1 << logn, W = a.W;
  const int logW = __ffs(W) - 1;  // W is a power of two
  typedef typename F::Base B;
  const B* tw = reinterpret_cast<const B*>(a.rt.ntt);  // read through L1 (keeps shared memory for data)
  const uint64_t C2 = 1ull << a.logC2;
  const uint64_t tiles = C2 >> logW;
  const uint64_t tile = bid % tiles;
  const uint64_t mc = bid / tiles;  // m * K + c
  const uint64_t c = mc % a.K, m = mc / a.K;
  const int lvl = a.logN - a.logC2;  // log2(K C1)
  const uint64_t col0 = tile * W;
  if (W <= ENC_THREADS) {
    // idx = threadIdx.x + ENC_THREADS i: the thread keeps column w and its row j1 advances by
    // js = ENC_THREADS / W, so the source and destination addresses advance by fixed strides and the
    // shared indices are the thread's first ones XOR terms shared by all threads (swz and brev are
    // linear over GF(2) and the bit fields are disjoint).
    const int w = threadIdx.x & (W - 1), r0 = threadIdx.x >> logW, js = ENC_THREADS >> logW;
    const int iters = (n * W + ENC_THREADS - 1) / ENC_THREADS;
    const bool active = threadIdx.x < n * W;
    const bool full = a.msg_len >= ((uint64_t)n << a.logC2);  // no zero padding in the message
    const F* p = a.src + m * a.msg_len + ((uint64_t)r0 << a.logC2) + col0 + w;
    const uint64_t pstep = (uint64_t)js << a.logC2;
    const int st = swz<F>(threadIdx.x);
    if (active) {
      #pragma unroll 4
      for (int i = 0; i < iters; ++i) {
        const int j1 = r0 + i * js;
        F x;
        if (full || (((uint64_t)j1 << a.logC2) + col0 + w) < a.msg_len)
          x = *p;
        else
          x = F::zero();
        if (c != 0 && j1 != 0) x = x.mul_base(level_root<B>(a.rt, lvl, c * (uint64_t)j1));
        sts(s, st ^ swz<F>(i * ENC_THREADS), x);
        p += pstep;
      }
    }
    __syncthreads();
    smem_ntt_dif<F, true>(s, logn, W, 1, W, true, tw);
    if (active) {
      const int sb = swz<F>((brev(r0, logn) << logW) + w);
      F* q = a.dst + ((mc << a.logC1) + r0) * C2 + col0 + w;
      const uint64_t qstep = (uint64_t)js * C2;
      #pragma unroll 4
      for (int i = 0; i < iters; ++i) {
        *q = lds(s, sb ^ swz<F>(brev(i * js, logn) << logW));
        q += qstep;
      }
    }
  } else {
    for (int idx = threadIdx.x; idx < n * W; idx += blockDim.x) {
      const int j1 = idx >> logW;
      const uint64_t j = ((uint64_t)j1 << a.logC2) + col0 + (idx & (W - 1));
      F x = j < a.msg_len ? a.src[m * a.msg_len + j] : F::zero();
      if (c != 0 && j1 != 0) x = x.mul_base(level_root<B>(a.rt, lvl, c * (uint64_t)j1));
      sts(s, swz<F>(idx), x);
    }
    __syncthreads();
    smem_ntt_dif<F, true>(s, logn, W, 1, W, true, tw);
    for (int idx = threadIdx.x; idx < n * W; idx += blockDim.x) {
      const int k1 = idx >> logW, w = idx & (W - 1);
      a.dst[((mc << a.logC1) + k1) * C2 + col0 + w] = lds(s, swz<F>((brev(k1, logn) << logW) + w));
    }
  }
}

template <class F>
__global__ void __launch_bounds__(ENC_THREADS, EncMinCtas<F>::value) encode_cols_kernel(EncArgs<F> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  encode_cols_body<F>(a, blockIdx.x, smem_raw);
}
template <class F>
__global__ void __launch_bounds__(ENC_THREADS, EncMinCtas<F>::value) encode_cols_multi_kernel(const EncJob<F>* jobs,
                                                                                             int njobs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int j = enc_job_of(jobs, njobs, blockIdx.x);
  const EncArgs<F> a = jobs[j].args;
  encode_cols_body<F>(a, blockIdx.x - jobs[j].cta_begin, smem_raw);
}

// Raises a kernel's dynamic shared-memory limit once per device. Each caller instantiation owns its
// flags; std::call_once makes concurrent first launches from several host threads wait for the one
// that sets the attribute.
static constexpr int ENC_MAX_DEVICES = 64;
template <class K>
static cudaError_t smem_attr_once(K kernel, std::once_flag* flags, cudaError_t* results) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= ENC_MAX_DEVICES)
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ENC_SMEM_ATTR);
  std::call_once(flags[dev], [&] {
    results[dev] = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ENC_SMEM_ATTR);
  });
  return results[dev];
}

template <class F, int KIND>
static cudaError_t run_rows(const EncArgs<F>& a, unsigned grid, size_t smem, cudaStream_t s) {
  static std::once_flag flags[ENC_MAX_DEVICES];
  static cudaError_t results[ENC_MAX_DEVICES];
  cudaError_t e = smem_attr_once(encode_rows_kernel<F, KIND>, flags, results);
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
                          uint32_t* leaves, int hash_kind, F* scratch, RootTab rt, cudaStream_t s,
                          const EncodeStaging* staging) {
  // Every root index below is taken modulo the codeword length, which must divide 2^log_order.
  if (p.logN > rt.log_order || p.logN > 32) return cudaErrorInvalidValue;
  const int groups = staging ? staging->groups : 1;
  if (groups < 1 || (size_t)groups > n_msgs) return cudaErrorInvalidValue;
  if (staging) {
    if (staging->bounds[0] != 0 || staging->bounds[groups] != n_msgs) return cudaErrorInvalidValue;
    for (int g = 0; g < groups; ++g)
      if (staging->bounds[g] >= staging->bounds[g + 1]) return cudaErrorInvalidValue;
  }
  auto wait_group = [&](int g) -> cudaError_t {
    return staging ? cudaStreamWaitEvent(s, staging->ready[g], 0) : cudaSuccess;
  };
  EncArgs<F> a;
  a.add_rows = 0;
  a.leaves = leaves;
  a.msg_len = msg_len;
  a.M = (int)n_msgs;
  a.m_magic = m_magic_of(n_msgs);
  a.logC = p.logC;
  a.logN = p.logN;
  a.logC1 = p.logC1;
  a.logC2 = p.logC2;
  a.K = 1ull << (p.logN - p.logC);
  a.G = p.cosets_per_cta;
  a.W = p.cols_per_cta;
  a.rt = rt;
  if (p.mode == 0) {
    for (int g = 0; g < groups; ++g) {
      cudaError_t e = wait_group(g);
      if (e != cudaSuccess) return e;
    }
    a.mode = 0;
    a.src = src;
    a.dst = dst;
    const size_t n = 1ull << p.logC;
    const size_t smem = (size_t)a.G * n_msgs * n * sizeof(F) + n * sizeof(typename F::Base) + 16;
    return dispatch_rows<F>(a, hash_kind, (unsigned)(a.K / a.G), smem, s);
  }
  // pass 1, one launch per message group (messages are independent in this pass; a group's
  // intermediate rows start at message m0's block [m0][c = 0][k1 = 0][j2 = 0])
  {
    static std::once_flag flags[ENC_MAX_DEVICES];
    static cudaError_t results[ENC_MAX_DEVICES];
    cudaError_t ea = smem_attr_once(encode_cols_kernel<F>, flags, results);
    if (ea != cudaSuccess) return ea;
    const size_t C1 = 1ull << p.logC1, C2 = 1ull << p.logC2;
    const size_t smem = (size_t)a.W * C1 * sizeof(F) + 16;
    for (int g = 0; g < groups; ++g) {
      cudaError_t e = wait_group(g);
      if (e != cudaSuccess) return e;
      const size_t m0 = staging ? staging->bounds[g] : 0, m1 = staging ? staging->bounds[g + 1] : n_msgs;
      EncArgs<F> c = a;
      c.src = src + m0 * msg_len;
      c.dst = scratch + m0 * a.K * C1 * C2;
      c.leaves = nullptr;
      const size_t grid = (m1 - m0) * a.K * (C2 / a.W);
      encode_cols_kernel<F><<<(unsigned)grid, ENC_THREADS, smem, s>>>(c);
      note_launch();
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
  }
  // pass 2
  a.mode = 1;
  a.src = scratch;
  a.dst = dst;
  const size_t C1 = 1ull << p.logC1, C2 = 1ull << p.logC2;
  const size_t smem = n_msgs * C2 * sizeof(F) + C2 * sizeof(typename F::Base) + 16;
  return dispatch_rows<F>(a, hash_kind, (unsigned)(a.K * C1), smem, s);
}

// Pass 1 of the four-step split for one message of one coset (K = 1) given by its nonzero
// coefficients grouped by column j2: CTA q writes the whole intermediate column
// I[k1][j2] = sum_e val_e w_C1^(k1 j1_e), k1 < C1, for j2 = col_j2[q] and entries
// [col_off[q], col_off[q + 1]); the caller zeroes the intermediate first (its other columns are zero).
template <class F>
__global__ void sparse_cols_kernel(const uint32_t* col_j2, const uint32_t* col_off, const uint32_t* ent_j1,
                                   const F* ent_val, int logC1, int logC2, RootTab rt, F* inter) {
  typedef typename F::Base B;
  const uint32_t j2 = col_j2[blockIdx.x], e0 = col_off[blockIdx.x], e1 = col_off[blockIdx.x + 1];
  const uint64_t C1 = 1ull << logC1;
  for (uint64_t k1 = threadIdx.x; k1 < C1; k1 += blockDim.x) {
    F acc = F::zero();
    for (uint32_t e = e0; e < e1; ++e) acc += ent_val[e].mul_base(level_root<B>(rt, logC1, (k1 * ent_j1[e]) & (C1 - 1)));
    inter[(k1 << logC2) + j2] = acc;
  }
}

template <class F>
cudaError_t launch_sparse_cols(const EncodePlan& p, const uint32_t* col_j2, const uint32_t* col_off,
                               const uint32_t* ent_j1, const F* ent_val, size_t ncols, F* inter, RootTab rt,
                               cudaStream_t s) {
  if (p.mode != 1 || p.logN != p.logC || p.logC1 < 1 || ncols == 0) return cudaErrorInvalidValue;
  sparse_cols_kernel<F><<<(unsigned)ncols, 256, 0, s>>>(col_j2, col_off, ent_j1, ent_val, p.logC1, p.logC2, rt, inter);
  note_launch();
  return cudaGetLastError();
}

// Pass 2 alone (the four-step row pass) of an encode whose intermediate `scratch` was produced
// elsewhere (launch_sparse_cols); no leaf hashing. With add_rows > 0 (one message) the evaluations
// at rows < add_rows are added into dst instead of being stored.
template <class F>
cudaError_t launch_encode_rows_pass(const EncodePlan& p, const F* scratch, size_t n_msgs, size_t msg_len, F* dst,
                                    RootTab rt, cudaStream_t s, size_t add_rows) {
  if (p.mode != 1 || p.logN > rt.log_order || p.logN > 32) return cudaErrorInvalidValue;
  if (add_rows && n_msgs != 1) return cudaErrorInvalidValue;
  EncArgs<F> a;
  a.add_rows = add_rows;
  a.leaves = nullptr;
  a.msg_len = msg_len;
  a.M = (int)n_msgs;
  a.m_magic = m_magic_of(n_msgs);
  a.logC = p.logC;
  a.logN = p.logN;
  a.logC1 = p.logC1;
  a.logC2 = p.logC2;
  a.K = 1ull << (p.logN - p.logC);
  a.G = p.cosets_per_cta;
  a.W = p.cols_per_cta;
  a.rt = rt;
  a.mode = 1;
  a.src = scratch;
  a.dst = dst;
  const size_t C1 = 1ull << p.logC1, C2 = 1ull << p.logC2;
  const size_t smem = n_msgs * C2 * sizeof(F) + C2 * sizeof(typename F::Base) + 16;
  return dispatch_rows<F>(a, HASH_COPY, (unsigned)(a.K * C1), smem, s);
}

// Multi-job encode: the host image holds the column-pass table then (16-byte aligned) the row-pass
// table, one EncJob per job with the CTA index its range starts at.
template <class F>
size_t encode_multi_table_bytes(size_t njobs) {
  return 2 * njobs * sizeof(EncJob<F>) + 64;
}

template <class F>
static EncArgs<F> enc_args_of(const EncodeJobDesc& d, RootTab rt) {
  EncArgs<F> a;
  a.add_rows = 0;
  a.leaves = d.leaves;
  a.msg_len = d.msg_len;
  a.M = (int)d.n_msgs;
  a.m_magic = m_magic_of(d.n_msgs);
  a.logC = d.plan.logC;
  a.logN = d.plan.logN;
  a.logC1 = d.plan.logC1;
  a.logC2 = d.plan.logC2;
  a.K = 1ull << (d.plan.logN - d.plan.logC);
  a.G = d.plan.cosets_per_cta;
  a.W = d.plan.cols_per_cta;
  a.rt = rt;
  return a;
}

template <class F>
int encode_multi_prepare(const EncodeJobDesc* jobs, size_t njobs, RootTab rt, void* host_image,
                         EncodeMultiLaunch* out) {
  EncodeMultiLaunch l{};
  l.rows_off = (njobs * sizeof(EncJob<F>) + 15) & ~(size_t)15;
  l.bytes = l.rows_off + njobs * sizeof(EncJob<F>);
  EncJob<F>* cols = reinterpret_cast<EncJob<F>*>(host_image);
  EncJob<F>* rows = reinterpret_cast<EncJob<F>*>(static_cast<uint8_t*>(host_image) + l.rows_off);
  for (size_t i = 0; i < njobs; ++i) {
    const EncodeJobDesc& d = jobs[i];
    const EncodePlan& p = d.plan;
    if (p.logN > rt.log_order || p.logN > 32) return WHIR_ERR_UNSUPPORTED;
    EncArgs<F> a = enc_args_of<F>(d, rt);
    const F* src = static_cast<const F*>(d.src);
    F* scratch = static_cast<F*>(d.scratch);
    if (p.mode == 0) {
      a.mode = 0;
      a.src = src;
      a.dst = static_cast<F*>(d.dst);
      const size_t n = 1ull << p.logC;
      l.rows_smem = std::max(l.rows_smem, (size_t)a.G * d.n_msgs * n * sizeof(F) + n * sizeof(typename F::Base) + 16);
      rows[l.nrows].args = a;
      rows[l.nrows].cta_begin = l.rows_grid;
      l.rows_grid += a.K / a.G;
      ++l.nrows;
    } else {
      const size_t C1 = 1ull << p.logC1, C2 = 1ull << p.logC2;
      EncArgs<F> c = a;
      c.src = src;
      c.dst = scratch;
      c.leaves = nullptr;
      c.mode = 1;
      l.cols_smem = std::max(l.cols_smem, (size_t)a.W * C1 * sizeof(F) + 16);
      cols[l.ncols].args = c;
      cols[l.ncols].cta_begin = l.cols_grid;
      l.cols_grid += d.n_msgs * a.K * (C2 / a.W);
      ++l.ncols;
      a.mode = 1;
      a.src = scratch;
      a.dst = static_cast<F*>(d.dst);
      l.rows_smem = std::max(l.rows_smem, d.n_msgs * C2 * sizeof(F) + C2 * sizeof(typename F::Base) + 16);
      rows[l.nrows].args = a;
      rows[l.nrows].cta_begin = l.rows_grid;
      l.rows_grid += a.K * C1;
      ++l.nrows;
    }
  }
  if (l.cols_grid > 0x7fffffffull || l.rows_grid > 0x7fffffffull) return WHIR_ERR_UNSUPPORTED;
  if (l.cols_smem > ENC_SMEM_ATTR || l.rows_smem > ENC_SMEM_ATTR) return WHIR_ERR_UNSUPPORTED;
  *out = l;
  return 0;
}

template <class F, int KIND>
static cudaError_t run_rows_multi(const EncJob<F>* tab, int n, unsigned grid, size_t smem, cudaStream_t s) {
  static std::once_flag flags[ENC_MAX_DEVICES];
  static cudaError_t results[ENC_MAX_DEVICES];
  cudaError_t e = smem_attr_once(encode_rows_multi_kernel<F, KIND>, flags, results);
  if (e != cudaSuccess) return e;
  encode_rows_multi_kernel<F, KIND><<<grid, ENC_THREADS, smem, s>>>(tab, n);
  note_launch();
  return cudaGetLastError();
}

template <class F>
cudaError_t launch_encode_multi(const EncodeMultiLaunch& l, const void* dev_image, int hash_kind, cudaStream_t s) {
  const EncJob<F>* cols = static_cast<const EncJob<F>*>(dev_image);
  const EncJob<F>* rows =
      reinterpret_cast<const EncJob<F>*>(static_cast<const uint8_t*>(dev_image) + l.rows_off);
  if (l.ncols) {
    static std::once_flag flags[ENC_MAX_DEVICES];
    static cudaError_t results[ENC_MAX_DEVICES];
    cudaError_t e = smem_attr_once(encode_cols_multi_kernel<F>, flags, results);
    if (e != cudaSuccess) return e;
    encode_cols_multi_kernel<F><<<(unsigned)l.cols_grid, ENC_THREADS, l.cols_smem, s>>>(cols, l.ncols);
    note_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (!l.nrows) return cudaSuccess;
  const unsigned g = (unsigned)l.rows_grid;
  switch (hash_kind) {
    case HASH_BLAKE3: return run_rows_multi<F, HASH_BLAKE3>(rows, l.nrows, g, l.rows_smem, s);
    case HASH_SHA2: return run_rows_multi<F, HASH_SHA2>(rows, l.nrows, g, l.rows_smem, s);
    case HASH_SHA3: return run_rows_multi<F, HASH_SHA3>(rows, l.nrows, g, l.rows_smem, s);
    case HASH_KECCAK: return run_rows_multi<F, HASH_KECCAK>(rows, l.nrows, g, l.rows_smem, s);
    default: return run_rows_multi<F, HASH_COPY>(rows, l.nrows, g, l.rows_smem, s);
  }
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

// ---------------------------------------------------------------------------------------------
// Canonical <-> in-memory form (Montgomery for Field192/Field256)
// ---------------------------------------------------------------------------------------------
template <class F, bool TO_INTERNAL>
__global__ void convert_kernel(F* v, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t* w = reinterpret_cast<uint64_t*>(v + i);
    if constexpr (TO_INTERNAL) {
      v[i] = Canon<F>::from(w);
    } else {
      uint64_t c[F::LIMBS];
      Canon<F>::to(v[i], c);
#pragma unroll
      for (int q = 0; q < F::LIMBS; ++q) w[q] = c[q];
    }
  }
}
template <class F, bool TO_INTERNAL>
cudaError_t launch_convert(F* v, size_t n, cudaStream_t s) {
  if (Canon<F>::IDENTITY || n == 0) return cudaSuccess;
  const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16);
  convert_kernel<F, TO_INTERNAL><<<grid, 256, 0, s>>>(v, n);
  note_launch();
  return cudaGetLastError();
}
template <class F>
cudaError_t launch_to_internal(F* v, size_t n, cudaStream_t s) {
  return launch_convert<F, true>(v, n, s);
}
template <class F>
cudaError_t launch_to_canonical(F* v, size_t n, cudaStream_t s) {
  return launch_convert<F, false>(v, n, s);
}

#define WHIR_ENCODE_INST(F)                                                                                      \
  template cudaError_t launch_encode<F>(const EncodePlan&, const F*, size_t, size_t, F*, uint32_t*, int, F*, RootTab, \
                                        cudaStream_t, const EncodeStaging*);                                     \
  template size_t encode_multi_table_bytes<F>(size_t);                                                           \
  template int encode_multi_prepare<F>(const EncodeJobDesc*, size_t, RootTab, void*, EncodeMultiLaunch*);        \
  template cudaError_t launch_encode_multi<F>(const EncodeMultiLaunch&, const void*, int, cudaStream_t);         \
  template cudaError_t launch_gather_rows<F>(const F*, size_t, const uint64_t*, size_t, F*, cudaStream_t);       \
  template cudaError_t launch_to_internal<F>(F*, size_t, cudaStream_t);                                         \
  template cudaError_t launch_to_canonical<F>(F*, size_t, cudaStream_t);                                         \
  template cudaError_t launch_sparse_cols<F>(const EncodePlan&, const uint32_t*, const uint32_t*, const uint32_t*,  \
                                             const F*, size_t, F*, RootTab, cudaStream_t);                        \
  template cudaError_t launch_encode_rows_pass<F>(const EncodePlan&, const F*, size_t, size_t, F*, RootTab,       \
                                                  cudaStream_t, size_t);

}  // namespace whir
