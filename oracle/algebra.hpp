// ORACLE — test infrastructure only. CPU restatement of the reference's algebra kernels:
//   NTT roots / interleaved Reed–Solomon encode  src/algebra/ntt/cooley_tukey.rs:51-127, 363-477
//   evaluation points, transpose_permute          cooley_tukey.rs:375-402, ntt/transpose.rs:11-15
//   next_order / divisors                          cooley_tukey.rs:364-368, ntt/utils.rs:69-84
//   sumcheck polynomial / fold                     src/algebra/sumcheck.rs:12-111
//   eval_eq / multilinear extend                   src/algebra/multilinear.rs:15-190
//   geometric_accumulate, univariate evaluate      src/algebra/mod.rs:105-177
// The oracle computes the same mathematical values with straightforward (multithreaded) loops:
// every operation is exact field arithmetic, so the reference's evaluation order does not change
// any output bit.
#pragma once
#include <algorithm>
#include <cassert>
#include <functional>
#include <stdexcept>
#include <thread>
#include <vector>

#include <type_traits>

#include "fields.hpp"

namespace oracle {

// Embedding helpers (src/algebra/embedding.rs:126-153): Identity maps a field to itself, Basefield
// maps the base prime field into an extension; mixed_mul multiplies a target element by a source one.
template <class T, class S>
inline T embed(const S& s) {
  if constexpr (std::is_same<T, S>::value)
    return s;
  else
    return T::from_base(s);
}
template <class T, class S>
inline T mixed_mul(const T& a, const S& s) {
  if constexpr (std::is_same<T, S>::value)
    return a * s;
  else
    return a.mul_base(s);
}

int num_threads();
// Runs fn(begin, end) over [0, n) split across threads; serial when n < min_parallel.
void parallel_for(size_t n, size_t min_parallel, const std::function<void(size_t, size_t)>& fn);

// ------------------------------------------------------------------------------------------
// Prime-field helpers that need multi-limb integers (root of unity exponents).
// ------------------------------------------------------------------------------------------
template <class B>
struct PrimeInfo;

template <>
struct PrimeInfo<Gl> {
  static constexpr int N = 1;
  static void pm1(uint64_t* out) { out[0] = GL_P - 1; }
  static Gl gen() { return Gl{7}; }
  // Order of the root the reference's NttEngine::new_from_fftfield picks: 2^32 * 3
  // (fields.rs:88-89 small subgroup base 15 power 1, keeps primes 2 and 3).
  static uint64_t engine_order() { return 3ULL << 32; }
  static int bits() { return 64; }
  static int bytes() { return 8; }
};
template <>
struct PrimeInfo<F192> {
  static constexpr int N = 3;
  static void pm1(uint64_t* out) {
    for (int i = 0; i < 3; ++i) out[i] = f192_params().p[i];
    out[0] -= 1;
  }
  static F192 gen() { return F192::from_u64(3); }
  static uint64_t engine_order() { return 1ULL << 48; }  // two-adicity 48, no small subgroup
  static int bits() { return f192_params().bits; }
  static int bytes() { return (f192_params().bits + 7) / 8; }
};
template <>
struct PrimeInfo<F256> {
  static constexpr int N = 4;
  static void pm1(uint64_t* out) {
    for (int i = 0; i < 4; ++i) out[i] = f256_params().p[i];
    out[0] -= 1;
  }
  static F256 gen() { return F256::from_u64(5); }
  static uint64_t engine_order() { return 9ULL << 28; }  // 2^28 * 3^2 (fields.rs:68-69)
  static int bits() { return f256_params().bits; }
  static int bytes() { return (f256_params().bits + 7) / 8; }
};

template <class B>
B prime_pow_limbs(B base, const uint64_t* e, int n) {
  B r = B::one();
  for (int i = n - 1; i >= 0; --i) {
    for (int b = 63; b >= 0; --b) {
      r = r * r;
      if ((e[i] >> b) & 1) r = r * base;
    }
  }
  return r;
}

// Primitive n-th root of unity g^((p-1)/n) of the base prime field; n must divide the engine order.
template <class B>
B prime_root(uint64_t n) {
  if (n == 0) return B::one();
  if (PrimeInfo<B>::engine_order() % n != 0) throw std::runtime_error("Subgroup of requested order does not exist.");
  constexpr int N = PrimeInfo<B>::N;
  uint64_t num[N];
  PrimeInfo<B>::pm1(num);
  // long division of num by n
  uint64_t q[N];
  u128 rem = 0;
  for (int i = N - 1; i >= 0; --i) {
    u128 cur = (rem << 64) | num[i];
    q[i] = (uint64_t)(cur / n);
    rem = cur % n;
  }
  return prime_pow_limbs<B>(PrimeInfo<B>::gen(), q, N);
}

// Sorted divisors of the engine order over primes {2, 3} (ntt/utils.rs:69-84).
template <class B>
std::vector<uint64_t> engine_divisors() {
  uint64_t order = PrimeInfo<B>::engine_order();
  std::vector<uint64_t> res{1};
  uint64_t rem = order;
  for (uint64_t p : {2ULL, 3ULL}) {
    uint64_t pk = 1;
    std::vector<uint64_t> existing = res;
    while (rem % p == 0) {
      pk *= p;
      rem /= p;
      for (uint64_t d : existing) res.push_back(d * pk);
    }
  }
  std::sort(res.begin(), res.end());
  return res;
}

template <class B>
bool next_order(uint64_t size, uint64_t* out) {
  static const std::vector<uint64_t> divs = engine_divisors<B>();
  auto it = std::lower_bound(divs.begin(), divs.end(), size);
  if (it == divs.end()) return false;
  *out = *it;
  return true;
}

// coset_size selection of interleaved_encode / evaluation_points (cooley_tukey.rs:387-390, 436-439).
template <class B>
uint64_t coset_size_for(uint64_t masked_len, uint64_t codeword_len) {
  uint64_t c;
  if (!next_order<B>(masked_len, &c)) throw std::runtime_error("message too long for NTT engine");
  while (codeword_len % c != 0) {
    if (!next_order<B>(c + 1, &c)) throw std::runtime_error("no coset size");
  }
  return c;
}

// Lift of a base prime field element to an extension / identity field.
template <class F>
inline F lift_base(typename F::Base b) {
  return F::from_base(b);
}

// In-place natural-order DFT out[k] = sum_j v[j] w^{jk} with w = root(n), mixed radix 2/3.
template <class F>
void dft_inplace(std::vector<F>& v) {
  typedef typename F::Base B;
  size_t n = v.size();
  if (n <= 1) return;
  if ((n & (n - 1)) == 0) {
    // iterative radix-2, bit-reversed input permutation then butterflies
    int logn = 0;
    while ((1ULL << logn) < n) ++logn;
    for (size_t i = 1, j = 0; i < n; ++i) {
      size_t bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) std::swap(v[i], v[j]);
    }
    std::vector<B> tw(n / 2);
    B w = prime_root<B>(n);
    tw[0] = B::one();
    for (size_t i = 1; i < n / 2; ++i) tw[i] = tw[i - 1] * w;
    for (size_t len = 2; len <= n; len <<= 1) {
      size_t step = n / len;
      for (size_t i = 0; i < n; i += len) {
        for (size_t j = 0; j < len / 2; ++j) {
          F u = v[i + j];
          F t = v[i + j + len / 2].mul_base(tw[j * step]);
          v[i + j] = u + t;
          v[i + j + len / 2] = u - t;
        }
      }
    }
    return;
  }
  // generic recursive split by the smallest prime factor (2 or 3)
  size_t r = (n % 2 == 0) ? 2 : 3;
  if (n % r != 0) throw std::runtime_error("NTT size must be 2^a 3^b");
  size_t m = n / r;
  std::vector<std::vector<F>> parts(r, std::vector<F>(m));
  for (size_t i = 0; i < m; ++i)
    for (size_t s = 0; s < r; ++s) parts[s][i] = v[i * r + s];
  for (size_t s = 0; s < r; ++s) dft_inplace(parts[s]);
  B w = prime_root<B>(n);
  for (size_t k = 0; k < n; ++k) {
    F acc = F::zero();
    B wk = w.pow(k);
    B f = B::one();
    for (size_t s = 0; s < r; ++s) {
      acc += parts[s][k % m].mul_base(f);
      f = f * wk;
    }
    v[k] = acc;
  }
}

// ReedSolomon::interleaved_encode (cooley_tukey.rs:411-477) in the default (permuted) order:
// output is codeword_len rows x n_msgs columns, row i = c*C + t holds msg(omega_N^{c + K t}).
template <class F>
std::vector<F> interleaved_encode(const std::vector<const F*>& msgs, size_t msg_len, const F* masks, size_t mask_len,
                                  size_t codeword_len) {
  typedef typename F::Base B;
  size_t n_msgs = msgs.size();
  std::vector<F> out;
  if (n_msgs == 0) return out;
  size_t masked = msg_len + mask_len;
  if (masked > codeword_len) throw std::runtime_error("masked message longer than codeword");
  if (PrimeInfo<B>::engine_order() % codeword_len != 0) throw std::runtime_error("unsupported codeword length");
  size_t C = coset_size_for<B>(masked, codeword_len);
  size_t K = codeword_len / C;
  out.assign(codeword_len * n_msgs, F::zero());
  B wN = prime_root<B>(codeword_len);
  parallel_for(n_msgs * K, 1, [&](size_t b, size_t e) {
    std::vector<F> buf(C);
    for (size_t job = b; job < e; ++job) {
      size_t m = job / K, c = job % K;
      B step = wN.pow(c);
      B tw = B::one();
      for (size_t j = 0; j < C; ++j) {
        F a = j < msg_len ? msgs[m][j] : (j < masked ? masks[m * mask_len + (j - msg_len)] : F::zero());
        buf[j] = a.mul_base(tw);
        tw = tw * step;
      }
      dft_inplace(buf);
      for (size_t t = 0; t < C; ++t) out[(c * C + t) * n_msgs + m] = buf[t];
    }
  });
  return out;
}

inline size_t transpose_permute(size_t index, size_t rows, size_t cols) {
  return index / cols + (index % cols) * rows;
}

template <class B>
std::vector<B> evaluation_points(size_t masked_len, size_t codeword_len, const std::vector<size_t>& idx) {
  if (masked_len > codeword_len) throw std::runtime_error("masked length exceeds codeword");
  if (PrimeInfo<B>::engine_order() % codeword_len != 0) throw std::runtime_error("unsupported codeword length");
  B g = prime_root<B>(codeword_len);
  size_t C = coset_size_for<B>(masked_len, codeword_len);
  size_t K = codeword_len / C;
  std::vector<B> res;
  for (size_t i : idx) {
    if (i >= codeword_len) throw std::runtime_error("index out of range");
    res.push_back(g.pow(transpose_permute(i, K, C)));
  }
  return res;
}

// ------------------------------------------------------------------------------------------
// Sumcheck algebra (src/algebra/sumcheck.rs)
// ------------------------------------------------------------------------------------------
inline size_t next_pow2(size_t n) {
  size_t p = 1;
  while (p < n) p <<= 1;
  return p;
}

template <class F>
void compute_sumcheck_polynomial(const std::vector<F>& a, const std::vector<F>& b, F* c0, F* c2) {
  size_t n = std::min(a.size(), b.size());
  if (n == 0) {
    *c0 = F::zero();
    *c2 = F::zero();
    return;
  }
  if (n == 1) {
    *c0 = a[0] * b[0];
    *c2 = F::zero();
    return;
  }
  size_t half = next_pow2(n) >> 1;
  size_t hi = n - half;  // length of the populated high half
  int T = num_threads();
  std::vector<F> p0(T, F::zero()), p2(T, F::zero());
  std::vector<std::thread> th;
  size_t chunk = (half + T - 1) / T;
  for (int t = 0; t < T; ++t) {
    th.emplace_back([&, t]() {
      size_t s = t * chunk, e = std::min(half, s + chunk);
      F acc0 = F::zero(), acc2 = F::zero();
      for (size_t i = s; i < e; ++i) {
        if (i < hi) {
          acc0 += a[i] * b[i];
          acc2 += (a[i + half] - a[i]) * (b[i + half] - b[i]);
        } else {
          F x = a[i] * b[i];
          acc0 += x;
          acc2 += x;
        }
      }
      p0[t] = acc0;
      p2[t] = acc2;
    });
  }
  for (auto& x : th) x.join();
  F s0 = F::zero(), s2 = F::zero();
  for (int t = 0; t < T; ++t) {
    s0 += p0[t];
    s2 += p2[t];
  }
  *c0 = s0;
  *c2 = s2;
}

template <class F>
void fold(std::vector<F>& v, const F& w) {
  size_t n = v.size();
  if (n <= 1) return;
  size_t half = next_pow2(n) >> 1;
  size_t hi = n - half;
  F one_minus = F::one() - w;
  parallel_for(half, 1 << 14, [&](size_t s, size_t e) {
    for (size_t i = s; i < e; ++i) {
      if (i < hi)
        v[i] = v[i] + (v[i + half] - v[i]) * w;
      else
        v[i] = v[i] * one_minus;
    }
  });
  v.resize(half);
  v.shrink_to_fit();
}

// acc[b] += scalar * prod_k (b_k ? x_k : 1 - x_k), point[0] is the most significant bit
// (multilinear.rs:170-190).
template <class F>
void eval_eq(std::vector<F>& acc, const std::vector<F>& point, const F& scalar) {
  size_t n = (size_t)1 << point.size();
  if (acc.size() != n) throw std::runtime_error("eval_eq size mismatch");
  // Split the point: high part table (first h coordinates) and low part table.
  size_t h = point.size() / 2, l = point.size() - h;
  auto table = [&](size_t off, size_t cnt, F s) {
    std::vector<F> t{s};
    for (size_t k = 0; k < cnt; ++k) {
      const F& x = point[off + k];
      std::vector<F> nt(t.size() * 2);
      for (size_t b = 0; b < t.size(); ++b) {
        F s1 = t[b] * x;
        nt[2 * b] = t[b] - s1;
        nt[2 * b + 1] = s1;
      }
      t.swap(nt);
    }
    return t;
  };
  std::vector<F> th = table(0, h, scalar), tl = table(h, l, F::one());
  size_t nl = tl.size();
  parallel_for(n, 1 << 14, [&](size_t s, size_t e) {
    for (size_t i = s; i < e; ++i) acc[i] += th[i / nl] * tl[i % nl];
  });
}

// acc[i] += sum_j scalars[j] * points[j]^i  (algebra/mod.rs:154-177)
template <class F>
void geometric_accumulate(std::vector<F>& acc, const std::vector<F>& scalars, const std::vector<F>& points) {
  if (scalars.empty()) return;
  size_t n = acc.size();
  parallel_for(n, 4096, [&](size_t s, size_t e) {
    std::vector<F> pw(scalars.size());
    for (size_t j = 0; j < scalars.size(); ++j) pw[j] = scalars[j] * points[j].pow(s);
    for (size_t i = s; i < e; ++i) {
      F sum = F::zero();
      for (size_t j = 0; j < pw.size(); ++j) {
        sum += pw[j];
        pw[j] *= points[j];
      }
      acc[i] += sum;
    }
  });
}

// Horner evaluation of a source-field coefficient vector at a target-field point
// (mixed_univariate_evaluate, algebra/mod.rs:105-129).
template <class T, class S>
T univariate_evaluate(const S* coeffs, size_t n, const T& x) {
  if (n == 0) return T::zero();
  int nt = num_threads();
  size_t chunk = std::max<size_t>(4096, (n + nt - 1) / nt);
  size_t parts = (n + chunk - 1) / chunk;
  std::vector<T> res(parts);
  parallel_for(parts, 2, [&](size_t b, size_t e) {
    for (size_t p = b; p < e; ++p) {
      size_t s = p * chunk, en = std::min(n, s + chunk);
      T acc = T::zero();
      for (size_t i = en; i-- > s;) acc = acc * x + embed<T, S>(coeffs[i]);
      res[p] = acc;
    }
  });
  T total = T::zero();
  T xc = x.pow(chunk);
  for (size_t p = parts; p-- > 0;) total = total * xc + res[p];
  return total;
}

// Multilinear extension of source-field evals at a target point, with implicit zero padding
// (mixed_multilinear_extend, multilinear.rs:15-151): sum_i evals[i] * eq(point, i).
template <class T, class S>
T multilinear_extend(const S* evals, size_t n, const std::vector<T>& point) {
  size_t full = (size_t)1 << point.size();
  if (n > full) throw std::runtime_error("evals longer than hypercube");
  std::vector<T> eq(full, T::zero());
  eval_eq(eq, point, T::one());
  T acc = T::zero();
  for (size_t i = 0; i < n; ++i) acc += mixed_mul<T, S>(eq[i], evals[i]);
  return acc;
}

}  // namespace oracle
