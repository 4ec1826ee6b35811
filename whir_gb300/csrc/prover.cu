// Device-resident WHIR prover and the C ABI (include/whir_gb300.h).
//
// The prover follows whir::Config::prove (src/protocols/whir/prover.rs:50-315) step for step. The
// committed vector, the covector, every codeword and every Merkle tree stay in HBM for the whole
// proof; the host only sees what the transcript needs: Merkle roots, sumcheck round messages
// (c0, c2), out-of-domain values, PoW nonces, the opened rows and their authentication paths, and
// the final (constant-size) vector.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/whir_gb300.h"
#include "field.cuh"
#include "hash.cuh"
#include "kernels.hpp"
#include "protocol.hpp"
#include "status.hpp"

using namespace whir;

namespace {
thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define CU(call)                                                                                 \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) throw Error(WHIR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
}  // namespace

// ------------------------------------------------------------------------------------------------
// Context
// ------------------------------------------------------------------------------------------------
// Kernel families timed by the optional per-family CUDA-event profiling.
enum ProfFamily { PF_ENCODE = 0, PF_MERKLE, PF_SUMCHECK, PF_EQ, PF_GEOMETRIC, PF_LIFT, PF_POW, PF_GATHER,
                  PF_UNIVARIATE, PF_COUNT };

static constexpr size_t MAIL_FLAG_OFF = 128;
static constexpr size_t MAIL_DATA_OFF = 256;
static constexpr size_t MAIL_DATA_BYTES = 512 * 1024;

struct whir_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  // Second stream for host-to-device copies of commit inputs that overlap the encode (see
  // encode_and_tree); everything else runs on `stream`.
  cudaStream_t up_stream = nullptr;
  // Root tables per base field (Goldilocks, Field192, Field256): lo (2^16) then hi entries.
  uint64_t* d_roots[3] = {nullptr, nullptr, nullptr};
  RootTab rts[3] = {};
  uint8_t* h_stage = nullptr;  // pinned staging for small transfers
  size_t h_stage_cap = 0;
  uint8_t* h_up = nullptr;  // pinned upload arena (see h2d)
  size_t up_cap = 0, up_off = 0;
  unsigned long long* d_pow = nullptr;
  // Host-mapped pinned mail area: the round kernels publish their (c0, c2) at offset 0 (see
  // SumcheckBuffers::wait_pair); small device results are copied to MAIL_DATA_OFF with a sequence
  // word at MAIL_FLAG_OFF (see d2h2).
  uint8_t* mail_h = nullptr;
  uint8_t* mail_d = nullptr;
  unsigned int mail_seq = 0;
  // Sumcheck reduction scratch: per-block partial pairs and the (arrival, sequence) counter pair.
  void* sc_parts = nullptr;
  size_t sc_parts_bytes = 0;
  unsigned int* sc_counter = nullptr;
  unsigned int sc_launches = 0;
  // Per-tile arrival counters of the split geometric accumulation (GR_MAX_TILES words, zeroed once).
  unsigned int* geo_counters = nullptr;
  // Device buffers released by finished operations, kept for reuse by exact size. All of the
  // context's work is issued on its one stream, so a buffer released in stream order can be handed
  // to later work as the stream-ordered pool would, without an allocator call per buffer.
  std::mutex cache_mu;
  std::multimap<size_t, void*> free_bufs;
  size_t cached_bytes = 0;
  uint64_t launches_at_create = 0;
  uint64_t h2d_bytes = 0, d2h_bytes = 0;
  // profiling: event pairs recorded around each kernel family on the context's stream
  bool profiling = false;
  std::vector<cudaEvent_t> event_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  double family_ms[PF_COUNT] = {0};
  uint64_t family_calls[PF_COUNT] = {0};
};

namespace {

cudaEvent_t take_event(whir_ctx* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) throw Error(WHIR_ERR_CUDA, "cudaEventCreate failed");
  return e;
}

// Resolves recorded event pairs into per-family milliseconds (waits for the stream).
void resolve_profile(whir_ctx* ctx) {
  if (ctx->pending.empty()) return;
  cudaStreamSynchronize(ctx->stream);
  for (auto& p : ctx->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.second.first, p.second.second);
    ctx->family_ms[p.first] += ms;
    ctx->family_calls[p.first] += 1;
    ctx->event_pool.push_back(p.second.first);
    ctx->event_pool.push_back(p.second.second);
  }
  ctx->pending.clear();
}

// Records a CUDA event pair around the kernels of one family when profiling is on.
struct ProfScope {
  whir_ctx* ctx;
  int fam;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(whir_ctx* c, int f) : ctx(c), fam(f) {
    if (!ctx->profiling) return;
    a = take_event(ctx);
    b = take_event(ctx);
    cudaEventRecord(a, ctx->stream);
  }
  ~ProfScope() {
    if (!a) return;
    cudaEventRecord(b, ctx->stream);
    ctx->pending.push_back({fam, {a, b}});
    if (ctx->pending.size() > 4096) resolve_profile(ctx);
  }
};

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

// Per-context cache of released device buffers (exact-size reuse, bounded). The bound holds every
// buffer of a d = 24 proof (about 2 GiB), so repeated proofs of one shape allocate nothing: a
// stream-ordered allocation that has to map new pool memory stalls the host for ~150 us.
static constexpr size_t BUF_CACHE_BYTES = 4ull << 30;        // bytes kept per context
static constexpr size_t BUF_CACHE_MAX_BLOCK = 512ull << 20;  // larger buffers go back to the pool

void* ctx_alloc(whir_ctx* ctx, size_t bytes) {
  {
    std::lock_guard<std::mutex> lk(ctx->cache_mu);
    auto it = ctx->free_bufs.find(bytes);
    if (it != ctx->free_bufs.end()) {
      void* p = it->second;
      ctx->free_bufs.erase(it);
      ctx->cached_bytes -= bytes;
      return p;
    }
  }
  void* p = nullptr;
  CU(cudaMallocAsync(&p, bytes, ctx->stream));
  return p;
}
void ctx_release(whir_ctx* ctx, void* p, size_t bytes) {
  {
    std::lock_guard<std::mutex> lk(ctx->cache_mu);
    if (bytes <= BUF_CACHE_MAX_BLOCK && ctx->cached_bytes + bytes <= BUF_CACHE_BYTES) {
      ctx->free_bufs.emplace(bytes, p);
      ctx->cached_bytes += bytes;
      return;
    }
  }
  cudaFreeAsync(p, ctx->stream);
}

// Stream-ordered device buffer (from the context's cache or the pool).
template <class T>
struct DBuf {
  whir_ctx* ctx = nullptr;
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(whir_ctx* c, size_t count) : ctx(c), n(count) {
    if (count) p = static_cast<T*>(ctx_alloc(c, count * sizeof(T)));
  }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : ctx(o.ctx), p(o.p), n(o.n) { o.p = nullptr; }
  DBuf& operator=(DBuf&& o) noexcept {
    release();
    ctx = o.ctx;
    p = o.p;
    n = o.n;
    o.p = nullptr;
    return *this;
  }
  void release() {
    if (p) ctx_release(ctx, p, n * sizeof(T));
    p = nullptr;
  }
  ~DBuf() { release(); }
};

void stage_reserve(whir_ctx* ctx, size_t bytes) {
  if (bytes <= ctx->h_stage_cap) return;
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  size_t cap = std::max<size_t>(bytes, 1 << 20);
  CU(cudaMallocHost((void**)&ctx->h_stage, cap));
  ctx->h_stage_cap = cap;
}

}  // namespace

// Copies up to two device segments into the context's host-mapped mail area and then publishes
// `seq` in the mail flag word (after a system-wide fence), so the host can poll for the data
// instead of synchronising the stream. The context's sticky device error word (set by a kernel whose
// bounded wait timed out) travels in the word after the flag. One block; 16-, 8- or 1-byte moves by
// alignment.
__global__ void __launch_bounds__(512) mail_copy_kernel(const uint8_t* s0, size_t b0, const uint8_t* s1, size_t b1,
                                                         uint8_t* dst, size_t off1, unsigned int* flag,
                                                         unsigned int seq, const unsigned int* dev_err) {
  auto copy = [](const uint8_t* src, size_t bytes, uint8_t* d) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(d) | bytes;
    if ((a & 15) == 0) {
      for (size_t i = threadIdx.x; i < bytes / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(d)[i] = reinterpret_cast<const uint4*>(src)[i];
    } else if ((a & 7) == 0) {
      for (size_t i = threadIdx.x; i < bytes / 8; i += blockDim.x)
        reinterpret_cast<uint64_t*>(d)[i] = reinterpret_cast<const uint64_t*>(src)[i];
    } else {
      for (size_t i = threadIdx.x; i < bytes; i += blockDim.x) d[i] = src[i];
    }
  };
  copy(s0, b0, dst);
  if (b1) copy(s1, b1, dst + off1);
  if (threadIdx.x == 0) reinterpret_cast<volatile unsigned int*>(flag)[1] = *reinterpret_cast<const volatile unsigned int*>(dev_err);
  __threadfence_system();
  __syncthreads();
  if (threadIdx.x == 0) *reinterpret_cast<volatile unsigned int*>(flag) = seq;
}

// out[j] = the root digest of tree j (its last node).
__global__ void gather_roots_kernel(const uint32_t* const* roots, int n, uint32_t* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n * 8; i += gridDim.x * blockDim.x)
    out[i] = roots[i >> 3][i & 7];
}

namespace {

// Device -> host copy of up to two segments, in two halves so that the host can enqueue more work
// before waiting. Segments that fit the mail area go through mail_copy_kernel and a bounded poll of
// its flag; larger ones are copied through pinned staging with a stream synchronisation at once.
struct MailFetch {
  void* dst0 = nullptr;
  void* dst1 = nullptr;
  size_t b0 = 0, b1 = 0, off1 = 0;
  unsigned int seq = 0;
  bool done = true;
};
MailFetch mail_begin(whir_ctx* ctx, void* dst0, const void* src0, size_t b0, void* dst1, const void* src1, size_t b1) {
  MailFetch f;
  f.dst0 = dst0;
  f.dst1 = dst1;
  f.b0 = b0;
  f.b1 = b1;
  f.off1 = (b0 + 15) & ~(size_t)15;
  if (!b0 && !b1) return f;
  ctx->d2h_bytes += b0 + b1;
  if (f.off1 + b1 <= MAIL_DATA_BYTES) {
    f.seq = ++ctx->mail_seq;
    f.done = false;
    mail_copy_kernel<<<1, 512, 0, ctx->stream>>>(static_cast<const uint8_t*>(src0), b0,
                                                 static_cast<const uint8_t*>(src1), b1, ctx->mail_d + MAIL_DATA_OFF,
                                                 f.off1, reinterpret_cast<unsigned int*>(ctx->mail_d + MAIL_FLAG_OFF),
                                                 f.seq, ctx->sc_counter + 3);
    CU(cudaGetLastError());
    note_launch();
  } else {
    stage_reserve(ctx, f.off1 + b1);
    if (b0) CU(cudaMemcpyAsync(ctx->h_stage, src0, b0, cudaMemcpyDeviceToHost, ctx->stream));
    if (b1) CU(cudaMemcpyAsync(ctx->h_stage + f.off1, src1, b1, cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    ctx->up_off = 0;  // every earlier upload has completed
    if (b0) memcpy(dst0, ctx->h_stage, b0);
    if (b1) memcpy(dst1, ctx->h_stage + f.off1, b1);
  }
  return f;
}
// A fetch whose bytes a kernel publishes itself (into the mail area, then the returned slot's
// sequence number): pass the slot to that kernel's launch, then wait with mail_end.
MailFetch mail_expect(whir_ctx* ctx, void* dst, size_t bytes, MailSlot* slot) {
  MailFetch f;
  f.dst0 = dst;
  f.b0 = bytes;
  f.seq = ++ctx->mail_seq;
  f.done = false;
  ctx->d2h_bytes += bytes;
  slot->data = ctx->mail_d + MAIL_DATA_OFF;
  slot->flag = reinterpret_cast<unsigned int*>(ctx->mail_d + MAIL_FLAG_OFF);
  slot->seq = f.seq;
  slot->dev_err = ctx->sc_counter + 3;
  return f;
}
// Waits (bounded) for a fetch started by mail_begin or mail_expect and copies its bytes out of the
// mail area.
void mail_end(whir_ctx* ctx, MailFetch& f) {
  if (f.done) return;
  const unsigned int* flag_h = reinterpret_cast<const unsigned int*>(ctx->mail_h + MAIL_FLAG_OFF);
  const auto t0 = std::chrono::steady_clock::now();
  for (uint64_t spin = 0; __atomic_load_n(flag_h, __ATOMIC_ACQUIRE) != f.seq; ++spin) {
    if ((spin & 1023) == 1023) {
      cudaError_t e = cudaStreamQuery(ctx->stream);
      if (e != cudaSuccess && e != cudaErrorNotReady) throw Error(WHIR_ERR_CUDA, cudaGetErrorString(e));
      if (e == cudaSuccess && __atomic_load_n(flag_h, __ATOMIC_ACQUIRE) != f.seq)
        throw Error(WHIR_ERR_INTERNAL, "device copy finished without publishing");
      if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(60))
        throw Error(WHIR_ERR_CUDA, "timed out waiting for a device result");
    }
  }
  if (__atomic_load_n(flag_h + 1, __ATOMIC_ACQUIRE) != 0)
    throw Error(WHIR_ERR_CUDA, "a bounded wait for a bulk copy timed out on the device");
  if (f.b0) memcpy(f.dst0, ctx->mail_h + MAIL_DATA_OFF, f.b0);
  if (f.b1) memcpy(f.dst1, ctx->mail_h + MAIL_DATA_OFF + f.off1, f.b1);
  f.done = true;
}
// Synchronous form: returns once the stream has executed everything enqueued before it.
void d2h2(whir_ctx* ctx, void* dst0, const void* src0, size_t b0, void* dst1, const void* src1, size_t b1) {
  MailFetch f = mail_begin(ctx, dst0, src0, b0, dst1, src1, b1);
  mail_end(ctx, f);
  ctx->up_off = 0;  // nothing was enqueued after the copy, so every earlier upload has completed
}
void d2h(whir_ctx* ctx, void* dst, const void* src, size_t bytes) { d2h2(ctx, dst, src, bytes, nullptr, nullptr, 0); }
// Host -> device copy of a small argument (stream ordered; host buffer reusable on return).
// Host -> device copy of a small argument without waiting: the bytes are staged in a pinned upload
// arena whose space is recycled only after the stream has been synchronised (every d2h() does).
void h2d(whir_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (!bytes) return;
  ctx->h2d_bytes += bytes;
  if (bytes > ctx->up_cap) {
    CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    ctx->up_off = 0;
    return;
  }
  if (ctx->up_off + bytes > ctx->up_cap) {
    CU(cudaStreamSynchronize(ctx->stream));
    ctx->up_off = 0;
  }
  uint8_t* slot = ctx->h_up + ctx->up_off;
  memcpy(slot, src, bytes);
  CU(cudaMemcpyAsync(dst, slot, bytes, cudaMemcpyHostToDevice, ctx->stream));
  ctx->up_off += (bytes + 255) & ~(size_t)255;
}

// Host arrays of canonical limbs <-> elements in their in-memory form.
template <class T>
std::vector<T> load_host(const uint64_t* p, size_t n) {
  std::vector<T> v(n);
  for (size_t i = 0; i < n; ++i) {
    if (!Canon<T>::ok(p + i * T::LIMBS)) throw Error(WHIR_ERR_INVALID, "non-canonical field element");
    v[i] = Canon<T>::from(p + i * T::LIMBS);
  }
  return v;
}
template <class T>
void store_host(const std::vector<T>& v, uint64_t* p) {
  for (size_t i = 0; i < v.size(); ++i) Canon<T>::to(v[i], p + i * T::LIMBS);
}
template <class T>
void store_one(const T& x, uint64_t* p) {
  Canon<T>::to(x, p);
}

template <class B>
struct RootSlot;
template <>
struct RootSlot<Gl> {
  static constexpr int value = 0;
};
template <>
struct RootSlot<F192> {
  static constexpr int value = 1;
};
template <>
struct RootSlot<F256> {
  static constexpr int value = 2;
};

// Device root tables of base field B, built on first use in this context: w = root(2^L),
// lo[i] = w^i (i < 2^16), hi[i] = w^(i 2^16) (i < 2^(L-16)), L = RootInfo<B>::TABLE_LOG.
template <class B>
const RootTab& root_tab(whir_ctx* ctx) {
  constexpr int k = RootSlot<B>::value;
  if (!ctx->d_roots[k]) {
    const int L = RootInfo<B>::TABLE_LOG;
    const size_t nlo = 1u << 16, nhi = (size_t)1 << (L - 16), nntt = ((size_t)1 << NTT_TW_LEVELS) - 1;
    const B w = RootInfo<B>::root(1ull << L);
    const B w16 = w.pow(1ull << 16);
    std::vector<B> tab(nlo + nhi + nntt);
    B x = B::one(), y = B::one();
    for (size_t i = 0; i < nlo; ++i) {
      tab[i] = x;
      x = x * w;
    }
    for (size_t i = 0; i < nhi; ++i) {
      tab[nlo + i] = y;
      y = y * w16;
    }
    for (int lev = 1; lev <= NTT_TW_LEVELS; ++lev) {
      const size_t h = (size_t)1 << (lev - 1);
      const B wl = w.pow(1ull << (L - lev));  // root(2^lev)
      B z = B::one();
      for (size_t q = 0; q < h; ++q) {
        tab[nlo + nhi + h - 1 + q] = z;
        z = z * wl;
      }
    }
    uint64_t* d = nullptr;
    CU(cudaMalloc((void**)&d, tab.size() * sizeof(B)));
    CU(cudaMemcpy(d, tab.data(), tab.size() * sizeof(B), cudaMemcpyHostToDevice));
    ctx->d_roots[k] = d;
    ctx->rts[k].lo = d;
    ctx->rts[k].hi = d + nlo * (sizeof(B) / 8);
    ctx->rts[k].ntt = d + (nlo + nhi) * (sizeof(B) / 8);
    ctx->rts[k].log_order = L;
  }
  return ctx->rts[k];
}

}  // namespace

// ------------------------------------------------------------------------------------------------
// Witness: irs_commit::Witness (irs_commit.rs:95-103) with the matrix and tree in HBM.
// ------------------------------------------------------------------------------------------------
struct whir_witness {
  whir_ctx* ctx = nullptr;
  int field = 0;
  size_t codeword_len = 0, num_cols = 0, layers = 0, elem_limbs = 0;
  DBuf<uint64_t> matrix;  // codeword_len x num_cols elements, elem_limbs u64 each
  DBuf<uint32_t> nodes;   // (2^(layers+1) - 1) x 8 words
  uint8_t root[32] = {0};
  const uint64_t* host_src = nullptr;  // host buffer the committed vectors were copied from
  DBuf<uint64_t> vectors;              // device copy of those vectors (commit from host memory)
  std::vector<uint64_t> ood_points;  // target limbs
  std::vector<uint64_t> ood_matrix;  // points x vectors, target limbs
  size_t num_vectors(size_t t_limbs) const {
    size_t np = ood_points.size() / t_limbs;
    return np ? ood_matrix.size() / t_limbs / np : 0;
  }
};


struct whir_prover_state {
  Transcript ts;
  const whir_config* cfg = nullptr;
};

namespace {

int hash_kind_or_throw(const uint8_t* id) {
  int k = engine_kind(id);
  if (k < 0) throw Error(WHIR_ERR_INVALID, "unknown hash engine id");
  return k;
}

// ------------------------------------------------------------------------------------------------
// Proof of work on the device (proof_of_work.rs:68-166)
// ------------------------------------------------------------------------------------------------
uint64_t grind(whir_ctx* ctx, int kind, const uint8_t chal[32], uint64_t threshold) {
  if (kind == HASH_COPY) throw Error(WHIR_ERR_INVALID, "Copy engine cannot hash 64-byte PoW inputs");
  uint32_t cw[8];
  for (int i = 0; i < 8; ++i)
    cw[i] = (uint32_t)chal[4 * i] | ((uint32_t)chal[4 * i + 1] << 8) | ((uint32_t)chal[4 * i + 2] << 16) |
            ((uint32_t)chal[4 * i + 3] << 24);
  double expect = 18446744073709551616.0 / ((double)threshold + 1.0);
  // The search kernel stops as soon as every block below the best hit is done, so the range per
  // launch can be generous (one launch almost always suffices).
  uint64_t chunk = 1ull << 22;
  while ((double)chunk < 64.0 * expect && chunk < (1ull << 36)) chunk <<= 1;
  const uint64_t limit = 1ull << 50;
  for (uint64_t start = 0; start < limit; start += chunk) {
    const unsigned long long init[2] = {~0ull, 0ull};  // best nonce, finished-CTA counter
    h2d(ctx, ctx->d_pow, init, sizeof(init));
    unsigned long long best;
    MailSlot slot;
    MailFetch f = mail_expect(ctx, &best, sizeof(best), &slot);
    {
      ProfScope prof(ctx, PF_POW);
      CU(launch_pow(cw, threshold, start, chunk, ctx->d_pow, kind, ctx->stream, slot));
    }
    mail_end(ctx, f);
    ctx->up_off = 0;  // nothing was enqueued after the search, so every earlier upload has completed
    if (best != ~0ull) return best;
  }
  throw Error(WHIR_ERR_POW, "Proof of Work failed to solve.");
}

void pow_prove(whir_ctx* ctx, const Pow& p, Transcript& ts) {
  if (p.threshold == UINT64_MAX) return;
  int kind = hash_kind_or_throw(p.hash_id);
  uint8_t chal[32];
  ts.verifier_bytes(chal, 32);
  uint64_t nonce = grind(ctx, kind, chal, p.threshold);
  uint8_t nb[8];
  for (int i = 0; i < 8; ++i) nb[i] = (uint8_t)(nonce >> (8 * i));
  ts.prover_bytes(nb, 8);
}

// ------------------------------------------------------------------------------------------------
// Interleaved RS commitment on the device (irs_commit.rs:292-350)
// ------------------------------------------------------------------------------------------------
// Inputs of at least this many bytes are uploaded in message groups that overlap the encode.
static constexpr size_t STAGED_UPLOAD_MIN_BYTES = 16u << 20;
static constexpr int STAGED_UPLOAD_MAX_GROUPS = 4;

// Canonical host messages to copy into the encode's input buffer while the encode runs (the
// Goldilocks family, whose in-memory form is the canonical one).
template <class F>
struct HostUpload {
  const F* host;
  F* dev;
};

template <class F>
void encode_and_tree(whir_ctx* ctx, const F* d_msgs, size_t n_msgs, size_t msg_len, size_t codeword_len, int kind,
                     whir_witness& w, const HostUpload<F>* upload = nullptr) {
  EncodePlan plan;
  int rc = plan_encode(n_msgs, msg_len, codeword_len, sizeof(F), &plan);
  if (rc) throw Error(rc, "encode shape unsupported on the device");
  if (kind == HASH_BLAKE3 && n_msgs * sizeof(F) > 1024)
    throw Error(WHIR_ERR_UNSUPPORTED, "Blake3 leaves longer than one chunk (1024 bytes) are not supported on the device");
  if (kind == HASH_COPY && n_msgs * sizeof(F) > 32) throw Error(WHIR_ERR_INVALID, "Copy engine needs leaves <= 32 bytes");
  w.codeword_len = codeword_len;
  w.num_cols = n_msgs;
  w.layers = layers_for(codeword_len);
  w.elem_limbs = F::LIMBS;
  w.matrix = DBuf<uint64_t>(ctx, codeword_len * n_msgs * F::LIMBS);
  w.nodes = DBuf<uint32_t>(ctx, ((2ull << w.layers) - 1) * 8);
  DBuf<F> scratch(ctx, plan.scratch_elems);
  // Staged upload: message groups are copied on the upload stream (after the work already queued on
  // the context's stream, which may still use the reused input buffer), each followed by an event
  // that the encode waits for before its first kernel reading that group.
  std::vector<cudaEvent_t> ready;
  std::vector<size_t> bounds;
  EncodeStaging staging{1, nullptr, nullptr};
  // If anything below throws after copies were issued, the context's stream still waits for them,
  // so the input buffer is not handed back to the cache while a copy may be writing into it.
  struct CopyFence {
    whir_ctx* ctx;
    std::vector<cudaEvent_t>* ready;
    bool armed = true;
    ~CopyFence() {
      if (armed)
        for (cudaEvent_t e : *ready) cudaStreamWaitEvent(ctx->stream, e, 0);
    }
  } fence{ctx, &ready};
  if (upload) {
    const size_t bytes = n_msgs * msg_len * sizeof(F);
    // Equal groups: smaller first groups (less of the copy exposed) measured slower overall, as the
    // narrower column-pass launches leave more of their last wave idle.
    const size_t ngroups = std::max<size_t>(
        1, std::min<size_t>({n_msgs, (size_t)STAGED_UPLOAD_MAX_GROUPS, bytes / STAGED_UPLOAD_MIN_BYTES}));
    for (size_t g = 0; g <= ngroups; ++g) bounds.push_back(n_msgs * g / ngroups);
    const int groups = (int)bounds.size() - 1;
    cudaEvent_t start = take_event(ctx);
    ready.push_back(start);
    CU(cudaEventRecord(start, ctx->stream));
    CU(cudaStreamWaitEvent(ctx->up_stream, start, 0));
    for (int g = 0; g < groups; ++g) {
      const size_t m0 = bounds[g], m1 = bounds[g + 1];
      CU(cudaMemcpyAsync(upload->dev + m0 * msg_len, upload->host + m0 * msg_len, (m1 - m0) * msg_len * sizeof(F),
                         cudaMemcpyHostToDevice, ctx->up_stream));
      cudaEvent_t e = take_event(ctx);
      ready.push_back(e);
      CU(cudaEventRecord(e, ctx->up_stream));
    }
    ctx->h2d_bytes += bytes;
    staging = EncodeStaging{groups, bounds.data(), ready.data() + 1};
  }
  {
    ProfScope prof(ctx, PF_ENCODE);
    CU(launch_encode<F>(plan, d_msgs, n_msgs, msg_len, reinterpret_cast<F*>(w.matrix.p), w.nodes.p, kind, scratch.p,
                        root_tab<typename F::Base>(ctx), ctx->stream, upload ? &staging : nullptr));
  }
  fence.armed = false;  // the encode enqueued the waits
  // A wait captures the event's state when it is enqueued, so the events can be reused at once.
  for (cudaEvent_t e : ready) ctx->event_pool.push_back(e);
  if (w.layers >= 1) {
    // the Merkle launch that computes the root publishes it to the host
    MailSlot slot;
    MailFetch f = mail_expect(ctx, w.root, 32, &slot);
    {
      ProfScope prof(ctx, PF_MERKLE);
      CU(launch_merkle(w.nodes.p, (int)w.layers, kind, ctx->stream, 0, slot));
    }
    mail_end(ctx, f);
    ctx->up_off = 0;  // nothing was enqueued after the tree, so every earlier upload has completed
  } else {
    d2h(ctx, w.root, w.nodes.p, 32);
  }
}

template <class T, class S>
T univariate_device(whir_ctx* ctx, const S* d_coeffs, size_t n, const T& x) {
  DBuf<T> parts(ctx, std::max<size_t>(1, (n + 8191) / 8192) + 1);
  size_t np = 0;
  DBuf<T> out(ctx, 1);
  {
    ProfScope prof(ctx, PF_UNIVARIATE);
    CU((launch_univariate_eval<T, S>(d_coeffs, n, x, parts.p, &np, ctx->stream)));
    CU(launch_reduce_singles<T>(parts.p, np, out.p, ctx->stream));
  }
  T r;
  d2h(ctx, &r, out.p, sizeof(T));
  return r;
}

// vectors: num_vectors contiguous device vectors of S.
// upload (optional): d_vecs is still to be filled from these host vectors; the copy overlaps the encode.
template <class S, class T>
std::unique_ptr<whir_witness> irs_commit(whir_ctx* ctx, const Irs& c, Transcript& ts, const S* d_vecs, int field,
                                         const HostUpload<S>* upload = nullptr) {
  auto w = std::make_unique<whir_witness>();
  w->ctx = ctx;
  w->field = field;
  int kind = hash_kind_or_throw(c.hash_id);
  // Messages: each vector split into interleaving_depth contiguous chunks (irs_commit.rs:317-320),
  // so the contiguous vector array already is the n_msgs x message_length message matrix.
  if (upload && c.num_cols * c.message_length() != c.num_vectors * c.vector_size) {
    // the message matrix does not tile the vectors exactly: copy everything before encoding
    CU(cudaMemcpyAsync(upload->dev, upload->host, c.num_vectors * c.vector_size * sizeof(S), cudaMemcpyHostToDevice,
                       ctx->stream));
    ctx->h2d_bytes += c.num_vectors * c.vector_size * sizeof(S);
    upload = nullptr;
  }
  encode_and_tree<S>(ctx, d_vecs, c.num_cols, c.message_length(), c.codeword_length, kind, *w, upload);
  ts.prover_bytes(w->root, 32);
  for (size_t i = 0; i < c.out_domain_samples; ++i) {
    put_raw(w->ood_points, challenge<T>(ts));
  }
  for (size_t i = 0; i < c.out_domain_samples; ++i) {
    T pt = get_raw<T>(&w->ood_points[i * T::LIMBS]);
    for (size_t v = 0; v < c.num_vectors; ++v) {
      T val = univariate_device<T, S>(ctx, d_vecs + v * c.vector_size, c.vector_size, pt);
      send_elem<T>(ts, val);
      put_raw(w->ood_matrix, val);
    }
  }
  return w;
}

// Several commitments (Config::commit of independent jobs, irs_commit.rs:292-350) with the device
// work of every job in shared launches: one column pass and one row pass (with the leaf hashes)
// covering every job's encode through a per-job table, Merkle trees built step by step with every
// job's tiles in one launch, and one fetch of all roots. The transcript steps (root, out-of-domain
// samples) then follow per job, exactly as in irs_commit. Every job has the embedding S -> T and
// commits with its own configuration cs[j].
template <class S, class T>
std::vector<std::unique_ptr<whir_witness>> irs_commit_batch(whir_ctx* ctx, const std::vector<const Irs*>& cs,
                                                            const std::vector<Transcript*>& tss,
                                                            const std::vector<const S*>& d_vecs, int field) {
  const size_t n = cs.size();
  std::vector<std::unique_ptr<whir_witness>> ws(n);
  std::vector<EncodeJobDesc> enc(n);
  std::vector<MerkleJobDesc> mk(n);
  std::vector<DBuf<S>> scratch(n);
  int kind = -1;
  for (size_t j = 0; j < n; ++j) {
    const Irs& c = *cs[j];
    const int k = hash_kind_or_throw(c.hash_id);
    if (kind >= 0 && k != kind) throw Error(WHIR_ERR_INVALID, "a batched commit needs one hash engine");
    kind = k;
    const size_t n_msgs = c.num_cols, msg_len = c.message_length(), cw = c.codeword_length;
    if (n_msgs * msg_len != c.num_vectors * c.vector_size) throw Error(WHIR_ERR_UNSUPPORTED, "message matrix shape");
    EncodePlan plan;
    int rc = plan_encode(n_msgs, msg_len, cw, sizeof(S), &plan);
    if (rc) throw Error(rc, "encode shape unsupported on the device");
    if (kind == HASH_BLAKE3 && n_msgs * sizeof(S) > 1024)
      throw Error(WHIR_ERR_UNSUPPORTED, "Blake3 leaves longer than one chunk (1024 bytes) are not supported");
    if (kind == HASH_COPY && n_msgs * sizeof(S) > 32) throw Error(WHIR_ERR_INVALID, "Copy engine needs leaves <= 32 bytes");
    auto w = std::make_unique<whir_witness>();
    w->ctx = ctx;
    w->field = field;
    w->codeword_len = cw;
    w->num_cols = n_msgs;
    w->layers = layers_for(cw);
    w->elem_limbs = S::LIMBS;
    w->matrix = DBuf<uint64_t>(ctx, cw * n_msgs * S::LIMBS);
    w->nodes = DBuf<uint32_t>(ctx, ((2ull << w->layers) - 1) * 8);
    scratch[j] = DBuf<S>(ctx, plan.scratch_elems);
    enc[j] = EncodeJobDesc{plan, d_vecs[j], n_msgs, msg_len, w->matrix.p, w->nodes.p, scratch[j].p};
    mk[j] = MerkleJobDesc{w->nodes.p, (int)w->layers};
    ws[j] = std::move(w);
  }
  if (n == 0) return ws;
  {
    ProfScope prof(ctx, PF_ENCODE);
    std::vector<uint8_t> image(encode_multi_table_bytes<S>(n));
    EncodeMultiLaunch l;
    const int rc = encode_multi_prepare<S>(enc.data(), n, root_tab<typename S::Base>(ctx), image.data(), &l);
    if (rc) throw Error(rc, "batched encode shape unsupported on the device");
    DBuf<uint8_t> dimg(ctx, l.bytes);
    h2d(ctx, dimg.p, image.data(), l.bytes);
    CU(launch_encode_multi<S>(l, dimg.p, kind, ctx->stream));
  }
  DBuf<uint32_t> roots(ctx, n * 8);
  {
    ProfScope prof(ctx, PF_MERKLE);
    std::vector<MerkleMultiLaunch> launches;
    std::vector<uint8_t> image;
    merkle_multi_plan(mk.data(), n, 0, launches, image);
    DBuf<uint8_t> dimg(ctx, std::max<size_t>(image.size(), 1));
    h2d(ctx, dimg.p, image.data(), image.size());
    CU(launch_merkle_multi(launches, dimg.p, kind, ctx->stream));
    std::vector<const uint32_t*> rp(n);
    for (size_t j = 0; j < n; ++j) rp[j] = ws[j]->nodes.p + ((2ull << ws[j]->layers) - 2) * 8;
    DBuf<const uint32_t*> drp(ctx, n);
    h2d(ctx, drp.p, rp.data(), n * sizeof(const uint32_t*));
    gather_roots_kernel<<<(unsigned)((n * 8 + 255) / 256), 256, 0, ctx->stream>>>(drp.p, (int)n, roots.p);
    CU(cudaGetLastError());
    note_launch();
  }
  std::vector<uint8_t> hroots(n * 32);
  d2h(ctx, hroots.data(), roots.p, n * 32);
  for (size_t j = 0; j < n; ++j) {
    const Irs& c = *cs[j];
    whir_witness& w = *ws[j];
    memcpy(w.root, hroots.data() + j * 32, 32);
    Transcript& ts = *tss[j];
    ts.prover_bytes(w.root, 32);
    for (size_t i = 0; i < c.out_domain_samples; ++i) put_raw(w.ood_points, challenge<T>(ts));
    for (size_t i = 0; i < c.out_domain_samples; ++i) {
      T pt = get_raw<T>(&w.ood_points[i * T::LIMBS]);
      for (size_t v = 0; v < c.num_vectors; ++v) {
        T val = univariate_device<T, S>(ctx, d_vecs[j] + v * c.vector_size, c.vector_size, pt);
        send_elem<T>(ts, val);
        put_raw(w.ood_matrix, val);
      }
    }
  }
  return ws;
}

// irs_commit::Config::open (irs_commit.rs:385-432) in two halves. irs_open_begin samples the query
// indices, computes the evaluation points (and their root exponents), launches the row and sibling
// gathers of every witness and starts their copy to the host; irs_open_end waits for the copy,
// writes the hints (Vec<F> submatrix, then the authentication nodes, per witness) and returns the
// opened rows (points x (witnesses * num_cols)) in the witnesses' field F. Hints are not absorbed
// by the sponge, so the caller may squeeze further challenges and enqueue more device work between
// the two halves without changing the transcript.
template <class F>
struct OpenState {
  size_t q = 0, nc = 0, nwit = 0, layers = 0;
  std::vector<uint64_t> idx;  // opened leaves in challenge order
  DBuf<uint64_t> d_idx;
  DBuf<F> d_rows;        // nwit x q x nc
  DBuf<uint32_t> d_sib;  // nwit x q x layers x 8 words: every query's path, repeats included
  std::vector<F> sub;
  std::vector<uint8_t> sib;
  MailFetch fetch;
};

template <class F>
void irs_open_begin(whir_ctx* ctx, const Irs& c, Transcript& ts, const std::vector<const whir_witness*>& ws,
                    size_t& npoints, OpenState<F>& st, std::vector<uint64_t>* exps = nullptr) {
  std::vector<uint64_t> idx = challenge_indices(ts, c.codeword_length, c.in_domain_samples, c.dedup);
  // The prover needs only the number of evaluation points (their values enter the device's STIR
  // accumulation as root exponents), so they are not computed on the host.
  npoints = idx.size();
  if (exps) {
    // point = w_N^e with e = transpose_permute(index, K, C) (cooley_tukey.rs:391-399)
    uint64_t C = 1;
    while (C < c.masked_message_length()) C <<= 1;
    const uint64_t K = c.codeword_length / C;
    exps->clear();
    for (uint64_t i : idx) exps->push_back(i / C + (i % C) * K);
  }
  st.nc = c.num_cols;
  st.q = idx.size();
  st.nwit = ws.size();
  st.layers = c.layers;
  // The device gathers every query's whole authentication path (repeats included); the host picks
  // the reference's deduplicated node order out of it in irs_open_end, after more device work has
  // been queued, so that walk is off the device's critical path.
  st.d_idx = DBuf<uint64_t>(ctx, std::max<size_t>(st.q, 1));
  h2d(ctx, st.d_idx.p, idx.data(), idx.size() * sizeof(uint64_t));
  st.idx = std::move(idx);
  const size_t per_rows = st.q * st.nc, per_sib = st.q * st.layers * 8;
  st.d_rows = DBuf<F>(ctx, std::max<size_t>(st.nwit * per_rows, 1));
  st.d_sib = DBuf<uint32_t>(ctx, std::max<size_t>(st.nwit * per_sib, 1));
  for (size_t k = 0; k < ws.size(); ++k) {
    const whir_witness* w = ws[k];
    if (w->codeword_len != c.codeword_length || w->num_cols != st.nc)
      throw Error(WHIR_ERR_INVALID, "witness shape mismatch");
    ProfScope prof(ctx, PF_GATHER);
    CU(launch_gather_rows<F>(reinterpret_cast<const F*>(w->matrix.p), st.nc, st.d_idx.p, st.q,
                             st.d_rows.p + k * per_rows, ctx->stream));
    CU(launch_gather_paths(w->nodes.p, st.d_idx.p, st.q, (int)st.layers, st.d_sib.p + k * per_sib, ctx->stream));
  }
  st.sub.resize(st.nwit * per_rows);
  st.sib.resize(st.nwit * per_sib * 4);
  st.fetch = mail_begin(ctx, st.sub.data(), st.d_rows.p, st.sub.size() * sizeof(F), st.sib.data(), st.d_sib.p,
                        st.sib.size());
}

template <class F>
void irs_open_end(whir_ctx* ctx, Transcript& ts, OpenState<F>& st, std::vector<F>& rows) {
  // Authentication nodes in the reference's order (merkle_tree.rs:145-186):
  // per layer, the siblings of the sorted distinct ancestors that are not themselves present; each
  // ancestor keeps a query that reaches it, whose gathered path holds the sibling's digest.
  std::vector<std::pair<uint64_t, uint32_t>> cur, next;  // (ancestor, query)
  for (size_t j = 0; j < st.q; ++j) cur.push_back({st.idx[j], (uint32_t)j});
  std::stable_sort(cur.begin(), cur.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
  cur.erase(std::unique(cur.begin(), cur.end(), [](const auto& x, const auto& y) { return x.first == y.first; }),
            cur.end());
  std::vector<uint32_t> pick;  // (query j, layer l) of each hint node, as j * layers + l
  for (size_t l = 0; l < st.layers; ++l) {
    next.clear();
    for (size_t i = 0; i < cur.size(); ++i) {
      const uint64_t a = cur[i].first;
      const uint32_t j = cur[i].second;
      if (i + 1 < cur.size() && cur[i + 1].first == (a ^ 1))
        ++i;
      else
        pick.push_back((uint32_t)(j * st.layers + l));
      next.push_back({a >> 1, j});
    }
    cur.swap(next);
  }
  const size_t nodes = pick.size();
  mail_end(ctx, st.fetch);
  const size_t nc = st.nc, q = st.q, stride = st.nwit * nc, per_rows = q * nc;
  std::vector<uint8_t> path(nodes * 32);
  rows.assign(q * stride, F::zero());
  for (size_t k = 0; k < st.nwit; ++k) {
    const F* sub = st.sub.data() + k * per_rows;
    // prover_hint_ark(&submatrix): ark-serialize compressed Vec<F> = u64 LE length + elements.
    uint8_t lb[8];
    const uint64_t len = per_rows;
    for (int i = 0; i < 8; ++i) lb[i] = (uint8_t)(len >> (8 * i));
    ts.hint_bytes(lb, 8);
    std::vector<uint8_t> eb(per_rows * 8 * F::LIMBS);
    for (size_t i = 0; i < per_rows; ++i) elem_bytes(sub[i], eb.data() + i * 8 * F::LIMBS);
    ts.hint_bytes(eb.data(), eb.size());
    const uint8_t* all = st.sib.data() + k * q * st.layers * 32;
    for (size_t n = 0; n < nodes; ++n) memcpy(path.data() + n * 32, all + (size_t)pick[n] * 32, 32);
    ts.hint_bytes(path.data(), path.size());
    for (size_t pi = 0; pi < q; ++pi)
      for (size_t j = 0; j < nc; ++j) rows[pi * stride + k * nc + j] = sub[pi * nc + j];
  }
}

template <class F>
void irs_open(whir_ctx* ctx, const Irs& c, Transcript& ts, const std::vector<const whir_witness*>& ws,
              size_t& npoints, std::vector<F>& rows, std::vector<uint64_t>* exps = nullptr) {
  OpenState<F> st;
  irs_open_begin<F>(ctx, c, ts, ws, npoints, st, exps);
  irs_open_end<F>(ctx, ts, st, rows);
}

// ------------------------------------------------------------------------------------------------
// Sumcheck on the device (protocols/sumcheck.rs:69-162), mask_length == 0.
// ------------------------------------------------------------------------------------------------
// Round-message buffers: per-block partials, the last-block counter pair (arrival count, launch
// sequence) and the output pair, which lives in the context's host-mapped mail words: the kernel's
// last block writes (c0, c2) there and then the launch sequence, and the host polls that word
// (wait_pair) instead of issuing a copy and synchronising the stream.
// The partials area and the counter pair are the context's (allocated once; the counter is zeroed
// at creation, the arrival count is re-armed by every last block and the launch sequence only grows,
// mirrored on the host in ctx->sc_launches).
template <class T>
struct SumcheckBuffers {
  whir_ctx* ctx;
  struct {
    T* p;
  } parts;
  struct {
    unsigned int* p;
  } counter;
  T* out;    // device alias of the mail words
  T* out_h;  // host view
  unsigned int& launches;
  SumcheckBuffers(whir_ctx* c, size_t n) : ctx(c), launches(c->sc_launches) {
    const size_t need = (2 * sumcheck_partials(n) + 2) * sizeof(T);
    if (need > ctx->sc_parts_bytes) throw Error(WHIR_ERR_INTERNAL, "sumcheck partials area too small");
    parts.p = reinterpret_cast<T*>(ctx->sc_parts);
    counter.p = ctx->sc_counter;
    out = reinterpret_cast<T*>(ctx->mail_d);
    out_h = reinterpret_cast<T*>(ctx->mail_h);
  }
  unsigned int* flag_h() { return reinterpret_cast<unsigned int*>(out_h + 2); }
  // Call before launching a round kernel that publishes into `out`.
  void arm() {
    __atomic_store_n(flag_h(), 0u, __ATOMIC_RELEASE);
    ++launches;
  }
  // Waits (bounded) for the armed launch's publication and copies (c0, c2).
  void wait_pair(T cc[2]) {
    const auto t0 = std::chrono::steady_clock::now();
    for (uint64_t spin = 0;; ++spin) {
      if (__atomic_load_n(flag_h(), __ATOMIC_ACQUIRE) == launches) break;
      if ((spin & 1023) == 1023) {
        cudaError_t e = cudaStreamQuery(ctx->stream);
        if (e != cudaSuccess && e != cudaErrorNotReady) throw Error(WHIR_ERR_CUDA, cudaGetErrorString(e));
        if (e == cudaSuccess && __atomic_load_n(flag_h(), __ATOMIC_ACQUIRE) != launches)
          throw Error(WHIR_ERR_INTERNAL, "round kernel finished without publishing its message");
        if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(60))
          throw Error(WHIR_ERR_CUDA, "timed out waiting for a sumcheck round");
      }
    }
    memcpy(cc, out_h, 2 * sizeof(T));
    ctx->d2h_bytes += 2 * sizeof(T);
  }
};

// `before_first_message` (optional) runs after the first round's kernel has been enqueued and
// before its message is read: the caller finishes host work that the first round message needs
// (the claimed sum) while the device computes.
template <class T>
std::vector<T> sumcheck_device(whir_ctx* ctx, const Sumcheck& c, Transcript& ts, T* a, T* b, size_t& n, T& sum,
                               const std::function<void()>& before_first_message = {}) {
  if (c.mask_length != 0) throw Error(WHIR_ERR_UNSUPPORTED, "masked sumcheck is not part of this prover");
  if (n != c.initial_size) throw Error(WHIR_ERR_INTERNAL, "sumcheck size mismatch");
  std::vector<T> rs;
  if (c.num_rounds == 0) {
    if (before_first_message) before_first_message();
    return rs;
  }
  SumcheckBuffers<T> buf(ctx, n);
  bool have = false;
  T prev = T::zero();
  for (size_t round = 0; round < c.num_rounds; ++round) {
    size_t np = 0;
    {
      ProfScope prof(ctx, PF_SUMCHECK);
      buf.arm();
      if (!have) {
        CU(launch_sumcheck_compute<T>(a, b, n, buf.parts.p, &np, ctx->stream, buf.out, buf.counter.p));
      } else {
        CU(launch_fold_compute<T>(a, b, n, prev, buf.parts.p, &np, ctx->stream, buf.out, buf.counter.p));
        n = n > 1 ? n / 2 : n;
      }
    }
    if (round == 0 && before_first_message) before_first_message();
    T cc[2];
    buf.wait_pair(cc);
    const T c0 = cc[0], c2 = cc[1];
    const T c1 = sum - c0.dbl() - c2;
    send_elem<T>(ts, c0);
    send_elem<T>(ts, c2);
    pow_prove(ctx, c.round_pow, ts);
    T r = challenge<T>(ts);
    rs.push_back(r);
    sum = (c2 * r + c1) * r + c0;
    prev = r;
    have = true;
  }
  {
    ProfScope prof(ctx, PF_SUMCHECK);
    CU(launch_fold2<T>(a, b, n, prev, ctx->stream));
  }
  n = n > 1 ? n / 2 : n;
  return rs;
}

// Initial sumcheck over a = map(x) and b = sum_l eq(point_l, .) * rlc_l without materialising
// either at full size: round 1 computes (c0, c2) from x and the eq tables, round 2 folds on the fly
// into the half-size buffers a_out / b_out, later rounds use the regular fold-and-compute kernel.
// The transcript interactions are exactly those of sumcheck_device.
template <class T, class S>
std::vector<T> initial_sumcheck_fused(whir_ctx* ctx, const Sumcheck& c, Transcript& ts, const S* x,
                                      const T* tables, int nforms, T* a, T* b, size_t& n, T& sum) {
  if (c.mask_length != 0) throw Error(WHIR_ERR_UNSUPPORTED, "masked sumcheck is not part of this prover");
  const int nvars = (int)layers_for(n);
  std::vector<T> rs;
  SumcheckBuffers<T> buf(ctx, n);
  T prev = T::zero();
  // Prover round messages and challenges (protocols/sumcheck.rs:104-155) once (c0, c2) is in buf.out.
  auto transcript_round = [&]() {
    T cc[2];
    buf.wait_pair(cc);
    const T c0 = cc[0], c2 = cc[1];
    const T c1 = sum - c0.dbl() - c2;
    send_elem<T>(ts, c0);
    send_elem<T>(ts, c2);
    pow_prove(ctx, c.round_pow, ts);
    T r = challenge<T>(ts);
    rs.push_back(r);
    sum = (c2 * r + c1) * r + c0;
    prev = r;
  };
  if (c.num_rounds >= 2 && (int)c.num_rounds <= nvars / 2 && nforms <= 16 && n == ((size_t)1 << nvars)) {
    // Every folded variable lies in the hi index of the eq tables: the covector stays factored as
    // lo x row factors (only the factors are folded) and is written once, after the last round.
    const int h = nvars / 2, l = nvars - h;
    const size_t hs = (size_t)1 << h;
    DBuf<T> fb(ctx, 2 * (size_t)nforms * hs);
    const T* F = tables;
    size_t fstride = hs + ((size_t)1 << l), m = n;
    int rlog = h;
    for (size_t round = 0; round < c.num_rounds; ++round) {
      size_t np = 0;
      {
        ProfScope prof(ctx, PF_SUMCHECK);
        buf.arm();
        if (round == 0) {
          CU((launch_first_compute_eq<T, S>(x, n, tables, nforms, nvars, buf.parts.p, &np, ctx->stream, buf.out,
                                            buf.counter.p)));
        } else {
          T* Fn = fb.p + (round & 1) * (size_t)nforms * hs;
          if (round == 1) {
            CU((launch_rows_fold_compute<T, S>(x, m, prev, F, fstride, rlog, tables, nforms, nvars, a, Fn,
                                               buf.parts.p, &np, ctx->stream, buf.out, buf.counter.p)));
          } else {
            CU((launch_rows_fold_compute<T, T>(a, m, prev, F, fstride, rlog, tables, nforms, nvars, a, Fn,
                                               buf.parts.p, &np, ctx->stream, buf.out, buf.counter.p)));
          }
          F = Fn;
          fstride = hs;
          rlog -= 1;
          m /= 2;
        }
      }
      transcript_round();
    }
    {
      ProfScope prof(ctx, PF_SUMCHECK);
      CU(launch_rows_finish<T>(a, m, prev, F, rlog, tables, nforms, nvars, b, ctx->stream));
    }
    n = m / 2;
    return rs;
  }
  for (size_t round = 0; round < c.num_rounds; ++round) {
    size_t np = 0;
    {
      ProfScope prof(ctx, PF_SUMCHECK);
      buf.arm();
      if (round == 0) {
        CU((launch_first_compute_eq<T, S>(x, n, tables, nforms, nvars, buf.parts.p, &np, ctx->stream, buf.out,
                                          buf.counter.p)));
      } else if (round == 1) {
        CU((launch_first_fold_compute_eq<T, S>(x, n, prev, tables, nforms, nvars, a, b, buf.parts.p, &np,
                                               ctx->stream, buf.out, buf.counter.p)));
        n /= 2;
      } else {
        CU(launch_fold_compute<T>(a, b, n, prev, buf.parts.p, &np, ctx->stream, buf.out, buf.counter.p));
        n = n > 1 ? n / 2 : n;
      }
    }
    transcript_round();
  }
  {
    ProfScope prof(ctx, PF_SUMCHECK);
    if (c.num_rounds == 1) {
      // Only one round: the final fold also reads x and the eq tables (its sums are unused).
      size_t np = 0;
      CU((launch_first_fold_compute_eq<T, S>(x, n, prev, tables, nforms, nvars, a, b, buf.parts.p, &np,
                                             ctx->stream)));
    } else {
      CU(launch_fold2<T>(a, b, n, prev, ctx->stream));
    }
  }
  n = n > 1 ? n / 2 : n;
  return rs;
}

// One tensor-product form of the initial covector: B(y) = scalar * prod_t (y_t ? beta[t] : alpha[t])
// over the index bits y_t, t = 0 the most significant (an eq form of an evaluation point p has
// (alpha, beta) = (1 - p_t, p_t); the geometric form of an out-of-domain point x has
// (1, x^(2^(n-1-t)))).
template <class T>
struct TensorForm {
  T scalar;
  std::vector<T> alpha, beta;
};

// Initial sumcheck (protocols/sumcheck.rs:69-162, mask_length == 0) over a = x_0 + sum_{j>=1}
// c_j lift(x_j) (the vector RLC, as lift + mixed_scalar_mul_add) and b = sum_f B_f for tensor
// forms B_f. The device makes one pass over the vectors for the 2^k sums V_{j,f}(z) (launch_tensor_sums);
// the host derives every round message from them: with the earlier challenges folded into V and
// into P_f = prod_{u<t} phi_{f,u}(r_u), round t's polynomial is
//   h_t(X) = sum_{j,f} c_j s_f P_f phi_{f,t}(X) (A_{j,f,0} + X (A_{j,f,1} - A_{j,f,0})),
//   A_{j,f,c} = sum_y V_{j,f}(c, y) prod_{u>t} phi_{f,u}(y_u),
// which gives the reference's (c0, c2) exactly (c0 = h_t(0), c2 its X^2 coefficient). After the last
// challenge one more pass writes the folded a and b (launch_tensor_fold). The transcript
// interactions (messages, round PoW, challenges) are those of sumcheck_device.
template <class T, class S>
std::vector<T> initial_sumcheck_tensor(whir_ctx* ctx, const Sumcheck& c, Transcript& ts, const S* x, size_t nvec,
                                       const std::vector<T>& vector_rlc, const std::vector<TensorForm<T>>& forms,
                                       T* a, T* b, size_t& n, T& sum) {
  const int nvars = (int)layers_for(n);
  const int k = (int)c.num_rounds;
  const int NF = (int)forms.size();
  const TensorShape sh =
      tensor_plan(nvars, k, (int)nvec, NF, n, sizeof(S), reinterpret_cast<uintptr_t>(x) % 16 == 0);
  const size_t rows = (size_t)1 << sh.R, cols = (size_t)1 << sh.C, per = rows + cols;
  const size_t nz = (size_t)1 << k;
  std::vector<T> rs;
  // out holds the 2^k sums per (vector, form), then an error word (one if a stage wait timed out).
  DBuf<T> tables(ctx, NF * per), parts(ctx, sh.grid() * NF), out(ctx, nvec * NF * nz + 1);
  std::vector<T> V(nvec * NF * nz + 1);
  {
    ProfScope prof(ctx, PF_SUMCHECK);
    std::vector<T> ab;
    for (const auto& f : forms)
      for (int t = k; t < nvars; ++t) {
        ab.push_back(f.alpha[t]);
        ab.push_back(f.beta[t]);
      }
    DBuf<T> dab(ctx, std::max<size_t>(ab.size(), 1));
    h2d(ctx, dab.p, ab.data(), ab.size() * sizeof(T));
    CU(launch_tensor_tables<T>(dab.p, NF, sh.R, sh.C, tables.p, ctx->stream));
    if (V.size() * sizeof(T) <= MAIL_DATA_BYTES) {
      // the last CTA of the sums pass publishes the sums to the host itself
      MailSlot slot;
      MailFetch fetch = mail_expect(ctx, V.data(), V.size() * sizeof(T), &slot);
      CU((launch_tensor_sums<T, S>(x, sh, tables.p, parts.p, out.p, ctx->sc_counter, ctx->stream, slot)));
      mail_end(ctx, fetch);
      ctx->up_off = 0;  // nothing was enqueued after the sums, so every earlier upload has completed
    } else {
      CU((launch_tensor_sums<T, S>(x, sh, tables.p, parts.p, out.p, ctx->sc_counter, ctx->stream)));
      d2h(ctx, V.data(), out.p, V.size() * sizeof(T));
    }
    if (!(V.back() == T::zero())) throw Error(WHIR_ERR_CUDA, "tensor sums: a bulk-copy stage wait timed out");
    V.pop_back();
  }
  std::vector<T> P(NF, T::one());
  for (int t = 0; t < k; ++t) {
    const size_t sz = nz >> t, half = sz >> 1;
    T c0 = T::zero(), c2 = T::zero();
    for (int f = 0; f < NF; ++f) {
      const TensorForm<T>& fm = forms[f];
      // weights of the remaining top variables t+1..k-1 inside a half
      std::vector<T> wy(half, T::one());
      for (size_t y = 0; y < half; ++y)
        for (int q = 0; q < k - t - 1; ++q) {
          const bool bit = (y >> (k - t - 2 - q)) & 1;
          wy[y] = wy[y] * (bit ? fm.beta[t + 1 + q] : fm.alpha[t + 1 + q]);
        }
      for (size_t j = 0; j < nvec; ++j) {
        const T* v = &V[(j * NF + f) * nz];
        T A0 = T::zero(), A1 = T::zero();
        for (size_t y = 0; y < half; ++y) {
          A0 += v[y] * wy[y];
          A1 += v[half + y] * wy[y];
        }
        const T coef = (j == 0 ? T::one() : vector_rlc[j]) * fm.scalar * P[f];
        c0 += coef * (fm.alpha[t] * A0);
        c2 += coef * ((fm.beta[t] - fm.alpha[t]) * (A1 - A0));
      }
    }
    const T c1 = sum - c0.dbl() - c2;
    send_elem<T>(ts, c0);
    send_elem<T>(ts, c2);
    pow_prove(ctx, c.round_pow, ts);
    const T r = challenge<T>(ts);
    rs.push_back(r);
    sum = (c2 * r + c1) * r + c0;
    for (size_t jf = 0; jf < nvec * (size_t)NF; ++jf) {
      T* v = &V[jf * nz];
      for (size_t y = 0; y < half; ++y) v[y] = v[y] + r * (v[half + y] - v[y]);
    }
    for (int f = 0; f < NF; ++f) P[f] = P[f] * (forms[f].alpha[t] + r * (forms[f].beta[t] - forms[f].alpha[t]));
  }
  {
    ProfScope prof(ctx, PF_SUMCHECK);
    std::vector<T> w(nvec * nz), kf(NF);
    for (size_t z = 0; z < nz; ++z) {
      T e = T::one();
      for (int t = 0; t < k; ++t) e = e * (((z >> (k - 1 - t)) & 1) ? rs[t] : T::one() - rs[t]);
      for (size_t j = 0; j < nvec; ++j) w[j * nz + z] = (j == 0 ? T::one() : vector_rlc[j]) * e;
    }
    for (int f = 0; f < NF; ++f) kf[f] = forms[f].scalar * P[f];
    DBuf<T> dw(ctx, w.size()), dk(ctx, kf.size());
    h2d(ctx, dw.p, w.data(), w.size() * sizeof(T));
    h2d(ctx, dk.p, kf.data(), kf.size() * sizeof(T));
    CU((launch_tensor_fold<T, S>(x, sh, dw.p, dk.p, tables.p, a, b, ctx->sc_counter + 3, ctx->stream)));
  }
  n >>= k;
  return rs;
}

// covector[i] += sum_j scalars[j] * w_N^(exps[j] * i) for i < len: the STIR constraints of the
// in-domain query points (UnivariateEvaluation::accumulate_many, linear_form/univariate_evaluation.rs
// 26-39). Small rounds use the root-table kernel; when len * queries exceeds the cost of one size-N
// NTT, the sum is computed as that NTT of the sparse vector S[e] = sum_{e_j = e} s_j
// (sum_e S[e] w_N^(e i) = S's polynomial evaluated at w_N^i), of which the first len values are added.
template <class T>
void accumulate_in_domain(whir_ctx* ctx, T* cov, size_t len, const std::vector<T>& scalars,
                          const std::vector<uint64_t>& exps, size_t N) {
  if (scalars.empty() || len == 0) return;
  const int logN = (int)layers_for(N);
  const double direct = 3.0 * (double)len * (double)scalars.size();
  const double ntt = (double)N * (double)(logN + 20);
  ProfScope prof(ctx, PF_GEOMETRIC);
  if (direct <= ntt || N < 64) {
    DBuf<T> ds(ctx, scalars.size());
    DBuf<uint64_t> de(ctx, exps.size());
    h2d(ctx, ds.p, scalars.data(), scalars.size() * sizeof(T));
    h2d(ctx, de.p, exps.data(), exps.size() * sizeof(uint64_t));
    const GeometricSplit sp = geometric_split_plan(len, scalars.size(), true);
    DBuf<T> parts(ctx, sp.split && sp.groups > 1 ? sp.groups * len : 0);
    CU(launch_geometric_roots<T>(cov, len, ds.p, de.p, scalars.size(), logN, root_tab<typename T::Base>(ctx),
                                 ctx->stream, parts.p, parts.p ? ctx->geo_counters : nullptr));
    return;
  }
  // Combine repeated query positions (indices are sampled with replacement).
  std::vector<std::pair<uint64_t, T>> sparse;
  for (size_t j = 0; j < scalars.size(); ++j) sparse.push_back({exps[j] % N, scalars[j]});
  std::sort(sparse.begin(), sparse.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
  std::vector<uint64_t> idx;
  std::vector<T> vals;
  for (auto& p : sparse) {
    if (!idx.empty() && idx.back() == p.first)
      vals.back() += p.second;
    else {
      idx.push_back(p.first);
      vals.push_back(p.second);
    }
  }
  EncodePlan plan;
  // Four-step with 2^10-point row transforms where the size allows (2^21: 2048 CTAs of 2^10 points
  // fill the GPU in several waves; the largest tile, 512 CTAs of 2^12 points, left most of a second
  // wave idle), and the plain plan otherwise.
  const int logN_ = (int)layers_for(N);
  const EncodeTuning four{1, std::max(logN_ - ENC_MAX_NTT_LOG, std::min(10, logN_ - 1)), 1, 1};
  int rc = logN_ > ENC_MAX_NTT_LOG ? plan_encode_tuned(1, N, N, sizeof(T), four, &plan) : -1;
  if (rc) rc = plan_encode(1, N, N, sizeof(T), &plan);
  if (rc) throw Error(rc, "NTT shape unsupported on the device");
  DBuf<T> scratch(ctx, plan.scratch_elems);
  if (plan.mode == 1) {
    // Four-step: with a few hundred nonzeros among N coefficients nearly every column of the
    // (C1 x C2) view is zero, so pass 1 is computed only for the nonzero columns, straight from the
    // sparse list (the intermediate is zeroed first), and pass 2 runs as usual.
    const uint64_t C2 = 1ull << plan.logC2;
    std::vector<std::pair<uint64_t, size_t>> bycol;  // (column j2, entry)
    for (size_t e = 0; e < idx.size(); ++e) bycol.push_back({idx[e] & (C2 - 1), e});
    std::sort(bycol.begin(), bycol.end());
    std::vector<uint32_t> col_j2, col_off, ent_j1;
    std::vector<T> ent_val;
    for (const auto& ce : bycol) {
      if (col_j2.empty() || col_j2.back() != ce.first) {
        col_j2.push_back((uint32_t)ce.first);
        col_off.push_back((uint32_t)ent_j1.size());
      }
      ent_j1.push_back((uint32_t)(idx[ce.second] >> plan.logC2));
      ent_val.push_back(vals[ce.second]);
    }
    col_off.push_back((uint32_t)ent_j1.size());
    DBuf<uint32_t> dj2(ctx, col_j2.size()), doff(ctx, col_off.size()), dj1(ctx, ent_j1.size());
    DBuf<T> dval(ctx, ent_val.size());
    h2d(ctx, dj2.p, col_j2.data(), col_j2.size() * sizeof(uint32_t));
    h2d(ctx, doff.p, col_off.data(), col_off.size() * sizeof(uint32_t));
    h2d(ctx, dj1.p, ent_j1.data(), ent_j1.size() * sizeof(uint32_t));
    h2d(ctx, dval.p, ent_val.data(), ent_val.size() * sizeof(T));
    CU(cudaMemsetAsync(scratch.p, 0, plan.scratch_elems * sizeof(T), ctx->stream));
    CU(launch_sparse_cols<T>(plan, dj2.p, doff.p, dj1.p, dval.p, col_j2.size(), scratch.p,
                             root_tab<typename T::Base>(ctx), ctx->stream));
    // pass 2 adds the evaluations at the first len points straight into the covector
    CU(launch_encode_rows_pass<T>(plan, scratch.p, 1, N, cov, root_tab<typename T::Base>(ctx), ctx->stream, len));
  } else {
    DBuf<T> dense(ctx, N), out(ctx, N);
    DBuf<uint64_t> di(ctx, idx.size());
    DBuf<T> dv(ctx, vals.size());
    CU(cudaMemsetAsync(dense.p, 0, N * sizeof(T), ctx->stream));
    h2d(ctx, di.p, idx.data(), idx.size() * sizeof(uint64_t));
    h2d(ctx, dv.p, vals.data(), vals.size() * sizeof(T));
    CU(launch_scatter<T>(dense.p, di.p, dv.p, idx.size(), ctx->stream));
    CU(launch_encode<T>(plan, dense.p, 1, N, out.p, nullptr, HASH_BLAKE3, scratch.p,
                        root_tab<typename T::Base>(ctx), ctx->stream));
    CU(launch_add<T>(cov, out.p, len, ctx->stream));
  }
}

template <class T>
std::vector<T> eq_weights_host(const std::vector<T>& point) {
  std::vector<T> t{T::one()};
  for (const T& x : point) {
    std::vector<T> nt(t.size() * 2);
    for (size_t b = 0; b < t.size(); ++b) {
      T s1 = t[b] * x;
      nt[2 * b] = t[b] - s1;
      nt[2 * b + 1] = s1;
    }
    t.swap(nt);
  }
  return t;
}

// Host accumulator of 64x64-bit products: exact sum as lo (128 bits) + hi * 2^128, reduced mod p
// once (2^128 = -2^32 mod p).
struct HostAcc {
  unsigned __int128 lo = 0;
  uint64_t hi = 0;
  void add(uint64_t a, uint64_t b) {
    const unsigned __int128 p = (unsigned __int128)a * b;
    lo += p;
    hi += lo < p;
  }
  uint64_t reduce() const { return gl_sub(gl_reduce((uint64_t)lo, (uint64_t)(lo >> 64)), hi << 32); }
};

// sum_k w[k] * map(v[k]) for the opened rows of a STIR round, with unreduced products for the
// Goldilocks family (the same field element as the reduced sum).
template <class T, class S>
T dot_host_wide(const T* w, const S* v, size_t n) {
  if constexpr (std::is_same_v<S, Gl> && (std::is_same_v<T, Gl> || std::is_same_v<T, Gl2> || std::is_same_v<T, Gl3>)) {
    HostAcc acc[T::DEG];
    for (size_t k = 0; k < n; ++k)
      for (int d = 0; d < T::DEG; ++d) acc[d].add(w[k].coeff(d).v, v[k].v);
    uint64_t c[T::DEG];
    for (int d = 0; d < T::DEG; ++d) c[d] = acc[d].reduce();
    return Canon<T>::from(c);
  } else if constexpr (std::is_same_v<T, Gl2> && std::is_same_v<S, Gl2>) {
    HostAcc a00, a11, a01;
    for (size_t k = 0; k < n; ++k) {
      a00.add(w[k].c0, v[k].c0);
      a11.add(w[k].c1, v[k].c1);
      a01.add(w[k].c0, v[k].c1);
      a01.add(w[k].c1, v[k].c0);
    }
    return Gl2{gl_add(a00.reduce(), gl_mul7(a11.reduce())), a01.reduce()};
  } else {
    T acc = T::zero();
    for (size_t k = 0; k < n; ++k) acc += Embed<T, S>::mul(w[k], v[k]);
    return acc;
  }
}

template <class T>
T dot_host(const std::vector<T>& a, const std::vector<T>& b) {
  T acc = T::zero();
  for (size_t i = 0; i < a.size(); ++i) acc += a[i] * b[i];
  return acc;
}

// ------------------------------------------------------------------------------------------------
// whir::Config::prove on the device
// ------------------------------------------------------------------------------------------------
template <class S, class T>
void prove_device(whir_ctx* ctx, const Config& cfg, Transcript& ts, const S* d_vectors, size_t nv,
                  const std::vector<const whir_witness*>& witnesses, const std::vector<std::vector<T>>& mle_points,
                  const std::vector<std::vector<T>>& covectors, const std::vector<T>& evaluations,
                  std::vector<T>& eval_point_out, std::vector<T>& rlc_out) {
  const size_t n = cfg.size();
  const size_t nforms = mle_points.size() + covectors.size();
  if (nv != witnesses.size() * cfg.initial.num_vectors) throw Error(WHIR_ERR_INVALID, "vector/witness count mismatch");
  if (evaluations.size() != nv * nforms) throw Error(WHIR_ERR_INVALID, "evaluation matrix size mismatch");
  eval_point_out.clear();
  rlc_out.clear();
  if (nv == 0) return;

  // Out-of-domain cross terms (prover.rs:98-128).
  std::vector<T> oods_points, oods_matrix;
  size_t voff = 0;
  for (const whir_witness* w : witnesses) {
    const size_t wn = w->num_vectors(T::LIMBS);
    const size_t np = w->ood_points.size() / T::LIMBS;
    for (size_t oi = 0; oi < np; ++oi) {
      const T pt = get_raw<T>(&w->ood_points[oi * T::LIMBS]);
      for (size_t j = 0; j < nv; ++j) {
        if (j >= voff && j < voff + wn) {
          oods_matrix.push_back(get_raw<T>(&w->ood_matrix[(oi * wn + (j - voff)) * T::LIMBS]));
        } else {
          T e = univariate_device<T, S>(ctx, d_vectors + j * n, n, pt);
          send_elem<T>(ts, e);
          oods_matrix.push_back(e);
        }
      }
      oods_points.push_back(pt);
    }
    voff += wn;
  }

  std::vector<T> vector_rlc = geometric_challenge<T>(ts, nv);
  std::vector<T> constraint_rlc = geometric_challenge<T>(ts, nforms + oods_points.size());
  const bool has_constraints = !constraint_rlc.empty();
  std::vector<T> init_rlc(constraint_rlc.begin(), constraint_rlc.begin() + nforms);
  std::vector<T> oods_rlc(constraint_rlc.begin() + nforms, constraint_rlc.end());
  // Tensor path: the covector is a sum of at most TS_MAX_FORMS tensor-product forms (evaluation
  // points and out-of-domain points; explicit covectors are not tensors) and the initial sumcheck
  // has rounds: the vectors are read twice in all (initial_sumcheck_tensor).
  const int nvars_all = (int)layers_for(n);
  const size_t k0 = cfg.initial_sumcheck.num_rounds;
  const bool tensor = has_constraints && covectors.empty() && mle_points.size() + oods_points.size() <= TS_MAX_FORMS &&
                      k0 >= 1 && k0 <= 10 && (int)k0 <= nvars_all && cfg.initial_sumcheck.mask_length == 0 &&
                      n == ((size_t)1 << nvars_all) && (nv << k0) * sizeof(T) <= 48 * 1024;
  // Fused path: one vector and a statement made only of multilinear-evaluation forms. The first
  // two sumcheck rounds then read the coefficients directly and evaluate the eq covector from
  // small tables, so neither the lifted vector nor the covector is written at full size.
  const bool fused = !tensor && has_constraints && nv == 1 && covectors.empty() && oods_points.empty() &&
                     !mle_points.empty() && n >= 8 && cfg.initial_sumcheck.num_rounds >= 1;
  const size_t alen = tensor ? n >> k0 : (fused ? n / 2 : n);
  DBuf<T> a(ctx, alen), b(ctx, alen);
  if (!fused && !tensor) {
    std::vector<const S*> vp(nv);
    for (size_t j = 0; j < nv; ++j) vp[j] = d_vectors + j * n;
    ProfScope prof(ctx, PF_LIFT);
    CU((launch_lift_rlc<T, S>(a.p, vp.data(), vector_rlc.data(), nv, n, ctx->stream)));
  }
  DBuf<T> eq_tables;
  if (fused) {
    const int nvars = (int)layers_for(n);
    const int h = nvars / 2, l = nvars - h;
    const size_t per = (1ull << h) + (1ull << l);
    eq_tables = DBuf<T>(ctx, per * mle_points.size());
    DBuf<T> pt(ctx, (size_t)nvars * mle_points.size());
    std::vector<T> allp;
    for (const auto& p : mle_points) allp.insert(allp.end(), p.begin(), p.end());
    h2d(ctx, pt.p, allp.data(), allp.size() * sizeof(T));
    ProfScope prof(ctx, PF_EQ);
    for (size_t k = 0; k < mle_points.size(); ++k) {
      CU(launch_eq_table<T>(pt.p + k * nvars, 0, h, init_rlc[k], eq_tables.p + k * per, ctx->stream));
      CU(launch_eq_table<T>(pt.p + k * nvars, h, l, T::one(), eq_tables.p + k * per + (1ull << h), ctx->stream));
    }
  } else if (has_constraints && !tensor) {
    CU(cudaMemsetAsync(b.p, 0, n * sizeof(T), ctx->stream));
    const int nvars = (int)layers_for(n);
    DBuf<T> pt(ctx, std::max(nvars, 1));
    DBuf<T> tables(ctx, (2ull << ((nvars + 1) / 2)) + 2);
    size_t k = 0;
    for (const auto& p : mle_points) {
      h2d(ctx, pt.p, p.data(), p.size() * sizeof(T));
      ProfScope prof(ctx, PF_EQ);
      CU(launch_eval_eq<T>(b.p, pt.p, nvars, init_rlc[k], tables.p, ctx->stream));
      ++k;
    }
    if (!covectors.empty()) {
      DBuf<T> cv(ctx, n);
      for (const auto& c : covectors) {
        h2d(ctx, cv.p, c.data(), n * sizeof(T));
        const T* vp = cv.p;
        // b += rlc * covector: reuse the RLC axpy with an identity embedding.
        std::vector<const T*> ptrs{b.p, vp};
        std::vector<T> coeffs{T::one(), init_rlc[k]};
        DBuf<T> tmp(ctx, n);
        CU((launch_lift_rlc<T, T>(tmp.p, ptrs.data(), coeffs.data(), 2, n, ctx->stream)));
        CU(cudaMemcpyAsync(b.p, tmp.p, n * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
        ++k;
      }
    }
  }
  T the_sum = T::zero();
  for (size_t f = 0; f < nforms; ++f) {
    T row = T::zero();
    for (size_t j = 0; j < nv; ++j) row += vector_rlc[j] * evaluations[f * nv + j];
    the_sum += init_rlc[f] * row;
  }
  if (!oods_points.empty() && !tensor) {
    DBuf<T> sp(ctx, 2 * oods_points.size());
    std::vector<T> packed(oods_rlc);
    packed.insert(packed.end(), oods_points.begin(), oods_points.end());
    h2d(ctx, sp.p, packed.data(), packed.size() * sizeof(T));
    ProfScope prof(ctx, PF_GEOMETRIC);
    CU(launch_geometric_accumulate<T>(b.p, n, sp.p, sp.p + oods_points.size(), oods_points.size(), ctx->stream));
  }
  for (size_t o = 0; o < oods_points.size(); ++o) {
    T row = T::zero();
    for (size_t j = 0; j < nv; ++j) row += vector_rlc[j] * oods_matrix[o * nv + j];
    the_sum += oods_rlc[o] * row;
  }

  size_t len = n;  // current logical length of a and b
  std::vector<T> folding;
  if (tensor) {
    std::vector<TensorForm<T>> forms;
    for (size_t f = 0; f < mle_points.size(); ++f) {
      TensorForm<T> fm{init_rlc[f], {}, {}};
      for (const T& p : mle_points[f]) {
        fm.alpha.push_back(T::one() - p);
        fm.beta.push_back(p);
      }
      forms.push_back(std::move(fm));
    }
    for (size_t o = 0; o < oods_points.size(); ++o) {
      TensorForm<T> fm{oods_rlc[o], std::vector<T>(nvars_all, T::one()), std::vector<T>(nvars_all)};
      T pw = oods_points[o];
      for (int t = nvars_all - 1; t >= 0; --t) {
        fm.beta[t] = pw;
        pw = pw * pw;
      }
      forms.push_back(std::move(fm));
    }
    folding = initial_sumcheck_tensor<T, S>(ctx, cfg.initial_sumcheck, ts, d_vectors, nv, vector_rlc, forms, a.p, b.p,
                                            len, the_sum);
  } else if (fused) {
    folding = initial_sumcheck_fused<T, S>(ctx, cfg.initial_sumcheck, ts, d_vectors, eq_tables.p,
                                           (int)mle_points.size(), a.p, b.p, len, the_sum);
  } else if (has_constraints) {
    folding = sumcheck_device<T>(ctx, cfg.initial_sumcheck, ts, a.p, b.p, len, the_sum);
  } else {
    for (size_t i = 0; i < cfg.initial_sumcheck.num_rounds; ++i) folding.push_back(challenge<T>(ts));
    pow_prove(ctx, cfg.initial_skip_pow, ts);
    for (const T& f : folding) {
      CU(launch_fold<T>(a.p, len, f, ctx->stream));
      len = len > 1 ? len / 2 : len;
    }
    CU(cudaMemsetAsync(b.p, 0, cfg.initial_sumcheck.final_size() * sizeof(T), ctx->stream));
  }
  std::vector<T> evaluation_point = folding;

  std::unique_ptr<whir_witness> prev;
  for (size_t ri = 0; ri < cfg.rounds.size(); ++ri) {
    const Round& rc = cfg.rounds[ri];
    if (len != rc.irs.vector_size) throw Error(WHIR_ERR_INTERNAL, "round vector size mismatch");
    std::unique_ptr<whir_witness> nw = irs_commit<T, T>(ctx, rc.irs, ts, a.p, cfg.field);
    pow_prove(ctx, rc.pow, ts);
    size_t npts = 0;
    std::vector<S> srows;
    std::vector<T> in_rows;
    std::vector<uint64_t> exps;
    const size_t prev_N = prev ? cfg.rounds[ri - 1].irs.codeword_length : cfg.initial.codeword_length;
    // The opening's rows come back while the device accumulates the STIR constraints and runs the
    // first sumcheck round: the rows only feed the claimed sum (hints are not absorbed).
    OpenState<S> open_s;
    OpenState<T> open_t;
    if (!prev) {
      irs_open_begin<S>(ctx, cfg.initial, ts, witnesses, npts, open_s, &exps);
    } else {
      irs_open_begin<T>(ctx, cfg.rounds[ri - 1].irs, ts, std::vector<const whir_witness*>{prev.get()}, npts, open_t,
                        &exps);
    }
    // STIR constraint points: the commitment's out-of-domain points, then the opened in-domain
    // points (only their count is needed here).
    std::vector<T> stir_points;
    std::vector<T> stir_evals;
    const size_t nood = nw->ood_points.size() / T::LIMBS;
    for (size_t o = 0; o < nood; ++o) {
      stir_points.push_back(get_raw<T>(&nw->ood_points[o * T::LIMBS]));
      stir_evals.push_back(get_raw<T>(&nw->ood_matrix[o * T::LIMBS]));
    }
    std::vector<T> stir_rlc = geometric_challenge<T>(ts, nood + npts);
    if (nood) {
      // Out-of-domain points are general extension elements.
      DBuf<T> sp(ctx, 2 * nood);
      std::vector<T> packed(stir_rlc.begin(), stir_rlc.begin() + nood);
      packed.insert(packed.end(), stir_points.begin(), stir_points.begin() + nood);
      h2d(ctx, sp.p, packed.data(), packed.size() * sizeof(T));
      ProfScope prof(ctx, PF_GEOMETRIC);
      CU(launch_geometric_accumulate<T>(b.p, len, sp.p, sp.p + nood, nood, ctx->stream));
    }
    accumulate_in_domain<T>(ctx, b.p, len, std::vector<T>(stir_rlc.begin() + nood, stir_rlc.end()), exps, prev_N);
    const std::vector<T> eqw = eq_weights_host(folding);
    auto finish_open = [&]() {
      if (!prev) {
        irs_open_end<S>(ctx, ts, open_s, srows);
      } else {
        irs_open_end<T>(ctx, ts, open_t, in_rows);
      }
      std::vector<T> wts;
      for (const T& x : vector_rlc)
        for (const T& y : eqw) wts.push_back(x * y);
      const size_t cols = npts == 0 ? 0 : (prev ? in_rows.size() : srows.size()) / npts;
      if (cols != wts.size()) throw Error(WHIR_ERR_INTERNAL, "opened row width mismatch");
      for (size_t pi = 0; pi < npts; ++pi)
        stir_evals.push_back(prev ? dot_host_wide<T, T>(wts.data(), &in_rows[pi * cols], cols)
                                  : dot_host_wide<T, S>(wts.data(), &srows[pi * cols], cols));
      the_sum += dot_host(stir_rlc, stir_evals);
    };
    folding = sumcheck_device<T>(ctx, rc.sumcheck, ts, a.p, b.p, len, the_sum, finish_open);
    evaluation_point.insert(evaluation_point.end(), folding.begin(), folding.end());
    prev = std::move(nw);
    vector_rlc = {T::one()};
  }

  if (len != cfg.final_sumcheck.initial_size) throw Error(WHIR_ERR_INTERNAL, "final vector size mismatch");
  std::vector<T> fin(len);
  d2h(ctx, fin.data(), a.p, len * sizeof(T));
  for (const T& x : fin) send_elem<T>(ts, x);
  pow_prove(ctx, cfg.final_pow, ts);
  {
    size_t npts = 0;
    if (!prev) {
      std::vector<S> rows;
      irs_open<S>(ctx, cfg.initial, ts, witnesses, npts, rows);
    } else {
      std::vector<T> rows;
      irs_open<T>(ctx, cfg.rounds.back().irs, ts, std::vector<const whir_witness*>{prev.get()}, npts, rows);
    }
  }
  std::vector<T> last = sumcheck_device<T>(ctx, cfg.final_sumcheck, ts, a.p, b.p, len, the_sum);
  evaluation_point.insert(evaluation_point.end(), last.begin(), last.end());
  eval_point_out = evaluation_point;
  rlc_out = init_rlc;
  CU(cudaStreamSynchronize(ctx->stream));
}

// Device copy, in the in-memory form of S, of a read-only input array of canonical limbs (host
// memory, or device memory with WHIR_DEVICE_PTRS); returns a device pointer valid for the call.
// Canonical device inputs of the Goldilocks family are used in place. Small operator inputs are
// checked for canonical form on the host; the polynomial vectors of commit/prove are taken as given
// (like the reference's ark-ff elements, they must be canonical).
template <class S>
const S* device_vectors(whir_ctx* ctx, const uint64_t* vectors, size_t count, uint32_t flags, DBuf<S>& holder,
                        bool validate = true) {
  const bool dev = (flags & WHIR_DEVICE_PTRS) != 0;
  if (dev && Canon<S>::IDENTITY) return reinterpret_cast<const S*>(vectors);
  if (validate && !dev)
    for (size_t i = 0; i < count; ++i)
      if (!Canon<S>::ok(vectors + i * S::LIMBS))
        throw Error(WHIR_ERR_INVALID, "non-canonical field element in input vector");
  holder = DBuf<S>(ctx, count);
  if (!count) return holder.p;
  if (!dev) ctx->h2d_bytes += count * sizeof(S);
  CU(cudaMemcpyAsync(holder.p, vectors, count * sizeof(S), dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(launch_to_internal<S>(holder.p, count, ctx->stream));
  return holder.p;
}

// An in/out array of canonical limbs for the operator entry points: with WHIR_DEVICE_PTRS the
// caller's device buffer is converted to the in-memory form in place (and back by finish());
// otherwise a device copy is made and finish() copies `back` elements of the result to the host.
template <class T>
struct InOut {
  whir_ctx* ctx;
  uint64_t* user;
  size_t n;
  bool dev;
  DBuf<T> own;
  T* p = nullptr;
  InOut(whir_ctx* c, uint64_t* u, size_t count, uint32_t flags) : ctx(c), user(u), n(count) {
    dev = (flags & WHIR_DEVICE_PTRS) != 0;
    if (dev) {
      p = reinterpret_cast<T*>(user);
    } else {
      for (size_t i = 0; i < n; ++i)
        if (!Canon<T>::ok(user + i * T::LIMBS)) throw Error(WHIR_ERR_INVALID, "non-canonical field element");
      own = DBuf<T>(ctx, n);
      p = own.p;
      if (n) {
        ctx->h2d_bytes += n * sizeof(T);
        CU(cudaMemcpyAsync(p, user, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
      }
    }
    CU(launch_to_internal<T>(p, n, ctx->stream));
  }
  // Converts the whole array back to canonical limbs and copies the first `back` elements home.
  void finish(size_t back) {
    CU(launch_to_canonical<T>(p, n, ctx->stream));
    if (!dev && back) {
      ctx->d2h_bytes += back * sizeof(T);
      CU(cudaMemcpyAsync(user, p, back * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
    }
    CU(cudaStreamSynchronize(ctx->stream));
  }
};

template <class Fn>
int guarded(Fn&& fn) {
  try {
    return fn();
  } catch (const Error& e) {
    return set_error(e.code, e.what());
  } catch (const std::bad_alloc&) {
    return set_error(WHIR_ERR_INTERNAL, "host allocation failed");
  } catch (const std::exception& e) {
    return set_error(WHIR_ERR_INTERNAL, e.what());
  }
}


// Calls f.template operator()<S, T>() for the embedding id.
template <class Fn>
int with_embedding(int field, Fn&& f) {
  switch (field) {
    case WHIR_GOLDILOCKS1: return f.template operator()<Gl, Gl>();
    case WHIR_GOLDILOCKS2: return f.template operator()<Gl, Gl2>();
    case WHIR_GOLDILOCKS3: return f.template operator()<Gl, Gl3>();
    case WHIR_FIELD192: return f.template operator()<F192, F192>();
    case WHIR_FIELD256: return f.template operator()<F256, F256>();
    default: throw Error(WHIR_ERR_INVALID, "unknown field id");
  }
}
// Calls f.template operator()<F>() for the field whose elements the operator works on.
template <class Fn>
int with_field(int field, Fn&& f) {
  switch (field) {
    case WHIR_GOLDILOCKS1: return f.template operator()<Gl>();
    case WHIR_GOLDILOCKS2: return f.template operator()<Gl2>();
    case WHIR_GOLDILOCKS3: return f.template operator()<Gl3>();
    case WHIR_FIELD192: return f.template operator()<F192>();
    case WHIR_FIELD256: return f.template operator()<F256>();
    default: throw Error(WHIR_ERR_INVALID, "unknown field id");
  }
}

void check_ctx(whir_ctx* ctx) {
  if (!ctx) throw Error(WHIR_ERR_INVALID, "null context");
  CU(cudaSetDevice(ctx->device));
}

}  // namespace

// ================================================================================================
// C ABI
// ================================================================================================
extern "C" {

const char* whir_last_error(void) { return g_last_error.c_str(); }

int whir_ctx_create(int device, whir_ctx** out) { return whir_ctx_create_priority(device, 0, out); }

int whir_ctx_create_priority(int device, int priority, whir_ctx** out) {
  return guarded([&] {
    if (!out) throw Error(WHIR_ERR_INVALID, "null output pointer");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
      cudaGetLastError();
      throw Error(WHIR_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= count) throw Error(WHIR_ERR_INVALID, "device index out of range");
    // Released through whir_ctx_destroy if any step below fails.
    std::unique_ptr<whir_ctx, int (*)(whir_ctx*)> ctx(new whir_ctx(), whir_ctx_destroy);
    ctx->device = device;
    CU(cudaSetDevice(device));
    // Stream priority: 0 = the default; a positive value raises it that many steps toward the
    // device's greatest priority (clamped), so the scheduler runs this context's kernels first.
    int least = 0, greatest = 0;
    CU(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int prio = std::max(greatest, least - std::max(0, priority));
    CU(cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, prio));
    CU(cudaStreamCreateWithPriority(&ctx->up_stream, cudaStreamNonBlocking, prio));
    // Keep freed pool memory cached across proofs.
    cudaMemPool_t pool;
    CU(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t thr = UINT64_MAX;
    CU(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    root_tab<Gl>(ctx.get());  // the other fields' tables are built on first use
    CU(cudaMalloc((void**)&ctx->d_pow, 2 * sizeof(unsigned long long)));
    ctx->sc_parts_bytes = (2 * sumcheck_partials(SIZE_MAX / 64) + 2) * 64;  // max blocks x largest element pair
    CU(cudaMalloc(&ctx->sc_parts, ctx->sc_parts_bytes));
    // (arrival count, launch sequence, error word of the bulk-staged sums, sticky device error word
    // that every mail publication carries to the host)
    CU(cudaMalloc((void**)&ctx->sc_counter, 4 * sizeof(unsigned int)));
    CU(cudaMemset(ctx->sc_counter, 0, 4 * sizeof(unsigned int)));
    CU(cudaMalloc((void**)&ctx->geo_counters, GR_MAX_TILES * sizeof(unsigned int)));
    CU(cudaMemset(ctx->geo_counters, 0, GR_MAX_TILES * sizeof(unsigned int)));
    CU(cudaHostAlloc((void**)&ctx->mail_h, MAIL_DATA_OFF + MAIL_DATA_BYTES, cudaHostAllocMapped));
    memset(ctx->mail_h, 0, MAIL_DATA_OFF + MAIL_DATA_BYTES);
    CU(cudaHostGetDevicePointer((void**)&ctx->mail_d, ctx->mail_h, 0));
    stage_reserve(ctx.get(), 1 << 20);
    ctx->up_cap = 8 << 20;
    CU(cudaMallocHost((void**)&ctx->h_up, ctx->up_cap));
    ctx->launches_at_create = kernel_launches();
    *out = ctx.release();
    return 0;
  });
}

int whir_ctx_destroy(whir_ctx* ctx) {
  if (!ctx) return 0;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->up_stream) cudaStreamSynchronize(ctx->up_stream);
  for (auto& p : ctx->pending) {
    cudaEventDestroy(p.second.first);
    cudaEventDestroy(p.second.second);
  }
  for (auto e : ctx->event_pool) cudaEventDestroy(e);
  for (uint64_t* r : ctx->d_roots)
    if (r) cudaFree(r);
  if (ctx->d_pow) cudaFree(ctx->d_pow);
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  if (ctx->h_up) cudaFreeHost(ctx->h_up);
  if (ctx->mail_h) cudaFreeHost(ctx->mail_h);
  if (ctx->sc_parts) cudaFree(ctx->sc_parts);
  for (auto& b : ctx->free_bufs) cudaFree(b.second);
  if (ctx->sc_counter) cudaFree(ctx->sc_counter);
  if (ctx->geo_counters) cudaFree(ctx->geo_counters);
  cudaStreamDestroy(ctx->stream);
  if (ctx->up_stream) cudaStreamDestroy(ctx->up_stream);
  delete ctx;
  return 0;
}

int whir_ctx_synchronize(whir_ctx* ctx) {
  return guarded([&] {
    check_ctx(ctx);
    CU(cudaStreamSynchronize(ctx->stream));
    return 0;
  });
}

uint64_t whir_ctx_launch_count(const whir_ctx* ctx) { return ctx ? kernel_launches() - ctx->launches_at_create : 0; }

void* whir_ctx_stream(const whir_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int whir_ctx_transfer_bytes(const whir_ctx* ctx, uint64_t* h2d_bytes, uint64_t* d2h_bytes) {
  if (!ctx) return set_error(WHIR_ERR_INVALID, "null context");
  if (h2d_bytes) *h2d_bytes = ctx->h2d_bytes;
  if (d2h_bytes) *d2h_bytes = ctx->d2h_bytes;
  return 0;
}

int whir_ctx_set_profiling(whir_ctx* ctx, int enabled) {
  return guarded([&] {
    check_ctx(ctx);
    resolve_profile(ctx);
    ctx->profiling = enabled != 0;
    for (int i = 0; i < PF_COUNT; ++i) {
      ctx->family_ms[i] = 0;
      ctx->family_calls[i] = 0;
    }
    return 0;
  });
}

int whir_ctx_profile(whir_ctx* ctx, double* ms, uint64_t* calls, size_t n_families) {
  return guarded([&] {
    check_ctx(ctx);
    resolve_profile(ctx);
    for (size_t i = 0; i < n_families && i < (size_t)PF_COUNT; ++i) {
      if (ms) ms[i] = ctx->family_ms[i];
      if (calls) calls[i] = ctx->family_calls[i];
    }
    return PF_COUNT;
  });
}

int whir_device_alloc(whir_ctx* ctx, size_t bytes, void** out) {
  return guarded([&] {
    check_ctx(ctx);
    CU(cudaMallocAsync(out, bytes, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return 0;
  });
}
int whir_device_free(whir_ctx* ctx, void* ptr) {
  return guarded([&] {
    check_ctx(ctx);
    CU(cudaFreeAsync(ptr, ctx->stream));
    return 0;
  });
}
int whir_host_alloc(size_t bytes, void** out) {
  return guarded([&] {
    if (!out) throw Error(WHIR_ERR_INVALID, "null argument");
    *out = nullptr;
    if (bytes == 0) return 0;
    cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
      *out = nullptr;
      throw Error(e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? WHIR_ERR_NO_DEVICE : WHIR_ERR_CUDA,
                  std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    }
    return 0;
  });
}
int whir_host_free(void* ptr) {
  return guarded([&] {
    if (ptr) CU(cudaFreeHost(ptr));
    return 0;
  });
}
int whir_memcpy_h2d(whir_ctx* ctx, void* dst, const void* src, size_t bytes) {
  return guarded([&] {
    check_ctx(ctx);
    CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return 0;
  });
}
int whir_memcpy_d2h(whir_ctx* ctx, void* dst, const void* src, size_t bytes) {
  return guarded([&] {
    check_ctx(ctx);
    CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return 0;
  });
}

int whir_config_new(int field, const whir_params* p, uint64_t size, whir_config** out) {
  return guarded([&] {
    if (!p || !out) throw Error(WHIR_ERR_INVALID, "null argument");
    Params wp;
    wp.unique_decoding = p->unique_decoding != 0;
    wp.starting_log_inv_rate = p->starting_log_inv_rate;
    wp.initial_folding_factor = p->initial_folding_factor;
    wp.folding_factor = p->folding_factor;
    wp.security_level = p->security_level;
    wp.pow_bits = p->pow_bits;
    wp.batch_size = p->batch_size;
    memcpy(wp.hash_id, p->hash_id, 32);
    auto c = std::make_unique<whir_config>();
    c->cfg = config_new(field, size, wp);
    *out = c.release();
    return 0;
  });
}
int whir_config_free(whir_config* cfg) {
  delete cfg;
  return 0;
}

int whir_config_json(const whir_config* cfg, char* buf, size_t cap) {
  return guarded([&] {
    if (!cfg) throw Error(WHIR_ERR_INVALID, "null config");
    const Config& c = cfg->cfg;
    std::string s;
    char tmp[512];
    auto irs = [&](const Irs& r) {
      snprintf(tmp, sizeof(tmp),
               "{\"num_vectors\":%zu,\"vector_size\":%zu,\"codeword_length\":%zu,\"interleaving_depth\":%zu,"
               "\"num_cols\":%zu,\"merkle_layers\":%zu,\"in_domain_samples\":%zu,\"out_domain_samples\":%zu,"
               "\"johnson_slack\":%.17g}",
               r.num_vectors, r.vector_size, r.codeword_length, r.interleaving_depth, r.num_cols, r.layers,
               r.in_domain_samples, r.out_domain_samples, r.johnson_slack);
      s += tmp;
    };
    auto sc = [&](const Sumcheck& x) {
      snprintf(tmp, sizeof(tmp), "{\"initial_size\":%zu,\"num_rounds\":%zu,\"round_pow_threshold\":%llu}",
               x.initial_size, x.num_rounds, (unsigned long long)x.round_pow.threshold);
      s += tmp;
    };
    s += "{\"initial_committer\":";
    irs(c.initial);
    s += ",\"initial_sumcheck\":";
    sc(c.initial_sumcheck);
    snprintf(tmp, sizeof(tmp), ",\"initial_skip_pow_threshold\":%llu,\"rounds\":[",
             (unsigned long long)c.initial_skip_pow.threshold);
    s += tmp;
    for (size_t i = 0; i < c.rounds.size(); ++i) {
      if (i) s += ",";
      s += "{\"irs\":";
      irs(c.rounds[i].irs);
      s += ",\"sumcheck\":";
      sc(c.rounds[i].sumcheck);
      snprintf(tmp, sizeof(tmp), ",\"pow_threshold\":%llu}", (unsigned long long)c.rounds[i].pow.threshold);
      s += tmp;
    }
    s += "],\"final_sumcheck\":";
    sc(c.final_sumcheck);
    snprintf(tmp, sizeof(tmp), ",\"final_pow_threshold\":%llu}", (unsigned long long)c.final_pow.threshold);
    s += tmp;
    if (!buf || s.size() + 1 > cap) throw Error(WHIR_ERR_INVALID, "buffer too small");
    memcpy(buf, s.c_str(), s.size() + 1);
    return 0;
  });
}

int whir_config_cbor(const whir_config* cfg, uint8_t* buf, size_t cap, size_t* len) {
  return guarded([&] {
    if (!cfg || !len) throw Error(WHIR_ERR_INVALID, "null argument");
    const std::vector<uint8_t> cb = config_bytes(cfg->cfg);
    *len = cb.size();
    if (buf && cap) memcpy(buf, cb.data(), std::min(cap, cb.size()));
    if (buf && cap < cb.size()) throw Error(WHIR_ERR_INVALID, "buffer too small for the configuration's CBOR");
    return 0;
  });
}

int whir_prover_state_new(const whir_config* cfg, const char* session, size_t session_len, whir_prover_state** out) {
  return guarded([&] {
    if (!cfg || !out) throw Error(WHIR_ERR_INVALID, "null argument");
    auto ps = std::make_unique<whir_prover_state>();
    ps->cfg = cfg;
    std::vector<uint8_t> cb = config_bytes(cfg->cfg);
    uint8_t pid[64], sid[32];
    sha3_512_host(cb.data(), cb.size(), pid);
    std::vector<uint8_t> st = cbor_text(std::string(session ? session : "", session ? session_len : 0));
    sha3_256_host(st.data(), st.size(), sid);
    ps->ts.init(pid, sid);
    *out = ps.release();
    return 0;
  });
}
int whir_prover_state_free(whir_prover_state* ps) {
  delete ps;
  return 0;
}
int whir_prover_state_proof(const whir_prover_state* ps, const uint8_t** narg, size_t* narg_len, const uint8_t** hints,
                            size_t* hints_len) {
  return guarded([&] {
    if (!ps) throw Error(WHIR_ERR_INVALID, "null state");
    if (narg) *narg = ps->ts.narg.data();
    if (narg_len) *narg_len = ps->ts.narg.size();
    if (hints) *hints = ps->ts.hints.data();
    if (hints_len) *hints_len = ps->ts.hints.size();
    return 0;
  });
}

int whir_commit(whir_ctx* ctx, const whir_config* cfg, whir_prover_state* ps, const uint64_t* vectors, uint32_t flags,
                whir_witness** out) {
  return guarded([&] {
    check_ctx(ctx);
    if (!cfg || !ps || !vectors || !out) throw Error(WHIR_ERR_INVALID, "null argument");
    const Config& c = cfg->cfg;
    return with_embedding(c.field, [&]<class S, class T>() {
      const size_t count = c.initial.num_vectors * c.size();
      DBuf<S> copy;
      std::unique_ptr<whir_witness> w;
      if (!(flags & WHIR_DEVICE_PTRS) && Canon<S>::IDENTITY && count * sizeof(S) >= STAGED_UPLOAD_MIN_BYTES) {
        // Large host input: the upload runs in message groups beside the encode's first pass.
        copy = DBuf<S>(ctx, count);
        const HostUpload<S> up{reinterpret_cast<const S*>(vectors), copy.p};
        w = irs_commit<S, T>(ctx, c.initial, ps->ts, copy.p, c.field, &up);
      } else {
        const S* d = device_vectors<S>(ctx, vectors, count, flags, copy, false);
        w = irs_commit<S, T>(ctx, c.initial, ps->ts, d, c.field);
      }
      CU(cudaStreamSynchronize(ctx->stream));
      if (!(flags & WHIR_DEVICE_PTRS)) {
        // Keep the device copy: prove() given the same host buffer reuses it instead of copying again.
        w->host_src = vectors;
        w->vectors = DBuf<uint64_t>();
        w->vectors.ctx = ctx;
        w->vectors.p = reinterpret_cast<uint64_t*>(copy.p);
        w->vectors.n = count * S::LIMBS;
        copy.p = nullptr;
      }
      *out = w.release();
      return 0;
    });
  });
}

int whir_commit_batch(whir_ctx* ctx, size_t n, const whir_config* const* cfgs, whir_prover_state* const* pss,
                      const uint64_t* const* vectors, uint32_t flags, whir_witness** out) {
  return guarded([&] {
    check_ctx(ctx);
    if (n && (!cfgs || !pss || !vectors || !out)) throw Error(WHIR_ERR_INVALID, "null argument");
    for (size_t j = 0; j < n; ++j) {
      if (!cfgs[j] || !pss[j] || !vectors[j]) throw Error(WHIR_ERR_INVALID, "null job argument");
      if (cfgs[j]->cfg.field != cfgs[0]->cfg.field) throw Error(WHIR_ERR_INVALID, "a batched commit needs one field");
      if (pss[j]->cfg != cfgs[j]) throw Error(WHIR_ERR_INVALID, "prover state of another configuration");
      out[j] = nullptr;
    }
    if (n == 0) return 0;
    return with_embedding(cfgs[0]->cfg.field, [&]<class S, class T>() {
      std::vector<const Irs*> cs(n);
      std::vector<Transcript*> tss(n);
      std::vector<const S*> dv(n);
      std::vector<DBuf<S>> copies(n);
      for (size_t j = 0; j < n; ++j) {
        const Config& c = cfgs[j]->cfg;
        cs[j] = &c.initial;
        tss[j] = &pss[j]->ts;
        dv[j] = device_vectors<S>(ctx, vectors[j], c.initial.num_vectors * c.size(), flags, copies[j], false);
      }
      auto ws = irs_commit_batch<S, T>(ctx, cs, tss, dv, cfgs[0]->cfg.field);
      CU(cudaStreamSynchronize(ctx->stream));
      for (size_t j = 0; j < n; ++j) {
        if (!(flags & WHIR_DEVICE_PTRS)) {
          // Keep the device copy: prove() given the same host buffer reuses it.
          ws[j]->host_src = vectors[j];
          ws[j]->vectors = DBuf<uint64_t>();
          ws[j]->vectors.ctx = ctx;
          ws[j]->vectors.p = reinterpret_cast<uint64_t*>(copies[j].p);
          ws[j]->vectors.n = copies[j].n * S::LIMBS;
          copies[j].p = nullptr;
        }
      }
      for (size_t j = 0; j < n; ++j) out[j] = ws[j].release();
      return 0;
    });
  });
}

// ---- autotuner ---------------------------------------------------------------------------------
}  // extern "C"

namespace {

// Event-timed minimum over `reps` runs of fn() on the context's stream (milliseconds).
template <class Fn>
double time_min(whir_ctx* ctx, int reps, Fn&& fn) {
  cudaEvent_t e0 = take_event(ctx), e1 = take_event(ctx);
  double best = 1e30;
  for (int r = 0; r < reps; ++r) {
    CU(cudaEventRecord(e0, ctx->stream));
    fn();
    CU(cudaEventRecord(e1, ctx->stream));
    CU(cudaEventSynchronize(e1));
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, e0, e1));
    best = std::min(best, (double)ms);
  }
  ctx->event_pool.push_back(e0);
  ctx->event_pool.push_back(e1);
  return best;
}

// Tunes the encode plan of one commitment shape (elements of F) and the Merkle tile height of its
// tree: every valid candidate is timed on the device and the fastest is recorded in the process-wide
// table that plan_encode / launch_merkle consult. Appends a JSON object to `report`.
template <class F>
void autotune_shape(whir_ctx* ctx, size_t n_msgs, size_t msg_len, size_t cw, int kind, int reps, std::string& report) {
  std::vector<std::pair<EncodeTuning, EncodePlan>> cands;
  size_t C = 1;
  while (C < msg_len) C <<= 1;
  const int logC = (int)layers_for(C);
  for (int G = 1; G <= 64; G *= 2) {
    EncodePlan p;
    EncodeTuning t{0, 0, 0, G};
    if (plan_encode_tuned(n_msgs, msg_len, cw, sizeof(F), t, &p) == 0) cands.push_back({t, p});
  }
  for (int l2 = 1; l2 < logC; ++l2)
    for (int W = 1; W <= 64; W *= 2) {
      EncodePlan p;
      EncodeTuning t{1, l2, W, 1};
      if (plan_encode_tuned(n_msgs, msg_len, cw, sizeof(F), t, &p) == 0) cands.push_back({t, p});
    }
  EncodePlan def;
  if (plan_encode_default(n_msgs, msg_len, cw, sizeof(F), &def)) return;
  size_t scratch_elems = 0;
  for (auto& c : cands) scratch_elems = std::max(scratch_elems, c.second.scratch_elems);
  const size_t layers = layers_for(cw);
  DBuf<F> src(ctx, std::max<size_t>(n_msgs * msg_len, 1)), dst(ctx, cw * n_msgs), scratch(ctx, scratch_elems);
  DBuf<uint32_t> nodes(ctx, ((2ull << layers) - 1) * 8);
  CU(cudaMemsetAsync(src.p, 0, std::max<size_t>(n_msgs * msg_len, 1) * sizeof(F), ctx->stream));
  CU(cudaMemsetAsync(nodes.p, 0, ((2ull << layers) - 1) * 32, ctx->stream));
  const RootTab rt = root_tab<typename F::Base>(ctx);
  double best = 1e30, def_ms = 0;
  EncodeTuning pick{};
  char buf[200];
  report += "{\"n_msgs\":" + std::to_string(n_msgs) + ",\"msg_len\":" + std::to_string(msg_len) +
            ",\"codeword_len\":" + std::to_string(cw) + ",\"elem_bytes\":" + std::to_string(sizeof(F)) +
            ",\"candidates\":[";
  bool first = true;
  for (auto& c : cands) {
    const double ms = time_min(ctx, reps, [&] {
      CU(launch_encode<F>(c.second, src.p, n_msgs, msg_len, dst.p, nodes.p, kind, scratch.p, rt, ctx->stream));
    });
    snprintf(buf, sizeof(buf), "%s[%d,%d,%d,%d,%.4f]", first ? "" : ",", c.first.mode, c.first.logC2, c.first.W,
             c.first.G, ms);
    report += buf;
    first = false;
    const bool is_def = c.second.mode == def.mode && c.second.logC2 == def.logC2 &&
                        c.second.cols_per_cta == def.cols_per_cta && c.second.cosets_per_cta == def.cosets_per_cta;
    if (is_def) def_ms = ms;
    if (ms < best) {
      best = ms;
      pick = c.first;
    }
  }
  if (!cands.empty()) encode_tuning_set(n_msgs, msg_len, cw, sizeof(F), pick);
  snprintf(buf, sizeof(buf), "],\"pick\":[%d,%d,%d,%d],\"pick_ms\":%.4f,\"default_ms\":%.4f", pick.mode,
           pick.logC2, pick.W, pick.G, best, def_ms);
  report += buf;
  // Merkle tile height for this tree
  int best_tl = merkle_tile_log;
  double mbest = 1e30;
  report += ",\"merkle\":[";
  first = true;
  for (int tl = 6; tl <= 10; ++tl) {
    const double ms = time_min(ctx, reps, [&] { CU(launch_merkle(nodes.p, (int)layers, kind, ctx->stream, tl)); });
    snprintf(buf, sizeof(buf), "%s[%d,%.4f]", first ? "" : ",", tl, ms);
    report += buf;
    first = false;
    if (ms < mbest) {
      mbest = ms;
      best_tl = tl;
    }
  }
  merkle_tuning_set((int)layers, best_tl);
  snprintf(buf, sizeof(buf), "],\"merkle_pick\":%d}", best_tl);
  report += buf;
}

}  // namespace

extern "C" {

int whir_autotune(whir_ctx* ctx, const whir_config* cfg, int reps, char* report, size_t cap) {
  return guarded([&] {
    check_ctx(ctx);
    if (!cfg) throw Error(WHIR_ERR_INVALID, "null config");
    const Config& c = cfg->cfg;
    reps = std::max(1, std::min(reps, 20));
    return with_embedding(c.field, [&]<class S, class T>() {
      std::string rep = "{\"shapes\":[";
      const int kind = hash_kind_or_throw(c.initial.hash_id);
      autotune_shape<S>(ctx, c.initial.num_cols, c.initial.message_length(), c.initial.codeword_length, kind, reps, rep);
      for (const Round& r : c.rounds) {
        rep += ",";
        autotune_shape<T>(ctx, r.irs.num_cols, r.irs.message_length(), r.irs.codeword_length,
                          hash_kind_or_throw(r.irs.hash_id), reps, rep);
      }
      rep += "]}";
      CU(cudaStreamSynchronize(ctx->stream));
      if (report && cap) {
        const size_t m = std::min(cap - 1, rep.size());
        memcpy(report, rep.data(), m);
        report[m] = 0;
        if (rep.size() >= cap) throw Error(WHIR_ERR_INVALID, "report buffer too small");
      }
      return 0;
    });
  });
}

int whir_autotune_export(char* buf, size_t cap, size_t* len) {
  return guarded([&] {
    if (!len) throw Error(WHIR_ERR_INVALID, "null argument");
    const std::string s = tuning_export();
    *len = s.size();
    if (buf && cap) {
      const size_t m = std::min(cap - 1, s.size());
      memcpy(buf, s.data(), m);
      buf[m] = 0;
      if (s.size() >= cap) throw Error(WHIR_ERR_INVALID, "buffer too small");
    }
    return 0;
  });
}

int whir_autotune_import(const char* text) {
  return guarded([&] {
    if (!text) throw Error(WHIR_ERR_INVALID, "null argument");
    const int rc = tuning_import(text);
    if (rc) throw Error(rc, "malformed or invalid tuning line");
    return 0;
  });
}

int whir_autotune_clear(void) {
  tuning_clear();
  return 0;
}

int whir_witness_free(whir_witness* w) {
  if (!w) return 0;
  cudaSetDevice(w->ctx->device);
  delete w;
  return 0;
}
int whir_witness_root(const whir_witness* w, uint8_t root[32]) {
  if (!w || !root) return set_error(WHIR_ERR_INVALID, "null argument");
  memcpy(root, w->root, 32);
  return 0;
}

int whir_prove(whir_ctx* ctx, const whir_config* cfg, whir_prover_state* ps, const uint64_t* vectors, uint32_t flags,
               whir_witness* const* witnesses, size_t n_witnesses, const uint64_t* mle_points, size_t n_points,
               const uint64_t* covectors, size_t n_covectors, const uint64_t* evaluations, uint64_t* eval_point_out,
               uint64_t* rlc_out) {
  return guarded([&] {
    check_ctx(ctx);
    if (!cfg || !ps) throw Error(WHIR_ERR_INVALID, "null argument");
    const Config& c = cfg->cfg;
    const size_t n = c.size();
    const size_t nvars = layers_for(n);
    const size_t nv = n_witnesses * c.initial.num_vectors;
    const size_t nforms = n_points + n_covectors;
    return with_embedding(c.field, [&]<class S, class T>() {
      std::vector<const whir_witness*> ws;
      for (size_t i = 0; i < n_witnesses; ++i) {
        if (!witnesses || !witnesses[i]) throw Error(WHIR_ERR_INVALID, "null witness");
        if (witnesses[i]->field != c.field || witnesses[i]->ctx != ctx) throw Error(WHIR_ERR_INVALID, "witness from another config/context");
        ws.push_back(witnesses[i]);
      }
      std::vector<std::vector<T>> pts, covs;
      for (size_t i = 0; i < n_points; ++i) pts.push_back(load_host<T>(mle_points + i * nvars * T::LIMBS, nvars));
      for (size_t i = 0; i < n_covectors; ++i) covs.push_back(load_host<T>(covectors + i * n * T::LIMBS, n));
      std::vector<T> evals = nforms * nv ? load_host<T>(evaluations, nforms * nv) : std::vector<T>();
      DBuf<S> holder;
      const S* d = nullptr;
      if (nv && !(flags & WHIR_DEVICE_PTRS) && ws.size() == 1 && ws[0]->host_src == vectors && ws[0]->vectors.p) {
        d = reinterpret_cast<const S*>(ws[0]->vectors.p);  // same host buffer as the commitment
      } else if (nv) {
        d = device_vectors<S>(ctx, vectors, nv * n, flags, holder, false);
      }
      std::vector<T> ep, rlc;
      prove_device<S, T>(ctx, c, ps->ts, d, nv, ws, pts, covs, evals, ep, rlc);
      if (eval_point_out) store_host<T>(ep, eval_point_out);
      if (rlc_out) store_host<T>(rlc, rlc_out);
      return 0;
    });
  });
}

// ---- operator-level entry points ---------------------------------------------------------------

int whir_rs_interleaved_encode(whir_ctx* ctx, int field, const uint64_t* msgs, size_t n_msgs, size_t msg_len,
                               const uint64_t* masks, size_t mask_len, size_t codeword_len, uint64_t* out,
                               uint32_t flags) {
  return guarded([&] {
    check_ctx(ctx);
    if (mask_len != 0 && !masks) throw Error(WHIR_ERR_INVALID, "null masks with mask_len > 0");
    if (n_msgs == 0) return 0;
    return with_field(field, [&]<class F>() {
      DBuf<F> in, mk, cat, outb;
      const F* d_in = device_vectors<F>(ctx, msgs, n_msgs * msg_len, flags, in);
      // Masked messages (cooley_tukey.rs:411-477): message m's coefficients are its msg_len values
      // followed by its mask_len mask values (masks laid out [n_msgs][mask_len]); the rows are
      // assembled on the device and encoded as messages of msg_len + mask_len coefficients.
      const size_t len = msg_len + mask_len;
      if (mask_len) {
        const F* d_mk = device_vectors<F>(ctx, masks, n_msgs * mask_len, flags, mk);
        cat = DBuf<F>(ctx, n_msgs * len);
        if (msg_len)
          CU(cudaMemcpy2DAsync(cat.p, len * sizeof(F), d_in, msg_len * sizeof(F), msg_len * sizeof(F), n_msgs,
                               cudaMemcpyDeviceToDevice, ctx->stream));
        CU(cudaMemcpy2DAsync(cat.p + msg_len, len * sizeof(F), d_mk, mask_len * sizeof(F), mask_len * sizeof(F),
                             n_msgs, cudaMemcpyDeviceToDevice, ctx->stream));
        d_in = cat.p;
      }
      F* d_out = (flags & WHIR_DEVICE_PTRS) ? reinterpret_cast<F*>(out) : (outb = DBuf<F>(ctx, codeword_len * n_msgs)).p;
      EncodePlan plan;
      int rc = plan_encode(n_msgs, len, codeword_len, sizeof(F), &plan);
      if (rc) throw Error(rc, "encode shape unsupported on the device");
      DBuf<F> scratch(ctx, plan.scratch_elems);
      CU(launch_encode<F>(plan, d_in, n_msgs, len, d_out, nullptr, HASH_BLAKE3, scratch.p,
                          root_tab<typename F::Base>(ctx), ctx->stream));
      CU(launch_to_canonical<F>(d_out, codeword_len * n_msgs, ctx->stream));
      if (!(flags & WHIR_DEVICE_PTRS))
        CU(cudaMemcpyAsync(out, d_out, codeword_len * n_msgs * sizeof(F), cudaMemcpyDeviceToHost, ctx->stream));
      CU(cudaStreamSynchronize(ctx->stream));
      return 0;
    });
  });
}

int whir_rs_evaluation_points(int field, size_t masked_len, size_t codeword_len, const uint64_t* indices, size_t n,
                              uint64_t* out) {
  return guarded([&] {
    return with_field(field, [&]<class F>() {
      typedef typename F::Base B;
      std::vector<uint64_t> idx(indices, indices + n);
      std::vector<B> pts = evaluation_points<B>(masked_len, codeword_len, idx);
      for (size_t i = 0; i < n; ++i) store_one<F>(F::from_base(pts[i]), out + i * F::LIMBS);
      return 0;
    });
  });
}

int whir_hash_many(whir_ctx* ctx, const uint8_t engine_id[32], size_t size, const uint8_t* in, size_t count,
                   uint8_t* out, uint32_t flags) {
  return guarded([&] {
    check_ctx(ctx);
    int kind = hash_kind_or_throw(engine_id);
    if (kind == HASH_COPY && size > 32) throw Error(WHIR_ERR_INVALID, "Copy engine only supports sizes up to 32 bytes");
    if (size % 4 != 0) throw Error(WHIR_ERR_UNSUPPORTED, "message sizes must be a multiple of 4 bytes on the device");
    if (kind == HASH_BLAKE3 && size > 1024) throw Error(WHIR_ERR_UNSUPPORTED, "Blake3 messages above 1024 bytes");
    if (count == 0) return 0;
    DBuf<uint8_t> din, dout;
    const uint8_t* pin = in;
    uint8_t* pout = out;
    if (!(flags & WHIR_DEVICE_PTRS)) {
      din = DBuf<uint8_t>(ctx, std::max<size_t>(size * count, 1));
      dout = DBuf<uint8_t>(ctx, 32 * count);
      if (size) CU(cudaMemcpyAsync(din.p, in, size * count, cudaMemcpyHostToDevice, ctx->stream));
      pin = din.p;
      pout = dout.p;
    }
    CU(launch_hash_many(pin, size, count, pout, kind, ctx->stream));
    if (!(flags & WHIR_DEVICE_PTRS)) CU(cudaMemcpyAsync(out, pout, 32 * count, cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return 0;
  });
}

int whir_merkle_nodes(whir_ctx* ctx, const uint8_t engine_id[32], const uint8_t* leaves, size_t n_leaves,
                      uint8_t* nodes_out, uint32_t flags) {
  return guarded([&] {
    check_ctx(ctx);
    int kind = hash_kind_or_throw(engine_id);
    if (kind == HASH_COPY) throw Error(WHIR_ERR_INVALID, "Copy engine cannot hash 64-byte nodes");
    const size_t layers = n_leaves ? layers_for(n_leaves) : 0;
    const size_t nn = (2ull << layers) - 1;
    DBuf<uint32_t> nodes(ctx, nn * 8);
    CU(cudaMemsetAsync(nodes.p, 0, nn * 32, ctx->stream));
    if (n_leaves)
      CU(cudaMemcpyAsync(nodes.p, leaves, n_leaves * 32,
                         (flags & WHIR_DEVICE_PTRS) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
    CU(launch_merkle(nodes.p, (int)layers, kind, ctx->stream));
    CU(cudaMemcpyAsync(nodes_out, nodes.p, nn * 32,
                       (flags & WHIR_DEVICE_PTRS) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return 0;
  });
}

int whir_sumcheck_polynomial(whir_ctx* ctx, int field, const uint64_t* a, const uint64_t* b, size_t n, uint64_t* c0,
                             uint64_t* c2, uint32_t flags) {
  return guarded([&] {
    check_ctx(ctx);
    if (n && (n & (n - 1))) throw Error(WHIR_ERR_UNSUPPORTED, "length must be a power of two on the device");
    return with_field(field, [&]<class T>() {
      if (n == 0) {
        store_one<T>(T::zero(), c0);
        store_one<T>(T::zero(), c2);
        return 0;
      }
      DBuf<T> ha, hb;
      const T* da = device_vectors<T>(ctx, a, n, flags, ha);
      const T* db = device_vectors<T>(ctx, b, n, flags, hb);
      DBuf<T> parts(ctx, 2 * sumcheck_partials(n) + 2), res(ctx, 2);
      size_t np;
      CU(launch_sumcheck_compute<T>(da, db, n, parts.p, &np, ctx->stream));
      CU(launch_reduce_pairs<T>(parts.p, np, res.p, ctx->stream));
      T r[2];
      d2h(ctx, r, res.p, sizeof(r));
      store_one<T>(r[0], c0);
      store_one<T>(r[1], c2);
      return 0;
    });
  });
}

int whir_fold(whir_ctx* ctx, int field, uint64_t* v, size_t n, const uint64_t* weight, uint32_t flags) {
  return guarded([&] {
    check_ctx(ctx);
    if (n && (n & (n - 1))) throw Error(WHIR_ERR_UNSUPPORTED, "length must be a power of two on the device");
    return with_field(field, [&]<class T>() {
      T w = load_host<T>(weight, 1)[0];
      if (n <= 1) return 0;
      InOut<T> dv(ctx, v, n, flags);
      CU(launch_fold<T>(dv.p, n, w, ctx->stream));
      dv.finish(n / 2);
      return 0;
    });
  });
}

int whir_eval_eq(whir_ctx* ctx, int field, uint64_t* acc, const uint64_t* point, size_t nvars, const uint64_t* scalar,
                 uint32_t flags) {
  return guarded([&] {
    check_ctx(ctx);
    return with_field(field, [&]<class T>() {
      T s = load_host<T>(scalar, 1)[0];
      const size_t n = 1ull << nvars;
      DBuf<T> hpt;
      InOut<T> io(ctx, acc, n, flags);
      T* dacc = io.p;
      const T* dpt = nvars ? device_vectors<T>(ctx, point, nvars, flags, hpt) : nullptr;
      DBuf<T> tables(ctx, (2ull << ((nvars + 1) / 2)) + 2);
      if (nvars == 0) {
        std::vector<T> one{s};
        DBuf<T> tmp(ctx, 1);
        h2d(ctx, tmp.p, one.data(), sizeof(T));
        std::vector<const T*> ptrs{dacc, tmp.p};
        std::vector<T> co{T::one(), T::one()};
        DBuf<T> out(ctx, 1);
        CU((launch_lift_rlc<T, T>(out.p, ptrs.data(), co.data(), 2, 1, ctx->stream)));
        CU(cudaMemcpyAsync(dacc, out.p, sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
      } else {
        CU(launch_eval_eq<T>(dacc, dpt, (int)nvars, s, tables.p, ctx->stream));
      }
      io.finish(n);
      return 0;
    });
  });
}

int whir_geometric_accumulate(whir_ctx* ctx, int field, uint64_t* acc, size_t n, const uint64_t* scalars,
                              const uint64_t* points, size_t m, uint32_t flags) {
  return guarded([&] {
    check_ctx(ctx);
    return with_field(field, [&]<class T>() {
      if (n == 0 || m == 0) return 0;
      DBuf<T> hs, hp;
      InOut<T> io(ctx, acc, n, flags);
      const T* ds = device_vectors<T>(ctx, scalars, m, flags, hs);
      const T* dp = device_vectors<T>(ctx, points, m, flags, hp);
      CU(launch_geometric_accumulate<T>(io.p, n, ds, dp, m, ctx->stream));
      io.finish(n);
      return 0;
    });
  });
}

int whir_univariate_evaluate(whir_ctx* ctx, int field, const uint64_t* coeffs, size_t n, const uint64_t* point,
                             uint64_t* out, uint32_t flags) {
  return guarded([&] {
    check_ctx(ctx);
    return with_embedding(field, [&]<class S, class T>() {
      T x = load_host<T>(point, 1)[0];
      T r = T::zero();
      if (n) {
        DBuf<S> hc;
        const S* dc = device_vectors<S>(ctx, coeffs, n, flags, hc);
        r = univariate_device<T, S>(ctx, dc, n, x);
      }
      store_one<T>(r, out);
      return 0;
    });
  });
}

int whir_lift(whir_ctx* ctx, int field, const uint64_t* src, size_t n, uint64_t* dst, uint32_t flags) {
  return guarded([&] {
    check_ctx(ctx);
    if (n && (!src || !dst)) throw Error(WHIR_ERR_INVALID, "null argument");
    return with_embedding(field, [&]<class S, class T>() {
      if (n == 0) return 0;
      const bool dev = (flags & WHIR_DEVICE_PTRS) != 0;
      DBuf<S> hs;
      DBuf<T> own;
      const S* ds = device_vectors<S>(ctx, src, n, flags, hs);
      T* dd = dev ? reinterpret_cast<T*>(dst) : (own = DBuf<T>(ctx, n)).p;
      const S* vecs[1] = {ds};
      const T coeffs[1] = {T::one()};
      CU((launch_lift_rlc<T, S>(dd, vecs, coeffs, 1, n, ctx->stream)));
      CU(launch_to_canonical<T>(dd, n, ctx->stream));
      if (!dev) {
        ctx->d2h_bytes += n * sizeof(T);
        CU(cudaMemcpyAsync(dst, dd, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
      }
      CU(cudaStreamSynchronize(ctx->stream));
      return 0;
    });
  });
}

int whir_multilinear_evaluate(whir_ctx* ctx, int field, const uint64_t* coeffs, size_t n, const uint64_t* point,
                              size_t nvars, uint64_t* out, uint32_t flags) {
  return guarded([&] {
    check_ctx(ctx);
    if (nvars > 62 || (nvars < 62 && n > (1ull << nvars))) throw Error(WHIR_ERR_INVALID, "more values than 2^nvars");
    return with_embedding(field, [&]<class S, class T>() {
      T r = T::zero();
      if (n) {
        std::vector<T> pt = load_host<T>(point, nvars);
        DBuf<S> hc;
        const S* dc = device_vectors<S>(ctx, coeffs, n, flags, hc, false);
        const int h = (int)nvars / 2, l = (int)nvars - h;
        DBuf<T> dp(ctx, std::max<size_t>(nvars, 1)), tables(ctx, (1ull << h) + (1ull << l));
        h2d(ctx, dp.p, pt.data(), nvars * sizeof(T));
        CU(launch_eq_table<T>(dp.p, 0, h, T::one(), tables.p, ctx->stream));
        CU(launch_eq_table<T>(dp.p, h, l, T::one(), tables.p + (1ull << h), ctx->stream));
        DBuf<T> parts(ctx, 152 * 8 + 1), res(ctx, 1);
        size_t np = 0;
        CU((launch_mle_dot<T, S>(dc, n, tables.p, (int)nvars, parts.p, &np, ctx->stream)));
        CU(launch_reduce_singles<T>(parts.p, np, res.p, ctx->stream));
        d2h(ctx, &r, res.p, sizeof(T));
      }
      store_one<T>(r, out);
      return 0;
    });
  });
}

int whir_pow_grind(whir_ctx* ctx, const uint8_t engine_id[32], const uint8_t challenge[32], uint64_t threshold,
                   uint64_t* nonce) {
  return guarded([&] {
    check_ctx(ctx);
    int kind = hash_kind_or_throw(engine_id);
    *nonce = grind(ctx, kind, challenge, threshold);
    return 0;
  });
}

}  // extern "C"
