// Commitment-side kernels: encode instantiations for the Goldilocks family (the encode kernels
// themselves, with the leaf hash fused into the kernel that writes each codeword row, are in
// encode.cuh), Merkle layers, generic hash_many, proof-of-work search and opening gathers.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

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

// Process-wide tuned choices (whir_autotune): encode plans by shape, Merkle tiles by tree height.
static std::mutex g_tune_mu;
static std::map<std::array<size_t, 4>, EncodeTuning> g_enc_tune;
static std::map<int, int> g_mk_tune;
extern int merkle_tile_log;

void encode_tuning_set(size_t n_msgs, size_t msg_len, size_t codeword_len, size_t eb, const EncodeTuning& t) {
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_enc_tune[{n_msgs, msg_len, codeword_len, eb}] = t;
}
bool encode_tuning_get(size_t n_msgs, size_t msg_len, size_t codeword_len, size_t eb, EncodeTuning* t) {
  std::lock_guard<std::mutex> g(g_tune_mu);
  auto it = g_enc_tune.find({n_msgs, msg_len, codeword_len, eb});
  if (it == g_enc_tune.end()) return false;
  *t = it->second;
  return true;
}
void merkle_tuning_set(int layers, int tile_log) {
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_mk_tune[layers] = tile_log;
}
int merkle_tile_log_for(int layers) {
  std::lock_guard<std::mutex> g(g_tune_mu);
  auto it = g_mk_tune.find(layers);
  return it == g_mk_tune.end() ? merkle_tile_log : it->second;
}
std::string tuning_export() {
  std::lock_guard<std::mutex> g(g_tune_mu);
  std::string s;
  char line[160];
  for (auto& kv : g_enc_tune) {
    snprintf(line, sizeof(line), "encode %zu %zu %zu %zu %d %d %d %d\n", kv.first[0], kv.first[1], kv.first[2],
             kv.first[3], kv.second.mode, kv.second.logC2, kv.second.W, kv.second.G);
    s += line;
  }
  for (auto& kv : g_mk_tune) {
    snprintf(line, sizeof(line), "merkle %d %d\n", kv.first, kv.second);
    s += line;
  }
  return s;
}
int tuning_import(const char* text) {
  std::vector<std::pair<std::array<size_t, 4>, EncodeTuning>> enc;
  std::vector<std::pair<int, int>> mk;
  const char* p = text;
  while (p && *p) {
    const char* e = strchr(p, '\n');
    std::string line(p, e ? (size_t)(e - p) : strlen(p));
    p = e ? e + 1 : nullptr;
    if (line.empty()) continue;
    size_t a, b, cw, eb;
    EncodeTuning t;
    int layers, tl;
    if (sscanf(line.c_str(), "encode %zu %zu %zu %zu %d %d %d %d", &a, &b, &cw, &eb, &t.mode, &t.logC2, &t.W, &t.G) ==
        8) {
      EncodePlan plan;
      if (plan_encode_tuned(a, b, cw, eb, t, &plan)) return WHIR_ERR_INVALID;
      enc.push_back({{a, b, cw, eb}, t});
    } else if (sscanf(line.c_str(), "merkle %d %d", &layers, &tl) == 2) {
      if (layers < 0 || tl < 1 || tl > 10) return WHIR_ERR_INVALID;
      mk.push_back({layers, tl});
    } else {
      return WHIR_ERR_INVALID;
    }
  }
  std::lock_guard<std::mutex> g(g_tune_mu);
  for (auto& x : enc) g_enc_tune[x.first] = x.second;
  for (auto& x : mk) g_mk_tune[x.first] = x.second;
  return 0;
}
void tuning_clear() {
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_enc_tune.clear();
  g_mk_tune.clear();
}

// A plan with explicit choices: mode 0 (whole cosets in one CTA, G cosets per CTA) or mode 1 (four
// step with a row-pass NTT of 2^logC2 points and W columns per column-pass CTA). Fails when the
// choice does not fit the kernels' limits.
int plan_encode_tuned(size_t n_msgs, size_t msg_len, size_t codeword_len, size_t eb, const EncodeTuning& t,
                      EncodePlan* p) {
  if (n_msgs == 0 || codeword_len == 0) return WHIR_ERR_INVALID;
  if (!is_pow2(codeword_len) || codeword_len > (1ull << 32)) return WHIR_ERR_UNSUPPORTED;
  size_t C = 1;
  while (C < msg_len) C <<= 1;
  if (C > codeword_len) return WHIR_ERR_INVALID;
  const size_t K = codeword_len / C;
  EncodePlan q{};
  q.logC = ilog2(C);
  q.logN = ilog2(codeword_len);
  if (t.mode == 0) {
    const size_t G = (size_t)t.G;
    if (!is_pow2(G) || G > K || n_msgs * C * eb * G > ENC_SMEM_BUDGET || q.logC > ENC_MAX_LOGN_SMEM)
      return WHIR_ERR_INVALID;
    q.mode = 0;
    q.cosets_per_cta = (int)G;
  } else if (t.mode == 1) {
    if (t.logC2 < 1 || t.logC2 >= q.logC || t.logC2 > ENC_MAX_LOGN_SMEM) return WHIR_ERR_INVALID;
    const size_t C2 = (size_t)1 << t.logC2, C1 = C / C2, W = (size_t)t.W;
    if (n_msgs * C2 * eb > ENC_SMEM_BUDGET || ilog2(C1) > ENC_MAX_LOGN_SMEM) return WHIR_ERR_INVALID;
    if (!is_pow2(W) || W > C2 || W > 256 || C1 * W * eb > ENC_SMEM_BUDGET) return WHIR_ERR_INVALID;
    q.mode = 1;
    q.logC1 = ilog2(C1);
    q.logC2 = t.logC2;
    q.cosets_per_cta = 1;
    q.cols_per_cta = (int)W;
    q.scratch_elems = n_msgs * K * C;
  } else {
    return WHIR_ERR_INVALID;
  }
  *p = q;
  return 0;
}

int plan_encode(size_t n_msgs, size_t msg_len, size_t codeword_len, size_t eb, EncodePlan* p) {
  EncodeTuning t;
  if (encode_tuning_get(n_msgs, msg_len, codeword_len, eb, &t) &&
      plan_encode_tuned(n_msgs, msg_len, codeword_len, eb, t, p) == 0)
    return 0;
  return plan_encode_default(n_msgs, msg_len, codeword_len, eb, p);
}

int plan_encode_default(size_t n_msgs, size_t msg_len, size_t codeword_len, size_t eb, EncodePlan* p) {
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
// Merkle layers (merkle_tree.rs:82-127): each CTA hashes a tile of 2^nlev consecutive nodes of one
// layer up nlev layers, writing every produced node to its slot. Two phases:
//   A. each thread reads 2^S consecutive nodes (S = nlev - 8 when the tile is wider than the CTA)
//      and hashes them up S layers in registers, with no barrier and every lane busy;
//   B. the CTA's (at most 256) phase-A results are hashed up the remaining layers in shared memory,
//      halving the active threads per layer.
// With 1024-node tiles three quarters of a tile's compressions run in phase A.
// ---------------------------------------------------------------------------------------------
static constexpr int MK_THREADS = 256;
static constexpr int MK_MAX_S = 2;                   // phase-A layers per thread
static constexpr int MK_MAX_TILE_LOG = 8 + MK_MAX_S;  // 1024 input digests per CTA
int merkle_tile_log = MK_MAX_TILE_LOG;                // tile height of a launch (1..MK_MAX_TILE_LOG)

template <int KIND>
__device__ __forceinline__ void hash_pair(const uint32_t* l, const uint32_t* r, uint32_t* out) {
  uint32_t m[16];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    m[q] = l[q];
    m[8 + q] = r[q];
  }
  hash64<KIND>(m, out);
}

template <int KIND, int S>
__device__ __forceinline__ void merkle_tile_body(uint32_t* nodes, int layers, int in_level, int nlev, uint64_t bid) {
  __shared__ uint4 buf[MK_THREADS * 2];  // phase-B digests
  // offset of level l: 2^(L+1) - 2^(L-l+1)
  auto level_off = [&](int l) -> uint64_t { return (2ull << layers) - (2ull << (layers - l)); };
  const uint64_t first = bid << nlev;  // first input node of the tile (in its level)
  const int width = 1 << (nlev - S);   // phase-A threads = phase-B inputs
  const int t = threadIdx.x;
  if (t < width) {
    uint32_t d[1 << S][8];
    const uint4* src = reinterpret_cast<const uint4*>(nodes + (level_off(in_level) + first + ((uint64_t)t << S)) * 8);
#pragma unroll
    for (int k = 0; k < (1 << S); ++k) {
      const uint4 a = src[2 * k], b = src[2 * k + 1];
      d[k][0] = a.x; d[k][1] = a.y; d[k][2] = a.z; d[k][3] = a.w;
      d[k][4] = b.x; d[k][5] = b.y; d[k][6] = b.z; d[k][7] = b.w;
    }
#pragma unroll
    for (int l = 1; l <= S; ++l) {
      const uint64_t off = level_off(in_level + l) + ((first >> l) + ((uint64_t)t << (S - l)));
#pragma unroll
      for (int k = 0; k < (1 << (S - l)); ++k) {
        uint32_t h[8];
        hash_pair<KIND>(d[2 * k], d[2 * k + 1], h);
        uint4* dst = reinterpret_cast<uint4*>(nodes + (off + k) * 8);
        dst[0] = make_uint4(h[0], h[1], h[2], h[3]);
        dst[1] = make_uint4(h[4], h[5], h[6], h[7]);
#pragma unroll
        for (int q = 0; q < 8; ++q) d[k][q] = h[q];
      }
    }
    buf[2 * t] = make_uint4(d[0][0], d[0][1], d[0][2], d[0][3]);
    buf[2 * t + 1] = make_uint4(d[0][4], d[0][5], d[0][6], d[0][7]);
  }
  __syncthreads();
  int cnt = width;
  for (int l = S + 1; l <= nlev; ++l) {
    cnt >>= 1;
    const uint64_t out_off = level_off(in_level + l) + (first >> l);
    const bool active = t < cnt;
    uint4 r0, r1;
    if (active) {
      uint32_t m[16], h[8];
      const uint4* p = buf + t * 4;
      const uint4 q0 = p[0], q1 = p[1], q2 = p[2], q3 = p[3];
      m[0] = q0.x; m[1] = q0.y; m[2] = q0.z; m[3] = q0.w;
      m[4] = q1.x; m[5] = q1.y; m[6] = q1.z; m[7] = q1.w;
      m[8] = q2.x; m[9] = q2.y; m[10] = q2.z; m[11] = q2.w;
      m[12] = q3.x; m[13] = q3.y; m[14] = q3.z; m[15] = q3.w;
      hash64<KIND>(m, h);
      r0 = make_uint4(h[0], h[1], h[2], h[3]);
      r1 = make_uint4(h[4], h[5], h[6], h[7]);
      uint4* dst = reinterpret_cast<uint4*>(nodes + (out_off + t) * 8);
      dst[0] = r0;
      dst[1] = r1;
    }
    __syncthreads();
    if (active) {
      buf[2 * t] = r0;
      buf[2 * t + 1] = r1;
    }
    __syncthreads();
  }
}

// Copies a result that this CTA has written to global memory into a mail slot and publishes it
// (call after a CTA barrier, from one thread).
__device__ __forceinline__ void mail_publish(const MailSlot& mail, const uint32_t* src, int words) {
  for (int i = 0; i < words; ++i) reinterpret_cast<volatile uint32_t*>(mail.data)[i] = src[i];
  reinterpret_cast<volatile unsigned int*>(mail.flag)[1] = *reinterpret_cast<const volatile unsigned int*>(mail.dev_err);
  __threadfence_system();
  *reinterpret_cast<volatile unsigned int*>(mail.flag) = mail.seq;
}

template <int KIND, int S>
__global__ void __launch_bounds__(MK_THREADS) merkle_tile_kernel(uint32_t* nodes, int layers, int in_level,
                                                                 int nlev, MailSlot mail) {
  merkle_tile_body<KIND, S>(nodes, layers, in_level, nlev, blockIdx.x);
  if (mail.data == nullptr) return;
  // the single CTA of the top tile: the root is the tree's last node
  __syncthreads();
  if (threadIdx.x == 0) mail_publish(mail, nodes + ((2ull << layers) - 2) * 8, 8);
}

// Several trees in one launch per tile step: tree j's tiles are CTAs [cta_begin_j, cta_begin_j+1).
struct MerkleStep {
  uint32_t* nodes;
  int layers, in_level, nlev, pad;
  uint64_t cta_begin;
};
template <int KIND, int S>
__global__ void __launch_bounds__(MK_THREADS) merkle_tile_multi_kernel(const MerkleStep* steps, int n) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (steps[mid].cta_begin <= blockIdx.x)
      lo = mid;
    else
      hi = mid - 1;
  }
  const MerkleStep st = steps[lo];
  merkle_tile_body<KIND, S>(st.nodes, st.layers, st.in_level, st.nlev, blockIdx.x - st.cta_begin);
}

// Steps: at step t every unfinished tree hashes its next min(tile height, remaining) layers. A
// step's trees are launched together per phase-A depth S (the kernel's template argument); every
// launch reads its own slice of the uploaded table.
void merkle_multi_plan(const MerkleJobDesc* jobs, size_t njobs, int tile_log, std::vector<MerkleMultiLaunch>& launches,
                       std::vector<uint8_t>& image) {
  launches.clear();
  std::vector<MerkleStep> tab;
  std::vector<int> level(njobs, 0), tl(njobs);
  for (size_t j = 0; j < njobs; ++j)
    tl[j] = std::max(1, std::min(tile_log > 0 ? tile_log : merkle_tile_log_for(jobs[j].layers), MK_MAX_TILE_LOG));
  for (;;) {
    bool any = false;
    for (int S = 0; S <= MK_MAX_S; ++S) {
      const size_t base = tab.size();
      uint64_t grid = 0;
      for (size_t j = 0; j < njobs; ++j) {
        if (level[j] >= jobs[j].layers) continue;
        const int nlev = std::min(tl[j], jobs[j].layers - level[j]);
        if (std::max(0, nlev - 8) != S) continue;
        tab.push_back(MerkleStep{jobs[j].nodes, jobs[j].layers, level[j], nlev, 0, grid});
        grid += (1ull << (jobs[j].layers - level[j])) >> nlev;
      }
      if (tab.size() == base) continue;
      any = true;
      launches.push_back(MerkleMultiLaunch{base * sizeof(MerkleStep), (int)(tab.size() - base), S, grid});
    }
    if (!any) break;
    for (size_t j = 0; j < njobs; ++j)
      if (level[j] < jobs[j].layers) level[j] += std::min(tl[j], jobs[j].layers - level[j]);
  }
  image.assign(reinterpret_cast<const uint8_t*>(tab.data()),
               reinterpret_cast<const uint8_t*>(tab.data()) + tab.size() * sizeof(MerkleStep));
}

template <int KIND>
static cudaError_t merkle_multi_run(const std::vector<MerkleMultiLaunch>& launches, const void* dev_image,
                                    cudaStream_t s) {
  for (const MerkleMultiLaunch& l : launches) {
    const MerkleStep* t = reinterpret_cast<const MerkleStep*>(static_cast<const uint8_t*>(dev_image) + l.offset);
    if (l.grid == 0 || l.grid > 0x7fffffffull) return cudaErrorInvalidValue;
    switch (l.S) {
      case 0: merkle_tile_multi_kernel<KIND, 0><<<(unsigned)l.grid, MK_THREADS, 0, s>>>(t, l.n); break;
      case 1: merkle_tile_multi_kernel<KIND, 1><<<(unsigned)l.grid, MK_THREADS, 0, s>>>(t, l.n); break;
      default: merkle_tile_multi_kernel<KIND, 2><<<(unsigned)l.grid, MK_THREADS, 0, s>>>(t, l.n); break;
    }
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_merkle_multi(const std::vector<MerkleMultiLaunch>& launches, const void* dev_image, int hash_kind,
                                cudaStream_t s) {
  switch (hash_kind) {
    case HASH_BLAKE3: return merkle_multi_run<HASH_BLAKE3>(launches, dev_image, s);
    case HASH_SHA2: return merkle_multi_run<HASH_SHA2>(launches, dev_image, s);
    case HASH_SHA3: return merkle_multi_run<HASH_SHA3>(launches, dev_image, s);
    case HASH_KECCAK: return merkle_multi_run<HASH_KECCAK>(launches, dev_image, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int KIND>
static cudaError_t merkle_run(uint32_t* nodes, int layers, cudaStream_t s, int tile_log, const MailSlot& mail) {
  tile_log = std::max(1, std::min(tile_log, MK_MAX_TILE_LOG));
  if (mail.data && layers < 1) return cudaErrorInvalidValue;
  int level = 0;
  while (level < layers) {
    const int nlev = std::min(tile_log, layers - level);
    const int S = std::max(0, nlev - 8);
    const unsigned grid = (unsigned)((1ull << (layers - level)) >> nlev);
    const MailSlot m = level + nlev == layers ? mail : MailSlot();  // the last launch is one CTA
    switch (S) {
      case 0: merkle_tile_kernel<KIND, 0><<<grid, MK_THREADS, 0, s>>>(nodes, layers, level, nlev, m); break;
      case 1: merkle_tile_kernel<KIND, 1><<<grid, MK_THREADS, 0, s>>>(nodes, layers, level, nlev, m); break;
      default: merkle_tile_kernel<KIND, 2><<<grid, MK_THREADS, 0, s>>>(nodes, layers, level, nlev, m); break;
    }
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    level += nlev;
  }
  return cudaSuccess;
}

cudaError_t launch_merkle(uint32_t* nodes, int layers, int kind, cudaStream_t s, int tile_log, const MailSlot& mail) {
  if (tile_log <= 0) tile_log = merkle_tile_log_for(layers);
  switch (kind) {
    case HASH_BLAKE3: return merkle_run<HASH_BLAKE3>(nodes, layers, s, tile_log, mail);
    case HASH_SHA2: return merkle_run<HASH_SHA2>(nodes, layers, s, tile_log, mail);
    case HASH_SHA3: return merkle_run<HASH_SHA3>(nodes, layers, s, tile_log, mail);
    case HASH_KECCAK: return merkle_run<HASH_KECCAK>(nodes, layers, s, tile_log, mail);
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
  unsigned long long* best;  // best[0]: lowest hit so far; best[1]: finished CTAs
  MailSlot mail;
};

static constexpr int POW_THREADS = 256;

// Thread t of the grid (T threads) tries nonces start + t, start + t + T, start + t + 2T, ... and
// stops at the first one at or above the best nonce known so far; a satisfying nonce lowers the best
// with atomicMin. Every nonce below the final best is tried by its thread, so the result is the
// lowest satisfying nonce of the range. The grid is one wave of resident CTAs, so the threads advance
// together and, once a hit is known, each does at most the hash in progress (no block claims, no
// barriers). The best nonce is re-read before every hash and the read of one iteration is used by the
// next, so its latency hides behind a hash.
template <int KIND>
__global__ void __launch_bounds__(POW_THREADS) pow_kernel(PowArgs a) {
  const uint64_t T = (uint64_t)gridDim.x * blockDim.x;
  unsigned long long known = *reinterpret_cast<volatile unsigned long long*>(a.best);
#pragma unroll 1
  for (uint64_t off = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; off < a.count; off += T) {
    const uint64_t nonce = a.start + off;
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
  if (a.mail.data == nullptr) return;
  // The last CTA to finish publishes the result (every CTA's atomicMin precedes its arrival).
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(a.best + 1, 1ull) == gridDim.x - 1) {
      const unsigned long long b = *reinterpret_cast<volatile unsigned long long*>(a.best);
      *reinterpret_cast<volatile unsigned long long*>(a.mail.data) = b;
      reinterpret_cast<volatile unsigned int*>(a.mail.flag)[1] =
          *reinterpret_cast<const volatile unsigned int*>(a.mail.dev_err);
      __threadfence_system();
      *reinterpret_cast<volatile unsigned int*>(a.mail.flag) = a.mail.seq;
    }
  }
}

cudaError_t launch_pow(const uint32_t challenge[8], uint64_t threshold, uint64_t start, uint64_t count,
                       unsigned long long* best, int kind, cudaStream_t s, const MailSlot& mail) {
  PowArgs a;
  for (int i = 0; i < 8; ++i) a.chal[i] = challenge[i];
  blake3_pow_prefix(a.chal, a.pre);
  a.threshold = threshold;
  a.start = start;
  a.count = count;
  a.best = best;
  a.mail = mail;
  // The grid is exactly the CTAs that fit on the GPU at once (by the kernel's registers), so every
  // thread starts at once; a larger grid would hold CTAs back until the first ones exit.
  auto resident = [&](auto kernel) -> unsigned {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
        cudaSuccess || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, POW_THREADS, 0) != cudaSuccess ||
        per_sm < 1 || sms < 1)
      return 152;
    return (unsigned)(sms * per_sm);
  };
  const uint64_t want = (count + POW_THREADS - 1) / POW_THREADS;
  switch (kind) {
    case HASH_BLAKE3: {
      static const unsigned r = resident(pow_kernel<HASH_BLAKE3>);
      pow_kernel<HASH_BLAKE3><<<(unsigned)std::min<uint64_t>(want, r), POW_THREADS, 0, s>>>(a);
      break;
    }
    case HASH_SHA2: {
      static const unsigned r = resident(pow_kernel<HASH_SHA2>);
      pow_kernel<HASH_SHA2><<<(unsigned)std::min<uint64_t>(want, r), POW_THREADS, 0, s>>>(a);
      break;
    }
    case HASH_SHA3: {
      static const unsigned r = resident(pow_kernel<HASH_SHA3>);
      pow_kernel<HASH_SHA3><<<(unsigned)std::min<uint64_t>(want, r), POW_THREADS, 0, s>>>(a);
      break;
    }
    case HASH_KECCAK: {
      static const unsigned r = resident(pow_kernel<HASH_KECCAK>);
      pow_kernel<HASH_KECCAK><<<(unsigned)std::min<uint64_t>(want, r), POW_THREADS, 0, s>>>(a);
      break;
    }
    default: return cudaErrorInvalidValue;
  }
  note_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------

__global__ void gather_paths_kernel(const uint32_t* nodes, const uint64_t* idx, uint64_t q, int layers, uint32_t* out) {
  const uint64_t total = q * (uint64_t)layers * 8;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t w = t & 7, jl = t >> 3, j = jl / (uint64_t)layers, l = jl - j * (uint64_t)layers;
    const uint64_t off = (2ull << layers) - (2ull << (layers - l));
    out[t] = nodes[(off + ((idx[j] >> l) ^ 1)) * 8 + w];
  }
}
cudaError_t launch_gather_paths(const uint32_t* nodes, const uint64_t* idx, size_t q, int layers, uint32_t* out,
                                cudaStream_t s) {
  if (q == 0 || layers <= 0) return cudaSuccess;
  const size_t total = q * (size_t)layers * 8;
  gather_paths_kernel<<<(unsigned)std::min<size_t>((total + 255) / 256, 4096), 256, 0, s>>>(nodes, idx, q, layers, out);
  note_launch();
  return cudaGetLastError();
}

}  // namespace whir
