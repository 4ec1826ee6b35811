// ORACLE — test infrastructure only. Fiat–Shamir transcript used by the oracle prover/verifier.
//
// The reference wraps spongefish 1.0.0-rc1 @ fcc277f8 (src/transcript/mod.rs:50-300); its sponge
// (`StdHash`) and codecs are a git dependency that is not available here, so transcript bytes are
// NOT pinned against the reference. This file defines the transcript the GPU library implements
// too, with the same interaction structure as the reference:
//   * DomainSeparator: protocol_id = SHA3-512(config bytes), session_id = SHA3-256(CBOR text
//     string of the session), absorbed in that order (mod.rs:110-137).
//   * Duplex sponge over Keccak-f[1600], rate 136 bytes: absorb XORs bytes into the rate; the first
//     squeeze after absorbing pads (0x01 at the position, 0x80 at the last rate byte) and permutes.
//   * prover_message: canonical little-endian bytes (ceil(bits/8) per base coefficient, extension
//     coefficients in increasing degree; digests 32 bytes; u64 nonces 8 bytes LE) appended to the
//     NARG string and absorbed.
//   * verifier_message<F>: per base coefficient, squeeze ceil(bits/8)+16 bytes, read little-endian,
//     reduce mod p. verifier_message<[u8;N]>: squeeze N bytes.
//   * hints (Merkle siblings, ark-compressed row matrices) go to a separate hint buffer, not absorbed
//     (mod.rs:213-233). Row matrices are serialized like ark-serialize's compressed Vec<F>: u64 LE
//     length, then each element's canonical bytes.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "hashes.hpp"

namespace oracle {

struct DuplexSponge {
  uint64_t st[25];
  size_t pos = 0;
  bool squeezing = false;
  static constexpr size_t RATE = 136;
  DuplexSponge() {
    for (int i = 0; i < 25; ++i) st[i] = 0;
  }
  uint8_t* bytes() { return (uint8_t*)st; }
  void absorb(const uint8_t* in, size_t n) {
    if (squeezing) {
      squeezing = false;
      pos = 0;
    }
    for (size_t i = 0; i < n; ++i) {
      if (pos == RATE) {
        keccak_f1600(st);
        pos = 0;
      }
      bytes()[pos++] ^= in[i];
    }
  }
  void squeeze(uint8_t* out, size_t n) {
    if (!squeezing) {
      if (pos == RATE) {
        keccak_f1600(st);
        pos = 0;
      }
      bytes()[pos] ^= 0x01;
      bytes()[RATE - 1] ^= 0x80;
      keccak_f1600(st);
      pos = 0;
      squeezing = true;
    }
    for (size_t i = 0; i < n; ++i) {
      if (pos == RATE) {
        keccak_f1600(st);
        pos = 0;
      }
      out[i] = bytes()[pos++];
    }
  }
};

// CBOR encoding of a text string (major type 3), as ciborium writes a Rust &str / String.
inline std::vector<uint8_t> cbor_text(const std::string& s) {
  std::vector<uint8_t> out;
  size_t n = s.size();
  if (n < 24) {
    out.push_back((uint8_t)(0x60 | n));
  } else if (n < 256) {
    out.push_back(0x78);
    out.push_back((uint8_t)n);
  } else if (n < 65536) {
    out.push_back(0x79);
    out.push_back((uint8_t)(n >> 8));
    out.push_back((uint8_t)n);
  } else {
    out.push_back(0x7a);
    for (int i = 3; i >= 0; --i) out.push_back((uint8_t)(n >> (8 * i)));
  }
  out.insert(out.end(), s.begin(), s.end());
  return out;
}

struct DomainSeparator {
  uint8_t protocol_id[64];
  uint8_t session_id[32];
  static DomainSeparator make(const std::vector<uint8_t>& config_bytes, const std::string& session) {
    DomainSeparator d;
    sha3_512(config_bytes.data(), config_bytes.size(), d.protocol_id);
    std::vector<uint8_t> c = cbor_text(session);
    sha3_256(c.data(), c.size(), d.session_id);
    return d;
  }
};

struct ProverState {
  DuplexSponge sponge;
  std::vector<uint8_t> narg;
  std::vector<uint8_t> hints;
  explicit ProverState(const DomainSeparator& ds) {
    sponge.absorb(ds.protocol_id, 64);
    sponge.absorb(ds.session_id, 32);
  }
  void prover_bytes(const uint8_t* b, size_t n) {
    narg.insert(narg.end(), b, b + n);
    sponge.absorb(b, n);
  }
  void verifier_bytes(uint8_t* out, size_t n) { sponge.squeeze(out, n); }
  void hint_bytes(const uint8_t* b, size_t n) { hints.insert(hints.end(), b, b + n); }
};

struct VerificationError : std::runtime_error {
  VerificationError() : std::runtime_error("verification failed") {}
};

struct VerifierState {
  DuplexSponge sponge;
  const uint8_t* narg;
  size_t narg_len, narg_pos = 0;
  const uint8_t* hints;
  size_t hints_len, hints_pos = 0;
  VerifierState(const DomainSeparator& ds, const uint8_t* n, size_t nl, const uint8_t* h, size_t hl)
      : narg(n), narg_len(nl), hints(h), hints_len(hl) {
    sponge.absorb(ds.protocol_id, 64);
    sponge.absorb(ds.session_id, 32);
  }
  void prover_bytes(uint8_t* out, size_t n) {
    if (narg_len - narg_pos < n) throw VerificationError();
    for (size_t i = 0; i < n; ++i) out[i] = narg[narg_pos + i];
    narg_pos += n;
    sponge.absorb(out, n);
  }
  void verifier_bytes(uint8_t* out, size_t n) { sponge.squeeze(out, n); }
  void hint_bytes(uint8_t* out, size_t n) {
    if (hints_len - hints_pos < n) throw VerificationError();
    for (size_t i = 0; i < n; ++i) out[i] = hints[hints_pos + i];
    hints_pos += n;
  }
  bool eof() const { return narg_pos == narg_len && hints_pos == hints_len; }
};

}  // namespace oracle
