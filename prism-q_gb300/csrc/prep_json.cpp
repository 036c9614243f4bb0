// PRISM-PREP topology JSON ingest: PrismPrepTopology
// (crates/prism-nhs/src/input.rs:1027-1140) into a prismq_topology.
//
// The steps follow the reference's load path for a production MD run:
//   1. parse (PrismPrepTopology::load, input.rs:1972, serde_json): the
//      required keys, integer-only index fields, deny_unknown_fields on the
//      harmonic contract;
//   2. validate (input.rs:1996-2290): array lengths, finite / positive values,
//      index ranges, distinct term atoms, symmetric duplicate-free strict
//      exclusions, canonical (i < j) unique exceptions that are exactly
//      representable in float32 and disjoint from the strict exclusions, the
//      harmonic contract (schema, units, counts, canonical SHA-256, :300-321)
//      and the exact-exception contract (schema, semantics, counts, the two
//      pair digests :1935-1969, the prmtop provenance hash);
//   3. nonbonded execution policy RequireExactV2 (:1429-1450);
//   4. harmonic lowering to U = k (x - x0)^2 (:467-520): k x (source
//      prefactor / 1.0) in binary64, then cast to float32;
//   5. hydrogen mass repartitioning (:2482-2560), binary64 on the inverse
//      masses, skipped only when the file records hmr_applied = true.
// Strict exclusions are kept as given; the engine removes exception pairs from
// the ordinary pair list itself (fused_engine.rs:11680-11700).
//
// Two pieces are restated from published specifications: SHA-256 (FIPS
// 180-4) and the canonical JSON that the reference hashes, which is Python's
// json.dumps(sort_keys=True, separators=(",", ":"), ensure_ascii=True)
// (input.rs:44-137).
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <set>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "pq_host.h"

namespace {

// --------------------------------------------------------------------------
// SHA-256 (FIPS 180-4).
// --------------------------------------------------------------------------
class Sha256 {
 public:
  Sha256() {
    static const uint32_t kInit[8] = {0x6a09e667u, 0xbb67ae85u, 0x3c6ef372u, 0xa54ff53au,
                                      0x510e527fu, 0x9b05688cu, 0x1f83d9abu, 0x5be0cd19u};
    std::memcpy(h_, kInit, sizeof(h_));
  }
  void update(const void* data, size_t n) {
    const uint8_t* p = static_cast<const uint8_t*>(data);
    total_ += n;
    while (n > 0) {
      const size_t take = std::min(n, (size_t)64 - fill_);
      std::memcpy(buf_ + fill_, p, take);
      fill_ += take;
      p += take;
      n -= take;
      if (fill_ == 64) {
        block(buf_);
        fill_ = 0;
      }
    }
  }
  void update_u64le(uint64_t v) {
    uint8_t b[8];
    for (int k = 0; k < 8; ++k) b[k] = (uint8_t)(v >> (8 * k));
    update(b, 8);
  }
  void update_f64le(double d) {
    uint64_t v;
    std::memcpy(&v, &d, 8);
    update_u64le(v);
  }
  std::string hex() {
    const uint64_t bits = total_ * 8;
    const uint8_t one = 0x80, zero = 0x00;
    update(&one, 1);
    while (fill_ != 56) update(&zero, 1);
    uint8_t len[8];
    for (int k = 0; k < 8; ++k) len[k] = (uint8_t)(bits >> (56 - 8 * k));
    update(len, 8);
    static const char* kHex = "0123456789abcdef";
    std::string out;
    for (uint32_t w : h_)
      for (int k = 28; k >= 0; k -= 4) out += kHex[(w >> k) & 0xF];
    return out;
  }

 private:
  static uint32_t rotr(uint32_t x, int r) { return (x >> r) | (x << (32 - r)); }
  void block(const uint8_t* b) {
    static const uint32_t K[64] = {
        0x428a2f98u, 0x71374491u, 0xb5c0fbcfu, 0xe9b5dba5u, 0x3956c25bu, 0x59f111f1u, 0x923f82a4u, 0xab1c5ed5u,
        0xd807aa98u, 0x12835b01u, 0x243185beu, 0x550c7dc3u, 0x72be5d74u, 0x80deb1feu, 0x9bdc06a7u, 0xc19bf174u,
        0xe49b69c1u, 0xefbe4786u, 0x0fc19dc6u, 0x240ca1ccu, 0x2de92c6fu, 0x4a7484aau, 0x5cb0a9dcu, 0x76f988dau,
        0x983e5152u, 0xa831c66du, 0xb00327c8u, 0xbf597fc7u, 0xc6e00bf3u, 0xd5a79147u, 0x06ca6351u, 0x14292967u,
        0x27b70a85u, 0x2e1b2138u, 0x4d2c6dfcu, 0x53380d13u, 0x650a7354u, 0x766a0abbu, 0x81c2c92eu, 0x92722c85u,
        0xa2bfe8a1u, 0xa81a664bu, 0xc24b8b70u, 0xc76c51a3u, 0xd192e819u, 0xd6990624u, 0xf40e3585u, 0x106aa070u,
        0x19a4c116u, 0x1e376c08u, 0x2748774cu, 0x34b0bcb5u, 0x391c0cb3u, 0x4ed8aa4au, 0x5b9cca4fu, 0x682e6ff3u,
        0x748f82eeu, 0x78a5636fu, 0x84c87814u, 0x8cc70208u, 0x90befffau, 0xa4506cebu, 0xbef9a3f7u, 0xc67178f2u};
    uint32_t w[64];
    for (int t = 0; t < 16; ++t)
      w[t] = (uint32_t)b[4 * t] << 24 | (uint32_t)b[4 * t + 1] << 16 | (uint32_t)b[4 * t + 2] << 8 | b[4 * t + 3];
    for (int t = 16; t < 64; ++t) {
      const uint32_t s0 = rotr(w[t - 15], 7) ^ rotr(w[t - 15], 18) ^ (w[t - 15] >> 3);
      const uint32_t s1 = rotr(w[t - 2], 17) ^ rotr(w[t - 2], 19) ^ (w[t - 2] >> 10);
      w[t] = w[t - 16] + s0 + w[t - 7] + s1;
    }
    uint32_t a = h_[0], bb = h_[1], c = h_[2], d = h_[3], e = h_[4], f = h_[5], g = h_[6], hh = h_[7];
    for (int t = 0; t < 64; ++t) {
      const uint32_t S1 = rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25);
      const uint32_t ch = (e & f) ^ (~e & g);
      const uint32_t t1 = hh + S1 + ch + K[t] + w[t];
      const uint32_t S0 = rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22);
      const uint32_t maj = (a & bb) ^ (a & c) ^ (bb & c);
      const uint32_t t2 = S0 + maj;
      hh = g;
      g = f;
      f = e;
      e = d + t1;
      d = c;
      c = bb;
      bb = a;
      a = t1 + t2;
    }
    h_[0] += a; h_[1] += bb; h_[2] += c; h_[3] += d;
    h_[4] += e; h_[5] += f; h_[6] += g; h_[7] += hh;
  }
  uint32_t h_[8];
  uint8_t buf_[64];
  size_t fill_ = 0;
  uint64_t total_ = 0;
};

// --------------------------------------------------------------------------
// JSON DOM and a recursive-descent reader (RFC 8259).
// --------------------------------------------------------------------------
struct JVal {
  enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
  bool b = false;
  bool is_int = false;  // a number written without fraction or exponent that fits int64
  double num = 0.0;
  long long ival = 0;
  std::string str;
  std::vector<JVal> arr;
  std::vector<std::pair<std::string, JVal>> obj;

  const JVal* get(const char* key) const {
    if (kind != Obj) return nullptr;
    for (const auto& kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
};

void put_utf8(unsigned cp, std::string& out) {
  if (cp < 0x80) {
    out += (char)cp;
  } else if (cp < 0x800) {
    out += (char)(0xC0 | (cp >> 6));
    out += (char)(0x80 | (cp & 0x3F));
  } else if (cp < 0x10000) {
    out += (char)(0xE0 | (cp >> 12));
    out += (char)(0x80 | ((cp >> 6) & 0x3F));
    out += (char)(0x80 | (cp & 0x3F));
  } else {
    out += (char)(0xF0 | (cp >> 18));
    out += (char)(0x80 | ((cp >> 12) & 0x3F));
    out += (char)(0x80 | ((cp >> 6) & 0x3F));
    out += (char)(0x80 | (cp & 0x3F));
  }
}

struct Parser {
  const char* p;
  const char* end;
  std::string err;
  int depth = 0;

  void ws() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
  }
  bool fail(const std::string& m) {
    if (err.empty()) err = m;
    return false;
  }
  bool lit(const char* s) {
    const size_t n = std::strlen(s);
    if ((size_t)(end - p) < n || std::memcmp(p, s, n) != 0) return false;
    p += n;
    return true;
  }
  bool hex4(unsigned* cp) {
    if (end - p < 4) return fail("truncated \\u escape");
    unsigned v = 0;
    for (int k = 0; k < 4; ++k) {
      const char c = p[k];
      v <<= 4;
      if (c >= '0' && c <= '9') v |= (unsigned)(c - '0');
      else if (c >= 'a' && c <= 'f') v |= (unsigned)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') v |= (unsigned)(c - 'A' + 10);
      else return fail("bad \\u escape");
    }
    p += 4;
    *cp = v;
    return true;
  }
  bool str(std::string& out) {
    if (p >= end || *p != '"') return fail("expected a string");
    ++p;
    out.clear();
    while (p < end && *p != '"') {
      const unsigned char c = (unsigned char)*p;
      if (c < 0x20) return fail("control character in string");
      if (c != '\\') {
        out += *p++;
        continue;
      }
      if (++p >= end) return fail("truncated escape");
      const char e = *p++;
      switch (e) {
        case '"': out += '"'; break;
        case '\\': out += '\\'; break;
        case '/': out += '/'; break;
        case 'b': out += '\b'; break;
        case 'f': out += '\f'; break;
        case 'n': out += '\n'; break;
        case 'r': out += '\r'; break;
        case 't': out += '\t'; break;
        case 'u': {
          unsigned cp;
          if (!hex4(&cp)) return false;
          if (cp >= 0xD800 && cp < 0xDC00) {  // high surrogate: a low one must follow
            unsigned lo;
            if (end - p < 2 || p[0] != '\\' || p[1] != 'u') return fail("unpaired surrogate");
            p += 2;
            if (!hex4(&lo)) return false;
            if (lo < 0xDC00 || lo >= 0xE000) return fail("unpaired surrogate");
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          } else if (cp >= 0xDC00 && cp < 0xE000) {
            return fail("unpaired surrogate");
          }
          put_utf8(cp, out);
          break;
        }
        default: return fail("bad escape");
      }
    }
    if (p >= end) return fail("unterminated string");
    ++p;
    return true;
  }
  bool number(JVal& v) {
    const char* s = p;
    if (p < end && *p == '-') ++p;
    const char* digits = p;
    while (p < end && *p >= '0' && *p <= '9') ++p;
    if (p == digits) return fail("expected a value");
    if (*digits == '0' && p - digits > 1) return fail("leading zero in number");
    bool integral = true;
    if (p < end && *p == '.') {
      integral = false;
      ++p;
      const char* f = p;
      while (p < end && *p >= '0' && *p <= '9') ++p;
      if (p == f) return fail("bad number");
    }
    if (p < end && (*p == 'e' || *p == 'E')) {
      integral = false;
      ++p;
      if (p < end && (*p == '+' || *p == '-')) ++p;
      const char* x = p;
      while (p < end && *p >= '0' && *p <= '9') ++p;
      if (p == x) return fail("bad exponent");
    }
    const std::string t(s, p);
    v.kind = JVal::Num;
    v.num = std::strtod(t.c_str(), nullptr);  // correctly rounded
    v.is_int = integral;
    if (integral) {
      errno = 0;
      v.ival = std::strtoll(t.c_str(), nullptr, 10);
      if (errno == ERANGE) v.is_int = false;
    }
    return true;
  }
  bool val(JVal& v) {
    if (++depth > 64) return fail("nesting deeper than 64");
    ws();
    if (p >= end) return fail("unexpected end of input");
    bool ok = true;
    if (*p == '{') {
      ++p;
      v.kind = JVal::Obj;
      ws();
      if (p < end && *p == '}') {
        ++p;
      } else {
        for (;;) {
          ws();
          std::string key;
          if (!str(key)) { ok = false; break; }
          ws();
          if (p >= end || *p != ':') { ok = fail("expected ':'"); break; }
          ++p;
          v.obj.emplace_back(std::move(key), JVal());
          if (!val(v.obj.back().second)) { ok = false; break; }
          ws();
          if (p < end && *p == ',') { ++p; continue; }
          if (p < end && *p == '}') { ++p; break; }
          ok = fail("expected ',' or '}'");
          break;
        }
      }
    } else if (*p == '[') {
      ++p;
      v.kind = JVal::Arr;
      ws();
      if (p < end && *p == ']') {
        ++p;
      } else {
        for (;;) {
          v.arr.emplace_back();
          if (!val(v.arr.back())) { ok = false; break; }
          ws();
          if (p < end && *p == ',') { ++p; continue; }
          if (p < end && *p == ']') { ++p; break; }
          ok = fail("expected ',' or ']'");
          break;
        }
      }
    } else if (*p == '"') {
      v.kind = JVal::Str;
      ok = str(v.str);
    } else if (lit("true")) {
      v.kind = JVal::Bool;
      v.b = true;
    } else if (lit("false")) {
      v.kind = JVal::Bool;
    } else if (lit("null")) {
      v.kind = JVal::Null;
    } else {
      ok = number(v);
    }
    --depth;
    return ok;
  }
};

// --------------------------------------------------------------------------
// Canonical JSON: Python json.dumps(sort_keys=True, separators=(",", ":"),
// ensure_ascii=True), for the integer / string / bool objects the reference
// hashes (input.rs:44-137).
// --------------------------------------------------------------------------
struct Err {
  std::string msg;
};

void canon_string(const std::string& s, std::string& out) {
  out += '"';
  for (size_t k = 0; k < s.size();) {
    const unsigned char c = (unsigned char)s[k];
    unsigned cp;
    size_t n;
    if (c < 0x80) { cp = c; n = 1; }
    else if ((c & 0xE0) == 0xC0) { cp = c & 0x1F; n = 2; }
    else if ((c & 0xF0) == 0xE0) { cp = c & 0x0F; n = 3; }
    else { cp = c & 0x07; n = 4; }
    if (k + n > s.size()) throw Err{"invalid UTF-8 in a hashed string"};
    for (size_t q = 1; q < n; ++q) cp = (cp << 6) | ((unsigned char)s[k + q] & 0x3F);
    k += n;
    char esc[16];
    switch (cp) {
      case '"': out += "\\\""; continue;
      case '\\': out += "\\\\"; continue;
      case '\b': out += "\\b"; continue;
      case '\f': out += "\\f"; continue;
      case '\n': out += "\\n"; continue;
      case '\r': out += "\\r"; continue;
      case '\t': out += "\\t"; continue;
      default: break;
    }
    if (cp >= 0x20 && cp < 0x7F) {
      out += (char)cp;
    } else if (cp < 0x10000) {
      std::snprintf(esc, sizeof(esc), "\\u%04x", cp);
      out += esc;
    } else {
      const unsigned v = cp - 0x10000;
      std::snprintf(esc, sizeof(esc), "\\u%04x\\u%04x", 0xD800 + (v >> 10), 0xDC00 + (v & 0x3FF));
      out += esc;
    }
  }
  out += '"';
}

void canon_value(const JVal& v, std::string& out) {
  switch (v.kind) {
    case JVal::Null: out += "null"; break;
    case JVal::Bool: out += v.b ? "true" : "false"; break;
    case JVal::Num:
      if (!v.is_int) throw Err{"hashed contract holds a non-integer number"};
      out += std::to_string(v.ival);
      break;
    case JVal::Str: canon_string(v.str, out); break;
    case JVal::Arr:
      out += '[';
      for (size_t k = 0; k < v.arr.size(); ++k) {
        if (k) out += ',';
        canon_value(v.arr[k], out);
      }
      out += ']';
      break;
    case JVal::Obj: {
      std::vector<const std::pair<std::string, JVal>*> kv;
      for (const auto& e : v.obj) kv.push_back(&e);
      std::sort(kv.begin(), kv.end(), [](const std::pair<std::string, JVal>* a,
                                         const std::pair<std::string, JVal>* b) { return a->first < b->first; });
      out += '{';
      for (size_t k = 0; k < kv.size(); ++k) {
        if (k) out += ',';
        canon_string(kv[k]->first, out);
        out += ':';
        canon_value(kv[k]->second, out);
      }
      out += '}';
      break;
    }
  }
}

// --------------------------------------------------------------------------
// Typed field access with the reference's serde types.
// --------------------------------------------------------------------------
const JVal& need(const JVal& o, const char* key, const std::string& where) {
  const JVal* v = o.get(key);
  if (!v) throw Err{where + ": missing field '" + key + "'"};
  return *v;
}
double f64(const JVal& v, const std::string& what) {
  if (v.kind != JVal::Num) throw Err{what + " must be a number"};
  return v.num;
}
float f32(const JVal& v, const std::string& what) {  // serde f32: the binary64 value cast to float32
  return (float)f64(v, what);
}
uint64_t usize(const JVal& v, const std::string& what) {
  if (v.kind != JVal::Num || !v.is_int || v.ival < 0) throw Err{what + " must be a non-negative integer"};
  return (uint64_t)v.ival;
}
int64_t i32(const JVal& v, const std::string& what) {
  if (v.kind != JVal::Num || !v.is_int || v.ival < INT32_MIN || v.ival > INT32_MAX)
    throw Err{what + " must be a 32-bit integer"};
  return v.ival;
}
bool boolean(const JVal& v, const std::string& what) {
  if (v.kind != JVal::Bool) throw Err{what + " must be true or false"};
  return v.b;
}
const std::string& text(const JVal& v, const std::string& what) {
  if (v.kind != JVal::Str) throw Err{what + " must be a string"};
  return v.str;
}
const std::vector<JVal>& array(const JVal& v, const std::string& what) {
  if (v.kind != JVal::Arr) throw Err{what + " must be an array"};
  return v.arr;
}
std::string at(const char* name, size_t k) { return std::string(name) + "[" + std::to_string(k) + "]"; }

bool is_hex64(const std::string& s) {
  if (s.size() != 64) return false;
  for (char c : s)
    if (!((c >= '0' && c <= '9') || (c >= 'a' && c <= 'f') || (c >= 'A' && c <= 'F'))) return false;
  return true;
}

// Parsed terms in the reference's own types (usize indices, binary64 values).
struct Bond { uint64_t i, j; double r0, k; };
struct Angle { uint64_t i, j, k; double theta0, force_k; };
struct Dih { uint64_t i, j, k, l; int64_t n; double phase, force_k; };
struct Exc { uint64_t i, j; double qq, sig, eps; };
struct Cluster { uint64_t c; std::vector<int64_t> h; std::vector<double> len; uint64_t nh; double inv_c, inv_h; };

double convention_prefactor(const std::string& c) {
  if (c == "OPENMM_FULL_K_HALF_ENERGY") return 0.5;  // input.rs:267
  if (c == "AMBER_NO_HALF_ENERGY") return 1.0;
  throw Err{"unknown harmonic energy convention '" + c + "'"};
}

// HarmonicParameterContract::validate_for_topology (input.rs:300-321), with
// serde(deny_unknown_fields).  Returns {bond prefactor, angle prefactor}.
std::pair<double, double> harmonic_contract(const JVal& c, size_t n_bonds, size_t n_angles) {
  static const char* kFields[] = {"schema_kind", "schema_version", "source_provider", "bond_convention",
                                  "angle_convention", "bond_coefficient_unit", "angle_coefficient_unit",
                                  "bond_equilibrium_unit", "angle_equilibrium_unit",
                                  "bond_uses_periodic_boundary_conditions",
                                  "angle_uses_periodic_boundary_conditions", "bond_count", "angle_count",
                                  "contract_sha256"};
  const std::string w = "harmonic_parameter_contract";
  if (c.kind != JVal::Obj) throw Err{w + " must be an object"};
  for (const auto& kv : c.obj) {
    bool known = false;
    for (const char* f : kFields) known |= kv.first == f;
    if (!known) throw Err{w + ": unknown field '" + kv.first + "'"};
  }
  const double pb = convention_prefactor(text(need(c, "bond_convention", w), w + ".bond_convention"));
  const double pa = convention_prefactor(text(need(c, "angle_convention", w), w + ".angle_convention"));
  const uint64_t version = usize(need(c, "schema_version", w), w + ".schema_version");
  if (version > 0xFFFFFFFFull) throw Err{w + ".schema_version out of range"};
  const bool ok = text(need(c, "schema_kind", w), w) == "prismos_harmonic_parameter_contract" && version == 1 &&
                  text(need(c, "source_provider", w), w).find_first_not_of(" \t\r\n\f\v") != std::string::npos &&
                  text(need(c, "bond_coefficient_unit", w), w) == "kcal/mol/angstrom^2" &&
                  text(need(c, "angle_coefficient_unit", w), w) == "kcal/mol/radian^2" &&
                  text(need(c, "bond_equilibrium_unit", w), w) == "angstrom" &&
                  text(need(c, "angle_equilibrium_unit", w), w) == "radian" &&
                  !boolean(need(c, "bond_uses_periodic_boundary_conditions", w), w) &&
                  !boolean(need(c, "angle_uses_periodic_boundary_conditions", w), w) &&
                  usize(need(c, "bond_count", w), w) == n_bonds && usize(need(c, "angle_count", w), w) == n_angles;
  if (!ok) throw Err{"harmonic source contract has unsupported schema, units, provider or term counts"};
  const std::string& given = text(need(c, "contract_sha256", w), w + ".contract_sha256");
  JVal body = c;
  body.obj.erase(std::remove_if(body.obj.begin(), body.obj.end(),
                                [](const std::pair<std::string, JVal>& kv) { return kv.first == "contract_sha256"; }),
                 body.obj.end());
  std::string canon;
  canon_value(body, canon);
  Sha256 h;
  h.update(canon.data(), canon.size());
  if (given != h.hex()) throw Err{"harmonic source contract canonical digest mismatch"};
  return {pb, pa};
}

void lower(const JVal& root, const prismq_prep_options& opt, pq::HostTopology& T, prismq_prep_report& R) {
  if (root.kind != JVal::Obj) throw Err{"top-level JSON value must be an object"};
  const std::string top = "PrismPrepTopology";
  // ---- required scalars and arrays (serde: no default on these fields) ----
  text(need(root, "source_pdb", top), "source_pdb");
  const uint64_t n = usize(need(root, "n_atoms", top), "n_atoms");
  const uint64_t n_res = usize(need(root, "n_residues", top), "n_residues");
  usize(need(root, "n_chains", top), "n_chains");
  if (n == 0 || n > (1ull << 28)) throw Err{"n_atoms must be in [1, 2^28]"};
  auto arr_of = [&](const char* key) -> const std::vector<JVal>& { return array(need(root, key, top), key); };
  const auto& positions = arr_of("positions");
  const auto& elements = arr_of("elements");
  const auto& atom_names = arr_of("atom_names");
  const auto& residue_names = arr_of("residue_names");
  const auto& residue_ids = arr_of("residue_ids");
  const auto& chain_ids = arr_of("chain_ids");
  const auto& charges = arr_of("charges");
  const auto& masses = arr_of("masses");
  const auto& ca = arr_of("ca_indices");
  const auto& bonds_j = arr_of("bonds");
  const auto& angles_j = arr_of("angles");
  const auto& dihs_j = arr_of("dihedrals");
  const auto& lj = arr_of("lj_params");
  const auto& excl_j = arr_of("exclusions");
  static const std::vector<JVal> kEmpty;
  const JVal* exc_v = root.get("nonbonded_exceptions");
  const auto& exc_j = exc_v ? array(*exc_v, "nonbonded_exceptions") : kEmpty;
  const JVal* hc_v = root.get("h_clusters");
  const auto& hc_j = hc_v ? array(*hc_v, "h_clusters") : kEmpty;
  for (const auto* list : {&elements, &atom_names, &residue_names, &chain_ids})
    for (const JVal& s : *list) text(s, "atom metadata entry");

  // ---- terms in the reference's types ----
  std::vector<Bond> bonds(bonds_j.size());
  for (size_t t = 0; t < bonds_j.size(); ++t) {
    const JVal& b = bonds_j[t];
    const std::string w = at("bonds", t);
    bonds[t] = {usize(need(b, "i", w), w + ".i"), usize(need(b, "j", w), w + ".j"), f64(need(b, "r0", w), w + ".r0"),
                f64(need(b, "k", w), w + ".k")};
  }
  std::vector<Angle> angles(angles_j.size());
  for (size_t t = 0; t < angles_j.size(); ++t) {
    const JVal& g = angles_j[t];
    const std::string w = at("angles", t);
    angles[t] = {usize(need(g, "i", w), w + ".i"), usize(need(g, "j", w), w + ".j"),
                 usize(need(g, "k_idx", w), w + ".k_idx"), f64(need(g, "theta0", w), w + ".theta0"),
                 f64(need(g, "force_k", w), w + ".force_k")};
  }
  std::vector<Dih> dihs(dihs_j.size());
  for (size_t t = 0; t < dihs_j.size(); ++t) {
    const JVal& d = dihs_j[t];
    const std::string w = at("dihedrals", t);
    // periodicity, phase, force_k and improper are serde(default)
    const JVal* per = d.get("periodicity");
    const JVal* ph = d.get("phase");
    const JVal* fk = d.get("force_k");
    if (const JVal* imp = d.get("improper")) boolean(*imp, w + ".improper");
    dihs[t] = {usize(need(d, "i", w), w + ".i"), usize(need(d, "j", w), w + ".j"),
               usize(need(d, "k_idx", w), w + ".k_idx"), usize(need(d, "l", w), w + ".l"),
               per ? i32(*per, w + ".periodicity") : 0, ph ? f64(*ph, w + ".phase") : 0.0,
               fk ? f64(*fk, w + ".force_k") : 0.0};
  }
  std::vector<Exc> excs(exc_j.size());
  for (size_t t = 0; t < exc_j.size(); ++t) {
    const JVal& e = exc_j[t];
    const std::string w = at("nonbonded_exceptions", t);
    excs[t] = {usize(need(e, "i", w), w + ".i"), usize(need(e, "j", w), w + ".j"),
               f64(need(e, "charge_product_e2", w), w + ".charge_product_e2"), f64(need(e, "sigma_A", w), w + ".sigma_A"),
               f64(need(e, "epsilon_kcal_mol", w), w + ".epsilon_kcal_mol")};
  }
  std::vector<Cluster> cls(hc_j.size());
  for (size_t t = 0; t < hc_j.size(); ++t) {
    const JVal& c = hc_j[t];
    const std::string w = at("h_clusters", t);
    Cluster& x = cls[t];
    i32(need(c, "type", w), w + ".type");
    x.c = usize(need(c, "central_atom", w), w + ".central_atom");
    for (const JVal& h : array(need(c, "hydrogen_atoms", w), w + ".hydrogen_atoms"))
      x.h.push_back(i32(h, w + ".hydrogen_atoms[]"));
    for (const JVal& l : array(need(c, "bond_lengths", w), w + ".bond_lengths"))
      x.len.push_back(f64(l, w + ".bond_lengths[]"));
    x.nh = usize(need(c, "n_hydrogens", w), w + ".n_hydrogens");
    x.inv_c = f64(need(c, "inv_mass_central", w), w + ".inv_mass_central");
    x.inv_h = f64(need(c, "inv_mass_h", w), w + ".inv_mass_h");
  }

  // ---- validate (input.rs:1996-2290) ----
  double bond_pref = 1.0, angle_pref = 1.0;
  const JVal* hcon = root.get("harmonic_parameter_contract");
  if (hcon && hcon->kind == JVal::Null) hcon = nullptr;
  if (hcon) std::tie(bond_pref, angle_pref) = harmonic_contract(*hcon, bonds.size(), angles.size());
  const std::pair<const char*, const std::vector<JVal>*> per_atom[] = {
      {"elements", &elements}, {"atom_names", &atom_names}, {"residue_names", &residue_names},
      {"residue_ids", &residue_ids}, {"chain_ids", &chain_ids}, {"charges", &charges}, {"masses", &masses},
      {"lj_params", &lj}, {"exclusions", &excl_j}};
  if (positions.size() != 3 * n)
    throw Err{"positions length " + std::to_string(positions.size()) + " != expected " + std::to_string(3 * n)};
  for (const auto& kv : per_atom)
    if (kv.second->size() != n)
      throw Err{std::string(kv.first) + " length " + std::to_string(kv.second->size()) + " != expected " +
                std::to_string(n)};
  uint64_t max_res = 0;
  for (size_t a = 0; a < n; ++a) max_res = std::max(max_res, usize(residue_ids[a], "residue_ids[]"));
  if (max_res >= n_res)
    throw Err{"max residue_id " + std::to_string(max_res) + " >= n_residues " + std::to_string(n_res)};
  T.n_atoms = (int32_t)n;
  T.positions.resize(3 * n);
  T.charges.resize(n);
  T.masses.resize(n);
  T.lj_sigma.resize(n);
  T.lj_epsilon.resize(n);
  for (size_t k = 0; k < 3 * n; ++k) {
    T.positions[k] = f32(positions[k], "positions[]");
    if (!std::isfinite(T.positions[k])) throw Err{"position value " + std::to_string(k) + " is non-finite"};
  }
  for (size_t a = 0; a < n; ++a) {
    T.charges[a] = f32(charges[a], "charges[]");
    if (!std::isfinite(T.charges[a])) throw Err{"charge value " + std::to_string(a) + " is non-finite"};
    T.masses[a] = f32(masses[a], "masses[]");
    if (!std::isfinite(T.masses[a]) || T.masses[a] <= 0.0f)
      throw Err{"mass value " + std::to_string(a) + " must be finite and positive"};
    const std::string w = at("lj_params", a);
    const double sig = f64(need(lj[a], "sigma", w), w + ".sigma"), eps = f64(need(lj[a], "epsilon", w), w + ".epsilon");
    if (!std::isfinite(sig) || !std::isfinite(eps) || sig < 0.0 || eps < 0.0)
      throw Err{"invalid LJ parameters for atom " + std::to_string(a)};
    T.lj_sigma[a] = (float)sig;
    T.lj_epsilon[a] = (float)eps;
  }
  std::set<uint64_t> ca_seen;
  for (const JVal& v : ca) {
    const uint64_t i = usize(v, "ca_indices[]");
    if (i >= n || !ca_seen.insert(i).second) throw Err{"invalid or duplicate CA atom index " + std::to_string(i)};
  }
  for (size_t t = 0; t < bonds.size(); ++t) {
    const Bond& b = bonds[t];
    if (b.i >= n || b.j >= n || b.i == b.j || !std::isfinite(b.r0) || !std::isfinite(b.k) || b.r0 <= 0.0 || b.k < 0.0)
      throw Err{"invalid bond term at index " + std::to_string(t)};
  }
  for (size_t t = 0; t < angles.size(); ++t) {
    const Angle& g = angles[t];
    if (g.i >= n || g.j >= n || g.k >= n || g.i == g.j || g.j == g.k || g.i == g.k || !std::isfinite(g.theta0) ||
        !std::isfinite(g.force_k) || g.theta0 <= 0.0 || g.theta0 > M_PI || g.force_k < 0.0)
      throw Err{"invalid angle term at index " + std::to_string(t)};
  }
  for (size_t t = 0; t < dihs.size(); ++t) {
    const Dih& d = dihs[t];
    if (d.i >= n || d.j >= n || d.k >= n || d.l >= n || d.n <= 0 || !std::isfinite(d.phase) ||
        !std::isfinite(d.force_k))
      throw Err{"invalid dihedral term at index " + std::to_string(t)};
  }
  std::vector<std::vector<uint64_t>> excl(n);
  for (size_t a = 0; a < n; ++a)
    for (const JVal& v : array(excl_j[a], at("exclusions", a))) excl[a].push_back(usize(v, "exclusions[][]"));
  std::set<std::pair<uint64_t, uint64_t>> strict;
  for (size_t a = 0; a < n; ++a) {
    std::set<uint64_t> local;
    for (uint64_t p : excl[a]) {
      if (p >= n || p == a || !local.insert(p).second)
        throw Err{"invalid, self, or duplicate strict exclusion (" + std::to_string(a) + ", " + std::to_string(p) + ")"};
      if (std::find(excl[p].begin(), excl[p].end(), (uint64_t)a) == excl[p].end())
        throw Err{"asymmetric strict exclusion (" + std::to_string(a) + ", " + std::to_string(p) + ")"};
      strict.insert({std::min<uint64_t>(a, p), std::max<uint64_t>(a, p)});
    }
  }
  std::set<std::pair<uint64_t, uint64_t>> exc_pairs;
  for (const Exc& e : excs) {
    const std::string pair = "(" + std::to_string(e.i) + ", " + std::to_string(e.j) + ")";
    if (e.i >= n || e.j >= n) throw Err{"nonbonded exception index out of range: " + pair};
    if (e.i >= e.j) throw Err{"nonbonded exception pair must be canonical i < j: " + pair};
    if (!std::isfinite(e.qq) || !std::isfinite(e.sig) || !std::isfinite(e.eps) || e.sig < 0.0 || e.eps < 0.0)
      throw Err{"invalid nonbonded exception parameters for pair " + pair};
    const std::pair<const char*, double> fields[] = {
        {"charge_product_e2", e.qq}, {"sigma_A", e.sig}, {"epsilon_kcal_mol", e.eps}};
    for (const auto& f : fields) {
      const float narrowed = (float)f.second;
      if (!std::isfinite(narrowed) || (f.second != 0.0 && narrowed == 0.0f) ||
          (f.second == 0.0 && std::signbit(f.second)))
        throw Err{std::string("nonbonded exception ") + f.first + " is not safely representable as f32 for pair " +
                  pair};
      const double error = std::fabs((double)narrowed - f.second);
      const double tol = std::max(1.0e-12, std::fabs(f.second) * 1.0e-6);
      if (error > tol)
        throw Err{std::string("nonbonded exception ") + f.first + " f32 conversion error exceeds tolerance for pair " +
                  pair};
    }
    if (!exc_pairs.insert({e.i, e.j}).second) throw Err{"duplicate nonbonded exception pair: " + pair};
    if (strict.count({e.i, e.j})) throw Err{"nonbonded exception overlaps strict exclusion: " + pair};
  }
  const JVal* econ = root.get("nonbonded_exception_contract");
  if (econ && econ->kind == JVal::Null) econ = nullptr;
  if (excs.empty() && econ) throw Err{"nonbonded exception contract is present but the exact pair vector is empty"};
  if (!excs.empty() && !econ) throw Err{"exact nonbonded exceptions require a versioned completeness/digest contract"};
  if (econ) {
    const std::string w = "nonbonded_exception_contract";
    const JVal& c = *econ;
    if (text(need(c, "schema_kind", w), w) != "prismos_exact_nonbonded_exceptions_v2" ||
        usize(need(c, "schema_version", w), w) != 2)
      throw Err{"unsupported nonbonded exception contract"};
    if (text(need(c, "semantics", w), w) != "OPENMM_NONBONDEDFORCE_ABSOLUTE_EXCEPTION_PARAMETERS_V1" ||
        text(need(c, "dynamic_charge_scaling_semantics", w), w) !=
            "EXCITED_STATE_MULTIPLIES_GROUND_STATE_CHARGE_PRODUCT_BY_PER_ATOM_SCALE_PRODUCT_V1")
      throw Err{"unsupported exact nonbonded exception semantics"};
    if (text(need(c, "pair_digest_algorithm", w), w) != "SHA256_PRISMOS_NBEX_ACTIVE_V1_LE_U64_U64_F64_F64_F64" ||
        text(need(c, "strict_exclusion_digest_algorithm", w), w) != "SHA256_PRISMOS_NBEX_STRICT_V1_LE_U64_U64")
      throw Err{"unsupported nonbonded exception digest algorithms"};
    if (!boolean(need(c, "complete", w), w) || boolean(need(c, "fallback_used", w), w) ||
        boolean(need(c, "hardcoded_uniform_scaling_allowed", w), w))
      throw Err{"exact nonbonded exception contract is incomplete or records fallback"};
    const uint64_t n_exact = usize(need(c, "exact_scaled_pair_count", w), w);
    const uint64_t n_strict = usize(need(c, "strict_exclusion_pair_count", w), w);
    if (n_exact != excs.size()) throw Err{"nonbonded exception count mismatch"};
    if (n_strict != strict.size()) throw Err{"strict exclusion count mismatch"};
    if (usize(need(c, "total_openmm_exception_count", w), w) != n_exact + n_strict)
      throw Err{"OpenMM exception completeness mismatch"};
    // active-pair digest over the (i, j)-sorted rows (input.rs:1935-1949)
    std::vector<const Exc*> rows;
    for (const Exc& e : excs) rows.push_back(&e);
    std::sort(rows.begin(), rows.end(),
              [](const Exc* a, const Exc* b) { return a->i != b->i ? a->i < b->i : a->j < b->j; });
    Sha256 ha;
    ha.update("PRISMOS_NBEX_ACTIVE_V1\0", 23);
    ha.update_u64le(rows.size());
    for (const Exc* e : rows) {
      ha.update_u64le(e->i);
      ha.update_u64le(e->j);
      ha.update_f64le(e->qq);
      ha.update_f64le(e->sig);
      ha.update_f64le(e->eps);
    }
    if (text(need(c, "pair_digest_sha256", w), w) != ha.hex()) throw Err{"nonbonded exception digest mismatch"};
    // strict-exclusion digest over the sorted canonical pair set (:1952-1969)
    Sha256 hs;
    hs.update("PRISMOS_NBEX_STRICT_V1\0", 23);
    hs.update_u64le(strict.size());
    for (const auto& pr : strict) {
      hs.update_u64le(pr.first);
      hs.update_u64le(pr.second);
    }
    if (text(need(c, "strict_exclusion_digest_sha256", w), w) != hs.hex())
      throw Err{"strict exclusion digest mismatch"};
    const JVal* prm = root.get("generated_prmtop_sha256");
    if (!prm || prm->kind != JVal::Str)
      throw Err{"exact nonbonded exceptions require generated_prmtop_sha256 provenance"};
    if (text(need(c, "source_prmtop_sha256", w), w) != prm->str || !is_hex64(prm->str))
      throw Err{"exact exception source prmtop hash is absent, malformed, or mismatched"};
  }

  // ---- nonbonded execution policy (input.rs:1429-1450) ----
  if (opt.require_exceptions && (excs.empty() || !econ))
    throw Err{"production nonbonded execution requires exact OpenMM exception parameters and a complete V2 contract"};

  // ---- harmonic lowering (input.rs:467-520) ----
  if (!hcon && opt.require_harmonic_contract)
    throw Err{"harmonic source convention is absent: refusing production lowering"};
  for (const Bond& b : bonds)
    if (!std::isfinite((float)b.r0) || (float)b.r0 <= 0.0f)
      throw Err{"harmonic equilibrium coordinate is not representable in the target float32 ABI"};
  for (const Angle& g : angles)
    if (!std::isfinite((float)g.theta0) || (float)g.theta0 <= 0.0f)
      throw Err{"harmonic equilibrium coordinate is not representable in the target float32 ABI"};
  const double bond_scale = bond_pref / 1.0, angle_scale = angle_pref / 1.0;  // target: AMBER_NO_HALF_ENERGY
  auto cast = [](double raw, double scale, const char* label, size_t index) -> float {
    const double mapped = raw * scale;
    const float dev = (float)mapped;
    if (!std::isfinite(raw) || raw < 0.0 || !std::isfinite(mapped) || !std::isfinite(dev) ||
        (raw > 0.0 && dev == 0.0f))
      throw Err{std::string(label) + " coefficient " + std::to_string(index) +
                " is invalid or not representable in the target float32 ABI"};
    return dev;
  };
  for (size_t t = 0; t < bonds.size(); ++t)
    T.bonds.push_back({(int32_t)bonds[t].i, (int32_t)bonds[t].j, (float)bonds[t].r0,
                       cast(bonds[t].k, bond_scale, "bond", t)});
  for (size_t t = 0; t < angles.size(); ++t)
    T.angles.push_back({(int32_t)angles[t].i, (int32_t)angles[t].j, (int32_t)angles[t].k, (float)angles[t].theta0,
                        cast(angles[t].force_k, angle_scale, "angle", t)});
  for (const Dih& d : dihs)
    T.dihedrals.push_back({(int32_t)d.i, (int32_t)d.j, (int32_t)d.k, (int32_t)d.l, (int32_t)d.n, (float)d.phase,
                           (float)d.force_k});
  for (const Exc& e : excs) T.exceptions.push_back({(int32_t)e.i, (int32_t)e.j, (float)e.qq, (float)e.sig, (float)e.eps});
  T.exclusion_offsets.assign(1, 0);
  for (size_t a = 0; a < n; ++a) {
    for (uint64_t p : excl[a]) T.exclusions.push_back((int32_t)p);
    T.exclusion_offsets.push_back((int32_t)T.exclusions.size());
  }
  R.bond_scale = bond_scale;
  R.angle_scale = angle_scale;
  R.exact_exceptions = (int32_t)excs.size();

  // ---- hydrogen mass repartitioning (input.rs:2482-2560) ----
  for (size_t t = 0; t < cls.size(); ++t) {
    const Cluster& x = cls[t];
    const std::string w = at("h_clusters", t);
    if (x.c >= n) throw Err{w + ".central_atom is out of range"};
    if (x.h.size() > 3 || x.len.size() > 3) throw Err{w + " lists more than three hydrogens"};
    for (int64_t h : x.h)
      if (h >= (int64_t)n) throw Err{w + ".hydrogen_atoms[] is out of range"};
  }
  const JVal* hmr = root.get("hmr_applied");
  if (hmr && hmr->kind != JVal::Bool && hmr->kind != JVal::Null) throw Err{"hmr_applied must be true, false or null"};
  const bool verified = hmr && hmr->kind == JVal::Bool && hmr->b;
  if (opt.apply_hmr && !verified) {
    const double factor = opt.hmr_factor;
    if (!(factor > 0.0) || !std::isfinite(factor)) throw Err{"hmr_factor must be positive"};
    R.hmr_performed = 1;
    for (Cluster& x : cls) {
      const double m_h = 1.0 / x.inv_h, m_c = 1.0 / x.inv_c;
      R.total_mass_before += m_c + (double)x.nh * m_h;
      const double m_h_new = m_h * factor;
      const double dm = m_h_new - m_h;
      const double m_c_new = m_c - (double)x.nh * dm;
      if (m_c_new < 1.0) {  // the central atom keeps at least 1 amu: cluster left as is
        R.total_mass_after += m_c + (double)x.nh * m_h;
        ++R.n_skipped;
        continue;
      }
      x.inv_h = 1.0 / m_h_new;
      x.inv_c = 1.0 / m_c_new;
      ++R.n_repartitioned;
      R.total_mass_after += m_c_new + (double)x.nh * m_h_new;
      T.masses[x.c] = (float)m_c_new;
      for (int64_t h : x.h)
        if (h >= 0) T.masses[h] = (float)m_h_new;
    }
  }
  for (const Cluster& x : cls) {
    prismq_hcluster h;
    std::memset(&h, 0, sizeof(h));
    h.central_atom = (int32_t)x.c;
    for (int k = 0; k < 3; ++k) {
      h.hydrogen_atoms[k] = k < (int)x.h.size() ? (int32_t)x.h[k] : -1;
      h.bond_lengths[k] = k < (int)x.len.size() ? (float)x.len[k] : 0.0f;
    }
    h.n_hydrogens = (int32_t)std::min<uint64_t>(x.nh, 0x7FFFFFFF);
    h.inv_mass_central = (float)x.inv_c;
    h.inv_mass_h = (float)x.inv_h;
    T.clusters.push_back(h);
  }
}

prismq_status parse_and_lower(const char* src, size_t len, const prismq_prep_options* opt_in,
                              prismq_topology_buf** out, prismq_prep_report* report) {
  if (!src || !out) {
    pq::set_last_error("NULL argument");
    return PRISMQ_E_INVALID;
  }
  *out = nullptr;
  prismq_prep_options opt;
  prismq_prep_options_default(&opt);
  if (opt_in) opt = *opt_in;
  Parser ps{src, src + len};
  JVal root;
  if (!ps.val(root)) {
    pq::set_last_error("JSON: " + ps.err + " at byte " + std::to_string(ps.p - src));
    return PRISMQ_E_INVALID;
  }
  ps.ws();
  if (ps.p != ps.end) {
    pq::set_last_error("JSON: trailing characters at byte " + std::to_string(ps.p - src));
    return PRISMQ_E_INVALID;
  }
  auto buf = std::make_unique<prismq_topology_buf>();
  prismq_prep_report rep;
  std::memset(&rep, 0, sizeof(rep));
  try {
    lower(root, opt, buf->topo, rep);
  } catch (const Err& e) {
    pq::set_last_error("PrismPrepTopology: " + e.msg);
    return PRISMQ_E_INVALID;
  }
  if (report) *report = rep;
  *out = buf.release();
  return PRISMQ_OK;
}

}  // namespace

extern "C" {

void prismq_prep_options_default(prismq_prep_options* opt) {
  if (!opt) return;
  std::memset(opt, 0, sizeof(*opt));
  opt->apply_hmr = 1;
  opt->require_harmonic_contract = 1;
  opt->require_exceptions = 1;
  opt->hmr_factor = 3.0;
}

prismq_status prismq_topology_from_prep_json(const char* text, size_t len, const prismq_prep_options* opt,
                                             prismq_topology_buf** out, prismq_prep_report* report) {
  return parse_and_lower(text, len, opt, out, report);
}

prismq_status prismq_topology_load_prep_json(const char* path, const prismq_prep_options* opt,
                                             prismq_topology_buf** out, prismq_prep_report* report) {
  if (!path || !out) {
    pq::set_last_error("NULL argument");
    return PRISMQ_E_INVALID;
  }
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    pq::set_last_error(std::string("cannot open ") + path);
    return PRISMQ_E_NOT_FOUND;
  }
  std::string content;
  char chunk[1 << 16];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) content.append(chunk, got);
  std::fclose(f);
  return parse_and_lower(content.data(), content.size(), opt, out, report);
}

}  // extern "C"
