// Nektar++ XML/FLD scene loader, hexahedra (the reference's load_xml_fld path,
// FEM-AABB/xml_fld_loader.cpp:16-402, restricted to hexes).
//
//  * geometry (FEM-AABB/xml_fld_geometry_parser.cpp:48-508): <VERTEX>,
//    <EDGE>, <FACE> (quad faces as edge loops), <ELEMENT> hexes given by 6
//    faces or 8 vertices, <CURVED> edges and faces (NUMPOINTS, point type);
//    XML comments are ignored.
//  * expansions (FEM-AABB/xml_fld_field_parser.cpp:202-289): <COMPOSITE>
//    lists and <E COMPOSITE=.. NUMMODES|NUMMODESPERDIR=.. FIELDS=..>; the
//    first NUMMODES in the file is the default.
//  * field (FEM-AABB/xml_fld_field_parser.cpp:165-200): FIELDS="..." names,
//    the <ELEMENTS> payload as ASCII numbers or base64 + zlib (inflate below)
//    of FP64 (or FP32) values, cast to FP32; slices assigned to elements in
//    expansion order, per field (FEM-AABB/xml_fld_loader.cpp:166-223).
//  * geometry build (FEM-AABB/xml_fld_geometry_builder.cpp:68-381): GLL nodal
//    grid from the trilinear corners, curved edges resampled onto it, curved
//    faces resampled (Legendre interpolation) and blended linearly into the
//    volume, then a tensor-product modal fit in FP64.
// Arithmetic is FP64 throughout (the reference mixes FP32 and FP64); results
// agree with the reference loader to FP32 rounding.
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <unordered_map>
#include <vector>

#include "ho_host.h"

namespace ho {
namespace {

struct V3d {
  double x, y, z;
};
V3d operator+(V3d a, V3d b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3d operator-(V3d a, V3d b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3d operator*(double s, V3d a) { return {s * a.x, s * a.y, s * a.z}; }

bool read_file(const std::string& path, std::string& out) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return false;
  std::ostringstream ss;
  ss << in.rdbuf();
  out = ss.str();
  return true;
}

std::string strip_comments(const std::string& t) {
  std::string out;
  size_t pos = 0;
  while (pos < t.size()) {
    const size_t a = t.find("<!--", pos);
    if (a == std::string::npos) {
      out.append(t, pos, std::string::npos);
      break;
    }
    out.append(t, pos, a - pos);
    const size_t b = t.find("-->", a + 4);
    if (b == std::string::npos) break;  // unclosed comment: drop the rest
    pos = b + 3;
  }
  return out;
}

std::string trim(const std::string& s) {
  const size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return {};
  return s.substr(a, s.find_last_not_of(" \t\r\n") - a + 1);
}

std::string upper(std::string s) {
  for (auto& c : s) c = static_cast<char>(std::toupper(static_cast<unsigned char>(c)));
  return s;
}

bool is_space(char c) { return std::isspace(static_cast<unsigned char>(c)) != 0; }

// Attribute value of KEY in a tag header: KEY="v" or KEY='v', the key not
// preceded by a letter or digit (so ID does not match EDGEID).
std::string attr(const std::string& tag, const std::string& key) {
  size_t pos = 0;
  while ((pos = tag.find(key, pos)) != std::string::npos) {
    const bool left_ok = pos == 0 || !std::isalnum(static_cast<unsigned char>(tag[pos - 1]));
    size_t q = pos + key.size();
    while (q < tag.size() && is_space(tag[q])) ++q;
    if (left_ok && q < tag.size() && tag[q] == '=') {
      ++q;
      while (q < tag.size() && is_space(tag[q])) ++q;
      if (q < tag.size() && (tag[q] == '"' || tag[q] == '\'')) {
        const size_t e = tag.find(tag[q], q + 1);
        if (e != std::string::npos) return tag.substr(q + 1, e - q - 1);
      }
    }
    pos += key.size();
  }
  return {};
}

// Block from <NAME up to (excluding) the first </NAME>, or empty.
std::string section(const std::string& t, const std::string& name) {
  const size_t a = t.find("<" + name), b = t.find("</" + name + ">");
  if (a == std::string::npos || b == std::string::npos || b <= a) return {};
  return t.substr(a, b - a);
}

struct Tag {
  std::string header, body;
};

// Every <NAME ...>body</NAME> and <NAME .../> in text; NAME must be followed
// by whitespace, '>' or '/', so <V does not match <VERTEX>.
std::vector<Tag> tags(const std::string& t, const std::string& name) {
  std::vector<Tag> out;
  const std::string open = "<" + name, close = "</" + name + ">";
  size_t pos = 0;
  while ((pos = t.find(open, pos)) != std::string::npos) {
    const size_t after = pos + open.size();
    if (after >= t.size() || !(is_space(t[after]) || t[after] == '>' || t[after] == '/')) {
      pos = after;
      continue;
    }
    const size_t gt = t.find('>', pos);
    if (gt == std::string::npos) break;
    Tag tg;
    tg.header = t.substr(pos, gt - pos + 1);
    if (t[gt - 1] == '/') {
      out.push_back(tg);
      pos = gt + 1;
      continue;
    }
    const size_t ce = t.find(close, gt);
    if (ce == std::string::npos) break;
    tg.body = t.substr(gt + 1, ce - gt - 1);
    out.push_back(tg);
    pos = ce + close.size();
  }
  return out;
}

// Whitespace-separated FP32 numbers up to the first token that does not
// parse (decimal -> float rounding, like reading floats from a stream).
std::vector<float> floats(const std::string& s) {
  std::vector<float> v;
  const char* p = s.c_str();
  for (;;) {
    while (*p && is_space(*p)) ++p;
    if (!*p) break;
    char* end = nullptr;
    const float f = std::strtof(p, &end);
    if (end == p) break;
    v.push_back(f);
    p = end;
  }
  return v;
}

// Whitespace-separated integers up to the first token that does not parse.
std::vector<int> ints(const std::string& s) {
  std::vector<int> v;
  const char* p = s.c_str();
  for (;;) {
    while (*p && is_space(*p)) ++p;
    if (!*p) break;
    char* end = nullptr;
    const long x = std::strtol(p, &end, 10);
    if (end == p) break;
    v.push_back(static_cast<int>(x));
    p = end;
  }
  return v;
}

// Modes attribute: "5" -> 5,5,5; "4,6" -> 4,6,1; "4,5,6". Tokens split at
// ',', ' ' or ';' and read with atoi.
std::array<unsigned, 3> parse_modes(const std::string& s) {
  std::vector<int> v;
  std::string tok;
  for (size_t i = 0; i <= s.size(); ++i) {
    const char c = i < s.size() ? s[i] : ',';
    if (c == ',' || c == ' ' || c == ';') {
      if (!tok.empty()) v.push_back(std::atoi(tok.c_str()));
      tok.clear();
    } else {
      tok.push_back(c);
    }
  }
  if (v.empty()) return {0, 0, 0};
  if (v.size() == 1) return {unsigned(v[0]), unsigned(v[0]), unsigned(v[0])};
  if (v.size() == 2) return {unsigned(v[0]), unsigned(v[1]), 1u};
  return {unsigned(v[0]), unsigned(v[1]), unsigned(v[2])};
}

std::vector<std::string> field_list(const std::string& s) {
  std::vector<std::string> out;
  std::stringstream ss(s);
  std::string tok;
  while (std::getline(ss, tok, ',')) {
    tok = trim(tok);
    if (!tok.empty()) out.push_back(tok);
  }
  return out;
}

// "lo-hi" (both read as %d, the dash right after lo) or a single id (atoi).
void id_range(const std::string& tok, int& lo, int& hi) {
  if (tok.find('-') == std::string::npos) {
    lo = hi = std::atoi(tok.c_str());
    return;
  }
  lo = hi = 0;
  const char* p = tok.c_str();
  char* end = nullptr;
  const long a = std::strtol(p, &end, 10);
  if (end == p) return;
  lo = static_cast<int>(a);
  if (*end != '-') return;
  p = end + 1;
  const long b = std::strtol(p, &end, 10);
  if (end != p) hi = static_cast<int>(b);
}

// ---- base64 + inflate (RFC 1950/1951) --------------------------------------
struct B64Table {
  int8_t v[256];
  B64Table() {
    std::memset(v, -1, sizeof(v));
    const char* a = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
    for (int i = 0; i < 64; ++i) v[static_cast<unsigned char>(a[i])] = static_cast<int8_t>(i);
  }
};

std::vector<uint8_t> base64(const std::string& in) {
  static const B64Table table;  // built once, thread-safe
  const int8_t* lut = table.v;
  std::vector<uint8_t> out;
  uint32_t acc = 0;
  int bits = 0;
  for (unsigned char c : in) {
    if (std::isspace(c)) continue;
    const int v = lut[c];
    if (v < 0) break;  // '=' padding or anything else ends the payload
    acc = (acc << 6) | static_cast<uint32_t>(v);
    bits += 6;
    if (bits >= 8) {
      bits -= 8;
      out.push_back(static_cast<uint8_t>((acc >> bits) & 0xFFu));
    }
  }
  return out;
}

class Inflater {
 public:
  Inflater(const uint8_t* d, size_t n) : d_(d), n_(n) {}
  // Input bytes used so far; bits of a partly used byte are discarded.
  size_t consumed() const { return pos_ - static_cast<size_t>(cnt_ / 8); }
  bool run(std::vector<uint8_t>& out) {
    int final_block = 0;
    do {
      if (!bits(1, final_block)) return false;
      int type;
      if (!bits(2, type)) return false;
      bool ok = false;
      if (type == 0) ok = stored(out);
      else if (type == 1) ok = fixed(out);
      else if (type == 2) ok = dynamic(out);
      if (!ok) return false;
    } while (!final_block);
    return true;
  }

 private:
  struct Huff {
    uint16_t count[16];
    uint16_t sym[320];
  };
  const uint8_t* d_;
  size_t n_, pos_ = 0;
  uint32_t buf_ = 0;
  int cnt_ = 0;

  bool bits(int need, int& v) {
    while (cnt_ < need) {
      if (pos_ >= n_) return false;
      buf_ |= static_cast<uint32_t>(d_[pos_++]) << cnt_;
      cnt_ += 8;
    }
    v = static_cast<int>(buf_ & ((1u << need) - 1u));
    buf_ >>= need;
    cnt_ -= need;
    return true;
  }
  bool stored(std::vector<uint8_t>& out) {
    buf_ = 0;
    cnt_ = 0;
    if (pos_ + 4 > n_) return false;
    const unsigned len = d_[pos_] | (d_[pos_ + 1] << 8), nlen = d_[pos_ + 2] | (d_[pos_ + 3] << 8);
    pos_ += 4;
    if ((len ^ 0xFFFFu) != nlen || pos_ + len > n_) return false;
    out.insert(out.end(), d_ + pos_, d_ + pos_ + len);
    pos_ += len;
    return true;
  }
  static bool build(Huff& h, const uint8_t* lens, int n) {
    std::memset(h.count, 0, sizeof(h.count));
    for (int i = 0; i < n; ++i) h.count[lens[i]]++;
    h.count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
      left <<= 1;
      left -= h.count[l];
      if (left < 0) return false;  // over-subscribed
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + h.count[l];
    for (int i = 0; i < n; ++i)
      if (lens[i]) h.sym[offs[lens[i]]++] = static_cast<uint16_t>(i);
    return true;
  }
  bool decode(const Huff& h, int& sym) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
      int b;
      if (!bits(1, b)) return false;
      code |= b;
      const int count = h.count[l];
      if (code - count < first) {
        sym = h.sym[index + (code - first)];
        return true;
      }
      index += count;
      first += count;
      first <<= 1;
      code <<= 1;
    }
    return false;
  }
  bool codes(std::vector<uint8_t>& out, const Huff& lit, const Huff& dist) {
    static const uint16_t lbase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59,
                                       67, 83, 99, 115, 131, 163, 195, 227, 258};
    static const uint8_t lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    static const uint16_t dbase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769,
                                       1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
    static const uint8_t dext[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8,
                                     9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
    for (;;) {
      int s;
      if (!decode(lit, s)) return false;
      if (s < 256) {
        out.push_back(static_cast<uint8_t>(s));
      } else if (s == 256) {
        return true;
      } else {
        s -= 257;
        if (s >= 29) return false;
        int e;
        if (!bits(lext[s], e)) return false;
        const size_t len = lbase[s] + e;
        int ds;
        if (!decode(dist, ds) || ds >= 30) return false;
        if (!bits(dext[ds], e)) return false;
        const size_t back = dbase[ds] + e;
        if (back > out.size()) return false;
        const size_t from = out.size() - back;
        for (size_t i = 0; i < len; ++i) out.push_back(out[from + i]);
      }
    }
  }
  bool fixed(std::vector<uint8_t>& out) {
    uint8_t l[288];
    for (int i = 0; i < 144; ++i) l[i] = 8;
    for (int i = 144; i < 256; ++i) l[i] = 9;
    for (int i = 256; i < 280; ++i) l[i] = 7;
    for (int i = 280; i < 288; ++i) l[i] = 8;
    Huff lit, dist;
    build(lit, l, 288);
    uint8_t dl[30];
    for (int i = 0; i < 30; ++i) dl[i] = 5;
    build(dist, dl, 30);
    return codes(out, lit, dist);
  }
  bool dynamic(std::vector<uint8_t>& out) {
    static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    int nlen, ndist, ncode;
    if (!bits(5, nlen) || !bits(5, ndist) || !bits(4, ncode)) return false;
    nlen += 257;
    ndist += 1;
    ncode += 4;
    if (nlen > 286 || ndist > 30) return false;
    uint8_t lens[320] = {0};
    for (int i = 0; i < ncode; ++i) {
      int v;
      if (!bits(3, v)) return false;
      lens[order[i]] = static_cast<uint8_t>(v);
    }
    Huff lencode;
    if (!build(lencode, lens, 19)) return false;
    std::memset(lens, 0, sizeof(lens));
    int idx = 0;
    while (idx < nlen + ndist) {
      int sym;
      if (!decode(lencode, sym)) return false;
      if (sym < 16) {
        lens[idx++] = static_cast<uint8_t>(sym);
        continue;
      }
      int rep = 0, val = 0;
      if (sym == 16) {
        if (idx == 0) return false;
        val = lens[idx - 1];
        if (!bits(2, rep)) return false;
        rep += 3;
      } else if (sym == 17) {
        if (!bits(3, rep)) return false;
        rep += 3;
      } else {
        if (!bits(7, rep)) return false;
        rep += 11;
      }
      if (idx + rep > nlen + ndist) return false;
      while (rep--) lens[idx++] = static_cast<uint8_t>(val);
    }
    Huff lit, dist;
    if (!build(lit, lens, nlen) || !build(dist, lens + nlen, ndist)) return false;
    return codes(out, lit, dist);
  }
};

uint32_t adler32(const std::vector<uint8_t>& d) {
  uint32_t a = 1, b = 0;
  for (uint8_t x : d) {
    a = (a + x) % 65521u;
    b = (b + a) % 65521u;
  }
  return (b << 16) | a;
}

// A zlib stream (RFC 1950: header, deflate data, Adler-32 of the output),
// else raw deflate data; false when neither decodes.
bool inflate_any(const std::vector<uint8_t>& in, std::vector<uint8_t>& out) {
  if (in.empty()) return false;
  if (in.size() >= 6 && (in[0] & 0x0F) == 8 && (in[0] >> 4) <= 7 && ((in[0] << 8) | in[1]) % 31 == 0 &&
      !(in[1] & 0x20)) {
    Inflater z(in.data() + 2, in.size() - 2);
    out.clear();
    if (z.run(out)) {
      const size_t tail = 2 + z.consumed();
      if (tail + 4 <= in.size()) {
        const uint32_t want = (uint32_t(in[tail]) << 24) | (uint32_t(in[tail + 1]) << 16) |
                              (uint32_t(in[tail + 2]) << 8) | uint32_t(in[tail + 3]);
        if (want == adler32(out)) return true;
      }
    }
  }
  Inflater r(in.data(), in.size());
  out.clear();
  return r.run(out);
}

// ---- geometry ----------------------------------------------------------------
struct CurvedPts {
  unsigned num = 0;
  bool even = false;  // PolyEvenlySpaced / uniform points, else GLL
  std::vector<V3d> pts;
};

struct Hex {
  int id = 0;
  std::array<int, 8> verts{};
  std::array<int, 12> edges{};
  std::array<int, 6> faces{};
};

const int kHexEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 4}, {1, 5},
                             {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {7, 4}};
const int kFaceVerts[6][4] = {{0, 1, 2, 3}, {0, 1, 5, 4}, {1, 2, 6, 5}, {3, 2, 6, 7}, {0, 3, 7, 4}, {4, 5, 6, 7}};

long long edge_key(int a, int b) {
  if (a > b) std::swap(a, b);
  return (static_cast<long long>(a) << 32) | static_cast<unsigned>(b);
}

bool node_type_even(const std::string& t) {
  const std::string u = upper(t);
  return u.find("EVENLY") != std::string::npos || u.find("POLY") != std::string::npos ||
         u.find("UNIFORM") != std::string::npos;
}

std::vector<double> nodes_of(unsigned n, bool even) {
  if (!even) return gll_nodes(static_cast<int>(n));
  std::vector<double> x(n);
  for (unsigned i = 0; i < n; ++i) x[i] = n == 1 ? 0.0 : -1.0 + 2.0 * i / (n - 1);
  return x;
}

double legendre_p(int n, double x) {
  double p0 = 1.0, p1 = x;
  if (n == 0) return 1.0;
  for (int k = 2; k <= n; ++k) {
    const double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = pk;
  }
  return p1;
}

bool dense_inverse(std::vector<double> a, int n, std::vector<double>& inv) {
  inv.assign(static_cast<size_t>(n) * n, 0.0);
  for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c])) piv = r;
    if (std::fabs(a[piv * n + c]) < 1e-300) return false;
    if (piv != c)
      for (int k = 0; k < n; ++k) {
        std::swap(a[c * n + k], a[piv * n + k]);
        std::swap(inv[c * n + k], inv[piv * n + k]);
      }
    const double s = 1.0 / a[c * n + c];
    for (int k = 0; k < n; ++k) {
      a[c * n + k] *= s;
      inv[c * n + k] *= s;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c || a[r * n + c] == 0.0) continue;
      const double f = a[r * n + c];
      for (int k = 0; k < n; ++k) {
        a[r * n + k] -= f * a[c * n + k];
        inv[r * n + k] -= f * inv[c * n + k];
      }
    }
  }
  return true;
}

// Curved edge points onto `target` GLL nodes through a Modified-A fit
// (FEM-AABB/xml_fld_math.cpp:540-590).
std::vector<V3d> resample_edge(const CurvedPts& ce, unsigned target, bool reverse) {
  const unsigned ns = static_cast<unsigned>(ce.pts.size());
  const std::vector<double> src = nodes_of(ns, ce.even);
  std::vector<double> V(static_cast<size_t>(ns) * ns), Vi;
  for (unsigned r = 0; r < ns; ++r)
    for (unsigned a = 0; a < ns; ++a) V[r * ns + a] = mod_a(static_cast<int>(a), src[r]);
  if (!dense_inverse(V, static_cast<int>(ns), Vi)) return {};
  std::vector<V3d> coef(ns, V3d{0, 0, 0});
  for (unsigned a = 0; a < ns; ++a)
    for (unsigned i = 0; i < ns; ++i) coef[a] = coef[a] + Vi[a * ns + i] * ce.pts[i];
  const std::vector<double> tgt = gll_nodes(static_cast<int>(target));
  std::vector<V3d> out(target, V3d{0, 0, 0});
  for (unsigned i = 0; i < target; ++i) {
    const double r = reverse ? tgt[target - 1 - i] : tgt[i];
    for (unsigned a = 0; a < ns; ++a) out[i] = out[i] + mod_a(static_cast<int>(a), r) * coef[a];
  }
  return out;
}

// Orient a curved face's point grid so its corners match the face's expected
// corners (one of the 8 axis swaps / flips, tolerance 1e-3); unmatched grids
// are kept as given (FEM-AABB/xml_fld_math.cpp:592-666).
std::vector<V3d> orient_grid(const std::vector<V3d>& g, unsigned dim, const std::array<V3d, 4>& want) {
  auto at = [&](unsigned i, unsigned j) { return g[j * dim + i]; };
  auto d2 = [](V3d a, V3d b) {
    const V3d d = a - b;
    return d.x * d.x + d.y * d.y + d.z * d.z;
  };
  for (int sw = 0; sw < 2; ++sw)
    for (int fr = 0; fr < 2; ++fr)
      for (int fs = 0; fs < 2; ++fs) {
        auto map = [&](unsigned i, unsigned j) {
          unsigned ri = sw ? j : i, sj = sw ? i : j;
          if (fr) ri = dim - 1 - ri;
          if (fs) sj = dim - 1 - sj;
          return at(ri, sj);
        };
        const double err = d2(map(0, 0), want[0]) + d2(map(dim - 1, 0), want[1]) +
                           d2(map(dim - 1, dim - 1), want[2]) + d2(map(0, dim - 1), want[3]);
        if (err < 1e-3) {
          std::vector<V3d> out(g.size());
          for (unsigned j = 0; j < dim; ++j)
            for (unsigned i = 0; i < dim; ++i) out[j * dim + i] = map(i, j);
          return out;
        }
      }
  return g;
}

// Legendre interpolation from n_src source nodes to n_tgt GLL nodes
// (FEM-AABB/xml_fld_math.cpp:233-265).
std::vector<double> legendre_interp(unsigned n_src, unsigned n_tgt, bool even_src) {
  const std::vector<double> s = nodes_of(n_src, even_src), t = gll_nodes(static_cast<int>(n_tgt));
  std::vector<double> V(static_cast<size_t>(n_src) * n_src), Vi;
  for (unsigned i = 0; i < n_src; ++i)
    for (unsigned j = 0; j < n_src; ++j) V[i * n_src + j] = legendre_p(static_cast<int>(j), s[i]);
  if (!dense_inverse(V, static_cast<int>(n_src), Vi)) return {};
  std::vector<double> M(static_cast<size_t>(n_tgt) * n_src, 0.0);
  for (unsigned i = 0; i < n_tgt; ++i)
    for (unsigned j = 0; j < n_src; ++j) {
      double acc = 0.0;
      for (unsigned k = 0; k < n_src; ++k) acc += legendre_p(static_cast<int>(k), t[i]) * Vi[k * n_src + j];
      M[i * n_src + j] = acc;
    }
  return M;
}

// Curved face points onto a dim_u x dim_v GLL grid (FEM-AABB/xml_fld_math.cpp:725-787).
std::vector<V3d> resample_face(const CurvedPts& cf, unsigned du, unsigned dv, const std::array<V3d, 4>& corners) {
  const unsigned n = static_cast<unsigned>(std::lround(std::sqrt(static_cast<double>(cf.pts.size()))));
  if (n * n != cf.pts.size() || du == 0 || dv == 0) return {};
  const std::vector<V3d> g = orient_grid(cf.pts, n, corners);
  const std::vector<double> R = legendre_interp(n, du, cf.even), C = legendre_interp(n, dv, cf.even);
  if (R.empty() || C.empty()) return {};
  std::vector<V3d> tmp(static_cast<size_t>(n) * du, V3d{0, 0, 0}), out(static_cast<size_t>(dv) * du, V3d{0, 0, 0});
  for (unsigned j = 0; j < n; ++j)
    for (unsigned i = 0; i < du; ++i)
      for (unsigned k = 0; k < n; ++k) tmp[j * du + i] = tmp[j * du + i] + R[i * n + k] * g[j * n + k];
  for (unsigned i = 0; i < du; ++i)
    for (unsigned j = 0; j < dv; ++j)
      for (unsigned k = 0; k < n; ++k) out[j * du + i] = out[j * du + i] + C[j * n + k] * tmp[k * du + i];
  return out;
}

}  // namespace

int load_xml_fld(const std::string& xml_path, const std::string& fld_path, HostScene& hs, std::string& err,
                 ModalFitter* fitter) {
  std::string raw;
  if (!read_file(xml_path, raw) || raw.empty()) {
    err = "cannot read " + xml_path;
    return HO_ERR_IO;
  }
  const std::string xml = strip_comments(raw);

  // vertices: <V ID=..> x y z </V> inside <VERTEX>, FP32 (missing values 0)
  std::vector<V3d> verts;
  for (const Tag& t : tags(section(xml, "VERTEX"), "V")) {
    const std::string ids = attr(t.header, "ID");
    const int id = ids.empty() ? static_cast<int>(verts.size()) : std::atoi(ids.c_str());
    if (id < 0) continue;
    std::vector<float> v = floats(t.body);
    v.resize(3, 0.f);
    if (id >= static_cast<int>(verts.size())) verts.resize(id + 1, V3d{0, 0, 0});
    verts[id] = V3d{v[0], v[1], v[2]};
  }
  if (verts.empty()) {
    err = "no <VERTEX> entries in " + xml_path;
    return HO_ERR_PARSE;
  }
  auto vertex = [&](int id) { return (id >= 0 && id < static_cast<int>(verts.size())) ? verts[id] : V3d{0, 0, 0}; };

  // default modes: the tag holding the first "NUMMODES" of the file
  std::array<unsigned, 3> default_modes = {1, 1, 1};
  {
    const size_t p = xml.find("NUMMODES");
    if (p != std::string::npos) {
      const size_t a = xml.rfind('<', p), b = xml.find('>', p);
      if (a != std::string::npos && b != std::string::npos && b > a) {
        const std::string m = attr(xml.substr(a, b - a + 1), "NUMMODES");
        if (!m.empty()) default_modes = parse_modes(m);
      }
    }
    if (default_modes[0] == 0) default_modes = {1, 1, 1};
  }

  // edges and quad faces (a face's vertices: its edge loop chained in order)
  std::unordered_map<int, std::array<int, 2>> edges;
  std::unordered_map<long long, int> edge_lookup;
  for (const Tag& t : tags(section(xml, "EDGE"), "E")) {
    const std::vector<int> v = ints(t.body);
    const std::string ids = attr(t.header, "ID");
    if (v.size() >= 2 && !ids.empty()) edges[std::atoi(ids.c_str())] = {v[0], v[1]};
  }
  for (const auto& kv : edges) edge_lookup[edge_key(kv.second[0], kv.second[1])] = kv.first;
  std::unordered_map<int, std::vector<int>> face_verts;
  for (const Tag& t : tags(section(xml, "FACE"), "Q")) {
    const std::vector<int> es = ints(t.body);
    const std::string ids = attr(t.header, "ID");
    if (es.empty() || ids.empty()) continue;
    std::vector<int> fv;
    auto first = edges.find(es[0]);
    if (first != edges.end()) {
      fv = {first->second[0], first->second[1]};
      for (size_t i = 1; i < es.size(); ++i) {
        auto it = edges.find(es[i]);
        if (it == edges.end()) continue;
        const int a = it->second[0], b = it->second[1];
        if (a == fv.back()) fv.push_back(b);
        else if (b == fv.back()) fv.push_back(a);
        else if (a == fv.front()) fv.insert(fv.begin(), b);
        else if (b == fv.front()) fv.insert(fv.begin(), a);
      }
    }
    std::vector<int> uniq;  // first four distinct
    for (int v : fv)
      if (uniq.size() < 4 && std::find(uniq.begin(), uniq.end(), v) == uniq.end()) uniq.push_back(v);
    face_verts[std::atoi(ids.c_str())] = uniq;
  }

  // hexes (<H> then <HEX>), in file order: 6 face ids or 8 vertex ids
  std::vector<Hex> hexes;
  const std::string elem_sec = section(xml, "ELEMENT");
  const std::string& elements = elem_sec.empty() ? xml : elem_sec;
  for (const char* name : {"H", "HEX"}) {
    for (const Tag& t : tags(elements, name)) {
      Hex h;
      const std::string ids = attr(t.header, "ID");
      h.id = ids.empty() ? static_cast<int>(hexes.size()) : std::atoi(ids.c_str());
      const std::vector<int> v = ints(t.body);
      h.faces.fill(-1);
      if (v.size() == 6) {
        std::array<std::vector<int>, 6> fv;
        bool all = true;
        for (int f = 0; f < 6; ++f) {
          h.faces[f] = v[f];
          auto it = face_verts.find(v[f]);
          if (it != face_verts.end()) fv[f] = it->second;
          all = all && fv[f].size() >= 3;
        }
        if (!all) continue;
        // corner c = the vertex shared by the three faces meeting there
        auto common = [&](int a, int b, int c) {
          for (int x : fv[a])
            if (std::count(fv[b].begin(), fv[b].end(), x) && std::count(fv[c].begin(), fv[c].end(), x)) return x;
          return -1;
        };
        static const int kCornerFaces[8][3] = {{0, 1, 4}, {0, 1, 2}, {0, 2, 3}, {0, 3, 4},
                                               {1, 4, 5}, {1, 2, 5}, {2, 3, 5}, {3, 4, 5}};
        bool ok = true;
        for (int c = 0; c < 8; ++c) {
          h.verts[c] = common(kCornerFaces[c][0], kCornerFaces[c][1], kCornerFaces[c][2]);
          ok = ok && h.verts[c] >= 0;
        }
        if (!ok) continue;
      } else if (v.size() == 8) {
        for (int c = 0; c < 8; ++c) h.verts[c] = v[c];
      } else {
        continue;
      }
      for (int e = 0; e < 12; ++e) {
        auto it = edge_lookup.find(edge_key(h.verts[kHexEdge[e][0]], h.verts[kHexEdge[e][1]]));
        h.edges[e] = it != edge_lookup.end() ? it->second : -1;
      }
      hexes.push_back(h);
    }
  }

  // curved edges and faces
  std::unordered_map<int, CurvedPts> cedges, cfaces;
  {
    const std::string cs = section(xml, "CURVED");
    auto read = [&](const Tag& t, const char* idkey, std::unordered_map<int, CurvedPts>& into) {
      const std::string id = attr(t.header, idkey), np = attr(t.header, "NUMPOINTS");
      if (id.empty() || np.empty()) return;
      CurvedPts c;
      c.num = static_cast<unsigned>(std::atoi(np.c_str()));
      c.even = node_type_even(attr(t.header, "TYPE"));
      const std::vector<float> v = floats(t.body);
      for (size_t i = 0; i + 2 < v.size(); i += 3) c.pts.push_back(V3d{v[i], v[i + 1], v[i + 2]});
      if (!c.pts.empty()) into[std::atoi(id.c_str())] = c;
    };
    for (const Tag& t : tags(cs, "E")) read(t, "EDGEID", cedges);
    for (const Tag& t : tags(cs, "F")) read(t, "FACEID", cfaces);
  }

  // field file; an unreadable or empty one leaves the elements without field
  std::string fld;
  if (!read_file(fld_path, fld)) fld.clear();
  std::vector<std::string> field_names;
  {
    const std::string up = upper(fld);
    const size_t p = up.find("FIELDS=\"");
    if (p != std::string::npos) {
      const size_t e = fld.find('"', p + 8);
      if (e != std::string::npos && e > p + 8) field_names = field_list(fld.substr(p + 8, e - p - 8));
    }
    if (field_names.empty()) field_names.push_back("u");
  }
  std::vector<float> coeffs;
  {
    // the <ELEMENTS> payload, else the longest text between two tags
    std::string payload;
    const size_t a = fld.find("<ELEMENTS");
    const size_t gt = a == std::string::npos ? a : fld.find('>', a);
    const size_t b = fld.find("</ELEMENTS>", gt == std::string::npos ? (a == std::string::npos ? 0 : a) : gt);
    if (a != std::string::npos && gt != std::string::npos && b != std::string::npos && b > gt) {
      payload = trim(fld.substr(gt + 1, b - gt - 1));
    } else {
      size_t pos = 0;
      for (;;) {
        const size_t o = fld.find('>', pos);
        if (o == std::string::npos) break;
        const size_t c = fld.find('<', o + 1);
        if (c == std::string::npos) break;
        std::string between = trim(fld.substr(o + 1, c - o - 1));
        if (between.size() > payload.size()) payload.swap(between);
        pos = c + 1;
      }
    }
    // ASCII when the payload starts with a number, else base64 of zlib (or
    // raw deflate, or plain) little-endian FP64 values (FP32 when the byte
    // count is a multiple of 4 only)
    coeffs = floats(payload);
    if (coeffs.empty() && !payload.empty()) {
      const std::vector<uint8_t> dec = base64(payload);
      std::vector<uint8_t> bytes;
      if (!dec.empty()) {
        if (!inflate_any(dec, bytes)) bytes = dec;
        if (bytes.size() % 8 == 0) {
          coeffs.resize(bytes.size() / 8);
          for (size_t i = 0; i < coeffs.size(); ++i) {
            double d;
            std::memcpy(&d, bytes.data() + 8 * i, 8);
            coeffs[i] = static_cast<float>(d);
          }
        } else if (bytes.size() % 4 == 0) {
          coeffs.resize(bytes.size() / 4);
          std::memcpy(coeffs.data(), bytes.data(), bytes.size());
        }
      }
    }
  }

  // composites <C ID=n> H[..] Q[..] P[..] T[..] </C>, read from the raw text
  std::unordered_map<int, std::vector<std::pair<char, int>>> composites;
  for (const Tag& t : tags(raw, "C")) {
    const std::string ids = attr(t.header, "ID");
    if (ids.empty() || t.body.find('<') != std::string::npos) continue;
    const int cid = std::atoi(ids.c_str());
    const std::string& b = t.body;
    for (size_t p = 0; p < b.size(); ++p) {
      const char ty = static_cast<char>(std::toupper(static_cast<unsigned char>(b[p])));
      if (!(ty == 'H' || ty == 'Q' || ty == 'P' || ty == 'T')) continue;
      size_t q = p + 1;
      while (q < b.size() && is_space(b[q])) ++q;
      if (q >= b.size() || b[q] != '[') continue;
      const size_t e = b.find(']', q);
      if (e == std::string::npos) break;
      const std::string inside = b.substr(q + 1, e - q - 1);
      if (trim(inside).find_first_not_of("0123456789-:, ") != std::string::npos) continue;
      std::stringstream ss(trim(inside));
      std::string tok;
      while (std::getline(ss, tok, ',')) {
        int lo, hi;
        id_range(tok, lo, hi);
        for (int v = lo; v <= hi; ++v) composites[cid].push_back({ty, v});
      }
      p = e;
    }
  }

  // expansions <E COMPOSITE="C[..]" NUMMODES|NUMMODESPERDIR=.. FIELDS=..>
  struct Rec {
    char typ;
    int id;
    std::array<unsigned, 3> modes;
    std::vector<std::string> fields;
  };
  std::vector<Rec> recs;
  for (size_t p = raw.find("<E"); p != std::string::npos; p = raw.find("<E", p + 2)) {
    if (p + 2 >= raw.size() || !is_space(raw[p + 2])) continue;
    const size_t gt = raw.find('>', p);
    if (gt == std::string::npos) break;
    const std::string header = raw.substr(p, gt - p + 1);
    const std::string comp = attr(header, "COMPOSITE");
    if (comp.empty()) continue;
    const std::string per = attr(header, "NUMMODESPERDIR"), nm = attr(header, "NUMMODES");
    const auto modes = !per.empty() ? parse_modes(per) : (!nm.empty() ? parse_modes(nm) : default_modes);
    const std::vector<std::string> fl = field_list(attr(header, "FIELDS"));
    const std::string ucomp = upper(comp);
    for (size_t c = ucomp.find("C["); c != std::string::npos; c = ucomp.find("C[", c + 2)) {
      const size_t e = comp.find(']', c);
      if (e == std::string::npos) break;
      const std::string tok = trim(comp.substr(c + 2, e - c - 2));
      if (tok.empty() || tok.find_first_not_of("0123456789-") != std::string::npos) continue;
      int lo, hi;
      id_range(tok, lo, hi);
      for (int cid = lo; cid <= hi; ++cid) {
        auto it = composites.find(cid);
        if (it == composites.end()) continue;
        for (const auto& el : it->second) recs.push_back(Rec{el.first, el.second, modes, fl});
      }
    }
  }
  const bool explicit_exp = !recs.empty();
  if (!explicit_exp)  // every hex, default modes, all fields; non-hex elements follow the hexes
    for (const Hex& h : hexes) recs.push_back(Rec{'H', h.id, default_modes, field_names});
  if (explicit_exp) {  // keep only the hexes that an expansion names
    std::unordered_map<int, bool> named;
    for (const Rec& r : recs)
      if (r.typ == 'H') named[r.id] = true;
    std::vector<Hex> kept;
    for (const Hex& h : hexes)
      if (named.count(h.id)) kept.push_back(h);
    hexes.swap(kept);
  }
  if (hexes.empty()) {
    err = "no hexahedra in " + xml_path + " (this renderer takes hexahedral elements)";
    return HO_ERR_PARSE;
  }
  std::unordered_map<int, size_t> hex_index;
  for (size_t i = 0; i < hexes.size(); ++i) hex_index[hexes[i].id] = i;
  std::unordered_map<int, std::array<unsigned, 3>> hex_modes;
  for (const Rec& r : recs)
    if (r.typ == 'H') {
      auto it = hex_modes.find(r.id);
      if (it == hex_modes.end()) {
        hex_modes[r.id] = r.modes;
      } else {
        for (int a = 0; a < 3; ++a) it->second[a] = std::max(it->second[a], r.modes[a]);
      }
    }

  // coefficient slices: per field, the elements in expansion order, each
  // taking its coefficient count; a hex's field is its first slice
  auto count_of = [](const Rec& r) -> size_t {
    const size_t m0 = r.modes[0], m1 = r.modes[1], m2 = r.modes[2];
    if (r.typ == 'H') return m0 * m1 * m2;
    if (r.typ == 'Q') return m0 * m1;
    size_t c = 0;
    if (r.typ == 'P') {
      for (size_t i = 0; i < m0; ++i) c += m1 * (m2 > i ? m2 - i : 0);
    } else {  // triangle
      for (size_t i = 0; i < m0; ++i) c += m1 > i ? m1 - i : 0;
    }
    return c;
  };
  struct Slice {
    size_t off, cnt;
    std::array<unsigned, 3> modes;
  };
  std::vector<std::vector<Slice>> slices(hexes.size());
  size_t base = 0;
  for (const std::string& fname : field_names) {
    size_t cursor = base;
    for (const Rec& r : recs) {
      const std::vector<std::string>& fl = r.fields.empty() ? field_names : r.fields;
      if (std::find(fl.begin(), fl.end(), fname) == fl.end()) continue;
      const size_t cnt = count_of(r);
      if (cnt == 0) continue;
      if (cursor + cnt > coeffs.size()) break;  // stream exhausted: the rest get no field
      if (r.typ == 'H') {
        auto it = hex_index.find(r.id);
        if (it != hex_index.end()) slices[it->second].push_back(Slice{cursor, cnt, r.modes});
      }
      cursor += cnt;
    }
    base = cursor;
  }

  // geometry: trilinear GLL grid, curved edges, curved faces, modal fit
  HostScene out;
  std::unique_ptr<ModalFitter> host_fit;
  ModalFitter* fit = fitter;
  if (!fit) {
    host_fit = make_host_fitter();
    fit = host_fit.get();
  }
  std::vector<double> soa;
  for (size_t hi = 0; hi < hexes.size(); ++hi) {
    const Hex& h = hexes[hi];
    std::array<unsigned, 3> bm = default_modes;
    auto itm = hex_modes.find(h.id);
    if (itm != hex_modes.end()) bm = itm->second;
    unsigned mo = std::max(bm[0], std::max(bm[1], bm[2]));
    for (int e : h.edges) {
      auto it = cedges.find(e);
      if (it != cedges.end()) mo = std::max(mo, it->second.num);
    }
    for (int f : h.faces) {
      auto it = cfaces.find(f);
      if (it != cfaces.end() && it->second.num > 0)
        mo = std::max(mo, static_cast<unsigned>(std::lround(std::sqrt(static_cast<double>(it->second.num)))));
    }
    const std::array<unsigned, 3> gm = {std::max(bm[0], mo), std::max(bm[1], mo), std::max(bm[2], mo)};
    for (int a = 0; a < 3; ++a)
      if (gm[a] < static_cast<unsigned>(kMinModes) || gm[a] > static_cast<unsigned>(kMaxModes)) {
        err = "hex " + std::to_string(h.id) + ": " + std::to_string(gm[a]) +
              " geometry modes in one direction; this renderer takes 2 to 9";
        return HO_ERR_RANGE;
      }
    const int nx = static_cast<int>(gm[0]), ny = static_cast<int>(gm[1]), nz = static_cast<int>(gm[2]);
    const std::vector<double> rn = gll_nodes(nx), sn = gll_nodes(ny), tn = gll_nodes(nz);
    auto idx = [&](int i, int j, int k) { return (static_cast<size_t>(k) * ny + j) * nx + i; };
    // Z-order corner z = (i, j, k) bits is XML vertex {0,1,3,2,4,5,7,6}[z]
    static const int kZ2Xml[8] = {0, 1, 3, 2, 4, 5, 7, 6};
    V3d corner[8];
    for (int z = 0; z < 8; ++z) corner[z] = vertex(h.verts[kZ2Xml[z]]);
    std::vector<V3d> nodal(static_cast<size_t>(nx) * ny * nz, V3d{0, 0, 0});
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          V3d p{0, 0, 0};
          for (int z = 0; z < 8; ++z) {
            const double w = 0.125 * (1.0 + ((z & 1) ? 1 : -1) * rn[i]) * (1.0 + ((z & 2) ? 1 : -1) * sn[j]) *
                             (1.0 + ((z & 4) ? 1 : -1) * tn[k]);
            p = p + w * corner[z];
          }
          nodal[idx(i, j, k)] = p;
        }
    // curved edges replace the grid's edge lines; local edges 2, 3, 10, 11
    // run against the grid axis
    static const bool kReverse[12] = {false, false, true, true, false, false, false, false, false, false, true, true};
    for (int e = 0; e < 12; ++e) {
      if (h.edges[e] < 0) continue;
      auto ce = cedges.find(h.edges[e]);
      if (ce == cedges.end()) continue;
      bool rev = kReverse[e];
      auto ei = edges.find(h.edges[e]);
      if (ei != edges.end() && ei->second[0] == h.verts[kHexEdge[e][1]] && ei->second[1] == h.verts[kHexEdge[e][0]])
        rev = !rev;
      const unsigned target = (e == 1 || e == 3 || e == 9 || e == 11) ? gm[1]
                              : (e >= 4 && e <= 7)                     ? gm[2]
                                                                       : gm[0];
      const std::vector<V3d> pts = resample_edge(ce->second, target, rev);
      if (pts.size() != target) continue;
      for (unsigned q = 0; q < target; ++q) {
        const int m = static_cast<int>(q);
        size_t at = 0;
        switch (e) {
          case 0: at = idx(m, 0, 0); break;
          case 1: at = idx(nx - 1, m, 0); break;
          case 2: at = idx(m, ny - 1, 0); break;
          case 3: at = idx(0, m, 0); break;
          case 4: at = idx(0, 0, m); break;
          case 5: at = idx(nx - 1, 0, m); break;
          case 6: at = idx(nx - 1, ny - 1, m); break;
          case 7: at = idx(0, ny - 1, m); break;
          case 8: at = idx(m, 0, nz - 1); break;
          case 9: at = idx(nx - 1, m, nz - 1); break;
          case 10: at = idx(m, ny - 1, nz - 1); break;
          default: at = idx(0, m, nz - 1); break;
        }
        nodal[at] = pts[q];
      }
    }
    // curved faces: the offset from the face's grid layer to the resampled
    // surface, blended linearly to zero at the opposite face
    for (int lf = 0; lf < 6; ++lf) {
      if (h.faces[lf] < 0) continue;
      auto cf = cfaces.find(h.faces[lf]);
      if (cf == cfaces.end()) continue;
      const unsigned du = (lf == 2 || lf == 4) ? gm[1] : gm[0];
      const unsigned dv = (lf == 0 || lf == 5) ? gm[1] : gm[2];
      std::array<V3d, 4> fc;
      for (int c = 0; c < 4; ++c) fc[c] = vertex(h.verts[kFaceVerts[lf][c]]);
      const std::vector<V3d> grid = resample_face(cf->second, du, dv, fc);
      if (grid.size() != static_cast<size_t>(du) * dv) continue;
      for (unsigned b = 0; b < dv; ++b)
        for (unsigned a = 0; a < du; ++a) {
          const V3d target = grid[b * du + a];
          const int A = static_cast<int>(a), B = static_cast<int>(b);
          if (lf == 0 || lf == 5) {
            const int kb = lf == 0 ? 0 : nz - 1;
            const V3d diff = target - nodal[idx(A, B, kb)];
            for (int k = 0; k < nz; ++k)
              nodal[idx(A, B, k)] = nodal[idx(A, B, k)] + (0.5 * (lf == 0 ? 1.0 - tn[k] : 1.0 + tn[k])) * diff;
          } else if (lf == 1 || lf == 3) {
            const int jb = lf == 1 ? 0 : ny - 1;
            const V3d diff = target - nodal[idx(A, jb, B)];
            for (int j = 0; j < ny; ++j)
              nodal[idx(A, j, B)] = nodal[idx(A, j, B)] + (0.5 * (lf == 1 ? 1.0 - sn[j] : 1.0 + sn[j])) * diff;
          } else {
            const int ib = lf == 4 ? 0 : nx - 1;
            const V3d diff = target - nodal[idx(ib, A, B)];
            for (int i = 0; i < nx; ++i)
              nodal[idx(i, A, B)] = nodal[idx(i, A, B)] + (0.5 * (lf == 4 ? 1.0 - rn[i] : 1.0 + rn[i])) * diff;
          }
        }
    }
    // modal fit (the fitter may run it later, in a batch)
    const size_t S = static_cast<size_t>(nx) * ny * nz;
    const int64_t goff = static_cast<int64_t>(out.geom.size());
    out.geom.resize(out.geom.size() + 3 * S);
    soa.resize(3 * S);
    for (size_t q = 0; q < S; ++q) {
      soa[q] = nodal[q].x;
      soa[S + q] = nodal[q].y;
      soa[2 * S + q] = nodal[q].z;
    }
    if (!fit->add(soa.data(), 3, nx, ny, nz, &out.geom, goff)) {
      err = fit->error();
      return HO_ERR_PARSE;
    }
    out.goff.push_back(goff);
    for (int q = 0; q < 3; ++q) out.gmodes.push_back(gm[q]);
    for (int v = 0; v < 8; ++v) {
      const V3d p = vertex(h.verts[v]);
      out.corners.push_back(static_cast<float>(p.x));
      out.corners.push_back(static_cast<float>(p.y));
      out.corners.push_back(static_cast<float>(p.z));
    }
    if (!slices[hi].empty()) {
      const Slice& sl = slices[hi].front();
      if (sl.modes[0] < 1 || sl.modes[0] > static_cast<unsigned>(kMaxModes) || sl.modes[1] < 1 ||
          sl.modes[1] > static_cast<unsigned>(kMaxModes) || sl.modes[2] < 1 ||
          sl.modes[2] > static_cast<unsigned>(kMaxModes)) {
        err = "hex " + std::to_string(h.id) + ": field modes outside 1 to 9";
        return HO_ERR_RANGE;
      }
      for (int q = 0; q < 3; ++q) out.fmodes.push_back(sl.modes[q]);
      out.foff.push_back(static_cast<int64_t>(out.field.size()));
      out.field.insert(out.field.end(), coeffs.begin() + sl.off, coeffs.begin() + sl.off + sl.cnt);
    } else {
      for (int q = 0; q < 3; ++q) out.fmodes.push_back(default_modes[q]);
      out.foff.push_back(-1);
    }
  }

  if (!fit->finish()) {
    err = fit->error();
    return HO_ERR_PARSE;
  }
  // append to the caller's scene only when the whole file loaded
  for (size_t e = 0; e < out.goff.size(); ++e) {
    hs.goff.push_back(static_cast<int64_t>(hs.geom.size()) + out.goff[e]);
    hs.foff.push_back(out.foff[e] < 0 ? -1 : static_cast<int64_t>(hs.field.size()) + out.foff[e]);
  }
  hs.geom.insert(hs.geom.end(), out.geom.begin(), out.geom.end());
  hs.field.insert(hs.field.end(), out.field.begin(), out.field.end());
  hs.corners.insert(hs.corners.end(), out.corners.begin(), out.corners.end());
  hs.gmodes.insert(hs.gmodes.end(), out.gmodes.begin(), out.gmodes.end());
  hs.fmodes.insert(hs.fmodes.end(), out.fmodes.begin(), out.fmodes.end());
  return HO_OK;
}

}  // namespace ho
