// VTK XML unstructured-grid (.vtu) scene loader, hexahedra (the reference's
// load_vtu_file, FEM-AABB/vtu_loader.cpp:156-343, restricted to hexes).
//
// What it reads, as the reference does: the first <Points> section's first
// ASCII <DataArray> (or the one named "Points") as x y z float triples; in the
// first <Cells> section the ASCII arrays named "connectivity", "offsets"
// (int, else long long narrowed to int) and "types". Arrays in other formats
// (binary, appended) are skipped. Cell c has offsets[c] - offsets[c-1] points
// (without offsets: 8 for a linear hex, 6 for a wedge, 4 for a quad, none for
// other types); a cell whose range is empty or runs past the connectivity
// ends the cell list. Hexahedra (VTK cell types 12, and 72 and 25 as the
// reference numbers its Lagrange and Bezier hexahedra) become trilinear
// elements whose 8 corners are the cell's first 8 points in the file's order
// (a higher-order VTK cell lists its corners first); wedges (13, 73, 26) become
// linear prisms from their first 6 points and quads (9, 70, 22) linear quads
// from their first 4, each taken in the file's order as the reference takes
// them; a point index outside the point list reads as the origin. No field.
// Other cells are skipped.
//
// The reference leaves the hexes' loader boxes zero-initialised, a point at
// the origin, which its BVH build takes as the element's box; here, as for
// every element, the box is computed from the geometry at BVH build time.
#include <algorithm>
#include <cctype>
#include <cstdint>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "ho_host.h"

namespace ho {

namespace {

bool slurp(const std::string& path, std::string& out) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return false;
  std::ostringstream ss;
  ss << in.rdbuf();
  out = ss.str();
  return !out.empty();
}

// Body of the first <NAME ...>body</NAME> at or after `from`, or empty.
std::string first_section(const std::string& t, const std::string& name) {
  const size_t open = t.find("<" + name);
  if (open == std::string::npos) return {};
  const size_t body = t.find('>', open);
  if (body == std::string::npos) return {};
  const size_t close = t.find("</" + name + ">", body + 1);
  if (close == std::string::npos) return {};
  return t.substr(body + 1, close - body - 1);
}

// Value of key="v" / key='v' at the first occurrence of `key=` in a tag
// header (as the reference matches it: no word boundary), or empty.
std::string attribute(const std::string& tag, const std::string& key) {
  const size_t p = tag.find(key + "=");
  if (p == std::string::npos) return {};
  const size_t q = p + key.size() + 1;
  if (q >= tag.size() || (tag[q] != '"' && tag[q] != '\'')) return {};
  const size_t e = tag.find(tag[q], q + 1);
  return e == std::string::npos ? std::string() : tag.substr(q + 1, e - q - 1);
}

// Numbers of the first ASCII <DataArray> in `sec` whose Name is `name` (any
// name when empty), read as T up to the first token that does not parse as a
// T (an int array stops at a value beyond int's range).
template <class T>
bool ascii_array(const std::string& sec, const std::string& name, std::vector<T>& out) {
  for (size_t at = sec.find("<DataArray"); at != std::string::npos; at = sec.find("<DataArray", at + 1)) {
    const size_t head_end = sec.find('>', at);
    if (head_end == std::string::npos) return false;
    const std::string head = sec.substr(at, head_end - at);
    std::string fmt = attribute(head, "format");
    std::transform(fmt.begin(), fmt.end(), fmt.begin(), [](unsigned char c) { return std::tolower(c); });
    if (!fmt.empty() && fmt != "ascii") continue;
    if (!name.empty() && attribute(head, "Name") != name) continue;
    const size_t end = sec.find("</DataArray>", head_end);
    if (end == std::string::npos) return false;
    std::istringstream in(sec.substr(head_end + 1, end - head_end - 1));
    out.clear();
    T v;
    while (in >> v) out.push_back(v);
    return !out.empty();
  }
  return false;
}

// An integer array as int, or, when not one value parses as int, as long
// long narrowed to int.
bool int_array(const std::string& sec, const std::string& name, std::vector<int>& out) {
  if (ascii_array(sec, name, out)) return true;
  std::vector<long long> wide;
  if (!ascii_array(sec, name, wide)) return false;
  out.assign(wide.size(), 0);
  for (size_t i = 0; i < wide.size(); ++i) out[i] = static_cast<int>(wide[i]);
  return true;
}

constexpr int kVtkHex = 12, kVtkWedge = 13, kVtkQuad = 9;
constexpr int kRefLagrangeHex = 72, kRefBezierHex = 25;
constexpr int kLagrangeWedge = 73, kBezierWedge = 26, kLagrangeQuad = 70, kBezierQuad = 22;

}  // namespace

int load_vtu(const std::string& path, HostScene& hs, std::string& err) {
  std::string text;
  if (!slurp(path, text)) {
    err = "cannot read " + path;
    return HO_ERR_IO;
  }
  const std::string points = first_section(text, "Points");
  if (points.empty()) {
    err = "no <Points> section";
    return HO_ERR_PARSE;
  }
  const std::string cells = first_section(text, "Cells");
  if (cells.empty()) {
    err = "no <Cells> section";
    return HO_ERR_PARSE;
  }
  std::vector<float> xyz;
  if (!ascii_array(points, "", xyz) && !ascii_array(points, "Points", xyz)) {
    err = "no ASCII point coordinates";
    return HO_ERR_PARSE;
  }
  if (xyz.size() % 3 != 0) {
    err = "point coordinates are not triples";
    return HO_ERR_PARSE;
  }
  std::vector<int> conn, offsets, types;
  if (!int_array(cells, "connectivity", conn)) {
    err = "no ASCII cell connectivity";
    return HO_ERR_PARSE;
  }
  int_array(cells, "offsets", offsets);
  if (!ascii_array(cells, "types", types)) {
    err = "no ASCII cell types";
    return HO_ERR_PARSE;
  }
  const int n_points = static_cast<int>(xyz.size() / 3);
  HostScene out;
  HostPrims& prims = out.prims;
  auto point = [&](int p, int a) { return p >= 0 && p < n_points ? xyz[3 * size_t(p) + a] : 0.0f; };
  size_t cursor = 0;
  for (size_t c = 0; c < types.size(); ++c) {
    const int type = types[c];
    int count = 0;
    if (c < offsets.size()) {
      count = offsets[c] - (c == 0 ? 0 : offsets[c - 1]);
    } else {
      count = type == kVtkHex ? 8 : type == kVtkWedge ? 6 : type == kVtkQuad ? 4 : 0;
    }
    if (count <= 0 || cursor + static_cast<size_t>(count) > conn.size()) break;
    const bool hex = type == kVtkHex || type == kRefLagrangeHex || type == kRefBezierHex;
    if (hex && count >= 8) {
      for (int v = 0; v < 8; ++v) {
        for (int a = 0; a < 3; ++a) out.corners.push_back(point(conn[cursor + v], a));
      }
      for (int a = 0; a < 3; ++a) {
        out.gmodes.push_back(0);
        out.fmodes.push_back(0);
      }
      out.goff.push_back(-1);
      out.foff.push_back(-1);
    }
    const bool wedge = type == kVtkWedge || type == kLagrangeWedge || type == kBezierWedge;
    const bool quad = type == kVtkQuad || type == kLagrangeQuad || type == kBezierQuad;
    if ((wedge && count >= 6) || (quad && count >= 4)) {
      const int nv = wedge ? 6 : 4;
      prims.kind.push_back(wedge ? 0 : 1);
      for (int v = 0; v < 6; ++v)
        for (int a = 0; a < 3; ++a) prims.verts.push_back(v < nv ? point(conn[cursor + v], a) : 0.0f);
      for (int a = 0; a < 3; ++a) {
        prims.gmodes.push_back(0);
        prims.fmodes.push_back(0);
      }
      prims.goff.push_back(-1);
      prims.foff.push_back(-1);
    }
    cursor += static_cast<size_t>(count);
  }
  if (out.goff.empty() && prims.size() == 0) {
    err = "no hexahedron, wedge or quad cells in " + path;
    return HO_ERR_PARSE;
  }
  // append only when the whole file loaded
  hs.corners.insert(hs.corners.end(), out.corners.begin(), out.corners.end());
  hs.gmodes.insert(hs.gmodes.end(), out.gmodes.begin(), out.gmodes.end());
  hs.fmodes.insert(hs.fmodes.end(), out.fmodes.begin(), out.fmodes.end());
  hs.goff.insert(hs.goff.end(), out.goff.begin(), out.goff.end());
  hs.foff.insert(hs.foff.end(), out.foff.begin(), out.foff.end());
  HostPrims& hp = hs.prims;
  hp.kind.insert(hp.kind.end(), prims.kind.begin(), prims.kind.end());
  hp.verts.insert(hp.verts.end(), prims.verts.begin(), prims.verts.end());
  hp.gmodes.insert(hp.gmodes.end(), prims.gmodes.begin(), prims.gmodes.end());
  hp.fmodes.insert(hp.fmodes.end(), prims.fmodes.begin(), prims.fmodes.end());
  hp.goff.insert(hp.goff.end(), prims.goff.begin(), prims.goff.end());
  hp.foff.insert(hp.foff.end(), prims.foff.begin(), prims.foff.end());
  return HO_OK;
}

}  // namespace ho
