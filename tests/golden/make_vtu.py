"""Generates the VTU loader fixtures under tests/golden/vtu: small ASCII VTK
XML unstructured grids (seeded, made here, not taken from any data set) and
vtu_ref.npz, what the reference's own loader (load_vtu_file,
FEM-AABB/vtu_loader.cpp:156-343, compiled into oracle/_ref/libref.so by
oracle/build_ref.sh) made of each: whether it succeeded, how many hexahedra,
prisms and quads it added, and their vertices.

Cases:
  grid      3x2x2 jittered linear hexes (type 12), Int32 arrays, a binary
            DataArray ahead of the ASCII points, PointData/CellData sections
  mixed     hexes of types 12, 72 (27 points) and 25 (27 points), a wedge, a
            quad and a tetrahedron (skipped), Int64 connectivity/offsets
  nooffsets no offsets array: counts guessed for types 12/13/9; a type-10 cell
            gets none and ends the cell list
  badrange  the offsets of the 4th cell run past the connectivity
  badindex  point indices -1 and beyond the point list (read as the origin)
  wide      a connectivity value beyond int's range: the int parse stops
            there, the long long retry is not taken, later cells fall off
  nohex     wedges and quads only

Run: python tests/golden/make_vtu.py (needs oracle/_ref/libref.so).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "vtu"
sys.path.insert(0, str(HERE.parent))


def grid_points(nx, ny, nz, rng, jitter=0.08):
    g = np.stack(np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij"), -1)
    p = g.transpose(2, 1, 0, 3).reshape(-1, 3).astype(np.float64)  # i fastest
    p /= max(nx, ny, nz)
    p += rng.uniform(-jitter, jitter, p.shape) / max(nx, ny, nz)
    return p


def grid_hexes(nx, ny, nz):
    def pid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)

    cells = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                cells.append([pid(i, j, k), pid(i + 1, j, k), pid(i + 1, j + 1, k), pid(i, j + 1, k),
                              pid(i, j, k + 1), pid(i + 1, j, k + 1), pid(i + 1, j + 1, k + 1), pid(i, j + 1, k + 1)])
    return cells


def fmt_points(p, style):
    if style == "sci":
        return " ".join(f"{v:.8e}" for v in p.reshape(-1))
    return "\n".join(" ".join(f"{v:.9g}" for v in row) for row in p.reshape(-1, 3))


def array(name, typ, values, fmt="ascii", extra=""):
    body = " ".join(str(v) for v in values)
    name_attr = f' Name="{name}"' if name else ""
    return f'        <DataArray type="{typ}"{name_attr}{extra} format="{fmt}">\n          {body}\n        </DataArray>'


def vtu(points_text, cells_xml, n_points, n_cells, point_prefix="", with_data=False):
    lines = ['<?xml version="1.0"?>',
             '<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">',
             "  <UnstructuredGrid>", f'    <Piece NumberOfPoints="{n_points}" NumberOfCells="{n_cells}">']
    if with_data:
        lines += ["      <PointData Scalars=\"u\">",
                  array("u", "Float32", ["0.5"] * n_points), "      </PointData>",
                  "      <CellData>", array("id", "Int32", list(range(n_cells))), "      </CellData>"]
    lines += ["      <Points>"]
    if point_prefix:
        lines.append(point_prefix)
    lines += ['        <DataArray type="Float32" Name="Points" NumberOfComponents="3" format="ascii">',
              "          " + points_text, "        </DataArray>", "      </Points>",
              "      <Cells>", cells_xml, "      </Cells>", "    </Piece>", "  </UnstructuredGrid>", "</VTKFile>", ""]
    return "\n".join(lines)


def cells_xml(conn, offsets, types, ctype="Int32", otype="Int32"):
    parts = [array("connectivity", ctype, conn)]
    if offsets is not None:
        parts.append(array("offsets", otype, offsets))
    parts.append(array("types", "UInt8", types))
    return "\n".join(parts)


def flat(cells):
    conn, off, c = [], [], 0
    for cell in cells:
        conn += list(cell)
        c += len(cell)
        off.append(c)
    return conn, off


def make_cases(rng):
    cases = {}
    # grid
    p = grid_points(3, 2, 2, rng)
    hexes = grid_hexes(3, 2, 2)
    conn, off = flat(hexes)
    binary = '        <DataArray type="Float32" Name="Points" NumberOfComponents="3" format="binary">AAAA</DataArray>'
    cases["grid"] = vtu(fmt_points(p, "g"), cells_xml(conn, off, [12] * len(hexes)), len(p), len(hexes),
                        point_prefix=binary, with_data=True)
    # mixed: corner points first, then extra (mid-edge etc.) points for the 27-point cells
    p = grid_points(2, 2, 1, rng)
    n0 = len(p)
    extra = rng.uniform(0.0, 1.0, (40, 3))
    p = np.concatenate([p, extra])
    hexes = grid_hexes(2, 2, 1)
    mids = list(range(n0, n0 + 19))
    cells = [hexes[0], hexes[1] + mids, hexes[2] + mids[::-1], [0, 1, 3, 9, 10, 12], [0, 1, 4, 3], [0, 1, 3, 9],
             hexes[3]]
    types = [12, 72, 25, 13, 9, 10, 12]
    conn, off = flat(cells)
    cases["mixed"] = vtu(fmt_points(p, "sci"), cells_xml(conn, off, types, "Int64", "Int64"), len(p), len(cells))
    # nooffsets
    p = grid_points(2, 1, 1, rng)
    hexes = grid_hexes(2, 1, 1)
    cells = [hexes[0], [0, 1, 3, 6, 7, 9], [0, 1, 4, 3], hexes[1], [0, 1, 3, 6], hexes[0]]
    types = [12, 13, 9, 12, 10, 12]
    conn, _ = flat(cells)
    cases["nooffsets"] = vtu(fmt_points(p, "g"), cells_xml(conn, None, types), len(p), len(cells))
    # badrange
    p = grid_points(3, 1, 1, rng)
    hexes = grid_hexes(3, 1, 1) + [grid_hexes(3, 1, 1)[0]]
    conn, off = flat(hexes)
    off[3] = len(conn) + 5
    cases["badrange"] = vtu(fmt_points(p, "g"), cells_xml(conn, off, [12] * 4), len(p), 4)
    # badindex
    p = grid_points(2, 1, 1, rng)
    hexes = grid_hexes(2, 1, 1)
    hexes[1][2] = -1
    hexes[1][6] = len(p) + 3
    conn, off = flat(hexes)
    cases["badindex"] = vtu(fmt_points(p, "g"), cells_xml(conn, off, [12, 12]), len(p), 2)
    # wide
    p = grid_points(3, 1, 1, rng)
    hexes = grid_hexes(3, 1, 1)
    hexes[1][5] = 3_000_000_000
    conn, off = flat(hexes)
    cases["wide"] = vtu(fmt_points(p, "g"), cells_xml(conn, off, [12] * 3, "Int64", "Int64"), len(p), 3)
    # nohex
    p = grid_points(1, 1, 1, rng)
    cells = [[0, 1, 2, 4, 5, 6], [0, 2, 3, 4, 6, 7], [0, 1, 3, 2]]
    conn, off = flat(cells)
    cases["nohex"] = vtu(fmt_points(p, "g"), cells_xml(conn, off, [13, 13, 9]), len(p), 3)
    return cases


def main():
    import oracle_bind as ob

    if not ob.ref_available():
        sys.exit("oracle/_ref/libref.so not built (oracle/build_ref.sh)")
    OUT.mkdir(exist_ok=True)
    rng = np.random.default_rng(11)
    ref = {}
    for name, text in make_cases(rng).items():
        path = OUT / f"{name}.vtu"
        path.write_text(text)
        try:
            rs = ob.RefScene(vtu=str(path))
            ok, counts, verts = True, rs.vtu_counts.copy(), rs.arrays().verts
            prisms, quads = rs.vtu_prisms, rs.vtu_quads
        except RuntimeError:
            ok, counts, verts = False, np.zeros(3, np.int64), np.zeros((0, 8, 3), np.float32)
            prisms, quads = np.zeros((0, 6, 3), np.float32), np.zeros((0, 4, 3), np.float32)
        ref[f"{name}_ok"] = np.array(ok)
        ref[f"{name}_counts"] = counts
        ref[f"{name}_verts"] = verts
        ref[f"{name}_prisms"] = prisms
        ref[f"{name}_quads"] = quads
        print(name, "ok" if ok else "failed", "hex/prism/quad", counts.tolist())
    np.savez_compressed(OUT / "vtu_ref.npz", **ref)


if __name__ == "__main__":
    main()
