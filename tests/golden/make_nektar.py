"""Writes small Nektar++-format meshes (XML) and fields (FLD) that exercise the
loader's format paths, and records what the reference's own loader
(oracle/_ref/libref.so, built from the reference sources by
oracle/build_ref.sh) makes of each. Run in a checkout that has the reference
sources:

    python tests/golden/make_nektar.py

Everything here is generated: a structured grid of hexes on [0,1]^3 bent by a
smooth map F that fixes the origin (the reference's vertex scan also matches
<VERTEX> and <VARIABLES>, which leaves vertex 0 at the origin, so vertex 0 is
placed there), with curved edges and faces sampled from F.

  nek_faces   12 hexes given by face ids; curved edges (GLL and evenly spaced
              points, random edge directions), curved faces (evenly spaced,
              grids written in random orientations); NUMMODES=5; one smooth
              field u (random modal coefficients decaying as 0.4^(i+j+k)),
              base64 + zlib FP64.
  nek_verts   8 hexes given by vertex ids; two composites with
              NUMMODESPERDIR="4,5,6" and NUMMODES="3"; fields u,v (the hex's
              field is u); ASCII coefficients; a stale curved face inside an
              XML comment.
  nek_raw     2 hexes, no expansion naming an existing composite (all hexes,
              default modes 6); base64 of raw deflate FP64.
  nek_fp32    3 hexes, NUMMODES=3, 81 coefficients as plain base64 FP32 (the
              byte count is not a multiple of 8).
  nek_origin  1 straight hex whose vertex 0 is NOT at the origin, no reference
              output: the product reads the file's vertex 0, the reference
              sets it to the origin (documented difference).
Each <name>.npz holds the reference loader's arrays.
"""
from __future__ import annotations

import base64
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "nektar"
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "tests"))


def gll(n: int) -> np.ndarray:
    if n == 2:
        return np.array([-1.0, 1.0])
    P = np.polynomial.legendre.Legendre.basis(n - 1)
    inner = np.sort(P.deriv().roots().real)
    return np.concatenate([[-1.0], inner, [1.0]])


def even(n: int) -> np.ndarray:
    return np.linspace(-1.0, 1.0, n)


def bend(p: np.ndarray, amp: float) -> np.ndarray:
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    s = np.sin
    d = np.stack([s(np.pi * y) * s(np.pi * z) + 0.5 * s(2 * np.pi * x) * y,
                  s(np.pi * z) * s(np.pi * x) + 0.5 * s(2 * np.pi * y) * z,
                  s(np.pi * x) * s(np.pi * y) + 0.5 * s(2 * np.pi * z) * x], -1)
    return p + amp * d


def fmt(v) -> str:
    return " ".join(f"{float(a):.9g}" for a in np.ravel(v))


class Mesh:
    """Structured nx x ny x nz hex grid; local vertex order 0-3 bottom
    counter-clockwise, 4-7 top; faces 0 bottom, 1 front (y-), 2 right (x+),
    3 back (y+), 4 left (x-), 5 top."""

    def __init__(self, nx, ny, nz, amp, rng, offset=(0.0, 0.0, 0.0)):
        self.rng = rng
        self.amp = amp
        self.n = (nx, ny, nz)
        g = np.stack(np.meshgrid(np.linspace(0, 1, nx + 1), np.linspace(0, 1, ny + 1), np.linspace(0, 1, nz + 1),
                                 indexing="ij"), -1)
        self.pos = bend(g.reshape(-1, 3), amp) + np.asarray(offset)

        def vid(i, j, k):
            return (i * (ny + 1) + j) * (nz + 1) + k

        self.vid = vid
        self.edges: dict[tuple[int, int], tuple[int, int, int]] = {}  # key -> (id, v0, v1)
        self.faces: dict[frozenset, tuple[int, list[int]]] = {}
        self.hexes = []
        for i in range(nx):
            for j in range(ny):
                for k in range(nz):
                    v = [vid(i, j, k), vid(i + 1, j, k), vid(i + 1, j + 1, k), vid(i, j + 1, k),
                         vid(i, j, k + 1), vid(i + 1, j, k + 1), vid(i + 1, j + 1, k + 1), vid(i, j + 1, k + 1)]
                    fl = []
                    for fv in ([0, 1, 2, 3], [0, 1, 5, 4], [1, 2, 6, 5], [3, 2, 6, 7], [0, 3, 7, 4], [4, 5, 6, 7]):
                        fl.append(self.face([v[a] for a in fv]))
                    self.hexes.append((v, fl))

    def edge(self, a, b):
        key = (min(a, b), max(a, b))
        if key not in self.edges:
            v0, v1 = (a, b) if self.rng.random() < 0.5 else (b, a)
            self.edges[key] = (len(self.edges), v0, v1)
        return self.edges[key][0]

    def face(self, fv):
        key = frozenset(fv)
        if key not in self.faces:
            loop = [self.edge(fv[q], fv[(q + 1) % 4]) for q in range(4)]
            r = int(self.rng.integers(4))
            loop = loop[r:] + loop[:r]
            self.faces[key] = (len(self.faces), list(fv), loop)
        return self.faces[key][0]

    # positions in the unbent parameter space, for sampling curved entities
    def param(self, v):
        nx, ny, nz = self.n
        k = v % (nz + 1)
        j = (v // (nz + 1)) % (ny + 1)
        i = v // ((ny + 1) * (nz + 1))
        return np.array([i / nx, j / ny, k / nz])

    def xml(self, elem_mode, curved_edges, curved_faces, tail, vertex_lines=None, comment=""):
        L = ['<?xml version="1.0" encoding="utf-8" ?>', "<NEKTAR>", '  <GEOMETRY DIM="3" SPACE="3">', "    <VERTEX>"]
        if vertex_lines is None:
            vertex_lines = [f'      <V ID="{q}"> {fmt(p)} </V>' for q, p in enumerate(self.pos)]
        L += vertex_lines
        L += ["    </VERTEX>", "    <EDGE>"]
        for (_, v0, v1), eid in sorted(((val, val[0]) for val in self.edges.values()), key=lambda t: t[1]):
            L.append(f'      <E ID="{eid}"> {v0} {v1} </E>')
        L += ["    </EDGE>", "    <FACE>"]
        for fid, _, loop in sorted(self.faces.values(), key=lambda t: t[0]):
            L.append(f'      <Q ID="{fid}"> {" ".join(map(str, loop))} </Q>')
        L += ["    </FACE>", "    <ELEMENT>"]
        for h, (v, fl) in enumerate(self.hexes):
            body = fl if elem_mode == "faces" else v
            L.append(f'      <H ID="{h}"> {" ".join(map(str, body))} </H>')
        L += ["    </ELEMENT>"]
        L += tail["composite"]
        L += ["    <CURVED>"]
        cid = 0
        for eid, npts, typ in curved_edges:
            (v0, v1) = next((val[1], val[2]) for val in self.edges.values() if val[0] == eid)
            nodes = gll(npts) if typ.startswith("Gauss") else even(npts)
            a, b = self.param(v0), self.param(v1)
            pts = bend(a[None] + (nodes[:, None] + 1) / 2 * (b - a)[None], self.amp)
            L.append(f'      <E ID="{cid}" EDGEID="{eid}" NUMPOINTS="{npts}" TYPE="{typ}"> {fmt(pts)} </E>')
            cid += 1
        for fid, npts in curved_faces:
            _, fv, _ = next(val for val in self.faces.values() if val[0] == fid)
            p0, p1, p3 = self.param(fv[0]), self.param(fv[1]), self.param(fv[3])
            u = even(npts)
            grid = np.array([[p0 + (a + 1) / 2 * (p1 - p0) + (b + 1) / 2 * (p3 - p0) for a in u] for b in u])
            pts = bend(grid, self.amp)  # [b][a], a fastest
            # write in one of the 8 orientations
            o = int(self.rng.integers(8))
            if o & 1:
                pts = pts[:, ::-1]
            if o & 2:
                pts = pts[::-1]
            if o & 4:
                pts = pts.transpose(1, 0, 2)
            L.append(f'      <F ID="{cid}" FACEID="{fid}" NUMPOINTS="{npts * npts}" TYPE="PolyEvenlySpaced"> '
                     f'{fmt(pts)} </F>')
            cid += 1
        L += [comment, "    </CURVED>", "  </GEOMETRY>"]
        L += tail["expansions"]
        L += ["  <CONDITIONS>", "    <VARIABLES>", '      <V ID="0"> u </V>', "    </VARIABLES>", "  </CONDITIONS>",
              "</NEKTAR>"]
        return "\n".join(L) + "\n"


def fld_text(fields: str, payload: str, compressed: str | None) -> str:
    attrs = f'FIELDS="{fields}" BASIS="Modified_A,Modified_A,Modified_A" SHAPE="Hexahedron"'
    if compressed:
        attrs += f' COMPRESSED="{compressed}"'
    return ('<?xml version="1.0" encoding="utf-8" ?>\n<NEKTAR>\n'
            f'  <ELEMENTS {attrs}>{payload}</ELEMENTS>\n</NEKTAR>\n')


def main():
    import oracle_bind as ob

    if not ob.ref_available():
        raise SystemExit("oracle/_ref/libref.so is missing: run oracle/build_ref.sh first")
    OUT.mkdir(exist_ok=True)
    rng = np.random.default_rng(20261203)
    cases = {}

    # nek_faces
    m = Mesh(3, 2, 2, 0.06, rng)
    eids = sorted(val[0] for val in m.edges.values())
    ce = [(e, int(rng.integers(3, 7)), "GaussLobattoLegendre" if rng.random() < 0.5 else "PolyEvenlySpaced")
          for e in rng.choice(eids, size=20, replace=False)]
    fids = sorted(val[0] for val in m.faces.values())
    cf = [(f, int(rng.integers(3, 6))) for f in rng.choice(fids, size=10, replace=False)]
    tail = {"composite": ["    <COMPOSITE>", f'      <C ID="0"> H[0-{len(m.hexes) - 1}] </C>', "    </COMPOSITE>",
                          "    <DOMAIN> C[0] </DOMAIN>"],
            "expansions": ["  <EXPANSIONS>", '    <E COMPOSITE="C[0]" NUMMODES="5" TYPE="MODIFIED" FIELDS="u" />',
                           "  </EXPANSIONS>"]}
    # smooth field: modal coefficients (i fastest) decaying as 0.4^(i+j+k)
    i, j, k = np.meshgrid(np.arange(5), np.arange(5), np.arange(5), indexing="ij")
    decay = (0.4 ** (i + j + k)).transpose(2, 1, 0).reshape(-1)
    coef = (rng.standard_normal((len(m.hexes), 125)) * decay).reshape(-1)
    payload = base64.b64encode(zlib.compress(coef.astype("<f8").tobytes())).decode()
    cases["nek_faces"] = (m.xml("faces", ce, cf, tail), fld_text("u", payload, "B64Z-LittleEndian"))

    # nek_verts
    m = Mesh(2, 2, 2, 0.05, rng)
    eids = sorted(val[0] for val in m.edges.values())
    ce = [(e, 4, "PolyEvenlySpaced") for e in rng.choice(eids, size=8, replace=False)]
    tail = {"composite": ["    <COMPOSITE>", '      <C ID="0"> H[0-3] </C>', '      <C ID="1"> H[4,5,6-7] </C>',
                          "    </COMPOSITE>", "    <DOMAIN> C[0-1] </DOMAIN>"],
            "expansions": ["  <EXPANSIONS>",
                           '    <E COMPOSITE="C[0]" NUMMODESPERDIR="4,5,6" TYPE="MODIFIED" FIELDS="u,v" />',
                           '    <E COMPOSITE="C[1]" NUMMODES="3" TYPE="MODIFIED" FIELDS="u,v" />', "  </EXPANSIONS>"]}
    n = 2 * (4 * 120 + 4 * 27)
    coef = rng.standard_normal(n)
    comment = ('      <!--\n      <F ID="99" FACEID="0" NUMPOINTS="9" TYPE="PolyEvenlySpaced"> '
               '0 0 0 1 0 0 1 1 0 0 1 0 0.5 0 0 1 0.5 0 0.5 1 0 0 0.5 0 0.5 0.5 0.7 </F>\n      -->')
    cases["nek_verts"] = (m.xml("verts", ce, [], tail, comment=comment),
                          fld_text("u,v", " " + " ".join(f"{c:.9g}" for c in coef) + " ", None))

    # nek_raw
    m = Mesh(2, 1, 1, 0.04, rng)
    tail = {"composite": ["    <COMPOSITE>", '      <C ID="0"> H[0-1] </C>', "    </COMPOSITE>"],
            "expansions": ["  <EXPANSIONS>", '    <E COMPOSITE="C[9]" NUMMODES="6" TYPE="MODIFIED" FIELDS="u" />',
                           "  </EXPANSIONS>"]}
    coef = rng.standard_normal(2 * 216)
    co = zlib.compressobj(9, zlib.DEFLATED, -15)
    raw = co.compress(coef.astype("<f8").tobytes()) + co.flush()
    cases["nek_raw"] = (m.xml("verts", [], [], tail), fld_text("u", base64.b64encode(raw).decode(), None))

    # nek_fp32
    m = Mesh(3, 1, 1, 0.05, rng)
    fids = sorted(val[0] for val in m.faces.values())
    cf = [(f, 3) for f in fids[:4]]
    tail = {"composite": ["    <COMPOSITE>", '      <C ID="0"> H[0-2] </C>', "    </COMPOSITE>"],
            "expansions": ["  <EXPANSIONS>", '    <E COMPOSITE="C[0]" NUMMODES="3" TYPE="MODIFIED" FIELDS="u" />',
                           "  </EXPANSIONS>"]}
    coef = rng.standard_normal(81).astype("<f4")
    cases["nek_fp32"] = (m.xml("faces", [], cf, tail), fld_text("u", base64.b64encode(coef.tobytes()).decode(), None))

    # nek_origin (no reference output)
    m = Mesh(1, 1, 1, 0.0, rng, offset=(2.0, -1.0, 0.5))
    tail = {"composite": ["    <COMPOSITE>", '      <C ID="0"> H[0] </C>', "    </COMPOSITE>"],
            "expansions": ["  <EXPANSIONS>", '    <E COMPOSITE="C[0]" NUMMODES="2" TYPE="MODIFIED" FIELDS="u" />',
                           "  </EXPANSIONS>"]}
    cases["nek_origin"] = (m.xml("verts", [], [], tail), fld_text("u", " ".join(["0.5"] * 8), None))

    for name, (xml, fld) in cases.items():
        (OUT / f"{name}.xml").write_text(xml)
        (OUT / f"{name}.fld").write_text(fld)
        if name == "nek_origin":
            continue
        a = ob.RefScene(xml=str(OUT / f"{name}.xml"), fld=str(OUT / f"{name}.fld")).arrays()
        np.savez_compressed(OUT / f"{name}.npz", geom_modes=a.geom_modes, geom_offset=a.geom_offset, geom=a.geom,
                            field_modes=a.field_modes, field_offset=a.field_offset, field=a.field, verts=a.verts)
        print(name, "hexes", a.n, "geom", a.geom.size, "field", a.field.size)


if __name__ == "__main__":
    main()
