"""The loader's modal fit on the GPU (HO_OPT_GPU_FIT = 1) against the host
fit (= 0): the same FP64 sums in the same order, so the FP32 coefficients
agree to a few units in the last place (the GPU and host compilers contract
multiply-adds differently). On the generated fixtures and on a generated
20^3-hex mesh at 9 modes per direction, where the fit is most of the load;
the two load times are printed."""
from __future__ import annotations

import sys
import time

import numpy as np
import pytest

import horender as hr
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

NEK = GOLDEN / "nektar"


def load(xml, fld, gpu_fit):
    ctx = hr.Context(0)
    ctx.set_option(hr.OPT_GPU_FIT, gpu_fit)
    t0 = time.perf_counter()
    ctx.load_xml_fld(str(xml), str(fld))
    dt = time.perf_counter() - t0
    assert ctx.get_option(hr.OPT_LAST_FIT_GPU) == gpu_fit
    return ctx, dt


def compare(xml, fld):
    a, ta = load(xml, fld, 0)
    b, tb = load(xml, fld, 1)
    with a, b:
        sa, sb = a.get_scene(), b.get_scene()
        for k in ("geom_modes", "geom_offsets", "field", "corners"):
            assert np.array_equal(sa[k], sb[k]), k
        scale = float(np.abs(sa["geom"]).max())
        err = float(np.abs(sa["geom"] - sb["geom"]).max())
        assert err <= 4e-7 * scale, (err, scale)
    return ta, tb, sa["geom"].size


@pytest.mark.parametrize("name", ["nek_faces", "nek_verts", "nek_raw", "nek_fp32", "nek_origin"])
def test_gpu_fit_equals_host_fit_on_fixtures(name):
    compare(NEK / f"{name}.xml", NEK / f"{name}.fld")


def test_gpu_fit_on_a_large_mesh(tmp_path):
    sys.path.insert(0, str(GOLDEN))
    from make_nektar import Mesh

    rng = np.random.default_rng(7)
    m = Mesh(20, 20, 20, 0.05, rng)
    eids = sorted(val[0] for val in m.edges.values())
    ce = [(int(e), 5, "GaussLobattoLegendre") for e in rng.choice(eids, size=200, replace=False)]
    n = len(m.hexes)
    tail = {"composite": ["    <COMPOSITE>", f'      <C ID="0"> H[0-{n - 1}] </C>', "    </COMPOSITE>",
                          "    <DOMAIN> C[0] </DOMAIN>"],
            "expansions": ["  <EXPANSIONS>", '    <E COMPOSITE="C[0]" NUMMODES="9" TYPE="MODIFIED" FIELDS="u" />',
                           "  </EXPANSIONS>"]}
    xml = tmp_path / "big.xml"
    xml.write_text(m.xml("faces", ce, [], tail))
    ta, tb, size = compare(xml, tmp_path / "absent.fld")  # geometry only
    print(f"{n} hexes at 9 modes ({size} coefficients): load with host fit {ta:.3f} s, with GPU fit {tb:.3f} s")
