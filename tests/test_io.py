"""Scenario front end (config file, XML scenarios, legacy-VTK masks) and VTS output, on the CPU.

The reference's own scenario files are read from their committed copies under
tests/golden/scenarios (the pipe mask gzip-compressed, checked against the SHA-256 of the
reference's file); everything else uses files written here in the same formats.
"""
import base64
import gzip
import hashlib
import struct
import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np
import pytest

from lbm_gb300 import io
from lbm_gb300 import scenario as S

REF_SCEN = Path(__file__).resolve().parent / "golden" / "scenarios"


def reference_scenarios(dest: Path) -> Path:
    """The reference's build/scenarios files laid out as the reference runs them (from build/:
    scenarios/<name>.xml, and scenarios/pipe.vtk, which pipe.xml names relative to the working
    directory) under dest; returns dest. The pipe mask is checked against the reference's hash."""
    sc = dest / "scenarios"
    sc.mkdir(parents=True, exist_ok=True)
    for name in ("cavity.xml", "pipe.xml", "shearflow.xml", "step.xml"):
        (sc / name).write_bytes((REF_SCEN / name).read_bytes())
    raw = gzip.decompress((REF_SCEN / "pipe.vtk.gz").read_bytes())
    assert hashlib.sha256(raw).hexdigest() == (REF_SCEN / "pipe.vtk.sha256").read_text().strip()
    (sc / "pipe.vtk").write_bytes(raw)
    return dest

STEP_XML = """<?xml version="1.0" ?>
<scenario name="Backward step">
    <!-- a comment, ignored -->
    <domain xl="12" yl="10" zl="18">
        <boundary extent="7 13 0 11 0 0"   condition="inflow" vx="0" vy="0" vz="0.04" />
        <boundary extent="0 6 0 11 0 9" condition="noslip" />
        <boundary extent="zmax" condition="outflow" rho-ref="1.0" />
        <boundary extent="y0"  condition="noslip" />
        <boundary extent="ymax"   condition="noslip" />
        <boundary extent="x0"  condition="noslip" />
        <boundary extent="xmax"   condition="noslip" />
    </domain>
</scenario>
"""

SHEAR_XML = """<?xml version="1.0" ?>
<scenario name="Shear">
    <domain xl="6" yl="7" zl="14">
        <boundary extent="z0" condition="pressure" rho-in="1.004" />
        <boundary extent="zmax" condition="outflow" />
        <boundary extent="x0" condition="freeslip" />
        <boundary extent="xmax" condition="freeslip" />
        <boundary extent="y0" condition="noslip" />
        <boundary extent="ymax" condition="noslip" />
    </domain>
</scenario>
"""


def write_mask_vtk(path, mask, origin=(-3.5, 1.25, 0.0), spacing=(2.0, 0.5, 0.5)):
    """mask[z, y, x] (1 fluid, 0 solid) as an ASCII legacy-VTK STRUCTURED_POINTS file."""
    zl, yl, xl = mask.shape
    vals = " ".join(str(int(v)) for v in mask.reshape(-1))
    Path(path).write_text(
        "# vtk DataFile Version 2.0\nmask written by the tests\nASCII\n\nDATASET STRUCTURED_POINTS\n"
        f"DIMENSIONS {xl} {yl} {zl}\n\nORIGIN {origin[0]} {origin[1]} {origin[2]}\n"
        f"SPACING {spacing[0]} {spacing[1]} {spacing[2]}\n\nPOINT_DATA {xl * yl * zl}\n"
        "SCALARS inputfluidMask unsigned_char\nLOOKUP_TABLE default\n\n" + vals + "\n")


def tube_mask(xl, yl, zl, r):
    z, y = np.meshgrid(np.arange(zl) - (zl - 1) / 2, np.arange(yl) - (yl - 1) / 2, indexing="ij")
    inside = (y * y + z * z) <= r * r
    return np.repeat(inside[:, :, None], xl, axis=2).astype(np.uint8)


def test_config_file_and_command_line(tmp_path):
    cfg = tmp_path / "config.cfg"
    out = tmp_path / "out"
    cfg.write_text("# comment\ncollision-model = bgk\ntau = 0.6\ntimesteps  = 40\n"
                   f"timesteps-per-plot = 10\noutput-dir = {out}\nscenario-file = s.xml\n")
    c = io.Config([str(cfg)])
    assert (c.tau, c.timesteps, c.timesteps_per_plot, c.scenario_xml) == (0.6, 40, 10, "s.xml")
    assert out.is_dir()
    (out / "stale.vts").write_text("x")
    c2 = io.Config([str(cfg), "--tau", "0.7", "-t", "5", "--unknown-option", "1"])
    assert (c2.tau, c2.timesteps) == (0.7, 5)  # the command line wins
    assert not (out / "stale.vts").exists()  # an existing output directory is emptied
    with pytest.raises(ValueError, match="tau"):
        io.Config(["--timesteps", "3", "--timesteps-per-plot", "0", "--scenario-file", "a.xml"],
                  prepare_output_dir=False)
    with pytest.raises(ValueError):
        io.Config([str(cfg), "--tau", "2.5"], prepare_output_dir=False)


def test_scenario_xml_faces_and_boxes():
    scn = io.parse_scenario(STEP_XML, q=19, tau=0.55)
    assert (scn.name, scn.xl, scn.yl, scn.zl, scn.tau) == ("Backward step", 12, 10, 18, 0.55)
    assert [b.condition for b in scn.boundaries] == ["inflow", "noslip", "outflow", "noslip", "noslip",
                                                     "noslip", "noslip"]
    assert scn.boundaries[0].extent == (7, 13, 0, 11, 0, 0)
    assert scn.boundaries[0].v == (0.0, 0.0, 0.04) and scn.boundaries[0].rho == 1.0
    assert scn.boundaries[2].extent == S.face_extent("zmax", 12, 10, 18)
    sh = io.parse_scenario(SHEAR_XML)
    assert sh.boundaries[0].condition == "pressure" and sh.boundaries[0].rho == 1.004
    assert sh.boundaries[1].rho == 1.0  # rho-ref defaults to 1


@pytest.mark.parametrize("bad, msg", [
    ("<scenario><domain xl='2' yl='2' zl='2'/></scenario>", "Scenario name is missing!"),
    ("<other name='x'/>", "Scenario node missing!"),
    ("<scenario name='x'></scenario>", "Domain node is missing!"),
    ("<scenario name='x'><domain xl='2'/></scenario>", "Neither vtk-file nor xl/yl/zl"),
    ("<scenario name='x'><domain xl='2' yl='2' zl='2'><boundary condition='noslip'/></domain></scenario>",
     'Missing attribute "extent" for node "boundary"!'),
    ("<scenario name='x'><domain xl='2' yl='2' zl='2'><boundary extent='z0' condition='magic'/></domain>"
     "</scenario>", "magic boundary condition not supported!"),
    ("<scenario name='x'><domain xl='2' yl='2' zl='2'><boundary extent='1 2 3' condition='noslip'/>"
     "</domain></scenario>", 'Extent "1 2 3" is not complete! Must be six values!'),
    ("<scenario name='x'><domain xl='2' yl='2' zl='2'><boundary extent='z0' condition='movingwall' "
     "vx='1'/></domain></scenario>", 'Missing attribute "vy" for node "boundary"!'),
    ("<scenario name='x'><domain", "could not be read"),
])
def test_scenario_errors(bad, msg):
    with pytest.raises(ValueError, match=msg.replace("(", r"\(").replace(")", r"\)")):
        io.parse_scenario(bad)


def test_vtk_mask_reader(tmp_path):
    mask = tube_mask(9, 8, 7, 2.6)
    write_mask_vtk(tmp_path / "tube.vtk", mask)
    dims, origin, spacing, m = io.read_vtk_points(tmp_path / "tube.vtk")
    assert dims == (9, 8, 7) and origin == (-3.5, 1.25, 0.0) and spacing == (2.0, 0.5, 0.5)
    assert np.array_equal(m, mask)
    xml = STEP_XML.replace('<domain xl="12" yl="10" zl="18">', '<domain vtk-file="tube.vtk">')
    scn = io.parse_scenario(xml, base_dir=tmp_path)
    assert (scn.xl, scn.yl, scn.zl) == (9, 8, 7) and scn.origin == origin and scn.spacing == spacing
    assert np.array_equal(scn.solid, 1 - mask)
    with pytest.raises(ValueError, match="does not exist or does not"):
        io.read_vtk_points(tmp_path / "missing.vtk")


def _decode(node):
    raw = base64.b64decode(node.text.strip())
    (n,) = struct.unpack("<I", raw[:4])
    return raw[4:4 + n]


def test_vts_document_roundtrip():
    xl, yl, zl = 4, 3, 2
    rng = np.random.default_rng(0)
    rho = 1 + 0.01 * rng.standard_normal((zl, yl, xl))
    u = 0.01 * rng.standard_normal((zl, yl, xl, 3))
    doc = io.vts_document(xl, yl, zl, (0.5, -1.0, 2.0), (2.0, 1.0, 0.25), rho, u)
    root = ET.fromstring(doc)
    assert root.get("type") == "StructuredGrid"
    arrays = {a.get("Name"): a for a in root.iter("DataArray")}
    vel = np.frombuffer(_decode(arrays["Velocity"]), dtype="<f8").reshape(-1, 3)
    den = np.frombuffer(_decode(arrays["Density"]), dtype="<f8")
    pts_node = next(a for a in root.iter("DataArray") if a.get("Name") is None)
    pts = np.frombuffer(_decode(pts_node), dtype="<f4").reshape(-1, 3)
    assert np.array_equal(vel, u.reshape(-1, 3)) and np.array_equal(den, rho.reshape(-1))
    # x fastest; coordinates xs*x + xo - 1 for x = 1..xl (vtk.hpp:33)
    assert np.allclose(pts[0], [2.0 * 1 + 0.5 - 1, 1.0 * 1 - 1.0 - 1, 0.25 * 1 + 2.0 - 1])
    assert np.allclose(pts[1], [2.0 * 2 + 0.5 - 1, 1.0 * 1 - 1.0 - 1, 0.25 * 1 + 2.0 - 1])
    assert np.allclose(pts[xl], [2.0 * 1 + 0.5 - 1, 1.0 * 2 - 1.0 - 1, 0.25 * 1 + 2.0 - 1])
    ascii_doc = io.vts_document(xl, yl, zl, (0, 0, 0), (1, 1, 1), rho, u, binary=False)
    a = {n.get("Name"): n for n in ET.fromstring(ascii_doc).iter("DataArray")}
    assert np.allclose(np.array(a["Density"].text.split(), dtype=float), rho.reshape(-1))


# ------------------------------------------------------------------------------------------
# the reference's own scenario files (committed copies)
# ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("name", ["cavity.xml", "step.xml", "shearflow.xml", "pipe.xml"])
def test_reference_scenario_files_parse(name, tmp_path, monkeypatch):
    base = reference_scenarios(tmp_path)
    monkeypatch.chdir(base)
    scn = io.parse_scenario((base / "scenarios" / name).read_text())
    assert scn.boundaries and scn.xl > 0
    if name == "pipe.xml":
        assert scn.name == "Pipe flow"
        assert (scn.xl, scn.yl, scn.zl) == (250, 54, 54)
        assert scn.solid is not None and 0 < scn.solid.mean() < 1
        assert [b.condition for b in scn.boundaries] == ["noslip", "noslip", "inflow", "outflow", "noslip",
                                                         "noslip"]
        assert scn.boundaries[2].v == (0.03, 0.0, 0.0)


@pytest.mark.parametrize("name, steps", [("step.xml", 30), ("shearflow.xml", 30), ("cavity.xml", 10),
                                         ("pipe.xml", 6)])
def test_reference_scenarios_port_equals_reference(name, steps, oracle_built, tmp_path, monkeypatch):
    # the parsed scenario run by the reference's own code and by the C port: bit for bit (the pipe
    # mask marks its solid cells in one field only, as the reference's VTK reader does)
    import oracle
    if not oracle.ref_available():
        pytest.skip("reference harness not built (needs the reference tree at build time)")
    base = reference_scenarios(tmp_path)
    monkeypatch.chdir(base)
    scn = io.parse_scenario((base / "scenarios" / name).read_text(), q=19, tau=0.6)
    mode = 1 if name == "pipe.xml" else 0
    try:
        ref = oracle.run_ref(scn, steps, solid_mode=mode, want_pops=False)
    except (OSError, RuntimeError) as e:
        pytest.skip(f"reference build unavailable: {e}")
    port = oracle.run_port(scn, steps, solid_mode=mode)
    assert np.array_equal(ref["rho"], port["rho"]) and np.array_equal(ref["u"], port["u"])


# ------------------------------------------------------------------------------------------
# the C++ driver (lbm_gb300_run): configuration and scenario errors come before any GPU work
# ------------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def driver(lbm_lib):
    from lbm_gb300 import _build
    return _build.build_driver()


def _run(driver, args, cwd):
    import subprocess
    return subprocess.run([str(driver), *args], capture_output=True, text=True, cwd=cwd, timeout=60)


def test_driver_requires_options(driver, tmp_path):
    r = _run(driver, ["--tau", "0.6"], tmp_path)
    assert r.returncode != 0 and "is required but missing" in r.stderr


def test_driver_scenario_errors(driver, tmp_path):
    (tmp_path / "bad.xml").write_text("<scenario><domain xl='2' yl='2' zl='2'/></scenario>")
    r = _run(driver, ["--tau", "0.6", "-t", "2", "--timesteps-per-plot", "0", "--scenario-file", "bad.xml",
                      "--output-dir", str(tmp_path / "o")], tmp_path)
    assert r.returncode != 0 and "Scenario name is missing!" in r.stderr
    r = _run(driver, ["--tau", "0.6", "-t", "2", "--timesteps-per-plot", "0", "--scenario-file", "none.xml",
                      "--output-dir", str(tmp_path / "o")], tmp_path)
    assert 'XML file "none.xml" could not be read properly!' in r.stderr


class _FakeDomain:
    """Sizes, placement and moments of a domain, without a GPU (for the writers' host logic)."""

    def __init__(self, xl=5, yl=4, zl=3, seed=0):
        self.xl, self.yl, self.zl = xl, yl, zl
        self.xo, self.yo, self.zo = 0.5, -1.0, 2.0
        self.xs, self.ys, self.zs = 2.0, 1.0, 0.25
        rng = np.random.default_rng(seed)
        self.rho = 1 + 0.01 * rng.standard_normal((zl, yl, xl))
        self.u = 0.05 * rng.standard_normal((zl, yl, xl, 3))

    def moments(self):
        return self.rho.copy(), self.u.copy()


def test_background_vts_writer_host_logic(tmp_path):
    dom = _FakeDomain()
    with io.VtkWriter(depth=1) as w:
        for t in (1, 2, 3):
            dom.rho += 0.001  # the loop moves on: each file keeps its own snapshot
            w.submit(dom, tmp_path, "bg", t)
            io.write_vtk_file(dom, tmp_path, "direct", t)
    for t in (1, 2, 3):
        assert (tmp_path / f"bg.{t}.vts").read_bytes() == (tmp_path / f"direct.{t}.vts").read_bytes()
    w = io.VtkWriter()
    w.submit(dom, tmp_path / "missing-dir", "x", 1)
    with pytest.raises(OSError):
        w.finish()
    w.close()
