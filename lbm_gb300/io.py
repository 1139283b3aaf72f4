"""Scenario front end and output, mirroring the reference's io layer:

- Config: the run configuration of io/configuration.h:15-145 (a `key = value` file plus command
  line options; the command line wins, as with boost::program_options there).
- parse_scenario / parse_scenario_file: the XML scenario format of io/scenario.h:21-188 (same
  node and attribute names, face names, extent rules, defaults and error messages).
- read_vtk_point_file: the legacy-VTK STRUCTURED_POINTS fluid mask of io/vtk.hpp:93-157
  (DIMENSIONS give xl, yl, zl; ORIGIN and SPACING the domain's; value 0 marks a solid no-slip cell).
- write_vtk_file: the `<name>.<t>.vts` StructuredGrid output of io/vtk.hpp:42-89 (point data
  "Velocity" and "Density" of the interior cells, points at xs*x + xo - 1 etc., vtk.hpp:19-37),
  from the device moments kernel.

No XML or VTK library is involved: the formats are parsed and written here.
"""
from __future__ import annotations

import base64
import os
import shlex
import struct
import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np

from . import scenario as S

__all__ = ["Config", "parse_config_file", "parse_scenario", "parse_scenario_file", "read_vtk_points",
           "read_vtk_point_file", "write_vtk_file", "vts_document"]

# option name -> (type, default, required) as declared in configuration.h:76-94
_OPTIONS = {
    "collision-model": (str, "bgk", False),
    "tau": (float, None, True),
    "timesteps": (int, None, True),
    "timesteps-per-plot": (int, None, True),
    "scenario-file": (str, None, True),
    "omp-threads": (int, 1, False),
    "output-dir": (str, "vtk", False),
}
_SHORT = {"-c": "collision-model", "-t": "timesteps", "-i": "input-file"}


def parse_config_file(path) -> dict:
    """`key = value` lines; `#` starts a comment; unknown keys are errors (as a boost config file
    parse without allow_unregistered)."""
    out = {}
    for n, raw in enumerate(Path(path).read_text().splitlines(), 1):
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        if "=" not in line:
            raise ValueError(f"{path}:{n}: expected 'key = value'")
        k, v = (t.strip() for t in line.split("=", 1))
        if k not in _OPTIONS:
            raise ValueError(f"unrecognised option '{k}'")
        out[k] = v
    return out


class Config:
    """configuration.h:15-145: Config(argv) reads the command line and an optional input file
    (first positional argument or -i/--input-file)."""

    def __init__(self, argv=(), prepare_output_dir: bool = True):
        args = list(argv)
        values, input_file = {}, None
        i = 0
        while i < len(args):
            a = args[i]
            if a in ("-h", "--help"):
                raise SystemExit("Usage: lbm_gb300_run [file] additional-options...")
            key = None
            if a.startswith("--"):
                key, _, val = a[2:].partition("=")
                if not _:
                    i += 1
                    val = args[i] if i < len(args) else None
            elif a in _SHORT:
                key = _SHORT[a]
                i += 1
                val = args[i] if i < len(args) else None
            else:
                input_file = a  # positional: the configuration file
                i += 1
                continue
            if key == "input-file":
                input_file = val
            elif key in _OPTIONS:
                values[key] = val
            # unknown options are allowed on the command line (allow_unregistered)
            i += 1
        self.input_file = input_file or ""
        if input_file:
            for k, v in parse_config_file(input_file).items():
                values.setdefault(k, v)  # the command line wins
        for k, (typ, default, required) in _OPTIONS.items():
            if k not in values:
                if required:
                    raise ValueError(f"the option '--{k}' is required but missing")
                values[k] = default
            values[k] = typ(values[k])
        self.collision_model = values["collision-model"]
        self.tau = values["tau"]
        self.timesteps = values["timesteps"]
        self.timesteps_per_plot = values["timesteps-per-plot"]
        self.scenario_xml = values["scenario-file"]
        self.omp_threads = values["omp-threads"]
        self.output_dir = values["output-dir"]
        self.output_filename = "output"
        if not (self.timesteps > 0 and 0.5 < self.tau < 2.0 and self.omp_threads > 0
                and self.collision_model == "bgk"):
            raise ValueError("invalid configuration: timesteps > 0, 0.5 < tau < 2, omp-threads > 0 "
                             "and collision-model = bgk are required")
        if prepare_output_dir:
            # configuration.h:131-143: create the directory, or empty an existing one
            d = Path(self.output_dir)
            if not d.exists():
                d.mkdir(parents=True)
            else:
                for f in d.iterdir():
                    if f.is_file():
                        f.unlink()

    def __repr__(self) -> str:
        return (f"Config(tau={self.tau}, timesteps={self.timesteps}, timesteps_per_plot="
                f"{self.timesteps_per_plot}, scenario_xml={self.scenario_xml!r}, output_dir={self.output_dir!r})")


# ------------------------------------------------------------------------------------------
# XML scenarios (scenario.h)
# ------------------------------------------------------------------------------------------
def _attr(node, name: str) -> str:
    v = node.get(name)
    if v is None:
        raise ValueError(f'Missing attribute "{name}" for node "{node.tag}"!')
    return v


def _condition(node) -> tuple:
    """scenario.h:29-92 -> (condition, velocity, rho)."""
    c = _attr(node, "condition")
    if c == "noslip" or c == "freeslip":
        return c, (0.0, 0.0, 0.0), 1.0
    if c == "movingwall" or c == "inflow":
        v = tuple(float(_attr(node, k)) for k in ("vx", "vy", "vz"))
        rho = float(node.get("rho-ref", 1.0)) if c == "inflow" else 1.0
        return c, v, rho
    if c == "outflow":
        return c, (0.0, 0.0, 0.0), float(node.get("rho-ref", 1.0))
    if c == "pressure":
        return c, (0.0, 0.0, 0.0), float(_attr(node, "rho-in"))
    raise ValueError(f"{c} boundary condition not supported!")


def _extent(text: str, xl: int, yl: int, zl: int) -> tuple:
    """scenario.h:94-128: a face name or six integers (extra values ignored)."""
    faces = ("z0", "zmax", "x0", "xmax", "y0", "ymax")
    if text in faces:
        return S.face_extent(text, xl, yl, zl)
    vals = [int(t) for t in text.split()]
    if len(vals) < 6:
        raise ValueError(f'Extent "{text}" is not complete! Must be six values!')
    return tuple(vals[:6])


def parse_scenario(xml_text: str, q: int = 19, tau: float = 1.0, base_dir=None) -> S.Scenario:
    """The scenario of an XML document as a Scenario (scenario.h:131-188). A domain given by
    vtk-file takes its size, origin, spacing and solid mask from that file, looked up relative to
    the working directory (as the reference does) or, failing that, to base_dir."""
    try:
        root = ET.fromstring(xml_text)
    except ET.ParseError as e:
        raise ValueError("XML file could not be read properly!") from e
    scen = root if root.tag == "scenario" else root.find("scenario")
    if scen is None:
        raise ValueError("Scenario node missing!")
    name = scen.get("name")
    if name is None:
        raise ValueError("Scenario name is missing!")
    dom = scen.find("domain")
    if dom is None:
        raise ValueError("Domain node is missing!")
    vtk = dom.get("vtk-file")
    solid, origin, spacing = None, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    if vtk is not None:
        path = Path(vtk)
        if not path.exists() and base_dir is not None and (Path(base_dir) / vtk).exists():
            path = Path(base_dir) / vtk
        (xl, yl, zl), origin, spacing, mask = read_vtk_points(path)
        solid = (mask == 0).astype(np.uint8)
    elif all(dom.get(k) is not None for k in ("xl", "yl", "zl")):
        xl, yl, zl = (int(dom.get(k)) for k in ("xl", "yl", "zl"))
        if not (xl > 0 and yl > 0 and zl > 0):
            raise ValueError("domain lengths must be positive")
    else:
        raise ValueError("Neither vtk-file nor xl/yl/zl attribute provided to domain node!")
    scn = S.Scenario(name, q, xl, yl, zl, tau, origin=origin, spacing=spacing)
    scn.solid = solid
    for b in dom.findall("boundary"):
        ext = _attr(b, "extent")
        cond, v, rho = _condition(b)
        scn.boundaries.append(S.Boundary(cond, _extent(ext, xl, yl, zl), v, rho))
    return scn


def parse_scenario_file(filename, cfg: Config | None = None, collision=None, q: int = 19,
                        precision: str = "fp64"):
    """scenario.h:131-188: reads the XML file, sets cfg.output_filename to the scenario's name and
    returns the Domain (collision: a BGKCollision, or tau from cfg)."""
    path = Path(filename)
    try:
        text = path.read_text()
    except OSError as e:
        raise ValueError(f'XML file "{filename}" could not be read properly!') from e
    tau = collision.tau if collision is not None else (cfg.tau if cfg is not None else 1.0)
    scn = parse_scenario(text, q=q, tau=tau, base_dir=path.parent)
    if cfg is not None:
        cfg.output_filename = scn.name
    return S.build_domain(scn, precision)


# ------------------------------------------------------------------------------------------
# legacy VTK fluid mask (vtk.hpp:93-157)
# ------------------------------------------------------------------------------------------
def read_vtk_points(path):
    """((xl, yl, zl), origin, spacing, mask[zl, yl, xl] uint8) of an ASCII legacy-VTK
    STRUCTURED_POINTS file with one point-data array (x fastest)."""
    try:
        text = Path(path).read_text()
    except OSError as e:
        raise ValueError(f'VTK file "{path}" does not exist or does not seem to be a valid structured '
                         'grids file!') from e
    toks = text.split()
    if len(toks) < 3 or "STRUCTURED_POINTS" not in toks:
        raise ValueError(f'VTK file "{path}" does not exist or does not seem to be a valid structured '
                         'grids file!')
    up = [t.upper() for t in toks]

    def after(key, n, conv):
        if key not in up:
            raise ValueError(f"VTK file {path}: {key} missing")
        k = up.index(key)
        return tuple(conv(t) for t in toks[k + 1:k + 1 + n])
    dims = after("DIMENSIONS", 3, int)
    origin = after("ORIGIN", 3, float) if "ORIGIN" in up else (0.0, 0.0, 0.0)
    spacing = after("SPACING", 3, float) if "SPACING" in up else (1.0, 1.0, 1.0)
    if "SPACING" not in up and "ASPECT_RATIO" in up:
        spacing = after("ASPECT_RATIO", 3, float)
    (npts,) = after("POINT_DATA", 1, int)
    if npts != dims[0] * dims[1] * dims[2] or min(dims) < 1:
        raise ValueError(f"VTK file {path}: POINT_DATA does not match DIMENSIONS")
    k = up.index("POINT_DATA") + 2
    # SCALARS name type [ncomp] / LOOKUP_TABLE name, then the values
    if k < len(up) and up[k] == "SCALARS":
        k += 3
        if k < len(up) and toks[k].isdigit() and up[k + 1] == "LOOKUP_TABLE":
            k += 1
        if up[k] == "LOOKUP_TABLE":
            k += 2
    vals = np.array(toks[k:k + npts], dtype=np.float64)
    if vals.size != npts:
        raise ValueError(f"VTK file {path}: expected {npts} values, found {vals.size}")
    mask = (vals != 0).astype(np.uint8).reshape(dims[2], dims[1], dims[0])
    return dims, origin, spacing, mask


def read_vtk_point_file(filename, collision, q: int = 19, precision: str = "fp64"):
    """vtk.hpp:93-157: a Domain sized, placed and spaced by the file, whose zero-valued points
    are solid no-slip cells."""
    from .domain import BGKCollision, Domain
    (xl, yl, zl), origin, spacing, mask = read_vtk_points(filename)
    from . import model as _model
    dom = Domain(xl, yl, zl, collision if collision is not None else BGKCollision(1.0), *origin, *spacing,
                 model=_model.get(q), precision=precision)
    dom.set_solid_mask((mask == 0).astype(np.uint8))
    return dom


# ------------------------------------------------------------------------------------------
# VTS output (vtk.hpp:42-89)
# ------------------------------------------------------------------------------------------
def _b64(arr: np.ndarray) -> str:
    raw = np.ascontiguousarray(arr).tobytes()
    return base64.b64encode(struct.pack("<I", len(raw)) + raw).decode("ascii")


def vts_document(xl, yl, zl, origin, spacing, rho, u, binary: bool = True) -> str:
    """A VTK XML StructuredGrid of the interior cells: point data "Velocity" (3 x Float64) and
    "Density" (Float64), points (Float32) at (xs*x + xo - 1, ys*y + yo - 1, zs*z + zo - 1) for
    x = 1..xl etc., x fastest (vtk.hpp:19-37, 60-83)."""
    xs, ys, zs = spacing
    xo, yo, zo = origin
    x = (xs * np.arange(1, xl + 1) + xo - 1).astype(np.float64)
    y = (ys * np.arange(1, yl + 1) + yo - 1).astype(np.float64)
    z = (zs * np.arange(1, zl + 1) + zo - 1).astype(np.float64)
    zz, yy, xx = np.meshgrid(z, y, x, indexing="ij")
    pts = np.stack([xx, yy, zz], axis=-1).reshape(-1, 3).astype(np.float32)
    vel = np.asarray(u, dtype=np.float64).reshape(-1, 3)
    den = np.asarray(rho, dtype=np.float64).reshape(-1)
    fmt = "binary" if binary else "ascii"

    def data(a):
        if binary:
            return _b64(a)
        return "\n".join(" ".join(repr(float(v)) for v in row) for row in np.atleast_2d(a.reshape(len(a), -1)))
    ext = f"0 {xl - 1} 0 {yl - 1} 0 {zl - 1}"
    return (
        '<?xml version="1.0"?>\n'
        '<VTKFile type="StructuredGrid" version="0.1" byte_order="LittleEndian" header_type="UInt32">\n'
        f'  <StructuredGrid WholeExtent="{ext}">\n'
        f'    <Piece Extent="{ext}">\n'
        '      <PointData Scalars="Density" Vectors="Velocity">\n'
        f'        <DataArray type="Float64" Name="Velocity" NumberOfComponents="3" format="{fmt}">\n'
        f'{data(vel)}\n'
        '        </DataArray>\n'
        f'        <DataArray type="Float64" Name="Density" format="{fmt}">\n'
        f'{data(den)}\n'
        '        </DataArray>\n'
        '      </PointData>\n'
        '      <CellData></CellData>\n'
        '      <Points>\n'
        f'        <DataArray type="Float32" NumberOfComponents="3" format="{fmt}">\n'
        f'{data(pts)}\n'
        '        </DataArray>\n'
        '      </Points>\n'
        '    </Piece>\n'
        '  </StructuredGrid>\n'
        '</VTKFile>\n')


def write_vtk_file(domain, output_dir, output_filename: str, t: int, binary: bool = True) -> Path:
    """vtk.hpp:42-89: <output_dir>/<output_filename>.<t>.vts from the domain's moments (computed on
    the device)."""
    rho, u = domain.moments()
    path = Path(output_dir) / f"{output_filename}.{t}.vts"
    _write_vts(path, domain, rho, u, binary)
    return path


def _write_vts(path: Path, domain, rho, u, binary: bool) -> None:
    doc = vts_document(domain.xl, domain.yl, domain.zl, (domain.xo, domain.yo, domain.zo),
                       (domain.xs, domain.ys, domain.zs), rho, u, binary)
    path.write_text(doc)


class _DomainGeometry:
    """The sizes, origin and spacing of a domain: what a queued file needs after the loop moved on."""

    def __init__(self, d):
        self.xl, self.yl, self.zl = d.xl, d.yl, d.zl
        self.xo, self.yo, self.zo = d.xo, d.yo, d.zo
        self.xs, self.ys, self.zs = d.xs, d.ys, d.zs


class VtkWriter:
    """Extension: write_vtk_file with the file written on a background thread. The reference writes
    on the time loop's thread (main.cpp:56-57); here submit() reads the moments back (one
    synchronising read) and returns, and the loop keeps launching steps while the file is encoded
    and written. At most `depth` snapshots wait in memory; a failed write is raised by the next
    submit() or by finish()."""

    def __init__(self, depth: int = 2):
        import queue
        import threading
        self._q = queue.Queue(maxsize=max(1, depth))
        self._error = None
        self._thread = threading.Thread(target=self._run, daemon=True)
        self._thread.start()

    def _run(self):
        while True:
            job = self._q.get()
            try:
                if job is None:
                    return
                _write_vts(*job)
            except BaseException as e:  # kept for the caller's thread
                if self._error is None:
                    self._error = e
            finally:
                self._q.task_done()

    def _raise(self):
        if self._error is not None:
            e, self._error = self._error, None
            raise e

    def submit(self, domain, output_dir, output_filename: str, t: int, binary: bool = True) -> Path:
        self._raise()
        rho, u = domain.moments()
        path = Path(output_dir) / f"{output_filename}.{t}.vts"
        self._q.put((path, _DomainGeometry(domain), rho, u, binary))
        return path

    def finish(self) -> None:
        """Waits for every submitted file; raises the first failure."""
        self._q.join()
        self._raise()

    def close(self) -> None:
        self.finish()
        self._q.put(None)
        self._thread.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
