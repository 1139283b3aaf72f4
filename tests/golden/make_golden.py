"""Generates tests/golden/*.npz from the reference's own solver.

Runs the reference's unmodified headers (compiled by oracle/Makefile into
oracle/_ref/libref_lbm.so with FP contraction off) on every case of tests/golden/cases.py and on
the 64^3 FP64 cavity, and stores the results. Also copies the reference's own scenario
files (build/scenarios/{cavity,pipe,shearflow,step}.xml as they are, and the 250 x 54 x 54
legacy-VTK mask pipe.vtk gzip-compressed, with the SHA-256 of the uncompressed file) into
tests/golden/scenarios/. Needs the reference tree (LBM_REFERENCE_DIR); run from the repo root:

    make -C oracle ref REF_DIR=$LBM_REFERENCE_DIR && python tests/golden/make_golden.py
"""
from __future__ import annotations

import gzip
import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle  # noqa: E402
from golden import cases  # noqa: E402

OUT = Path(__file__).resolve().parent


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def copy_scenarios() -> None:
    src = oracle.checkers.reference_dir() / "build" / "scenarios"
    dst = OUT / "scenarios"
    dst.mkdir(exist_ok=True)
    for name in ("cavity.xml", "pipe.xml", "shearflow.xml", "step.xml"):
        (dst / name).write_bytes((src / name).read_bytes())
    raw = (src / "pipe.vtk").read_bytes()
    (dst / "pipe.vtk.gz").write_bytes(gzip.compress(raw, compresslevel=9, mtime=0))
    (dst / "pipe.vtk.sha256").write_text(hashlib.sha256(raw).hexdigest() + "\n")
    print("scenario files copied; pipe.vtk", len(raw), "bytes")


def main() -> None:
    copy_scenarios()
    for name, (make, steps) in cases.CASES.items():
        scn = make()
        r = oracle.run_ref(scn, steps, threads=1)
        np.savez_compressed(OUT / f"{name}.npz", pops=r["pops"], rho=r["rho"], u=r["u"], steps=steps)
        print(name, scn.xl, scn.yl, scn.zl, steps)
    make, steps = cases.CAVITY64
    scn = make()
    r = oracle.run_ref(scn, steps, threads=8, want_pops=False)
    rho = r["rho"].reshape(-1)
    u = r["u"].reshape(-1, 3)
    idx = cases.CAVITY64_SAMPLE
    np.savez_compressed(OUT / "cavity64_q19_1000.npz", sample_index=idx, rho=rho[idx], u=u[idx],
                        rho_sha256=sha(rho), u_sha256=sha(u), steps=steps)
    print("cavity64", sha(rho), sha(u))


if __name__ == "__main__":
    main()
