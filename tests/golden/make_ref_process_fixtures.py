"""Generate end-to-end fixtures from the reference's own decomposition loop.

Runs oracle/_ref (the VisACD host sources compiled in place, with the FP64
oracle for visibility and scoring and this project's stand-ins for OpenVDB,
qhull and CDT) on seeded synthetic meshes and records the number of parts, the
final concavity and per-part sizes and volumes. The GPU tests compare
visacd.process() against these files. Needs the reference tree (development
container); the fixtures are committed so the GPU machine does not.

    python tests/golden/make_ref_process_fixtures.py
"""
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle.ref as R  # noqa: E402
from visacd_gb300 import meshgen as mg  # noqa: E402

CASES = [
    # the torus the reference's small config names: 64 x 32 grid, R 1, r 0.35
    {"name": "torus_64x32_c0.04_n32", "mesh": ["torus", 64, 32, 42], "concavity": 0.04,
     "num_parts": 32, "seed": 42, "mode": "concavity"},
    {"name": "blob_s3_c0.02_n8", "mesh": ["blob", 3, 7], "concavity": 0.02, "num_parts": 8,
     "seed": 3, "mode": "concavity"},
    {"name": "torus_32x16_edge_n6", "mesh": ["torus", 32, 16, 5], "concavity": 0.04,
     "num_parts": 6, "seed": 11, "mode": "edge"},
    # the large concave blob: icosphere subdivision 5 with 8 seeded bumps
    {"name": "blob_s5_c0.02_n64", "mesh": ["blob", 5, 2026], "concavity": 0.02, "num_parts": 64,
     "seed": 42, "mode": "concavity"},
    # hull merging on (multimerge_ch after the split loop)
    {"name": "blob_s3_c0.02_n12_merge", "mesh": ["blob", 3, 11], "concavity": 0.02,
     "num_parts": 12, "seed": 5, "mode": "concavity", "merging": True},
]


def make_mesh(spec):
    if spec[0] == "torus":
        return mg.torus(R=1.0, r=0.35, nu=spec[1], nv=spec[2], perturb=0.02, seed=spec[3])
    return mg.displaced_blob(spec[1], seed=spec[2])


def volume(v, t):
    p0, p1, p2 = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    return float(np.sum(np.einsum("ij,ij->i", p0, np.cross(p1, p2))) / 6.0)


def main():
    out = {}
    for c in CASES:
        v, t = make_mesh(c["mesh"])
        t0 = time.time()
        n, conc, parts = R.process(v, t, c["concavity"], c["num_parts"], c["seed"], c["mode"],
                                   use_merging=c.get("merging", False))
        out[c["name"]] = {**c, "num_parts": c["num_parts"], "result_parts": n, "concavity_out": conc,
                          "part_vertices": [len(p["vertices"]) for p in parts],
                          "part_triangles": [len(p["triangles"]) for p in parts],
                          "part_volumes": [volume(p["vertices"], p["triangles"]) for p in parts],
                          "seconds": time.time() - t0}
        print(c["name"], n, conc, f"{time.time() - t0:.1f}s", flush=True)
    (Path(__file__).parent / "ref_process.json").write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
