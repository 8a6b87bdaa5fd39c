"""Generates tests/golden/golden.json: seeded inputs, their camera matrices (as
exact hex doubles, so no platform's libm is involved when a test replays
them) and FNV-1a-64 digests of the oracle's outputs.

The reference ships no tests or golden vectors, and its GLSL kernels cannot run
without OpenGL; these digests pin the oracle (and through it the CUDA path) to
fixed outputs.  Inputs are regenerated by the product's host generator, whose
own digest is part of each case.

    python tests/golden/make_golden.py          # rewrite golden.json
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from compute_rasterizer_gb300 import _lib as L  # noqa: E402
from compute_rasterizer_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.json"

QUIRKS = {"loop_las": O.L0_X12,
          "loop_las_prefetch": O.INCLUSIVE_END | O.DISPATCH_BY_POINTS | O.UVEC4_BASE,
          "loop_las_hqs": O.L0_X12 | O.INCLUSIVE_END | O.DISPATCH_BY_POINTS}


def hexs(m) -> list[str]:
    return [float(x).hex() for x in np.asarray(m, np.float64).reshape(16)]


def unhex(h) -> np.ndarray:
    return np.array([float.fromhex(x) for x in h], np.float64)


def dg(a: np.ndarray) -> str:
    return f"{O.fnv(a):016x}"


def terrain_inputs(case):
    p = synth.synth_params(L.SYNTH_TERRAIN, case["extent"], case["seed"])
    rec, hdr = synth.las_records_host(p, case["n"])
    batches, lo, md, hi, rgba = synth.encode_las(rec, case["n"], hdr)
    return hdr, batches, lo, md, hi, rgba


def run_case(case) -> dict:
    """Recompute a case's digests with the host generator and the oracle."""
    out = {}
    if case["kind"] == "terrain":
        hdr, batches, lo, md, hi, rgba = terrain_inputs(case)
        out["batches"], out["low"], out["med"], out["hig"], out["rgba"] = (
            dg(batches), dg(lo), dg(md), dg(hi), dg(rgba))
        bmin = np.array(hdr.min[:])[None]
        for cname, cam in case["cameras"].items():
            view, proj = unhex(cam["view"]), unhex(cam["proj"])
            w, h = cam["width"], cam["height"]
            for m in case["methods"]:
                fr = O.make_frame(view, proj, w, h, bmin, 1, QUIRKS[m["method"]], m["payload"])
                if m["method"] == "loop_las_hqs":
                    depth, accum, img = O.hqs(fr, batches, case["n"], lo, md, hi, rgba)
                    out[f"{cname}/hqs/depth"] = dg(depth)
                    out[f"{cname}/hqs/accum"] = dg(accum)
                    out[f"{cname}/hqs/image"] = dg(img)
                    continue
                fb = O.raster_batched(fr, batches, case["n"], lo, md, hi, rgba,
                                      threads=case.get("threads", 1))
                key = f"{cname}/{m['method']}/{'color' if m['payload'] else 'index'}"
                out[key + "/fb"] = dg(fb)
                img = (O.resolve_color(w, h, fb) if m["payload"] else
                       O.resolve_index(w, h, fb, rgba))
                out[key + "/image"] = dg(img)
    elif case["kind"] == "plain":
        v = synth.uniform_vertices_host(case["seed"], case["n"], case["size"])
        out["vertices"] = dg(v)
        cam = case["camera"]
        fb, img, _ = O.plain(unhex(cam["view"]), unhex(cam["proj"]), cam["width"], cam["height"], v)
        out["fb"] = dg(fb)
        out["image"] = dg(img)
    return out


def config1_camera(width=1920, height=1080):
    view = synth.look_at([150.0, 150.0, 150.0], [50.0, 50.0, 50.0], [0.0, 0.0, 1.0])
    proj = synth.perspective(60.0, width / height, 0.1, 1000.0)
    return {"view": hexs(view), "proj": hexs(proj), "width": width, "height": height}


def terrain_case(name, n, extent, seed, width, height, threads=1):
    from helpers import camera_views
    case = {"kind": "terrain", "n": n, "extent": extent, "seed": seed}
    hdr, batches = terrain_inputs(case)[:2]
    views = camera_views(np.array(hdr.min[:]), np.array(hdr.max[:]), batches)
    proj = synth.perspective(60.0, width / height, 0.1, 200000.0)
    cams = {k: {"view": hexs(v), "proj": hexs(proj), "width": width, "height": height}
            for k, v in views.items()}
    methods = [{"method": "loop_las", "payload": 0}, {"method": "loop_las_prefetch", "payload": 0},
               {"method": "loop_las", "payload": 1}, {"method": "loop_las_hqs", "payload": 0}]
    return {"name": name, "kind": "terrain", "n": n, "extent": extent, "seed": seed,
            "cameras": cams, "methods": methods, "threads": threads}


def main():
    cases = [
        terrain_case("terrain_62674_200m", 62674, 200.0, 7, 320, 240),
        terrain_case("terrain_1m_1km", 1_000_000, 1000.0, 21, 640, 360, threads=8),
        {"name": "plain_100k", "kind": "plain", "n": 100_000, "seed": 1, "size": 100.0,
         "camera": config1_camera(320, 180)},
        {"name": "plain_uniform_4194304_1080p", "kind": "plain", "n": 4_194_304, "seed": 1,
         "size": 100.0, "camera": config1_camera()},
    ]
    for c in cases:
        c["digests"] = run_case(c)
        print(c["name"], len(c["digests"]), "digests")
    OUT.write_text(json.dumps({"note": "digests: FNV-1a 64 of the raw little-endian arrays",
                               "cases": cases}, indent=1))
    print("wrote", OUT)


if __name__ == "__main__":
    main()
