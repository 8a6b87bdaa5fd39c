"""Writes tests/golden/laz/*.laz and tests/golden/laz.json: LAZ files (LAS
point formats 0-3 and the LAS 1.4 formats 6-8) whose point data the
reference's vendored LASzip compressed (libs/laszip/src, built
into oracle/_ref/liblaszipref.so by oracle/Makefile from the reference
checkout), over the deterministic records of tests/helpers.laz_records.  The
CPU tests decode them with the product's reader, compare the product writer's
bytes with them, and the GPU tests load them into clouds.

    CR_REFERENCE=<path to the reference checkout> python tests/golden/make_laz_fixtures.py
"""
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parent.parent))

import numpy as np  # noqa: E402

import helpers  # noqa: E402
from oracle import oracle as O  # noqa: E402

# name, point format, points, seed, extra bytes, chunk size (-1 variable), points per variable chunk
CASES = [
    ("fmt0_3chunks", 0, 3000, 1, 0, 1000, 0),
    ("fmt1_extra2", 1, 3000, 2, 2, 1000, 0),
    ("fmt2_12k", 2, 12000, 3, 0, 5000, 0),
    ("fmt3_variable", 3, 5000, 4, 0, -1, 1700),
    # LAS 1.4, LASzip's layered coder
    ("fmt6_channels", 6, 4000, 5, 0, 1500, 0),
    ("fmt7_extra3", 7, 4000, 6, 3, 50000, 0),
    ("fmt8_variable", 8, 5000, 7, 0, -1, 1800),
]


def main():
    O.build()
    if not O.LAZREF.exists():
        sys.exit("oracle/_ref/liblaszipref.so missing: set CR_REFERENCE to the reference checkout")
    out_dir = HERE / "laz"
    out_dir.mkdir(exist_ok=True)
    meta = []
    for name, fmt, n, seed, extra, chunk, var_every in CASES:
        rec, bpp = helpers.laz_records(fmt, n, seed, extra)
        data = helpers.laszip_file(rec, n, fmt, bpp, chunk, var_every)
        (out_dir / f"{name}.laz").write_bytes(data)
        meta.append({"name": name, "point_format": fmt, "points": n, "seed": seed, "extra": extra,
                     "chunk_size": chunk, "var_chunk": var_every, "bytes_per_point": bpp,
                     "records_fnv": O.fnv(rec), "file_fnv": O.fnv(np.frombuffer(data, np.uint8)),
                     "file_bytes": len(data)})
        print(name, len(data))
    (HERE / "laz.json").write_text(json.dumps({"source": "point data written by the reference's "
                                               "vendored LASzip (libs/laszip/src)", "cases": meta},
                                              indent=1) + "\n")


if __name__ == "__main__":
    main()
