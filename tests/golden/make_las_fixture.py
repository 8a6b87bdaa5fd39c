"""Writes tests/golden/las_5points_14.json from the LAS 1.4 example file that
ships with the reference's vendored laszip (libs/laszip/example/5points_14.las,
1,086 bytes: 5 points of format 6 after two VLRs): the file's bytes, and its
header fields decoded here with `struct` at the offsets the reference reads
(LasLoaderSparse.cpp:493-526), independently of the library's parser.

    python tests/golden/make_las_fixture.py <path to the reference checkout>
    (or CR_REFERENCE=<path> python tests/golden/make_las_fixture.py)
"""
import json
import os
import struct
import sys
from pathlib import Path

arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CR_REFERENCE")
if not arg:
    sys.exit("usage: make_las_fixture.py <path to the reference checkout> (or set CR_REFERENCE)")
ref = Path(arg)
data = (ref / "libs" / "laszip" / "example" / "5points_14.las").read_bytes()
u = lambda fmt, off: struct.unpack_from("<" + fmt, data, off)[0]
fields = {
    "version_major": data[24], "version_minor": data[25],
    "num_points": u("Q", 247) if (data[24], data[25]) >= (1, 4) else u("I", 107),
    "offset_to_points": u("I", 96), "point_format": data[104] % 128,
    "bytes_per_point": u("H", 105),
    "scale": [u("d", 131 + 8 * k) for k in range(3)],
    "offset": [u("d", 155 + 8 * k) for k in range(3)],
    "max": [u("d", 179 + 16 * k) for k in range(3)],
    "min": [u("d", 187 + 16 * k) for k in range(3)],
}
out = Path(__file__).resolve().parent / "las_5points_14.json"
out.write_text(json.dumps({"source": "libs/laszip/example/5points_14.las of the reference",
                           "bytes_hex": data.hex(), "fields": fields}, indent=1) + "\n")
print(out, len(data), fields)
