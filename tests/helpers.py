"""Shared test workloads: small seeded clouds, cameras, and GPU-vs-oracle runs."""
from __future__ import annotations

import numpy as np

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import default_params, make_view, synth
from oracle import oracle as O

QUIRKS = {L.METHOD_LOOP_LAS: O.L0_X12,
          L.METHOD_LOOP_LAS_PREFETCH: O.INCLUSIVE_END | O.DISPATCH_BY_POINTS | O.UVEC4_BASE,
          L.METHOD_LOOP_LAS_HQS: O.L0_X12 | O.INCLUSIVE_END | O.DISPATCH_BY_POINTS}


def terrain_las(n=62674, extent=200.0, seed=7, kind=L.SYNTH_TERRAIN, **kw):
    p = synth.synth_params(kind, extent, seed, **kw)
    rec, hdr = synth.las_records_host(p, n)
    return p, rec, hdr


def encoded(n=62674, extent=200.0, seed=7, **kw):
    p, rec, hdr = terrain_las(n, extent, seed, **kw)
    batches, lo, md, hi, rgba = synth.encode_las(rec, n, hdr)
    return dict(n=n, hdr=hdr, rec=rec, batches=batches, lo=lo, md=md, hi=hi, rgba=rgba,
                box_min=synth.header_min(hdr), box_max=synth.header_max(hdr))


def cameras(cl, width=320, height=240):
    """Far (levels 2-4), near (levels 0-1) and partly-outside views of a cloud."""
    views = camera_views(cl["box_min"], cl["box_max"], cl["batches"])
    proj = synth.perspective(60.0, width / height, 0.1, 200000.0)
    return {k: (v, proj, width, height) for k, v in views.items()}


def camera_views(bmin, bmax, batches):
    """far: the reference's zoom-to-cloud pose (levels 2-4); near: 1.5 m from a
    batch centre (30-bit for that batch, 20-bit around it); mid: 30 m above the
    same batch (20-bit); corner: partly outside the cloud (culling)."""
    yaw, pitch, radius, target = synth.zoom_to_cloud(bmin, bmax)
    size = bmax - bmin
    b = batches[len(batches) // 2]
    centre = bmin + 0.5 * np.array([b["min_x"] + b["max_x"], b["min_y"] + b["max_y"],
                                    b["min_z"] + b["max_z"]], np.float64)
    return {
        "far": synth.orbit_view(yaw, pitch, radius, target),
        "near": synth.orbit_view(0.3, -0.35, 1.5, centre),
        "mid": synth.orbit_view(1.1, -1.2, 30.0, centre),
        "corner": synth.orbit_view(2.0, -0.5, 0.3 * float(np.linalg.norm(size)), bmin + 0.1 * size),
    }


def oracle_frame(cam, box_mins, quirks, payload=O.PAYLOAD_INDEX, culling=1):
    view, proj, w, h = cam
    return O.make_frame(view, proj, w, h, box_mins, culling=culling, quirks=quirks,
                        payload=payload)


def gpu_raw(ctx, cloud, cam, method, payload=L.PAYLOAD_INDEX, quirks=L.QUIRKS_METHOD_DEFAULT,
            culling=1, fb_kind=None, clear=L.DEFAULT_CLEAR, **kw):
    """Rasterize only (no resolve); returns the Framebuffer."""
    view, proj, w, h = cam
    kind = fb_kind if fb_kind is not None else (
        L.FB_HQS if method == L.METHOD_LOOP_LAS_HQS else L.FB_U64)
    fb = ctx.framebuffer(w, h, kind)
    fb.clear(0xFF800000 if kind == L.FB_HQS else clear)
    params = default_params(method, payload=payload, quirks=quirks, frustum_culling=culling,
                            resolve=0, clear_after=0, **kw)
    ctx.render(cloud, make_view(view, proj, w, h), params, fb)
    ctx.sync()
    return fb, params


def first_diff(a, b, n=5):
    idx = np.nonzero(a != b)[0][:n]
    return [(int(i), hex(int(a[i])), hex(int(b[i]))) for i in idx]


IDENTITY = np.eye(4).reshape(16)


def handmade_cloud(points, colors, box_min=(-1.0, -1.0, 0.0), box_max=(1.0, 1.0, 1.0),
                   first_point=0, pad_before=0):
    """One batch whose 10-bit words are given directly: points are integer
    (X, Y, Z) in [0, 1023]; the decoded position is box_min + X * size / 1024.
    With identity view and projection, NDC = decoded position and w = 1."""
    pts = np.asarray(points, np.uint32).reshape(-1, 3)
    n = pad_before + len(pts)
    lo = np.zeros(n, np.uint32)
    lo[pad_before:] = pts[:, 0] | (pts[:, 1] << 10) | (pts[:, 2] << 20)
    rgba = np.zeros(n, np.uint32)
    rgba[pad_before:] = np.asarray(colors, np.uint32)
    b = np.zeros(1, L.BATCH_DTYPE)
    b["min_x"], b["min_y"], b["min_z"] = box_min
    b["max_x"], b["max_y"], b["max_z"] = box_max
    b["num_points"] = len(pts)
    b["first_point"] = pad_before
    zeros = np.zeros(n, np.uint32)
    return dict(n=n, batches=b, lo=lo, md=zeros.copy(), hi=zeros.copy(), rgba=rgba,
                box_min=np.zeros(3), box_max=np.ones(3))


def identity_cam(w=64, h=32):
    return (IDENTITY, IDENTITY, w, h)


def build_method_demo(out_dir):
    """Compiles tests/cpp/method_demo.cpp against include/cr_method.hpp and the
    in-tree library; returns the executable's path."""
    import subprocess
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    libdir = root / "compute_rasterizer_gb300" / "_build"
    exe = Path(out_dir) / "method_demo"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{root / 'include'}",
           str(root / "tests" / "cpp" / "method_demo.cpp"), f"-L{libdir}", "-lcr_raster",
           f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def many_file_cloud(nfiles=300, seed=11, extent=3000.0, base=10241, spread=2999):
    """A terrain cut into `nfiles` LAS files the way the reference's loader
    sees a tiled dataset: consecutive runs of the Morton-ordered records, each
    file its own boxMin (the min of its points) and file_index, encoded by the
    host layout builder at its sparse offset.  Every file holds more than
    10,240 points (two batch records), and the file sizes vary, so the files'
    first points fall on every value of firstPoint % 4."""
    sizes = [base + (i * 7919) % spread for i in range(nfiles)]
    n = int(sum(sizes))
    p, rec, hdr = terrain_las(n, extent, seed)
    scale = np.array(hdr.scale[:], np.float64)
    offset = np.array(hdr.offset[:], np.float64)
    rec2 = rec.reshape(n, L.LAS_FORMAT2_BYTES)
    xyz = rec2[:, :12].copy().view("<i4").reshape(n, 3).astype(np.float64) * scale + offset
    parts = [[], [], [], [], []]
    box_mins = np.zeros((nfiles, 3), np.float64)
    off = 0
    for i, sz in enumerate(sizes):
        bmin = xyz[off:off + sz].min(axis=0)
        box_mins[i] = bmin
        out = synth.encode_las(np.ascontiguousarray(rec2[off:off + sz]).reshape(-1), sz, hdr,
                               sparse_offset=off, file_index=i, box_min=bmin)
        for k in range(5):
            parts[k].append(out[k])
        off += sz
    batches, lo, md, hi, rgba = (np.concatenate(x) for x in parts)
    return dict(n=n, hdr=hdr, batches=batches, lo=lo, md=md, hi=hi, rgba=rgba,
                box_min=box_mins, box_max=synth.header_max(hdr), world_min=synth.header_min(hdr),
                sizes=sizes)


def many_file_cameras(cl, width=480, height=270):
    """far: the whole tiled cloud (10-bit); mid and near: 120 m and 5 m from
    a batch centre of a file in the middle (levels 1-4, and 0-4: 20/30-bit
    batches of several files next to 10-bit ones, the rest culled)."""
    bmin, bmax = cl["world_min"], cl["box_max"]
    yaw, pitch, radius, target = synth.zoom_to_cloud(bmin, bmax)
    b = cl["batches"][len(cl["batches"]) // 2]
    fmin = cl["box_min"][b["file_index"]]
    centre = fmin + 0.5 * np.array([b["min_x"] + b["max_x"], b["min_y"] + b["max_y"],
                                    b["min_z"] + b["max_z"]], np.float64)
    proj = synth.perspective(60.0, width / height, 0.1, 200000.0)
    views = {"far": synth.orbit_view(yaw, pitch, radius, target),
             "mid": synth.orbit_view(1.1, -0.6, 120.0, centre),
             "near": synth.orbit_view(0.3, -0.35, 5.0, centre)}
    return {k: (v, proj, width, height) for k, v in views.items()}


def pixel_grid_cloud(firsts, counts, total, width=1024, height=32):
    """Batches over one stream whose point g (global index) decodes, under the
    identity camera of a width x height view, to its own pixel
    (g % width, g // width): X = g % 1024 (width 1024), Y = (g // 1024) * 32.
    Every batch has the AABB (-1, -1, 0) - (1, 1, 1); `firsts` / `counts` are
    the batches' first_point / num_points (any alignment).  A rendered index
    payload therefore shows exactly which points a method visited."""
    assert width == 1024 and height == 32 and total + 64 <= width * height
    g = np.arange(total + 64, dtype=np.uint32)
    lo = (g % 1024) | (((g // 1024) * 32) << 10)
    lo[total:] = 0
    b = np.zeros(len(firsts), L.BATCH_DTYPE)
    b["min_x"], b["min_y"], b["min_z"] = -1.0, -1.0, 0.0
    b["max_x"], b["max_y"], b["max_z"] = 1.0, 1.0, 1.0
    b["first_point"] = firsts
    b["num_points"] = counts
    zeros = np.zeros(total + 64, np.uint32)
    rgba = (g * 2654435761).astype(np.uint32) & np.uint32(0xFFFFFF)
    return dict(n=total, batches=b, lo=lo.astype(np.uint32), md=zeros.copy(), hi=zeros.copy(),
                rgba=rgba, box_min=np.zeros((1, 3)))


def las2_visits(first, num_points, inclusive=True, threads=128, per_thread=80):
    """The batch-local indices compute_loop_las2/render.cs:319-341 visits: per
    thread base = firstPoint / 4 + tid, index = 4 * (base + i * 128) + j, uint
    localIndex = index - firstPoint, `localIndex > numPoints` returns (`>=` when
    not inclusive).  A literal restatement of the shader's loop, in Python."""
    out = []
    m = 0xFFFFFFFF
    for t in range(threads):
        base = first // 4 + t
        done = False
        for i in range(per_thread // 4):
            for j in range(4):
                index = (4 * (base + i * threads) + j) & m
                local = (index - first) & m
                if local > num_points or (not inclusive and local == num_points):
                    done = True
                    break
                out.append(local)
            if done:
                break
    return sorted(out)


LAZ_BASE_BYTES = {0: 20, 1: 28, 2: 26, 3: 34, 6: 30, 7: 36, 8: 38}


def _mix(seed: int, i: np.ndarray, lane: int) -> np.ndarray:
    """splitmix64 of (seed, index, lane): integer-only, the same on every host."""
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + i.astype(np.uint64) * np.uint64(0xBF58476D1CE4E5B9)
             + np.uint64(lane) * np.uint64(0x94D049BB133111EB))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def laz_records(fmt: int, n: int, seed: int, extra: int = 0) -> tuple[np.ndarray, int]:
    """LAS point format 0-3 records (plus `extra` bytes) whose every field
    varies the way scans do: coordinates as random walks, intensity drifting,
    runs of equal return bytes, classes and source IDs, scan angle steps, GPS
    times rising with repeats and jumps (so LASzip's four time sequences and
    full 64-bit codes are used), 8- and 16-bit and grey colours.  Integer-only
    arithmetic: the same bytes on every host.  -> (records uint8, bpp)."""
    if fmt >= 6:
        return _laz_records14(fmt, n, seed, extra)
    bpp = LAZ_BASE_BYTES[fmt] + extra
    i = np.arange(n, dtype=np.uint64)
    h = [_mix(seed, i, lane) for lane in range(16)]
    out = np.zeros((n, bpp), np.uint8)
    step = lambda hh, r: (hh % np.uint64(2 * r + 1)).astype(np.int64) - r
    xyz = np.stack([1_000_000 + np.cumsum(step(h[0], 1000)), 2_000_000 + np.cumsum(step(h[1], 1000)),
                    50_000 + np.cumsum(step(h[2], 120))], axis=1).astype("<i4")
    out[:, :12] = xyz.view(np.uint8).reshape(n, 12)
    inten = (30000 + np.cumsum(step(h[3], 40))) % 65536
    out[:, 12:14] = inten.astype("<u2").view(np.uint8).reshape(n, 2)
    nret = 1 + (h[4] % np.uint64(5)).astype(np.int64)
    ret = np.minimum(1 + (h[5] % np.uint64(5)).astype(np.int64), nret)
    flags = (ret | (nret << 3) | ((h[6] & np.uint64(1)).astype(np.int64) << 6)
             | ((h[6] % np.uint64(97) == 0).astype(np.int64) << 7)).astype(np.uint8)
    keep = (h[7] % np.uint64(10)) < 7
    flags[keep] = flags[0]
    out[:, 14] = flags
    out[:, 15] = (_mix(seed, i // np.uint64(100), 20) % np.uint64(20)).astype(np.uint8)
    out[:, 16] = (np.cumsum(step(h[8], 1)) % 256).astype(np.uint8)
    ud = (h[9] % np.uint64(256)).astype(np.uint8)
    ud[(h[10] % np.uint64(20)) != 0] = 7
    out[:, 17] = ud
    out[:, 18:20] = (_mix(seed, i // np.uint64(5000), 21) % np.uint64(65536)).astype("<u2") \
        .view(np.uint8).reshape(n, 2)
    off = 20
    if fmt in (1, 3):
        ticks = (100_000 << 20) + np.cumsum((h[11] % np.uint64(64)).astype(np.int64))
        jump = (h[12] % np.uint64(997)) == 0
        ticks[jump] += ((h[13][jump] % np.uint64(2 << 34)).astype(np.int64) - (1 << 34))
        same = (h[12] % np.uint64(20)) == 1
        ticks[same] = ticks[0]
        t = ticks.astype(np.float64) / float(1 << 20)
        out[:, off:off + 8] = t.astype("<f8").view(np.uint8).reshape(n, 8)
        off += 8
    if fmt in (2, 3):
        rgb = np.stack([(h[14] >> np.uint64(8 * k)) % np.uint64(256) for k in range(3)], axis=1)
        wide = (h[15] % np.uint64(8)) != 0
        rgb[wide] *= np.uint64(256)
        grey = (h[15] % np.uint64(5)) == 0
        rgb[grey, 1] = rgb[grey, 0]
        rgb[grey, 2] = rgb[grey, 0]
        out[:, off:off + 6] = rgb.astype("<u2").view(np.uint8).reshape(n, 6)
        off += 6
    if extra:
        out[:, off:] = ((i[:, None] // np.uint64(7) + np.arange(extra, dtype=np.uint64)[None, :] * np.uint64(3))
                        % np.uint64(256)).astype(np.uint8)
    return out.reshape(-1), bpp


def _laz_records14(fmt: int, n: int, seed: int, extra: int) -> tuple[np.ndarray, int]:
    """LAS 1.4 point format 6/7/8 records for laz_records: pulses of 1-5
    returns (a few of up to 15, a few with return 0 or past the count) sharing
    one GPS time, runs on all four scanner channels with single-point
    switches, classes past 31, classification flags, negative scan angles."""
    bpp = LAZ_BASE_BYTES[fmt] + extra
    i = np.arange(n, dtype=np.uint64)
    h = [_mix(seed, i, lane) for lane in range(20)]
    step = lambda hh, r: (hh % np.uint64(2 * r + 1)).astype(np.int64) - r
    out = np.zeros((n, bpp), np.uint8)
    xyz = np.stack([5_000_000 + np.cumsum(step(h[0], 900)), -3_000_000 + np.cumsum(step(h[1], 900)),
                    20_000 + np.cumsum(step(h[2], 150))], axis=1).astype("<i4")
    out[:, :12] = xyz.view(np.uint8).reshape(n, 12)
    out[:, 12:14] = ((20000 + np.cumsum(step(h[3], 60))) % 65536).astype("<u2").view(np.uint8).reshape(n, 2)
    # pulses: a new pulse where the hash says so; return numbers count up inside it
    start = (h[4] % np.uint64(3)) == 0
    start[0] = True
    pulse = np.cumsum(start) - 1
    first_idx = np.nonzero(start)[0]
    r = (np.arange(n) - first_idx[pulse]) + 1
    sizes = np.diff(np.append(first_idx, n))
    nret = sizes[pulse]
    big = (_mix(seed, pulse.astype(np.uint64), 30) % np.uint64(50)) == 0
    nret = np.where(big, np.minimum(nret + 9, 15), nret)
    odd = (h[5] % np.uint64(97)) == 0
    r = np.where(odd, (h[6] % np.uint64(16)).astype(np.int64), r)
    r, nret = np.minimum(r, 15), np.minimum(nret, 15)
    out[:, 14] = (r | (nret << 4)).astype(np.uint8)
    run = _mix(seed, i // np.uint64(777), 31) % np.uint64(4)
    flip = (h[7] % np.uint64(211)) == 0
    channel = np.where(flip, (run + np.uint64(1) + h[8] % np.uint64(3)) % np.uint64(4), run).astype(np.int64)
    cflags = np.where((h[9] % np.uint64(50)) == 0, (h[10] % np.uint64(16)).astype(np.int64), 0)
    sdir = (_mix(seed, i // np.uint64(300), 32) & np.uint64(1)).astype(np.int64)
    edge = ((h[11] % np.uint64(400)) == 0).astype(np.int64)
    out[:, 15] = (cflags | (channel << 4) | (sdir << 6) | (edge << 7)).astype(np.uint8)
    cls = (_mix(seed, i // np.uint64(150), 33) % np.uint64(8)).astype(np.int64)
    cls = np.choose(cls, [2, 2, 3, 5, 6, 40, 64, 200])
    out[:, 16] = cls.astype(np.uint8)
    out[:, 17] = np.where((h[12] % np.uint64(30)) == 0, (h[13] % np.uint64(256)).astype(np.int64), 9) \
        .astype(np.uint8)
    angle = (np.cumsum(step(h[14], 3)) % 60001) - 30000
    angle = np.where((h[15] % np.uint64(4)) == 0, angle, np.roll(angle, 1))
    out[:, 18:20] = angle.astype("<i2").view(np.uint8).reshape(n, 2)
    out[:, 20:22] = (_mix(seed, i // np.uint64(4000), 34) % np.uint64(65536)).astype("<u2") \
        .view(np.uint8).reshape(n, 2)
    pticks = (300_000 << 20) + np.cumsum((_mix(seed, np.arange(len(first_idx), dtype=np.uint64), 35)
                                          % np.uint64(4096)).astype(np.int64))
    ticks = pticks[pulse]
    jump = (h[16] % np.uint64(1499)) == 0
    ticks[jump] += ((h[17][jump] % np.uint64(2 << 36)).astype(np.int64) - (1 << 36))
    out[:, 22:30] = (ticks.astype(np.float64) / float(1 << 20)).astype("<f8").view(np.uint8).reshape(n, 8)
    off = 30
    if fmt in (7, 8):
        rgb = np.stack([(h[18] >> np.uint64(8 * k)) % np.uint64(256) for k in range(4)], axis=1)
        wide = (h[19] % np.uint64(8)) != 0
        rgb[wide] *= np.uint64(256)
        grey = (h[19] % np.uint64(5)) == 0
        rgb[grey, 1] = rgb[grey, 0]
        rgb[grey, 2] = rgb[grey, 0]
        k = 3 if fmt == 7 else 4
        out[:, off:off + 2 * k] = rgb[:, :k].astype("<u2").view(np.uint8).reshape(n, 2 * k)
        off += 2 * k
    if extra:
        out[:, off:] = ((i[:, None] // np.uint64(5) + np.arange(extra, dtype=np.uint64)[None, :] * np.uint64(7))
                        % np.uint64(256)).astype(np.uint8)
    return out.reshape(-1), bpp


LAZ_SCALE, LAZ_OFFSET = (0.001, 0.001, 0.001), (0.0, 0.0, 0.0)


def laz_box(records: np.ndarray, n: int, bpp: int):
    xyz = records.reshape(n, bpp)[:, :12].copy().view("<i4").reshape(n, 3).astype(np.float64) * 0.001
    return tuple(xyz.min(0)), tuple(xyz.max(0))


def laszip_file(records: np.ndarray, n: int, fmt: int, bpp: int, chunk: int = 50000, var_every: int = 0,
                compressor: int = 2, item_version: int = 0) -> bytes:
    """A LAZ file whose point data LASzip itself wrote (the reference's vendored
    codec built into oracle/_ref), under the same LAS header and VLR framing
    as compute_rasterizer_gb300.las.laz_bytes."""
    from compute_rasterizer_gb300 import las
    if fmt >= 6 and compressor == 2:
        compressor = 3  # LAS 1.4 points take LASzip's layered coder
    lz = O.laszipref()
    vlr = np.zeros(256, np.uint8)
    vn = lz.lzref_vlr(fmt, bpp, compressor, chunk & 0xFFFFFFFF, item_version, vlr.ctypes.data, 256)
    assert vn > 0
    bmin, bmax = laz_box(records, n, bpp)
    head = las._header(n, LAZ_SCALE, LAZ_OFFSET, bmin, bmax, fmt | 128, bpp, (1, 4) if fmt >= 6 else (1, 2),
                       [("laszip encoder", 22204, vlr[:vn].tobytes())])
    pre = np.frombuffer(head, np.uint8).copy()
    rec = np.ascontiguousarray(records, np.uint8)
    out = np.zeros(n * bpp * 2 + 65536, np.uint8)
    size = lz.lzref_compress(pre.ctypes.data, pre.size, rec.ctypes.data, n, fmt, bpp, compressor,
                             chunk & 0xFFFFFFFF, item_version, var_every, out.ctypes.data, out.size)
    assert size > 0, size
    return out[:size].tobytes()
