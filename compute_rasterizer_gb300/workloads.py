"""The benchmark workloads: synthetic clouds and cameras.

Seeded, so every run renders the same frames:
  * terrain_frame      1 view, the reference's zoom-to-cloud pose
                       (src/main.cpp:251-270), 1920x1080.
  * flight_path        5 poses along a seeded flight over a terrain, 2560x1440.
  * multiview_64       16 stereo pairs at 1440x1600 per eye (IPD 0.064 m,
                       parallel eye axes: each eye translate(-+ipd/2, 0, 0) *
                       V_head, as a headset composes them) flying over the
                       cloud + 32 random orbit poses at 512x512.
  * serving            8 resident terrains of 10-500 M points, Poisson
                       arrivals, clouds drawn Zipf(1.1), one random orbit
                       camera per request at one of five resolutions.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib as L
from . import synth


def _perspective(fovy, w, h, znear=0.1, zfar=200000.0):
    return synth.perspective(fovy, w / h, znear, zfar)


def terrain_frame(box_min, box_max, width=1920, height=1080):
    yaw, pitch, radius, target = synth.zoom_to_cloud(box_min, box_max)
    return synth.orbit_view(yaw, pitch, radius, target), _perspective(60.0, width, height), width, height


def flight_path(box_min, box_max, n=5, seed=2, width=2560, height=1440):
    """Poses along a seeded flight: orbit cameras drifting over the cloud."""
    rng = np.random.default_rng(seed)
    bmin, bmax = np.asarray(box_min, float), np.asarray(box_max, float)
    size = bmax - bmin
    cams = []
    start = bmin + size * np.array([0.2, 0.2, 0.5])
    end = bmin + size * np.array([0.8, 0.7, 0.5])
    for i in range(n):
        t = i / max(1, n - 1)
        target = start + t * (end - start)
        yaw = 0.6 + 1.5 * t + rng.uniform(-0.2, 0.2)
        pitch = -0.45 - 0.3 * rng.uniform()
        radius = float(np.linalg.norm(size[:2])) * (0.08 + 0.25 * rng.uniform())
        cams.append((synth.orbit_view(yaw, pitch, radius, target), _perspective(60.0, width, height),
                     width, height))
    return cams


def _look_dir(yaw, pitch):
    return np.array([math.cos(pitch) * math.cos(yaw), math.cos(pitch) * math.sin(yaw), math.sin(pitch)])


def eye_view(head_view, dx: float) -> np.ndarray:
    """translate(dx, 0, 0) * head_view (column-major doubles): an eye's view
    from the head's; only the x translation (element 12) changes."""
    v = np.array(head_view, dtype=np.float64).reshape(16).copy()
    v[12] = v[12] + dx
    return v


def multiview_64(box_min, box_max, seed=4, ipd=0.064, compose_eyes=True):
    """16 stereo pairs (1440x1600 per eye) + 32 random poses (512x512).
    compose_eyes=False builds each eye by look_at from its own position
    instead: the same cameras up to rounding, but the eyes' projection rows
    no longer agree bit for bit, so a multi-view plan cannot share them."""
    rng = np.random.default_rng(seed)
    bmin, bmax = np.asarray(box_min, float), np.asarray(box_max, float)
    size = bmax - bmin
    up = np.array([0.0, 0.0, 1.0])
    cams = []
    for _ in range(16):
        centre = bmin + size * np.array([rng.uniform(0.15, 0.85), rng.uniform(0.15, 0.85), 1.0])
        centre[2] = bmax[2] + rng.uniform(20.0, 150.0)
        d = _look_dir(rng.uniform(-math.pi, math.pi), rng.uniform(-0.6, -0.15))
        head = synth.look_at(centre, centre + d, up)
        right = np.cross(d, up)
        right /= np.linalg.norm(right)
        for side in (-0.5, 0.5):  # the eye at centre + side * ipd * right
            if compose_eyes:
                view = eye_view(head, -side * ipd)
            else:
                eye = centre + side * ipd * right
                view = synth.look_at(eye, eye + d, up)
            cams.append((view, _perspective(90.0, 1440, 1600), 1440, 1600))
    yaw0, pitch0, radius0, target0 = synth.zoom_to_cloud(bmin, bmax)
    for _ in range(32):
        target = bmin + size * np.array([rng.uniform(0.1, 0.9), rng.uniform(0.1, 0.9), 0.5])
        view = synth.orbit_view(rng.uniform(-math.pi, math.pi), rng.uniform(-1.3, -0.25),
                                radius0 * rng.uniform(0.1, 1.0), target)
        cams.append((view, _perspective(60.0, 512, 512), 512, 512))
    return cams


def multiview_cloud_params(seed=4, extent=4500.0):
    """Terrain plus 2000 boxes (10-60 m tall, 20k points on their faces)."""
    return synth.synth_params(L.SYNTH_TERRAIN_BOXES, extent, seed, num_boxes=2000,
                              points_per_box=20000, box_min_height=10.0, box_max_height=60.0)


SERVING_CLOUD_MPOINTS = (10, 25, 50, 100, 200, 300, 400, 500)
SERVING_RESOLUTIONS = ((256, 256), (512, 512), (1280, 720), (1920, 1080), (3840, 2160))


def serving_cloud_params(i: int, n: int):
    """Terrain i of the serving set: the 1B-point terrain's density (10 points
    per square metre), so the extent grows with sqrt(n)."""
    return synth.synth_params(L.SYNTH_TERRAIN, math.sqrt(n / 10.0), 100 + i)


def zipf_weights(k: int, s: float = 1.1) -> np.ndarray:
    w = 1.0 / np.arange(1, k + 1, dtype=np.float64) ** s
    return w / w.sum()


def serving_requests(boxes, n: int, rate: float, seed: int = 5, zipf_s: float = 1.1,
                     resolutions=SERVING_RESOLUTIONS):
    """n requests with Poisson arrivals at `rate` per second.

    boxes: [(box_min, box_max)] of the resident clouds, most popular first.
    Returns (arrival_us[n], cameras) with cameras[i] = (cloud, view, proj, W, H).
    """
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1e6 / rate, size=n)
    arrival = np.cumsum(gaps) - gaps[0]
    clouds = rng.choice(len(boxes), size=n, p=zipf_weights(len(boxes), zipf_s))
    res = rng.integers(0, len(resolutions), size=n)
    cams = []
    for i in range(n):
        c = int(clouds[i])
        bmin, bmax = (np.asarray(b, float) for b in boxes[c])
        _, _, radius, target = synth.zoom_to_cloud(bmin, bmax)
        w, h = resolutions[int(res[i])]
        view = synth.orbit_view(rng.uniform(-math.pi, math.pi), rng.uniform(-1.2, -0.3),
                                radius * rng.uniform(0.5, 1.2), target)
        cams.append((c, view, _perspective(60.0, w, h), w, h))
    return arrival, cams
