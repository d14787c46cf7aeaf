"""Seeded workloads of the benchmark configurations (seeds: scene 1,
colours 2, edits 3, cameras 4, serving trace 5).

Cameras are built as the reference's get_trace_params (dag_tracer.cu:71-113)
builds Tracer::TracePathsParams, with the scene's bounding box equal to the
voxel cube [0, 2^depth]^3 so that world and voxel space coincide.
"""
import math

import numpy as np

from . import scene

SEED_SCENE, SEED_COLORS, SEED_EDITS, SEED_CAMERAS, SEED_SERVING = 1, 2, 3, 4, 5

SPHERE_REMOVE, SPHERE_ADD, BOX_REMOVE, BOX_ADD = 0, 1, 2, 3


def color_tree_levels(depth):
    """C_colorTreeLevels per depth: the reference's 10, lowered on shallow
    scenes where 10 would reach the leaf level."""
    return min(10, depth - 5)


def top_bucket_bits(depth):
    """BUCKETS_BITS_FOR_TOP_LEVELS: the reference's 10, raised to 12 on scenes
    of depth 11 to 15 whose level 8 holds over 10^5 nodes, and to 14 from depth
    16 (over 5 * 10^5 nodes at level 8)."""
    return 10 if depth <= 10 else (12 if depth <= 15 else 14)


def low_bucket_bits(depth):
    """BUCKETS_BITS_FOR_LOW_LEVELS: the reference's 16, raised to 17 from depth
    16, where the shell scene's lowest interior level would average more
    than the 4096 words a bucket holds."""
    return 16 if depth <= 15 else 17


# ---------------------------------------------------------------- cameras --

def _norm(v):
    v = np.asarray(v, np.float64)
    return v / math.sqrt(float(v @ v))


def trace_params(position, target, width, height, fov_deg=90.0, up=(0.0, 1.0, 0.0)):
    """get_trace_params (dag_tracer.cu:71-113) for a camera at `position`
    looking at `target`; returns dict(position, ray_min, ray_ddx, ray_ddy)."""
    position = np.asarray(position, np.float64)
    forward = _norm(np.asarray(target, np.float64) - position)
    right = _norm(np.cross(forward, np.asarray(up, np.float64)))
    upv = np.cross(right, forward)
    fov = fov_deg / 2.0 * (math.pi / 180.0)
    aspect = float(width) / float(height)
    X = right * math.sin(fov) * aspect
    Y = upv * math.sin(fov)
    Z = forward * math.cos(fov)
    bottom_left = position + Z - Y - X
    bottom_right = position + Z - Y + X
    top_left = position + Z + Y - X
    dx = (bottom_right - bottom_left) * (1.0 / width)
    dy = (top_left - bottom_left) * (1.0 / height)
    return dict(position=position.tolist(), ray_min=bottom_left.tolist(), ray_ddx=dx.tolist(),
                ray_ddy=dy.tolist())


def orbit_camera(depth, width, height, seed=SEED_CAMERAS):
    """One seeded pose at distance 1.5 E from the centre, outside the box,
    looking at the centre (90 degree FOV)."""
    rng = np.random.default_rng(seed)
    e = float(1 << depth)
    centre = np.array([e / 2, e / 2, e / 2])
    theta = rng.uniform(0, 2 * math.pi)
    elev = rng.uniform(0.15, 0.6)
    d = np.array([math.cos(theta) * math.cos(elev), math.sin(elev), math.sin(theta) * math.cos(elev)])
    return trace_params(centre + 1.5 * e * d, centre, width, height)


def catmull_rom_path(depth, n_poses, width, height, seed=SEED_CAMERAS):
    """n_poses cameras on a closed Catmull-Rom spline through 8 seeded
    control points outside the bounding box, looking at points near the
    centre."""
    rng = np.random.default_rng(seed)
    e = float(1 << depth)
    centre = np.array([e / 2, e / 2, e / 2])
    ctrl = []
    for k in range(8):
        theta = 2 * math.pi * k / 8 + rng.uniform(-0.3, 0.3)
        elev = rng.uniform(0.1, 0.7)
        dist = rng.uniform(0.9, 1.4) * e
        ctrl.append(centre + dist * np.array([math.cos(theta) * math.cos(elev), math.sin(elev),
                                              math.sin(theta) * math.cos(elev)]))
    ctrl = np.array(ctrl)
    looks = centre + rng.uniform(-0.15, 0.15, (8, 3)) * e
    poses = []
    for i in range(n_poses):
        u = 8.0 * i / n_poses
        k = int(u)
        t = u - k
        p0, p1, p2, p3 = (ctrl[(k + j) % 8] for j in (-1, 0, 1, 2))
        pos = 0.5 * ((2 * p1) + (-p0 + p2) * t + (2 * p0 - 5 * p1 + 4 * p2 - p3) * t * t +
                     (-p0 + 3 * p1 - 3 * p2 + p3) * t ** 3)
        look = looks[k] * (1 - t) + looks[(k + 1) % 8] * t
        poses.append(trace_params(pos, look, width, height))
    return poses


# ------------------------------------------------------------------ edits --

def _centres(depth, n, rng):
    pts = scene.surface_points(SEED_SCENE, depth, n, rng).astype(np.float64)
    return pts + 0.5


def carve_edits(depth, n=16, r_range=(16.0, 48.0), seed=SEED_EDITS):
    """Sphere carves with uniform radius centred on seeded surface voxels."""
    rng = np.random.default_rng(seed)
    c = _centres(depth, n, rng)
    r = rng.uniform(r_range[0], r_range[1], n)
    return [(SPHERE_REMOVE, tuple(float(np.float32(v)) for v in c[i]), float(np.float32(r[i]))) for i in range(n)]


def mixed_edits(depth, n, r_range=(4.0, 512.0), seed=SEED_EDITS, mix=(0.5, 0.3, 0.2)):
    """Batch mix: 50% sphere carve, 30% sphere fill, 20% box fill, radius
    log-uniform in r_range, centres on seeded surface voxels."""
    rng = np.random.default_rng(seed)
    c = _centres(depth, n, rng)
    lr = rng.uniform(math.log(r_range[0]), math.log(r_range[1]), n)
    u = rng.uniform(0, 1, n)
    tools = np.where(u < mix[0], SPHERE_REMOVE, np.where(u < mix[0] + mix[1], SPHERE_ADD, BOX_ADD))
    return [(int(tools[i]), tuple(float(np.float32(v)) for v in c[i]), float(np.float32(math.exp(lr[i]))))
            for i in range(n)]


def paint_copy_edits(depth, n_paint=512, n_copy=32, paint_r=(8.0, 256.0), copy_radius=128.0, copy_offset=2048,
                     seed=SEED_EDITS):
    """Colours / copy workload: n_paint sphere paints (radius log-uniform in
    paint_r, random RGB8 target) centred on surface voxels, then n_copy copies
    of a (2 * copy_radius)^3 region around a surface voxel moved by a seeded
    integer offset in [-copy_offset, copy_offset]^3 (both regions kept inside
    the volume).  Tuples: (tool, centre, radius, rgb) / (tool, centre, radius,
    source, dest)."""
    rng = np.random.default_rng(seed + 100)
    e = float(1 << depth)
    c = _centres(depth, n_paint + n_copy, rng)
    out = []
    lr = rng.uniform(math.log(paint_r[0]), math.log(paint_r[1]), n_paint)
    rgb = rng.integers(0, 1 << 24, n_paint)
    for i in range(n_paint):
        out.append((4, tuple(float(np.float32(v)) for v in c[i]), float(np.float32(math.exp(lr[i]))), int(rgb[i])))
    lo, hi = copy_radius + 1, e - copy_radius - 1
    for i in range(n_copy):
        src = np.clip(np.floor(c[n_paint + i]), lo, hi)
        off = rng.integers(-copy_offset, copy_offset + 1, 3).astype(np.float64)
        dst = np.clip(src + off, lo, hi)
        out.append((5, tuple(float(v) for v in src), float(copy_radius), (0.0, 0.0, 0.0),
                    tuple(float(v) for v in dst - src)))
    return out


def noise_fill_edits(depth, n_noise=64, n_fill=32, noise_r=(8.0, 64.0), fill_r=(8.0, 48.0), seed=SEED_EDITS):
    """Noise spheres (SphereNoiseEditor adding, radius log-uniform in noise_r)
    centred on surface voxels, then flood fills (radius log-uniform in
    fill_r) started 3 voxels above surface voxels.  Tuples (tool, centre,
    radius); tools 7 (noise, adding) and 8 (fill)."""
    rng = np.random.default_rng(seed + 200)
    c = _centres(depth, n_noise + n_fill, rng)
    out = []
    lr = rng.uniform(math.log(noise_r[0]), math.log(noise_r[1]), n_noise)
    for i in range(n_noise):
        out.append((7, tuple(float(np.float32(v)) for v in c[i]), float(np.float32(math.exp(lr[i])))))
    lf = rng.uniform(math.log(fill_r[0]), math.log(fill_r[1]), n_fill)
    for i in range(n_fill):
        p = c[n_noise + i] + np.array([0.0, 3.0, 0.0])
        out.append((8, tuple(float(np.float32(v)) for v in p), float(np.float32(math.exp(lf[i])))))
    return out


def replay_text(depth, n_frames, edits_per_frame=2, replay_depth=16, seed=SEED_EDITS):
    """A replay in the reference's CSV format (replay.h): n_frames frames,
    each a camera pose and edits_per_frame sphere carves / fills, positions
    and radii recorded at replay_depth (scaled to depth on replay)."""
    rng = np.random.default_rng(seed + 300)
    s = float(1 << replay_depth) / float(1 << depth)
    c = _centres(depth, n_frames * edits_per_frame, rng)
    lines = []
    for f in range(n_frames):
        a = 2 * math.pi * f / max(1, n_frames)
        lines.append("SetLocation,%f,%f,%f" % (50 + 80 * math.cos(a), 70.0, 50 + 80 * math.sin(a)))
        fwd = _norm(np.array([50.0, 50.0, 50.0]) - np.array([50 + 80 * math.cos(a), 70.0, 50 + 80 * math.sin(a)]))
        right = _norm(np.cross(fwd, [0.0, 1.0, 0.0]))
        up = np.cross(right, fwd)
        lines.append("SetRotation," + ",".join("%f" % v for v in list(-right) + list(up) + list(fwd)))
        for k in range(edits_per_frame):
            p = c[f * edits_per_frame + k] * s
            r = float(rng.uniform(8, 48)) * s
            lines.append("EditSphere,%f,%f,%f,%f,%s" % (p[0], p[1], p[2], r, "true" if k % 2 else "false"))
        lines.append("EndFrame")
    return "\n".join(lines) + "\n"


RESOLUTIONS = ((1280, 720), (1920, 1080), (3840, 2160))


def serving_trace(depth, n, rate_per_s, seed=SEED_SERVING, edit_fraction=0.7, r_range=(4.0, 1024.0),
                  resolutions=RESOLUTIONS, poses=64):
    """Poisson arrivals at rate_per_s: edit_fraction edits (sphere carve,
    sphere fill, sphere paint in equal parts; radius log-uniform in r_range;
    centres on surface voxels; random paint colour), the rest renders at a
    seeded resolution and a seeded pose of the Catmull-Rom path.  Returns
    (kind, arrival_ms, payload) tuples: ("edit", t, (tool, centre, radius,
    rgb)) / ("render", t, (width, height, camera params))."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1000.0 / rate_per_s, n))
    kinds = rng.uniform(0, 1, n) < edit_fraction
    c = _centres(depth, n, rng)
    lr = rng.uniform(math.log(r_range[0]), math.log(r_range[1]), n)
    tools = rng.choice([SPHERE_REMOVE, SPHERE_ADD, 4], n)
    rgb = rng.integers(0, 1 << 24, n)
    res = rng.integers(0, len(resolutions), n)
    pose = rng.integers(0, poses, n)
    cams = {}
    out = []
    for i in range(n):
        if kinds[i]:
            out.append(("edit", float(t[i]), (int(tools[i]), tuple(float(np.float32(v)) for v in c[i]),
                                              float(np.float32(math.exp(lr[i]))), int(rgb[i]))))
        else:
            w, h = resolutions[res[i]]
            if (w, h) not in cams:
                cams[(w, h)] = catmull_rom_path(depth, poses, w, h)
            out.append(("render", float(t[i]), (w, h, cams[(w, h)][pose[i]])))
    return out
