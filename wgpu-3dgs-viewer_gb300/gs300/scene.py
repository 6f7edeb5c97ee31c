"""Seeded synthetic scenes and orbit cameras.

The distributions are the ones the render-path benchmarks are quoted on: positions N(0, 2²)
per axis, log-scales N(-4, 0.5²) per axis, uniform random unit quaternions (normalised
N(0, 1)⁴), opacity sigmoid(N(0, 1)), SH degree 3 with DC ~ N(0.5, 0.2²) and the 45 higher
coefficients ~ N(0, 0.05²).  The DC term and opacity are folded into the record's RGBA8 colour
as the reference model does (rgb = 0.5 + SH_C0·dc, src/shader/utils.wesl:94).
"""
import math

import numpy as np

from .records import (
    FORMAT_FP32,
    FORMAT_HALF_SH_BF16,
    FORMAT_HALF_SH_FP16,
    GAUSSIAN_DTYPE,
    GAUSSIAN_POD_DTYPE,
    GAUSSIAN_POD_HALF_DTYPE,
    Camera,
)

SH_C0 = 0.28209479177387814


def quat_to_mat(q):
    """(..., 4) quaternions x, y, z, w -> (..., 3, 3) rotation matrices (float64)."""
    q = np.asarray(q, dtype=np.float64)
    x, y, z, w = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    m = np.empty(q.shape[:-1] + (3, 3))
    m[..., 0, 0] = 1 - 2 * (y * y + z * z)
    m[..., 0, 1] = 2 * (x * y - w * z)
    m[..., 0, 2] = 2 * (x * z + w * y)
    m[..., 1, 0] = 2 * (x * y + w * z)
    m[..., 1, 1] = 1 - 2 * (x * x + z * z)
    m[..., 1, 2] = 2 * (y * z - w * x)
    m[..., 2, 0] = 2 * (x * z - w * y)
    m[..., 2, 1] = 2 * (y * z + w * x)
    m[..., 2, 2] = 1 - 2 * (x * x + y * y)
    return m


def cov3d_from(rot, scale):
    """Unique entries (xx, xy, xz, yy, yz, zz) of R·S·Sᵀ·Rᵀ, float64."""
    r = quat_to_mat(rot)
    m = r * np.asarray(scale, dtype=np.float64)[..., None, :]
    s = m @ np.swapaxes(m, -1, -2)
    return np.stack([s[..., 0, 0], s[..., 0, 1], s[..., 0, 2], s[..., 1, 1], s[..., 1, 2], s[..., 2, 2]], axis=-1)


def pack_color(rgba_u8):
    c = np.asarray(rgba_u8, dtype=np.uint32)
    return c[..., 0] | (c[..., 1] << 8) | (c[..., 2] << 16) | (c[..., 3] << 24)


def pack_gaussians(gaussians):
    """core::Gaussian records (GAUSSIAN_DTYPE) -> gs_gaussian_pod records."""
    g = np.asarray(gaussians, dtype=GAUSSIAN_DTYPE)
    out = np.zeros(g.shape, dtype=GAUSSIAN_POD_DTYPE)
    out["pos"] = g["pos"]
    out["color"] = pack_color(g["color"])
    out["sh"] = g["sh"]
    out["cov3d"] = cov3d_from(g["rot"], g["scale"]).astype(np.float32)
    return out


def pack_gaussians_half(gaussians, fmt):
    """core::Gaussian records -> gs_gaussian_pod_half records (rotation, scale to binary16; SH to
    binary16 or bfloat16; round to nearest even)."""
    g = np.asarray(gaussians, dtype=GAUSSIAN_DTYPE)
    out = np.zeros(g.shape, dtype=GAUSSIAN_POD_HALF_DTYPE)
    out["pos"] = g["pos"]
    out["color"] = pack_color(g["color"])
    out["rot"] = g["rot"].astype(np.float16).view(np.uint16)
    out["scale"] = g["scale"].astype(np.float16).view(np.uint16)
    if fmt == FORMAT_HALF_SH_FP16:
        out["sh"] = g["sh"].astype(np.float16).view(np.uint16)
    elif fmt == FORMAT_HALF_SH_BF16:
        out["sh"] = _f32_to_bf16_bits(g["sh"])
    else:
        raise ValueError(f"not a half record format: {fmt}")
    return out


def gaussian(pos=(0.0, 0.0, 1.0), rot=(0.0, 0.0, 0.0, 1.0), color=(255, 0, 0, 255), scale=(1.0, 1.0, 1.0), sh=None):
    """One core::Gaussian, defaulting to the reference tests' red Gaussian (tests/e2e/viewer.rs:74-80)."""
    g = np.zeros((), dtype=GAUSSIAN_DTYPE)
    g["pos"] = pos
    g["rot"] = rot
    g["color"] = color
    g["scale"] = scale
    if sh is not None:
        g["sh"] = np.asarray(sh, dtype=np.float32).reshape(45)
    return g


def _f32_to_bf16_bits(x):
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    return r.astype(np.uint16)


def synth_attributes(n, seed, translate_fraction=0.0, translate_std=0.1):
    """Raw attributes of a seeded scene (float32 arrays, uint8 colours)."""
    rng = np.random.default_rng(seed)
    pos = rng.normal(0.0, 2.0, size=(n, 3)).astype(np.float32)
    log_scale = rng.normal(-4.0, 0.5, size=(n, 3))
    scale = np.exp(log_scale).astype(np.float32)
    q = rng.normal(0.0, 1.0, size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    rot = q.astype(np.float32)
    opacity = 1.0 / (1.0 + np.exp(-rng.normal(0.0, 1.0, size=n)))
    dc = rng.normal(0.5, 0.2, size=(n, 3))
    sh = rng.normal(0.0, 0.05, size=(n, 45)).astype(np.float32)
    if translate_fraction > 0.0:
        sel = rng.random(n) < translate_fraction
        pos[sel] += rng.normal(0.0, translate_std, size=(int(sel.sum()), 3)).astype(np.float32)
    rgb = np.clip(0.5 + SH_C0 * dc, 0.0, 1.0)
    color = np.empty((n, 4), dtype=np.uint8)
    color[:, :3] = np.rint(rgb * 255.0).astype(np.uint8)
    color[:, 3] = np.rint(opacity * 255.0).astype(np.uint8)
    return {"pos": pos, "scale": scale, "rot": rot, "color": color, "sh": sh}


def synth_scene(n, seed=0, fmt=FORMAT_FP32, translate_fraction=0.0, chunk=1 << 20):
    """A seeded synthetic scene as device-ready records of format `fmt`."""
    a = synth_attributes(n, seed, translate_fraction)
    if fmt == FORMAT_FP32:
        out = np.zeros(n, dtype=GAUSSIAN_POD_DTYPE)
        out["pos"] = a["pos"]
        out["color"] = pack_color(a["color"])
        out["sh"] = a["sh"]
        for s in range(0, n, chunk):
            e = min(n, s + chunk)
            out["cov3d"][s:e] = cov3d_from(a["rot"][s:e], a["scale"][s:e]).astype(np.float32)
        return out
    out = np.zeros(n, dtype=GAUSSIAN_POD_HALF_DTYPE)
    out["pos"] = a["pos"]
    out["color"] = pack_color(a["color"])
    out["rot"] = a["rot"].astype(np.float16).view(np.uint16)
    out["scale"] = a["scale"].astype(np.float16).view(np.uint16)
    if fmt == FORMAT_HALF_SH_FP16:
        out["sh"] = a["sh"].astype(np.float16).view(np.uint16)
    elif fmt == FORMAT_HALF_SH_BF16:
        out["sh"] = _f32_to_bf16_bits(a["sh"])
    else:
        raise ValueError(f"unknown record format {fmt}")
    return out


def orbit_camera(k, radius=8.0, frames=120, pitch=0.1, yaw0=0.1, fovy_deg=60.0, z_near=0.1, z_far=1e4):
    """Camera k of an orbit around the origin: yaw_k = 2πk/frames + yaw0, looking at the origin."""
    yaw = 2.0 * math.pi * k / frames + yaw0
    fwd = np.array([math.cos(pitch) * math.sin(yaw), math.sin(pitch), math.cos(pitch) * math.cos(yaw)])
    pos = -radius * fwd
    return Camera.new(z_near, z_far, math.radians(fovy_deg), pos=tuple(float(v) for v in pos), pitch=pitch, yaw=yaw)


def random_orbit_camera(rng, radius_lo=6.0, radius_hi=12.0, pitch_max=0.3):
    """A camera on a random orbit around the origin: radius uniform in [radius_lo, radius_hi], yaw
    uniform, pitch uniform in [-pitch_max, pitch_max] (fovy 60°, z 0.1..1e4), looking at the origin."""
    radius = float(rng.uniform(radius_lo, radius_hi))
    yaw = float(rng.uniform(0.0, 2.0 * math.pi))
    pitch = float(rng.uniform(-pitch_max, pitch_max))
    fwd = np.array([math.cos(pitch) * math.sin(yaw), math.sin(pitch), math.cos(pitch) * math.cos(yaw)])
    pos = -radius * fwd
    return Camera.new(0.1, 1e4, math.radians(60.0), pos=tuple(float(v) for v in pos), pitch=pitch, yaw=yaw)


def given_camera():
    """The reference tests' camera: yaw 0.1, pitch 0.1, z 0.1..1e4, fovy 60° (tests/common/given.rs:6-12)."""
    return Camera.new(0.1, 1e4, math.radians(60.0), pos=(0.0, 0.0, 0.0), pitch=0.1, yaw=0.1)
