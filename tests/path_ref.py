"""CPU restatement of the path-tracing layer (test infrastructure): the same
hashed random numbers, jittered primary rays, Lambertian scatter, sky and
albedos as ho_path.cu, with every bounce's rays traced by the oracle (FP32).
It follows the reference's render loop (FEM-AABB/raytracer.cu:410-476,
ray_color :362-406, scatter :60-98)."""
from __future__ import annotations

import numpy as np

M32 = np.uint64(0xFFFFFFFF)


def pcg_hash(v):
    """Jarzynski and Olano's PCG hash, on uint32 arrays."""
    v = np.asarray(v, np.uint64) & M32
    state = (v * np.uint64(747796405) + np.uint64(2891336453)) & M32
    word = (((state >> ((state >> np.uint64(28)) + np.uint64(4))) ^ state) * np.uint64(277803737)) & M32
    return ((word >> np.uint64(22)) ^ word) & M32


def path_u01(key, bounce, dim):
    h = pcg_hash(pcg_hash((np.asarray(key, np.uint64) + pcg_hash(np.uint64(bounce * 8 + dim))) & M32)
                 ^ np.uint64(0x85EBCA6B))
    return (h >> np.uint64(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)


def path_key(path, seed):
    s_lo = np.uint64(seed & 0xFFFFFFFF)
    s_hi = np.uint64((seed >> 32) & 0xFFFFFFFF)
    return (pcg_hash((np.asarray(path, np.uint64) & M32) ^ pcg_hash(s_lo ^ np.uint64(0x9E3779B9))) ^ s_hi) & M32


def camera_basis(cam, W, H):
    """origin, lower-left corner, horizontal and vertical spans (float32)."""
    f = np.float32
    lookfrom, lookat, vup = (np.asarray(x, f) for x in (cam.lookfrom, cam.lookat, cam.vup))
    theta = f(cam.vfov_deg) * f(3.14159265) / f(180.0)
    h = f(np.tan(theta / f(2.0)))
    vh = f(2.0) * h
    vw = f(W) / f(H) * vh
    w = lookfrom - lookat
    focus = f(np.sqrt((w * w).sum()))
    w = w * (f(1.0) / focus)
    u = np.cross(vup, w).astype(f)
    u = u * (f(1.0) / f(np.sqrt((u * u).sum())))
    v = np.cross(w, u).astype(f)
    horiz = focus * vw * u
    vert = focus * vh * v
    llc = lookfrom - horiz / f(2.0) - vert / f(2.0) - focus * w
    return lookfrom, llc, horiz, vert


def path_trace(osc, cam, W, H, iso, iso_on, spp, max_depth, seed):
    """Image (H, W, 3) uint8 and the ray queries traced."""
    npix = W * H
    o, llc, horiz, vert = camera_basis(cam, W, H)
    accum = np.zeros((npix, 3), np.float64)
    pix_all = np.arange(npix)
    x = (pix_all % W).astype(np.float32)
    y = (pix_all // W).astype(np.float32)
    traced = 0
    for sample in range(spp):
        key = path_key(pix_all.astype(np.uint64) + np.uint64(npix * sample), seed)
        u = (x + path_u01(key, 0, 0)) / np.float32(W)
        v = (y + path_u01(key, 0, 1)) / np.float32(H)
        d = llc[None, :] + u[:, None] * horiz[None, :] + v[:, None] * vert[None, :] - o[None, :]
        d = d / np.sqrt((d * d).sum(axis=1))[:, None]
        rays = np.concatenate([np.broadcast_to(o, d.shape), d], axis=1).astype(np.float32)
        att = np.ones((npix, 3), np.float64)
        pix = pix_all.copy()
        for bounce in range(max_depth):
            if rays.shape[0] == 0:
                break
            hits, _ = osc.trace(rays, iso, iso_on, precision=32)
            traced += rays.shape[0]
            miss = hits["kind"] == 0
            dm = rays[miss, 3:].astype(np.float64)
            un = dm / np.sqrt((dm * dm).sum(axis=1))[:, None]
            t = 0.5 * (un[:, 1] + 1.0)
            sky = np.stack([(1 - t) + t * 0.5, (1 - t) + t * 0.7, (1 - t) + t * 1.0], axis=1)
            np.add.at(accum, pix[miss], att[miss] * sky)
            hit = ~miss
            blue = (hits["kind"] == 1) & (hits["face"] == 0)
            alb = np.where(blue[:, None], np.array([0.1, 0.2, 0.8]), 0.5)
            att = att * alb
            if bounce + 1 >= max_depth:
                break
            keep = hit
            rd = rays[keep, 3:].astype(np.float64)
            ro = rays[keep, :3].astype(np.float64)
            th = hits["t"][keep][:, None]
            n = hits["n"][keep].copy()
            flip = (n * rd).sum(axis=1) > 0
            n[flip] = -n[flip]
            k = key[keep]
            z = 1.0 - 2.0 * path_u01(k, bounce + 1, 0).astype(np.float64)
            rr = np.sqrt(np.maximum(0.0, 1.0 - z * z))
            phi = 2.0 * np.pi * path_u01(k, bounce + 1, 1).astype(np.float64)
            dn = n + np.stack([rr * np.cos(phi), rr * np.sin(phi), z], axis=1)
            small = (dn * dn).sum(axis=1) < 1e-12
            dn[small] = n[small]
            rays = np.concatenate([ro + th * rd, dn], axis=1).astype(np.float32)
            att = att[keep]
            pix = pix[keep]
            key = k
    img = np.minimum(1.0, np.sqrt(accum / spp))
    return (255.99 * img).astype(np.uint8).reshape(H, W, 3), traced
