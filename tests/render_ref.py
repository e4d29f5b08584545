"""float32 numpy restatement of pcisph_render (test reference for tests/test_gpu_render.py): per pixel, the
nearest ray-sphere hit over all particles (ties to the lower index), shaded with the density colour map,
+y lighting with 0.2 ambient, and the 5..20 depth falloff."""
import numpy as np

f32 = np.float32


def basis(cam):
    eye, target, up = (np.array(v, np.float32) for v in (cam.eye, cam.target, cam.up))
    fwd = target - eye
    fwd = fwd / np.linalg.norm(fwd)
    right = np.cross(fwd, up)
    right = right / np.linalg.norm(right)
    return eye, right.astype(f32), np.cross(right, fwd).astype(f32), fwd.astype(f32)


def render(pos, density, radius, rest_density, cam, width, height):
    eye, right, up, fwd = basis(cam)
    tx = f32(np.tan(0.5 * cam.fov_x_degrees * np.pi / 180.0))
    ty = tx * f32(height) / f32(width)
    d = pos[:, :3].astype(f32) - eye
    v = np.stack([d @ right, d @ up, d @ fwd], 1).astype(f32)
    px, py = np.meshgrid(np.arange(width), np.arange(height))
    nx = ((px + f32(0.5)) / f32(width)) * f32(2) - f32(1)
    ny = f32(1) - ((py + f32(0.5)) / f32(height)) * f32(2)
    r = np.stack([nx * tx, ny * ty, np.ones_like(nx, dtype=f32)], -1).astype(f32)   # (h, w, 3)
    rr = (r * r).sum(-1)[..., None]
    rs = np.einsum("hwc,nc->hwn", r, v)
    ss = (v * v).sum(-1)[None, None, :]
    disc = rs * rs - rr * (ss - f32(radius) ** 2)
    t = np.where(disc >= 0, (rs - np.sqrt(np.maximum(disc, 0))) / rr, np.inf)
    t = np.where((t > 0) & (v[None, None, :, 2] > radius), t, np.inf)
    best = np.argmin(t, -1)
    tb = np.take_along_axis(t, best[..., None], -1)[..., 0]
    out = np.zeros((height, width, 3), np.float32)
    hitmask = np.isfinite(tb)
    tb = np.where(hitmask, tb, 0).astype(np.float32)
    c = v[best]
    h = r * tb[..., None] - c
    nrm_y = (h[..., 0] * right[1] + h[..., 1] * up[1] + h[..., 2] * fwd[1]) / f32(radius)
    rho = density[best] if density is not None else np.full(best.shape, rest_density, np.float32)
    cmax, cneu, cmin = np.array([1, .3, 0], f32), np.array([.5, .3, .5], f32), np.array([0, .3, 1], f32)
    hi = np.clip((rho - rest_density) / (f32(1.05) * rest_density - rest_density), 0, 1)[..., None]
    lo = np.clip((rho - f32(0.95) * rest_density) / (rest_density - f32(0.95) * rest_density), 0, 1)[..., None]
    diffuse = np.where((rho > rest_density)[..., None], cneu + (cmax - cneu) * hi, cmin + (cneu - cmin) * lo)
    light = np.maximum(0, nrm_y)[..., None]
    fall = (1 - (tb - 5) / 15)[..., None]
    out = np.where(hitmask[..., None], (light * diffuse + f32(0.2)) * fall, 0)
    return (np.clip(out, 0, 1) * 255 + 0.5).astype(np.uint8)
