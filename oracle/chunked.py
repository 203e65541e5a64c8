"""A float64 PyTorch renderer that follows reference/backward_reference.py:87-157
statement by statement, but evaluates one 16x16 pixel tile at a time over only
the splats whose tile rectangle covers it. TEST INFRASTRUCTURE ONLY (it makes the
committed golden vectors; see tests/golden/make_golden.py).

Why tiles: the reference's render() is dense over pixels x splats, which at
256x256 x 16,384 Gaussians is ~8.6 GB per intermediate tensor. Restricting a
tile to its covering splats is exact: every other splat has `covered` false, so
its alpha is 0 and it multiplies the transmittance by 1, and the covering splats
keep the global stable depth order. make_golden.py checks this restatement
against the reference's own render() on scenes small enough for the dense form.
"""

from __future__ import annotations

import math

import torch
import torch.nn.functional as F

TILE = 16
NEAR_CULL = 0.2
BLUR = 0.3
SH_C1 = 0.4886025119029199
SH_C2 = [1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792, 0.5462742152789498]
SH_C3 = [-0.5900435899266435, 2.890611442640554, -0.4570457994644658, 0.3731763325901154, -0.4570457994644658,
         1.445305721320277, -0.5900435899266435]


def rotation_matrices(raw):
    w, x, y, z = (raw / raw.norm(dim=1, keepdim=True)).unbind(1)
    return torch.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
        2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
        2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y),
    ], dim=1).reshape(-1, 3, 3)


def sh_basis(d):
    x, y, z = d.unbind(1)
    xx, yy, zz = x * x, y * y, z * z
    return torch.stack([
        -SH_C1 * y, SH_C1 * z, -SH_C1 * x,
        SH_C2[0] * x * y, SH_C2[1] * y * z, SH_C2[2] * (2 * zz - xx - yy), SH_C2[3] * x * z, SH_C2[4] * (xx - yy),
        SH_C3[0] * y * (3 * xx - yy), SH_C3[1] * x * y * z, SH_C3[2] * y * (4 * zz - xx - yy),
        SH_C3[3] * z * (2 * zz - 3 * xx - 3 * yy), SH_C3[4] * x * (4 * zz - xx - yy),
        SH_C3[5] * z * (xx - yy), SH_C3[6] * x * (xx - 3 * yy),
    ], dim=1)


def as_matrix(column_major):
    return torch.tensor([float(v) for v in column_major], dtype=torch.float64).reshape(4, 4).T


def render(params, view, proj, background, width, height, sh_degree):
    """(H*W, 3) float64 image; params = (position, scale, rotation, opacity, color, sh(N,15,3))."""
    position, scale, rotation, opacity, color, sh = params
    f64 = torch.float64
    w = view[:3, :3]
    t = position @ w.T + view[:3, 3]
    depth = -t[:, 2]
    r = rotation_matrices(rotation)
    m = r * scale[:, None, :]
    cov3d = m @ m.transpose(1, 2)
    fx = proj[0, 0] * width / 2
    fy = proj[1, 1] * height / 2
    limit_x = 1.3 * width / 2 / fx
    limit_y = 1.3 * height / 2 / fy
    tx = torch.clamp(t[:, 0] / depth, -limit_x, limit_x) * depth
    ty = torch.clamp(t[:, 1] / depth, -limit_y, limit_y) * depth
    zero = torch.zeros_like(depth)
    j = torch.stack([fx / depth, zero, fx * tx / depth**2, zero, -fy / depth, -fy * ty / depth**2], dim=1)
    jw = j.reshape(-1, 2, 3) @ w
    cov = jw @ cov3d @ jw.transpose(1, 2)
    a = cov[:, 0, 0] + BLUR
    b = cov[:, 1, 0]
    c = cov[:, 1, 1] + BLUR
    det = a * c - b * b
    conic = torch.stack([c / det, -b / det, a / det], dim=1)
    clip = torch.cat([t, torch.ones_like(depth)[:, None]], dim=1) @ proj.T
    ndc = clip[:, :2] / clip[:, 3:]
    size = torch.tensor([width, height], dtype=f64)
    mean = (ndc * torch.tensor([0.5, -0.5], dtype=f64) + 0.5) * size
    camera_position = -(w.T @ view[:3, 3])
    offset = position - camera_position
    direction = offset / offset.norm(dim=1, keepdim=True)
    count = (sh_degree + 1) ** 2 - 1
    shaded = torch.clamp(color + (sh_basis(direction)[:, :count, None] * sh[:, :count, :]).sum(1), min=0)
    with torch.no_grad():
        mid = 0.5 * (a + c)
        radius = torch.ceil(3 * torch.sqrt(mid + torch.sqrt(torch.clamp(mid * mid - det, min=0.1))))
        offscreen = ((mean + radius[:, None] < 0) | (mean - radius[:, None] > size)).any(dim=1)
        visible = (depth > NEAR_CULL) & (det > 0) & ~offscreen
        tiles = torch.tensor([math.ceil(width / TILE), math.ceil(height / TILE)])
        low = torch.minimum(torch.clamp(torch.floor((mean - radius[:, None]) / TILE), min=0), tiles)
        high = torch.minimum(torch.clamp(torch.floor((mean + radius[:, None]) / TILE) + 1, min=0), tiles)
        order = torch.argsort(depth.detach(), stable=True)
        rank = torch.empty_like(order)
        rank[order] = torch.arange(order.numel())
    image = torch.zeros((height * width, 3), dtype=f64)
    pieces, where = [], []
    for ty_ in range(int(tiles[1])):
        for tx_ in range(int(tiles[0])):
            with torch.no_grad():
                cover = visible & (low[:, 0] <= tx_) & (high[:, 0] > tx_) & (low[:, 1] <= ty_) & (high[:, 1] > ty_)
                idx = torch.nonzero(cover).flatten()
                idx = idx[torch.argsort(rank[idx])]  # global stable depth order
                ys, xs = torch.meshgrid(torch.arange(ty_ * TILE, min((ty_ + 1) * TILE, height)),
                                        torch.arange(tx_ * TILE, min((tx_ + 1) * TILE, width)), indexing="ij")
                px, py = xs.flatten(), ys.flatten()
            pixel_index = py * width + px
            if idx.numel() == 0:
                pieces.append(background.expand(px.numel(), 3))
                where.append(pixel_index)
                continue
            centers = torch.stack([px + 0.5, py + 0.5], dim=1).to(f64)
            mu, co, op = mean[idx], conic[idx], opacity[idx]
            d = centers[:, None, :] - mu[None, :, :]
            power = -0.5 * (co[:, 0] * d[..., 0] ** 2 + co[:, 2] * d[..., 1] ** 2) - co[:, 1] * d[..., 0] * d[..., 1]
            alpha = torch.clamp(op * torch.exp(power), max=0.99)
            with torch.no_grad():
                blended = (power <= 0) & (alpha >= 1 / 255)
            alpha = torch.where(blended, alpha, 0)
            with torch.no_grad():
                before = torch.cumprod(torch.cat([torch.ones_like(alpha[:, :1]), 1 - alpha[:, :-1]], dim=1), dim=1)
                stops = blended & (before * (1 - alpha) < 0.0001)
                used = torch.cumsum(stops.to(torch.int64), dim=1) == 0
            alpha = torch.where(used, alpha, 0)
            trans = torch.cumprod(torch.cat([torch.ones_like(alpha[:, :1]), 1 - alpha[:, :-1]], dim=1), dim=1)
            final = trans[:, -1] * (1 - alpha[:, -1])
            pieces.append((alpha * trans) @ shaded[idx] + final[:, None] * background)
            where.append(pixel_index)
    order_all = torch.cat(where)
    values = torch.cat(pieces)
    image = image.index_put((order_all,), values)
    return image


def ssim_window(size: int = 11, sigma: float = 1.5):
    """The normalized 11x11 Gaussian window, one per channel
    (reference/loss_reference.py:26-29)."""
    g = torch.tensor([math.exp(-((x - size // 2) ** 2) / (2 * sigma**2)) for x in range(size)], dtype=torch.float64)
    g = g / g.sum()
    return (g[:, None] @ g[None, :]).expand(3, 1, size, size).contiguous()


def loss(render, target, lam: float = 0.2):
    """0.8 x L1 + 0.2 x (1 - SSIM) of two (3, H, W) float64 images, SSIM with
    zero padding and C1 = 0.01^2, C2 = 0.03^2, averaged over every pixel and
    channel (reference/loss_reference.py:32-50)."""
    w = ssim_window()
    a, b = render[None], target[None]
    blur = lambda image: F.conv2d(image, w, padding=5, groups=3)  # noqa: E731
    mu_a, mu_b = blur(a), blur(b)
    var_a = blur(a * a) - mu_a**2
    var_b = blur(b * b) - mu_b**2
    cov = blur(a * b) - mu_a * mu_b
    c1, c2 = 0.01**2, 0.03**2
    s = ((2 * mu_a * mu_b + c1) * (2 * cov + c2)) / ((mu_a**2 + mu_b**2 + c1) * (var_a + var_b + c2))
    return (1 - lam) * (render - target).abs().mean() + lam * (1 - s.mean())
