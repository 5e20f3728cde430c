"""Synthetic analytic-SDF scenes standing in for the reference's COLMAP
captures (datasets/colmap.py), which are not available here.

A scene is an analytic signed distance function with a procedural albedo.
Target views are rendered by sphere tracing the analytic SDF; cameras sit on
a sphere around the origin and look at it; pixel directions follow the
reference's OpenGL convention (models/ray_utils.py:9-20: x right, y up, -z
forward, pixel centres)."""
from __future__ import annotations

import math

import torch


def sdf_sphere(p, r=0.5, c=(0.0, 0.0, 0.0)):
    return (p - torch.tensor(c, device=p.device, dtype=p.dtype)).norm(dim=-1) - r


def sdf_torus(p, R=0.3, r=0.1, c=(0.0, 0.0, 0.0)):
    q = p - torch.tensor(c, device=p.device, dtype=p.dtype)
    xz = torch.sqrt(q[..., 0] ** 2 + q[..., 2] ** 2) - R
    return torch.sqrt(xz ** 2 + q[..., 1] ** 2) - r


def sdf_box(p, half=0.1, c=(0.0, 0.0, 0.0)):
    q = (p - torch.tensor(c, device=p.device, dtype=p.dtype)).abs() - half
    outside = q.clamp(min=0).norm(dim=-1)
    inside = q.max(dim=-1).values.clamp(max=0)
    return outside + inside


class Scene:
    name = "scene"
    radius = 0.5

    def sdf(self, p):
        raise NotImplementedError

    def albedo(self, p):
        """0.5 + 0.5 sin(4 pi x + phase_c) sin(4 pi y) sin(4 pi z), phase per channel."""
        ph = torch.tensor([0.0, 2.0 * math.pi / 3, 4.0 * math.pi / 3], device=p.device,
                          dtype=p.dtype)
        s = torch.sin(4 * math.pi * p[..., 1:2]) * torch.sin(4 * math.pi * p[..., 2:3])
        return 0.5 + 0.5 * torch.sin(4 * math.pi * p[..., 0:1] + ph) * s


class SphereScene(Scene):
    """Sphere of radius 0.5 (the small, CPU-runnable configuration)."""
    name = "sphere"
    radius = 1.0

    def sdf(self, p):
        return sdf_sphere(p, 0.5)


class UnionScene(Scene):
    """Union of a torus (R 0.3, r 0.1), a box (edge 0.2) and a sphere (r 0.15)
    inside the radius-0.5 box (the full training configuration)."""
    name = "torus_box_sphere"
    radius = 0.5

    def sdf(self, p):
        return torch.minimum(torch.minimum(sdf_torus(p, 0.3, 0.1),
                                           sdf_box(p, 0.1, (0.0, 0.25, 0.0))),
                             sdf_sphere(p, 0.15, (0.0, -0.25, 0.1)))


def look_at_c2w(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)):
    """Camera-to-world (3x4) looking from eye at target, OpenGL axes."""
    eye = torch.as_tensor(eye, dtype=torch.float64)
    f = torch.as_tensor(target, dtype=torch.float64) - eye
    f = f / f.norm()
    u = torch.as_tensor(up, dtype=torch.float64)
    if abs(float(f @ u)) > 0.99:
        u = torch.tensor([0.0, 0.0, 1.0], dtype=torch.float64)
    r = torch.linalg.cross(f, u)
    r = r / r.norm()
    u = torch.linalg.cross(r, f)
    return torch.stack([r, u, -f, eye], dim=1).float()


def sphere_poses(n, radius, seed):
    g = torch.Generator().manual_seed(seed)
    v = torch.randn(n, 3, generator=g, dtype=torch.float64)
    v = v / v.norm(dim=-1, keepdim=True) * radius
    return torch.stack([look_at_c2w(e.tolist()) for e in v])


def pixel_directions(W, H, fov_deg, device="cpu"):
    """models/ray_utils.py:9-20 with fx = fy = W / (2 tan(fov/2)), centre (W/2, H/2)."""
    f = W / (2 * math.tan(math.radians(fov_deg) / 2))
    i, j = torch.meshgrid(torch.arange(W, dtype=torch.float32, device=device) + 0.5,
                          torch.arange(H, dtype=torch.float32, device=device) + 0.5, indexing="xy")
    return torch.stack([(i - W / 2) / f, -(j - H / 2) / f, -torch.ones_like(i)], -1)


def rays_from(dirs_cam, c2w):
    """models/ray_utils.py:23-43 for (N,3) directions and (N,3,4) poses, then
    the normalisation of systems/neus.py:95."""
    d = (dirs_cam[:, None, :] * c2w[:, :3, :3]).sum(-1)
    o = c2w[:, :, 3]
    return torch.cat([o, torch.nn.functional.normalize(d, p=2, dim=-1)], dim=-1)


@torch.no_grad()
def render_analytic(scene: Scene, rays, background=(1.0, 1.0, 1.0), n_iter=128,
                    far=8.0):
    """Sphere-trace the analytic SDF; hit pixels take the albedo at the hit
    point, misses the background.  rays (N,6) -> rgb (N,3)."""
    o, d = rays[:, :3].double(), rays[:, 3:6].double()
    t = torch.zeros(len(rays), dtype=torch.float64, device=rays.device)
    for _ in range(n_iter):
        s = scene.sdf(o + d * t[:, None])
        t = torch.where(t < far, t + s, t)
    p = o + d * t[:, None]
    hit = scene.sdf(p).abs() < 1e-4
    bg = torch.tensor(background, dtype=torch.float64, device=rays.device)
    rgb = torch.where(hit[:, None], scene.albedo(p), bg)
    return rgb.float()


class TargetViews:
    """n_views images of H x W rendered from poses on a sphere, kept on a device,
    with Gaussian noise; sample_rays draws (image, x, y) uniformly like the
    reference's batch_image_sampling (systems/neus.py:39-55)."""

    def __init__(self, scene: Scene, n_views, W, H, fov_deg, cam_radius, seed=0, noise=0.01,
                 device="cuda", chunk=1 << 20):
        self.scene, self.W, self.H = scene, W, H
        self.c2w = sphere_poses(n_views, cam_radius, seed).to(device)
        self.dirs = pixel_directions(W, H, fov_deg, device).reshape(-1, 3)
        g = torch.Generator(device=device).manual_seed(seed + 1)
        imgs = []
        for v in range(n_views):
            rgbs = []
            for s in range(0, W * H, chunk):
                dd = self.dirs[s:s + chunk]
                rays = rays_from(dd, self.c2w[v:v + 1].expand(len(dd), 3, 4))
                rgbs.append(render_analytic(scene, rays))
            img = torch.cat(rgbs)
            img = img + noise * torch.randn(img.shape, generator=g, device=device)
            imgs.append(img)
        self.images = torch.stack(imgs)  # (V, H*W, 3)
        self.device = device

    def sample_rays(self, n, generator=None):
        V = self.images.shape[0]
        idx = torch.randint(0, V, (n,), device=self.device, generator=generator)
        pix = torch.randint(0, self.W * self.H, (n,), device=self.device, generator=generator)
        rays = rays_from(self.dirs[pix], self.c2w[idx])
        return rays, self.images[idx, pix]


def analytic_occupancy(scene: Scene, res=128, band=None, device="cuda"):
    """Cells whose centre lies within ``band`` (default: 2 cell diagonals) of
    the analytic surface: the occupancy a converged grid settles to."""
    r = scene.radius
    cell = 2 * r / res
    band = band if band is not None else 2 * cell * math.sqrt(3)
    c = (torch.arange(res, device=device, dtype=torch.float32) + 0.5) * cell - r
    X, Y, Z = torch.meshgrid(c, c, c, indexing="ij")
    p = torch.stack([X, Y, Z], -1).reshape(-1, 3)
    return scene.sdf(p).abs() < band
