"""Seeded synthetic tilt series: ellipsoid phantoms, per-axis affine projection
maps (written as the reference's TXBR grammar) and analytic parallel-beam
line integrals with Gaussian or Poisson noise.

The reference ships no data; these stand in for its electron-tomography
inputs with the sizes of the benchmark configurations.

Geometry of one axis with in-plane angle phi and tilts theta (1-based
detector coordinates, detector centre cu = (PX+1)/2, cv = (PY+1)/2, volume
centre c):
    x = cu + e_u . (p - c),  e_u = (cos t cos f, cos t sin f, sin t)
    y = cv + a   . (p - c),  a   = (-sin f, cos f, 0)
i.e. x_coef = [cu - e_u.c, e_u], y_coef = [cv - a.c, a] per angle, which the
reference evaluates as c0 + c1 X + c2 Y + c3 Z - 1 (FunctionOnGPU.cu:16-18).
The ray through detector pixel (u, v) runs along d = e_u x a.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Ellipsoids:
    centre: np.ndarray   # [n, 3] voxel coordinates (X, Y, Z)
    semi: np.ndarray     # [n, 3] semi-axes in voxels
    rot: np.ndarray      # [n, 3, 3] columns are the principal axes
    density: np.ndarray  # [n]

    @property
    def Q(self) -> np.ndarray:
        """Quadric matrices R diag(1/s^2) R^T, [n, 3, 3]."""
        return np.einsum("nij,nj,nkj->nik", self.rot, 1.0 / self.semi ** 2, self.rot)


def random_ellipsoids(rng: np.random.Generator, n: int, vol) -> Ellipsoids:
    """n ellipsoids, centres uniform inside vol, semi-axes 5-25 % of the lateral
    extent (z clipped to half the thickness), random rotation, density U(0,1)."""
    lo = np.array([vol.Xstart, vol.Ystart, vol.Zstart], np.float64)
    ext = np.array([vol.X, vol.Y, vol.Z], np.float64)
    centre = lo + rng.uniform(0.0, 1.0, (n, 3)) * (ext - 1)
    lateral = min(vol.X, vol.Y)
    semi = rng.uniform(0.05, 0.25, (n, 3)) * lateral
    semi[:, 2] = np.minimum(semi[:, 2], 0.5 * vol.Z)
    semi = np.maximum(semi, 1.0)
    g = rng.normal(size=(n, 3, 3))
    q, r = np.linalg.qr(g)
    q = q * np.sign(np.einsum("nii->ni", r))[:, None, :]
    density = rng.uniform(0.0, 1.0, n)
    return Ellipsoids(centre, semi, q, density)


def axis_maps(px: int, py: int, tilts_deg, phi_deg: float, vol) -> tuple[np.ndarray, np.ndarray]:
    """Per-angle affine maps [A*4] for x and y (TXBR coefficient order)."""
    c = np.array([(vol.Xstart + vol.Xend - 1) / 2.0, (vol.Ystart + vol.Yend - 1) / 2.0,
                  (vol.Zstart + vol.Zend - 1) / 2.0])
    cu, cv = (px + 1) / 2.0, (py + 1) / 2.0
    f = np.deg2rad(phi_deg)
    a = np.array([-np.sin(f), np.cos(f), 0.0])
    xs, ys = [], []
    for t in np.deg2rad(np.asarray(tilts_deg, np.float64)):
        eu = np.array([np.cos(t) * np.cos(f), np.cos(t) * np.sin(f), np.sin(t)])
        xs += [cu - eu @ c, *eu]
        ys += [cv - a @ c, *a]
    return np.array(xs), np.array(ys)


def line_integrals(ell: Ellipsoids, x_coef: np.ndarray, y_coef: np.ndarray, px: int, py: int,
                   chunk: int = 1 << 16) -> np.ndarray:
    """Analytic parallel-beam line integrals [A, py, px] in FP64 through the
    detector pixel centres of every angle (rays of the affine maps above)."""
    A = len(x_coef) // 4
    out = np.zeros((A, py, px), np.float64)
    Q = ell.Q
    uu, vv = np.meshgrid(np.arange(px, dtype=np.float64), np.arange(py, dtype=np.float64))
    uu, vv = uu.reshape(-1), vv.reshape(-1)
    for k in range(A):
        xc, yc = x_coef[4 * k:4 * k + 4], y_coef[4 * k:4 * k + 4]
        eu, ea = xc[1:], yc[1:]
        d = np.cross(eu, ea)
        d /= np.linalg.norm(d)
        # Point of the ray: eu.p = u+1 - xc0, ea.p = v+1 - yc0, d.p = 0.
        M = np.stack([eu, ea, d])
        Minv = np.linalg.inv(M)
        img = np.zeros(px * py)
        for s in range(0, uu.size, chunk):
            rhs = np.stack([uu[s:s + chunk] + 1 - xc[0], vv[s:s + chunk] + 1 - yc[0],
                            np.zeros(min(chunk, uu.size - s))])
            p0 = (Minv @ rhs).T  # [m, 3]
            acc = np.zeros(p0.shape[0])
            for e in range(len(ell.density)):
                q = Q[e]
                r = p0 - ell.centre[e]
                alpha = d @ q @ d
                beta = r @ (q @ d)
                gamma = np.einsum("mi,ij,mj->m", r, q, r) - 1.0
                disc = beta * beta - alpha * gamma
                ok = disc > 0
                acc[ok] += ell.density[e] * 2.0 * np.sqrt(disc[ok]) / alpha
            img[s:s + chunk] = acc
        out[k] = img.reshape(py, px)
    return out


def add_noise(rng: np.random.Generator, proj: np.ndarray, kind: str, level: float) -> tuple[np.ndarray, dict]:
    """Gaussian: sigma = level * max.  Poisson: dose = level e-/px, mu with max(mu L) = 2."""
    if kind == "gaussian":
        sigma = level * float(proj.max())
        return proj + rng.normal(0.0, sigma, proj.shape), {"sigma": sigma}
    if kind == "poisson":
        mu = 2.0 / max(float(proj.max()), 1e-12)
        counts = rng.poisson(level * np.exp(-mu * proj))
        data = -np.log(np.maximum(counts, 1) / level) / mu
        return data, {"mu": mu, "dose": level}
    if kind == "none":
        return proj.copy(), {}
    raise ValueError(kind)


def voxelize(ell: Ellipsoids, vol) -> np.ndarray:
    """Phantom sampled at voxel centres [Z, Y, X] (additive densities)."""
    z, y, x = np.meshgrid(np.arange(vol.Zstart, vol.Zend), np.arange(vol.Ystart, vol.Yend),
                          np.arange(vol.Xstart, vol.Xend), indexing="ij")
    p = np.stack([x, y, z], -1).reshape(-1, 3).astype(np.float64)
    out = np.zeros(p.shape[0])
    Q = ell.Q
    for e in range(len(ell.density)):
        r = p - ell.centre[e]
        out += ell.density[e] * (np.einsum("mi,ij,mj->m", r, Q[e], r) <= 1.0)
    return out.reshape(vol.Z, vol.Y, vol.X)


def txbr_text(x_coef: np.ndarray, y_coef: np.ndarray, vol) -> str:
    """TXBR text in the grammar the reference parses (MrcFileIOBaseFunction.cpp:72-134):
    one 'l' line per angle, 'x-k: c0 c1 c2 c3' and 'y-k: ...' coefficient lines,
    and 'x->S:1:E' style bound lines (fields 2 and 4 are start and end)."""
    lines = []
    A = len(x_coef) // 4
    for k in range(A):
        lines.append(f"l {k}")
        lines.append(f"x-{k}: " + " ".join(repr(float(v)) for v in x_coef[4 * k:4 * k + 4]))
        lines.append(f"y-{k}: " + " ".join(repr(float(v)) for v in y_coef[4 * k:4 * k + 4]))
    lines.append(f"x->{vol.Xstart}:1:{vol.Xend}")
    lines.append(f"y->{vol.Ystart}:1:{vol.Yend}")
    lines.append(f"z->{vol.Zstart}:1:{vol.Zend}")
    return "\n".join(lines) + "\n"


@dataclass
class Case:
    """A synthetic reconstruction input: K axes on one volume frame."""
    vol: object
    axes: list            # list of mtr.AxisData-like objects (x_coef, y_coef, data)
    ellipsoids: Ellipsoids
    meta: dict = field(default_factory=dict)


def make_case(vol, n_px: int, tilts_deg, phis_deg, n_ellipsoids: int, noise: str, level: float, seed: int,
              axis_cls=None, py: int | None = None) -> Case:
    """Build a case with analytic projections (numpy, FP64 then float32)."""
    rng = np.random.default_rng(seed)
    ell = random_ellipsoids(rng, n_ellipsoids, vol)
    py = py or n_px
    axes, meta = [], {"seed": seed, "noise": noise}
    for phi in phis_deg:
        xc, yc = axis_maps(n_px, py, tilts_deg, phi, vol)
        proj = line_integrals(ell, xc, yc, n_px, py)
        proj, info = add_noise(rng, proj, noise, level)
        meta.setdefault("noise_params", []).append(info)
        data = proj.astype(np.float32)
        axes.append(axis_cls(xc, yc, data) if axis_cls else (xc, yc, data))
    return Case(vol, axes, ell, meta)


def line_integrals_torch(ell: Ellipsoids, x_coef: np.ndarray, y_coef: np.ndarray, px: int, py: int,
                         device="cuda", ell_chunk: int = 32) -> "object":
    """Same analytic line integrals as line_integrals(), evaluated with torch
    in FP64 on a CUDA device for the large benchmark sizes; returns a float32
    CUDA tensor [A, py, px].

    Along the ray through detector pixel (u, v) the offset from an ellipsoid's
    centre is r = c + u e1 + v e2 + t d, so beta = (Q d).r is linear and
    gamma = r^T Q r - 1 quadratic in (u, v): their coefficients are formed per
    ellipsoid on the host and only the polynomials are evaluated per pixel."""
    import torch

    A = len(x_coef) // 4
    f64 = dict(dtype=torch.float64, device=device)
    out = torch.empty((A, py, px), dtype=torch.float32, device=device)
    u = torch.arange(px, **f64)[None, None, :]
    v = torch.arange(py, **f64)[None, :, None]
    Q, m, rho = np.asarray(ell.Q, np.float64), np.asarray(ell.centre, np.float64), np.asarray(ell.density, np.float64)
    for k in range(A):
        xc, yc = x_coef[4 * k:4 * k + 4], y_coef[4 * k:4 * k + 4]
        eu, ea = np.asarray(xc[1:]), np.asarray(yc[1:])
        d = np.cross(eu, ea)
        d /= np.linalg.norm(d)
        Minv = np.linalg.inv(np.stack([eu, ea, d]))
        e1, e2 = Minv[:, 0], Minv[:, 1]
        c = e1 * (1.0 - xc[0]) + e2 * (1.0 - yc[0]) - m                       # [n,3]
        Qd = Q @ d                                                               # [n,3]
        Qc, Qe1, Qe2 = np.einsum("nij,nj->ni", Q, c), Q @ e1, Q @ e2
        coef = np.stack([
            Qd @ d,                                                              # alpha
            np.einsum("ni,ni->n", Qd, c), Qd @ e1, Qd @ e2,                      # beta: 1, u, v
            np.einsum("ni,ni->n", c, Qc) - 1.0, 2 * np.einsum("ni,ni->n", Qc, np.broadcast_to(e1, c.shape)),
            2 * np.einsum("ni,ni->n", Qc, np.broadcast_to(e2, c.shape)),         # gamma: 1, u, v
            Qe1 @ e1, 2 * (Qe1 @ e2), Qe2 @ e2,                                  # gamma: uu, uv, vv
            rho], axis=1)
        C = torch.as_tensor(coef, **f64)[:, :, None, None]                       # [n,11,1,1]
        acc = torch.zeros((py, px), **f64)
        for s in range(0, len(rho), ell_chunk):
            K = C[s:s + ell_chunk]
            al, b0, bu, bv, g0, gu, gv, guu, guv, gvv, dens = K.unbind(1)
            beta = b0 + bu * u + bv * v
            gamma = g0 + (gu + guu * u + guv * v) * u + (gv + gvv * v) * v
            disc = beta * beta - al * gamma
            acc += (dens * 2.0 * torch.sqrt(torch.clamp(disc, min=0.0)) / al).sum(0)
        out[k] = acc.to(torch.float32)
    return out


def make_case_torch(vol, n_px: int, tilts_deg, phis_deg, n_ellipsoids: int, noise: str, level: float, seed: int,
                    device="cuda") -> dict:
    """Large-size counterpart of make_case: projections stay on the device
    (float32 tensors); noise is drawn with a seeded torch generator."""
    import torch

    rng = np.random.default_rng(seed)
    ell = random_ellipsoids(rng, n_ellipsoids, vol)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    axes = []
    meta = {"seed": seed, "noise": noise, "noise_params": []}
    for phi in phis_deg:
        xc, yc = axis_maps(n_px, n_px, tilts_deg, phi, vol)
        proj = line_integrals_torch(ell, xc, yc, n_px, n_px, device)
        if noise == "gaussian":
            sigma = level * float(proj.max())
            proj += sigma * torch.randn(proj.shape, generator=gen, device=device)
            meta["noise_params"].append({"sigma": sigma})
        elif noise == "poisson":
            mu = 2.0 / max(float(proj.max()), 1e-12)
            counts = torch.poisson(level * torch.exp(-mu * proj.double()), generator=gen)
            proj = (-torch.log(torch.clamp(counts, min=1.0) / level) / mu).float()
            meta["noise_params"].append({"mu": mu, "dose": level})
        axes.append((xc, yc, proj.contiguous()))
    return {"vol": vol, "axes": axes, "ellipsoids": ell, "meta": meta}
