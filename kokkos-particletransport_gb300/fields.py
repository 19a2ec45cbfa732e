"""Synthetic 2D MHD background fields and the compact field file format.

The compact field file is the one the reference reads in
``include/AthenaFieldReader.hpp:277-285`` (written by ``apps/athena2bin.py``):

    int32 nx, int32 ny
    float64 x_edges[nx + 1], y_edges[ny + 1]
    float64 Bx[nx*ny], By[nx*ny], Bz[nx*ny], Vx[nx*ny], Vy[nx*ny], Vz[nx*ny]

little-endian, component arrays row-major with x fastest
(``source_index = j * nx + i``).  The reference reader rejects non-uniform
edges (``AthenaFieldReader.hpp:167-193``); this package accepts them as a
stated extension (stretched y edges of the scale configuration).

The generators below build the seeded synthetic backgrounds that stand in for
the reference's (absent) Athena++ reconnection data: a Harris current sheet
with a guide field and inflow, optional magnetic islands from a flux function,
optional non-uniform y edges and seeded multiplicative noise per frame.
"""
from __future__ import annotations

import dataclasses
import os
from typing import Optional

import numpy as np

COMPONENTS = ("Bx", "By", "Bz", "Vx", "Vy", "Vz")


@dataclasses.dataclass
class CompactField:
    """One frame of a 2D background field: face edges plus six cell arrays.

    ``b`` and ``v`` have shape (3, ny, nx) (x fastest in memory), matching the
    file's component order.
    """

    x_edges: np.ndarray
    y_edges: np.ndarray
    b: np.ndarray
    v: np.ndarray

    @property
    def nx(self) -> int:
        return int(self.x_edges.size - 1)

    @property
    def ny(self) -> int:
        return int(self.y_edges.size - 1)

    def file_bytes(self) -> int:
        return 8 + 8 * (self.nx + 1 + self.ny + 1) + 48 * self.nx * self.ny


def write_compact_field(path: str, field: CompactField) -> None:
    """Write ``field`` in the compact binary layout (little-endian)."""
    nx, ny = field.nx, field.ny
    with open(path, "wb") as stream:
        stream.write(np.asarray([nx, ny], dtype="<i4").tobytes())
        stream.write(np.ascontiguousarray(field.x_edges, dtype="<f8").tobytes())
        stream.write(np.ascontiguousarray(field.y_edges, dtype="<f8").tobytes())
        for comp in range(3):
            stream.write(np.ascontiguousarray(field.b[comp], dtype="<f8").tobytes())
        for comp in range(3):
            stream.write(np.ascontiguousarray(field.v[comp], dtype="<f8").tobytes())


def read_compact_field(path: str) -> CompactField:
    """Read a compact field file; raises ValueError on a malformed file."""
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.size < 8:
        raise ValueError("compact field: file too short for the header")
    nx, ny = (int(v) for v in raw[:8].view("<i4"))
    if nx <= 0 or ny <= 0:
        raise ValueError("compact field: dimensions must be positive")
    expected = 8 + 8 * (nx + 1 + ny + 1) + 48 * nx * ny
    if raw.size != expected:
        raise ValueError(
            f"compact field: expected {expected} bytes for {nx}x{ny}, found {raw.size}")
    body = raw[8:].view("<f8")
    x_edges = body[: nx + 1].copy()
    y_edges = body[nx + 1: nx + 1 + ny + 1].copy()
    arrays = body[nx + ny + 2:].reshape(6, ny, nx)
    return CompactField(x_edges, y_edges, arrays[:3].copy(), arrays[3:].copy())


def stretched_edges(n: int, lower: float, upper: float, strength: float = 4.0) -> np.ndarray:
    """Face edges whose spacing grows as 1 + strength*(y/half)^2, spanning [lower, upper].

    The local spacing d(edge)/ds is proportional to 1 + strength*(y/h)^2 with
    h = (upper-lower)/2 about the centre; the map is integrated numerically
    and normalised so the edges land exactly on [lower, upper].
    """
    centre = 0.5 * (lower + upper)
    half = 0.5 * (upper - lower)
    fine = np.linspace(lower, upper, 64 * n + 1)
    density = 1.0 / (1.0 + strength * ((fine - centre) / half) ** 2)
    cumulative = np.concatenate([[0.0], np.cumsum(0.5 * (density[1:] + density[:-1]))])
    cumulative /= cumulative[-1]
    edges = np.interp(np.linspace(0.0, 1.0, n + 1), cumulative, fine)
    edges[0], edges[-1] = lower, upper
    return edges


def harris_field(nx: int, ny: int, *, x_range=(-1.0, 1.0), y_range=(-2.0, 2.0),
                 sheet_width: float = 0.1, guide: float = 0.1, perturbation: float = 0.05,
                 inflow: float = 0.05, outflow: float = 0.1, island_amplitude: float = 0.0,
                 island_count: int = 8, island_width2: float = 0.04,
                 y_edges: Optional[np.ndarray] = None, noise: float = 0.0,
                 seed: int = 0) -> CompactField:
    """Harris sheet with guide field, inflow and optional islands (cell centres).

    Bx = tanh(y/w), By = eps*sin(pi x)*cos(pi y/4), Bz = guide,
    Vx = outflow*x*sech^2(y/w), Vy = -inflow*tanh(y/w), Vz = 0.
    Islands add B += z_hat x grad(psi) with
    psi = A*cos(island_count/2 * 2 pi x / Lx)*exp(-y^2/island_width2), i.e.
    Bx += dpsi/dy, By -= dpsi/dx.  ``noise`` > 0 multiplies every component by
    (1 + noise*N(0,1)) drawn from ``seed``.
    """
    x_edges = np.linspace(x_range[0], x_range[1], nx + 1)
    if y_edges is None:
        y_edges = np.linspace(y_range[0], y_range[1], ny + 1)
    y_edges = np.asarray(y_edges, dtype=np.float64)
    xc = 0.5 * (x_edges[1:] + x_edges[:-1])
    yc = 0.5 * (y_edges[1:] + y_edges[:-1])
    X, Y = np.meshgrid(xc, yc)  # shape (ny, nx), x fastest
    t = np.tanh(Y / sheet_width)
    sech2 = 1.0 / np.cosh(Y / sheet_width) ** 2
    bx = t.copy()
    by = perturbation * np.sin(np.pi * X) * np.cos(np.pi * Y / 4.0)
    bz = np.full_like(X, guide)
    if island_amplitude != 0.0:
        lx = x_range[1] - x_range[0]
        k = np.pi * island_count / lx
        g = np.exp(-Y * Y / island_width2)
        # psi = A cos(k x) g(y): dpsi/dy = A cos(kx) g * (-2y/w2); dpsi/dx = -A k sin(kx) g
        bx = bx + island_amplitude * np.cos(k * X) * g * (-2.0 * Y / island_width2)
        by = by + island_amplitude * k * np.sin(k * X) * g
    vx = outflow * X * sech2
    vy = -inflow * t
    vz = np.zeros_like(X)
    b = np.stack([bx, by, bz])
    v = np.stack([vx, vy, vz])
    if noise > 0.0:
        rng = np.random.default_rng(seed)
        b = b * (1.0 + noise * rng.standard_normal(b.shape))
        v = v * (1.0 + noise * rng.standard_normal(v.shape))
    return CompactField(x_edges, y_edges, np.ascontiguousarray(b), np.ascontiguousarray(v))


def field_file_path(field_dir: str, frame: int) -> str:
    """``FIELD_DIR/fieldNNNNN.bin`` as in the reference (src/main.cpp:413-418)."""
    return os.path.join(field_dir, f"field{frame:05d}.bin")


def ghosted_faces(edges) -> np.ndarray:
    """The n + 5 face coordinates of a stored library grid axis from its n + 1
    physical faces: the two ghost faces on each side continue the axis
    periodically (face -k = face n-k minus the width), face -2 first."""
    e = np.asarray(edges, dtype=np.float64)
    n = e.size - 1
    w = e[-1] - e[0]
    return np.concatenate([e[n - 2:n] - w, e, e[1:3] + w])


def cell_centres(faces) -> np.ndarray:
    """Cell centres of a stored axis: the midpoints of adjacent faces."""
    f = np.asarray(faces, dtype=np.float64)
    return 0.5 * (f[:-1] + f[1:])


def _ghosted_centres(n: int, edges, centres):
    if centres is not None:
        return np.asarray(centres, dtype=np.float64)
    d = (edges[-1] - edges[0]) / n
    return edges[0] + (np.arange(-2, n + 2) + 0.5) * d


def library_parker_basis(nx: int, ny: int, x_edges, y_edges, readme: bool = True,
                         centres=None) -> np.ndarray:
    """Synthetic smooth periodic coefficient fields for the library Parker solver
    on every ghosted cell centre (of a uniform grid, or the given (xc, yc)
    centres of a stored one), in the packed order of ParkerSolver.hpp:96-116:
    B(3) V(3) drift curl(3) diffusion primary(3) secondary(3) kappa_par
    kappa_perp div V (points x 18, x fastest).  readme = False gives the
    constant-ratio branch (secondary zero)."""
    xc = _ghosted_centres(nx, x_edges, None if centres is None else centres[0])
    yc = _ghosted_centres(ny, y_edges, None if centres is None else centres[1])
    y, x = np.meshgrid(yc, xc, indexing="ij")
    kx, ky = np.pi, np.pi / 2.0
    out = np.zeros((ny + 4, nx + 4, 18))
    out[..., 0] = np.tanh(np.sin(ky * y) / 0.3) + 0.05
    out[..., 1] = 0.1 * np.sin(kx * x) * np.cos(ky * y)
    out[..., 2] = 0.2
    out[..., 3] = 0.1 * np.cos(kx * x)
    out[..., 4] = -0.05 * np.sin(ky * y)
    out[..., 6] = 0.02 * np.sin(kx * x + ky * y)
    out[..., 7] = 0.02 * np.cos(kx * x - ky * y)
    out[..., 8] = 0.01 * np.sin(ky * y)
    out[..., 9] = 1e-3 * np.cos(kx * x)
    out[..., 10] = 1e-3 * np.sin(ky * y)
    if readme:
        out[..., 12] = 5e-4 * np.sin(kx * x)
        out[..., 13] = 5e-4 * np.cos(ky * y)
    out[..., 15] = 0.01 * (1.2 + np.sin(kx * x) * np.cos(ky * y))
    out[..., 16] = 0.05 * out[..., 15] if not readme else 1e-3 * (1.1 + np.cos(kx * x))
    out[..., 17] = 0.1 * np.cos(kx * x) * np.sin(ky * y)
    return out.reshape(-1, 18)


def library_focus_basis(nx: int, ny: int, x_edges, y_edges, centres=None) -> np.ndarray:
    """Smooth periodic focused-transport fields on every ghosted cell centre in
    the packed order B(3) b(3) V(3) grad-drift(3) curvature-drift(3) perp-adv(3)
    |B| kpar kperp divV focusing bb:gradV b.dV/dt sigma^2 Lc."""
    parker = library_parker_basis(nx, ny, x_edges, y_edges, True,
                                  centres).reshape(ny + 4, nx + 4, 18)
    xc = _ghosted_centres(nx, x_edges, None if centres is None else centres[0])
    yc = _ghosted_centres(ny, y_edges, None if centres is None else centres[1])
    y, x = np.meshgrid(yc, xc, indexing="ij")
    kx, ky = np.pi, np.pi / 2.0
    out = np.zeros((ny + 4, nx + 4, 27))
    b = parker[..., 0:3]
    bmag = np.sqrt((b * b).sum(-1))
    out[..., 0:3] = b
    out[..., 3:6] = b / bmag[..., None]
    out[..., 6:9] = parker[..., 3:6]
    out[..., 9] = 0.01 * np.sin(kx * x)
    out[..., 10] = 0.01 * np.cos(ky * y)
    out[..., 12] = 0.005 * np.cos(kx * x + ky * y)
    out[..., 13] = 0.005 * np.sin(kx * x)
    out[..., 14] = 0.002
    out[..., 15] = 1e-4 * np.sin(ky * y)
    out[..., 16] = 1e-4 * np.cos(kx * x)
    out[..., 18] = bmag
    out[..., 19] = 0.01 * (1.2 + np.sin(kx * x) * np.cos(ky * y))
    out[..., 20] = 5e-4 * (1.1 + np.cos(kx * x))
    out[..., 21] = 0.1 * np.cos(kx * x) * np.sin(ky * y)
    out[..., 22] = 0.2 * np.sin(kx * x - ky * y)
    out[..., 23] = 0.05 * np.cos(ky * y)
    out[..., 24] = 0.02 * np.sin(kx * x)
    out[..., 25] = 0.1 * (1.0 + 0.5 * np.sin(kx * x) * np.sin(ky * y))
    out[..., 26] = 0.05 * (1.0 + 0.2 * np.cos(kx * x))
    return out.reshape(-1, 27)
