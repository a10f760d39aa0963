"""Initial particle lattices for the dam-break cases (host-side setup).

This restates the parts of SmoothedParticles.jl's setup layer that the
dam-break inputs need, in IEEE double with the reference's expression order so
that the particle sets -- and their order, which is the particle index order
the cell lists depend on -- are the reference's:

* ``covering(::Squaregrid, s)``  src/grids.jl:52-66   (i outer, j inner)
* ``covering(::CubicGrid, s)``   src/grids.jl:128-144 (i outer, j, k inner)
* ``is_inside(x, ::Box)``         src/geometry.jl:24-30; ``Rectangle`` :37-39
* ``Circle``                      src/geometry.jl:50-67
* ``Ball``                        src/geometry.jl:247-260
* ``BoundaryLayer``               src/geometry.jl:198-234
* ``Specification``               src/geometry.jl:179-196
* ``boundarybox`` of a union      src/geometry.jl:117-127

The lattices are setup-time work (not on the accelerated path); they run once
per case on the host with numpy.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

FLUID = 0
WALL = 1


@dataclass(frozen=True)
class Box:
    """Axis-aligned box (geometry.jl:15-43). ``Rectangle`` has x3 in [0, 0]."""
    lo: tuple
    hi: tuple

    def inside(self, x: np.ndarray) -> np.ndarray:
        """geometry.jl:24-30; comparisons are False for NaN."""
        m = np.ones(x.shape[0], dtype=bool)
        for d in range(3):
            m &= (self.lo[d] <= x[:, d]) & (x[:, d] <= self.hi[d])
        return m


def rectangle(x1_min, x2_min, x1_max, x2_max) -> Box:
    return Box((float(x1_min), float(x2_min), 0.0), (float(x1_max), float(x2_max), 0.0))


def box3(x1_min, x2_min, x3_min, x1_max, x2_max, x3_max) -> Box:
    return Box((float(x1_min), float(x2_min), float(x3_min)),
               (float(x1_max), float(x2_max), float(x3_max)))


def _lattice_axis(lo: float, hi: float, dr: float) -> np.ndarray:
    """Int64(floor(lo/dr)):Int64(ceil(hi/dr)) (grids.jl:55-58, :131-136)."""
    i_min = int(math.floor(lo / dr))
    i_max = int(math.ceil(hi / dr))
    return np.arange(i_min, i_max + 1, dtype=np.int64)


def _points(dim: int, bbox: Box, dr: float) -> np.ndarray:
    """Lattice points ``i*dr`` covering ``bbox`` in the reference's loop order."""
    I = _lattice_axis(bbox.lo[0], bbox.hi[0], dr)
    J = _lattice_axis(bbox.lo[1], bbox.hi[1], dr)
    if dim == 2:
        gi, gj = np.meshgrid(I, J, indexing="ij")
        x = np.zeros((gi.size, 3))
        x[:, 0] = gi.ravel().astype(np.float64) * dr
        x[:, 1] = gj.ravel().astype(np.float64) * dr
        return x
    K = _lattice_axis(bbox.lo[2], bbox.hi[2], dr)
    gi, gj, gk = np.meshgrid(I, J, K, indexing="ij")
    x = np.empty((gi.size, 3))
    x[:, 0] = gi.ravel().astype(np.float64) * dr
    x[:, 1] = gj.ravel().astype(np.float64) * dr
    x[:, 2] = gk.ravel().astype(np.float64) * dr
    return x


def ball_offsets(dim: int, dr: float, width: float) -> np.ndarray:
    """covering(grid, Ball(0,0,0,width)) (geometry.jl:201-205, :253-255):
    ``(x1-0)^2 + (x2-0)^2 + (x3-0)^2 <= r^2`` evaluated left to right."""
    bb = Box((-width, -width, -width), (width, width, width))
    x = _points(dim, bb, dr)
    s = (x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) + x[:, 2] * x[:, 2]
    return x[s <= width * width]


def fill_box(dim: int, dr: float, shape: Box) -> np.ndarray:
    """covering(grid, shape) for a Box/Rectangle."""
    x = _points(dim, shape, dr)
    return x[shape.inside(x)]


def circle(dim: int, dr: float, cx: float, cy: float, r: float) -> np.ndarray:
    """covering(Squaregrid, Circle) (geometry.jl:60-67)."""
    bb = rectangle(cx - r, cy - r, cx + r, cy + r)
    x = _points(dim, bb, dr)
    a = x[:, 0] - cx
    b = x[:, 1] - cy
    return x[(a * a + b * b) <= r * r]


def boundary_layer(dim: int, dr: float, shape: Box, width: float, keep=None) -> np.ndarray:
    """covering(grid, Specification(BoundaryLayer(shape, grid, width), keep)).

    A lattice point is in the layer when it is outside ``shape`` and some
    ``x + dx`` (``dx`` a lattice offset within ``width``) is inside it
    (geometry.jl:209-219).  ``keep(x)`` is the Specification predicate.  The
    bounding box is ``shape`` grown by ``width`` (geometry.jl:221-233).
    """
    lo = tuple(shape.lo[d] - width for d in range(3))
    hi = tuple(shape.hi[d] + width for d in range(3))
    if dim == 2:
        lo = (lo[0], lo[1], 0.0)
        hi = (hi[0], hi[1], 0.0)
    bb = Box(lo, hi)
    dxs = ball_offsets(dim, dr, width)
    I = _lattice_axis(bb.lo[0], bb.hi[0], dr)
    J = _lattice_axis(bb.lo[1], bb.hi[1], dr)
    K = _lattice_axis(bb.lo[2], bb.hi[2], dr) if dim == 3 else np.zeros(1, np.int64)
    # blocks of consecutive i keep memory bounded; the order stays i outer
    step = max(1, (1 << 21) // (J.size * K.size))
    out = []
    for i0 in range(0, I.size, step):
        x = _block(dim, I[i0:i0 + step], J, K, dr)
        cand = ~shape.inside(x)
        if keep is not None:
            cand &= keep(x)
        xc = x[cand]
        hit = np.zeros(xc.shape[0], dtype=bool)
        for dx in dxs:
            hit |= shape.inside(xc + dx)
        out.append(xc[hit])
    return np.concatenate(out) if out else np.zeros((0, 3))


def _block(dim: int, I: np.ndarray, J: np.ndarray, K: np.ndarray, dr: float) -> np.ndarray:
    """Lattice points i*dr, j*dr(, k*dr) for i in I, j in J(, k in K), i outer."""
    if dim == 2:
        gi, gj = np.meshgrid(I, J, indexing="ij")
        x = np.zeros((gi.size, 3))
        x[:, 0] = gi.ravel().astype(np.float64) * dr
        x[:, 1] = gj.ravel().astype(np.float64) * dr
        return x
    gi, gj, gk = np.meshgrid(I, J, K, indexing="ij")
    x = np.empty((gi.size, 3))
    x[:, 0] = gi.ravel().astype(np.float64) * dr
    x[:, 1] = gj.ravel().astype(np.float64) * dr
    x[:, 2] = gk.ravel().astype(np.float64) * dr
    return x


@dataclass
class Case:
    """A particle set plus the physical parameters of one run."""
    name: str
    dim: int
    dr: float
    x: np.ndarray            # n x 3, reference particle order
    type: np.ndarray         # int32, FLUID / WALL
    v: np.ndarray = None     # n x 3
    params: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.x.shape[0]

    @property
    def n_fluid(self) -> int:
        return int((self.type == FLUID).sum())


@dataclass
class Shapes:
    """The shapes of a case as the device generator takes them (no particles)."""
    name: str
    dim: int
    dr: float
    shapes: list             # dicts: kind, type, dr, lo, hi, width, keep_axis, keep_max
    params: dict = field(default_factory=dict)


def _dam_break_setup(dim, dr, col_width, col_height, box_width, box_height, depth, h_factor,
                     wall_layers, lid, alpha, eps_xsph, g, rho0):
    if h_factor is None:
        h_factor = 2.4 if dim == 2 else 2.0
    width = wall_layers * dr
    if dim == 2:
        fluid_shape = rectangle(0.0, 0.0, col_width, col_height)
        box = rectangle(0.0, 0.0, box_width, box_height)
        vaxis = 1
    else:
        fluid_shape = box3(0.0, 0.0, 0.0, col_width, depth, col_height)
        box = box3(0.0, 0.0, 0.0, box_width, depth, box_height)
        vaxis = 2
    h = h_factor * dr
    H = 2.0 * h
    dmin = [box.lo[d] - width for d in range(3)]
    dmax = [box.hi[d] + width for d in range(3)]
    if dim == 2:
        dmin[2] = dmax[2] = 0.0
    c0 = 10.0 * math.sqrt((2.0 * g) * col_height)
    gravity = [0.0, 0.0, 0.0]
    gravity[vaxis] = -g
    mass = rho0 * (dr * dr) if dim == 2 else rho0 * ((dr * dr) * dr)
    params = dict(dim=dim, h=H, domain_min=dmin, domain_max=dmax, mass=mass, rho0=rho0,
                  c0=c0, h_smooth=h, alpha=alpha, eps_xsph=eps_xsph, gravity=gravity,
                  dt=(0.1 * h) / c0, col_height=col_height,
                  vertical_axis=vaxis)
    return fluid_shape, box, width, vaxis, params


def dam_break(dim: int, dr: float, *, col_width: float = 1.0, col_height: float = 2.0,
              box_width: float = 4.0, box_height: float = 3.0, depth: float = 1.0,
              h_factor: float | None = None, wall_layers: int = 3, lid: bool = False,
              alpha: float = 0.02, eps_xsph: float = 0.5, g: float = 9.81,
              rho0: float = 1000.0, name: str | None = None) -> Case:
    """The WCSPH dam break: fluid column plus ``wall_layers`` wall layers.

    2D: column ``col_width x col_height`` in a ``box_width x box_height`` box,
    gravity along -y.  3D: block ``col_width x depth x col_height`` in a
    ``box_width x depth x box_height`` tank, gravity along -z.  The smoothing
    length is ``h = h_factor*dr`` (2.4 in 2D, 2.0 in 3D by default) and the
    neighbour radius (kernel support) is ``H = 2h``.  Without a lid the wall
    layer keeps only points below the box top, as collapse_dry.jl:93 does.
    The domain is ``box + walls``, whose bounding box is the box grown by the
    wall width (collapse_dry.jl:94).
    """
    fluid_shape, box, width, vaxis, params = _dam_break_setup(
        dim, dr, col_width, col_height, box_width, box_height, depth, h_factor, wall_layers,
        lid, alpha, eps_xsph, g, rho0)
    xf = fill_box(dim, dr, fluid_shape)
    keep = None if lid else (lambda x, a=vaxis, top=box_height: x[:, a] < top)
    xw = boundary_layer(dim, dr, box, width, keep)
    x = np.concatenate([xf, xw])
    typ = np.concatenate([np.full(xf.shape[0], FLUID, np.int32), np.full(xw.shape[0], WALL, np.int32)])
    return Case(name or f"dam_break_{dim}d_dr{dr:g}", dim, dr, x, typ,
                np.zeros_like(x), params)


def dam_break_shapes(dim: int, dr: float, *, col_width: float = 1.0, col_height: float = 2.0,
                     box_width: float = 4.0, box_height: float = 3.0, depth: float = 1.0,
                     h_factor: float | None = None, wall_layers: int = 3, lid: bool = False,
                     alpha: float = 0.02, eps_xsph: float = 0.5, g: float = 9.81,
                     rho0: float = 1000.0, name: str | None = None) -> Shapes:
    """The same dam break as ``dam_break`` for the device generator
    (``ParticleSystem.generate``): the fluid box and the wall layer, whose
    particles the GPU produces in the same order and bit for bit."""
    fluid_shape, box, width, vaxis, params = _dam_break_setup(
        dim, dr, col_width, col_height, box_width, box_height, depth, h_factor, wall_layers,
        lid, alpha, eps_xsph, g, rho0)
    shapes = [dict(kind="box", type=FLUID, dr=dr, lo=fluid_shape.lo, hi=fluid_shape.hi),
              dict(kind="layer", type=WALL, dr=dr, lo=box.lo, hi=box.hi, width=width,
                   keep_axis=-1 if lid else vaxis, keep_max=box_height)]
    return Shapes(name or f"dam_break_{dim}d_dr{dr:g}", dim, dr, shapes, params)


def collision_2d(dr: float = 0.02, c0: float = 20.0) -> Case:
    """The two colliding circles of tests/test_collision_2d.jl:15-58.

    Circles of radius 0.4 centred at (-0.5, -0.1) and (0.5, 0.1) moving at
    +1 and -1 m/s along x, domain [-10, 10]^2, kernel support ``2.4*dr``
    (the test uses h as the support), no walls, no gravity, no viscosity and
    no XSPH.  The equation of state is the test's linear one,
    P = c^2 (rho - rho0) with P/rho0^2 in the pressure force
    (test_collision_2d.jl:71-78), c = 20.
    """
    H = 2.4 * dr
    x1 = circle(2, dr, -0.5 * 1.0, -0.5 * 0.2, 0.4)
    x2 = circle(2, dr, 0.5 * 1.0, 0.5 * 0.2, 0.4)
    x = np.concatenate([x1, x2])
    v = np.zeros_like(x)
    v[: x1.shape[0], 0] = 1.0
    v[x1.shape[0]:, 0] = -1.0
    typ = np.zeros(x.shape[0], np.int32)
    rho0 = 1000.0
    params = dict(dim=2, h=H, domain_min=[-10.0, -10.0, 0.0], domain_max=[10.0, 10.0, 0.0],
                  mass=rho0 * (dr * dr), rho0=rho0, c0=c0, h_smooth=0.5 * H, alpha=0.0,
                  eps_xsph=0.0, gravity=[0.0, 0.0, 0.0], dt=(0.1 * H) / c0, col_height=0.0,
                  vertical_axis=1, eos=1)
    return Case("collision_2d", 2, dr, x, typ, v, params)
