"""Tight-binding inputs for the KPM engine: lattices, flakes and modifiers.

pybinding itself cannot be imported next to this package (its compiled core is
not built), so this module restates the part of its model builder that the
KPM path consumes: a Hamiltonian CSR matrix in pybinding's site order plus the
site positions and sublattice ranges used by ``find_nearest`` and the
conductivity's position operator.

Site order follows the reference exactly, because the stochastic DOS assigns
random-vector entries by site index:

* foundation bounds: lattice coordinates of the shape vertices, truncated and
  padded by one cell (``cppcore/src/system/Foundation.cpp:6-23``);
* positions generated sublattice-major, then c, b, a with ``a`` fastest, in
  float32 (``Foundation.cpp:25-48``);
* polygon membership by ray casting in float32
  (``cppcore/src/system/Shape.cpp:54-88``);
* dangling sites removed until every site keeps ``min_neighbors`` neighbours
  (``Foundation.cpp:50-101``), which is the k-core of the site graph;
* final indices: valid sites, sublattice-major (``Foundation.cpp:127-164``);
* CSR rows hold sorted column indices; hoppings are inserted for the owning
  sublattice and mirrored as their conjugate (``hamiltonian/Hamiltonian.hpp:74-100``);
  zero onsite energies are not stored (``HamiltonianModifiers.hpp:143-152``).

The scalar type follows ``cppcore/src/Model.cpp:178-204``: float32 unless a
modifier asks for complex numbers (complex64) or double precision.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

# graphene constants, pybinding/repository/graphene/constants.py:3-8
GRAPHENE_A = 0.24595
GRAPHENE_A_CC = 0.142
GRAPHENE_T = -2.8
GRAPHENE_BETA = 3.37
# pybinding/constants.py:11-12
HBAR = 6.58211899 * 10 ** -16
PHI0 = 2 * math.pi * HBAR


@dataclass
class System:
    """Site positions and sublattice layout of a built system; ``orbitals`` per site (one
    sublattice kind per system here, so every site has the same number)."""
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    sub_ranges: dict = field(default_factory=dict)  # name -> (start, end)
    orbitals: int = 1

    @property
    def positions(self):
        return self.x, self.y, self.z

    @property
    def num_sites(self):
        return int(self.x.size)

    @property
    def hamiltonian_size(self):
        return self.num_sites * self.orbitals

    def sublattice_range(self, sublattice=""):
        """cppcore/src/system/System.cpp:50-66"""
        if not sublattice:
            return 0, self.num_sites
        if sublattice not in self.sub_ranges:
            raise RuntimeError("There is no sublattice named '{}'".format(sublattice))
        return self.sub_ranges[sublattice]

    def find_nearest(self, position, sublattice=""):
        """Index of the site closest to ``position`` (float32 distances, first minimum wins).

        Mirrors ``System::find_nearest`` (``cppcore/src/system/System.cpp:68-82``).
        """
        p = np.zeros(3, np.float32)
        pos = np.asarray(position, dtype=np.float32).ravel()
        p[:pos.size] = pos
        start, end = self.sublattice_range(sublattice)
        dx = self.x[start:end] - p[0]
        dy = self.y[start:end] - p[1]
        dz = self.z[start:end] - p[2]
        d = np.sqrt(dx * dx + dy * dy + dz * dz)
        return int(start + np.argmin(d))

    def to_hamiltonian_indices(self, system_index):
        """The Hamiltonian rows of site ``i``: ``i * orbitals + k`` for its orbitals k
        (System.cpp:33-48, one sublattice kind)."""
        first = int(system_index) * self.orbitals
        return np.arange(first, first + self.orbitals, dtype=np.int32)

    def contains_mask(self, contains):
        return np.asarray(contains(self.x, self.y, self.z), dtype=bool)


@dataclass
class Model:
    """The part of ``pybinding.Model`` that the KPM path reads."""
    hamiltonian: sp.csr_matrix
    system: System
    is_complex: bool = False
    is_double: bool = False
    name: str = ""

    @property
    def is_multiorbital(self):
        return self.system is not None and self.system.orbitals > 1


# --------------------------------------------------------------------------- shapes

def rectangle(x, y=None):
    """Vertices of ``pb.rectangle`` (pybinding/shape.py:263-279), float32."""
    y = y or x
    x0, y0 = x / 2, y / 2
    return np.array([[x0, y0], [x0, -y0], [-x0, -y0], [-x0, y0]], dtype=np.float32)


def regular_polygon(num_sides, radius, angle=0.0):
    """Vertices of ``pb.regular_polygon`` (pybinding/shape.py:282-300), float32."""
    angles = [angle + 2 * n * math.pi / num_sides for n in range(num_sides)]
    return np.array([(radius * math.sin(a), radius * math.cos(a)) for a in angles], dtype=np.float32)


def hexagon_ac(side_width):
    """Vertices and lattice offset of ``graphene.hexagon_ac`` (repository/graphene/shape.py:8-35):
    a hexagon with armchair edges, its width adjusted to a whole number of edge atoms, and
    the lattice moved by (-a/2, 0) so that a carbon hexagon sits at the centre. Returns
    ``(vertices, lattice_offset)`` for :func:`build_honeycomb`."""
    side_atoms = math.ceil((side_width / GRAPHENE_A_CC + 1) * 2 / 3)
    side_atoms += side_atoms % 2
    side_width = (3 / 2 * side_atoms - 1) * GRAPHENE_A_CC - GRAPHENE_A_CC / 2
    x0 = side_width * math.sqrt(3) / 2
    y0 = side_width
    v = np.array([(0, y0), (x0, y0 / 2), (x0, -y0 / 2), (0, -y0), (-x0, -y0 / 2), (-x0, y0 / 2)], dtype=np.float32)
    return v, (-GRAPHENE_A / 2, 0.0)


def polygon_contains(vertices, px, py):
    """Ray-casting point-in-polygon test in float32 (``Shape.cpp:54-88``)."""
    vx = np.asarray(vertices[:, 0], np.float32)
    vy = np.asarray(vertices[:, 1], np.float32)
    px = np.asarray(px, np.float32)
    py = np.asarray(py, np.float32)
    inside = np.zeros(px.shape, dtype=bool)
    n = vx.size
    eps = np.finfo(np.float32).eps
    tiny = np.finfo(np.float32).tiny
    j = n - 1
    for i in range(n):
        x1, x2, y1, y2 = vx[i], vx[j], vy[i], vy[j]
        diff = abs(np.float32(y1 - y2))
        scale = abs(np.float32(y1 + y2))
        if diff <= eps * scale or diff <= tiny:   # num::approx_equal
            j = i
            continue
        k = np.float32((x2 - x1) / (y2 - y1))
        intersects_y = (y1 > py) != (y2 > py)
        x_side = k * (py - y1) + x1
        intersects_x = px > x_side
        inside ^= intersects_y & intersects_x
        j = i
    return inside


# --------------------------------------------------------------------------- builder

def _k_core(valid, nbr, min_neighbors):
    """Remove valid sites until each keeps ``min_neighbors`` valid neighbours.

    ``nbr`` is (num_sites, max_hops) with -1 for hoppings that leave the foundation.
    Equivalent to the recursive clearing of ``Foundation.cpp:73-101``: both compute
    the unique k-core of the valid-site graph.
    """
    valid = valid.copy()
    has = nbr >= 0
    safe = np.where(has, nbr, 0)
    while True:
        cnt = np.sum(has & valid[safe], axis=1)
        drop = valid & (cnt < min_neighbors)
        if not drop.any():
            return valid
        valid &= ~drop


def _honeycomb_frame(vertices, a, a_cc, float_constants, lattice_offset=(0.0, 0.0)):
    """Lattice vectors, sublattice offsets and the foundation (origin, s0 x s1 cells) of a
    honeycomb lattice cut by the polygon ``vertices``, all float32 values as the reference
    computes them (``Foundation.cpp:6-23``, ``Lattice.cpp:190-200``). ``lattice_offset`` is
    the shape's lattice offset (``Model.cpp:30-34``): it moves the sites, not the bounds."""
    f32 = np.float32
    if float_constants:
        af, accf = f32(a), f32(a_cc)
        v0 = np.array([af, 0, 0], f32)
        v1 = np.array([af / f32(2), af / f32(2) * np.sqrt(f32(3)), 0], f32)
        sub_pos = [np.array([0, -accf / f32(2), 0], f32), np.array([0, accf / f32(2), 0], f32)]
    else:
        v0 = np.array([a, 0, 0], f32)
        v1 = np.array([a / 2, a / 2 * math.sqrt(3), 0], f32)
        sub_pos = [np.array([0, -a_cc / 2, 0], f32), np.array([0, a_cc / 2, 0], f32)]

    # Foundation bounds: solve [v0 v1] v = p for each vertex, truncate, pad by one
    m = np.array([[v0[0], v1[0]], [v0[1], v1[1]]], dtype=np.float64)
    coords = np.linalg.solve(m, np.asarray(vertices, np.float64).T).T
    ic = np.trunc(coords).astype(np.int64)
    lo = ic.min(axis=0) - 1
    hi = ic.max(axis=0) + 1
    s0, s1 = int(hi[0] - lo[0] + 1), int(hi[1] - lo[1] + 1)

    # origin = offset + lo0*v0 + lo1*v1 (float32, Lattice.cpp:190-200)
    origin = np.zeros(3, f32)
    origin[:2] = np.asarray(lattice_offset, f32)[:2]
    origin = origin + f32(lo[0]) * v0
    origin = origin + f32(lo[1]) * v1
    return v0, v1, sub_pos, origin, s0, s1


# hoppings owned by A (non-conjugate) -> B as cell offsets along (a1, a2); B holds the conjugates
_HONEYCOMB_HOPS = [(0, 0), (1, -1), (0, -1)]


def _scalar_type(is_complex, is_double):
    if is_complex:
        return np.complex128 if is_double else np.complex64
    return np.float64 if is_double else np.float32


def _hopping_energies(dtype, t, nhops, rows, cols, sx, sy, sz, hopping_modifiers):
    hop = np.full(nhops, t, dtype=dtype)
    for mod in hopping_modifiers:
        hop = np.asarray(mod(hop, sx[rows], sy[rows], sz[rows], sx[cols], sy[cols], sz[cols]))
        hop = hop.astype(dtype) if np.iscomplexobj(dtype(0)) else np.real(hop).astype(dtype)
    return hop


def _onsite_energies(dtype, sx, sy, sz, sub_of, onsite_modifiers):
    onsite = np.zeros(sx.size, dtype=dtype)
    for mod in onsite_modifiers:
        onsite = np.asarray(mod(onsite, sx, sy, sz, sub_of)).astype(dtype)
    return onsite


def build_honeycomb(vertices, onsite_modifiers=(), hopping_modifiers=(),
                    is_complex=False, is_double=False, min_neighbors=2,
                    t=GRAPHENE_T, a=GRAPHENE_A, a_cc=GRAPHENE_A_CC, name="graphene",
                    float_constants=False, device=None, lattice_offset=(0.0, 0.0)):
    """Monolayer graphene (``repository/graphene/lattice.py:6-66``) cut by a polygon.

    ``float_constants`` derives the lattice vectors in float32 arithmetic, as the
    C++ test fixture does (``cppcore/tests/fixtures.cpp``, ``min_neighbors=1``);
    the Python repository lattice computes them in double and sets
    ``min_neighbors=2``.

    Modifiers are callables in the reference's numpy style:
    ``onsite(energy, x, y, z, sub)`` and ``hopping(energy, x1, y1, z1, x2, y2, z2)``
    returning the new energy array.

    ``lattice_offset`` moves the lattice against the shape, as a shape's ``lattice_offset``
    does in the reference (``hexagon_ac`` sets one).

    ``device="gpu"`` builds the sites and the CSR matrix on the GPU (``kpm_lattice.h``);
    the modifiers still run here on the numpy arrays. Both builds give identical models.
    """
    f32 = np.float32
    v0, v1, sub_pos, origin, s0, s1 = _honeycomb_frame(vertices, a, a_cc, float_constants, lattice_offset)
    dtype = _scalar_type(is_complex, is_double)
    if device is not None:
        if device != "gpu":
            raise ValueError("device must be None (host build) or 'gpu'")
        return _build_honeycomb_gpu(vertices, v0, v1, sub_pos, origin, s0, s1, onsite_modifiers,
                                    hopping_modifiers, dtype, min_neighbors, t, is_complex, is_double, name)
    rel_ab = _HONEYCOMB_HOPS
    rel = [rel_ab, [(-da, -db) for da, db in rel_ab]]

    bb = np.arange(s1)
    aa = np.arange(s0)
    xs, ys, zs = [], [], []
    for n in range(2):
        ps = origin + sub_pos[n]
        pb = np.empty((s1, 3), f32)
        pb[0] = ps
        pb[1:] = ps[None, :] + bb[1:, None].astype(f32) * v1[None, :]
        pa = pb[:, None, :] + aa[None, :, None].astype(f32) * v0[None, None, :]
        xs.append(pa[..., 0].ravel())
        ys.append(pa[..., 1].ravel())
        zs.append(pa[..., 2].ravel())
    x = np.concatenate(xs)
    y = np.concatenate(ys)
    z = np.concatenate(zs)
    block = s0 * s1
    total = 2 * block

    valid = polygon_contains(np.asarray(vertices, np.float32), x, y)

    # neighbour table in foundation (flat) indices
    nbr = np.full((total, 3), -1, np.int64)
    a_idx = np.tile(aa, s1)
    b_idx = np.repeat(bb, s0)
    for n in range(2):
        other = 1 - n
        for h, (da, db) in enumerate(rel[n]):
            na, nb = a_idx + da, b_idx + db
            ok = (na >= 0) & (na < s0) & (nb >= 0) & (nb < s1)
            tgt = other * block + nb * s0 + na
            nbr[n * block:(n + 1) * block, h] = np.where(ok, tgt, -1)

    valid = _k_core(valid, nbr, min_neighbors)

    final = np.full(total, -1, np.int64)
    nvalid = int(valid.sum())
    final[valid] = np.arange(nvalid)
    na_valid = int(valid[:block].sum())
    sub_ranges = {"A": (0, na_valid), "B": (na_valid, nvalid)}
    sx, sy, sz = x[valid], y[valid], z[valid]

    # hoppings owned by A sites (row = A site, col = B site)
    a_sites = np.nonzero(valid[:block])[0]
    rows, cols = [], []
    for h in range(3):
        tgt = nbr[a_sites, h]
        ok = tgt >= 0
        ok[ok] &= valid[tgt[ok]]
        rows.append(final[a_sites[ok]])
        cols.append(final[tgt[ok]])
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    sub_of = np.zeros(nvalid, np.int8)
    sub_of[na_valid:] = 1

    hop = _hopping_energies(dtype, t, rows.size, rows, cols, sx, sy, sz, hopping_modifiers)
    onsite = _onsite_energies(dtype, sx, sy, sz, sub_of, onsite_modifiers)

    r_all = [rows, cols]
    c_all = [cols, rows]
    v_all = [hop, np.conj(hop)]
    nz = onsite != 0
    if nz.any():
        d = np.nonzero(nz)[0]
        r_all.append(d)
        c_all.append(d)
        v_all.append(onsite[d])
    h = _csr_sorted(np.concatenate(r_all), np.concatenate(c_all), np.concatenate(v_all), nvalid, dtype)
    system = System(sx, sy, sz, sub_ranges)
    return Model(h, system, is_complex=is_complex, is_double=is_double, name=name)


def _build_honeycomb_gpu(vertices, v0, v1, sub_pos, origin, s0, s1, onsite_modifiers, hopping_modifiers, dtype,
                         min_neighbors, t, is_complex, is_double, name):
    """The device build behind ``build_honeycomb(device="gpu")``: positions, polygon
    membership, dangling-site removal, numbering and the CSR rows run as CUDA kernels."""
    from ._native import LatticeBuild
    b = LatticeBuild.honeycomb(s0, s1, origin, v0, v1, sub_pos, _HONEYCOMB_HOPS,
                               np.asarray(vertices, np.float32), min_neighbors)
    try:
        n, n0, nh, _ = b.sizes()
        sx, sy, sz = b.sites()
        hop_values = None
        if hopping_modifiers:
            rows, cols = b.hoppings()
            hop_values = _hopping_energies(dtype, t, nh, rows, cols, sx, sy, sz, hopping_modifiers)
        onsite = None
        if onsite_modifiers:
            sub_of = np.zeros(n, np.int8)
            sub_of[n0:] = 1
            onsite = _onsite_energies(dtype, sx, sy, sz, sub_of, onsite_modifiers)
        indptr, indices, values = b.csr(dtype, hopping=None if hop_values is not None else t,
                                        hopping_values=hop_values, onsite=onsite)
    finally:
        b.close()
    h = sp.csr_matrix((values, indices, indptr), shape=(n, n))
    h.has_sorted_indices = True
    system = System(sx, sy, sz, {"A": (0, n0), "B": (n0, n)})
    return Model(h, system, is_complex=is_complex, is_double=is_double, name=name)


def _csr_sorted(rows, cols, vals, n, dtype):
    """CSR with sorted column indices per row from (row, col, value) triples without
    duplicates: a counting sort by row (COO -> CSR, O(nnz)) and a per-row sort of the few
    columns of each row, instead of a global lexicographic sort."""
    m = sp.coo_matrix((np.asarray(vals).astype(dtype), (rows.astype(np.int32), cols.astype(np.int32))),
                      shape=(n, n)).tocsr()
    m.sort_indices()
    m.indptr = m.indptr.astype(np.int32, copy=False)
    m.indices = m.indices.astype(np.int32, copy=False)
    return m


# --------------------------------------------------------------------------- modifiers

def constant_potential(magnitude):
    """``pb.constant_potential`` (pybinding/modifier.py:391-402)."""
    def f(energy, x, y, z, sub):
        return energy + energy.dtype.type(magnitude)
    return f


def mass_term(delta):
    """``graphene.mass_term`` (repository/graphene/modifiers.py:9-24)."""
    def f(energy, x, y, z, sub):
        e = energy.copy()
        e[sub == 0] += delta
        e[sub == 1] -= delta
        return e
    return f


def constant_magnetic_field(magnitude):
    """Peierls phase of a perpendicular field (repository/graphene/modifiers.py:62-81).

    Computed in the precision of the numpy inputs as the reference's modifier is
    (float32 positions, complex64 energies).
    """
    scale = 1e-18
    const = scale * 2 * math.pi / PHI0

    def f(energy, x1, y1, z1, x2, y2, z2):
        vp_x = 0.5 * magnitude * (y1 + y2)
        peierls = vp_x * (x1 - x2)
        return energy * np.exp(1j * const * peierls)
    return f


def strained_hopping(displacement):
    """Hopping ``t * exp(-beta (d/a_cc - 1))`` for displaced sites
    (repository/graphene/modifiers.py:84-90); ``displacement(x, y) -> (ux, uy)``."""
    def f(energy, x1, y1, z1, x2, y2, z2):
        ux1, uy1 = displacement(x1, y1)
        ux2, uy2 = displacement(x2, y2)
        dx = (x1 + ux1) - (x2 + ux2)
        dy = (y1 + uy1) - (y2 + uy2)
        dz = z1 - z2
        d = np.sqrt(dx * dx + dy * dy + dz * dz)
        return energy * np.exp(-GRAPHENE_BETA * (d / GRAPHENE_A_CC - 1))
    return f


def sinusoidal_strain(amplitude, period):
    """Smooth in-plane displacement ``u = amplitude * period/(2 pi) * sin(2 pi x/period)``
    along x: a strain field of peak magnitude ``amplitude``."""
    def disp(x, y):
        k = 2 * np.pi / period
        ux = (amplitude / k) * np.sin(k * x)
        return ux.astype(x.dtype), np.zeros_like(y)
    return disp


def anderson_disorder(width, seed):
    """Onsite energies uniform in [-width/2, width/2] from a seeded numpy generator."""
    def f(energy, x, y, z, sub):
        rng = np.random.default_rng(seed)
        return energy + rng.uniform(-width / 2, width / 2, size=energy.shape).astype(energy.dtype)
    return f


# --------------------------------------------------------------------------- synthetic configs

GRAPHENE_SITE_DENSITY = 4 / (math.sqrt(3) * GRAPHENE_A ** 2)  # sites per nm^2


def graphene_flake(num_sites, aspect=1.0, **kw):
    """A rectangular graphene flake with about ``num_sites`` sites."""
    area = num_sites / GRAPHENE_SITE_DENSITY
    w = math.sqrt(area * aspect)
    h = area / w
    return build_honeycomb(rectangle(w, h), **kw)


def simple_cubic_periodic(L, t=-1.0, onsite=None, dtype=np.float32, device=None):
    """Simple cubic L^3 lattice with periodic boundaries, 6 hoppings per site.

    Site index = (z*L + y)*L + x. ``onsite`` is an optional array of L^3 energies
    (zeros, in ``dtype``, are not stored). The periodic wrap makes the Hamiltonian real
    at k = 0. ``device="gpu"`` builds the CSR matrix on the GPU (``kpm_lattice.h``, L >= 3).
    """
    n = L ** 3
    f32 = np.float32
    ons = None if onsite is None else np.asarray(onsite, dtype)
    if device is not None:
        if device != "gpu":
            raise ValueError("device must be None (host build) or 'gpu'")
        from ._native import LatticeBuild
        b = LatticeBuild.cubic(L)
        try:
            sx, sy, sz = b.sites()
            indptr, indices, values = b.csr(dtype, hopping=t, onsite=ons)
        finally:
            b.close()
        h = sp.csr_matrix((values, indices, indptr), shape=(n, n))
        h.has_sorted_indices = True
        return Model(h, System(sx, sy, sz, {"A": (0, n)}), name="cubic")
    idx = np.arange(n, dtype=np.int64)
    xi = idx % L
    yi = (idx // L) % L
    zi = idx // (L * L)
    rows, cols = [], []
    for dx, dy, dz in [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]:
        j = (((zi + dz) % L) * L + (yi + dy) % L) * L + (xi + dx) % L
        rows.append(idx)
        cols.append(j)
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    vals = np.full(rows.size, t, dtype)
    if ons is not None:
        nz = np.nonzero(ons)[0]
        rows = np.concatenate([rows, nz])
        cols = np.concatenate([cols, nz])
        vals = np.concatenate([vals, ons[nz]])
    h = _csr_sorted(rows, cols, vals, n, dtype)
    system = System(xi.astype(f32), yi.astype(f32), zi.astype(f32), {"A": (0, n)})
    return Model(h, system, name="cubic")


# --------------------------------------------------------------------------- 3-band TMD monolayers
# Nearest-neighbour three-band model of group-6 transition-metal dichalcogenides (metal d_z2,
# d_xy, d_x2-y2 orbitals on a triangular lattice; Liu et al., Phys. Rev. B 88, 085433 (2013),
# the parameters pybinding/repository/group6_tmd.py:7-14 uses):
#            a (nm), eps1,  eps2,   t0,     t1,    t2,    t11,   t12,   t22
TMD_3BAND = {
    "MoS2": (0.3190, 1.046, 2.104, -0.184, 0.401, 0.507, 0.218, 0.338, 0.057),
    "WS2": (0.3191, 1.130, 2.275, -0.206, 0.567, 0.536, 0.286, 0.384, -0.061),
    "MoSe2": (0.3326, 0.919, 2.065, -0.188, 0.317, 0.456, 0.211, 0.290, 0.130),
    "WSe2": (0.3325, 0.943, 2.179, -0.207, 0.457, 0.486, 0.263, 0.329, 0.034),
    "MoTe2": (0.3557, 0.605, 1.972, -0.169, 0.228, 0.390, 0.207, 0.239, 0.252),
    "WTe2": (0.3560, 0.606, 2.102, -0.175, 0.342, 0.410, 0.233, 0.270, 0.190),
}


def _tmd_hopping_blocks(t0, t1, t2, t11, t12, t22):
    """The 3 x 3 hopping matrices of the bonds a1, -a2 and a1 - a2 (the three a metal site owns).
    The bond along a1 (angle 0) has E(R1) below; a bond at angle phi is the C3-related matrix
    U(phi) E(R1) U(phi)^T, where U rotates (d_z2, d_xy, d_x2-y2) by phi (the d_xy / d_x2-y2 pair
    turns by 2 phi), and reversing a bond transposes its matrix: -a2 points at 240 degrees and
    a1 - a2 at 300 degrees, the reverse of the bond at 120 degrees."""
    e1 = np.array([[t0, -t1, t2], [t1, t11, -t12], [t2, t12, t22]])

    def rotate(deg):
        c, s = math.cos(math.radians(2 * deg)), math.sin(math.radians(2 * deg))
        u = np.array([[1.0, 0, 0], [0, c, s], [0, -s, c]])
        return u @ e1 @ u.T
    return [((1, 0), e1), ((0, -1), rotate(240)), ((1, -1), rotate(120).T)]


def build_tmd_3band(vertices, material="MoS2", min_neighbors=1, is_double=False, name=None):
    """A group-6 TMD monolayer (three orbitals per metal site) cut by the polygon ``vertices``, in
    pybinding's site and Hamiltonian order: sites of the triangular lattice a1 = (a, 0),
    a2 = (a/2, a sqrt(3)/2) inside the polygon (foundation and float32 positions as for the
    honeycomb builder), dangling sites removed down to ``min_neighbors`` (the lattice default 1),
    Hamiltonian row 3 i + k for orbital k of site i (``System.cpp:33-48``), onsite
    diag(eps1, eps2, eps2), each bond's 3 x 3 block stored for the owning site and its transpose
    for the other (``Hamiltonian.hpp:74-100``). Real; float32 unless ``is_double``."""
    f32 = np.float32
    a, eps1, eps2, t0, t1, t2, t11, t12, t22 = TMD_3BAND[material]
    v0 = np.array([a, 0, 0], f32)
    v1 = np.array([a / 2, a / 2 * math.sqrt(3), 0], f32)
    m = np.array([[v0[0], v1[0]], [v0[1], v1[1]]], dtype=np.float64)
    coords = np.linalg.solve(m, np.asarray(vertices, np.float64).T).T
    ic = np.trunc(coords).astype(np.int64)
    lo = ic.min(axis=0) - 1
    hi = ic.max(axis=0) + 1
    s0, s1 = int(hi[0] - lo[0] + 1), int(hi[1] - lo[1] + 1)
    origin = np.zeros(3, f32) + f32(lo[0]) * v0
    origin = origin + f32(lo[1]) * v1
    bb = np.arange(s1)
    aa = np.arange(s0)
    pb = np.empty((s1, 3), f32)
    pb[0] = origin
    pb[1:] = origin[None, :] + bb[1:, None].astype(f32) * v1[None, :]
    pa = pb[:, None, :] + aa[None, :, None].astype(f32) * v0[None, None, :]
    x, y, z = pa[..., 0].ravel(), pa[..., 1].ravel(), pa[..., 2].ravel()
    total = s0 * s1
    valid = polygon_contains(np.asarray(vertices, np.float32), x, y)
    blocks = _tmd_hopping_blocks(t0, t1, t2, t11, t12, t22)
    a_idx = np.tile(aa, s1)
    b_idx = np.repeat(bb, s0)
    offsets = [d for d, _ in blocks] + [(-da, -db) for (da, db), _ in blocks]
    nbr = np.full((total, len(offsets)), -1, np.int64)
    for h, (da, db) in enumerate(offsets):
        na, nb = a_idx + da, b_idx + db
        ok = (na >= 0) & (na < s0) & (nb >= 0) & (nb < s1)
        nbr[:, h] = np.where(ok, nb * s0 + na, -1)
    valid = _k_core(valid, nbr, min_neighbors)
    final = np.full(total, -1, np.int64)
    nvalid = int(valid.sum())
    final[valid] = np.arange(nvalid)
    dtype = np.float64 if is_double else np.float32
    sites = np.nonzero(valid)[0]
    rows, cols, vals = [], [], []
    for h, (_, e) in enumerate(blocks):
        tgt = nbr[sites, h]
        ok = tgt >= 0
        ok[ok] &= valid[tgt[ok]]
        i, j = final[sites[ok]], final[tgt[ok]]
        for p in range(3):
            for q in range(3):
                rows += [3 * i + p, 3 * j + q]
                cols += [3 * j + q, 3 * i + p]
                vals += [np.full(i.size, e[p, q]), np.full(i.size, e[p, q])]
    diag = np.array([eps1, eps2, eps2])
    d = np.arange(3 * nvalid)
    rows.append(d)
    cols.append(d)
    vals.append(np.tile(diag, nvalid))
    h = _csr_sorted(np.concatenate(rows), np.concatenate(cols), np.concatenate(vals).astype(dtype), 3 * nvalid,
                    dtype)
    metal = material[:2] if material[1].islower() else material[:1]
    system = System(x[valid], y[valid], z[valid], {metal: (0, nvalid)}, orbitals=3)
    return Model(h, system, is_double=is_double, name=name or material)

