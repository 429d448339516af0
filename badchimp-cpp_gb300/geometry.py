"""Geometry: seeded porous media and the reference's sparse node numbering.

Two parts:

* ``sphere_pack`` / ``channel_2d`` make voxel masks (1 = fluid, 0 = solid).
  The reference has no 3D sphere-pack generator; this one places spheres of a
  fixed radius with centres drawn from ``numpy.random.default_rng(seed)``
  uniformly in the box (periodic distance, overlap allowed) until the fluid
  fraction reaches the target porosity.

* ``build_lattice`` turns a mask into the arrays the reference's ``Grid`` and
  ``Nodes`` hold after reading a ``.vtklb`` file written by
  ``PythonScripts/vtklb.py``: the node numbering, the neighbour table
  ``neigList_[node*nQ + q]`` (src/lbsolver/LBgrid.h:119, 160), the positions
  ``pos_`` (LBgrid.h:120) and the node types of ``Nodes::setupNodeType``
  (src/lbsolver/LBnodes.h:141-209).  The numbering rules restated here are the
  single-rank case of ``vtklb.setup_processor_labels`` and
  ``write_neighbors_fast`` (PythonScripts/vtklb.py:6-45, 84-114, 182-218):

  - node 0 is the ghost node;
  - fluid nodes are numbered 1..Nf in C order of the interior (x slowest);
  - then every solid that is a lattice neighbour of a fluid node, in C order of
    the array padded by a one-node rim; a periodic rim position is a separate
    node (the rim copies the opposite interior layer, vtklb.py:97-114);
  - a neighbour outside the padded array, or at an unlisted position, is node 0,
    except that a rim position holding fluid maps to the interior fluid node it
    copies (vtklb.py:34-39).

Everything is plain numpy so that tables for 256^3 boxes build in seconds.
"""

from __future__ import annotations

import numpy as np

# Lattice velocity sets in the reference's order, rest direction last
# (src/lbsolver/LBd2q9.h:33, src/lbsolver/LBd3q19.h:33; PythonScripts/vtklb.py:171-176).
D2Q9_C = np.array([[1, 0], [1, 1], [0, 1], [-1, 1], [-1, 0], [-1, -1], [0, -1], [1, -1], [0, 0]],
                  dtype=np.int64)
D3Q19_C = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, -1, 0], [1, 0, 1], [1, 0, -1],
                    [0, 1, 1], [0, 1, -1], [-1, 0, 0], [0, -1, 0], [0, 0, -1], [-1, -1, 0],
                    [-1, 1, 0], [-1, 0, -1], [-1, 0, 1], [0, -1, -1], [0, -1, 1], [0, 0, 0]],
                   dtype=np.int64)
LATTICE_C = {"D2Q9": D2Q9_C, "D3Q19": D3Q19_C}
LATTICE_Q = {"D2Q9": 9, "D3Q19": 19}


def lattice_name(q: int) -> str:
    if q == 9:
        return "D2Q9"
    if q == 19:
        return "D3Q19"
    raise ValueError(f"unsupported lattice with {q} directions")


def tagged_pack(shape, radius: float, porosity: float, seed: int, blob_radius: float = 5.0,
                blob_spacing: int = 24, ghost_layers: bool = True):
    """A synthetic input of the std_one_phase step (src/std_one_phase/main.cpp):
    a box periodic in x and y whose z faces are pressure boundaries, with the
    node attributes that step reads, as voxel arrays.  The reference's own
    inputs are level-set phase distributions in rock images, which are not
    available; this stands in for them.

    * mask: a periodic sphere pack (``sphere_pack``); with ghost_layers the
      faces z = 0 and z = nz-1 are pressure ghost nodes (solid, tag 3);
    * phase 2: balls of ``blob_radius`` on a regular grid of spacing
      ``blob_spacing`` inside the box, each an interior domain (label 1, 2, ...)
      when it has at least one node without interface bits; phase 1 elsewhere;
    * nodetags: 0 solid, 1 / 2 fluid phase, 3 pressure ghost, +4 next to the
      other phase, +8 next to a solid, +16 next to a pressure ghost (D3Q19
      neighbours; beyond the z faces the neighbour is node 0, tag -1);
    * force: 1 on fluid, 0 on solid; interior_domains: the labels.

    Returns (mask, attrs) with int32 arrays ``nodetags``, ``interior_domains``
    and ``force`` of the mask's shape."""
    shape = tuple(int(n) for n in shape)
    nx, ny, nz = shape
    mask = sphere_pack(shape, radius, porosity, seed)[0].copy()
    ghost = np.zeros(shape, dtype=bool)
    if ghost_layers:
        mask[:, :, 0] = 0
        mask[:, :, -1] = 0
        ghost[:, :, 0] = ghost[:, :, -1] = True
    fluid = mask == 1
    phase = np.where(fluid, 1, 0).astype(np.int64)
    labels = np.zeros(shape, dtype=np.int64)
    x, y, z = (np.arange(n) for n in shape)
    h = blob_spacing
    cz = np.arange(h // 2 + 2, nz - h // 2 - 1, h)
    blobs = [(a, b, c) for a in range(h // 2, nx, h) for b in range(h // 2, ny, h) for c in cz]
    r2 = float(blob_radius) ** 2
    ri = int(np.ceil(blob_radius))
    for k, (a, b, c) in enumerate(blobs, start=1):
        sx, sy, sz = (slice(max(v - ri, 0), min(v + ri + 1, n)) for v, n in ((a, nx), (b, ny), (c, nz)))
        d2 = (x[sx, None, None] - a) ** 2 + (y[None, sy, None] - b) ** 2 + (z[None, None, sz] - c) ** 2
        sel = (d2 <= r2) & fluid[sx, sy, sz]
        phase[sx, sy, sz][sel] = 2
        labels[sx, sy, sz][sel] = k
    tags = np.where(ghost, 3, phase).astype(np.int64)
    base = tags.copy()
    other = np.where(phase == 1, 2, 1)
    for c in D3Q19_C[:18]:
        nb = np.roll(base, shift=(-c[0], -c[1]), axis=(0, 1))
        if c[2] != 0:
            nb = np.roll(nb, shift=-c[2], axis=2)
            if c[2] > 0:
                nb[:, :, -1] = -1
            else:
                nb[:, :, 0] = -1
        tags[fluid & ((nb & 3) == other) & ((nb & 3) != 0)] |= 4
        tags[fluid & ((nb & 3) == 0) & (nb >= 0)] |= 8
        tags[fluid & ((nb & 3) == 3)] |= 16
    # drop the labels of blobs that have no interior (untagged) node
    present = np.unique(labels[labels > 0])
    keep = np.unique(labels[(labels > 0) & (tags < 3)])
    remap = np.zeros(int(labels.max()) + 1, dtype=np.int64)
    remap[keep] = np.arange(1, keep.size + 1)
    labels = remap[labels]
    del present
    attrs = {"nodetags": tags.astype(np.int32), "interior_domains": labels.astype(np.int32),
             "force": fluid.astype(np.int32)}
    return mask, attrs


def channel_2d(nx: int = 256, ny: int = 64) -> np.ndarray:
    """2D channel: solid rows y=0 and y=ny-1, fluid in between (x periodic by the caller)."""
    geo = np.ones((nx, ny), dtype=np.int8)
    geo[:, 0] = 0
    geo[:, ny - 1] = 0
    return geo


def sphere_pack(shape, radius: float, porosity: float, seed: int, max_spheres: int = 10_000_000):
    """Periodic random pack of solid spheres; returns (mask, centres, porosity).

    Spheres of radius ``radius`` (voxel ``i`` is solid when its periodic
    distance to a centre is <= radius) are added one at a time, centres drawn
    uniformly in the box from ``default_rng(seed)``, until the fluid fraction is
    at most ``porosity``.
    """
    shape = tuple(int(n) for n in shape)
    nd = len(shape)
    rng = np.random.default_rng(seed)
    solid = np.zeros(shape, dtype=bool)
    total = solid.size
    nsolid = 0
    centres = []
    r = float(radius)
    ri = int(np.ceil(r))
    offs = np.arange(-ri, ri + 1)
    grids = np.meshgrid(*([offs] * nd), indexing="ij")
    while (total - nsolid) / total > porosity:
        if len(centres) >= max_spheres:
            break
        c = rng.uniform(0.0, 1.0, size=nd) * np.asarray(shape, dtype=np.float64)
        centres.append(c)
        base = np.floor(c).astype(np.int64)
        d2 = np.zeros(grids[0].shape, dtype=np.float64)
        idx = []
        for d in range(nd):
            p = base[d] + grids[d]
            diff = p - c[d]
            d2 += diff * diff
            idx.append(np.mod(p, shape[d]))
        inside = d2 <= r * r
        sel = tuple(ix[inside] for ix in idx)
        before = np.count_nonzero(solid[sel])
        solid[sel] = True
        nsolid += np.count_nonzero(solid[sel]) - before
    mask = (~solid).astype(np.int8)
    return mask, np.asarray(centres), float(np.count_nonzero(mask)) / total


def build_lattice(geo: np.ndarray, lattice: str, periodic: str = "") -> dict:
    """Node numbering, neighbour table, positions and node types for one rank.

    ``geo`` holds 1 for fluid and 0 for solid.  Returns a dict with
    ``neigh`` (int32 [N*Q], row 0 all zero), ``types`` (int16 [N]),
    ``pos`` (int32 [N*nD], -1 for node 0), ``nf`` (fluid count) and ``ns``
    (stored boundary-solid count); N = 1 + nf + ns.  Built on the host cores by
    the library's bclbm_lattice_build; ``build_lattice_numpy`` is the same
    numbering in numpy.
    """
    from . import native

    c = LATTICE_C[lattice]
    nq, nd = c.shape
    geo = np.asarray(geo)
    if geo.ndim != nd:
        raise ValueError(f"{lattice} needs a {nd}-D geometry, got {geo.ndim}-D")
    if not np.all((geo == 0) | (geo == 1)):
        raise ValueError("geometry must hold 0 (solid) and 1 (fluid) only")
    bits = sum(1 << d for d, ax in enumerate("xyz"[:nd]) if ax in periodic.lower())
    neigh, types, pos, nf, ns = native.lattice_tables(geo, nq, bits)
    return {"neigh": neigh, "types": types, "pos": pos, "nf": nf, "ns": ns, "nq": nq, "nd": nd, "lattice": lattice}


def read_vtklb(path, lattice: str, attributes=()) -> dict:
    """The tables of a .vtklb file (written by the reference's vtklb.py) as
    ``build_lattice`` returns them, read by the library's bclbm_lattice_read_vtklb
    (one rank, ASCII, no 2 GiB limit); ``attributes`` names SCALARS to return
    as per-node arrays (key ``attributes``)."""
    from . import native

    nq = LATTICE_Q[lattice]
    neigh, types, pos, nf, ns, attrs = native.read_vtklb(path, nq, tuple(attributes))
    return {"neigh": neigh, "types": types, "pos": pos, "nf": nf, "ns": ns, "nq": nq, "nd": 2 if nq == 9 else 3,
            "lattice": lattice, "attributes": attrs}


def build_lattice_numpy(geo: np.ndarray, lattice: str, periodic: str = "") -> dict:
    """``build_lattice`` in plain numpy (the same arrays, bit for bit)."""
    c = LATTICE_C[lattice]
    nq, nd = c.shape
    geo = np.asarray(geo)
    if geo.ndim != nd:
        raise ValueError(f"{lattice} needs a {nd}-D geometry, got {geo.ndim}-D")
    if not np.all((geo == 0) | (geo == 1)):
        raise ValueError("geometry must hold 0 (solid) and 1 (fluid) only")
    periodic = periodic.lower()
    pshape = tuple(n + 2 for n in geo.shape)
    interior = tuple([slice(1, -1)] * nd)
    P = np.full(pshape, -1, dtype=np.int8)
    P[interior] = geo
    fluid_int = np.zeros(pshape, dtype=bool)
    fluid_int[interior] = geo == 1
    nf = int(np.count_nonzero(fluid_int))
    label = np.zeros(pshape, dtype=np.int32)
    label[fluid_int] = np.arange(1, nf + 1, dtype=np.int32)
    for d, ax in enumerate("xyz"[:nd]):
        if ax in periodic:
            lo = [slice(None)] * nd
            hi = [slice(None)] * nd
            src_lo = [slice(None)] * nd
            src_hi = [slice(None)] * nd
            lo[d], src_lo[d] = 0, -2
            hi[d], src_hi[d] = -1, 1
            P[tuple(lo)] = P[tuple(src_lo)]
            P[tuple(hi)] = P[tuple(src_hi)]
            label[tuple(lo)] = label[tuple(src_lo)]
            label[tuple(hi)] = label[tuple(src_hi)]

    # flat indices into the padded array; a lattice step is a constant offset
    strides = np.cumprod((1,) + pshape[::-1][:-1])[::-1].astype(np.int64)
    offs = c @ strides
    Pf = P.reshape(-1)
    labelf = label.reshape(-1)
    fpos = np.flatnonzero(fluid_int)  # C order == label order; all interior
    added = np.zeros(Pf.size, dtype=bool)
    for off in offs:
        p = fpos + off
        added[p[Pf[p] == 0]] = True
    spos = np.flatnonzero(added)
    ns = int(spos.size)
    local = np.zeros(Pf.size, dtype=np.int32)
    local[fpos] = np.arange(1, nf + 1, dtype=np.int32)
    local[spos] = np.arange(nf + 1, nf + ns + 1, dtype=np.int32)

    n_nodes = 1 + nf + ns
    scoord = np.unravel_index(spos, pshape)
    neigh = np.zeros((n_nodes, nq), dtype=np.int32)
    for q in range(nq):
        # fluid nodes are interior: every neighbour is inside the padded array
        p = fpos + offs[q]
        nb = local[p]
        img = (nb == 0) & (Pf[p] == 1)
        neigh[1:nf + 1, q] = np.where(img, labelf[p], nb)
        # stored solids may sit on the rim: neighbours outside the array are node 0
        ok = np.ones(ns, dtype=bool)
        for d in range(nd):
            x = scoord[d] + c[q, d]
            ok &= (x >= 0) & (x < pshape[d])
        ps = spos[ok] + offs[q]
        nbs = local[ps]
        imgs = (nbs == 0) & (Pf[ps] == 1)
        col = np.zeros(ns, dtype=np.int32)
        col[ok] = np.where(imgs, labelf[ps], nbs)
        neigh[nf + 1:, q] = col
    pos = np.full((n_nodes, nd), -1, dtype=np.int32)
    fcoord = np.unravel_index(fpos, pshape)
    for d in range(nd):
        pos[1:nf + 1, d] = fcoord[d] - 1
        pos[nf + 1:, d] = scoord[d] - 1

    types = node_types(neigh, nf)
    return {"neigh": neigh.reshape(-1), "types": types, "pos": pos.reshape(-1),
            "nf": nf, "ns": ns, "nq": nq, "nd": nd, "lattice": lattice}


def node_types(neigh: np.ndarray, nf: int) -> np.ndarray:
    """Nodes::setupNodeType (src/lbsolver/LBnodes.h:156-209) for one rank.

    Nodes 1..nf are fluid, the rest solid, node 0 the default ghost (-1).
    Solids are 1 with a fluid neighbour, else 0; fluids are 2 with a solid
    neighbour (node 0 counts as solid), else 3.
    """
    neigh = np.asarray(neigh).reshape(-1, neigh.shape[-1] if neigh.ndim == 2 else 1)
    n_nodes = neigh.shape[0]
    fluid = np.zeros(n_nodes, dtype=bool)
    fluid[1:nf + 1] = True
    nbr_fluid = fluid[neigh]
    types = np.zeros(n_nodes, dtype=np.int16)
    has_fluid = nbr_fluid.any(axis=1)
    has_solid = (~nbr_fluid).any(axis=1)
    types[fluid] = np.where(has_solid[fluid], 2, 3)
    solid = ~fluid
    types[solid] = np.where(has_fluid[solid], 1, 0)
    types[0] = -1
    return types


def bounce_back_links(neigh: np.ndarray, types: np.ndarray, nodes: np.ndarray, nq: int) -> list:
    """Link classes of BoundaryHalwWayHelper (src/lbsolver/LBhalfwayhelperclass.h:128-159).

    For each listed node: (node, beta, gamma, delta) with beta the unknown
    direction of each fluid/solid pair, gamma and delta one direction of each
    fluid/fluid and solid/solid pair, for the first nQ/2 directions in order.
    """
    npairs = (nq - 1) // 2
    neigh = np.asarray(neigh).reshape(-1, nq)
    fluid = np.asarray(types) > 1
    out = []
    for node in nodes:
        beta, gamma, delta = [], [], []
        for q in range(npairs):
            a = fluid[neigh[node, q]]
            b = fluid[neigh[node, q + npairs]]
            if a and b:
                gamma.append(q)
            elif a:
                beta.append(q)
            elif b:
                beta.append(q + npairs)
            else:
                delta.append(q)
        out.append((int(node), beta, gamma, delta))
    return out
