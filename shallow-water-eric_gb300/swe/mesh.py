"""Mesh I/O and synthetic mesh generators (host side).

* ``read_fem`` / ``load_mesh_free_format`` read the reference's unformatted
  ``.FEM`` files (gfortran sequential records, 4-byte markers) and renumber
  nodes in first-touch element order exactly like
  SFEMaNS/FEMSUB_OBJET/prep_mesh.f90:759-1035.
* ``dirichlet_nodes`` follows SFEMaNS/FEMSUB/dir_nodes.f90:243-292,495-511.
* ``lattice_mesh`` / ``jittered_mesh`` build the synthetic P1 meshes used by
  the workloads (structured right-triangle lattice; jittered-lattice
  Delaunay triangulation).

Meshes are dicts with ``jj`` (3, me) int32 1-based, counter-clockwise;
``rr`` (2, np) float64; ``jjs`` (2, mes) boundary edges 1-based; ``sides``
(mes,) side ids.
"""
from __future__ import annotations

import gzip
import struct
from pathlib import Path

import numpy as np


def _records(buf: bytes):
    off = 0
    out = []
    while off < len(buf):
        (n,) = struct.unpack_from("<i", buf, off)
        out.append(buf[off + 4: off + 4 + n])
        (n2,) = struct.unpack_from("<i", buf, off + 4 + n)
        if n2 != n:
            raise ValueError("corrupt record markers in .FEM file")
        off += 8 + n
    return out


def read_fem(path):
    """Raw content of a P1 ``.FEM`` file (no renumbering); a ``.gz`` name
    is read through gzip."""
    path = Path(path)
    buf = gzip.decompress(path.read_bytes()) if path.suffix == ".gz" else path.read_bytes()
    recs = _records(buf)
    np_, nw, me, nws, mes = struct.unpack("<5i", recs[0][:20])
    if (nw, nws) != (3, 2):
        raise ValueError("only P1 triangle meshes are supported")
    a = np.frombuffer(recs[1], dtype="<i4")
    jj = a[: 3 * me].reshape(me, 3).T
    neigh = a[3 * me: 6 * me].reshape(me, 3).T
    i_d = a[6 * me: 7 * me]
    b = np.frombuffer(recs[2], dtype="<i4")
    jjs = b[: 2 * mes].reshape(mes, 2).T
    neighs = b[2 * mes: 3 * mes]
    sides = b[3 * mes: 4 * mes]
    rr = np.frombuffer(recs[3], dtype="<f8")[: 2 * np_].reshape(np_, 2).T
    return dict(np=np_, me=me, mes=mes, jj=jj.copy(), neigh=neigh.copy(), i_d=i_d.copy(),
                jjs=jjs.copy(), neighs=neighs.copy(), sides=sides.copy(), rr=rr.copy())


def load_mesh_free_format(path, list_dom=(1,)):
    """Read and renumber like prep_mesh.f90:759-1035 (P1, 2D)."""
    raw = read_fem(path)
    jj_l, neigh_l, i_d_l = raw["jj"], raw["neigh"], raw["i_d"]
    me, np_ = raw["me"], raw["np"]
    dom = set(int(d) for d in list_dom)
    nouv_nd = np.zeros(np_ + 1, np.int64)
    virgin = np.ones(np_ + 1, bool)
    nouv_el = np.zeros(me + 1, np.int64)
    ancien_el = []
    ancien_nd = []
    for m in range(me):
        if int(i_d_l[m]) not in dom:
            continue
        ancien_el.append(m)
        nouv_el[m + 1] = len(ancien_el)
        for n in range(3):
            i = int(jj_l[n, m])
            if virgin[i]:
                virgin[i] = False
                ancien_nd.append(i)
                nouv_nd[i] = len(ancien_nd)
    ae = np.array(ancien_el)
    jj = nouv_nd[jj_l[:, ae]].astype(np.int32)
    # boundary sides (the side-switching branch only matters for multi-domain
    # meshes; with one domain every side keeps its element)
    jjs_l, neighs_l, sides_l = raw["jjs"], raw["neighs"], raw["sides"]
    keep = []
    for ms in range(raw["mes"]):
        m1 = int(neighs_l[ms])
        ok = int(i_d_l[m1 - 1]) in dom
        if not ok:
            # the element on the other side of the face
            for n in range(3):
                if int(jj_l[n, m1 - 1]) not in (int(jjs_l[0, ms]), int(jjs_l[1, ms])):
                    break
            m2 = int(neigh_l[n, m1 - 1])
            ok = m2 != 0 and int(i_d_l[m2 - 1]) in dom
        if ok:
            keep.append(ms)
    keep = np.array(keep, dtype=np.int64)
    jjs = nouv_nd[jjs_l[:, keep]].astype(np.int32)
    sides = sides_l[keep].astype(np.int32)
    rr = raw["rr"][:, np.array(ancien_nd) - 1].copy()
    return dict(jj=np.asfortranarray(jj), rr=np.asfortranarray(rr), jjs=jjs, sides=sides)


def write_fem(path, mesh):
    """Write a P1 mesh as an unformatted ``.FEM`` file (one domain, id 1)."""
    jj, rr, jjs, sides = mesh["jj"], mesh["rr"], mesh["jjs"], mesh["sides"]
    me, np_, mes = jj.shape[1], rr.shape[1], jjs.shape[1]
    neigh = np.zeros((3, me), np.int32)
    neighs = np.ones(mes, np.int32)

    def rec(b: bytes):
        return struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))

    out = rec(struct.pack("<5i", np_, 3, me, 2, mes))
    out += rec(np.ascontiguousarray(jj.T, "<i4").tobytes() + np.ascontiguousarray(neigh.T, "<i4").tobytes()
               + np.ones(me, "<i4").tobytes())
    out += rec(np.ascontiguousarray(jjs.T, "<i4").tobytes() + neighs.astype("<i4").tobytes()
               + sides.astype("<i4").tobytes())
    out += rec(np.ascontiguousarray(rr.T, "<f8").tobytes())
    Path(path).write_bytes(out)


def dirichlet_nodes(jjs, sides, dir_list):
    """Sorted unique nodes of boundary edges on the listed sides (1-based)."""
    if len(dir_list) == 0:
        return np.zeros(0, np.int32)
    sel = np.isin(sides, np.asarray(dir_list))
    return np.unique(jjs[:, sel].ravel()).astype(np.int32)


def _ccw(jj, rr):
    x, y = rr[0], rr[1]
    a, b, c = jj[0] - 1, jj[1] - 1, jj[2] - 1
    cross = (x[b] - x[a]) * (y[c] - y[a]) - (y[b] - y[a]) * (x[c] - x[a])
    flip = cross < 0
    jj = jj.copy()
    jj[1, flip], jj[2, flip] = jj[2, flip].copy(), jj[1, flip].copy()
    return jj


def _rect_boundary(jj, rr, x0, x1, y0, y1, tol):
    """Boundary edges of a rectangle mesh with side ids 1=x-min, 2=y-min,
    3=x-max, 4=y-max."""
    e = np.concatenate([jj[[0, 1]].T, jj[[1, 2]].T, jj[[2, 0]].T]) - 1
    key = np.sort(e, axis=1)
    uniq, cnt = np.unique(key, axis=0, return_counts=True)
    b = uniq[cnt == 1]
    x, y = rr[0], rr[1]
    side = np.zeros(len(b), np.int32)
    xm = 0.5 * (x[b[:, 0]] + x[b[:, 1]])
    ym = 0.5 * (y[b[:, 0]] + y[b[:, 1]])
    side[np.abs(xm - x0) < tol] = 1
    side[np.abs(ym - y0) < tol] = 2
    side[np.abs(xm - x1) < tol] = 3
    side[np.abs(ym - y1) < tol] = 4
    return (b.T + 1).astype(np.int32), side


def lattice_mesh(nx, ny, x0=0.0, x1=1.0, y0=0.0, y1=1.0):
    """(nx x ny)-vertex structured right-triangle lattice, every cell cut
    along its SW->NE diagonal.  Node n = i + nx*j (x fastest), 1-based."""
    xs = np.linspace(x0, x1, nx)
    ys = np.linspace(y0, y1, ny)
    X, Y = np.meshgrid(xs, ys)           # (ny, nx)
    rr = np.vstack([X.ravel(), Y.ravel()])
    i, j = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1))
    i, j = i.ravel(), j.ravel()
    sw = i + nx * j
    se, nw_, ne = sw + 1, sw + nx, sw + nx + 1
    t1 = np.vstack([sw, se, ne])
    t2 = np.vstack([sw, ne, nw_])
    jj = (np.hstack([t1, t2]) + 1).astype(np.int32)
    # order elements cell by cell (t1, t2 of the same cell adjacent)
    order = np.arange(jj.shape[1]).reshape(2, -1).T.ravel()
    jj = jj[:, order]
    tol = 1e-9 * max(x1 - x0, y1 - y0)
    jjs, sides = _rect_boundary(jj, rr, x0, x1, y0, y1, tol)
    return dict(jj=np.asfortranarray(jj), rr=np.asfortranarray(rr), jjs=jjs, sides=sides)


def jittered_mesh(nx, ny, x0, x1, y0, y1, jitter=0.3, seed=0):
    """Jittered (nx x ny) lattice, Delaunay-triangulated.  Interior points move
    by U(-jitter, jitter)*spacing per axis; boundary points only along their
    side, corners stay fixed, so the domain stays the rectangle."""
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    dx = (x1 - x0) / (nx - 1)
    dy = (y1 - y0) / (ny - 1)
    xs = np.linspace(x0, x1, nx)
    ys = np.linspace(y0, y1, ny)
    X, Y = np.meshgrid(xs, ys)
    jx = rng.uniform(-jitter, jitter, X.shape) * dx
    jy = rng.uniform(-jitter, jitter, Y.shape) * dy
    jx[:, 0] = 0; jx[:, -1] = 0
    jy[0, :] = 0; jy[-1, :] = 0
    X = X + jx
    Y = Y + jy
    rr = np.vstack([X.ravel(), Y.ravel()])
    tri = Delaunay(rr.T, qhull_options="Qbb Qc Qz Q12").simplices.T.astype(np.int64)
    jj = _ccw((tri + 1).astype(np.int32), rr)
    x, y = rr[0], rr[1]
    a, b, c = jj[0] - 1, jj[1] - 1, jj[2] - 1
    area = 0.5 * ((x[b] - x[a]) * (y[c] - y[a]) - (y[b] - y[a]) * (x[c] - x[a]))
    if jj.shape[1] != 2 * (nx - 1) * (ny - 1) or not (area > 1e-12 * dx * dy).all():
        raise RuntimeError("degenerate Delaunay triangulation of the jittered lattice")
    # element order: by centroid row then x, so that element (and first-touch
    # node) order follows the lattice
    cy = (y[a] + y[b] + y[c]) / 3
    cx = (x[a] + x[b] + x[c]) / 3
    order = np.lexsort((cx, np.floor(cy / dy)))
    jj = np.ascontiguousarray(jj[:, order])
    # the hull is the rectangle and every lattice boundary point is a hull
    # vertex (boundary points only move along their side), so the boundary
    # edges join consecutive lattice boundary points: 1=x-min 2=y-min 3=x-max 4=y-max
    i = np.arange(nx)
    j = np.arange(ny)
    segs = [(j * nx, 1, ny), (i, 2, nx), (j * nx + nx - 1, 3, ny), (i + nx * (ny - 1), 4, nx)]
    jjs = np.hstack([np.vstack([n[:-1], n[1:]]) for n, _, _ in segs]) + 1
    sides = np.concatenate([np.full(k - 1, sd) for _, sd, k in segs])
    return dict(jj=np.asfortranarray(jj), rr=np.asfortranarray(rr), jjs=jjs.astype(np.int32),
                sides=sides.astype(np.int32))


def concat_meshes(meshes):
    """Concatenate independent meshes into one node/element space (batching)."""
    jj, rr, off = [], [], 0
    node_off, elem_off = [0], [0]
    for m in meshes:
        jj.append(m["jj"] + off)
        rr.append(m["rr"])
        off += m["rr"].shape[1]
        node_off.append(off)
        elem_off.append(elem_off[-1] + m["jj"].shape[1])
    return (np.asfortranarray(np.hstack(jj)), np.asfortranarray(np.hstack(rr)),
            np.array(node_off, np.int64), np.array(elem_off, np.int64))
