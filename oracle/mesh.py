"""CPU restatement of the Node Editor's chunk meshers (test infrastructure only).

Follows reference tools/NodeEditor/MeshNoisePreview.cpp: BuildBloxel3DMesh
(:443-540), BloxelAddQuadAO (:542-590) and BuildHeightMap2DMesh (:956-1004), with
the chunk size as a parameter (the editor uses 128).  Densities come from the
CPU oracle through GenPositionArray3D/2D with the editor's grid position arrays
(GridPositions3D/2D, :31-76).  All arithmetic is float32 (numpy scalars), in the
reference's operation order, so the GPU mesher can be compared bit for bit.

The heightmap's lighting uses Magnum's vector operations, restated as: dot =
sum of products accumulated left to right from zero, cross = (a.y*b.z - b.y*a.z,
a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y), normalized = v * (1 / sqrt(dot)).  Magnum is
not vendored, so these forms are assumptions (the bloxel mesher needs none).
"""
from __future__ import annotations

import numpy as np

from oracle.oracle import OracleTree

F = np.float32
LIGHT_DIR = (F(0.6), F(1.0), F(0.4))       # MeshNoisePreview.h:158
AMBIENT_LIGHT = F(0.3)                       # :159
AO_STRENGTH = F(0.9)                         # :160


def grid_positions_3d(size_gen: int, start: int):
    """GridPositions3D<SizeGen, StartOffset> (MeshNoisePreview.cpp:31-55), x fastest."""
    r = np.arange(size_gen, dtype=np.int64) + start
    z, y, x = np.meshgrid(r, r, r, indexing="ij")
    return x.ravel().astype(np.float32), y.ravel().astype(np.float32), z.ravel().astype(np.float32)


def grid_positions_2d(size_gen: int):
    r = np.arange(size_gen, dtype=np.int64)
    y, x = np.meshgrid(r, r, indexing="ij")
    return x.ravel().astype(np.float32), y.ravel().astype(np.float32)


def bloxel_densities(root, size: int, pos, seed: int, up_axis_z: bool = False):
    """The (size+2)^3 density array and OutputMinMax of BuildBloxel3DMesh (:447-455)."""
    gx, gy, gz = grid_positions_3d(size + 2, -1)
    ys, zs = (gz, gy) if up_axis_z else (gy, gz)
    off = (float(pos[0]), float(pos[2] if up_axis_z else pos[1]), float(pos[1] if up_axis_z else pos[2]))
    return OracleTree(root).positions([gx, ys, zs], off, seed)


def _bloxel_quad(verts, idx, density, iso, i, facing, oa, ob, light, p00, p01, p11, p10):
    """BloxelAddQuadAO (:542-590)."""
    f = i + facing
    sa0 = int(density[f - oa] <= iso)
    sa1 = int(density[f + oa] <= iso)
    sb0 = int(density[f - ob] <= iso)
    sb1 = int(density[f + ob] <= iso)
    c00 = int((sa0 & sb0) or density[f - oa - ob] <= iso)
    c01 = int((sa0 & sb1) or density[f - oa + ob] <= iso)
    c10 = int((sa1 & sb0) or density[f + oa - ob] <= iso)
    c11 = int((sa1 & sb1) or density[f + oa + ob] <= iso)
    ao_adjust = F(AO_STRENGTH / F(3.0))
    ao00 = F(sa0 + sb0 + c00) * ao_adjust
    ao01 = F(sa1 + sb0 + c10) * ao_adjust
    ao10 = F(sa0 + sb1 + c01) * ao_adjust
    ao11 = F(sa1 + sb1 + c11) * ao_adjust
    shift = (iso - density[i]) * F(4)
    light = F(light - shift)
    light = F(light * abs(light))
    light = light if AMBIENT_LIGHT < light else AMBIENT_LIGHT          # std::max(AMBIENT_LIGHT, light)
    base = len(verts)
    verts.append((*p00, F(F(1) - ao00) * light))
    verts.append((*p01, F(F(1) - ao01) * light))
    verts.append((*p10, F(F(1) - ao10) * light))
    verts.append((*p11, F(F(1) - ao11) * light))
    rot = 2 * int(F(ao00 + ao11) > F(ao01 + ao10))
    idx += [base, base + 3 - rot, base + 2, base + 3, base + rot, base + 1]


def bloxel_mesh(density: np.ndarray, minmax, size: int, pos, iso: float):
    """BuildBloxel3DMesh (:443-540) on a given density array.  Returns
    (vertices float32[n, 4] = x, y, z, light; indices uint32; minAir; maxSolid)."""
    iso = F(iso)
    density = np.asarray(density, np.float32)
    sg = size + 2
    sx, sy, sz = 1, sg, sg * sg
    verts, idx = [], []
    min_air, max_solid = F(np.inf), F(-np.inf)
    px, py, pz = (F(p) for p in pos)
    if minmax[0] > iso:
        return np.zeros((0, 4), np.float32), np.zeros(0, np.uint32), F(py), max_solid
    if minmax[1] < iso:
        return np.zeros((0, 4), np.float32), np.zeros(0, np.uint32), min_air, F(F(py - F(1.0)) + F(size))
    sun = tuple(F(c * F(F(1) - AMBIENT_LIGHT)) for c in LIGHT_DIR)
    one = F(1)
    i = sx + sy + sz
    for z in range(size):
        zf = F(F(z) + pz)
        for y in range(size):
            yf = F(F(y) + py)
            for x in range(size):
                xf = F(F(x) + px)
                if density[i] <= iso:
                    max_solid = max_solid if yf < max_solid else yf        # std::max(yf, maxSolid)
                    x1, y1, z1 = F(xf + one), F(yf + one), F(zf + one)
                    if density[i + sx] > iso:
                        _bloxel_quad(verts, idx, density, iso, i, sx, sy, sz, F(sun[0] + AMBIENT_LIGHT),
                                     (x1, yf, zf), (x1, y1, zf), (x1, y1, z1), (x1, yf, z1))
                    if density[i - sx] > iso:
                        _bloxel_quad(verts, idx, density, iso, i, -sx, -sy, sz, F(one - sun[0]),
                                     (xf, y1, zf), (xf, yf, zf), (xf, yf, z1), (xf, y1, z1))
                    if density[i + sy] > iso:
                        _bloxel_quad(verts, idx, density, iso, i, sy, sz, sx, F(sun[1] + AMBIENT_LIGHT),
                                     (xf, y1, zf), (xf, y1, z1), (x1, y1, z1), (x1, y1, zf))
                    if density[i - sy] > iso:
                        _bloxel_quad(verts, idx, density, iso, i, -sy, -sz, sx, F(one - sun[1]),
                                     (xf, yf, z1), (xf, yf, zf), (x1, yf, zf), (x1, yf, z1))
                    if density[i + sz] > iso:
                        _bloxel_quad(verts, idx, density, iso, i, sz, sx, sy, F(sun[2] + AMBIENT_LIGHT),
                                     (xf, yf, z1), (x1, yf, z1), (x1, y1, z1), (xf, y1, z1))
                    if density[i - sz] > iso:
                        _bloxel_quad(verts, idx, density, iso, i, -sz, -sx, sy, F(one - sun[2]),
                                     (x1, yf, zf), (xf, yf, zf), (xf, y1, zf), (x1, y1, zf))
                else:
                    min_air = min_air if min_air < yf else yf              # std::min(yf, minAir)
                i += 1
            i += sx * 2
        i += sy * 2
    return (np.array(verts, np.float32).reshape(-1, 4), np.array(idx, np.uint32), min_air, max_solid)


def heightmap_densities(root, size: int, pos, seed: int):
    """The (size+1)^2 density array of BuildHeightMap2DMesh (:958-962): x = pos.x, y = pos.z."""
    gx, gy = grid_positions_2d(size + 1)
    return OracleTree(root).positions([gx, gy], (float(pos[0]), float(pos[2])), seed)


def _dot(a, b):
    acc = F(0)
    for u, v in zip(a, b):
        acc = F(acc + F(u * v))
    return acc


def _cross(a, b):
    return (F(F(a[1] * b[2]) - F(b[1] * a[2])), F(F(a[2] * b[0]) - F(b[2] * a[0])), F(F(a[0] * b[1]) - F(b[0] * a[1])))


def _normalized(v):
    inv = F(F(1) / F(np.sqrt(_dot(v, v))))
    return tuple(F(c * inv) for c in v)


def _sub(a, b):
    return tuple(F(u - w) for u, w in zip(a, b))


def _add(a, b):
    return tuple(F(u + w) for u, w in zip(a, b))


def heightmap_mesh(density: np.ndarray, size: int, pos, multiplier: float):
    """BuildHeightMap2DMesh (:956-1004) on a given density array."""
    density = np.asarray(density, np.float32)
    mul = F(multiplier)
    sg = size + 1
    verts, idx = [], []
    px, pz = F(pos[0]), F(pos[2])
    i = 0
    for y in range(size):
        yf = F(F(y) + pz)
        for x in range(size):
            xf = F(F(x) + px)
            x1, y1 = F(xf + F(1)), F(yf + F(1))
            v00 = (xf, F(density[i] * mul), yf)
            v01 = (xf, F(density[i + sg] * mul), y1)
            v10 = (x1, F(density[i + 1] * mul), yf)
            v11 = (x1, F(density[i + 1 + sg] * mul), y1)
            n = _add(_normalized(_cross(_sub(v10, v11), _sub(v00, v11))), _normalized(_cross(_sub(v01, v00), _sub(v11, v00))))
            ln = tuple(F(l * c) for l, c in zip(LIGHT_DIR, _normalized(n)))
            light = _dot(ln, ln)
            base = len(verts)
            for v in (v00, v01, v10, v11):
                verts.append((*v, light))
            rot = 2 * int(_dot(_add(v00, v11), _add(v00, v11)) < _dot(_add(v01, v10), _add(v01, v10)))
            idx += [base, base + 3 - rot, base + 2, base + 3, base + rot, base + 1]
            i += 1
        i += 1
    return np.array(verts, np.float32).reshape(-1, 4), np.array(idx, np.uint32)
