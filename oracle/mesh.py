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


# ---- dual marching cubes: BuildDmc3DMesh (:592-769), DmcGetVertIndex (:771-953)

# Cell corners are numbered x + 2y + 4z; edge k joins DMC_EDGE_CORNERS[k] (the numbering of the
# reference's util/DmcTable.inl).  Faces list their corners in cyclic order; face edge k joins
# corner k and corner k + 1.
DMC_EDGE_CORNERS = ((0, 1), (1, 5), (4, 5), (0, 4), (2, 3), (3, 7), (6, 7), (2, 6), (0, 2), (1, 3), (5, 7), (4, 6))
DMC_FACES = (((0, 2, 6, 4), (8, 7, 11, 3)), ((1, 3, 7, 5), (9, 5, 10, 1)), ((0, 1, 5, 4), (0, 1, 2, 3)),
             ((2, 3, 7, 6), (4, 5, 6, 7)), ((0, 1, 3, 2), (0, 9, 4, 8)), ((4, 5, 7, 6), (2, 10, 6, 11)))


def dmc_dual_points(case: int):
    """The dual points of one marching-cubes case (bit k = corner k above the iso level), each
    as the bit set of the cut edges of one surface piece: the reference's kDualPointsList row,
    derived from the face contours.  A face with two cut edges joins them; on an ambiguous face
    (four cut edges) every corner above the iso level is cut off on its own."""
    cut = [((case >> a) & 1) != ((case >> b) & 1) for a, b in DMC_EDGE_CORNERS]
    label = list(range(12))

    def root(e):
        while label[e] != e:
            e = label[e]
        return e

    def join(a, b):
        ra, rb = root(a), root(b)
        label[max(ra, rb)] = min(ra, rb)

    for corners, edges in DMC_FACES:
        ce = [e for e in edges if cut[e]]
        if len(ce) == 2:
            join(*ce)
        elif len(ce) == 4:
            for k, c in enumerate(corners):
                if (case >> c) & 1:
                    join(edges[(k + 3) % 4], edges[k])
    pieces = {}
    for e in range(12):
        if cut[e]:
            pieces[root(e)] = pieces.get(root(e), 0) | (1 << e)
    return list(pieces.values())


def dmc_table():
    return [dmc_dual_points(c) for c in range(256)]


def dmc_table_digest(table) -> str:
    """sha256 of the table in a canonical text form (per case, its point codes sorted)."""
    import hashlib
    text = "\n".join(f"{c}:" + ",".join(str(v) for v in sorted(x for x in row if x)) for c, row in enumerate(table))
    return hashlib.sha256(text.encode()).hexdigest()


def dmc_densities(root, size: int, pos, seed: int, up_axis_z: bool = False):
    """The (size+4)^3 density array and OutputMinMax of BuildDmc3DMesh (:594-603)."""
    gx, gy, gz = grid_positions_3d(size + 4, -2)
    ys, zs = (gz, gy) if up_axis_z else (gy, gz)
    off = (float(pos[0]), float(pos[2] if up_axis_z else pos[1]), float(pos[1] if up_axis_z else pos[2]))
    return OracleTree(root).positions([gx, ys, zs], off, seed)


def _sqrt_newton(x):
    """SqrtNewtonRaphson (:21-24) in float32."""
    curr, prev = F(x), F(0)
    while curr != prev:
        curr, prev = F(F(0.5) * F(curr + F(x / curr))), curr
    return curr


def _normalise_constexpr(v):
    """NormaliseConstExpr (:26-30); Magnum's vector / scalar divides each component."""
    len_sqr = F(F(F(v[0] * v[0]) + F(v[1] * v[1])) + F(v[2] * v[2]))
    s = _sqrt_newton(len_sqr)
    return tuple(F(c / s) for c in v)


def _lroundf(v) -> int:
    """C lroundf: nearest integer, halves away from zero."""
    a = int(np.floor(abs(float(v)) + 0.5))
    return a if v >= 0 else -a


def dmc_mesh(density: np.ndarray, minmax, size: int, pos, iso: float):
    """BuildDmc3DMesh (:592-769) on a given density array.  Returns (vertices float32[n, 4] =
    x, y, z, light; indices uint32; minAir; maxSolid)."""
    iso = F(iso)
    d = np.asarray(density, np.float32)
    sg = size + 4
    SX, SY, SZ = 1, sg, sg * sg
    px, py, pz = (int(p) for p in pos)
    if minmax[0] > iso:
        return np.zeros((0, 4), np.float32), np.zeros(0, np.uint32), F(py), F(-np.inf)
    if minmax[1] < iso:
        return np.zeros((0, 4), np.float32), np.zeros(0, np.uint32), F(np.inf), F(F(F(py) - F(1.0)) + F(size))
    table = dmc_table()
    nl = _normalise_constexpr(tuple(F(-c) for c in LIGHT_DIR))
    shade_a = F(F(0.5) - F(AMBIENT_LIGHT * F(0.5)))
    shade_b = F(F(0.5) + F(AMBIENT_LIGHT * F(0.5)))
    corner = (0, SX, SY, SX + SY, SZ, SX + SZ, SY + SZ, SX + SY + SZ)
    verts, idx, vmap = [], [], {}

    def t(a, b):
        return F(F(iso - d[a]) / F(d[b] - d[a]))

    def lerp(a, b, w):                       # ImLerp
        return F(a + F(F(b - a) * w))

    def vert_index(ci, edge, off):
        """DmcGetVertIndex (:771-953)."""
        case = 0
        for k, o in enumerate(corner):
            if d[ci + o] > iso:
                case |= 1 << k
        code = next(p for p in table[case] if p & (1 << edge))
        key = (ci << 12) | code
        if key in vmap:
            return vmap[key]
        x = y = z = F(0)
        one = F(1)
        if code & 1: x = F(x + t(ci, ci + SX))
        if code & 2: x = F(x + one); z = F(z + t(ci + SX, ci + SX + SZ))
        if code & 4: x = F(x + t(ci + SZ, ci + SX + SZ)); z = F(z + one)
        if code & 8: z = F(z + t(ci, ci + SZ))
        if code & 16: x = F(x + t(ci + SY, ci + SX + SY)); y = F(y + one)
        if code & 32: x = F(x + one); y = F(y + one); z = F(z + t(ci + SX + SY, ci + SX + SY + SZ))
        if code & 64: x = F(x + t(ci + SY + SZ, ci + SX + SY + SZ)); y = F(y + one); z = F(z + one)
        if code & 128: y = F(y + one); z = F(z + t(ci + SY, ci + SY + SZ))
        if code & 256: y = F(y + t(ci, ci + SY))
        if code & 512: x = F(x + one); y = F(y + t(ci + SX, ci + SX + SY))
        if code & 1024: x = F(x + one); y = F(y + t(ci + SX + SZ, ci + SX + SY + SZ)); z = F(z + one)
        if code & 2048: y = F(y + t(ci + SZ, ci + SY + SZ)); z = F(z + one)
        n = F(bin(code).count("1"))
        v = (F(x / n), F(y / n), F(z / n))
        ox, oy, oz = SX & _lroundf(-v[0]), SY & _lroundf(-v[1]), SZ & _lroundf(-v[2])
        dd = [F(c + F(0.5)) for c in v]
        dd = [F(c - F(np.floor(c))) for c in dd]
        der = [F(0), F(0), F(0)]
        cur = ci
        for zz in (-1, 0):
            cz = F(abs(F(F(zz) + v[2])))
            for yy in (-1, 0):
                cy = F(abs(F(F(yy) + v[1])))
                for xx in (-1, 0):
                    cx = F(abs(F(F(xx) + v[0])))
                    if xx:
                        k = cur + ox
                        der[0] = F(der[0] + F(F(cy * cz) * lerp(F(d[k - SX] - d[k]), F(d[k] - d[k + SX]), dd[0])))
                    if yy:
                        k = cur + oy
                        der[1] = F(der[1] + F(F(cx * cz) * lerp(F(d[k - SY] - d[k]), F(d[k] - d[k + SY]), dd[1])))
                    if zz:
                        k = cur + oz
                        der[2] = F(der[2] + F(F(cx * cy) * lerp(F(d[k - SZ] - d[k]), F(d[k] - d[k + SZ]), dd[2])))
                    cur += SX
                cur += SY - SX * 2
            cur += SZ - SY * 2
        with np.errstate(divide="ignore", invalid="ignore"):
            light = F(F(_dot(nl, _normalized(tuple(der))) * shade_a) + shade_b)
        light = F(light * light)
        light = light if light < F(1) else F(1)              # std::min(1.0f, light): NaN -> 1
        vmap[key] = len(verts)
        verts.append((F(v[0] + off[0]), F(v[1] + off[1]), F(v[2] + off[2]), light))
        return vmap[key]

    def quad(q, flip_cond):
        rot = 2 * int(abs(F(verts[q[0]][3] - verts[q[3]][3])) > abs(F(verts[q[1]][3] - verts[q[2]][3])))
        flip = 2 * int(flip_cond)
        idx.extend([q[flip], q[3 - rot], q[2 - flip], q[3 - flip], q[rot], q[1 + flip]])

    min_air, max_solid = F(np.inf), F(-np.inf)
    one = F(1)
    ci = (SX + SY + SZ) * 2
    for z in range(size):
        cz = F(pz + z)
        for y in range(size):
            cy = F(py + y)
            for x in range(size):
                cx = F(px + x)
                dens = d[ci]
                inside = dens <= iso
                dx = d[ci + SX]
                if inside != (dx <= iso):
                    q = [vert_index(ci, 0, (cx, cy, cz)), vert_index(ci - SZ, 2, (cx, cy, F(cz - one))),
                         vert_index(ci - SY, 4, (cx, F(cy - one), cz)), vert_index(ci - SY - SZ, 6, (cx, F(cy - one), F(cz - one)))]
                    quad(q, dens < dx)
                dy = d[ci + SY]
                if inside != (dy <= iso):
                    q = [vert_index(ci, 8, (cx, cy, cz)), vert_index(ci - SX, 9, (F(cx - one), cy, cz)),
                         vert_index(ci - SZ, 11, (cx, cy, F(cz - one))), vert_index(ci - SX - SZ, 10, (F(cx - one), cy, F(cz - one)))]
                    quad(q, dens < dy)
                    ys = [verts[k][1] for k in q]
                    if inside:
                        max_solid = max([max_solid] + ys)
                    else:
                        min_air = min([min_air] + ys)
                dz = d[ci + SZ]
                if inside != (dz <= iso):
                    q = [vert_index(ci, 3, (cx, cy, cz)), vert_index(ci - SY, 7, (cx, F(cy - one), cz)),
                         vert_index(ci - SX, 1, (F(cx - one), cy, cz)), vert_index(ci - SX - SY, 5, (F(cx - one), F(cy - one), cz))]
                    quad(q, dens < dz)
                ci += SX
            ci += SX * (sg - size)
        ci += SY * (sg - size)
    return (np.array(verts, np.float32).reshape(-1, 4), np.array(idx, np.uint32), min_air, max_solid)
